"""The FP64 call that allocates nothing (kwg_fd1d_price_device_static).

Some callers cannot call cudaMalloc: a pricing step inside a host application whose
device memory belongs to another allocator or is held to a fixed budget, or a
latency-critical path where cudaMalloc's implicit synchronisation is not allowed.
For them the library keeps its scratch in one fixed 64 MiB device array.  This test
calls that entry point through the C ABI twice in a row, on batches of different
sizes so the second call runs over the first call's leftovers, and checks both
against the allocating entry point (kwg_fd1d_price_device) to the FP64 parity
tolerance of the other GPU tests.  It lives in its own file, collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10
PRICE_FLOOR = 1e-12


def _static_fn():
    import kwg

    L = kwg.lib()
    fn = L.kwg_fd1d_price_device_static
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(kwg.Fd1dParams), ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    fn.restype = ctypes.c_int
    return fn


def _device_batch(opts):
    import torch

    d_o = torch.from_numpy(opts.view(np.uint8).copy()).cuda()
    d_p = torch.full((len(opts),), float("nan"), dtype=torch.float64, device="cuda")
    d_s = torch.full((len(opts),), -1, dtype=torch.int32, device="cuda")
    return d_o, d_p, d_s


def test_static_scratch_matches_allocating_call(ctx):
    import torch

    import kwg
    import portfolio

    fn = _static_fn()
    stream = torch.cuda.Stream()
    err = ctypes.create_string_buffer(256)
    cases = [(portfolio.american_portfolio(700, seed=11), kwg.params(t_dim=300, x_dim=1024, scale=5.0, density=0.25)),
             (portfolio.american_portfolio(97, seed=12), kwg.params(t_dim=129, x_dim=257, scale=5.0, density=np.inf))]
    for opts, prm in cases:
        d_o, d_p, d_s = _device_batch(opts)
        rc = fn(d_o.data_ptr(), len(opts), ctypes.byref(prm), d_p.data_ptr(), d_s.data_ptr(), stream.cuda_stream,
                err, 256)
        assert rc == kwg.KWG_OK, err.value.decode()
        w_o, w_p, w_s = _device_batch(opts)
        rc = ctx.fd1d_price_device(w_o.data_ptr(), len(opts), prm, w_p.data_ptr(), w_s.data_ptr(),
                                   stream.cuda_stream)
        assert rc == kwg.KWG_OK, ctx.last_error()
        stream.synchronize()
        got, want = d_p.cpu().numpy(), w_p.cpu().numpy()
        assert (d_s.cpu().numpy() == 0).all() and (w_s.cpu().numpy() == 0).all()
        rel = np.max(np.abs(got - want) / np.maximum(np.abs(want), PRICE_FLOOR))
        assert rel <= REL_TOL, rel


def test_static_scratch_rejects_oversized_batches(ctx):
    import torch

    import kwg
    import portfolio

    fn = _static_fn()
    err = ctypes.create_string_buffer(256)
    opts = portfolio.american_portfolio(4096, seed=3)  # 4096 x 1024 nodes needs ~336 MB > 64 MiB
    prm = kwg.params(t_dim=16, x_dim=1024)
    d_o, d_p, d_s = _device_batch(opts)
    rc = fn(d_o.data_ptr(), len(opts), ctypes.byref(prm), d_p.data_ptr(), d_s.data_ptr(), None, err, 256)
    assert rc == kwg.KWG_ERR_INVALID
    assert "scratch" in err.value.decode()
    torch.cuda.synchronize()
    assert torch.isnan(d_p).all()  # nothing was launched
