"""The FP64 call that allocates nothing (kwg_fd1d_price_device_static).

Some callers cannot call cudaMalloc: a pricing step inside a host application whose
device memory belongs to another allocator or is held to a fixed budget, or a
latency-critical path where cudaMalloc's implicit synchronisation is not allowed.
For them the library keeps its scratch in one fixed 64 MiB device array.  These
tests call that entry point through the C ABI twice in a row, on batches of
different sizes and option mixes (so the second call runs over the first call's
leftovers), and check
  * that its prices are bit-identical to the allocating entry point's
    (kwg_fd1d_price_device, same Thomas solver),
  * that they match the oracle to the FP64 parity tolerance of the other GPU tests,
  * that the device's free memory is the same before and after the calls,
  * that oversized batches, strict mode and device dedup are refused before any
    launch.
The file is collected last."""
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


def _mixed(n, seed):
    """American and European puts and calls, interleaved in caller order."""
    import portfolio

    o = portfolio.american_portfolio(n, seed=seed)
    o["e"][1::3] = 0
    o["w"][::2] = -o["w"][::2]
    return o


def _cases():
    import kwg
    import portfolio

    return [
        (portfolio.american_portfolio(700, seed=11),
         kwg.params(t_dim=300, x_dim=1024, scale=5.0, density=0.25, solver=kwg.SOLVER_THOMAS)),
        (_mixed(97, seed=12), kwg.params(t_dim=129, x_dim=257, scale=5.0, density=np.inf, solver=kwg.SOLVER_THOMAS)),
        (_mixed(301, seed=13), kwg.params(t_dim=200, x_dim=512, scale=5.0, density=0.25, solver=kwg.SOLVER_THOMAS,
                                          block_warps=2)),
        # one 4-warp block per SM: the streaming solver's big stages
        (_mixed(250, seed=14), kwg.params(t_dim=150, x_dim=640, scale=5.0, density=np.inf, solver=kwg.SOLVER_THOMAS,
                                          block_warps=4, sm_blocks=1)),
    ]


def test_static_scratch_matches_allocating_call_and_oracle(ctx):
    import torch

    import kwg
    import kwor

    fn = _static_fn()
    stream = torch.cuda.Stream()
    err = ctypes.create_string_buffer(256)
    for opts, prm in _cases():
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
        np.testing.assert_array_equal(got, want)
        rc, msg, ref, _ = kwor.fd1d_price(opts, t_dim=prm.t_dim, x_dim=prm.x_dim, scale=prm.scale,
                                          density=prm.density)
        assert rc == 0, msg
        rel = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), PRICE_FLOOR))
        assert rel <= REL_TOL, rel


def test_static_scratch_allocates_nothing(ctx):
    import torch

    import kwg

    fn = _static_fn()
    err = ctypes.create_string_buffer(256)
    batches = [(_device_batch(o), p) for o, p in _cases()]
    # warm-up: the first call on the device does the set-up (module load, address look-up)
    (d_o, d_p, d_s), prm = batches[0]
    assert fn(d_o.data_ptr(), d_p.numel(), ctypes.byref(prm), d_p.data_ptr(), d_s.data_ptr(), None, err, 256) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        for (d_o, d_p, d_s), prm in batches:
            rc = fn(d_o.data_ptr(), d_p.numel(), ctypes.byref(prm), d_p.data_ptr(), d_s.data_ptr(), None, err, 256)
            assert rc == kwg.KWG_OK, err.value.decode()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    for (_, d_p, d_s), _ in batches:
        assert (d_s == 0).all() and not torch.isnan(d_p).any()


def test_static_scratch_rejects_what_it_cannot_do(ctx):
    import torch

    import kwg
    import portfolio

    fn = _static_fn()
    err = ctypes.create_string_buffer(256)
    big = portfolio.american_portfolio(4096, seed=3)  # 4096 x 1024 nodes needs ~336 MB > 64 MiB
    small = portfolio.american_portfolio(64, seed=4)
    refused = [(big, kwg.params(t_dim=16, x_dim=1024), "scratch"),
               (small, kwg.params(t_dim=16, x_dim=64, strict=1), "strict"),
               (small, kwg.params(t_dim=16, x_dim=64, solver=kwg.SOLVER_PCR), "Thomas")]
    dd = kwg.params(t_dim=16, x_dim=64)
    dd.device_dedup = 1
    refused.append((small, dd, "device_dedup"))
    for opts, prm, word in refused:
        d_o, d_p, d_s = _device_batch(opts)
        rc = fn(d_o.data_ptr(), len(opts), ctypes.byref(prm), d_p.data_ptr(), d_s.data_ptr(), None, err, 256)
        assert rc == kwg.KWG_ERR_INVALID
        assert word in err.value.decode()
        torch.cuda.synchronize()
        assert torch.isnan(d_p).all()  # nothing was launched
