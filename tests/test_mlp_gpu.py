"""Tensor-core (tcgen05) GEMM and the MLP surrogate built on it, against FP32 / FP64
references on the same BF16 inputs."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gemm(a, b):
    import torch

    import kwg

    m, k = a.shape
    n = b.shape[0]
    c = torch.full((m, n), float("nan"), dtype=torch.float32, device="cuda")
    rc = kwg.lib().kwg_gemm_bf16(a.data_ptr(), b.data_ptr(), c.data_ptr(), m, n, k, None)
    assert rc == 0
    torch.cuda.synchronize()
    return c


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (128, 128, 128), (256, 384, 320), (200, 100, 192)])
def test_gemm_matches_torch(built, m, n, k):
    """C = A B^T with BF16 inputs and FP32 accumulation: every product is exact in
    FP32, so only the summation order differs from the FP32 reference."""
    import torch

    g = torch.Generator(device="cpu").manual_seed(m * 7 + n * 3 + k)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(n, k, generator=g).to(torch.bfloat16).cuda()
    c = gemm(a, b)
    ref = a.double() @ b.double().T
    err = (c.double() - ref).abs().max().item()
    assert err <= 1e-4 * max(1.0, ref.abs().max().item()), err


# ----------------------------------------------------------------------------- surrogate network

def _features(n, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, (n, 5)).astype(np.float32)


def _padded(f):
    x = np.zeros((len(f), 128))
    x[:, :5] = f
    return x


@pytest.fixture(scope="module")
def net(built):
    import kwg

    s = kwg.Surrogate(0, seed=7)
    yield s
    s.close()


@pytest.mark.parametrize("n", [1, 300, 4096])
def test_forward_matches_oracle(net, n):
    """GPU forward (split-BF16 inputs, BF16 weights, FP32 accumulation, FP32 head)
    against the FP64 oracle applying the same roundings."""
    import torch

    import mlp_oracle as mo

    p = mo.random_params(11)
    net.set_params(p)
    f = _features(n, n)
    d_f = torch.from_numpy(f).cuda()
    d_y = torch.empty(n, dtype=torch.float32, device="cuda")
    net.forward(d_f.data_ptr(), n, d_y.data_ptr())
    y = d_y.cpu().numpy().astype(np.float64)
    yo, _ = mo.forward(p, _padded(f))
    assert np.max(np.abs(y - yo)) <= 2e-4 * max(1.0, np.max(np.abs(yo)))


@pytest.mark.parametrize("floors", [False, True])
def test_gradients_match_oracle(net, floors):
    """Every parameter's gradient of the loss (tensor-core backward, split-K weight
    gradients) against the oracle's, per weight and bias block; with floors, a third
    of the rows are early-exercise rows with the one-sided loss."""
    import torch

    import kwg
    import mlp_oracle as mo

    n = 300
    p = mo.random_params(12)
    net.set_params(p)
    f = _features(n, 5)
    rng = np.random.default_rng(6)
    t = rng.normal(size=n).astype(np.float32)
    fl = None
    if floors:
        fl = np.where(np.arange(n) % 3 == 0, rng.normal(size=n), -mo.NO_FLOOR).astype(np.float32)
    d_f, d_t = torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()
    d_fl = torch.from_numpy(fl).cuda() if floors else None
    d_g = torch.full((kwg.MLP_PARAMS,), float("nan"), dtype=torch.float32, device="cuda")
    loss = net.gradients(d_f.data_ptr(), d_t.data_ptr(), n, d_g.data_ptr(), d_fl.data_ptr() if floors else 0)
    g = d_g.cpu().numpy().astype(np.float64)
    lo, go = mo.gradients(p, _padded(f), t.astype(np.float64), floor=None if fl is None else fl.astype(np.float64))
    assert abs(loss - lo) <= 1e-4 * lo
    W, NW = mo.W, mo.N_WEIGHTS
    for l in range(mo.LAYERS):
        for a, b in ((l * W * W, (l + 1) * W * W), (NW + l * W, NW + (l + 1) * W)):
            ref = go[a:b]
            assert np.linalg.norm(g[a:b] - ref) <= 5e-3 * np.linalg.norm(ref), (l, a)
    # inactive entries (layer-1 inputs 5..127, head outputs 1..127) get exactly 0
    g0 = g[:W * W].reshape(W, W)
    assert np.all(g0[:, 5:] == 0)
    g4 = g[4 * W * W:5 * W * W].reshape(W, W)
    assert np.all(g4[1:] == 0) and np.all(g[NW + 4 * W + 1:] == 0)


def _fd_prices(ctx, opts, **kw):
    import kwg

    rc, p, st = ctx.fd1d_price(opts, kwg.params(**kw))
    assert rc == kwg.KWG_OK, ctx.last_error()
    assert (st == 0).all()
    return p


def european(opts):
    """Black-Scholes price of the same contracts with European exercise."""
    import kwor

    e = opts.copy()
    e["e"] = 0
    return kwor.bs_price(e)


LABEL_GRID = dict(t_dim=256, x_dim=256, scale=5.0, density=math.inf)


@pytest.fixture(scope="module")
def trained(ctx, built):
    """A surrogate trained on the GPU on FD64 prices of 16384 options (S=100,
    K~U[80,120], vol~U[0.1,0.6], r,q~U[0,0.1], T~U[0.25,2]; 256 x 256 uniform grid) generated by the GPU solver."""
    import torch

    import kwg
    import portfolio

    opts = portfolio.american_portfolio(16384, seed=101)
    prices = _fd_prices(ctx, opts, **LABEL_GRID)
    d_o = torch.from_numpy(opts.view(np.uint8).copy()).cuda()
    d_p = torch.from_numpy(prices).cuda()
    s = kwg.Surrogate(0, seed=3)
    last = s.train(d_o.data_ptr(), d_p.data_ptr(), len(opts), epochs=60, batch=256, lr=2e-3, seed=6)
    yield s, opts, prices, last
    s.close()


def test_training_reduces_loss(trained):
    """The loss on the (scaled) premium targets of the training set, before and
    after training, through the same gradient entry point the training uses."""
    import torch

    import kwg
    import kwor

    s, opts, prices, last = trained
    _, _, _, y_scale = s.get_params()
    sub, price = opts[:4096], prices[:4096]
    d_o = torch.from_numpy(sub.view(np.uint8).copy()).cuda()
    d_f = torch.empty((len(sub), 5), dtype=torch.float32, device="cuda")
    d_b = torch.empty(len(sub), dtype=torch.float64, device="cuda")
    s.featurize(d_o.data_ptr(), len(sub), d_f.data_ptr(), 0, d_b.data_ptr())
    base = d_b.cpu().numpy()
    k = sub["k"]
    intr = np.maximum(0.0, np.where(sub["w"] < 0, k - sub["s"], sub["s"] - k))
    t = ((price - base) / k * y_scale).astype(np.float32)
    exercise = (intr > 0) & (price - intr <= 1e-6 * k)
    fl = np.where(exercise, (intr - base) / k * y_scale, -1e30).astype(np.float32)
    d_t, d_fl = torch.from_numpy(t).cuda(), torch.from_numpy(fl).cuda()
    d_g = torch.empty(kwg.MLP_PARAMS, dtype=torch.float32, device="cuda")
    after = s.gradients(d_f.data_ptr(), d_t.data_ptr(), len(sub), d_g.data_ptr(), d_fl.data_ptr())
    fresh = kwg.Surrogate(0, seed=3)
    before = fresh.gradients(d_f.data_ptr(), d_t.data_ptr(), len(sub), d_g.data_ptr(), d_fl.data_ptr())
    fresh.close()
    assert after < 1e-2 * before, (before, after, last)
    assert after < 5e-3  # targets are scaled to unit standard deviation


def test_training_recovers_from_loss_spikes(ctx):
    """A learning rate far too large for Adam makes the loss blow up; the training
    returns to its best epoch's parameters with fresh moments and half the rate each
    time, and ends with finite parameters whose loss is the kept epoch's."""
    import torch

    import kwg
    import portfolio

    opts = portfolio.american_portfolio(4096, seed=202)
    prices = _fd_prices(ctx, opts, t_dim=64, x_dim=128, scale=5.0, density=math.inf)
    d_o = torch.from_numpy(opts.view(np.uint8).copy()).cuda()
    d_p = torch.from_numpy(prices).cuda()
    s = kwg.Surrogate(0, seed=4)
    try:
        # lr 1e4 overflows within the first epochs; halving 24 times brings it to ~6e-4
        last = s.train(d_o.data_ptr(), d_p.data_ptr(), len(opts), epochs=24, batch=256, lr=1e4, seed=8)
        h = s.train_history()
        losses = h["losses"]
        best, kept, restarts = math.inf, -1, 0  # the rule, replayed on the history
        for i, v in enumerate(losses):
            if np.isfinite(v) and v < best:
                best, kept = v, i
            elif not np.isfinite(v) or v > 3 * best:
                restarts += 1
        assert restarts >= 1
        assert h["restarts"] == restarts and h["best_epoch"] == kept, (h, restarts, kept)
        assert last == (losses[kept] if kept >= 0 else losses[-1])
        p, _, _, _ = s.get_params()
        assert np.isfinite(p).all()
        d_out = torch.empty(len(opts), dtype=torch.float64, device="cuda")
        s.price_device(d_o.data_ptr(), len(opts), d_out.data_ptr())
        torch.cuda.synchronize()
        assert torch.isfinite(d_out).all()
    finally:
        s.close()


def test_training_keeps_the_best_epoch(trained):
    """The training history: one mean loss per epoch, the kept epoch is the one with
    the lowest loss, and the loss train() reports is that epoch's."""
    s, _, _, last = trained
    h = s.train_history()
    assert len(h["losses"]) == 60
    assert np.isfinite(h["losses"]).all()
    assert h["best_epoch"] == int(np.argmin(h["losses"]))
    assert last == h["losses"][h["best_epoch"]]
    assert h["restarts"] >= 0
    assert h["losses"][h["best_epoch"]] < 1e-2 * h["losses"][0]


def test_trained_network_beats_analytic_prices(trained, ctx):
    """What the network gains: on fresh options, the surrogate price (analytic base +
    learned premium) is far closer to FD64 than the same method without the network,
    i.e. the Barone-Adesi-Whaley base alone, or the European price."""
    import torch

    import mlp_oracle as mo
    import portfolio

    s = trained[0]
    test = portfolio.american_portfolio(4096, seed=202)
    fd = _fd_prices(ctx, test, **LABEL_GRID)
    d_o = torch.from_numpy(test.view(np.uint8).copy()).cuda()
    d_p = torch.empty(len(test), dtype=torch.float64, device="cuda")
    d_in = torch.empty(len(test), dtype=torch.uint8, device="cuda")
    s.price_device(d_o.data_ptr(), len(test), d_p.data_ptr(), d_in.data_ptr())
    torch.cuda.synchronize()
    assert d_in.cpu().numpy().all()
    p99 = {name: np.quantile(np.abs(v - fd), 0.99) for name, v in
           (("net", d_p.cpu().numpy()), ("baw", mo.baw(test)), ("euro", european(test)))}
    assert p99["net"] <= 0.2 * p99["baw"], p99
    assert p99["net"] <= 0.02 * p99["euro"], p99
    assert p99["net"] <= 0.05, p99


def test_featurize_matches_oracle(net):
    """Features, in-box flags and the analytic base price (device Barone-Adesi-Whaley:
    FP64 European leg, FP32 safeguarded Newton for the critical price; the oracle:
    FP64 bisection) on in-box, out-of-box and European contracts."""
    import torch

    import mlp_oracle as mo
    import portfolio

    net.set_params(mo.random_params(1), mo.BOX_LO, mo.BOX_HI, 1.0)
    o = portfolio.american_portfolio(5000, seed=55)
    o["k"][::7] *= 1.5       # log K/S above the box
    o["z"][3::11] = 2.0      # vol sqrt T above the box
    o["e"][5::13] = 0        # European
    o["r"][6::17] = 0.0      # puts never exercised early
    o["q"][8::19] = 0.0      # calls never exercised early
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_f = torch.empty((len(o), 5), dtype=torch.float32, device="cuda")
    d_in = torch.empty(len(o), dtype=torch.uint8, device="cuda")
    d_b = torch.empty(len(o), dtype=torch.float64, device="cuda")
    net.featurize(d_o.data_ptr(), len(o), d_f.data_ptr(), d_in.data_ptr(), d_b.data_ptr())
    torch.cuda.synchronize()
    f_ref, in_ref = mo.features(o)
    assert np.array_equal(d_in.cpu().numpy().astype(bool), in_ref)
    assert np.max(np.abs(d_f.cpu().numpy() - f_ref)) <= 1e-6 * max(1.0, np.abs(f_ref).max())
    # the European leg is FP64, the critical price and the premium term FP32
    b_ref = mo.baw(o)
    assert np.max(np.abs(d_b.cpu().numpy() - b_ref) / o["k"]) <= 1e-6


def test_save_load_roundtrip(trained, tmp_path):
    import kwg

    s = trained[0]
    path = str(tmp_path / "w.npz")
    s.save(path)
    t = kwg.Surrogate(0, seed=99)
    t.load(path)
    a, b = s.get_params(), t.get_params()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[3] == b[3]
    t.close()


def test_surrogate_routes_and_audits(trained, ctx):
    """Out-of-box options (K/S far outside, European exercise) go to FD, a seeded
    audit fraction is priced both ways and its error reported, the rest keeps the
    network price."""
    import torch

    import kwg
    import portfolio

    s = trained[0]
    opts = portfolio.american_portfolio(3000, seed=303)
    opts["z"][::50] = 2.0  # vol sqrt(T) >= 1 is outside the box (and the spot stays on the FD grid)
    opts["e"][1::50] = 0
    oob = np.zeros(len(opts), bool)
    oob[::50] = oob[1::50] = True
    fd = kwg.params(precision=kwg.FP32, **LABEL_GRID)
    prices, route, audit = s.price(ctx, opts, fd, audit_frac=0.1, seed=3)
    assert (route != kwg.ROUTE_FD_FAILED).all()
    assert np.array_equal(route == kwg.ROUTE_OUT_OF_BOX, oob)
    aud = route == kwg.ROUTE_AUDIT
    n_in = (~oob).sum()
    assert abs(aud.sum() - 0.1 * n_in) <= 5 * math.sqrt(0.1 * 0.9 * n_in)
    assert audit.audited == aud.sum() and audit.out_of_box == oob.sum()
    # FD-routed prices are the FD solver's
    fd.strict = 0
    rc, fdp, st = ctx.fd1d_price(opts[route != 0], fd)
    assert rc == 0 and (st == 0).all()
    assert np.allclose(prices[route != 0], fdp, rtol=1e-12, atol=0)
    # network prices elsewhere; the audit statistics compare the two
    d_o = torch.from_numpy(opts.view(np.uint8).copy()).cuda()
    d_p = torch.empty(len(opts), dtype=torch.float64, device="cuda")
    s.price_device(d_o.data_ptr(), len(opts), d_p.data_ptr())
    torch.cuda.synchronize()
    net_p = d_p.cpu().numpy()
    assert np.array_equal(prices[route == 0], net_p[route == 0])
    e = np.abs(net_p[aud] - prices[aud])
    assert math.isclose(audit.audit_abs_max, e.max(), rel_tol=1e-12)
    assert math.isclose(audit.audit_abs_sum, e.sum(), rel_tol=1e-9)


@pytest.mark.parametrize("n", [1, 1000, 2 * 128 * 152 + 5])
def test_fused_price_matches_layer_path(net, n):
    """The fused persistent pricing kernel (weights resident in shared memory,
    activations on chip) against the layer-by-layer tensor-core path: features and
    base price from kwg_mlp_featurize, y from kwg_mlp_forward, then
    max(intrinsic, base + K y / y_scale)."""
    import torch

    import mlp_oracle as mo
    import portfolio

    y_scale = 250.0
    net.set_params(mo.random_params(21), mo.BOX_LO, mo.BOX_HI, y_scale)
    o = portfolio.american_portfolio(n, seed=n)
    if n > 10:
        o["e"][3::10] = 0
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_p = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    d_in = torch.empty(n, dtype=torch.uint8, device="cuda")
    net.price_device(d_o.data_ptr(), n, d_p.data_ptr(), d_in.data_ptr())
    d_f = torch.empty((n, 5), dtype=torch.float32, device="cuda")
    d_in2 = torch.empty(n, dtype=torch.uint8, device="cuda")
    d_b = torch.empty(n, dtype=torch.float64, device="cuda")
    net.featurize(d_o.data_ptr(), n, d_f.data_ptr(), d_in2.data_ptr(), d_b.data_ptr())
    d_y = torch.empty(n, dtype=torch.float32, device="cuda")
    net.forward(d_f.data_ptr(), n, d_y.data_ptr())
    torch.cuda.synchronize()
    y = d_y.cpu().numpy().astype(np.float64)
    v = d_b.cpu().numpy() + o["k"] * (y.astype(np.float32) / np.float32(y_scale)).astype(np.float64)
    intr = np.maximum(0.0, np.where(o["w"] < 0, o["k"] - o["s"], o["s"] - o["k"]))
    want = np.where(o["e"] != 0, np.maximum(v, intr), v)
    got = d_p.cpu().numpy()
    assert np.array_equal(d_in.cpu().numpy(), d_in2.cpu().numpy())
    assert np.max(np.abs(got - want) / o["k"]) <= 1e-12


def test_committed_weights_meet_the_error_target(ctx, built):
    """The shipped network (kwinto-cuda_gb300/surrogate_weights.npz, trained by
    train_surrogate.py on 2M FD64 prices at 1024 x 1024) on 8192 fresh options of the
    same distributions: p99 absolute error vs FD64 at 1024 x 1024 within 1e-3."""
    import os

    import torch

    import kwg
    import portfolio

    path = os.path.join(os.path.dirname(kwg.__file__), "surrogate_weights.npz")
    s = kwg.Surrogate(0)
    s.load(path)
    o = portfolio.american_portfolio(8192, seed=31337)
    fd = _fd_prices(ctx, o, t_dim=1024, x_dim=1024, scale=5.0, density=math.inf)
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_p = torch.empty(len(o), dtype=torch.float64, device="cuda")
    d_in = torch.empty(len(o), dtype=torch.uint8, device="cuda")
    s.price_device(d_o.data_ptr(), len(o), d_p.data_ptr(), d_in.data_ptr())
    torch.cuda.synchronize()
    s.close()
    assert d_in.cpu().numpy().all()
    err = np.abs(d_p.cpu().numpy() - fd)
    assert np.quantile(err, 0.99) <= 1e-3, np.quantile(err, 0.99)
