"""The MLP oracle (test infrastructure for the surrogate's GPU kernels): its
backward pass against central finite differences of its own FP64 forward."""
import numpy as np

import mlp_oracle as mo


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    p = mo.random_params(3)
    x = np.zeros((24, mo.W))
    x[:, :5] = rng.uniform(-1, 1, (24, 5))
    t = rng.normal(size=24)
    _, g = mo.gradients(p, x, t, exact=True)
    idx = [0, 3, 130, mo.W * mo.W + 17 * mo.W + 5, 2 * mo.W * mo.W + 99, 3 * mo.W * mo.W + 127 * mo.W + 64,
           4 * mo.W * mo.W + 7, mo.N_WEIGHTS + 5, mo.N_WEIGHTS + 2 * mo.W + 40, mo.N_WEIGHTS + 4 * mo.W]
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss(pp, x, t, exact=True) - mo.loss(pm, x, t, exact=True)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_floor_gradients_match_finite_differences():
    """The one-sided early-exercise loss: rows with a floor only penalise y above it."""
    rng = np.random.default_rng(4)
    p = mo.random_params(4)
    x = np.zeros((30, mo.W))
    x[:, :5] = rng.uniform(-1, 1, (30, 5))
    t = rng.normal(size=30)
    y, _ = mo.forward(p, x, exact=True)
    fl = np.full(30, -mo.NO_FLOOR)
    fl[::3] = y[::3] - 0.3   # active: y above the floor
    fl[1::6] = y[1::6] + 0.3  # inactive: y below the floor, zero residual
    _, g = mo.gradients(p, x, t, exact=True, floor=fl)
    h = 1e-6
    for i in [1, 200, mo.W * mo.W + 300, 4 * mo.W * mo.W + 3, mo.N_WEIGHTS + mo.W + 9, mo.N_WEIGHTS + 4 * mo.W]:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss(pp, x, t, True, fl) - mo.loss(pm, x, t, True, fl)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
    assert np.all(mo.residual(y, t, fl)[1::6] == 0.0)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 0.0, 65504.0])
    r = mo.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even
    assert r[2] == 1.0 + 2 ** -7        # above the midpoint: rounds up
    assert abs(r[3] + 3.140625) == 0.0
    assert r[4] == 0.0 and r[5] == 65536.0


def test_rounded_gradients_close_to_exact():
    """The BF16 roundings perturb the gradient by BF16-relative amounts only."""
    rng = np.random.default_rng(5)
    p = mo.random_params(5)
    x = np.zeros((64, mo.W))
    x[:, :5] = rng.uniform(-1, 1, (64, 5))
    t = rng.normal(size=64)
    _, g0 = mo.gradients(p, x, t, exact=True)
    _, g1 = mo.gradients(p, x, t)
    assert np.linalg.norm(g1 - g0) <= 0.03 * np.linalg.norm(g0)


def _opts(**fields):
    import kwg

    n = max(np.size(v) for v in fields.values())
    o = np.zeros(n, kwg.OPTION_DTYPE)
    for k, v in fields.items():
        o[k] = v
    return o


def test_baw_published_calls():
    """Barone-Adesi & Whaley (1987), American calls, K = 100, T = 0.25, r = 0.08,
    cost of carry b = -0.04 (q = 0.12), sigma = 0.2: 0.03, 0.59, 3.52, 10.31, 20.00
    at S = 80, 90, 100, 110, 120 (two decimals as published)."""
    o = _opts(s=[80.0, 90.0, 100.0, 110.0, 120.0], k=100.0, t=0.25, r=0.08, q=0.12, z=0.2, w=1, e=1)
    assert np.array_equal(np.round(mo.baw(o), 2), [0.03, 0.59, 3.52, 10.31, 20.00])


def test_baw_bounds_and_limits():
    import portfolio

    o = portfolio.american_portfolio(4000, seed=9)
    b, e = mo.baw(o), mo.european(o)
    intr = np.maximum(0, np.where(o["w"] < 0, o["k"] - o["s"], o["s"] - o["k"]))
    assert np.all(b >= e) and np.all(b >= intr - 1e-12 * o["k"])
    # no early exercise: puts with r = 0, calls with q = 0, European contracts
    o2 = o.copy()
    o2["r"][o2["w"] < 0] = 0.0
    o2["q"][o2["w"] > 0] = 0.0
    assert np.array_equal(mo.baw(o2), mo.european(o2))
    o3 = o.copy()
    o3["e"] = 0
    assert np.array_equal(mo.baw(o3), mo.european(o3))
