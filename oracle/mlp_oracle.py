"""CPU oracle of the MLP surrogate.  TEST INFRASTRUCTURE ONLY.

FP64 NumPy forward and backward of the network the GPU runs (5 -> 128 -> 128 -> 128
-> 128 -> 1, SiLU, MSE loss), rounding to BF16 exactly where the GPU does:
  * weights are BF16;
  * the input of layers 1-4 is the BF16 pair hi = bf16(a), lo = bf16(a - hi), so the
    layer sees hi + lo (the GPU stores [W | W] and doubles K);
  * the output layer is an FP32 dot product of the unrounded layer-4 activations;
  * the backward uses hi activations for the weight gradients, and BF16 dy / dZ as
    the operands of its GEMMs; bias gradients are unrounded sums.
Accumulation is FP64 here and FP32 on the tensor cores, so results agree to
FP32/BF16 rounding, not bit for bit.  Parameter layout: 5 weight matrices [out][in]
of 128 x 128, then 5 biases of 128.
"""
from __future__ import annotations

import numpy as np

W = 128
LAYERS = 5
N_WEIGHTS = LAYERS * W * W


def bf16(x) -> np.ndarray:
    """Round to BF16 (nearest-even) and back to float64."""
    f = np.asarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, np.float64)
    ws = [p[l * W * W:(l + 1) * W * W].reshape(W, W) for l in range(LAYERS)]
    bs = [p[N_WEIGHTS + l * W:N_WEIGHTS + (l + 1) * W] for l in range(LAYERS)]
    return ws, bs


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _identity(x):
    return np.asarray(x, np.float64)


def split(a):
    """hi + lo of the BF16 pair the GPU feeds the tensor cores."""
    hi = bf16(a)
    return hi + bf16(np.asarray(a, np.float64) - hi)


def forward(params, x, exact=False):
    """x: [n][128] inputs (features in columns 0..4).  Returns (y [n], cache).
    exact=True skips every rounding (the plain FP64 network, for finite differences)."""
    rnd = _identity if exact else bf16
    pair = _identity if exact else split
    ws, bs = unpack(params)
    a = np.asarray(x, np.float64)
    acts, zs = [a], []
    for l in range(4):
        z = pair(a) @ rnd(ws[l]).T + bs[l]
        zs.append(z)
        a = silu(z)
        acts.append(a)
    y = a @ rnd(ws[4][0]) + bs[4][0]
    return y, (acts, zs)


NO_FLOOR = 1e30


def residual(y, t, floor=None):
    """e = y - t, or max(0, y - floor) on early-exercise rows (floor > -NO_FLOOR)."""
    if floor is None:
        return y - t
    f = np.asarray(floor, np.float64)
    return np.where(f > -NO_FLOOR, np.maximum(0.0, y - f), y - t)


def loss(params, x, t, exact=False, floor=None):
    y, _ = forward(params, x, exact)
    return float(np.mean(residual(y, t, floor) ** 2))


def gradients(params, x, t, exact=False, floor=None):
    """Loss mean(e^2) (e from residual()) and the gradient of every parameter (flat, FP64)."""
    rnd = _identity if exact else bf16
    ws, bs = unpack(params)
    n = len(t)
    y, (acts, zs) = forward(params, x, exact)
    e = residual(y, t, floor)
    mse = float(np.mean(e * e))
    dy = 2.0 * e / n
    g = np.zeros(N_WEIGHTS + LAYERS * W)
    dY = np.zeros((n, W))
    dY[:, 0] = rnd(dy)
    gw = [None] * LAYERS
    gb = [None] * LAYERS
    gw[4] = dY.T @ rnd(acts[4])
    gb[4] = np.zeros(W)
    gb[4][0] = dy.sum()
    da = dY @ rnd(ws[4])
    for l in range(3, -1, -1):
        dz = da * dsilu(zs[l])
        gb[l] = dz.sum(0)
        dzb = rnd(dz)
        gw[l] = dzb.T @ rnd(acts[l])
        if l > 0:
            da = dzb @ rnd(ws[l])
    for l in range(LAYERS):
        g[l * W * W:(l + 1) * W * W] = gw[l].ravel()
        g[N_WEIGHTS + l * W:N_WEIGHTS + (l + 1) * W] = gb[l]
    return mse, g

BOX_LO = np.array([-0.25, 0.04, 0.0, 0.0, -1.0])
BOX_HI = np.array([0.20, 0.86, 0.2, 0.2, 1.0])


def features(opts, box_lo=BOX_LO, box_hi=BOX_HI):
    """Options -> (normalised features [n][5], in-box flags): log(K/S), vol sqrt(T),
    r T, q T and put/call (-1/+1), each mapped from [lo, hi] to [-1, 1].  Only
    American options (e != 0) count as in the box."""
    raw = np.stack([np.log(opts["k"] / opts["s"]), opts["z"] * np.sqrt(opts["t"]), opts["r"] * opts["t"],
                    opts["q"] * opts["t"], np.where(opts["w"] < 0, -1.0, 1.0)], axis=1)
    inside = (opts["e"] != 0) & np.all((raw >= box_lo) & (raw <= box_hi), axis=1)
    return 2.0 * (raw - box_lo) / (box_hi - box_lo) - 1.0, inside


def random_params(seed):
    """He-uniform weights on the active entries and small random biases (FP32
    values as float64), for the parity tests."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_WEIGHTS + LAYERS * W)
    for l in range(LAYERS):
        fan_in = W if l else 5
        outs = 1 if l == LAYERS - 1 else W
        w = np.zeros((W, W))
        w[:outs, :fan_in] = rng.uniform(-1, 1, (outs, fan_in)) * np.sqrt(6.0 / fan_in)
        p[l * W * W:(l + 1) * W * W] = w.ravel()
        p[N_WEIGHTS + l * W:N_WEIGHTS + l * W + outs] = rng.uniform(-0.1, 0.1, outs)
    return p.astype(np.float32).astype(np.float64)


def european(opts):
    """Black-Scholes European price of each contract (exercise flag ignored)."""
    from scipy.special import ndtr

    S, K, T, z, r, q = (np.asarray(opts[f], np.float64) for f in ("s", "k", "t", "z", "r", "q"))
    w = np.where(opts["w"] < 0, -1.0, 1.0)
    zt = z * np.sqrt(T)
    d1 = (np.log(S / K) + (r - q + 0.5 * z * z) * T) / zt
    return w * (S * ndtr(w * d1) * np.exp(-q * T) - K * ndtr(w * (d1 - zt)) * np.exp(-r * T))


def baw(opts):
    """Barone-Adesi & Whaley (1987) American price with dividend yield q: the
    quadratic approximation E(S) + A (S / S_c)^qe on the continuation side of the
    critical price S_c and the intrinsic value beyond it (E the European price).
    S_c is the root of w (S - K) - E(S) - w (1 - e^{-qT} N(w d1(S))) S / qe, found here
    by bisection in log S over [log K - 60, log K] (puts) / [log K, log K + 60]
    (calls); no sign change there, puts with r <= 0 and calls with q <= 0 price as
    European.  European contracts (e == 0) get the European price."""
    from scipy.special import ndtr

    S, K, T, z, r, q = (np.asarray(opts[f], np.float64) for f in ("s", "k", "t", "z", "r", "q"))
    w = np.where(opts["w"] < 0, -1.0, 1.0)
    eu = european(opts)
    s2, zt = z * z, z * np.sqrt(T)
    nn = 2 * (r - q) / s2
    with np.errstate(divide="ignore", invalid="ignore"):
        mk = np.where(r * T < 1e-12, 2 / (s2 * T), 2 * r / (s2 * -np.expm1(-r * T)))
    qe = 0.5 * (-(nn - 1) + w * np.sqrt((nn - 1) ** 2 + 4 * mk))
    dq, dr, lk = np.exp(-q * T), np.exp(-r * T), np.log(K)
    mu = (r - q + 0.5 * s2) * T

    def g(u):
        s = np.exp(u)
        d1 = (u - lk + mu) / zt
        nd1 = ndtr(w * d1)
        e = w * (s * dq * nd1 - K * dr * ndtr(w * (d1 - zt)))
        return w * (s - K) - e - w * (1 - dq * nd1) * s / qe

    lo = np.where(w < 0, lk - 60, lk)
    hi = np.where(w < 0, lk, lk + 60)
    has_root = g(np.where(w < 0, lo, hi)) > 0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        ex_side = (g(mid) > 0) == (w < 0)  # put: g > 0 below S_c
        lo = np.where(ex_side, mid, lo)
        hi = np.where(ex_side, hi, mid)
    u = 0.5 * (lo + hi)
    sc = np.exp(u)
    d1c = (u - lk + mu) / zt
    a = w * (sc / qe) * (1 - dq * ndtr(w * d1c))
    cont = np.where(w < 0, S > sc, S < sc)
    with np.errstate(over="ignore", invalid="ignore"):
        v = np.where(cont, eu + a * np.exp(qe * np.log(S / sc)), w * (S - K))
    never = np.where(w < 0, ~(r > 0), ~(q > 0)) | ~has_root | (opts["e"] == 0)
    return np.where(never, eu, np.maximum(v, eu))
