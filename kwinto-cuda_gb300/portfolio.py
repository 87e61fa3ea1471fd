"""Seeded synthetic portfolios for the FD1D workloads, and the reference's CSV format.

Random numbers: counter-based splitmix64.  Field f of option i takes the 64-bit
output of splitmix64's finaliser applied to  seed*2^40 + f*2^32 + i + 1  times the
golden-ratio increment, and the top 53 bits give a uniform double in [0, 1).  The
same function is used by tests, the benchmark and the oracle runs, so every
workload is reproducible from (workload, seed, n).

Workloads (the shapes the reference logs use, log/*_1024_32768.log):
  american_128x512     128 American options, half puts half calls, S=100,
                       K~U[80,120], vol~U[0.1,0.6], r~U[0,0.1], q~U[0,0.1],
                       T~U[0.25,2]; 512x512 grid, scale 5, density 0.25 (the
                       reference default)
  american_32768x1024  the same distributions, 32768 options, 1024x1024, uniform grid
  american_65536x2048  the same distributions, 65536 options, 2048x2048
  uneven_portfolio     131072 options: T log-uniform [1/52, 5], K/S lognormal(0, 0.2),
                       vol~U[0.05,0.8], r,q~U[0,0.08]; per-option x_dim by vol*sqrt(T)
                       bucket, t_dim = clamp(ceil(512 sqrt(T)), 64, 2048)
"""
from __future__ import annotations

import math

import numpy as np

from kwg import OPTION_DTYPE

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def uniforms(seed: int, field: int, n: int, start: int = 0) -> np.ndarray:
    """n uniform doubles in [0,1) for (seed, field), options start..start+n-1."""
    with np.errstate(over="ignore"):
        ctr = (np.uint64(seed) << np.uint64(40)) + (np.uint64(field) << np.uint64(32)) + \
            np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = ctr * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _normals(seed: int, field: int, n: int, start: int = 0) -> np.ndarray:
    u1 = uniforms(seed, field, n, start)
    u2 = uniforms(seed, field + 1, n, start)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


def american_portfolio(n: int, seed: int = 42, start: int = 0) -> np.ndarray:
    """American options: S=100, K~U[80,120], vol~U[0.1,0.6], r,q~U[0,0.1],
    T~U[0.25,2]; puts on even indices, calls on odd ones."""
    o = np.zeros(n, OPTION_DTYPE)
    o["s"] = 100.0
    o["k"] = 80.0 + 40.0 * uniforms(seed, 0, n, start)
    o["z"] = 0.1 + 0.5 * uniforms(seed, 1, n, start)
    o["r"] = 0.1 * uniforms(seed, 2, n, start)
    o["q"] = 0.1 * uniforms(seed, 3, n, start)
    o["t"] = 0.25 + 1.75 * uniforms(seed, 4, n, start)
    o["e"] = 1
    idx = np.arange(start, start + n)
    o["w"] = np.where(idx % 2 == 0, -1, 1).astype(np.int8)
    return o


WORKLOADS = {
    "american_128x512": dict(n=128, x_dim=512, t_dim=512, scale=5.0, density=0.25),
    "american_32768x1024": dict(n=32768, x_dim=1024, t_dim=1024, scale=5.0, density=math.inf),
    "american_65536x2048": dict(n=65536, x_dim=2048, t_dim=2048, scale=5.0, density=0.25),
}

# The reference has no uniform-grid mode; its closest setting is a large density.
# At d = 1e6 its grid differs from the exactly uniform one by ~1e-12 relative.
REFERENCE_UNIFORM_DENSITY = 1e6


def uneven_portfolio(n: int = 131072, seed: int = 42, start: int = 0):
    """Uneven batch.  Returns (options, x_dim[n], t_dim[n])."""
    o = np.zeros(n, OPTION_DTYPE)
    o["s"] = 100.0
    lo, hi = math.log(1.0 / 52.0), math.log(5.0)
    o["t"] = np.exp(lo + (hi - lo) * uniforms(seed, 10, n, start))
    o["k"] = 100.0 * np.exp(0.2 * _normals(seed, 11, n, start))
    o["z"] = 0.05 + 0.75 * uniforms(seed, 13, n, start)
    o["r"] = 0.08 * uniforms(seed, 14, n, start)
    o["q"] = 0.08 * uniforms(seed, 15, n, start)
    o["e"] = 1
    o["w"] = np.where(uniforms(seed, 16, n, start) < 0.5, -1, 1).astype(np.int8)
    zs = o["z"] * np.sqrt(o["t"])
    x_dim = np.select([zs < 0.1, zs < 0.2, zs < 0.4, zs < 0.8], [128, 256, 512, 1024], 2048).astype(np.int32)
    t_dim = np.clip(np.ceil(512.0 * np.sqrt(o["t"])), 64, 2048).astype(np.int32)
    return o, x_dim, t_dim


# ----------------------------------------------------------------------------- CSV (src/Utils/kwPortfolio.cpp)

_CSV_COLS = ("exercise", "strike", "dividend_rate", "interest_rate", "spot", "expiry", "price", "parity",
             "volatility")


def load_csv(path_or_text: str, is_text: bool = False):
    """Portfolio::load (src/Utils/kwPortfolio.cpp:13-84): named columns, e=="a" is
    American, w=="c" is a call.  Returns (options, prices) or raises ValueError with
    the reference's message when a column is missing."""
    text = path_or_text if is_text else open(path_or_text).read()
    lines = text.splitlines()
    header = lines[0].split(",")
    col = {name: header.index(name) if name in header else -1 for name in _CSV_COLS}
    if any(v == -1 for v in col.values()):
        e, k, q, r, s, t, v, w, z = (col[c] for c in ("exercise", "strike", "dividend_rate", "interest_rate",
                                                       "spot", "expiry", "price", "parity", "volatility"))
        raise ValueError(f"Portfolio::load : Some option data is missing: e={e}, k={k}, q={q}, r={r}, s={s}, "
                         f"t={t}, v={v}, w={w}, z={z}")
    rows = [ln.split(",") for ln in lines[1:] if ln]
    o = np.zeros(len(rows), OPTION_DTYPE)
    prices = np.zeros(len(rows))
    for i, vals in enumerate(rows):
        o[i] = (float(vals[col["expiry"]]), float(vals[col["strike"]]), float(vals[col["volatility"]]),
                float(vals[col["interest_rate"]]), float(vals[col["dividend_rate"]]), float(vals[col["spot"]]),
                1 if vals[col["exercise"]] == "a" else 0, 1 if vals[col["parity"]] == "c" else -1)
        prices[i] = float(vals[col["price"]])
    return o, prices


def price_stats(assets: np.ndarray, want: np.ndarray, got: np.ndarray, tolerance: float = 0.5) -> dict:
    """Portfolio::printPricesStats (src/Utils/kwPortfolio.cpp:101-163).  Options whose
    reference price is below `tolerance` are skipped; "rmse" is, as in the reference,
    the standard deviation of |error| (sqrt(E[d^2] - E[d]^2)), not the RMS."""
    keep = ~(want < tolerance)
    w, g = want[keep], got[keep]
    ad = np.abs(w - g)
    rd = ad / w
    out = dict(total=int(keep.sum()))
    if out["total"] == 0:
        return out
    out["rmse"] = float(np.sqrt(np.mean(ad * ad) - np.mean(ad) ** 2))
    out["rrmse"] = float(np.sqrt(np.mean(rd * rd) - np.mean(rd) ** 2))
    out["mae"] = float(ad.max())
    out["mre"] = float(rd.max())
    idx = np.flatnonzero(keep)
    out["mae_index"] = int(idx[int(np.argmax(ad))])
    out["mre_index"] = int(idx[int(np.argmax(rd))])
    return out
