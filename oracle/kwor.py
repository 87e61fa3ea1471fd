"""ctypes wrappers of the two CPU oracles.  TEST INFRASTRUCTURE ONLY.

  oracle/libkwor.so        C restatement of the reference FD1D pricer (fd1d_oracle.c)
  oracle/_ref/libkwref.so  the reference's own sources + ref_harness.cpp (built only
                           where the reference sources are present)

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the product path never does.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(_HERE, "libkwor.so")
REF_SO = os.path.join(_HERE, "_ref", "libkwref.so")

OK, OUT_OF_GRID, SOLVER_ERROR, BAD_INPUT = 0, 1, 2, 3

# kw::Option layout (src/Core/kwAsset.h:12-22): 6 f64, u8, i8, padded to 56 bytes.
# numpy operations such as concatenate drop the padding, so every entry point
# converts its input to this exact layout before handing the buffer to C.
OPTION_DTYPE = np.dtype({"names": ["t", "k", "z", "r", "q", "s", "e", "w"],
                         "formats": ["<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "u1", "i1"],
                         "offsets": [0, 8, 16, 24, 32, 40, 48, 49], "itemsize": 56})


def _as_options(opts):
    return np.ascontiguousarray(np.asarray(opts).astype(OPTION_DTYPE, copy=False))


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("density", ctypes.c_double),
        ("scale", ctypes.c_double),
        ("theta", ctypes.c_double),
        ("t_dim", ctypes.c_int64),
        ("x_dim", ctypes.c_int64),
        ("uniform", ctypes.c_int32),
        ("const_dt", ctypes.c_int32),
    ]


_oracle = None
_ref = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            raise RuntimeError(f"{ORACLE_SO} missing: run `make -C oracle`")
        L = ctypes.CDLL(ORACLE_SO)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.kwor_fd1d_price.argtypes = [vp, sz, ctypes.POINTER(OracleParams), ctypes.c_int, vp, vp,
                                      ctypes.c_char_p, sz]
        L.kwor_fd1d_price.restype = ctypes.c_int
        L.kwor_fd1d_bs_price.argtypes = L.kwor_fd1d_price.argtypes
        L.kwor_fd1d_bs_price.restype = ctypes.c_int
        L.kwor_bs_price.argtypes = [vp, sz, vp]
        L.kwor_bs_price.restype = None
        L.kwor_fd1d_solve_grid.argtypes = [vp, ctypes.POINTER(OracleParams), vp, vp]
        L.kwor_fd1d_solve_grid.restype = ctypes.c_int
        L.kwor_dedup.argtypes = [vp, sz, vp, vp]
        L.kwor_dedup.restype = sz
        _oracle = L
    return _oracle


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError(f"{REF_SO} missing: run `make -C oracle ref` where the reference sources exist")
        L = ctypes.CDLL(REF_SO)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.kwref_price.argtypes = [ctypes.c_char_p, vp, sz, ctypes.c_double, ctypes.c_double, ctypes.c_long,
                                  ctypes.c_long, vp, ctypes.c_char_p, sz, vp]
        L.kwref_price.restype = ctypes.c_int
        L.kwref_pool_size.argtypes = []
        L.kwref_pool_size.restype = ctypes.c_int
        _ref = L
    return _ref


def make_params(t_dim=512, x_dim=512, scale=50.0, density=0.25, theta=0.5, const_dt=False) -> OracleParams:
    p = OracleParams()
    p.uniform = 1 if math.isinf(density) else 0
    p.density = 1.0 if p.uniform else density
    p.scale, p.theta, p.t_dim, p.x_dim, p.const_dt = scale, theta, t_dim, x_dim, int(const_dt)
    return p


def fd1d_price(opts: np.ndarray, nthreads: int = 0, bs: bool = False, **kw):
    """Oracle prices: returns (rc, message, prices, status)."""
    L = oracle_lib()
    p = make_params(**kw)
    n = len(opts)
    opts = _as_options(opts)
    prices = np.zeros(n)
    status = np.zeros(n, np.int32)
    err = ctypes.create_string_buffer(512)
    fn = L.kwor_fd1d_bs_price if bs else L.kwor_fd1d_price
    rc = fn(opts.ctypes.data, n, ctypes.byref(p), nthreads or os.cpu_count() or 1, prices.ctypes.data,
            status.ctypes.data, err, 512)
    return rc, err.value.decode(), prices, status


def dedup(opts: np.ndarray):
    """kwor_dedup (src/Pricer/kwFd1d.cpp:28-65): (asset2pde, pde2asset), PDEs in key order."""
    o = _as_options(opts)
    n = len(o)
    a2p = np.zeros(n, np.uint32)
    p2a = np.zeros(n, np.uint32)
    m = oracle_lib().kwor_dedup(o.ctypes.data, n, a2p.ctypes.data, p2a.ctypes.data) if n else 0
    return a2p, p2a[:m].copy()


def bs_price(opts: np.ndarray) -> np.ndarray:
    opts = _as_options(opts)
    out = np.zeros(len(opts))
    oracle_lib().kwor_bs_price(opts.ctypes.data, len(opts), out.ctypes.data)
    return out


def solve_grid(opt: np.ndarray, **kw):
    """One PDE: returns (rc, x-grid, final V)."""
    p = make_params(**kw)
    x = np.zeros(p.x_dim)
    v = np.zeros(p.x_dim)
    one = _as_options(np.asarray(opt).reshape(1))
    rc = oracle_lib().kwor_fd1d_solve_grid(one.ctypes.data, ctypes.byref(p), x.ctypes.data, v.ctypes.data)
    return rc, x, v


def ref_price(opts: np.ndarray, pricer: str = "FD1D", density=-1.0, scale=-1.0, t_dim=-1, x_dim=-1):
    """The reference itself: returns (rc, message, prices, seconds).  Negative
    arguments leave the key unset (reference default)."""
    L = ref_lib()
    n = len(opts)
    opts = _as_options(opts)
    prices = np.full(n, np.nan)
    err = ctypes.create_string_buffer(1024)
    secs = ctypes.c_double(0)
    rc = L.kwref_price(pricer.encode(), opts.ctypes.data, n, density, scale, t_dim, x_dim, prices.ctypes.data,
                       err, 1024, ctypes.byref(secs))
    return rc, err.value.decode(), prices, secs.value
