"""kwg -- Python host mirror of the reference's pricer interface over libkwg.so.

The reference (gituliar/kwinto-cuda) exposes pricing as C++:

    kw::Config                    typed string->value map     src/Core/kwConfig.h:21-73
    kw::Pricer::init / price      abstract pricer             src/Pricer/kwPricer.h:12-22
    kw::PricerFactory::create     keyed on PRICER             src/Pricer/kwPricerFactory.h:15-41
    kw::Fd1d_Pricer               FD1D.* keys                 src/Pricer/kwFd1d.cpp:9-19

This module mirrors those names, argument meanings and error behaviour (an error
is a non-empty string; "" means success) on top of the C ABI in include/kwg.h.
The GPU library must be built (``__graft_entry__.build()``); importing this module
without it raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkwg.so")

# kw::Option layout (src/Core/kwAsset.h:12-22): t k z r q s (f64), e (u8), w (i8); 56 bytes.
OPTION_DTYPE = np.dtype(
    {
        "names": ["t", "k", "z", "r", "q", "s", "e", "w"],
        "formats": ["<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "u1", "i1"],
        "offsets": [0, 8, 16, 24, 32, 40, 48, 49],
        "itemsize": 56,
    }
)

KWG_OK, KWG_ERR_INVALID, KWG_ERR_CUDA, KWG_ERR_OUT_OF_GRID, KWG_ERR_SOLVER = 0, 1, 2, 3, 4
STATUS_OK, STATUS_OUT_OF_GRID, STATUS_SOLVER, STATUS_BAD_INPUT = 0, 1, 2, 3
FP64, FP32 = 0, 1
SOLVER_AUTO, SOLVER_THOMAS, SOLVER_PCR = 0, 1, 2


class Fd1dParams(ctypes.Structure):
    """struct kwg_fd1d_params (include/kwg.h)."""

    _fields_ = [
        ("t_dim", ctypes.c_int32),
        ("x_dim", ctypes.c_int32),
        ("theta", ctypes.c_double),
        ("scale", ctypes.c_double),
        ("density", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("solver", ctypes.c_int32),
        ("strict", ctypes.c_int32),
        ("device_dedup", ctypes.c_int32),
        ("block_warps", ctypes.c_int32),
        ("option_warps", ctypes.c_int32),
        ("sm_blocks", ctypes.c_int32),
    ]


class Audit(ctypes.Structure):
    """struct kwg_audit (include/kwg.h)."""

    _fields_ = [
        ("audited", ctypes.c_int64),
        ("out_of_box", ctypes.c_int64),
        ("audit_abs_max", ctypes.c_double),
        ("audit_abs_sum", ctypes.c_double),
    ]


MLP_WIDTH, MLP_LAYERS, MLP_IN = 128, 5, 5
MLP_PARAMS = MLP_LAYERS * MLP_WIDTH * MLP_WIDTH + MLP_LAYERS * MLP_WIDTH
ROUTE_NETWORK, ROUTE_AUDIT, ROUTE_OUT_OF_BOX, ROUTE_FD_FAILED = 0, 1, 2, 3

class Tuning(ctypes.Structure):
    """struct kwg_tuning (include/kwg.h)."""

    _fields_ = [
        ("solver", ctypes.c_int32),
        ("block_warps", ctypes.c_int32),
        ("option_warps", ctypes.c_int32),
        ("sm_blocks", ctypes.c_int32),
        ("thomas_ms", ctypes.c_double * 3),
        ("pcr_ms", ctypes.c_double),
        ("fp32_ms", ctypes.c_double * 3),
        ("spread_ms", ctypes.c_double),
        ("fp32_8w_ms", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {"solver": {SOLVER_THOMAS: "thomas", SOLVER_PCR: "pcr"}.get(self.solver, self.solver),
                "block_warps": self.block_warps, "option_warps": self.option_warps, "sm_blocks": self.sm_blocks,
                "thomas_ms_by_block_warps": {1: self.thomas_ms[0], 2: self.thomas_ms[1], 4: self.thomas_ms[2]},
                "thomas_ms_one_4warp_block_per_sm": self.spread_ms,
                "pcr_ms": self.pcr_ms,
                "fp32_ms_by_option_warps": {1: self.fp32_ms[0], 2: self.fp32_ms[1], 4: self.fp32_ms[2],
                                            8: self.fp32_8w_ms}}


_lib = None


def lib() -> ctypes.CDLL:
    """Loads libkwg.so once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"kwg: {LIB_PATH} is missing; run __graft_entry__.build() first")
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, i32, dp = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p
    L.kwg_fd1d_params_default.argtypes = [ctypes.POINTER(Fd1dParams)]
    L.kwg_fd1d_params_default.restype = None
    L.kwg_fd1d_dedup.argtypes = [vp, vp, vp, sz, vp, vp]
    L.kwg_fd1d_dedup.restype = sz
    L.kwg_create.argtypes = [i32]
    L.kwg_create.restype = vp
    L.kwg_destroy.argtypes = [vp]
    L.kwg_destroy.restype = None
    L.kwg_last_error.argtypes = [vp]
    L.kwg_last_error.restype = ctypes.c_char_p
    L.kwg_last_launch_count.argtypes = [vp]
    L.kwg_last_launch_count.restype = i32
    L.kwg_fd1d_price.argtypes = [vp, vp, sz, ctypes.POINTER(Fd1dParams), dp, dp]
    L.kwg_fd1d_price.restype = i32
    L.kwg_fd1d_bs_price.argtypes = [vp, vp, sz, ctypes.POINTER(Fd1dParams), dp, dp]
    L.kwg_fd1d_bs_price.restype = i32
    L.kwg_fd1d_price_device.argtypes = [vp, vp, sz, ctypes.POINTER(Fd1dParams), dp, dp, vp]
    L.kwg_fd1d_price_device.restype = i32
    L.kwg_fd1d_price_uneven.argtypes = [vp, vp, vp, vp, sz, ctypes.POINTER(Fd1dParams), dp, dp]
    L.kwg_fd1d_price_uneven.restype = i32
    L.kwg_autotune_ex.argtypes = [vp, ctypes.POINTER(Fd1dParams), sz, ctypes.POINTER(Tuning)]
    L.kwg_autotune_ex.restype = i32
    L.kwg_autotune_uneven.argtypes = [vp, vp, vp, vp, sz, ctypes.POINTER(Fd1dParams), ctypes.POINTER(Tuning)]
    L.kwg_autotune_uneven.restype = i32
    L.kwg_selftest_waits.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
    L.kwg_selftest_waits.restype = i32
    L.kwg_autotune.argtypes = [vp, ctypes.POINTER(Fd1dParams), sz, ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double)]
    L.kwg_autotune.restype = i32
    L.kwg_gemm_bf16.argtypes = [vp, vp, vp, i32, i32, i32, vp]
    L.kwg_gemm_bf16.restype = i32
    L.kwg_set_profiling.argtypes = [vp, i32]
    L.kwg_set_profiling.restype = i32
    L.kwg_profile_read.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_double)]
    L.kwg_profile_read.restype = i32
    u64, f32, dbl = ctypes.c_uint64, ctypes.c_float, ctypes.c_double
    L.kwg_mlp_create.argtypes = [i32, u64]
    L.kwg_mlp_create.restype = vp
    L.kwg_mlp_destroy.argtypes = [vp]
    L.kwg_mlp_destroy.restype = None
    L.kwg_mlp_last_error.argtypes = [vp]
    L.kwg_mlp_last_error.restype = ctypes.c_char_p
    L.kwg_mlp_set_params.argtypes = [vp, vp, vp, vp, f32]
    L.kwg_mlp_get_params.argtypes = [vp, vp, vp, vp, ctypes.POINTER(f32)]
    L.kwg_mlp_forward.argtypes = [vp, vp, i32, vp]
    L.kwg_mlp_gradients.argtypes = [vp, vp, vp, vp, i32, vp, ctypes.POINTER(dbl)]
    L.kwg_mlp_featurize.argtypes = [vp, vp, i32, vp, vp, vp]
    L.kwg_mlp_train.argtypes = [vp, vp, vp, i32, i32, i32, f32, u64, ctypes.POINTER(dbl)]
    L.kwg_mlp_price_device.argtypes = [vp, vp, i32, vp, vp]
    L.kwg_mlp_train_history.argtypes = [vp, vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.kwg_mlp_train_history.restype = i32
    L.kwg_surrogate_price.argtypes = [vp, vp, vp, sz, ctypes.POINTER(Fd1dParams), dbl, u64, dp, dp,
                                      ctypes.POINTER(Audit)]
    for name in ("set_params", "get_params", "forward", "gradients", "featurize", "train", "price_device"):
        getattr(L, "kwg_mlp_" + name).restype = i32
    L.kwg_surrogate_price.restype = i32
    _lib = L
    return L


def dedup(opts, x_dims=None, t_dims=None) -> tuple[np.ndarray, np.ndarray]:
    """The PDE grouping every pricing call uses (kwg_fd1d_dedup; the reference's key,
    src/Pricer/kwFd1d.cpp:28-65, plus the grid shape when x_dims/t_dims are given):
    (asset2pde, pde2asset).  Host only."""
    o = np.ascontiguousarray(opts, dtype=OPTION_DTYPE)
    n = len(o)
    a2p = np.zeros(n, np.int32)
    p2a = np.zeros(n, np.uint32)
    if n == 0:
        return a2p, p2a
    xp = tp = None
    if x_dims is not None and t_dims is not None:
        xd = np.ascontiguousarray(x_dims, np.int32)
        td = np.ascontiguousarray(t_dims, np.int32)
        if xd.shape != (n,) or td.shape != (n,):
            raise ValueError("dedup: x_dims and t_dims need one entry per option")
        xp, tp = xd.ctypes.data, td.ctypes.data
    m = lib().kwg_fd1d_dedup(o.ctypes.data, xp, tp, n, a2p.ctypes.data, p2a.ctypes.data)
    return a2p, p2a[:m].copy()


def default_params() -> Fd1dParams:
    p = Fd1dParams()
    lib().kwg_fd1d_params_default(ctypes.byref(p))
    return p


class Context:
    """Owns a kwg_ctx (device buffers + stream) on one CUDA device."""

    def __init__(self, device: int = 0):
        self._L = lib()
        self.device = device
        self.ptr = self._L.kwg_create(device)
        if not self.ptr:
            raise RuntimeError(f"kwg_create({device}) failed: no usable CUDA device")

    def close(self):
        if self.ptr:
            self._L.kwg_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return self._L.kwg_last_error(self.ptr).decode()

    def launch_count(self) -> int:
        return self._L.kwg_last_launch_count(self.ptr)

    def set_profiling(self, on: bool):
        self._L.kwg_set_profiling(self.ptr, 1 if on else 0)

    def profile_read(self, with_bytes: bool = False):
        """(summed solve-kernel ms, launches[, bytes read+written]) since the last read."""
        ms, cnt, nb = ctypes.c_double(0), ctypes.c_int(0), ctypes.c_double(0)
        rc = self._L.kwg_profile_read(self.ptr, ctypes.byref(ms), ctypes.byref(cnt), ctypes.byref(nb))
        if rc:
            raise RuntimeError(self.last_error())
        return (ms.value, cnt.value, nb.value) if with_bytes else (ms.value, cnt.value)

    def selftest_waits(self):
        """(timed_out, completed) of the bounded-wait self-test; (1, 1) is correct."""
        a, b = ctypes.c_int32(-1), ctypes.c_int32(-1)
        rc = self._L.kwg_selftest_waits(self.ptr, ctypes.byref(a), ctypes.byref(b))
        if rc:
            raise RuntimeError(self.last_error())
        return a.value, b.value

    def autotune(self, params: Fd1dParams, m: int):
        """Times the FP64 solvers on a synthetic batch of m options; records the faster
        one for KWG_SOLVER_AUTO.  Returns (thomas_ms, pcr_ms); -1 if not applicable."""
        a, b = ctypes.c_double(0), ctypes.c_double(0)
        rc = self._L.kwg_autotune(self.ptr, ctypes.byref(params), m, ctypes.byref(a), ctypes.byref(b))
        if rc:
            raise RuntimeError(self.last_error())
        return a.value, b.value

    def autotune_ex(self, params: Fd1dParams, m: int) -> Tuning:
        """Times options-per-block and Thomas vs PCR (FP64) or threads-per-option (FP32) on
        a synthetic batch of m options of params' shape; records and returns the choice."""
        t = Tuning()
        if self._L.kwg_autotune_ex(self.ptr, ctypes.byref(params), m, ctypes.byref(t)):
            raise RuntimeError(self.last_error())
        return t

    def autotune_uneven(self, opts: np.ndarray, x_dims, t_dims, params: Fd1dParams) -> Tuning:
        """The same on an uneven batch; the choice applies to uneven calls of its size."""
        opts = np.ascontiguousarray(opts, dtype=OPTION_DTYPE)
        xd = np.ascontiguousarray(x_dims, dtype=np.int32)
        td = np.ascontiguousarray(t_dims, dtype=np.int32)
        t = Tuning()
        if self._L.kwg_autotune_uneven(self.ptr, opts.ctypes.data, xd.ctypes.data, td.ctypes.data, len(opts),
                                       ctypes.byref(params), ctypes.byref(t)):
            raise RuntimeError(self.last_error())
        return t

    def fd1d_price(self, opts: np.ndarray, params: Fd1dParams):
        """Host arrays in, host arrays out. Returns (rc, prices, status)."""
        opts = np.ascontiguousarray(opts, dtype=OPTION_DTYPE)
        n = len(opts)
        prices = np.empty(n, np.float64)
        status = np.empty(n, np.int32)
        rc = self._L.kwg_fd1d_price(
            self.ptr, opts.ctypes.data, n, ctypes.byref(params), prices.ctypes.data, status.ctypes.data
        )
        return rc, prices, status

    def fd1d_bs_price(self, opts: np.ndarray, params: Fd1dParams):
        """FD1D-BS control variate, host arrays.  Returns (rc, prices, status)."""
        opts = np.ascontiguousarray(opts, dtype=OPTION_DTYPE)
        n = len(opts)
        prices = np.empty(n, np.float64)
        status = np.empty(n, np.int32)
        rc = self._L.kwg_fd1d_bs_price(
            self.ptr, opts.ctypes.data, n, ctypes.byref(params), prices.ctypes.data, status.ctypes.data
        )
        return rc, prices, status

    def fd1d_price_uneven(self, opts: np.ndarray, x_dims, t_dims, params: Fd1dParams):
        """Per-option grids.  Returns (rc, prices, status)."""
        opts = np.ascontiguousarray(opts, dtype=OPTION_DTYPE)
        xd = np.ascontiguousarray(x_dims, dtype=np.int32)
        td = np.ascontiguousarray(t_dims, dtype=np.int32)
        n = len(opts)
        prices = np.empty(n, np.float64)
        status = np.empty(n, np.int32)
        rc = self._L.kwg_fd1d_price_uneven(self.ptr, opts.ctypes.data, xd.ctypes.data, td.ctypes.data, n,
                                           ctypes.byref(params), prices.ctypes.data, status.ctypes.data)
        return rc, prices, status

    def fd1d_price_device(self, d_opts: int, n: int, params: Fd1dParams, d_prices: int, d_status: int,
                          stream: int = 0) -> int:
        """Device pointers in and out (e.g. torch tensors' data_ptr()); asynchronous."""
        return self._L.kwg_fd1d_price_device(self.ptr, d_opts, n, ctypes.byref(params), d_prices, d_status,
                                             stream or None)


class Surrogate:
    """Owns a kwg_mlp: the MLP surrogate of the FD1D price (no reference counterpart)."""

    def __init__(self, device: int = 0, seed: int = 1):
        self._L = lib()
        self.ptr = self._L.kwg_mlp_create(device, seed)
        if not self.ptr:
            raise RuntimeError(f"kwg_mlp_create({device}) failed: no usable CUDA device")

    def close(self):
        if self.ptr:
            self._L.kwg_mlp_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return self._L.kwg_mlp_last_error(self.ptr).decode()

    def _check(self, rc: int):
        if rc:
            raise RuntimeError(f"kwg_mlp error {rc}: {self.last_error()}")

    def get_params(self):
        """(params float32[MLP_PARAMS], box_lo[5], box_hi[5], y_scale)."""
        p = np.empty(MLP_PARAMS, np.float32)
        lo, hi = np.empty(MLP_IN), np.empty(MLP_IN)
        ys = ctypes.c_float(0)
        self._check(self._L.kwg_mlp_get_params(self.ptr, p.ctypes.data, lo.ctypes.data, hi.ctypes.data,
                                               ctypes.byref(ys)))
        return p, lo, hi, ys.value

    def set_params(self, params, box_lo=None, box_hi=None, y_scale: float = 1.0):
        p = np.ascontiguousarray(params, np.float32)
        if p.size != MLP_PARAMS:
            raise ValueError(f"expected {MLP_PARAMS} parameters, got {p.size}")
        lo = None if box_lo is None else np.ascontiguousarray(box_lo, np.float64)
        hi = None if box_hi is None else np.ascontiguousarray(box_hi, np.float64)
        self._check(self._L.kwg_mlp_set_params(self.ptr, p.ctypes.data, None if lo is None else lo.ctypes.data,
                                               None if hi is None else hi.ctypes.data, y_scale))

    def save(self, path: str):
        p, lo, hi, ys = self.get_params()
        np.savez(path, params=p, box_lo=lo, box_hi=hi, y_scale=np.float32(ys))

    def load(self, path: str):
        z = np.load(path)
        self.set_params(z["params"], z["box_lo"], z["box_hi"], float(z["y_scale"]))

    def forward(self, d_x: int, n: int, d_y: int):
        self._check(self._L.kwg_mlp_forward(self.ptr, d_x, n, d_y))

    def gradients(self, d_x: int, d_t: int, n: int, d_grad: int, d_floor: int = 0) -> float:
        loss = ctypes.c_double(0)
        self._check(self._L.kwg_mlp_gradients(self.ptr, d_x, d_t, d_floor or None, n, d_grad, ctypes.byref(loss)))
        return loss.value

    def featurize(self, d_opts: int, n: int, d_x: int = 0, d_inside: int = 0, d_base: int = 0):
        """Features [n][5], in-box flags and analytic base prices (BAW) of device options."""
        self._check(self._L.kwg_mlp_featurize(self.ptr, d_opts, n, d_x or None, d_inside or None, d_base or None))

    def train(self, d_opts: int, d_prices: int, n: int, epochs: int, batch: int, lr: float, seed: int = 1) -> float:
        loss = ctypes.c_double(0)
        self._check(self._L.kwg_mlp_train(self.ptr, d_opts, d_prices, n, epochs, batch, lr, seed,
                                          ctypes.byref(loss)))
        return loss.value

    def train_history(self) -> dict:
        """The last train() run: per-epoch mean losses, the epoch whose parameters the
        network kept, and the returns to them after a loss spike."""
        best, restarts = ctypes.c_int(0), ctypes.c_int(0)
        n = self._L.kwg_mlp_train_history(self.ptr, None, 0, ctypes.byref(best), ctypes.byref(restarts))
        if n < 0:
            raise RuntimeError("kwg_mlp_train_history: invalid arguments")
        losses = np.zeros(n)
        self._L.kwg_mlp_train_history(self.ptr, losses.ctypes.data if n else None, n, None, None)
        return {"losses": losses, "best_epoch": best.value, "restarts": restarts.value}

    def price_device(self, d_opts: int, n: int, d_prices: int, d_inside: int = 0):
        self._check(self._L.kwg_mlp_price_device(self.ptr, d_opts, n, d_prices, d_inside or None))

    def price(self, ctx: Context, opts: np.ndarray, fd: Fd1dParams, audit_frac: float = 0.01, seed: int = 1):
        """Host options -> (prices, route, Audit): the network inside its training box,
        FD outside it and on the seeded audit sample."""
        opts = np.ascontiguousarray(opts, dtype=OPTION_DTYPE)
        n = len(opts)
        prices = np.empty(n, np.float64)
        route = np.empty(n, np.int32)
        a = Audit()
        self._check(self._L.kwg_surrogate_price(ctx.ptr, self.ptr, opts.ctypes.data, n, ctypes.byref(fd),
                                                audit_frac, seed, prices.ctypes.data, route.ctypes.data,
                                                ctypes.byref(a)))
        return prices, route, a


# ----------------------------------------------------------------------------- kw::Config


class Config:
    """kw::Config (src/Core/kwConfig.h:21-73): separate double / integer / string maps;
    ``get`` looks in the map matching the type of its default."""

    def __init__(self):
        self._d: dict[str, float] = {}
        self._i: dict[str, int] = {}
        self._s: dict[str, str] = {}

    def set(self, key: str, value):
        if isinstance(value, bool) or isinstance(value, (int, np.integer)):
            self._i[key] = int(value)
        elif isinstance(value, (float, np.floating)):
            self._d[key] = float(value)
        elif isinstance(value, str):
            self._s[key] = value
        else:
            raise TypeError(f"Config.set: unsupported type {type(value).__name__}")

    def get(self, key: str, default):
        if isinstance(default, bool) or isinstance(default, (int, np.integer)):
            return self._i.get(key, int(default))
        if isinstance(default, (float, np.floating)):
            return self._d.get(key, float(default))
        if isinstance(default, str):
            return self._s.get(key, default)
        raise TypeError(f"Config.get: unsupported default type {type(default).__name__}")

    def erase(self, key: str):
        for m in (self._d, self._i, self._s):
            m.pop(key, None)


# ----------------------------------------------------------------------------- kw::Pricer


@dataclass
class Option:
    """kw::Option (src/Core/kwAsset.h:12-22)."""

    t: float
    k: float
    z: float
    r: float
    q: float
    s: float
    e: int
    w: int


def to_array(assets) -> np.ndarray:
    """List of Option (or tuples in kw::Option field order) -> OPTION_DTYPE array."""
    if isinstance(assets, np.ndarray) and assets.dtype == OPTION_DTYPE:
        return assets
    out = np.zeros(len(assets), OPTION_DTYPE)
    for i, a in enumerate(assets):
        if isinstance(a, Option):
            a = (a.t, a.k, a.z, a.r, a.q, a.s, a.e, a.w)
        out[i] = tuple(a)
    return out


class Pricer:
    """kw::Pricer (src/Pricer/kwPricer.h:12-22). Errors are strings, "" = success."""

    def init(self, config: Config) -> str:  # pragma: no cover - interface
        raise NotImplementedError

    def price(self, assets, prices: list) -> str:  # pragma: no cover - interface
        raise NotImplementedError


_PRECISIONS = {"FP64": FP64, "FP32": FP32}
_SOLVERS = {"AUTO": SOLVER_AUTO, "THOMAS": SOLVER_THOMAS, "PCR": SOLVER_PCR}


class Fd1dGpuPricer(Pricer):
    """Drop-in for kw::Fd1d_Pricer (src/Pricer/kwFd1d.cpp:9-160) on the GPU.

    Reads the reference keys FD1D.DENSITY (0.25), FD1D.SCALE (50.),
    FD1D.T_GRID_SIZE (512), FD1D.X_GRID_SIZE (512) with the reference defaults,
    plus FD1D.THETA (0.5), FD1D.PRECISION ("FP64"|"FP32"), FD1D.SOLVER
    ("AUTO"|"THOMAS"|"PCR"), FD1D.STRICT (1: fail the whole call on the first
    out-of-grid asset like the reference, src/Pricer/kwFd1d.cpp:154-155; 0: NaN and a
    per-option status), FD1D.DEVICE (0)."""

    def __init__(self):
        self.params = default_params()
        self.ctx: Context | None = None
        self.status = np.zeros(0, np.int32)

    def init(self, config: Config) -> str:
        p = self.params
        p.density = config.get("FD1D.DENSITY", 0.25)
        p.scale = config.get("FD1D.SCALE", 50.0)
        p.t_dim = config.get("FD1D.T_GRID_SIZE", 512)
        p.x_dim = config.get("FD1D.X_GRID_SIZE", 512)
        p.theta = config.get("FD1D.THETA", 0.5)
        prec = config.get("FD1D.PRECISION", "FP64")
        solver = config.get("FD1D.SOLVER", "AUTO")
        if prec not in _PRECISIONS:
            return f"Fd1dGpu_Pricer::init: unknown FD1D.PRECISION = {prec}"
        if solver not in _SOLVERS:
            return f"Fd1dGpu_Pricer::init: unknown FD1D.SOLVER = {solver}"
        p.precision = _PRECISIONS[prec]
        p.solver = _SOLVERS[solver]
        p.strict = config.get("FD1D.STRICT", 1)
        try:
            self.ctx = Context(config.get("FD1D.DEVICE", 0))
        except RuntimeError as ex:
            return f"Fd1dGpu_Pricer::init: {ex}"
        return ""

    _name = "Fd1dGpu_Pricer"

    def _solve(self, arr):
        return self.ctx.fd1d_price(arr, self.params)

    def price(self, assets, prices: list) -> str:
        arr = to_array(assets)
        if len(arr) == 0:
            return ""
        if self.ctx is None:
            return f"{self._name}::price: init was not called"
        rc, out, status = self._solve(arr)
        self.status = status
        prices[:] = out.tolist()
        if rc != KWG_OK:
            return f"{self._name}::price: " + self.ctx.last_error()
        return ""

    def price_array(self, arr: np.ndarray):
        """Fast path: OPTION_DTYPE array -> (error, prices ndarray, status ndarray)."""
        rc, out, status = self._solve(arr)
        return ("" if rc == KWG_OK else f"{self._name}::price: " + self.ctx.last_error()), out, status


class Fd1dBsGpuPricer(Fd1dGpuPricer):
    """Drop-in for kw::Fd1d_BlackScholes_Pricer (src/Pricer/kwFd1d_BlackScholes.cpp:15-42):
    FD(asset) + BS(European copy) - FD(European copy), same FD1D.* keys."""

    _name = "Fd1dBsGpu_Pricer"

    def _solve(self, arr):
        return self.ctx.fd1d_bs_price(arr, self.params)


class PricerFactory:
    """kw::PricerFactory (src/Pricer/kwPricerFactory.h:15-41).  "FD1D" / "FD1D-GPU"
    create the GPU FD pricer, "FD1D-BS" / "FD1D-BS-GPU" its control-variate form
    (the drop-ins); unknown keys are an error."""

    @staticmethod
    def create(config: Config):
        mode = config.get("PRICER", "")
        if not mode:
            return "PricerFactory: Missing PRICER key", None
        if mode in ("FD1D", "FD1D-GPU"):
            pricer = Fd1dGpuPricer()
        elif mode in ("FD1D-BS", "FD1D-BS-GPU"):
            pricer = Fd1dBsGpuPricer()
        else:
            return f"PricerFactory: Unknown PRICER = {mode}", None
        err = pricer.init(config)
        if err:
            return "PricerFactory: " + err, None
        return "", pricer


def params(t_dim=512, x_dim=512, theta=0.5, scale=50.0, density=0.25, precision=FP64, solver=SOLVER_AUTO,
           strict=0, block_warps=0, option_warps=0, sm_blocks=0) -> Fd1dParams:
    p = default_params()
    p.t_dim, p.x_dim, p.theta, p.scale, p.density = t_dim, x_dim, theta, scale, density
    p.precision, p.solver, p.strict = precision, solver, strict
    p.block_warps, p.option_warps, p.sm_blocks = block_warps, option_warps, sm_blocks
    return p


UNIFORM = math.inf  # density value selecting the uniform grid
