"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a container where the reference sources are mounted:
    make -C oracle ref && python tests/golden/make_golden.py /root/reference

Sources of truth:
  * test/kwPricer_test.cpp:16-28  -- 12 options with expected prices (read as text)
  * test/portfolio_qdfp.csv.zst   -- 6000 American puts with QuantLib QdFp prices
  * test/portfolio_fd1d.csv.zst   -- 6000 American puts (strike grid), QdFp prices
  * oracle/_ref/libkwref.so       -- the reference's own pricer (src/ compiled as is)
Every reference run is made twice and must agree bit for bit (its thread pool's
wait() can return early, src/kwThreadPool.cpp:58-72, so a torn run is rejected).
"""
from __future__ import annotations

import ctypes
import ctypes.util
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "kwinto-cuda_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import kwor  # noqa: E402
import portfolio  # noqa: E402
from kwg import OPTION_DTYPE  # noqa: E402


def zstd_decompress(path: str) -> str:
    lib = ctypes.CDLL(ctypes.util.find_library("zstd") or "libzstd.so.1")
    lib.ZSTD_getFrameContentSize.restype = ctypes.c_ulonglong
    lib.ZSTD_getFrameContentSize.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    lib.ZSTD_decompress.restype = ctypes.c_size_t
    lib.ZSTD_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
    lib.ZSTD_isError.argtypes = [ctypes.c_size_t]
    lib.ZSTD_isError.restype = ctypes.c_uint
    src = open(path, "rb").read()
    size = lib.ZSTD_getFrameContentSize(src, len(src))
    if size >= 2**63:
        raise RuntimeError(f"{path}: frame size unknown")
    dst = ctypes.create_string_buffer(size)
    got = lib.ZSTD_decompress(dst, size, src, len(src))
    if lib.ZSTD_isError(got):
        raise RuntimeError(f"{path}: zstd error")
    return dst.raw[:got].decode()


def ref_twice(opts, **kw):
    rc1, msg1, p1, _ = kwor.ref_price(opts, **kw)
    rc2, msg2, p2, _ = kwor.ref_price(opts, **kw)
    if rc1 != rc2 or not np.array_equal(p1, p2, equal_nan=True):
        raise RuntimeError("reference runs disagree (thread-pool race); rerun")
    return rc1, msg1, p1


def parse_pricer_test(ref: str):
    """The m_testData table of test/kwPricer_test.cpp: {{t, k, z, r, q, s, e, w}, price}."""
    text = open(os.path.join(ref, "test", "kwPricer_test.cpp")).read()
    rows = re.findall(r"\{\{([^{}]*)\},\s*([0-9.eE+-]+)\}", text)
    opts = np.zeros(len(rows), OPTION_DTYPE)
    want = np.zeros(len(rows))
    for i, (fields, price) in enumerate(rows):
        v = [float(x) for x in fields.split(",")]
        opts[i] = (v[0], v[1], v[2], v[3], v[4], v[5], int(v[6]), int(v[7]))
        want[i] = float(price)
    return opts, want


def main(ref: str):
    out = {}
    # 1. kwPricer_test table, priced by the reference at its defaults.
    opts, want = parse_pricer_test(ref)
    assert len(opts) == 12, len(opts)
    rc, msg, fd = ref_twice(opts, pricer="FD1D")
    assert rc == 0, msg
    rc, msg, fdbs = ref_twice(opts, pricer="FD1D-BS")
    assert rc == 0, msg
    rc, msg, bs = ref_twice(opts, pricer="BS")
    assert rc == 0, msg
    np.savez_compressed(os.path.join(HERE, "pricer_test.npz"), opts=opts, want=want, ref_fd1d=fd,
                        ref_fd1d_bs=fdbs, ref_bs=bs)
    out["pricer_test"] = dict(n=12, tol=1.3e-3, max_abs_fd1d=float(np.max(np.abs(fd - want))))

    # 2. Portfolio fixtures (6000 puts each), reference FD1D at 512x512 defaults.
    for name in ("qdfp", "fd1d"):
        text = zstd_decompress(os.path.join(ref, "test", f"portfolio_{name}.csv.zst"))
        o, qd = portfolio.load_csv(text, is_text=True)
        amer = o[o["e"] == 1]
        qd = qd[o["e"] == 1]
        rc, msg, fd = ref_twice(amer, pricer="FD1D", t_dim=512, x_dim=512)
        assert rc == 0, msg
        np.savez_compressed(os.path.join(HERE, f"portfolio_{name}.npz"), opts=amer, quantlib=qd, ref_fd1d=fd)
        out[f"portfolio_{name}"] = dict(n=int(len(amer)), max_abs_vs_quantlib=float(np.max(np.abs(fd - qd))))

    # 3. Synthetic workloads at their grids (reference has no uniform mode: d = 1e6).
    o1 = portfolio.american_portfolio(128, seed=42)
    rc, msg, p1 = ref_twice(o1, pricer="FD1D", density=0.25, scale=5.0, t_dim=512, x_dim=512)
    assert rc == 0, msg
    o2 = portfolio.american_portfolio(256, seed=42)
    rc, msg, p2 = ref_twice(o2, pricer="FD1D", density=portfolio.REFERENCE_UNIFORM_DENSITY, scale=5.0,
                            t_dim=1024, x_dim=1024)
    assert rc == 0, msg
    o4 = portfolio.american_portfolio(32, seed=42)
    rc, msg, p4 = ref_twice(o4, pricer="FD1D", density=0.25, scale=5.0, t_dim=2048, x_dim=2048)
    assert rc == 0, msg
    np.savez_compressed(os.path.join(HERE, "synthetic.npz"), small_opts=o1, small_ref=p1,
                        batch1024_opts=o2, batch1024_ref=p2, fine2048_opts=o4, fine2048_ref=p4)
    out["synthetic"] = dict(small=len(o1), batch1024_sample=len(o2), fine2048_sample=len(o4))

    # 4. Edge cases: European options, calls/puts, duplicates (dedup path), odd grids,
    #    and an out-of-grid spot (the reference fails the whole call).
    e = np.zeros(8, OPTION_DTYPE)
    e[0] = (1.0, 100.0, 0.2, 0.06, 0.02, 100.0, 0, -1)
    e[1] = (1.0, 100.0, 0.2, 0.06, 0.02, 100.0, 0, 1)
    e[2] = (0.5, 90.0, 0.3, 0.01, 0.05, 100.0, 1, 1)
    e[3] = (0.5, 110.0, 0.3, 0.01, 0.05, 100.0, 1, 1)   # same PDE key as e[2]
    e[4] = (0.5, 90.0, 0.3, 0.01, 0.05, 95.0, 1, 1)     # same key again, other spot
    e[5] = (2.0, 100.0, 0.6, 0.1, 0.0, 100.0, 1, -1)
    e[6] = (0.02, 100.0, 0.05, 0.0, 0.0, 100.0, 1, -1)  # very short, low vol
    e[7] = (1.0, 100.0, 0.2, 0.06, 0.02, 100.0, 1, -1)
    cases = {}
    for name, kw in {"default": {}, "x3_t2": dict(x_dim=3, t_dim=2), "x7_t5": dict(x_dim=7, t_dim=5),
                     "x64_t33": dict(x_dim=64, t_dim=33, scale=5.0)}.items():
        rc, msg, p = ref_twice(e, pricer="FD1D", **kw)
        assert rc == 0, (name, msg)
        cases[name] = p
    bad = e.copy()
    bad[3]["s"] = 1e12  # log(s/k) = 22.8, outside the default half-width 50*0.3*sqrt(0.5)
    rc, msg, _ = ref_twice(bad, pricer="FD1D")
    assert rc != 0
    np.savez_compressed(os.path.join(HERE, "edge.npz"), opts=e, bad_opts=bad, **{f"ref_{k}": v for k, v in
                                                                                cases.items()})
    out["edge"] = dict(cases=list(cases), bad_message=msg)
    with open(os.path.join(HERE, "golden_manifest.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
