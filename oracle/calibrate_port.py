"""Speed of the oracle port against the reference itself, on one host.  TEST
INFRASTRUCTURE ONLY.

The timed CPU baseline on a host without the reference's sources is the oracle port
(fd1d_oracle.c, bit-exact to the reference).  Its speed is not the reference's:
the reference allocates its grids per call, recomputes the stencil with divisions
at every node-step (src/Math/kwFd1d.cpp:86-102), allocates the Thomas scratch per
solve (src/Math/kwMath.cpp:26) and runs its jobs on kw::ThreadPool
(src/kwThreadPool.cpp:43-72).  This script times both on the same options, grid and
thread count -- the reference through PricerFactory("FD1D") in oracle/_ref, the port
through kwor_fd1d_price -- and writes the ratio to port_calibration.json, which the
reference arm of bench.py reports beside the port's rate.

    make -C oracle && make -C oracle ref && python oracle/calibrate_port.py [N_OPTIONS]
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "kwinto-cuda_gb300"))

import numpy as np  # noqa: E402

import kwor  # noqa: E402
import portfolio  # noqa: E402

OUT = os.path.join(HERE, "port_calibration.json")


def main(n: int = 512, repeats: int = 3) -> dict:
    if not kwor.ref_available():
        raise SystemExit("oracle/_ref/libkwref.so missing: make -C oracle ref (needs the reference sources)")
    opts = portfolio.american_portfolio(n, seed=42)
    grid = dict(t_dim=1024, x_dim=1024, scale=5.0)
    threads = kwor.ref_lib().kwref_pool_size()  # the reference's pool: hardware_concurrency()
    ref_s, port_s = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        rc, msg, ref, _ = kwor.ref_price(opts, density=portfolio.REFERENCE_UNIFORM_DENSITY, **grid)
        ref_s.append(time.perf_counter() - t0)
        if rc != 0:
            raise SystemExit(msg)
        t0 = time.perf_counter()
        rc, msg, port, _ = kwor.fd1d_price(opts, nthreads=threads, density=portfolio.REFERENCE_UNIFORM_DENSITY,
                                           **grid)
        port_s.append(time.perf_counter() - t0)
        if rc != 0:
            raise SystemExit(msg)
    rec = {
        "workload": f"{n} options of the 32768-option batch (seed 42), 1024x1024, scale 5, density 1e6",
        "threads": threads,
        "host": f"{platform.machine()}, {os.cpu_count()} cores",
        "reference_options_per_sec": n / min(ref_s),
        "port_options_per_sec": n / min(port_s),
        "port_over_reference": min(ref_s) / min(port_s),
        "max_rel_diff": float(np.max(np.abs(ref - port) / np.abs(ref))),
        "timing": f"best of {repeats}, wall time of one pricing call",
    }
    with open(OUT, "w") as f:
        json.dump(rec, f, indent=1)
        f.write("\n")
    return rec


if __name__ == "__main__":
    print(json.dumps(main(int(sys.argv[1]) if len(sys.argv) > 1 else 512), indent=1))
