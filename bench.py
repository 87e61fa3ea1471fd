"""Benchmark: batched FD1D American-option pricing on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step"): one batch of 32768 American options (half puts, half calls,
S=100, K~U[80,120], vol~U[0.1,0.6], r,q~U[0,0.1], T~U[0.25,2]), 1024 x 1024 grid,
theta 0.5, scale 5, uniform x-grid, FP64 -- the reference's largest logged shape
(log/z800_1024_32768.log).  Synthetic, seeded (kwinto-cuda_gb300/portfolio.py).

Reported on one JSON line (rank 0):
  value      options/s with inputs resident in HBM (kwg_fd1d_price_device), CUDA
             events on the launching stream, K steps after W warm-up steps; the
             per-step working set (2.4 GB of coefficients, payoff and state) is far larger
             than L2, so no flush is needed between steps.
  e2e        the same metric through the reference-facing call (kwg_fd1d_price: host
             options in, host prices out; dedup, H2D and D2H inside the timing).
  roofline   of the solve kernel, from its own CUDA events inside the timed region:
             achieved = 32 B per node-step (the streaming scheme's algorithmic bytes)
             over the launch time; the kernel's own count of requested bytes beside it.
  variants   FP64 and FP32 rates and their errors against the FP64 oracle.
  cpu_baseline  the oracle (C restatement of the reference, all host cores) on a
             bounded sample of the same workload; its prices are the FP64 parity check
             of the resident run.
With --impl reference the reference's CPU implementation runs instead (oracle/_ref
when it was built here from the reference sources, else the oracle port, with the
port/reference speed ratio measured by oracle/calibrate_port.py).  --gpus N without
a launcher re-runs the script as N ranks through torch.distributed.run.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "kwinto-cuda_gb300"))

N_OPTIONS = 32768
X_DIM = T_DIM = 1024
SCALE = 5.0
DENSITY = math.inf  # uniform grid
WORKLOAD = "fd1d_american_32768x1024x1024"
# The reference's own published FD64 number for this exact shape (its benchmark log
# log/z800_1024_32768.log:87-93, GTX 1070): 32768 options per 39,901.747 ms.
REF_PUBLISHED_OPS = 32768 / 39.901747
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def node_steps(n, x_dim=None, t_dim=None):
    return n * (x_dim or X_DIM) * ((t_dim or T_DIM) - 1)


# Traffic of the FP64 streaming solve per node and step: V and the sweep value read and
# written (32 B, the algorithmic bytes of the scheme) plus what the kernel also reads:
# outside the uniform grid's frozen middle region three factor coefficients (24 B),
# and the payoff (8 B) where it is not +0 for the whole tile.  The kernel counts the
# bytes it requests itself (kwg_profile_read).
FP64_FLOPS_PER_NODE_STEP = 6  # 3 FMA per node-step at theta = 1/2
ALGO_BYTES_PER_NODE_STEP = 32  # FP64 streaming scheme: V read + write, sweep value write + read


def workload_config():
    """The `config` both arms print (same keys and values, so the two lines compare)."""
    return {"workload": WORKLOAD, "options_per_batch": N_OPTIONS, "x_dim": X_DIM, "t_dim": T_DIM, "theta": 0.5,
            "scale": SCALE, "grid": "uniform", "precision": "fp64",
            "l2": "working set 2.4 GB per step > 129 MB L2 (no flush needed)"}


CALIBRATION_FILE = os.path.join(ROOT, "oracle", "port_calibration.json")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join("/tmp", f"kwg_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        d = json.load(open(PEAKS_FILE))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def cpu_oracle_rate(opts_all, budget_s=12.0):
    """The oracle (C restatement, all host cores) on a bounded sample of the workload:
    the first n options of the batch, n grown until one call takes budget_s / 4.
    Returns (options/s, threads, n, seconds, the n oracle prices)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import kwor

    threads = os.cpu_count() or 1
    n = 32
    while True:
        sample = opts_all[:n]
        t0 = time.perf_counter()
        rc, msg, want, _ = kwor.fd1d_price(sample, nthreads=threads, t_dim=T_DIM, x_dim=X_DIM, scale=SCALE,
                                           density=DENSITY)
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(msg)
        if dt >= budget_s / 4 or n >= len(opts_all):
            return n / dt, threads, n, dt, want
        n = min(len(opts_all), int(n * max(2.0, budget_s / 4 / max(dt, 1e-3))))


def max_rel(got, want):
    """Max relative error (prices of this workload are >= ~3e-4, so no floor is needed
    beyond guarding an exact zero)."""
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-300)))


def uneven_oracle_check(opts, x_dims, t_dims, prices, status, sample=4096):
    """FP64 prices of the uneven batch against the oracle on an evenly spaced sample,
    one oracle call per (x_dim, t_dim) group as the reference requires (one grid shape
    per Fd1d_Pricer::init, src/Pricer/kwFd1d.cpp:15-16), the groups spread over the
    host cores.  Out-of-grid status must agree; prices are compared where both are OK."""
    import concurrent.futures as cf

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import kwor

    idx = np.linspace(0, len(opts) - 1, min(sample, len(opts))).astype(np.int64)
    groups = {}
    for i in idx:
        groups.setdefault((int(x_dims[i]), int(t_dims[i])), []).append(i)

    def one(key):
        ii = np.array(groups[key])
        rc, msg, want, st = kwor.fd1d_price(opts[ii], nthreads=1, t_dim=key[1], x_dim=key[0], scale=SCALE,
                                            density=DENSITY)
        return ii, want, st

    t0 = time.perf_counter()
    worst, n_ok, status_mismatch = 0.0, 0, 0
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        for ii, want, st in ex.map(one, sorted(groups, key=lambda k: -k[0] * k[1])):
            status_mismatch += int(((st != 0) != (status[ii] != 0)).sum())
            ok = (st == 0) & (status[ii] == 0)
            if ok.any():
                worst = max(worst, max_rel(prices[ii][ok], want[ok]))
                n_ok += int(ok.sum())
    return {"max_rel_err_vs_oracle": worst, "oracle_sample": int(len(idx)), "oracle_sample_priced": n_ok,
            "oracle_groups": len(groups), "status_mismatch": status_mismatch,
            "oracle_s": time.perf_counter() - t0}


def measured_traffic(ns):
    """DRAM bytes per solve launch from the committed ncu summary (dram__bytes_read +
    dram__bytes_write of one captured launch, per node-step), scaled to ns node-steps."""
    path = os.path.join(ROOT, "profiles", "fd1d_solve_fp64_32768x1024.md")
    try:
        for line in open(path):
            if line.startswith("traffic per full launch (bytes):"):
                return float(line.split(":")[1]) / node_steps(32768, 1024, 1024) * ns
    except (OSError, ValueError):
        pass
    return None


def fp64_peak_tflops(dev):
    """FP64 peak of this GPU, measured as cuBLAS DGEMM 4096^3 (best of 5)."""
    import torch

    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize(dev)
        best = max(best, 2 * 4096**3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    return best


def run_reference(args):
    """--impl reference: the reference's CPU implementation on the host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import kwor
    import portfolio

    threads = os.cpu_count() or 1
    per_step = args.ref_options
    use_ref = kwor.ref_available()
    kind = "reference" if use_ref else "port"

    def one(i):
        o = portfolio.american_portfolio(per_step, seed=42, start=(i * per_step) % N_OPTIONS)
        t0 = time.perf_counter()
        if use_ref:
            rc, msg, _, _ = kwor.ref_price(o, density=portfolio.REFERENCE_UNIFORM_DENSITY, scale=SCALE,
                                           t_dim=T_DIM, x_dim=X_DIM)
        else:
            rc, msg, _, _ = kwor.fd1d_price(o, nthreads=threads, t_dim=T_DIM, x_dim=X_DIM, scale=SCALE,
                                            density=DENSITY)
        if rc != 0:
            raise RuntimeError(msg)
        return time.perf_counter() - t0

    for i in range(args.warmup):
        one(i)
    total = sum(one(args.warmup + i) for i in range(args.steps))
    value = per_step * args.steps / total
    cores = kwor.ref_lib().kwref_pool_size() if use_ref else threads
    sample = (f"{per_step} options per step of the {N_OPTIONS}-option batch, {X_DIM}x{T_DIM}, "
              + ("reference src/ compiled from source, density 1e6 (its closest to uniform)" if use_ref
                 else "oracle C restatement (bit-exact port of the reference), uniform grid"))
    baseline = {"value": value, "unit": "options/s", "cores": cores, "kind": kind, "sample": sample}
    if not use_ref:
        # the port's speed against the reference's own build, both timed on one host
        # (oracle/calibrate_port.py): the reference is estimated at value / port_over_reference
        try:
            cal = json.load(open(CALIBRATION_FILE))
            baseline["calibration"] = dict(cal, reference_estimate_options_per_sec=value / cal["port_over_reference"])
        except (OSError, ValueError, KeyError):
            baseline["calibration"] = None
    line = {
        "impl": "reference", "metric": "options_per_sec_fd64_1024x1024", "value": value, "unit": "options/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": value / REF_PUBLISHED_OPS, "dtype": "f64",
        "data": "synthetic (seeded splitmix64; American, S=100, K~U[80,120], vol~U[0.1,0.6], r,q~U[0,0.1], T~U[0.25,2])",
        "config": workload_config(),
        "cpu_baseline": baseline,
        "e2e": {"value": value, "unit": "options/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


SURROGATE_OPTIONS = 1_000_000
SURROGATE_WEIGHTS = os.path.join(ROOT, "kwinto-cuda_gb300", "surrogate_weights.npz")
SURROGATE_AUDIT = 0.01
SURROGATE_CHECK = 32768  # options of the batch re-priced with FD64 for the error report


def surrogate_variant(args, ctx, rank, ws, fd32_rate, barrier, max_over_ranks):
    """1M fresh options through kwg_surrogate_price (host arrays in and out: the
    network inside its training box, FD32 at 1024 x 1024 for out-of-box options and a
    1% seeded audit).  Error vs FD64 (1024 x 1024) on a seeded subsample of the batch."""
    import torch

    import kwg
    import portfolio

    n = args.surrogate_options
    if args.surrogate_train > 0:
        # the network this run prices with is trained here, end to end: FD64 labels on
        # the GPU, the library's tcgen05 training kernels, a held-out check
        import train_surrogate

        net, meta = train_surrogate.train(ctx, n=args.surrogate_train, grid=X_DIM)
        meta["source"] = "trained in this run (train_surrogate.train)"
    else:
        if not os.path.exists(SURROGATE_WEIGHTS):
            return {"unavailable": "surrogate_weights.npz not trained (kwinto-cuda_gb300/train_surrogate.py)"}
        net = kwg.Surrogate(torch.cuda.current_device())
        net.load(SURROGATE_WEIGHTS)
        meta = json.loads(str(np.load(SURROGATE_WEIGHTS)["meta"])) if "meta" in np.load(SURROGATE_WEIGHTS) else {}
        meta["source"] = "committed surrogate_weights.npz (metadata of the run that trained it)"
    opts = portfolio.american_portfolio(n, seed=5005, start=rank * n)
    fd = kwg.params(t_dim=T_DIM, x_dim=X_DIM, scale=SCALE, density=DENSITY, precision=kwg.FP32)
    # the FD32 launch shape for the audit's batch size (~1 % of the options), as a
    # caller would tune it once
    fd_tuning = ctx.autotune_ex(fd, max(1, int(round(n * SURROGATE_AUDIT)))).as_dict()
    for i in range(max(1, args.warmup)):
        prices, route, audit = net.price(ctx, opts, fd, SURROGATE_AUDIT, seed=100 + i)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        prices, route, audit = net.price(ctx, opts, fd, SURROGATE_AUDIT, seed=1000 + i)
    dt = max_over_ranks(time.perf_counter() - t0) / args.steps
    barrier()
    # network alone, inputs resident (device-timed)
    d_o = torch.from_numpy(opts.view(np.uint8).copy()).cuda()
    d_p = torch.empty(n, dtype=torch.float64, device="cuda")
    net.price_device(d_o.data_ptr(), n, d_p.data_ptr())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        net.price_device(d_o.data_ptr(), n, d_p.data_ptr())
    e1.record()
    torch.cuda.synchronize()
    net_ms = e0.elapsed_time(e1) / args.steps
    # error vs FD64 on a seeded subsample (all routes)
    idx = np.sort(np.random.default_rng(77).choice(n, size=min(SURROGATE_CHECK, n), replace=False))
    p64 = kwg.params(t_dim=T_DIM, x_dim=X_DIM, scale=SCALE, density=DENSITY, precision=kwg.FP64)
    rc, ref, st = ctx.fd1d_price(opts[idx], p64)
    if rc != 0:
        raise RuntimeError(ctx.last_error())
    err = np.abs(prices[idx] - ref)
    net.close()
    rate = ws * n / dt
    return {"options_per_sec_e2e": rate, "ms_per_batch_e2e": dt * 1e3, "options": n,
            "speedup_vs_fd32": rate / fd32_rate, "fd32_options_per_sec": fd32_rate,
            "network_ms_resident": net_ms, "network_options_per_sec_resident": n / (net_ms / 1e3),
            "routed_network": int((route == kwg.ROUTE_NETWORK).sum()),
            "routed_audit": int(audit.audited), "routed_out_of_box": int(audit.out_of_box),
            "routed_fd_failed": int((route == kwg.ROUTE_FD_FAILED).sum()),
            "audit_abs_max": audit.audit_abs_max,
            "audit_abs_mean": audit.audit_abs_sum / max(1, audit.audited),
            "check_sample": len(idx), "p99_abs_err_vs_fd64": float(np.quantile(err, 0.99)),
            "max_abs_err_vs_fd64": float(err.max()), "mean_abs_err_vs_fd64": float(err.mean()),
            "training": meta,
            "fd32_audit_tuning": {"option_warps": fd_tuning["option_warps"],
                                  "fp32_ms_by_option_warps": fd_tuning["fp32_ms_by_option_warps"]},
            "workload": "1M fresh options (seeded; S=100, K~U[80,120], vol~U[0.1,0.6], r,q~U[0,0.1], T~U[0.25,2]), 1% audit, FD32 fallback at "
                        "1024x1024; kwg_surrogate_price (host arrays, H2D/D2H inside the timing)"}


def run_ours(args):
    import torch

    import kwg
    import portfolio
    import shard

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = kwg.Context(local)
    # a dedicated non-default stream: the kernels and the timing events share it
    # (a NULL stream handle would mean the context's own stream to the C ABI)
    stream = torch.cuda.Stream(dev)

    if args.scaling == "strong":
        # one batch for the whole job: every rank deduplicates it alike and prices the
        # options of its share of the PDEs (split by work); prices are gathered after
        full = portfolio.american_portfolio(N_OPTIONS, seed=42)
        own = shard.strong_shard(full, rank, ws, x_dim=X_DIM, t_dim=T_DIM)
        opts = full[own]
        n_loc, n_job = len(opts), N_OPTIONS
    else:
        # each rank prices its own batch (weak scaling), drawn from its own window of the stream
        opts = shard.portfolio_shard(N_OPTIONS, rank, seed=42)
        n_loc, n_job = N_OPTIONS, ws * N_OPTIONS
    prm = kwg.params(t_dim=T_DIM, x_dim=X_DIM, scale=SCALE, density=DENSITY, precision=kwg.FP64)
    d_opts = torch.from_numpy(opts.view(np.uint8).copy()).to(dev)
    d_prices = torch.empty(n_loc, dtype=torch.float64, device=dev)
    d_status = torch.empty(n_loc, dtype=torch.int32, device=dev)

    # ---------------------------------------------------------------- autotuner: launch shapes
    # options per block and Thomas vs PCR (FP64), threads per option (FP32), on this shape
    tune64 = ctx.autotune_ex(prm, n_loc).as_dict()
    tune32 = ctx.autotune_ex(kwg.params(t_dim=T_DIM, x_dim=X_DIM, scale=SCALE, density=DENSITY,
                                        precision=kwg.FP32), n_loc).as_dict()

    def step(params=prm):
        rc = ctx.fd1d_price_device(d_opts.data_ptr(), n_loc, params, d_prices.data_ptr(), d_status.data_ptr(),
                                   stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(ctx.last_error())
        return ctx.launch_count()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x):
        return shard.max_over_ranks(x)

    # ---------------------------------------------------------------- resident (value)
    for _ in range(args.warmup):
        step()
    barrier()
    ctx.set_profiling(True)
    clocks = Clocks(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        launches += step()
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    solve_ms, solve_n, solve_bytes = ctx.profile_read(with_bytes=True)
    ctx.set_profiling(False)
    ms = max_over_ranks(e0.elapsed_time(e1))
    value = n_job * args.steps / (ms / 1e3)
    status = d_status.cpu().numpy()
    gpu_prices = d_prices.cpu().numpy()
    if not (status == 0).all():
        raise RuntimeError(f"{int((status != 0).sum())} options failed")
    if args.scaling == "strong":
        # the 8-byte prices of every rank's share, assembled for the whole batch
        whole = shard.gather_prices(N_OPTIONS, own, gpu_prices)
        if np.isnan(whole).any():
            raise RuntimeError("strong scaling: some options were priced by no rank")

    # ---------------------------------------------------------------- end to end (e2e)
    prices_host = np.empty(n_loc)
    for _ in range(max(1, args.warmup)):
        rc, prices_host, _ = ctx.fd1d_price(opts, prm)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc, prices_host, st = ctx.fd1d_price(opts, prm)
        if rc != 0:
            raise RuntimeError(ctx.last_error())
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    barrier()
    e2e_value = n_job * args.steps / e2e_s
    if not np.array_equal(prices_host, gpu_prices):
        raise RuntimeError("host and device entry points disagree")
    # bytes the host call moves per step (include/kwg.h packing): per PDE t,z,r,q (f64) + w,e;
    # per asset s,k (f64) + pde index (i32); back: price (f64) + status (i32) per asset.
    h2d = n_loc * (4 * 8 + 2) + n_loc * (2 * 8 + 4)
    d2h = n_loc * (8 + 4)

    # ---------------------------------------------------------------- FP32 variant (resident)
    prm32 = kwg.params(t_dim=T_DIM, x_dim=X_DIM, scale=SCALE, density=DENSITY, precision=kwg.FP32)
    for _ in range(args.warmup):
        step(prm32)
    barrier()
    ctx.set_profiling(True)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        launches32 = step(prm32)
    f1.record(stream)
    barrier()
    solve32_ms, solve32_n = ctx.profile_read()
    ctx.set_profiling(False)
    ms32 = max_over_ranks(f0.elapsed_time(f1))
    value32 = n_job * args.steps / (ms32 / 1e3)
    p32 = d_prices.cpu().numpy()
    if not (d_status.cpu().numpy() == 0).all():
        raise RuntimeError("FP32: options failed")
    err32 = np.abs(p32 - gpu_prices)

    # ---------------------------------------------------------------- FD1D-BS control variate (host API)
    # on the benchmark's uniform grid and on the reference's default sinh grid
    # (density 0.25), where the coefficients stream at every node and the American and
    # European PDEs of an option share one record (twin tiles)
    fd1d_bs = {}
    for bs_name, bs_density in (("uniform", DENSITY), ("sinh_density_0.25", 0.25)):
        prm_bs = kwg.params(t_dim=T_DIM, x_dim=X_DIM, scale=SCALE, density=bs_density, precision=kwg.FP64)
        for _ in range(max(1, args.warmup)):
            rc, pbs, stbs = ctx.fd1d_bs_price(opts, prm_bs)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rc, pbs, stbs = ctx.fd1d_bs_price(opts, prm_bs)
            if rc != 0:
                raise RuntimeError(ctx.last_error())
        dtbs = max_over_ranks(time.perf_counter() - t0) / args.steps
        leg = {"options_per_sec_e2e": n_job / dtbs, "ms_per_batch_e2e": dtbs * 1e3, "density": bs_density,
               "pdes_solved": 2 * n_loc, "launches": ctx.launch_count()}
        if not args.no_cpu and rank == 0:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import kwor

            idx = np.arange(0, n_loc, max(1, n_loc // 512))
            rcb, msgb, wantbs, _ = kwor.fd1d_price(opts[idx], bs=True, t_dim=T_DIM, x_dim=X_DIM, scale=SCALE,
                                                   density=bs_density)
            if rcb != 0:
                raise RuntimeError(msgb)
            # a deep out-of-the-money control-variate price is a cancellation residue:
            # below 1e-3 the error is taken absolutely (relative to 1e-3)
            leg["max_rel_err_vs_oracle"] = float(np.max(np.abs(pbs[idx] - wantbs) / np.maximum(np.abs(wantbs), 1e-3)))
            leg["oracle_sample"] = len(idx)
        fd1d_bs[bs_name] = leg

    # ---------------------------------------------------------------- uneven batch (131072 options, per-option grids)
    uneven = {}
    if not args.no_uneven:
        o3, xd3, td3 = portfolio.uneven_portfolio(131072, seed=42, start=rank * 131072)
        ns3 = int((xd3.astype(np.int64) * (td3.astype(np.int64) - 1)).sum())
        uneven["tuning"] = {}
        for name, prec in (("fp64", kwg.FP64), ("fp32", kwg.FP32)):
            p3 = kwg.params(scale=SCALE, density=DENSITY, precision=prec)
            uneven["tuning"][name] = ctx.autotune_uneven(o3, xd3, td3, p3).as_dict()
            for _ in range(max(1, args.warmup)):
                rc, pr3, st3 = ctx.fd1d_price_uneven(o3, xd3, td3, p3)  # first call captures the graph
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                rc, pr3, st3 = ctx.fd1d_price_uneven(o3, xd3, td3, p3)
                if rc != 0:
                    raise RuntimeError(ctx.last_error())
            dt3 = max_over_ranks(time.perf_counter() - t0) / args.steps
            ctx.set_profiling(True)
            ctx.fd1d_price_uneven(o3, xd3, td3, p3)
            sms, sn = ctx.profile_read()
            ctx.set_profiling(False)
            uneven[name] = {"options_per_sec_e2e": ws * len(o3) / dt3, "ms_per_batch_e2e": dt3 * 1e3,
                            "solve_ms": sms, "solve_launches": sn, "node_steps": ns3,
                            "out_of_grid": int((st3 == kwg.STATUS_OUT_OF_GRID).sum()),
                            "failed_other": int(((st3 != 0) & (st3 != kwg.STATUS_OUT_OF_GRID)).sum())}
            if name == "fp64":
                ref64 = pr3.copy()
                if not args.no_cpu and rank == 0:
                    uneven[name].update(uneven_oracle_check(o3, xd3, td3, pr3, st3))
            else:
                ok = st3 == 0
                e = np.abs(pr3[ok] - ref64[ok])
                uneven[name]["max_abs_err_vs_fd64"] = float(e.max())
                uneven[name]["p99_abs_err_vs_fd64"] = float(np.percentile(e, 99))

    # ---------------------------------------------------------------- surrogate + FD32 fallback (1M fresh options)
    surrogate = surrogate_variant(args, ctx, rank, ws, value32, barrier, max_over_ranks) if not args.no_surrogate \
        else {"skipped": "--no-surrogate"}

    # ---------------------------------------------------------------- precision study (65536 options, 2048 x 2048)
    fine = {"skipped": "--no-fine-study"}
    if not args.no_fine_study:
        o4 = portfolio.american_portfolio(65536, seed=44, start=rank * 65536)
        res4 = {}
        # threads per option of the FP32 solver on this shape (2, 4 or 8 warps at 2048 nodes)
        tune4 = ctx.autotune_ex(kwg.params(t_dim=2048, x_dim=2048, scale=SCALE, density=0.25, precision=kwg.FP32),
                                len(o4)).as_dict()
        for name, prec in (("fp64", kwg.FP64), ("fp32", kwg.FP32)):
            p4 = kwg.params(t_dim=2048, x_dim=2048, scale=SCALE, density=0.25, precision=prec)
            rc, pr4, st4 = ctx.fd1d_price(o4, p4)  # warm-up (allocations)
            barrier()
            t0 = time.perf_counter()
            rc, pr4, st4 = ctx.fd1d_price(o4, p4)
            if rc != 0:
                raise RuntimeError(ctx.last_error())
            dt4 = max_over_ranks(time.perf_counter() - t0)
            res4[name] = (pr4, st4, dt4)
        p64_, s64_, t64_ = res4["fp64"]
        p32_, s32_, t32_ = res4["fp32"]
        ok4 = (s64_ == 0) & (s32_ == 0)
        e_abs = np.abs(p32_[ok4] - p64_[ok4])
        e_rel = e_abs / np.maximum(np.abs(p64_[ok4]), 1e-12)
        fine = {"options": len(o4), "x_dim": 2048, "t_dim": 2048, "density": 0.25, "scale": SCALE,
                   "fd64_options_per_sec_e2e": ws * len(o4) / t64_, "fd32_options_per_sec_e2e": ws * len(o4) / t32_,
                   "fd32_speedup": t64_ / t32_,
                   "fd32_max_abs_err_vs_fd64": float(e_abs.max()),
                   "fd32_p99_abs_err_vs_fd64": float(np.percentile(e_abs, 99)),
                   "fd32_max_rel_err_vs_fd64": float(e_rel.max()),
                   "fd32_p99_rel_err_vs_fd64": float(np.percentile(e_rel, 99)),
                   "failed": int((~ok4).sum()),
                   "fp32_tuning": {"option_warps": tune4["option_warps"],
                                   "fp32_ms_by_option_warps": tune4["fp32_ms_by_option_warps"]}}
        if not args.no_cpu and rank == 0:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import kwor

            idx = np.linspace(0, len(o4) - 1, 256).astype(int)
            rc4, msg4, want4, _ = kwor.fd1d_price(o4[idx], t_dim=2048, x_dim=2048, scale=SCALE, density=0.25)
            if rc4 != 0:
                raise RuntimeError(msg4)
            fine["fd64_max_rel_err_vs_oracle"] = float(np.max(np.abs(p64_[idx] - want4) / np.abs(want4)))
            fine["oracle_sample"] = len(idx)

    # ---------------------------------------------------------------- precision, 128 options, 512 x 512 (sinh grid)
    small = {}
    if rank == 0:
        o1 = portfolio.american_portfolio(128, seed=42)
        kw1 = dict(t_dim=512, x_dim=512, scale=SCALE, density=0.25)
        rc1, p1_64, s1_64 = ctx.fd1d_price(o1, kwg.params(**kw1))
        rc2, p1_32, s1_32 = ctx.fd1d_price(o1, kwg.params(precision=kwg.FP32, **kw1))
        if rc1 != 0 or rc2 != 0:
            raise RuntimeError(ctx.last_error())
        ok1 = (s1_64 == 0) & (s1_32 == 0)
        small = {"options": len(o1), "x_dim": 512, "t_dim": 512, "density": 0.25, "scale": SCALE,
                 "fd32_max_abs_err_vs_fd64": float(np.abs(p1_32[ok1] - p1_64[ok1]).max()), "failed": int((~ok1).sum())}
        if not args.no_cpu:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import kwor

            rc3, msg3, want1, _ = kwor.fd1d_price(o1, **kw1)
            if rc3 != 0:
                raise RuntimeError(msg3)
            small["fd64_max_rel_err_vs_oracle"] = float(np.max(np.abs(p1_64[ok1] - want1[ok1]) / np.abs(want1[ok1])))
            small["fd32_max_abs_err_vs_oracle"] = float(np.abs(p1_32[ok1] - want1[ok1]).max())

    tuned = {"fp64": tune64, "fp32": tune32, "uneven_131072": uneven.pop("tuning", None)}

    if ws > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return
    fp64_peak = fp64_peak_tflops(dev)

    # ---------------------------------------------------------------- roofline (solve kernel)
    # achieved: the algorithmic bytes of the streaming two-sweep scheme, 32 B per
    # node-step in FP64 (V read and written, the sweep value written and read back),
    # over the solve kernel's CUDA-event time.  The kernel's own count of the bytes it
    # requests (payoff and, outside the frozen middle region, coefficients on top) is
    # reported beside it as achieved_requested.
    hbm, peak_src = peaks()
    per_launch_s = solve_ms / 1e3 / max(solve_n, 1)
    ns = node_steps(n_loc)
    algo_bytes = ALGO_BYTES_PER_NODE_STEP * ns
    achieved = algo_bytes / per_launch_s / 1e9
    req_bytes = solve_bytes / max(solve_n, 1)
    achieved_req = req_bytes / per_launch_s / 1e9
    fp64_tflops = FP64_FLOPS_PER_NODE_STEP * ns / per_launch_s / 1e12
    traffic = measured_traffic(ns)

    # ---------------------------------------------------------------- CPU baseline and FP64 parity
    # the oracle prices of the CPU-baseline sample are the parity check of the whole
    # resident run (the first n options of the batch)
    if not args.no_cpu:
        cpu_rate, cpu_threads, cpu_n, cpu_s, cpu_want = cpu_oracle_rate(opts)
        err, nerr = max_rel(gpu_prices[:cpu_n], cpu_want), cpu_n
    else:
        cpu_rate, cpu_threads, cpu_n, cpu_s = None, 0, 0, 0.0
        err, nerr = None, 0
    if err is not None and err > 1e-10:
        raise RuntimeError(f"FP64 parity broken: max rel err {err:.3e} > 1e-10 on {nerr} options")

    line = {
        "metric": "options_per_sec_fd64_1024x1024",
        "value": value,
        "unit": "options/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": args.scaling,
        "vs_baseline": value / REF_PUBLISHED_OPS,
        "dtype": "f64",
        "data": "synthetic (seeded splitmix64; American, S=100, K~U[80,120], vol~U[0.1,0.6], r,q~U[0,0.1], T~U[0.25,2])",
        "config": workload_config(),
        "launch": {"solver": tune64["solver"], "block_warps": tune64["block_warps"],
                   "sm_blocks": tune64["sm_blocks"], "chosen_by": "kwg_autotune_ex on this shape"},
        "e2e": {"value": e2e_value, "unit": "options/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": {"bound": "hbm", "kernel": "fd1d_solve_fp64", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo_bytes,
                     "algorithmic_bytes_per_node_step": ALGO_BYTES_PER_NODE_STEP,
                     "basis": "32 B per node-step (V read + write, sweep value write + read), FP64 streaming scheme",
                     "achieved_requested": achieved_req, "frac_requested": achieved_req / hbm,
                     "requested_bytes_per_node_step": req_bytes / ns,
                     "requested_basis": "bytes the kernel itself requests (state 32 B + payoff 8 B where nonzero "
                                        "+ coefficients 24 B outside the frozen middle region), counted in the kernel",
                     "traffic_per_node_step": traffic / ns if traffic else None,
                     "node_steps_per_launch": ns, "launch_ms": per_launch_s * 1e3,
                     "fp64_tflops": fp64_tflops, "fp64_peak_tflops": fp64_peak,
                     "fp64_frac": fp64_tflops / fp64_peak if fp64_peak else None,
                     "fp64_peak_source": "measured here: cuBLAS DGEMM 4096^3"},
        "cpu_baseline": ({"value": cpu_rate, "unit": "options/s", "cores": cpu_threads, "kind": "port",
                          "sample": f"{cpu_n} options of the batch at 1024x1024 ({cpu_s:.1f} s), oracle C "
                                    f"restatement, {cpu_threads} threads"} if cpu_rate else None),
        "variants": {"fd64": {"options_per_sec": value, "max_rel_err_vs_oracle": err,
                              "oracle_sample": nerr,
                              "oracle_sample_is": "the CPU-baseline sample: the first n options of the batch"},
                     "fd32": {"options_per_sec": value32, "ms_per_step": ms32 / args.steps,
                              "solve_ms": solve32_ms / max(solve32_n, 1),
                              "speedup_vs_fd64": value32 / value,
                              "max_abs_err_vs_fd64": float(err32.max()),
                              "p99_abs_err_vs_fd64": float(np.percentile(err32, 99)),
                              "gpu_launches_per_step": launches32},
                     "uneven_131072": dict(uneven, workload="131072 options, per-option x_dim in "
                                            "{128..2048} by vol*sqrt(T), t_dim=clamp(ceil(512 sqrt(T)),64,2048), "
                                            "uniform grids, scale 5; kwg_fd1d_price_uneven (host API, CUDA graph)"),
                     "fd1d_bs_32768x1024": fd1d_bs,
                     "precision_65536x2048": fine,
                     "precision_128x512": small,
                     "autotune": tuned,
                     "surrogate_1m": surrogate},
    }
    print(json.dumps(line), flush=True)


def relaunch(n: int) -> int:
    """--gpus N without a launcher: run this script as N ranks, one process per GPU,
    through torch.distributed.run on this node (rendezvous on 127.0.0.1)."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-options", type=int, default=256, help="options per reference step")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="weak: every rank prices its own batch (default); strong: the ranks split one batch")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-batch (131072 options) variant")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate (1M options) variant")
    ap.add_argument("--no-fine-study", action="store_true", help="skip the 65536-option 2048x2048 precision study")
    ap.add_argument("--surrogate-options", type=int, default=SURROGATE_OPTIONS)
    ap.add_argument("--surrogate-train", type=int, default=2_000_000,
                    help="options to label and train the surrogate on in this run (0: load the committed weights)")
    ap.add_argument("--options", type=int, default=N_OPTIONS,
                    help="options per batch (default 32768; smaller values are for profiling captures)")
    ap.add_argument("--t-dim", type=int, default=T_DIM,
                    help="time steps (default 1024; shorter runs are for profiling captures)")
    args = ap.parse_args()
    globals()["N_OPTIONS"] = args.options
    globals()["T_DIM"] = args.t_dim
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch(args.gpus))
    ws = dist_env()[0]
    if ws != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={ws}; reporting the {ws} ranks that run",
              file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
