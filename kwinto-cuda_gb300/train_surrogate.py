"""Trains the MLP surrogate on the GPU and writes its weights.

Labels are FD64 prices the GPU solver generates (kwg_fd1d_price_device) for options
drawn from the 32768-option workload's distributions (S = 100, K ~ U[80, 120],
vol ~ U[0.1, 0.6], r, q ~ U[0, 0.1], T ~ U[0.25, 2], puts and calls alternating),
on the uniform 1024 x 1024 grid over +-5 sigma sqrt(T).  Training runs in the
library's tcgen05 forward/backward kernels (kwg_mlp_train).  The weights, the
training box and the held-out error (network vs FD64 on fresh options) go to an .npz
that kwg.Surrogate.load() reads.

    python kwinto-cuda_gb300/train_surrogate.py --n 2000000 --out kwinto-cuda_gb300/surrogate_weights.npz
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import kwg  # noqa: E402
import portfolio  # noqa: E402

TRAIN_SEED, TEST_SEED = 1001, 2002


def fd64_device(ctx, d_opts, n: int, grid: int, chunk: int = 262144):
    """FD64 prices of n device options (torch uint8 tensor of n * 56 bytes)."""
    import torch

    prices = torch.empty(n, dtype=torch.float64, device="cuda")
    status = torch.empty(n, dtype=torch.int32, device="cuda")
    p = kwg.params(t_dim=grid, x_dim=grid, scale=5.0, density=math.inf)
    p.strict = 0
    stream = torch.cuda.current_stream().cuda_stream
    for c0 in range(0, n, chunk):
        c = min(chunk, n - c0)
        rc = ctx.fd1d_price_device(d_opts.data_ptr() + c0 * kwg.OPTION_DTYPE.itemsize, c, p,
                                   prices.data_ptr() + 8 * c0, status.data_ptr() + 4 * c0, stream)
        if rc:
            raise RuntimeError(f"FD64 labels: {ctx.last_error()}")
    torch.cuda.synchronize()
    bad = int((status != 0).sum().item())
    if bad:
        raise RuntimeError(f"FD64 labels: {bad} options failed")
    return prices


def evaluate(net: kwg.Surrogate, ctx, n: int, grid: int, seed: int = TEST_SEED) -> dict:
    """Network prices vs FD64 on n fresh options."""
    import torch

    opts = portfolio.american_portfolio(n, seed=seed)
    d_o = torch.from_numpy(opts.view(np.uint8).copy()).cuda()
    fd = fd64_device(ctx, d_o, n, grid).cpu().numpy()
    d_p = torch.empty(n, dtype=torch.float64, device="cuda")
    net.price_device(d_o.data_ptr(), n, d_p.data_ptr())
    torch.cuda.synchronize()
    err = np.abs(d_p.cpu().numpy() - fd)
    return {"n": n, "max_abs": float(err.max()), "p99_abs": float(np.quantile(err, 0.99)),
            "p999_abs": float(np.quantile(err, 0.999)), "mean_abs": float(err.mean())}


def train(ctx, n: int = 2_000_000, grid: int = 1024, epochs: int = 150, batch: int = 4096, lr: float = 2e-3,
          seed: int = 1, test: int = 65536):
    """Labels n options with FD64 on the GPU, trains a fresh network on them and
    measures its held-out error on `test` fresh options: (network, metadata with the
    measured label and training times)."""
    import torch

    opts = portfolio.american_portfolio(n, seed=TRAIN_SEED)
    d_o = torch.from_numpy(opts.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d_p = fd64_device(ctx, d_o, n, grid)
    t_label = time.perf_counter() - t0
    net = kwg.Surrogate(ctx.device, seed=seed)
    t0 = time.perf_counter()
    loss = net.train(d_o.data_ptr(), d_p.data_ptr(), n, epochs, batch, lr, seed)
    t_train = time.perf_counter() - t0
    hist = net.train_history()
    report = evaluate(net, ctx, test, grid)
    meta = {"n_train": n, "grid": grid, "epochs": epochs, "batch": batch, "lr": lr, "seed": seed,
            "label_s": t_label, "train_s": t_train, "final_loss": loss, "kept_epoch": hist["best_epoch"],
            "spike_restarts": hist["restarts"], "last_epoch_loss": float(hist["losses"][-1]),
            "heldout": report}
    del d_o, d_p
    return net, meta


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--n", type=int, default=2_000_000, help="training options")
    ap.add_argument("--grid", type=int, default=1024, help="x_dim = t_dim of the FD64 labels")
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--test", type=int, default=65536, help="held-out options for the error report")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                  "surrogate_weights.npz"))
    a = ap.parse_args(argv)

    ctx = kwg.Context(0)
    net, meta = train(ctx, a.n, a.grid, a.epochs, a.batch, a.lr, a.seed, a.test)
    p, lo, hi, ys = net.get_params()
    np.savez(a.out, params=p, box_lo=lo, box_hi=hi, y_scale=np.float32(ys), meta=json.dumps(meta))
    print(json.dumps(meta))
    net.close()
    ctx.close()


if __name__ == "__main__":
    main()
