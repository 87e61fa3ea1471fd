"""kwinto -- command-line pricing of a portfolio CSV on the GPU.

Mirrors `kwinto price` (src/kwinto.cpp:15-120) without docopt: the same options and
defaults, the same flow (Portfolio::load -> PricerFactory -> Pricer::price ->
Portfolio::printPricesStats, src/Utils/kwPortfolio.cpp:13-163) and the same report.
"FD1D" and "FD1D-BS" (the default, as in the reference) run on the GPU through
libkwg.so; two options are added for the GPU path: --precision and --device.

    python kwinto-cuda_gb300/kwinto.py price [options] <path>

As in the reference, -e is parsed and checked but the statistics skip options whose
reference price is below 0.5 (Portfolio::printPricesStats does not take -e).
"""
from __future__ import annotations

import argparse
import math
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

VERSION = "kwinto-cuda GB300 (sm_103a)"
STATS_TOLERANCE = 0.5  # src/Utils/kwPortfolio.cpp:109


def option_string(o) -> str:
    """Option::asString (src/Core/kwAsset.h:29-43): std::to_string prints %f."""
    return (f"<Option e={'amer' if o['e'] else 'euro'} k={o['k']:f} q={o['q']:f} r={o['r']:f} s={o['s']:f} "
            f"t={o['t']:f} w={'Call' if o['w'] > 0 else 'Put'} z={o['z']:f}>")


def parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="kwinto", description="kwinto - Options Pricing Analytics")
    ap.add_argument("--version", action="version", version=VERSION)
    sub = ap.add_subparsers(dest="command", required=True)
    p = sub.add_parser("price", help="price the options of a CSV file")
    p.add_argument("path", help="CSV file with options data")
    p.add_argument("--density", default="0.25", help="Density of the x-grid distribution [default: 0.25]")
    p.add_argument("--scale", default="50.0", help="Scale of the x-grid distribution [default: 50.0]")
    p.add_argument("-e", default="0.5", help="Reject option prices less than <num> from RRMS error stats")
    p.add_argument("-p", default="FD1D-BS", help="Pricer name [default: FD1D-BS]")
    p.add_argument("-t", type=int, default=512, help="Use <num> points for t-grid [default: 512]")
    p.add_argument("-x", type=int, default=512, help="Use <num> points for x-grid [default: 512]")
    p.add_argument("-v", action="store_true", help="Show extra details, be verbose")
    p.add_argument("--precision", default="FP64", choices=["FP64", "FP32"], help="GPU arithmetic [default: FP64]")
    p.add_argument("--device", type=int, default=0, help="CUDA device [default: 0]")
    return ap


def _number(text: str, what: str) -> float:
    try:
        return float(text)
    except ValueError:
        raise ValueError(f"cmdPrice: Fail to parse '{what}': {text!r} is not a number") from None


def cmd_price(args, out, factory=None) -> str:
    """Returns "" or the error message, like the reference's cmdPrice."""
    import kwg
    import portfolio

    factory = factory or kwg.PricerFactory
    try:
        density = _number(args.density, "--density <num>")
        scale = _number(args.scale, "--scale <num>")
        _number(args.e, "-e <num>")
    except ValueError as ex:
        return str(ex)
    config = kwg.Config()
    config.set("PRICER", args.p)
    config.set("FD1D.DENSITY", density)
    config.set("FD1D.SCALE", scale)
    config.set("FD1D.T_GRID_SIZE", int(args.t))
    config.set("FD1D.X_GRID_SIZE", int(args.x))
    config.set("FD1D.PRECISION", args.precision)
    config.set("FD1D.DEVICE", int(args.device))
    try:
        assets, want = portfolio.load_csv(args.path)
    except (OSError, ValueError) as ex:
        return f"cmdPrice: {ex}"
    print("Portfolio", file=out)
    print(f"    Assets : {len(assets)}", file=out)
    print("", file=out)
    err, pricer = factory.create(config)
    if err:
        return f"cmdPrice: Portfolio::price : {err}"
    prices = [0.0] * len(assets)
    err = pricer.price(assets, prices)
    if err:
        return f"cmdPrice: Portfolio::price : {err}"
    import numpy as np

    st = portfolio.price_stats(assets, want, np.asarray(prices), tolerance=STATS_TOLERANCE)
    print("Price Statistics", file=out)
    if st["total"]:
        print(f"       RMSE : {st['rmse']:e}", file=out)
        print(f"      RRMSE : {st['rrmse']:e}", file=out)
        print(f"        MAE : {st['mae']:e}", file=out)
        print(f"        MRE : {st['mre']:e}", file=out)
        print(f"  MAE Asset : {option_string(assets[st['mae_index']])}", file=out)
        print(f"  MRE Asset : {option_string(assets[st['mre_index']])}", file=out)
    else:  # the reference divides by zero here and prints nan
        for name in ("RMSE", "RRMSE"):
            print(f"{name:>11} : {math.nan}", file=out)
    print(f"      total : {st['total']} options", file=out)
    print("", file=out)
    return ""


def main(argv=None, out=sys.stdout, factory=None) -> int:
    args = parser().parse_args(argv)
    print(VERSION + "\n", file=out)
    if args.v:
        print("Command-Line Arguments", file=out)
        for k, v in sorted(vars(args).items()):
            print(f"    {k}: {v}", file=out)
        print("", file=out)
    err = cmd_price(args, out, factory) if args.command == "price" else ""
    if err:
        print(err, file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
