"""Host-side logic and the C-ABI library surface; no GPU needed."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "kwg.h")).read()
    return sorted(set(re.findall(r"\b(kwg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    import kwg

    declared = _declared_symbols()
    assert "kwg_fd1d_price" in declared and "kwg_create" in declared
    L = ctypes.CDLL(kwg.LIB_PATH)
    for name in declared:
        assert hasattr(L, name), f"libkwg.so does not export {name}"
    out = subprocess.run(["nm", "-D", "--defined-only", kwg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (kwg_[a-z0-9_]+)$", out, re.M))
    assert set(declared) <= exported


def test_option_layout_matches_kw_option():
    import kwg

    assert kwg.OPTION_DTYPE.itemsize == 56
    assert kwg.OPTION_DTYPE.fields["e"][1] == 48 and kwg.OPTION_DTYPE.fields["w"][1] == 49


def test_ctypes_mirrors_match_the_header(tmp_path):
    """Size and every field offset of the structs in include/kwg.h, from a C program
    compiled against the header, equal those of the ctypes mirrors in kwg.py."""
    import kwg

    structs = {"kwg_option": None, "kwg_fd1d_params": kwg.Fd1dParams, "kwg_tuning": kwg.Tuning,
               "kwg_audit": kwg.Audit}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "kwg.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} size %zu\\n", sizeof({name}));')
        fields = [f[0] for f in cls._fields_] if cls else list(kwg.OPTION_DTYPE.names)
        for f in fields:
            lines.append(f'printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for name, cls in structs.items():
        if cls is None:
            assert got[(name, "size")] == kwg.OPTION_DTYPE.itemsize
            for f in kwg.OPTION_DTYPE.names:
                assert got[(name, f)] == kwg.OPTION_DTYPE.fields[f][1], (name, f)
            continue
        assert got[(name, "size")] == ctypes.sizeof(cls), name
        for f in cls._fields_:
            assert got[(name, f[0])] == getattr(cls, f[0]).offset, (name, f[0])


def _canonical(a2p):
    """Group labels renumbered by first occurrence, so equal partitions compare equal."""
    first = {}
    return np.array([first.setdefault(int(g), len(first)) for g in a2p])


def test_dedup_matches_the_oracle(built):
    """The hash-table dedup every pricing call uses groups options exactly as the
    oracle's restatement of the reference's sort (src/Pricer/kwFd1d.cpp:28-65):
    repeated keys, keys that differ only in spot or strike, and +0.0 / -0.0 rates."""
    import sys

    import kwg
    import portfolio

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import kwor

    rng = np.random.default_rng(1)
    o = portfolio.american_portfolio(3000, seed=8)
    dup = o[rng.integers(0, len(o), 2000)]
    dup["s"][:500] *= 1.1
    dup["k"][500:1000] *= 0.9
    zp = o[:10].copy()
    zp["r"] = 0.0
    zm = zp.copy()
    zm["r"] = -0.0
    o = np.concatenate([o, dup, zp, zm])
    o = o[rng.permutation(len(o))]
    a2p, p2a = kwg.dedup(o)
    ra2p, rp2a = kwor.dedup(o)
    assert len(p2a) == len(rp2a) < len(o)
    assert np.array_equal(_canonical(a2p), _canonical(ra2p))
    assert (a2p[p2a] == np.arange(len(p2a))).all()  # each PDE's first option maps to it
    assert (np.diff(p2a.astype(np.int64)) > 0).all()  # PDEs numbered by first option


def test_dedup_nan_keys_and_grid_shapes(built):
    """A NaN field matches nothing (the reference's sort would merge such a key with
    a neighbour); with per-option grid shapes, equal keys on different grids are
    different PDEs."""
    import kwg
    import portfolio

    o = portfolio.american_portfolio(4, seed=3)
    o = np.concatenate([o, o])
    o["z"][[1, 5]] = np.nan
    a2p, p2a = kwg.dedup(o)
    assert a2p[0] == a2p[4] and a2p[2] == a2p[6] and a2p[3] == a2p[7]
    assert a2p[1] != a2p[5] and len(p2a) == 5
    xd = np.array([128] * 4 + [256] * 4, np.int32)
    td = np.full(8, 64, np.int32)
    a2p2, p2a2 = kwg.dedup(o, xd, td)
    assert len(p2a2) == 8 and len(set(a2p2.tolist())) == 8
    assert kwg.dedup(o[:0])[1].size == 0


def test_params_default_is_reference_default(built):
    import kwg

    p = kwg.default_params()
    assert (p.t_dim, p.x_dim, p.theta, p.scale, p.density) == (512, 512, 0.5, 50.0, 0.25)
    assert (p.precision, p.solver, p.strict) == (kwg.FP64, kwg.SOLVER_AUTO, 0)


def test_create_without_gpu_fails_cleanly(built):
    import torch

    import kwg

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        kwg.Context(0)
    assert kwg.lib().kwg_create(0) is None


def test_config_typed_maps():
    """kw::Config (src/Core/kwConfig.h:21-73): a key set as double is not visible
    through an integer default and vice versa."""
    import kwg

    c = kwg.Config()
    c.set("FD1D.T_GRID_SIZE", 1024)
    c.set("FD1D.DENSITY", 1.5)
    c.set("PRICER", "FD1D")
    assert c.get("FD1D.T_GRID_SIZE", 512) == 1024
    assert c.get("FD1D.T_GRID_SIZE", 512.0) == 512.0
    assert c.get("FD1D.DENSITY", 0.25) == 1.5
    assert c.get("PRICER", "") == "FD1D"
    c.erase("PRICER")
    assert c.get("PRICER", "") == ""


def test_factory_errors():
    """kw::PricerFactory::create (src/Pricer/kwPricerFactory.h:15-41) messages."""
    import kwg

    c = kwg.Config()
    err, p = kwg.PricerFactory.create(c)
    assert err == "PricerFactory: Missing PRICER key" and p is None
    c.set("PRICER", "NOPE")
    err, p = kwg.PricerFactory.create(c)
    assert err == "PricerFactory: Unknown PRICER = NOPE"


def test_portfolio_generator_is_deterministic_and_in_range():
    import portfolio

    a = portfolio.american_portfolio(1000, seed=42)
    b = portfolio.american_portfolio(1000, seed=42)
    assert a.tobytes() == b.tobytes()
    # a window of the stream equals the same slice of the full stream
    c = portfolio.american_portfolio(100, seed=42, start=500)
    assert c.tobytes() == a[500:600].tobytes()
    assert (a["k"] >= 80).all() and (a["k"] < 120).all()
    assert (a["z"] >= 0.1).all() and (a["z"] < 0.6).all()
    assert (a["t"] >= 0.25).all() and (a["t"] < 2.0).all()
    assert (a["w"] == -1).sum() == 500 and (a["e"] == 1).all()
    u = portfolio.uniforms(7, 3, 200000)
    assert abs(u.mean() - 0.5) < 5e-3 and u.min() >= 0 and u.max() < 1


def test_uneven_buckets():
    import portfolio

    o, xd, td = portfolio.uneven_portfolio(20000, seed=42)
    assert set(np.unique(xd)) <= {128, 256, 512, 1024, 2048}
    assert td.min() >= 64 and td.max() <= 2048
    assert (o["t"] >= 1 / 52 - 1e-12).all() and (o["t"] <= 5 + 1e-12).all()


def test_csv_loader_and_stats():
    """Portfolio::load / printPricesStats (src/Utils/kwPortfolio.cpp:13-163)."""
    import portfolio

    text = ("expiry,spot,strike,volatility,interest_rate,dividend_rate,parity,exercise,price\n"
            "1,100,100,0.2,0.05,0,p,a,6.09\n"
            "0.5,90,100,0.3,0.02,0.01,c,e,3.5\n"
            "0.5,90,100,0.3,0.02,0.01,c,e,0.2\n")
    o, p = portfolio.load_csv(text, is_text=True)
    assert len(o) == 3 and o[0]["e"] == 1 and o[0]["w"] == -1 and o[1]["w"] == 1 and o[1]["e"] == 0
    assert o[1]["s"] == 90 and o[1]["t"] == 0.5 and p[0] == 6.09
    got = p + np.array([0.01, -0.03, 5.0])
    st = portfolio.price_stats(o, p, got)
    assert st["total"] == 2  # the 0.2 price is below the 0.5 filter
    assert st["mae"] == pytest.approx(0.03) and st["mae_index"] == 1
    assert st["rmse"] == pytest.approx(0.01)  # std-dev of |err| {0.01, 0.03}
    with pytest.raises(ValueError, match="Some option data is missing"):
        portfolio.load_csv("expiry,spot\n1,2\n", is_text=True)


def test_golden_fixtures_are_consistent():
    g = golden("pricer_test.npz")
    assert g["opts"].shape == (12,) and np.max(np.abs(g["ref_fd1d"] - g["want"])) <= 1.3e-3
    q = golden("portfolio_qdfp.npz")
    assert len(q["opts"]) == 6000 and np.max(np.abs(q["ref_fd1d"] - q["quantlib"])) <= 0.005
