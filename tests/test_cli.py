"""The `kwinto price` command-line flow (src/kwinto.cpp:15-120): option parsing, the
portfolio CSV, the pricer factory and the statistics report.  The CPU tests plug the
oracle in as the pricer; the GPU test runs the real one."""
import io
import os

import numpy as np
import pytest

from conftest import golden

COLS = ("exercise", "strike", "dividend_rate", "interest_rate", "spot", "expiry", "price", "parity", "volatility")


def write_csv(path, opts, prices):
    with open(path, "w") as f:
        f.write(",".join(COLS) + "\n")
        for o, p in zip(opts, prices):
            f.write(",".join([
                "a" if o["e"] else "e", repr(float(o["k"])), repr(float(o["q"])), repr(float(o["r"])),
                repr(float(o["s"])), repr(float(o["t"])), repr(float(p)), "c" if o["w"] > 0 else "p",
                repr(float(o["z"]))]) + "\n")


class OracleFactory:
    """PricerFactory stand-in that prices with the oracle (CPU), keyed like the reference."""

    last_config = None

    @staticmethod
    def create(config):
        import kwg
        import kwor

        OracleFactory.last_config = config
        mode = config.get("PRICER", "")
        if mode not in ("FD1D", "FD1D-BS"):
            return f"PricerFactory: Unknown PRICER = {mode}", None
        kw = dict(t_dim=config.get("FD1D.T_GRID_SIZE", 512), x_dim=config.get("FD1D.X_GRID_SIZE", 512),
                  scale=config.get("FD1D.SCALE", 50.0), density=config.get("FD1D.DENSITY", 0.25))

        class P(kwg.Pricer):
            def price(self, assets, prices):
                rc, msg, p, _ = kwor.fd1d_price(kwg.to_array(assets), bs=(mode == "FD1D-BS"), **kw)
                prices[:] = list(p)
                return "" if rc == 0 else msg

        return "", P()


def run(argv, factory=OracleFactory):
    import kwinto

    out = io.StringIO()
    rc = kwinto.main(argv, out=out, factory=factory)
    return rc, out.getvalue()


def test_price_report_matches_the_statistics(tmp_path, capsys):
    import kwor
    import portfolio

    g = golden("pricer_test.npz")
    path = str(tmp_path / "p.csv")
    write_csv(path, g["opts"], g["want"])
    rc, text = run(["price", path, "-t", "128", "-x", "128"])
    assert rc == 0, capsys.readouterr().err
    assert "    Assets : 12" in text and "Price Statistics" in text
    cfg = OracleFactory.last_config
    assert cfg.get("PRICER", "") == "FD1D-BS" and cfg.get("FD1D.DENSITY", 0.0) == 0.25
    assert cfg.get("FD1D.SCALE", 0.0) == 50.0 and cfg.get("FD1D.T_GRID_SIZE", 0) == 128
    rc2, msg, p, _ = kwor.fd1d_price(g["opts"], bs=True, t_dim=128, x_dim=128, scale=50.0, density=0.25)
    st = portfolio.price_stats(g["opts"], g["want"], p)
    assert f"        MAE : {st['mae']:e}" in text
    assert f"       RMSE : {st['rmse']:e}" in text
    assert f"      total : {st['total']} options" in text


def test_option_string_follows_the_reference():
    import kwinto

    g = golden("pricer_test.npz")
    s = kwinto.option_string(g["opts"][0])
    assert s.startswith("<Option e=") and s.endswith(">") and " w=" in s and " z=" in s


def test_errors(tmp_path, capsys):
    g = golden("pricer_test.npz")
    path = str(tmp_path / "p.csv")
    write_csv(path, g["opts"], g["want"])
    assert run(["price", path, "--density", "abc"])[0] == 1
    assert "Fail to parse '--density <num>'" in capsys.readouterr().err
    assert run(["price", path, "-p", "NOPE"])[0] == 1
    assert "Unknown PRICER = NOPE" in capsys.readouterr().err
    bad = str(tmp_path / "bad.csv")
    open(bad, "w").write("expiry,spot\n1,2\n")
    assert run(["price", bad])[0] == 1
    assert "Some option data is missing" in capsys.readouterr().err


@pytest.mark.gpu
def test_cli_on_the_gpu(tmp_path, built):
    """The QuantLib portfolio (6000 American puts) through the real GPU pricers at the
    reference defaults: within the reference test's 0.005 of QuantLib."""
    import kwg
    import portfolio

    g = golden("portfolio_qdfp.npz")
    path = str(tmp_path / "qdfp.csv")
    write_csv(path, g["opts"], g["quantlib"])
    for pricer in ("FD1D", "FD1D-BS"):
        rc, text = run(["price", path, "-p", pricer], factory=kwg.PricerFactory)
        assert rc == 0
        mae = float([ln for ln in text.splitlines() if ln.strip().startswith("MAE :")][0].split(":")[1])
        assert mae <= 0.005
