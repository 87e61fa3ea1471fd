"""Failure detection without a GPU fault.

* The bounded waits every kernel uses give up and report, and the context stays
  usable: a self-test kernel waits on an mbarrier that nothing arrives on.
* Host-injected faults become per-option statuses (NaN price + code) while the rest
  of the batch prices normally; strict mode turns the first one into the call's
  error, like the reference's whole-batch failure (src/Pricer/kwFd1d.cpp:154-155).
  The injected degenerate factorisation (vol = 1e200, finite, but sigma^2 overflows:
  the operator's rows and so the LU pivots are not finite) has no reference
  counterpart; the reference would silently price garbage (src/Math/kwFd1d.cpp:46-48
  only prints solver errors).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(ctx):
    import kwg
    import portfolio

    assert ctx.selftest_waits() == (1, 1)
    o = portfolio.american_portfolio(64, seed=3)
    rc, p, st = ctx.fd1d_price(o, kwg.params(t_dim=64, x_dim=64, scale=5.0))
    assert rc == kwg.KWG_OK and (st == 0).all() and np.isfinite(p).all()


@pytest.mark.parametrize("precision,solver", [(0, 1), (0, 2), (1, 0)], ids=["fp64-thomas", "fp64-pcr", "fp32"])
def test_degenerate_factorisation_is_a_per_option_status(ctx, precision, solver):
    import kwg
    import portfolio

    o = portfolio.american_portfolio(100, seed=4)
    bad = o.copy()
    bad["z"][[7, 50]] = 1e200
    prm = kwg.params(t_dim=64, x_dim=128, scale=5.0, precision=precision, solver=solver)
    rc, want, st0 = ctx.fd1d_price(o, prm)
    assert rc == 0 and (st0 == 0).all()
    rc, got, st = ctx.fd1d_price(bad, prm)
    assert rc == kwg.KWG_OK
    assert st[7] == kwg.STATUS_SOLVER and st[50] == kwg.STATUS_SOLVER
    assert np.isnan(got[[7, 50]]).all()
    keep = np.ones(len(o), bool)
    keep[[7, 50]] = False
    assert (st[keep] == 0).all()
    assert np.array_equal(got[keep], want[keep])
    prm.strict = 1
    rc, _, _ = ctx.fd1d_price(bad, prm)
    assert rc == kwg.KWG_ERR_SOLVER
    assert "asset 7" in ctx.last_error()
