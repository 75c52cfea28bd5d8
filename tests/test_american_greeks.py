"""CPU: the American Greeks' host logic (lsmc.american_greeks) with the GPU pricer
replaced by a smooth function of the scenario, so the stencils, the 8%-of-spot default
bump, the time stencil and the call's rate-shortcut boundary are checked without a
device (american.rs:555-557, 1487-1687)."""
import math

import pytest

from kiyosi_gb300 import lsmc
from kiyosi_gb300.errors import UnsupportedOperationError
from kiyosi_gb300.greeks import symmetric_shift
from kiyosi_gb300.instruments import AmericanOption
from kiyosi_gb300.market import BlackScholesMertonParameters, HestonParameters, PricingContext
from kiyosi_gb300.pricing import MonteCarloVanillaEngine


def _value(ctx, expiry=1.0):
    m = ctx.model
    return (0.1 * ctx.spot ** 2 / 100.0 + 3.0 * m.volatility ** 2 - 7.0 * m.rate + 2.0 * m.dividend
            + 0.5 * ctx.spot * m.volatility + 4.0 * expiry + 0.01 * ctx.spot * expiry)


@pytest.fixture
def calls(monkeypatch):
    seen = []

    def fake(engine, option, contexts, seed, shortcut=True):
        seen.append((len(contexts), shortcut, seed))
        return [_value(c, option.expiry) for c in contexts]
    monkeypatch.setattr(lsmc, "price_american_scenarios", fake)
    return seen


def test_put_greeks_follow_the_stencils(calls):
    engine = MonteCarloVanillaEngine(path_count=1024, step_count=10, seed=5)
    ctx = PricingContext(BlackScholesMertonParameters(0.05, 0.02, 0.2), 100.0)
    res = engine.price_with_greeks(AmericanOption("put", 100.0, 1.0), ctx,
                                   ["delta", "gamma", "vega", "rho", "dividend_rho", "theta", "charm"])
    h = symmetric_shift(100.0, 8.0)  # 8% of spot
    v = symmetric_shift(0.2, 1e-4)

    def at(spot=100.0, vol=0.2, rate=0.05, div=0.02):
        return _value(PricingContext(BlackScholesMertonParameters(rate, div, vol), spot))
    p0 = at()
    assert res.price == p0
    assert res.greeks["delta"] == (at(spot=100.0 + h) - at(spot=100.0 - h)) / h / 2.0
    assert res.greeks["gamma"] == ((at(spot=100.0 + h) - p0) - (p0 - at(spot=100.0 - h))) / h / h
    assert res.greeks["vega"] == (at(vol=0.2 + v) - at(vol=0.2 - v)) / (2.0 * v)
    assert math.isclose(res.greeks["rho"], -7.0, rel_tol=1e-6)
    assert math.isclose(res.greeks["dividend_rho"], 2.0, rel_tol=1e-6)
    # The stencil is one day each way (no valuation start); the fake's time terms give
    # theta -(4 + 0.01 S) and charm -0.01.
    assert math.isclose(res.greeks["theta"], -5.0, rel_tol=1e-9)
    assert math.isclose(res.greeks["charm"], -0.01, rel_tol=1e-6)
    # One batch per instant (valuation, a day later, a day earlier), on the engine's seed.
    assert len(calls) == 3 and all(c[1] and c[2] == 5 for c in calls)


def test_call_rho_crossing_the_no_early_exercise_boundary(calls):
    """A call with no dividend at a zero rate: the rho stencil crosses r = 0, so both legs
    are priced on the exercise grid (shortcut off), as american.rs:1606-1656 does."""
    engine = MonteCarloVanillaEngine(path_count=1024, step_count=10, seed=5)
    ctx = PricingContext(BlackScholesMertonParameters(0.0, 0.0, 0.2), 100.0)
    res = engine.price_with_greeks(AmericanOption("call", 100.0, 1.0), ctx, ["rho", "dividend_rho"])
    assert math.isclose(res.greeks["rho"], -7.0, rel_tol=1e-6)
    assert [c[1] for c in calls] == [True, False, False]


def test_american_greeks_need_bsm():
    engine = MonteCarloVanillaEngine(path_count=1024, step_count=10, seed=5)
    ctx = PricingContext(HestonParameters(0.03, 0.0, 0.04, 2.0, 0.04, 0.5, -0.7), 100.0)
    with pytest.raises(UnsupportedOperationError):
        engine.price_with_greeks(AmericanOption("put", 100.0, 1.0), ctx, ["delta"])


def test_greeks_at_expiry_use_the_terminal_payoff(calls):
    engine = MonteCarloVanillaEngine(path_count=1024, step_count=10, seed=5)
    ctx = PricingContext(BlackScholesMertonParameters(0.05, 0.02, 0.2), 90.0)
    res = engine.price_with_greeks(AmericanOption("put", 100.0, 0.0), ctx, ["delta", "vega"])
    assert res.price == 10.0 and res.greeks["vega"] == 0.0
    assert res.greeks["delta"] == -1.0
    assert not calls
