"""Structured notes under local volatility against the reference's QuantLib fixture.

The reference holds QuantLib 1.43 Monte Carlo prices of eight structured contracts under
a fixed local-volatility surface (python/tests/quantlib_reference/
local_volatility_structured.json, made by local_volatility_paths.py and read by
python/tests/test_local_volatility_structured.py).  The contracts: snowball, ternary and
Phoenix notes with daily or expiry-only knock-in, a binary snowball and an accumulator;
spot 101, r = 0.04, q = 0.01, 2025-01-01 to 2025-04-01 on a weekday calendar,
knock-out observations on Feb 3, Mar 3 and Apr 1 at 110 / 108 / 105, knock-in 95.
The surface: vols 0.32 / 0.24 / 0.16 at spots 60 / 100 / 160, the same at both
times, bilinear and clamped.  QuantLib steps log-Euler paths with 4 steps per calendar
day (360 steps on its TimeGrid of the trading dates), antithetic pairs and a put
control variate.

Here the same contracts are priced by this package's local-volatility Monte Carlo
(log-Euler with the surface read at each step's start, the same 360-step grid from
plans.refine_grid) and compared within K_SE combined standard errors plus twice the
fixture's own fine-minus-coarse time bias; a semantic error (a wrong coupon accrual,
strict/inclusive barrier, a missed observation) moves a price by 1e-3 or more, far
outside the band.
"""
import json
import math
import os
from datetime import date, timedelta

import pytest

from kiyosi_gb300 import plans
from kiyosi_gb300.instruments import Accumulator, AutocallableNote, Observation
from kiyosi_gb300.market import LocalVolatilitySurface, PricingContext
from oracle import loader

from helpers import gpu_price, pack, settings

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "local_volatility_structured.json")
START, END = date(2025, 1, 1), date(2025, 4, 1)
OBSERVATION_DAYS = ((date(2025, 2, 3) - START).days, (date(2025, 3, 3) - START).days, (END - START).days)
KNOCK_OUT = (110.0, 108.0, 105.0)
YEAR = 365.0
TIME_STEPS = 360  # 4 steps per calendar day over 90 days, the fixture's grid
K_SE = 4.0


def _fixture():
    return json.load(open(GOLDEN))


def market(spot=101.0):
    surface = LocalVolatilitySurface(0.04, 0.01, [0.0, 90.0 / YEAR], [60.0, 100.0, 160.0],
                                     [[0.32, 0.24, 0.16]] * 2)
    return PricingContext(surface, spot)


def trading_times():
    """Weekdays after the valuation date through expiry, as A/365F year fractions."""
    days = [d for d in range(1, (END - START).days + 1)
            if (START + timedelta(days=d)).weekday() < 5]
    return [d / YEAR for d in days]


def contracts():
    """The fixture's contracts in this package's terms.  The valuation instant
    (2025-01-01 00:00, a weekday) is itself a monitoring and accumulation date."""
    expiry = 90.0 / YEAR
    daily = [0.0] + trading_times()
    snow_obs = [Observation(d / YEAR, knock_out_level=k, coupon_rate=0.08)
                for d, k in zip(OBSERVATION_DAYS, KNOCK_OUT)]
    phoenix_obs = [Observation(d / YEAR, knock_out_level=k, coupon_barrier_level=95.0)
                   for d, k in zip(OBSERVATION_DAYS, KNOCK_OUT)]
    loss = dict(initial_spot=100.0, knock_in_level=95.0, upper_strike=100.0, lower_strike=60.0)
    out = {"accumulator": Accumulator("call", 100.0, 110.0, expiry, accumulation_times=daily,
                                      knock_out_times=daily, daily_quantity=1.0, acceleration=2.0,
                                      quantity=3.0)}
    for suffix, times in (("daily", daily), ("terminal", None)):
        out[f"snowball_{suffix}"] = AutocallableNote(expiry=expiry, observations=snow_obs,
                                                     knock_in_times=times, maturity_coupon_rate=0.06,
                                                     barrier_state="no_event", **loss)
        out[f"ternary_{suffix}"] = AutocallableNote(initial_spot=100.0, expiry=expiry,
                                                    observations=snow_obs, knock_in_level=95.0,
                                                    knock_in_times=times, maturity_coupon_rate=0.06,
                                                    fixed_knock_in_coupon=0.01,
                                                    barrier_state="no_event")
        out[f"phoenix_{suffix}"] = AutocallableNote(expiry=expiry, observations=phoenix_obs,
                                                    knock_in_times=times, period_coupon=0.08,
                                                    barrier_state="no_event", **loss)
    out["binary_snowball"] = AutocallableNote(initial_spot=100.0, expiry=expiry,
                                              observations=snow_obs, maturity_coupon_rate=0.06)
    return out


def book(ctx):
    names = list(contracts())
    plan_list = []
    for name in names:
        c = contracts()[name]
        if isinstance(c, Accumulator):
            plan_list.append(plans.accumulator(c, ctx, time_steps=TIME_STEPS))
        else:
            plan_list.append(plans.autocallable(c, ctx, time_steps=TIME_STEPS))
    return names, pack(plan_list)


def band(name, our_se):
    ref = _fixture()
    r = ref["reference"]["results"][name]
    bias = ref["time_refinement"]["results"][name]
    combined = math.sqrt(r["standard_error"] ** 2 + our_se ** 2)
    return (K_SE * combined + r["control_reference_error"]
            + 2.0 * (abs(bias["fine_minus_coarse"]) + K_SE * bias["standard_error"]))


def test_grid_is_the_fixture_time_grid():
    ctx = market()
    names, packed = book(ctx)
    for i, name in enumerate(names):
        assert packed.contracts[i]["step_count"] == TIME_STEPS, name
    refined = plans.refine_grid(trading_times(), TIME_STEPS)
    assert len(refined) == TIME_STEPS
    assert all(abs(b - a - 0.25 / YEAR) < 1e-15 for a, b in zip([0.0] + refined, refined))


def _check(names, estimates):
    ref = _fixture()["reference"]["results"]
    worst = 0.0
    for name, e in zip(names, estimates):
        limit = band(name, e.standard_error)
        err = abs(e.price - ref[name]["price"])
        assert err <= limit, (name, e.price, ref[name]["price"], err, limit)
        worst = max(worst, err / limit)
    return worst


def test_oracle_matches_quantlib_fixture():
    """2^16 antithetic pseudo-random paths on the CPU oracle."""
    ctx = market()
    names, packed = book(ctx)
    _check(names, loader.price_book(ctx, packed, settings(1 << 16, 2718, antithetic=True)))


@pytest.mark.gpu
def test_gpu_matches_quantlib_fixture_and_oracle(native):
    """2^22 paths on the GPU (FP64 and FP32) against the fixture; FP64 against the
    oracle on the same random numbers at 2^16 paths."""
    ctx = market()
    names, packed = book(ctx)
    s = settings(1 << 16, 2718, antithetic=True)
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= 1e-10 * max(1.0, abs(r.price)), (g.price, r.price)
    for precision, schedule in (("fp64", "plain"), ("fp32", "persistent")):
        big = settings(1 << 22, 2718, precision=precision, schedule=schedule)
        _check(names, gpu_price(native, ctx, packed, big))
