"""Vanishing volatility: the reference's exact threshold answers
(crates/kiyosi/tests/monte_carlo_thresholds.rs:27-209).

With r = q = 0, spot 100 and sigma = 1e-18 or 1e-200, every spot stays within an ulp of
100, so a barrier, knock-out or knock-in level at 100 is decided by the sign of the
path's sub-ulp log return alone.  The reference compares log returns with log-space
thresholds, so half of the paths fall on each side and the prices are exact halves
(antithetic pairs make them exact to rounding).  The oracle and the GPU's FP64 kernels
restate those comparisons.  FP32 cannot carry such plans (a diffusion of 1e-200
underflows, a daily quantity of 1e200 overflows): kgpu_price_book refuses FP32 for them
and the engines price those contracts with the FP64 kernels.

Times: the reference's dates are 2025-01-01 / 2026-01-01 (365 days, one year), and the
one-day notes run 2025-01-01 00:00 to 2025-01-02 00:00 valued at 12:00 (half a day
before expiry, half a day after the effective time).
"""
import math

import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.errors import UnsupportedOperationError
from kiyosi_gb300.instruments import (Accumulator, AutocallableNote, BarrierOption,
                                      DoubleBarrierOption, Observation)
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from oracle import loader

from helpers import gpu_price, pack, settings

VOLS = (1e-18, 1e-200)
HALF_DAY = 0.5 / 365.0


def context(volatility):
    return PricingContext(BlackScholesMertonParameters(0.0, 0.0, volatility), 100.0)


def _ncdf(x):
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


def barrier_cases():
    """(option, expected price): scheduled single and double barriers observed once at
    expiry, rebate 2 at expiry; exactly half of the paths touch, so 6.0."""
    out = []
    for option_type, strike in (("call", 90.0), ("put", 110.0)):
        for kind, lower, upper in (("up_and_in", 80.0, 100.0), ("up_and_out", 80.0, 100.0),
                                   ("down_and_in", 100.0, 120.0), ("down_and_out", 100.0, 120.0)):
            out.append(BarrierOption(option_type, strike, 1.0, barrier=100.0, barrier_type=kind,
                                     rebate=2.0, observation_times=[1.0]))
            double = "knock_in" if kind.endswith("_in") else "knock_out"
            out.append(DoubleBarrierOption(option_type, strike, 1.0, lower=lower, upper=upper,
                                           barrier_type=double, rebate=2.0, observation_times=[1.0]))
    return out


def binary_snowball():
    return AutocallableNote(initial_spot=100.0, expiry=1.0, maturity_coupon_rate=0.02,
                            observations=[Observation(1.0, knock_out_level=100.0, coupon_rate=0.12)])


def one_day_notes():
    """(note, expected): ternary snowballs (knock-in 100 daily or at expiry, coupons 0.12
    / 0.02) pay 1 + 0.07/365; the Phoenix note (coupon barrier 100, coupon 0.12) 1.06."""
    obs = [Observation(HALF_DAY, knock_out_level=120.0, coupon_rate=0.0)]
    out = []
    for times in ([-HALF_DAY, HALF_DAY], None):
        out.append((AutocallableNote(initial_spot=100.0, expiry=HALF_DAY, effective_time=-HALF_DAY,
                                     observations=obs, knock_in_level=100.0, knock_in_times=times,
                                     maturity_coupon_rate=0.12, fixed_knock_in_coupon=0.02,
                                     barrier_state="no_event"), 1.0 + 0.07 / 365.0))
    phoenix = AutocallableNote(initial_spot=100.0, expiry=HALF_DAY, effective_time=-HALF_DAY,
                               observations=[Observation(HALF_DAY, knock_out_level=120.0,
                                                         coupon_barrier_level=100.0)],
                               knock_in_level=80.0, upper_strike=100.0, lower_strike=100.0,
                               period_coupon=0.12)
    out.append((phoenix, 1.06))
    return out


def accumulators(volatility):
    """(option, expected, relative tolerance): knock-out at 100 with one unit held
    settles 10 or accumulates to 20, so 15; a daily quantity of 1/sigma with
    acceleration 2 is minus the analytic at-the-money vanilla over sigma (2%)."""
    out = []
    for option_type, strike, barrier in (("call", 90.0, 120.0), ("put", 110.0, 80.0)):
        out.append((Accumulator(option_type, strike, 100.0, HALF_DAY, accumulation_times=[HALF_DAY],
                                knock_out_times=[HALF_DAY], daily_quantity=1.0, acceleration=1.0,
                                quantity=1.0), 15.0, None))
        # The at-the-money vanilla as sigma -> 0: 100 sigma sqrt(t) phi(0), for either side.
        vanilla = 100.0 * volatility * math.sqrt(HALF_DAY) / math.sqrt(2.0 * math.pi)
        out.append((Accumulator(option_type, 100.0, barrier, HALF_DAY, accumulation_times=[HALF_DAY],
                                knock_out_times=[HALF_DAY], daily_quantity=1.0 / volatility,
                                acceleration=2.0, quantity=0.0), -vanilla / volatility, 0.02))
    return out


def all_cases(volatility):
    """(plan, expected, tolerance kind) of every case at one volatility; antithetic."""
    ctx = context(volatility)
    cases = [(plans.barrier(o, ctx), 6.0, None) for o in barrier_cases()]
    cases += [(plans.autocallable(n, ctx), v, None) for n, v in one_day_notes()]
    cases += [(plans.accumulator(o, ctx), v, tol) for o, v, tol in accumulators(volatility)]
    return ctx, cases


def _check(cases, estimates):
    for (plan, expected, tol), e in zip(cases, estimates):
        if tol is None:
            assert abs(e.price - expected) < 1e-12, (e.price, expected)
        else:
            assert abs(e.price - expected) < tol * abs(expected), (e.price, expected)


@pytest.mark.parametrize("volatility", VOLS)
def test_thresholds_on_the_oracle(volatility):
    ctx, cases = all_cases(volatility)
    priced = [(c, i) for i, c in enumerate(cases) if not isinstance(c[0], plans.Known)]
    assert len(priced) == len(cases)
    est = loader.price_book(ctx, pack([c[0] for c in cases]), settings(65536, 42, antithetic=True))
    _check(cases, est)


@pytest.mark.parametrize("volatility", VOLS)
def test_binary_snowball_thresholds_on_the_oracle(volatility):
    ctx = context(volatility)
    packed = pack([plans.autocallable(binary_snowball(), ctx)])
    plain = loader.price_book(ctx, packed, settings(65536, 42))[0]
    assert abs(plain.price - 1.07) < 4.0 * plain.standard_error
    assert abs(plain.standard_error - 0.05 / 256.0) < 1e-6
    paired = loader.price_book(ctx, packed, settings(65536, 42, antithetic=True))[0]
    assert abs(paired.price - 1.07) < 1e-12
    assert abs_status(paired) == "zero_observed_variance"


def abs_status(e):
    return abi.UNCERTAINTY_NAMES[e.uncertainty_status]


@pytest.mark.gpu
@pytest.mark.parametrize("volatility", VOLS)
def test_thresholds_on_gpu(native, volatility):
    ctx, cases = all_cases(volatility)
    packed = pack([c[0] for c in cases] + [plans.autocallable(binary_snowball(), ctx)])
    s = settings(65536, 42, antithetic=True)
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= 1e-12 * max(1.0, abs(r.price)), (g.price, r.price)
        assert g.uncertainty_status == r.uncertainty_status
    _check(cases, got)
    # Non-antithetic binary snowball: the standard error of a fair coin between 1.02 and 1.12.
    one = pack([plans.autocallable(binary_snowball(), ctx)])
    g = gpu_price(native, ctx, one, settings(65536, 42))[0]
    assert abs(g.standard_error - 0.05 / 256.0) < 1e-6
    assert abs(g.price - 1.07) < 4.0 * g.standard_error


@pytest.mark.gpu
def test_fp32_refuses_plans_it_cannot_represent(native):
    from kiyosi_gb300.pricing import MonteCarloAccumulatorEngine, MonteCarloAutocallableEngine
    ctx = context(1e-200)
    packed = pack([plans.autocallable(binary_snowball(), ctx)])
    for schedule in ("plain", "persistent"):
        with pytest.raises(UnsupportedOperationError):
            gpu_price(native, ctx, packed, settings(65536, 42, precision="fp32", schedule=schedule))
    # The engines price such contracts with the FP64 kernels instead.
    fp64 = MonteCarloAutocallableEngine(path_count=65536, seed=42, antithetic=True)
    fp32 = MonteCarloAutocallableEngine(path_count=65536, seed=42, antithetic=True, precision="fp32")
    note, expected = one_day_notes()[0]
    assert fp32.price(note, ctx) == fp64.price(note, ctx)
    acc, expected, tol = accumulators(1e-18)[1]
    engine = MonteCarloAccumulatorEngine(path_count=65536, seed=42, precision="fp32",
                                         schedule="persistent")
    assert abs(engine.price(acc, context(1e-18)) - expected) < tol * abs(expected)


def test_fp32_rule_keeps_ordinary_plans_and_refuses_vanishing_ones():
    from kiyosi_gb300 import workloads
    from kiyosi_gb300.instruments import EuropeanOption
    ordinary = [(workloads.c2_context(), plans.autocallable(workloads.snowball_c2(), workloads.c2_context())),
                (workloads.heston_context(), plans.asian(workloads.heston_asian_c3(), workloads.heston_context(), None)),
                (workloads.bsm(), plans.european(EuropeanOption("call", 100.0, 1.0), workloads.bsm()))]
    lv_ctx = PricingContext(workloads.lv_surface(), 100.0)
    notes, _ = workloads.lv_book(64)
    ordinary += [(lv_ctx, plans.autocallable(n, lv_ctx)) for n in notes]
    for ctx, plan in ordinary:
        assert plans.fp32_representable(plan, ctx)
    for volatility in VOLS:
        ctx = context(volatility)
        assert not plans.fp32_representable(plans.autocallable(binary_snowball(), ctx), ctx)
