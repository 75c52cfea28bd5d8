"""Native delta and gamma of the digital, barrier and Asian engines: each path's
likelihood-ratio or pathwise sample, averaged like the price.

CPU checks of the oracle:
- kiyosi's independent continuous double-barrier deltas and gammas
  (crates/kiyosi/tests/double_barrier_monte_carlo.rs:121-157: the reference allows
  0.003; the oracle lands within 1e-7);
- digital likelihood-ratio Greeks against the closed forms;
- scheduled-barrier and average-price Greeks against finite differences of the
  quadrature or of common-random-number prices.

GPU checks: the CUDA samples against the oracle's on the same random numbers.
"""
import math

import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.instruments import (ArithmeticAveragePriceOption, BarrierOption, DigitalOption,
                                      DoubleBarrierOption, GeometricAveragePriceOption)
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from oracle import loader

from barrier_quadrature import scheduled_barrier_value
from helpers import gpu_price, pack, settings


def _ctx(spot=100.0, vol=0.2, rate=0.04, dividend=0.01):
    return PricingContext(BlackScholesMertonParameters(rate, dividend, vol), spot)


def _triple(ctx, plan, paths, seed, **kw):
    """(price, delta, gamma) of one plan, the three priced in one book."""
    book = pack([plan, plans.greek_output(plan, "delta"), plans.greek_output(plan, "gamma")])
    return tuple(e.price for e in loader.price_book(ctx, book, settings(paths, seed, **kw)))


@pytest.mark.parametrize("kind,delta,gamma", [
    ("call", -0.009437716341942348, -0.006614552070516311),
    ("put", -0.031725540191196444, -0.008683048910995694)])
def test_double_barrier_likelihood_greeks_match_reference(kind, delta, gamma):
    ctx = _ctx()
    option = DoubleBarrierOption(kind, 100.0, 1.0, lower=80.0, upper=120.0)
    for seed in (17, 42, 103):
        _, d, g = _triple(ctx, plans.barrier(option, ctx), 32768, seed, sobol=True)
        assert abs(d - delta) < 0.003 and abs(g - gamma) < 0.003
        # The survival weight's derivatives carry almost all of the estimate.
        assert abs(d - delta) < 1e-7 and abs(g - gamma) < 1e-8, (seed, d, g)


def test_digital_likelihood_greeks_near_closed_forms():
    ctx = _ctx(100.0, 0.25, 0.05, 0.02)
    t = 1.0
    sq = 0.25 * math.sqrt(t)
    d1 = (math.log(100.0 / 105.0) + (0.05 - 0.02 + 0.5 * 0.25 ** 2) * t) / sq
    d2 = d1 - sq
    pdf = math.exp(-0.5 * d2 * d2) / math.sqrt(2 * math.pi)
    delta = 10.0 * math.exp(-0.05 * t) * pdf / (100.0 * sq)
    gamma = -10.0 * math.exp(-0.05 * t) * pdf * d1 / (100.0 ** 2 * sq * sq)
    option = DigitalOption("call", 105.0, t, payout=10.0)
    _, d, g = _triple(ctx, plans.digital(option, ctx), 1 << 18, 42)
    assert abs(d - delta) < 0.01 * abs(delta) + 2e-3, (d, delta)
    assert abs(g - gamma) < 0.05 * abs(gamma) + 5e-4, (g, gamma)


def test_continuous_single_barrier_greeks_match_bumped_prices():
    """The likelihood-ratio delta against a wide central difference of common-random-
    number prices (the conditional survival weight makes both smooth in the spot)."""
    option = BarrierOption("call", 100.0, 1.0, barrier=85.0, barrier_type="down_and_out", rebate=1.0)
    ctx = _ctx()
    _, d, g = _triple(ctx, plans.barrier(option, ctx), 1 << 17, 7)
    h = 0.5
    up = _triple(_ctx(100.0 + h), plans.barrier(option, _ctx(100.0 + h)), 1 << 17, 7)[0]
    down = _triple(_ctx(100.0 - h), plans.barrier(option, _ctx(100.0 - h)), 1 << 17, 7)[0]
    mid = _triple(ctx, plans.barrier(option, ctx), 1 << 17, 7)[0]
    assert abs(d - (up - down) / (2 * h)) < 0.02, (d, (up - down) / (2 * h))
    assert abs(g - (up - 2 * mid + down) / (h * h)) < 0.01


def test_scheduled_barrier_greeks_match_quadrature_differences():
    """The scheduled double barrier of double_barrier_monte_carlo.rs:352-403 (one date
    plus expiry, knock-out, rebate 2 at expiry): delta within 0.025 and gamma within
    0.01 of the quadrature's central differences, the reference's bars."""
    dates = [180.0 / 365.0, 1.0]
    option = DoubleBarrierOption("call", 100.0, 1.0, lower=80.0, upper=120.0, rebate=2.0,
                                 observation_times=dates)
    ctx = _ctx()
    _, d, g = _triple(ctx, plans.barrier(option, ctx), 65536, 42, sobol=True)
    h = 0.5
    q = lambda s: scheduled_barrier_value(_ctx(s), 1.0, 100.0, 1.0, dates, 80.0, 120.0, False, 2.0)  # noqa: E731
    qd = (q(100.0 + h) - q(100.0 - h)) / (2 * h)
    qg = (q(100.0 + h) - 2 * q(100.0) + q(100.0 - h)) / (h * h)
    assert abs(d - qd) < 0.025, (d, qd)
    assert abs(g - qg) < 0.01, (g, qg)


@pytest.mark.parametrize("option", [
    GeometricAveragePriceOption("call", 100.0, 1.0),
    ArithmeticAveragePriceOption("call", 100.0, 1.0),
    ArithmeticAveragePriceOption("put", 104.0, 1.0, averaging_start=0.25)])
def test_average_native_greeks_match_bumped_prices(option):
    """Pathwise delta and gamma against a central difference of common-random-number
    prices (with the control's exact delta and gamma added back for arithmetic ones)."""
    ctx = _ctx()
    plan = plans.average(option, ctx, 50)
    book = pack([plan, plans.greek_output(plan, "delta"), plans.greek_output(plan, "gamma")])
    _, d, g = (e.price for e in loader.price_book(ctx, book, settings(1 << 16, 3)))
    h = 0.5
    price = lambda s: loader.price_book(_ctx(s), pack([plans.average(option, _ctx(s), 50)]),  # noqa: E731
                                        settings(1 << 16, 3))[0].price
    up, mid, down = price(100.0 + h), price(100.0), price(100.0 - h)
    assert abs(d - (up - down) / (2 * h)) < 0.01, (d, (up - down) / (2 * h))
    assert abs(g - (up - 2 * mid + down) / (h * h)) < 0.005, (g, (up - 2 * mid + down) / (h * h))


@pytest.mark.gpu
@pytest.mark.parametrize("sobol", [False, True])
def test_native_greek_samples_gpu_parity(native, sobol):
    ctx = PricingContext(BlackScholesMertonParameters(0.03, 0.01, 0.3), 100.0)
    options = [DigitalOption("put", 95.0, 1.0, payout=5.0),
               BarrierOption("call", 100.0, 1.0, barrier=80.0, barrier_type="down_and_out", rebate=1.0),
               BarrierOption("put", 100.0, 1.0, barrier=120.0, barrier_type="up_and_in",
                             observation_times=[i / 12 for i in range(1, 13)]),
               DoubleBarrierOption("call", 100.0, 1.0, lower=75.0, upper=130.0),
               ArithmeticAveragePriceOption("call", 100.0, 1.0),
               GeometricAveragePriceOption("put", 100.0, 1.0)]
    base = []
    for o in options:
        p = (plans.digital(o, ctx) if isinstance(o, DigitalOption) else
             plans.average(o, ctx, 32) if isinstance(o, (ArithmeticAveragePriceOption,
                                                         GeometricAveragePriceOption))
             else plans.barrier(o, ctx))
        base += [plans.greek_output(p, "delta"), plans.greek_output(p, "gamma")]
    packed = pack(base)
    s = settings(1 << 14, 29, sobol=sobol)
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= 1e-11 * max(1.0, abs(r.price)), (g.price, r.price)
    got32 = gpu_price(native, ctx, packed, settings(1 << 14, 29, sobol=sobol, precision="fp32",
                                                    schedule="persistent"))
    for r, g in zip(ref, got32):
        assert abs(g.price - r.price) <= 0.5 * max(r.sample_error, 1e-4 * abs(r.price)), (g.price, r.price)
