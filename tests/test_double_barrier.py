"""Double barriers (barrier.rs:231-452 with an upper level; double_barrier.rs:6-112).

CPU checks of the oracle:
- kiyosi's independent continuous knock-out prices
  (crates/kiyosi/tests/double_barrier_monte_carlo.rs:121-157: call 1.0838814592583166,
  put 1.5760435147766145, within 0.003 at 32,768 Sobol paths for seeds 17, 42, 103).
  The conditional survival weight makes the estimate land within 1e-6;
- continuity where the survival sum switches from the image series to the spectral
  series (the volatilities of double_barrier_monte_carlo.rs:232-278), and extreme bands;
- the scheduled cases of double_barrier_monte_carlo.rs:352-403 against a
  transition-density quadrature (the reference uses a finite-difference engine, within
  0.04);
- host resolution rules.

GPU checks: the CUDA path against the oracle on the same random numbers.
"""
import math

import pytest

from kiyosi_gb300 import abi, analytic, plans
from kiyosi_gb300.errors import InvalidInputError, UnsupportedOperationError
from kiyosi_gb300.instruments import DoubleBarrierOption
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from oracle import loader

from barrier_quadrature import scheduled_barrier_value
from helpers import gpu_price, pack, settings


def _market(sigma=0.2):
    """double_barrier_monte_carlo.rs:20-28."""
    return PricingContext(BlackScholesMertonParameters(0.04, 0.01, sigma), 100.0)


def _option(kind="call", **kw):
    base = dict(lower=80.0, upper=120.0, barrier_type="knock_out")
    base.update(kw)
    return DoubleBarrierOption(kind, 100.0, 1.0, **base)


def _oracle(ctx, options, paths, seed, **kw):
    return loader.price_book(ctx, pack([plans.barrier(o, ctx) for o in options]),
                             settings(paths, seed, **kw))


@pytest.mark.parametrize("kind,reference", [("call", 1.0838814592583166), ("put", 1.5760435147766145)])
def test_continuous_knock_out_matches_independent_reference(kind, reference):
    ctx = _market()
    plan = plans.barrier(_option(kind), ctx)
    assert plan.record["payoff"] == abi.PAYOFF_DOUBLE_BARRIER
    for seed in (17, 42, 103):
        (e,) = _oracle(ctx, [_option(kind)], 32768, seed, sobol=True)
        assert abs(e.price - reference) < 0.003
        assert abs(e.price - reference) < 1e-6, (seed, e.price)


def test_image_and_spectral_series_agree_at_the_switch():
    """variance (sigma / log 1.5)^2 crosses 0.25 between the first two volatilities."""
    band = math.log(1.5)
    low, high, wide = 0.20273255202675663, 0.20273255608140772, 0.3040988310811233
    assert (low / band) ** 2 < 0.25 <= (high / band) ** 2
    a, = _oracle(_market(low), [_option()], 65536, 42)
    b, = _oracle(_market(high), [_option()], 65536, 42)
    assert abs(a.price - b.price) < 1e-6
    c, = _oracle(_market(wide), [_option()], 65536, 42)
    assert 0.0 < c.price < a.price
    narrow, = _oracle(_market(), [_option(lower=99.99, upper=100.01)], 65536, 42)
    assert narrow.price == 0.0
    wide_band, = _oracle(_market(), [_option(lower=0.01, upper=10000.0)], 65536, 42)
    vanilla = analytic.european_price(1.0, 100.0, 1.0, _market())
    assert abs(wide_band.price - vanilla) < 3.0 * wide_band.standard_error


@pytest.mark.parametrize("kind", ["call", "put"])
@pytest.mark.parametrize("barrier_type,timing", [("knock_out", "at_expiry"), ("knock_out", "at_hit"),
                                                 ("knock_in", "at_expiry")])
@pytest.mark.parametrize("final", [False, True])
def test_scheduled_double_matches_quadrature(kind, barrier_type, timing, final):
    """One observation on 2025-06-30, optionally plus expiry, rebate 2; 65,536 Sobol
    paths with seed 42, the reference test's engine."""
    ctx = _market()
    dates = [180.0 / 365.0] + ([1.0] if final else [])
    option = _option(kind, barrier_type=barrier_type, rebate=2.0, rebate_timing=timing,
                     observation_times=dates)
    plan = plans.barrier(option, ctx)
    assert plan.record["flags"] & abi.C_DOUBLE
    (e,) = _oracle(ctx, [option], 65536, 42, sobol=True)
    expected = scheduled_barrier_value(ctx, option.sign, 100.0, 1.0, dates, 80.0, 120.0,
                                       barrier_type == "knock_in", 2.0, timing == "at_hit")
    assert abs(e.price - expected) < 0.04
    assert abs(e.price - expected) < 0.005, (e.price, expected)


def test_double_resolution_and_validation():
    ctx = _market()
    # Spot outside the band: a knock-out pays its rebate, a knock-in is the vanilla.
    out = plans.barrier(_option(lower=100.0, rebate=1.5), ctx)
    assert out.value == 1.5 * math.exp(-0.04)
    touched_in = plans.barrier(_option(upper=100.0, barrier_type="knock_in"), ctx)
    assert touched_in.value == analytic.european_price(1.0, 100.0, 1.0, ctx)
    # A call struck at or above the upper barrier needs a touch to pay: a knock-out is
    # worthless without a rebate.
    assert plans.barrier(DoubleBarrierOption("call", 130.0, 1.0, lower=80.0, upper=120.0), ctx).value == 0.0
    # ... unless its last observation is before expiry.
    early = DoubleBarrierOption("call", 130.0, 1.0, lower=80.0, upper=120.0, observation_times=[0.25])
    (e,) = _oracle(ctx, [early], 1 << 15, 42)
    assert e.price > 0.01
    with pytest.raises(InvalidInputError):
        _option(lower=120.0, upper=80.0)
    with pytest.raises(InvalidInputError):
        _option(barrier_type="knock_in", rebate=1.0, rebate_timing="at_hit")
    with pytest.raises(UnsupportedOperationError):
        plans.barrier(_option(rebate=1.0, rebate_timing="at_hit"), ctx)


@pytest.mark.gpu
@pytest.mark.parametrize("sobol", [False, True])
def test_double_barrier_gpu_parity(native, sobol):
    ctx = PricingContext(BlackScholesMertonParameters(0.03, 0.01, 0.3), 100.0)
    monthly = [i / 12 for i in range(1, 13)]
    options = [_option("call"), _option("put", rebate=1.0),
               _option("call", barrier_type="knock_in", rebate=0.5),
               DoubleBarrierOption("put", 100.0, 2.0, lower=60.0, upper=150.0),  # spectral series
               _option("call", observation_times=monthly, rebate=1.0, rebate_timing="at_hit"),
               _option("put", barrier_type="knock_in", observation_times=[i / 52 for i in range(1, 50)])]
    packed = pack([plans.barrier(o, ctx) for o in options])
    s = settings(1 << 14, 13, sobol=sobol)
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= 1e-12 * max(1.0, abs(r.price)), (g.price, r.price)
    for schedule in ("plain", "persistent"):
        got32 = gpu_price(native, ctx, packed, settings(1 << 14, 13, sobol=sobol, precision="fp32",
                                                        schedule=schedule))
        for r, g in zip(ref, got32):
            se = max(r.sample_error, 1e-4 * abs(r.price))
            assert abs(g.price - r.price) <= 0.5 * se, (schedule, g.price, r.price)
