"""Autocallable pins held by the reference, restated on the oracle (CPU) and the GPU.

* crates/kiyosi/tests/autocallable_monte_carlo.rs:226-253: a binary snowball that only
  observes at expiry is the discounted principal plus a cash-or-nothing digital; the
  Monte Carlo price (32,768 paths, seed 42) lies within 4 standard errors of that, and
  the 95% interval is 2 x 1.959963984540054 standard errors wide (to 1e-14).
* crates/kiyosi/tests/snowball.rs:35-58: valued at expiry, the note settles to its
  exact payment -- knock-in is strict, knock-out inclusive.
* instruments/autocallable/pricing.rs:12-69 (`initial`, `expiry_payment`): knocked-out
  notes settle at 0, knocked-in history and a spot below the level on a monitoring
  date at valuation take the knocked-in redemption, an observation at valuation fixes
  its coupon and settles a knock-out.

The GPU twins price the same plans through the C ABI: FP64 within 1e-12 relative of
the oracle, FP32 within half a standard error.
"""
import math

import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.errors import InvalidInputError, MissingHistoryError
from kiyosi_gb300.instruments import AutocallableNote, Observation
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from kiyosi_gb300.pricing import MonteCarloAutocallableEngine
from oracle import loader

from helpers import compare_gpu_oracle, pack, settings

Z95 = 1.959963984540054


def _ncdf(x):
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


def _market(spot=100.0):
    # market() of the reference tests: r = 0.04, q = 0.01, sigma = 0.3
    return PricingContext(BlackScholesMertonParameters(0.04, 0.01, 0.3), spot)


def _bsm_terms(ctx, strike, t):
    m = ctx.model
    sd = m.volatility * math.sqrt(t)
    d1 = (math.log(ctx.spot / strike) + (m.rate - m.dividend) * t) / sd + 0.5 * sd
    return d1, d1 - sd


def _binary_snowball():
    """BinarySnowballTerms::new(0.0, 2025-01-01, 2026-01-01, [(2026-01-01, 100, 0.1)]):
    365 days = 1 year on Actual/365 Fixed, no knock-in, zero maturity coupon."""
    return AutocallableNote(initial_spot=100.0, expiry=1.0,
                            observations=[Observation(1.0, knock_out_level=100.0, coupon_rate=0.1)])


def _binary_expected(ctx):
    _, d2 = _bsm_terms(ctx, 100.0, 1.0)
    return math.exp(-0.04) + 0.1 * math.exp(-0.04) * _ncdf(d2)


def _estimate(e):
    return e.price, e.standard_error if e.uncertainty_status == 0 else None, e.sample_error


@pytest.mark.parametrize("sobol", [False, True])
def test_binary_snowball_matches_discounted_principal_plus_digital(sobol):
    ctx = _market()
    packed = pack([plans.autocallable(_binary_snowball(), ctx)])
    s = settings(32768, 42, sobol=sobol)
    price, se, sample_error = _estimate(loader.price_book(ctx, packed, s)[0])
    expected = _binary_expected(ctx)
    # Sobol estimates carry no standard error (MonteCarloUncertaintyStatus::UnsupportedSampling);
    # the i.i.d. sample error bounds them from above.
    error = se if not sobol else sample_error
    assert abs(price - expected) < 4.0 * error, (price, expected, error)
    if not sobol:
        lower, upper = price - Z95 * se, price + Z95 * se
        assert abs(upper - lower - 2.0 * Z95 * se) < 1e-14


def _at_expiry_snowball(coupon=0.08):
    """snowball.rs terms valued at expiry: effective 2025-01-01, expiry 2025-04-01 (90
    days earlier than valuation), knock-out 110 at expiry with coupon 0.08, knock-in 80
    at expiry, strikes 100 / 60, maturity coupon 0.06, no event so far."""
    return AutocallableNote(initial_spot=100.0, expiry=0.0, effective_time=-90.0 / 365.0,
                            observations=[Observation(0.0, knock_out_level=110.0, coupon_rate=coupon)],
                            knock_in_level=80.0, upper_strike=100.0, lower_strike=60.0,
                            maturity_coupon_rate=0.06, barrier_state="no_event")


def test_valuation_at_expiry_settles_strict_knock_in_and_inclusive_knock_out():
    term = 90.0 / 365.0
    note = _at_expiry_snowball()
    engine = MonteCarloAutocallableEngine(path_count=4096, seed=1)
    for spot, expected in ((60.0, 0.6), (70.0, 0.7), (80.0, 1.0 + 0.06 * term),
                           (110.0, 1.0 + 0.08 * term)):
        ctx = _market(spot)
        plan = plans.autocallable(note, ctx)
        assert isinstance(plan, plans.Known)
        assert abs(plan.value - expected) < 1e-14
        assert abs(engine.price(note, ctx) - expected) < 1e-14


def test_history_is_checked_against_the_schedule():
    past_ko = [Observation(-0.1, knock_out_level=103.0, coupon_rate=0.1),
               Observation(0.5, knock_out_level=103.0, coupon_rate=0.1)]
    base = dict(initial_spot=100.0, expiry=0.5, effective_time=-0.2, knock_in_level=80.0,
                upper_strike=100.0, maturity_coupon_rate=0.1)
    ctx = _market()
    with pytest.raises(MissingHistoryError):
        plans.autocallable(AutocallableNote(observations=past_ko, **base), ctx)
    future = [Observation(0.5, knock_out_level=103.0, coupon_rate=0.1)]
    with pytest.raises(InvalidInputError, match="knock-out predates"):
        plans.autocallable(AutocallableNote(observations=future, barrier_state="knocked_out", **base), ctx)
    with pytest.raises(InvalidInputError, match="knock-in predates"):
        plans.autocallable(AutocallableNote(observations=future, barrier_state="knocked_in", **base), ctx)
    with pytest.raises(InvalidInputError, match="outside contract life"):
        AutocallableNote(initial_spot=100.0, expiry=0.5, effective_time=0.1, observations=future)
    # Past daily monitoring also needs the history.
    daily = [-0.1, 0.0, 0.25, 0.5]
    with pytest.raises(MissingHistoryError):
        plans.autocallable(AutocallableNote(observations=future, knock_in_times=daily, **base), ctx)
    # A knocked-out note settles at zero.
    knocked_out = AutocallableNote(observations=past_ko, barrier_state="knocked_out", **base)
    assert plans.autocallable(knocked_out, ctx).value == 0.0


def _seasoned_downside(state, spot_ki_check=False):
    """A seasoned snowball with no knock-out left: principal plus the capped downside,
    (min(S, 100) - 100) / 100 at expiry once knocked in."""
    times = [-0.25 + 0.25 * i / 63 for i in range(63)] + [0.5 * (i + 1) / 126 for i in range(126)]
    if spot_ki_check:
        times = [t for t in times if t < 0.0] + [0.0] + [t for t in times if t > 0.0]
    return AutocallableNote(initial_spot=100.0, expiry=0.5, effective_time=-0.25,
                            observations=[Observation(-0.2, knock_out_level=120.0, coupon_rate=0.1)],
                            knock_in_level=80.0, knock_in_times=times, upper_strike=100.0,
                            lower_strike=0.0, maturity_coupon_rate=0.1, barrier_state=state)


def _knocked_in_price(ctx, t=0.5):
    """exp(-r t) - put(K = 100) / 100 under BSM."""
    m = ctx.model
    d1, d2 = _bsm_terms(ctx, 100.0, t)
    put = 100.0 * math.exp(-m.rate * t) * _ncdf(-d2) - ctx.spot * math.exp(-m.dividend * t) * _ncdf(-d1)
    return math.exp(-m.rate * t) - put / 100.0


def _seasoned_cases():
    """(context, note, analytic price or None) of the seasoned cases."""
    high = _market(100.0)
    low = _market(79.0)
    phoenix = AutocallableNote(
        initial_spot=100.0, expiry=0.5, effective_time=-0.5, period_coupon=0.02,
        observations=[Observation(-0.25, knock_out_level=105.0, coupon_barrier_level=90.0),
                      Observation(0.0, knock_out_level=105.0, coupon_barrier_level=90.0),
                      Observation(0.25, knock_out_level=105.0, coupon_barrier_level=90.0),
                      Observation(0.5, knock_out_level=105.0, coupon_barrier_level=90.0)],
        knock_in_level=70.0, upper_strike=100.0, lower_strike=0.0, barrier_state="no_event")
    return [
        (high, _seasoned_downside("knocked_in"), _knocked_in_price(high)),
        (low, _seasoned_downside("no_event", spot_ki_check=True), _knocked_in_price(low)),
        (_market(95.0), phoenix, None),
    ]


def test_seasoned_plans_carry_the_valuation_state():
    (hi, ki_note, _), (lo, below_note, _), (mid, phoenix, _) = _seasoned_cases()
    for ctx, note in ((hi, ki_note), (lo, below_note)):
        plan = plans.autocallable(note, ctx)
        assert plan.contract[0]["flags"] & abi.C_KNOCKED_IN
        assert not plan.contract[0]["flags"] & abi.C_BRIDGE  # no daily grid once knocked in
        assert len(plan.steps) == 1  # expiry only: monitoring no longer matters
    plan = plans.autocallable(phoenix, mid)
    assert plan.contract[0]["initial_cash"] == 0.02  # coupon at valuation, undiscounted
    assert len(plan.events) == 2  # the valuation-date observation is settled, not stepped
    # Spot at the knock-out level on the valuation date settles the note.
    settled = plans.autocallable(phoenix, _market(105.0))
    assert settled.value == phoenix.knock_out_payment(phoenix.observations[1]) + 0.02


def test_seasoned_prices_on_the_oracle():
    for ctx, note, expected in _seasoned_cases():
        packed = pack([plans.autocallable(note, ctx)])
        e = loader.price_book(ctx, packed, settings(1 << 16, 42))[0]
        if expected is not None:
            assert abs(e.price - expected) < 4.0 * e.standard_error, (e.price, expected)
    # The coupon fixed at valuation adds to the price of the same note without it, on
    # the same random numbers.
    ctx, phoenix, _ = _seasoned_cases()[2]
    without = AutocallableNote(**{**phoenix.__dict__,
                                  "observations": [o for o in phoenix.observations if o.time != 0.0]})
    s = settings(1 << 14, 5)
    a = loader.price_book(ctx, pack([plans.autocallable(phoenix, ctx)]), s)[0].price
    b = loader.price_book(ctx, pack([plans.autocallable(without, ctx)]), s)[0].price
    assert abs(a - (b + 0.02)) < 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("sobol", [False, True])
def test_binary_snowball_pin_on_gpu(native, sobol):
    ctx = _market()
    packed = pack([plans.autocallable(_binary_snowball(), ctx)])
    s = settings(32768, 42, sobol=sobol)
    ref, got = compare_gpu_oracle(native, ctx, packed, s)
    error = got[0].standard_error if not sobol else got[0].sample_error
    assert abs(got[0].price - _binary_expected(ctx)) < 4.0 * error


@pytest.mark.gpu
def test_seasoned_notes_on_gpu(native):
    for ctx, note, expected in _seasoned_cases():
        packed = pack([plans.autocallable(note, ctx)])
        ref, got = compare_gpu_oracle(native, ctx, packed, settings(1 << 16, 42))
        if expected is not None:
            assert abs(got[0].price - expected) < 4.0 * got[0].standard_error
