"""Continuously averaged price options: kiyosi's MonteCarloAsianEngine
(engines/monte_carlo/asian.rs).

CPU checks of the oracle against kiyosi's known answers:
- the conditioned first-interval integration converges to the values in kiyosi's test
  (crates/kiyosi/tests/asian_monte_carlo.rs:349-386, within 0.001);
- exact geometric sampling matches the closed-form geometric price
  (benchmarks/quantlib/references/digitals_asian.json) and ignores the step count
  (asian_monte_carlo.rs:227-263);
- arithmetic prices sit near the two-moment lognormal fit of the same reference file;
- the geometric control variate leaves the price within the sampling error and cuts
  the sample error several times over.

GPU checks: the CUDA path against the oracle on the same random numbers. FP64 must
match within 1e-12 relative, FP32 within 0.5 SE; price_strikes must replay scalar
prices.
"""
import math

import pytest

from kiyosi_gb300 import abi, analytic, plans
from kiyosi_gb300.errors import InvalidInputError, UnsupportedOperationError
from kiyosi_gb300.instruments import ArithmeticAveragePriceOption as Arithmetic
from kiyosi_gb300.instruments import GeometricAveragePriceOption as Geometric
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from oracle import loader

from helpers import gpu_price, pack, settings


def _ctx(spot=100.0, sigma=0.2, rate=0.04, dividend=0.01):
    return PricingContext(BlackScholesMertonParameters(rate, dividend, sigma), spot)


def _oracle(ctx, options, step_count, paths, seed, control=True, **kw):
    plan_list = [plans.average(o, ctx, step_count, control) for o in options]
    return loader.price_book(ctx, pack(plan_list), settings(paths, seed, **kw)), plan_list


@pytest.mark.parametrize("spot,expected", [(1.9, 0.193174), (2.0, 0.246416), (2.1, 0.306220)])
def test_conditioned_integration_converges(spot, expected):
    ctx = _ctx(spot, 0.5, 0.05, 0.0)
    option = Arithmetic("call", 2.0, 1.0)
    (fine,), _ = _oracle(ctx, [option], 64, 65536, 42, sobol=True, antithetic=True)
    (coarse,), _ = _oracle(ctx, [option], 2, 65536, 42, sobol=True, antithetic=True)
    assert abs(fine.price - expected) < 0.001, fine.price
    assert abs(fine.price - expected) < abs(coarse.price - expected)


def test_geometric_matches_closed_form_and_ignores_steps():
    """Reference file values: call S = K = 100; put S = 110, K = 105; r 4%, q 1%,
    sigma 20%, one year."""
    for option, ctx, reference in ((Geometric("call", 100.0, 1.0), _ctx(100.0), 5.035867546515377),
                                   (Geometric("put", 105.0, 1.0), _ctx(110.0), 2.3556936178500534)):
        (a,), (plan,) = _oracle(ctx, [option], 2, 16384, 42, sobol=True, antithetic=True)
        (b,), _ = _oracle(ctx, [option], 10000, 16384, 42, sobol=True, antithetic=True)
        assert plan.record["payoff"] == abi.PAYOFF_AVERAGE_GEOMETRIC
        assert abs(a.price - reference) < 0.01, a.price
        assert a.price == b.price


def test_single_fixing_is_the_european_option():
    """Averaging that starts at expiry is one fixing: the terminal spot's vanilla."""
    ctx = _ctx(100.0, 0.25, 0.03, 0.0)
    for kind in ("call", "put"):
        option = Arithmetic(kind, 95.0, 0.75, averaging_start=0.75)
        (e,), (plan,) = _oracle(ctx, [option], 50, 1 << 17, 9)
        assert plan.record["payoff"] == abi.PAYOFF_AVERAGE_GEOMETRIC
        reference = analytic.european_price(option.sign, 95.0, 0.75, ctx)
        assert abs(e.price - reference) < 4.0 * e.standard_error, (kind, e.price, reference)


def test_arithmetic_near_the_two_moment_fit():
    """The two-moment lognormal fit of the reference file is an approximation; the
    converged Monte Carlo price lies within 0.04 of it."""
    for option, ctx, fit in ((Arithmetic("call", 100.0, 1.0), _ctx(100.0), 5.246501860362811),
                             (Arithmetic("put", 105.0, 1.0), _ctx(110.0), 2.276320528271724)):
        (e,), (plan,) = _oracle(ctx, [option], 200, 1 << 16, 42)
        assert plan.record["flags"] & abi.C_AVERAGE_CONTROL
        assert abs(e.price - fit) < 0.04, (e.price, fit)


def test_control_variate_keeps_the_price_and_cuts_the_error():
    ctx = _ctx(100.0)
    option = Arithmetic("call", 100.0, 1.0)
    (with_control,), _ = _oracle(ctx, [option], 50, 1 << 16, 5)
    (plain,), (plan,) = _oracle(ctx, [option], 50, 1 << 16, 5, control=False)
    assert not plan.record["flags"] & abi.C_AVERAGE_CONTROL
    assert abs(with_control.price - plain.price) < 4.0 * plain.standard_error
    assert with_control.standard_error < plain.standard_error / 5.0


def test_lead_interval_and_far_strikes():
    """A forward start draws one more normal (the lead interval); strikes far from the
    money run without the control."""
    ctx = _ctx(100.0)
    lead = plans.average(Arithmetic("call", 100.0, 1.0, averaging_start=0.25), ctx, 50)
    assert lead.record["flags"] & abi.C_AVERAGE_LEAD and lead.record["step_count"] == 50
    far = plans.average(Arithmetic("call", 180.0, 1.0), ctx, 50)
    assert not far.record["flags"] & abi.C_AVERAGE_CONTROL and far.record["step_count"] == 49
    (a, b), _ = _oracle(ctx, [Arithmetic("call", 100.0, 1.0, averaging_start=0.25),
                              Arithmetic("call", 100.0, 1.0)], 50, 1 << 15, 3)
    assert a.price > b.price  # less averaging, more variance


def test_validation():
    ctx = _ctx()
    with pytest.raises(InvalidInputError):
        Arithmetic("call", 100.0, 1.0, averaging_start=1.5)
    with pytest.raises(InvalidInputError):
        plans.average(Arithmetic("call", 100.0, 1.0), ctx, 1)
    with pytest.raises(UnsupportedOperationError):
        plans.average(Arithmetic("call", 100.0, 1.0), _ctx(sigma=0.0), 50)
    assert plans.average(Arithmetic("put", 100.0, 0.0), ctx, 50).value == 0.0


def _gpu_options():
    ctx = _ctx(100.0, 0.3, 0.03, 0.01)
    options = [Arithmetic("call", 100.0, 1.0), Arithmetic("put", 104.0, 1.0),
               Arithmetic("call", 100.0, 2.0, averaging_start=0.5), Arithmetic("put", 60.0, 1.0),
               Geometric("call", 98.0, 1.0), Geometric("put", 100.0, 1.5, averaging_start=0.5),
               Arithmetic("call", 100.0, 0.5, averaging_start=0.5)]
    return ctx, options


@pytest.mark.gpu
@pytest.mark.parametrize("sobol,antithetic", [(False, False), (False, True), (True, False)])
def test_average_gpu_parity(native, sobol, antithetic):
    ctx, options = _gpu_options()
    packed = pack([plans.average(o, ctx, 64) for o in options])
    s = settings(1 << 14, 31, sobol=sobol, antithetic=antithetic)
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= 1e-12 * max(1.0, abs(r.price)), (g.price, r.price)
        assert g.executed_steps == r.executed_steps
    for schedule in ("plain",) if antithetic else ("plain", "persistent"):
        got32 = gpu_price(native, ctx, packed, settings(1 << 14, 31, sobol=sobol, antithetic=antithetic,
                                                        precision="fp32", schedule=schedule))
        for r, g in zip(ref, got32):
            se = max(r.sample_error, 1e-4 * abs(r.price))
            assert abs(g.price - r.price) <= 0.5 * se, (schedule, g.price, r.price)


@pytest.mark.gpu
def test_average_engine_strike_batch_replays_scalar_prices(native):
    from kiyosi_gb300.pricing import MonteCarloAsianEngine
    ctx = _ctx(100.0)
    engine = MonteCarloAsianEngine(path_count=4096, seed=7, step_count=16)
    template = Arithmetic("call", 100.0, 1.0)
    strikes = [95.0, 105.0, 100.0, 95.0, 140.0]
    prices = engine.price_strikes(template, ctx, strikes)
    scalar = [engine.price(Arithmetic("call", k, 1.0), ctx) for k in strikes]
    assert prices == scalar
    assert prices[0] == prices[3] and prices[0] > prices[2] > prices[1] > prices[4]
