"""Discretely monitored single barriers (barrier.rs:240-449, scheduled branch).

CPU checks of the oracle:
- kiyosi's own closed-form check of at-hit rebates
  (crates/kiyosi/tests/barrier_monte_carlo.rs:728-765);
- a quadrature of the discrete-monitoring transition density, standing in for kiyosi's
  QuadratureBarrierEngine in the dense knock-in test (barrier_monte_carlo.rs:35-81, same
  tolerance);
- the resolution rules and the Sobol dimension limit.

GPU checks: the CUDA path against the oracle on the same random numbers, with
conditioned knock-ins, at-hit rebates and an unobserved expiry leg. FP64 must match
within 1e-12 relative; FP32 plain and persistent must land within 0.5 SE.
"""
import math

import numpy as np
import pytest

from kiyosi_gb300 import abi, analytic, plans
from kiyosi_gb300.errors import InvalidInputError
from kiyosi_gb300.instruments import BarrierOption
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from oracle import loader

from helpers import gpu_price, pack, settings


def _market(rate=0.04):
    """barrier_monte_carlo.rs:25-32: r, q = 0.01, sigma = 0.2, spot 100."""
    return PricingContext(BlackScholesMertonParameters(rate, 0.01, 0.2), 100.0)


def _day(days):
    return days / 365.0  # ACT/365 year fractions from 2025-01-01


def _quadrature(option: BarrierOption, ctx: PricingContext, nodes=3001):
    """Discounted value of a scheduled barrier by propagating the surviving density of
    x = log(S / S0) across the observation dates on a grid (trapezoid rule), then
    pricing the vanilla from the last observation with the analytic BSM formula.
    Knock-ins by in/out parity: vanilla - knock-out(no rebate) + rebate x P(survive)."""
    m = ctx.model
    r, q, sigma, spot = m.rate, m.dividend, m.volatility, ctx.spot
    drift = r - q - 0.5 * sigma * sigma
    dates = [t for t in option.observation_times if t > 0.0]
    b = math.log(option.barrier / spot)
    span = 8.0 * sigma * math.sqrt(option.expiry) + abs(drift) * option.expiry
    x = np.linspace(b, b + span, nodes) if not option.is_up else np.linspace(b - span, b, nodes)
    w = np.full(nodes, x[1] - x[0])
    w[0] = w[-1] = 0.5 * (x[1] - x[0])
    density = None
    previous = 0.0
    for t in dates:
        dt = t - previous
        s = sigma * math.sqrt(dt)
        if density is None:
            density = np.exp(-0.5 * ((x - drift * dt) / s) ** 2) / (s * math.sqrt(2 * math.pi))
        else:
            kernel = np.exp(-0.5 * ((x[:, None] - x[None, :] - drift * dt) / s) ** 2) / (
                s * math.sqrt(2 * math.pi))
            density = kernel @ (density * w)
        previous = t
    last = dates[-1]
    tau = option.expiry - last
    if tau > 0.0:
        sub = PricingContext(BlackScholesMertonParameters(r, q, sigma), 1.0)
        inner = np.array([analytic.european_price(option.sign, option.strike / (spot * math.exp(v)),
                                                  tau, sub) * spot * math.exp(v) for v in x])
    else:
        inner = np.maximum(option.sign * (spot * np.exp(x) - option.strike), 0.0)
    survive = float(np.sum(density * w))
    knock_out = math.exp(-r * last) * float(np.sum(density * w * inner))
    rebate_leg = option.rebate * math.exp(-r * option.expiry) * (1.0 - survive)
    if not option.is_knock_in:
        return knock_out + rebate_leg
    vanilla = analytic.european_price(option.sign, option.strike, option.expiry, ctx)
    return vanilla - knock_out + option.rebate * math.exp(-r * option.expiry) * survive


def _oracle(ctx, options, path_count, seed, **kw):
    return loader.price_book(ctx, pack([plans.barrier(o, ctx) for o in options]),
                             settings(path_count, seed, **kw))


def test_scheduled_at_hit_rebate_uses_the_fixing_discount():
    """barrier_monte_carlo.rs:728-765: one observation on 2025-07-01; the at-hit rebate
    adds 10 e^(-r t) P(S_t >= 120), within 0.025; an observation before expiry is not
    extended to expiry, so an up-and-out call struck above its barrier is worth more
    than 0.01 and matches the quadrature within 0.04."""
    ctx = _market(0.04)
    t = _day(181)
    kw = dict(barrier=120.0, barrier_type="up_and_out", observation_times=[t])
    with_rebate, without = _oracle(ctx, [BarrierOption("put", 100.0, 1.0, rebate=10.0,
                                                       rebate_timing="at_hit", **kw),
                                         BarrierOption("put", 100.0, 1.0, **kw)], 131072, 42)
    threshold = (math.log(1.2) - 0.01 * t) / (0.2 * math.sqrt(t))
    probability = 0.5 * math.erfc(threshold / math.sqrt(2.0))
    difference = with_rebate.price - without.price
    assert abs(difference - 10.0 * math.exp(-0.04 * t) * probability) < 0.025
    early = BarrierOption("call", 130.0, 1.0, barrier=120.0, barrier_type="up_and_out",
                          observation_times=[_day(90)])
    value = _oracle(ctx, [early], 131072, 42)[0].price
    assert value > 0.01
    assert abs(value - _quadrature(early, ctx)) < 0.04


@pytest.mark.parametrize("sampling", [("pcg32", True, 42), ("sobol", False, 91)])
def test_dense_scheduled_knock_in_matches_quadrature(sampling):
    """barrier_monte_carlo.rs:35-81: 16 observations (day 60 + 18 i) and an unobserved
    expiry leg, so hits with more than 8 dates left are priced analytically from the
    hit; 65,536 paths within 0.12 of the quadrature, and much closer in practice."""
    ctx = _market(0.04)
    option = BarrierOption("call", 100.0, 1.0, barrier=99.0, barrier_type="down_and_in",
                           rebate=2.0, observation_times=[_day(60 + 18 * i) for i in range(16)])
    plan = plans.barrier(option, ctx)
    assert plan.record["flags"] & abi.C_CONDITION_ON_HIT and plan.record["step_count"] == 17
    name, antithetic, seed = sampling
    e = _oracle(ctx, [option], 65536, seed, sobol=name == "sobol", antithetic=antithetic)[0]
    expected = _quadrature(option, ctx)
    assert abs(e.price - expected) < 0.12
    assert abs(e.price - expected) < 0.03, (e.price, expected)


def test_scheduled_knock_out_values_between_continuous_and_vanilla():
    """Fewer observations touch less often: continuous < monthly < vanilla for a
    knock-out, on the oracle at 2^16 paths (differences far above the SE), and the
    monthly value agrees with the quadrature."""
    ctx = _market(0.04)
    kw = dict(barrier=85.0, barrier_type="down_and_out")
    monthly = BarrierOption("call", 100.0, 1.0, observation_times=[i / 12 for i in range(1, 13)], **kw)
    values = [e.price for e in _oracle(ctx, [BarrierOption("call", 100.0, 1.0, **kw), monthly], 1 << 16, 3)]
    vanilla = analytic.european_price(1.0, 100.0, 1.0, ctx)
    assert values[0] < values[1] < vanilla
    assert abs(values[1] - _quadrature(monthly, ctx)) < 4.0 * 0.07


def test_in_out_parity_without_conditioning():
    """With eight dates or fewer nothing is conditioned: knock-in + knock-out (no
    rebates) is the intrinsic value of every path, so it matches the vanilla price
    within the sampling error."""
    ctx = _market(0.03)
    obs = [0.25, 0.5, 0.75]
    pair = [BarrierOption("put", 100.0, 1.0, barrier=110.0, barrier_type=f"up_and_{x}",
                          observation_times=obs) for x in ("in", "out")]
    a, b = _oracle(ctx, pair, 1 << 16, 11)
    vanilla = analytic.european_price(-1.0, 100.0, 1.0, ctx)
    assert abs(a.price + b.price - vanilla) < 4.0 * (a.sample_error + b.sample_error)


def test_scheduled_resolution_rules():
    """monitoring.rs:293-320 and analytic/barrier.rs:20-78 at valuation time 0."""
    ctx = _market(0.04)
    # The spot beyond a scheduled barrier is no hit unless today is an observation date.
    beyond = BarrierOption("call", 100.0, 1.0, barrier=101.0, barrier_type="down_and_out",
                           observation_times=[0.5, 1.0])
    assert isinstance(plans.barrier(beyond, ctx), plans.ContractPlan)
    today = BarrierOption("call", 100.0, 1.0, barrier=101.0, barrier_type="down_and_out",
                          rebate=1.0, observation_times=[0.0, 0.5, 1.0])
    assert plans.barrier(today, ctx).value == 1.0 * math.exp(-0.04)
    knocked_in = BarrierOption("call", 100.0, 1.0, barrier=101.0, barrier_type="down_and_in",
                               observation_times=[0.0, 0.5])
    assert plans.barrier(knocked_in, ctx).value == analytic.european_price(1.0, 100.0, 1.0, ctx)
    # A knock-out whose payoff needs the barrier crossed is worthless without a rebate ...
    dead = BarrierOption("call", 130.0, 1.0, barrier=120.0, barrier_type="up_and_out",
                         observation_times=[0.5, 1.0])
    assert plans.barrier(dead, ctx).value == 0.0
    # ... unless the last observation is before expiry (the expiry leg is unobserved).
    assert isinstance(plans.barrier(BarrierOption("call", 130.0, 1.0, barrier=120.0,
                                                  barrier_type="up_and_out",
                                                  observation_times=[0.5]), ctx),
                      plans.ContractPlan)
    with pytest.raises(InvalidInputError):
        BarrierOption("call", 100.0, 1.0, barrier=90.0, barrier_type="down_and_in",
                      rebate=1.0, rebate_timing="at_hit", observation_times=[0.5])
    with pytest.raises(InvalidInputError):
        BarrierOption("call", 100.0, 1.0, barrier=90.0, observation_times=[0.5, 0.25])
    with pytest.raises(InvalidInputError):
        BarrierOption("call", 100.0, 1.0, barrier=90.0, observation_times=[])


def test_sobol_dimensions_count_the_unobserved_expiry_leg():
    """barrier_monte_carlo.rs:948-983: 21,201 observations plus the expiry leg exceed
    the Sobol table's 21,201 dimensions."""
    ctx = _market(0.04)
    option = BarrierOption("put", 100.0, 100.0, barrier=120.0, barrier_type="up_and_out",
                           observation_times=[(i + 1) / 300.0 for i in range(21201)])
    with pytest.raises(InvalidInputError):
        _oracle(ctx, [option], 1, 42, sobol=True)


def _gpu_cases():
    ctx = PricingContext(BlackScholesMertonParameters(0.03, 0.01, 0.3), 100.0)
    monthly = [i / 12 for i in range(1, 13)]
    weekly = [i / 52 for i in range(1, 50)]  # the expiry leg is unobserved
    options = [
        BarrierOption("call", 100.0, 1.0, barrier=80.0, barrier_type="down_and_out", rebate=1.5,
                      rebate_timing="at_hit", observation_times=monthly),
        BarrierOption("put", 100.0, 1.0, barrier=115.0, barrier_type="up_and_in", rebate=0.5,
                      observation_times=monthly),
        BarrierOption("call", 95.0, 1.0, barrier=90.0, barrier_type="down_and_in",
                      observation_times=weekly),
        BarrierOption("put", 105.0, 1.0, barrier=125.0, barrier_type="up_and_out", rebate=2.0,
                      observation_times=weekly),
        BarrierOption("call", 100.0, 1.0, barrier=120.0, barrier_type="up_and_in",
                      observation_times=[0.25, 0.5, 0.75]),
    ]
    return ctx, pack([plans.barrier(o, ctx) for o in options])


@pytest.mark.gpu
@pytest.mark.parametrize("sobol,antithetic", [(False, False), (False, True), (True, False)])
def test_scheduled_barrier_gpu_parity(native, sobol, antithetic):
    """FP64 plain within 1e-12 of the oracle (the conditioned leg's erfc may differ
    by an ulp between libraries); FP32 plain and persistent within 0.5 SE, with the
    same executed steps (early exits at the same dates)."""
    ctx, packed = _gpu_cases()
    s = settings(1 << 14, 23, sobol=sobol, antithetic=antithetic)
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= 1e-12 * max(1.0, abs(r.price)), (g.price, r.price)
        assert g.executed_steps == r.executed_steps
    # The persistent schedule does not pair antithetic samples (it rejects them).
    for schedule in ("plain",) if antithetic else ("plain", "persistent"):
        got32 = gpu_price(native, ctx, packed, settings(1 << 14, 23, sobol=sobol, antithetic=antithetic,
                                                        precision="fp32", schedule=schedule))
        for r, g in zip(ref, got32):
            se = max(r.sample_error, 1e-3 * abs(r.price))
            assert abs(g.price - r.price) <= 0.5 * se, (schedule, g.price, r.price)
