"""Host-side plans: the per-step transitions, events and thresholds the reference's
engines build before sampling, packed into the kgpu_* structs of include/kgpu.h.

Each builder restates one reference planning routine:
  european()       EuropeanPayoff::new           engines/monte_carlo.rs:1170-1222
  digital()        MonteCarloDigitalEngine        engines/monte_carlo/digital.rs:75-110
  path_vanilla()   path_samples over a uniform grid with transition() (monte_carlo.rs:2123)
  asian()          arithmetic average of fixing spots on a uniform grid
  autocallable()   prepare_sample_on_grid        engines/monte_carlo/autocallable.rs:293-430
                   BridgePlan::new               autocallable.rs:464-515
                   CashEvent::{new, discounted_payment} autocallable.rs:532-562
  accumulator()    MonteCarloAccumulatorEngine   engines/monte_carlo/accumulator.rs:91-160
A builder returns either a Known value (no sampling) or a ContractPlan; BookBuilder
packs plans into one kgpu_book.
"""
import math
from dataclasses import dataclass, field, replace
from typing import Callable, List, Optional

import numpy as np

from . import abi, analytic
from .errors import UnsupportedOperationError, ComputationFailureError, InvalidInputError
from .instruments import (Accumulator, AsianOption, AutocallableNote, BarrierOption,
                          DigitalOption, EuropeanOption)
from .market import (BlackScholesMertonParameters, HestonParameters, LocalVolatilitySurface,
                     PricingContext, discounted_product, log_ratio, safe_log_returns)

STEP_DTYPE = np.dtype(abi.Step)
EVENT_DTYPE = np.dtype(abi.Event)
INTERVAL_DTYPE = np.dtype(abi.BridgeInterval)
DAILY_DTYPE = np.dtype(abi.BridgeDaily)
CONTRACT_DTYPE = np.dtype(abi.Contract)


@dataclass
class Known:
    """A price that needs no sampling (expiry reached, sigma = 0, settled note)."""
    value: float


def _fp32_ok(values) -> bool:
    a = np.abs(np.asarray(values, dtype=np.float64).ravel())
    ok = (a == 0.0) | ~np.isfinite(a) | ((a >= 2.0 ** -100) & (a <= 2.0 ** 120))
    return bool(ok.all())


def fp32_representable(plan, ctx: PricingContext) -> bool:
    """Whether FP32 kernels can carry `plan`: every finite nonzero value of the plan and
    the model lies within [2^-100, 2^120] in magnitude (the rule kgpu_price_book
    applies before an FP32 launch; a diffusion of 1e-200 or a daily quantity of 1e200
    is priced in FP64)."""
    if not isinstance(plan, ContractPlan):
        return True
    c = plan.contract[0]
    first = list(CONTRACT_DTYPE.names).index("strike")
    last = list(CONTRACT_DTYPE.names).index("greek_log_weight")
    if not _fp32_ok([c[n] for n in CONTRACT_DTYPE.names[first:last + 1]]):
        return False
    if not fp32_model_ok(ctx):
        return False
    st = plan.steps
    if not (_fp32_ok(st["drift"]) and _fp32_ok(st["diffusion"]) and _fp32_ok(st["discount"])):
        return False
    if len(plan.events) and not (_fp32_ok(plan.events["knock_out"]) and _fp32_ok(plan.events["coupon_barrier"])
                                 and _fp32_ok(plan.events["payment"])):
        return False
    if c["flags"] & abi.C_BRIDGE:
        if not (_fp32_ok(plan.intervals["drift"]) and _fp32_ok(plan.intervals["diffusion"])):
            return False
        if plan.daily is not None and not (_fp32_ok(plan.daily["weight"]) and _fp32_ok(plan.daily["width"])):
            return False
    return True


def fp32_model_ok(ctx: PricingContext) -> bool:
    """The model half of fp32_representable."""
    m = ctx.kgpu_model()
    return _fp32_ok([m.spot, m.rate, m.dividend, m.volatility, m.v0, m.kappa, m.theta, m.xi, m.rho])


@dataclass
class ContractPlan:
    contract: np.ndarray                 # one CONTRACT_DTYPE record
    steps: np.ndarray                    # STEP_DTYPE[step_count]
    flags: np.ndarray                    # uint8[step_count]
    events: np.ndarray = field(default_factory=lambda: np.zeros(0, EVENT_DTYPE))
    intervals: np.ndarray = field(default_factory=lambda: np.zeros(0, INTERVAL_DTYPE))
    daily: Optional[np.ndarray] = None   # DAILY_DTYPE[step_count] when bridged
    # exact [price, delta, gamma] of an arithmetic average's geometric control
    control_expected: Optional[tuple] = None
    # an analytic part added to the sampled mean (a continuous knock-out's at-hit
    # rebate, barrier.rs:484-498), as a function of the context
    addend: Optional[Callable] = None

    @property
    def record(self):
        return self.contract[0]


def _unstable():
    return ComputationFailureError("Monte Carlo produced a non-finite parameter, path or result")


def transition(rate, dividend, sigma, time, discount_time):
    """transition (engines/monte_carlo.rs:2123-2137)."""
    drift = (rate - dividend - 0.5 * sigma * sigma) * time
    diffusion = sigma * math.sqrt(time)
    log_discount = -rate * discount_time
    if not (math.isfinite(drift) and math.isfinite(diffusion) and math.isfinite(log_discount)):
        raise _unstable()
    return drift, diffusion, log_discount


def _new_contract(payoff: int, spot: float) -> np.ndarray:
    """A zeroed contract record of `payoff` valued at `spot` (the scenario's spot: a
    book may hold contracts valued at different spots, as Greek stencils do)."""
    c = np.zeros(1, CONTRACT_DTYPE)
    c["payoff"] = payoff
    c["sign"] = 1.0
    c["spot"] = spot
    return c


_GRID_CACHE: dict = {}


def _grid_steps(ctx: PricingContext, times: List[float]):
    """Per-step records of a grid ending at `times` (ascending, > 0).  Under BSM the
    records depend only on the flat parameters and the dates, so books whose notes share
    a grid build it once (the cached array is read-only)."""
    model = ctx.model
    if isinstance(model, BlackScholesMertonParameters):
        key = (model.rate, model.dividend, model.volatility, tuple(times))
        cached = _GRID_CACHE.get(key)
        if cached is None:
            if len(_GRID_CACHE) >= 256:
                _GRID_CACHE.clear()
            cached = _grid_steps_uncached(ctx, times)
            cached.flags.writeable = False
            _GRID_CACHE[key] = cached
        return cached
    return _grid_steps_uncached(ctx, times)


def _grid_steps_uncached(ctx: PricingContext, times: List[float]):
    model = ctx.model
    n = len(times)
    steps = np.zeros(n, STEP_DTYPE)
    previous = 0.0
    for i, t in enumerate(times):
        dt = t - previous
        if isinstance(model, BlackScholesMertonParameters):
            drift, diffusion, log_discount = transition(model.rate, model.dividend,
                                                        model.volatility, dt, t)
        else:
            drift, diffusion, log_discount = dt, math.sqrt(dt), -model.rate * t
        steps[i] = (drift, diffusion, previous, math.exp(log_discount))
        previous = t
    return steps


def _uniform_times(expiry: float, count: int) -> List[float]:
    return [expiry * (i + 1) / count for i in range(count)]


def european(option: EuropeanOption, ctx: PricingContext):
    """EuropeanPayoff::new (monte_carlo.rs:1170-1222): exact terminal sampling."""
    model = ctx.model
    if not isinstance(model, BlackScholesMertonParameters):
        raise InvalidInputError("the European Monte Carlo engine requires BSM parameters")
    sign = option.sign
    time = option.expiry
    if time == 0.0:
        return Known(max(sign * (ctx.spot - option.strike), 0.0))
    rate, dividend, sigma = model.rate, model.dividend, model.volatility
    if sigma == 0.0:
        forward = ctx.spot * math.exp((rate - dividend) * time)
        return Known(max(sign * (forward - option.strike), 0.0) * math.exp(-rate * time))
    diffusion = sigma * math.sqrt(time)
    carry = (rate - dividend) * time
    half_variance = (0.5 * diffusion) * diffusion
    drift = carry - half_variance
    if not (math.isfinite(drift) and math.isfinite(diffusion)):
        raise _unstable()
    moneyness = (log_ratio(ctx.spot, option.strike) + carry) - half_variance
    log_scale = (math.log(ctx.spot) - dividend * time) if sign > 0 else (
        math.log(option.strike) - rate * time)
    c = _new_contract(abi.PAYOFF_EUROPEAN, ctx.spot)
    c["strike"] = option.strike
    c["sign"] = sign
    c["diffusion"] = diffusion
    c["half_variance"] = half_variance
    c["moneyness"] = moneyness
    c["log_scale"] = log_scale
    c["step_count"] = 1
    steps = np.zeros(1, STEP_DTYPE)
    steps[0] = (drift, diffusion, 0.0, math.exp(-rate * time))
    return ContractPlan(c, steps, np.zeros(1, np.uint8))


def digital(option: DigitalOption, ctx: PricingContext):
    """MonteCarloDigitalEngine::native (digital.rs:75-121): d2 standardisation, cash or
    asset payment exp(exponent)."""
    model = ctx.model
    sign = option.sign
    time = option.expiry
    if time == 0.0:
        hit = (ctx.spot > option.strike) if sign > 0 else (ctx.spot < option.strike)
        return Known((option.payout if option.payout is not None else ctx.spot) if hit else 0.0)
    rate, dividend, sigma = model.rate, model.dividend, model.volatility
    root = math.sqrt(time)
    width = sigma * root
    carry = (rate - dividend) * time
    moneyness = log_ratio(ctx.spot, option.strike) + carry
    d2 = moneyness / width - 0.5 * width
    asset = option.payout is None
    amount = ctx.spot if asset else option.payout
    drift = (-dividend - 0.5 * sigma * sigma) * time if asset else -rate * time
    c = _new_contract(abi.PAYOFF_DIGITAL, ctx.spot)
    c["flags"] = abi.C_ASSET_DIGITAL if asset else 0
    c["strike"] = amount
    c["sign"] = sign
    c["diffusion"] = width
    c["moneyness"] = d2
    c["log_scale"] = drift
    c["step_count"] = 1
    # native delta / gamma samples (digital.rs:110-140)
    c["greek_log_spot"] = math.log(ctx.spot)
    c["greek_log_width"] = math.log(sigma) + math.log(root)
    c["greek_log_amount"] = math.log(amount)
    steps = np.zeros(1, STEP_DTYPE)
    steps[0] = (drift, width, 0.0, math.exp(-rate * time))
    return ContractPlan(c, steps, np.zeros(1, np.uint8))


def _barrier_resolution(option: BarrierOption, ctx: PricingContext):
    """resolved_price (engines/analytic/barrier.rs:20-78) with the state of
    instruments/monitoring.rs:293-320, valuation at the option's start: a barrier is
    touched now when today is monitored (always for continuous monitoring, an
    observation time of 0 for scheduled) and the spot is at or beyond it.  Returns the
    settled price, or None when the option must be sampled."""
    from .instruments import DoubleBarrierOption
    rate = ctx.model.rate
    spot, time = ctx.spot, option.expiry
    knock_in = option.is_knock_in
    times = option.observation_times
    monitored = option.continuous or times[0] == 0.0
    if isinstance(option, DoubleBarrierOption):
        hit = spot <= option.lower or spot >= option.upper
    else:
        hit = spot >= option.barrier if option.is_up else spot <= option.barrier
    touched = monitored and hit
    finished = time == 0.0 or (not option.continuous and times[-1] <= 0.0)

    def cash():
        if option.rebate == 0.0:
            return 0.0
        return analytic.discounted_product(option.rebate, 1.0, -rate * time)

    if touched and not knock_in:
        return option.rebate if option.rebate_timing == "at_hit" else cash()
    if not touched and finished and knock_in:
        return cash()
    if isinstance(option, DoubleBarrierOption):
        # DoubleBarrierOption::payoff_requires_touch (instruments/double_barrier.rs)
        needs = option.strike >= option.upper if option.sign > 0.0 else option.strike <= option.lower
    elif option.is_up:
        needs = option.sign > 0.0 and option.strike >= option.barrier
    else:
        needs = option.sign < 0.0 and option.strike <= option.barrier
    requires_touch = (option.continuous or times[-1] == time) and needs
    fixed = option.rebate == 0.0 and requires_touch
    if fixed and not knock_in:
        return 0.0
    if touched or finished or fixed:
        return analytic.european_price(option.sign, option.strike, time, ctx)
    return None


def barrier(option, ctx: PricingContext):
    """MonteCarloBarrierEngine::native (barrier.rs:231-452) for single and double barriers.
    Barriers settled at valuation resolve first (analytic/barrier.rs:20-78): a touched
    knock-out pays its rebate, a touched knock-in is the analytic vanilla option.
    Continuous monitoring draws one terminal normal per path and weights it by the
    Brownian-bridge survival (single) or the killed-density series (double,
    double_barrier.rs); scheduled monitoring steps date by date (one normal per
    observation, plus an unobserved expiry leg when the last observation is earlier)."""
    from .instruments import DoubleBarrierOption
    model = ctx.model
    if not isinstance(model, BlackScholesMertonParameters):
        raise UnsupportedOperationError("the Monte Carlo barrier engine requires BSM parameters")
    resolved = _barrier_resolution(option, ctx)
    if resolved is not None:
        return Known(resolved)
    double = isinstance(option, DoubleBarrierOption)
    rate, dividend, sigma = model.rate, model.dividend, model.volatility
    spot, time = ctx.spot, option.expiry
    level = option.lower if double else option.barrier
    up = False if double else option.is_up
    knock_in = option.is_knock_in
    at_hit = option.rebate_timing == "at_hit"
    if sigma == 0.0:
        raise UnsupportedOperationError("zero volatility: the barrier is deterministic")
    carry_rate = rate - dividend
    half_variance_rate = 0.5 * sigma * sigma
    drift = carry_rate - half_variance_rate

    def mean_distance(elapsed, lvl):
        return (log_ratio(spot, lvl) + carry_rate * elapsed) - half_variance_rate * elapsed

    if not option.continuous:
        return _scheduled_barrier(option, ctx, drift, half_variance_rate, mean_distance)
    addend = None
    if at_hit and not knock_in and option.rebate != 0.0:
        if double:
            raise UnsupportedOperationError("at-hit rebates of continuous double knock-outs are not sampled")

        def addend(scenario: PricingContext, option=option, up=up):
            # hit_value (analytic/barrier.rs:361-425) at the scenario's market
            m = scenario.model
            return analytic.hit_value(option.rebate, abs(log_ratio(option.barrier, scenario.spot)), up,
                                      m.rate - m.dividend - 0.5 * m.volatility * m.volatility,
                                      m.volatility, option.expiry, m.rate)
        addend(ctx)  # unsupported branches fail before sampling
    width = sigma * math.sqrt(time)
    mean = drift * time
    if not (width > 0.0 and math.isfinite(width) and math.isfinite(mean)):
        raise _unstable()
    c = _new_contract(abi.PAYOFF_DOUBLE_BARRIER if double else abi.PAYOFF_BARRIER, ctx.spot)
    c["flags"] = (abi.C_BARRIER_UP if up else 0) | (abi.C_BARRIER_IN if knock_in else 0)
    if double:
        c["band"] = log_ratio(option.upper, level)
        c["band_initial"] = -log_ratio(level, spot)
    c["strike"] = option.strike
    c["sign"] = option.sign
    c["diffusion"] = width
    c["moneyness"] = mean_distance(time, option.strike)
    c["barrier_drift"] = mean
    c["barrier_distance"] = abs(log_ratio(level, spot))
    c["barrier_moneyness"] = mean_distance(time, level)
    # An at-hit knock-out rebate is valued analytically, not on the paths.
    c["rebate"] = 0.0 if addend is not None else option.rebate
    c["spot"] = spot
    c["log_discount"] = -rate * time
    c["step_count"] = 1
    steps = np.zeros(1, STEP_DTYPE)
    steps[0] = (mean, width, 0.0, math.exp(-rate * time))
    return ContractPlan(c, steps, np.zeros(1, np.uint8), addend=addend)


def _scheduled_barrier(option: BarrierOption, ctx: PricingContext, drift, half_variance_rate,
                       mean_distance):
    """The scheduled branch of barrier.rs:240-449: one grid step and one event record per
    remaining observation (plus the unobserved expiry leg).  Step i holds the cumulative
    mean drift * t_i and the width sigma sqrt(t_i - t_(i-1)); event i holds the noise
    level at which date i touches the barrier, the discount and asset log weights of a
    hit, and the remaining time and its root for the conditioned vanilla."""
    from .instruments import DoubleBarrierOption
    model = ctx.model
    rate, dividend, sigma = model.rate, model.dividend, model.volatility
    double = isinstance(option, DoubleBarrierOption)
    spot, time = ctx.spot, option.expiry
    level = option.lower if double else option.barrier
    dates = [t for t in option.observation_times if t > 0.0]
    legs = [(t, True) for t in dates]
    if not dates or dates[-1] != time:
        legs.append((time, False))
    n = len(legs)
    steps = np.zeros(n, STEP_DTYPE)
    events = np.zeros(n, EVENT_DTYPE)
    previous = 0.0
    width_sum = 0.0
    for i, (date, observe) in enumerate(legs):
        dt = date - previous
        width = sigma * math.sqrt(dt)
        mean = drift * date
        if not (width > 0.0 and math.isfinite(width) and math.isfinite(mean)):
            raise _unstable()
        remaining = time - date
        discount = -rate * date
        steps[i] = (mean, width, date, math.exp(discount))
        events[i]["knock_out"] = -mean_distance(date, level) if observe else 0.0
        events[i]["coupon_barrier"] = remaining
        upper_touch = -mean_distance(date, option.upper) if (double and observe) else 0.0
        events[i]["payment"] = (discount, discount - dividend * remaining, math.sqrt(remaining),
                                upper_touch)
        events[i]["has_knock_out"] = 1 if observe else 0
        events[i]["step"] = i
        width_sum += width
        previous = date
    # Both normal samplers stay within ten standard deviations; paths that could still
    # leave the representable range are checked step by step.
    bounded = abs(math.log(spot)) + 10.0 * width_sum + abs(drift * time) < 600.0
    knock_in = option.is_knock_in
    condition = knock_in and n > 8 and bounded
    if condition:
        # Conditioned hits price a vanilla of width sigma sqrt(remaining); the narrow-width
        # regimes of that pricing are not sampled.
        narrowest = min(sigma * float(events[i]["payment"][2]) for i in range(n - 8))
        if not narrowest >= 1e-5:
            raise UnsupportedOperationError("conditioned knock-in widths below 1e-5 are not sampled")
    c = _new_contract(abi.PAYOFF_BARRIER_DISCRETE, ctx.spot)
    c["flags"] = ((abi.C_BARRIER_UP if (not double and option.is_up) else 0)
                  | (abi.C_DOUBLE if double else 0) | (abi.C_BARRIER_IN if knock_in else 0)
                  | (abi.C_REBATE_AT_HIT if option.rebate_timing == "at_hit" else 0)
                  | (abi.C_CONDITION_ON_HIT if condition else 0)
                  | (0 if bounded else abi.C_CHECK_STEPS))
    c["strike"] = option.strike
    c["sign"] = option.sign
    c["moneyness"] = mean_distance(time, option.strike)
    c["half_variance"] = half_variance_rate
    c["rebate"] = option.rebate
    c["spot"] = spot
    c["log_discount"] = -rate * time
    c["volatility"] = sigma
    c["dividend"] = dividend
    c["step_count"] = n
    c["event_count"] = n
    return ContractPlan(c, steps, np.zeros(n, np.uint8), events)


def _geometric_control_values(sign, log_discount, log_spot, log_forward, log_strike, width):
    """ArithmeticParameters::geometric_values (asian.rs:1062-1085): the control's exact
    [price, delta, gamma]."""
    d1 = (log_forward - log_strike) / width + 0.5 * width
    d2 = d1 - width
    log_asset = log_forward + log_discount + analytic.log_normal_cdf(sign * d1)
    log_cash = log_strike + log_discount + analytic.log_normal_cdf(sign * d2)
    if sign > 0.0:
        price = analytic.positive_difference(log_asset, log_cash)
    else:
        price = analytic.positive_difference(log_cash, log_asset)
    delta = sign * math.exp(log_asset - log_spot)
    gamma = math.exp(log_forward + log_discount - 2.0 * log_spot - math.log(width) - 0.5 * d1 * d1
                     - 0.5 * math.log(2.0 * math.pi))
    return (price, delta, gamma)


def average(option, ctx: PricingContext, step_count: int = 50, control: bool = True):
    """MonteCarloAsianEngine::prepare (asian.rs:374-551) for flat BSM rates, valuation at
    the contract's effective time (no realized average).

    Geometric averages and single fixings sample their exact lognormal law in one
    dimension.  Arithmetic averages integrate n = `step_count` trapezoid intervals.
    The first interval is conditioned on the others and integrated in closed form, so
    n - 1 normals are drawn, plus one for a lead interval when averaging starts later.
    Near the money a geometric payoff on the same grid is the control variate
    (geometric_control, asian.rs:1016-1060): samples are residuals and the control's
    exact mean is carried in `control_mean`.  `control=False` builds the plan without
    it, as the reference does when the controlled mean comes out negative."""
    from .instruments import GeometricAveragePriceOption
    model = ctx.model
    if not isinstance(model, BlackScholesMertonParameters):
        raise UnsupportedOperationError("the Monte Carlo Asian engine requires BSM parameters")
    if not (2 <= int(step_count) <= 10_000):
        raise InvalidInputError("step_count must be in 2..=10000")
    geometric = isinstance(option, GeometricAveragePriceOption)
    spot, strike, sign = ctx.spot, option.strike, option.sign
    tau = option.expiry
    if tau == 0.0:
        return Known(max(sign * (spot - strike), 0.0))
    rate, dividend, sigma = model.rate, model.dividend, model.volatility
    if sigma == 0.0:
        raise UnsupportedOperationError("zero volatility: the average is deterministic")
    single = option.period == 0.0
    lead = 0.0 if single else option.averaging_start
    future = tau if single else tau - option.averaging_start
    weight = 1.0 if single else future / option.period
    carry = rate - dividend
    drift_rate = carry - 0.5 * sigma * sigma
    log_discount = -rate * tau
    c_sign = sign
    if geometric or single:
        variance_time = tau if single else lead + future / 3.0
        if single:
            moneyness = log_ratio(spot, strike) + ((-dividend * tau) - log_discount)
            drift = -0.5 * sigma * sigma * tau
        else:
            moneyness = weight * log_ratio(spot, strike)
            drift = weight * drift_rate * (lead + future / 2.0)
        width = sigma * (weight * math.sqrt(variance_time))
        log_width = math.log(sigma) + math.log(weight) + 0.5 * math.log(variance_time)
        initial_moneyness = moneyness + 0.0
        if not (math.isfinite(drift) and math.isfinite(width)):
            raise _unstable()
        c = _new_contract(abi.PAYOFF_AVERAGE_GEOMETRIC, ctx.spot)
        c["strike"] = strike
        c["sign"] = c_sign
        c["moneyness"] = initial_moneyness + drift
        c["diffusion"] = width
        c["log_scale"] = log_width
        c["avg_log_strike"] = math.log(strike)
        c["log_discount"] = log_discount
        c["spot"] = spot
        c["step_count"] = 1
        # native delta / gamma samples (GeometricParameters::geometric)
        c["greek_log_spot"] = math.log(spot)
        c["greek_log_weight"] = math.log(weight)
        c["greek_log_base_width"] = math.log(sigma) + 0.5 * math.log(variance_time)
        return ContractPlan(c, np.zeros(1, STEP_DTYPE), np.zeros(1, np.uint8))
    n = int(step_count)
    dt = future / float(n)
    interval_forward = carry * dt
    drift = drift_rate * dt
    width = sigma * math.sqrt(dt)
    lead_drift = drift_rate * lead
    lead_width = sigma * math.sqrt(lead)
    if not all(math.isfinite(v) for v in (drift, width, lead_drift, lead_width, interval_forward)):
        raise _unstable()
    if width < 1e-5:
        raise UnsupportedOperationError("average-price intervals narrower than 1e-5 are not sampled")
    has_lead = lead > 0.0
    dims = n - 1 + (1 if has_lead else 0)
    half = 0.5 / float(n)
    rest = 1.0 - half
    log_spot = math.log(spot)
    c = _new_contract(abi.PAYOFF_AVERAGE_ARITHMETIC, ctx.spot)
    c["strike"] = strike
    c["sign"] = c_sign
    c["spot"] = spot
    c["log_discount"] = log_discount
    c["avg_drift"] = drift
    c["avg_width"] = width
    c["avg_lead_drift"] = lead_drift
    c["avg_lead_width"] = lead_width
    c["avg_interval_forward"] = interval_forward
    c["avg_weight"] = weight
    c["avg_log_spot"] = log_spot
    c["avg_log_scale"] = log_spot + math.log(weight)
    c["avg_log_strike"] = math.log(strike)
    c["avg_fraction"] = 1.0 / float(n)
    c["avg_half"] = half
    c["avg_log_fraction"] = math.log(1.0 / float(n))
    c["avg_log_half"] = math.log(half)
    c["avg_rest"] = rest
    c["avg_log_rest"] = math.log(rest)
    # prior_weight ((realized - strike) / spot) + weight ((spot - strike) / spot), no history
    c["avg_baseline"] = 0.0 * ((0.0 - strike) / spot) + weight * ((spot - strike) / spot)
    c["greek_log_width"] = math.log(sigma) + 0.5 * math.log(dt)  # ArithmeticParameters::log_width
    c["step_count"] = dims
    expected = None
    flags = abi.C_AVERAGE_LEAD if has_lead else 0
    if control:
        # geometric_control (asian.rs:1016-1060)
        first_weight = 1.0 - 0.5 / float(n)
        log_asset_scale = log_spot + math.log(weight)
        log_strike = math.log(strike)
        usable = not (width > 0.8 or abs(log_discount) > 50.0 or abs(log_spot) > 200.0
                      or abs(log_asset_scale) > 200.0)
        if usable:
            mean = lead_drift + first_weight * drift
            for step in range(1, n):
                mean += (first_weight - float(step) / float(n)) * drift
            variance = lead_width * lead_width + width * width * (float(n) / 3.0 - 1.0 / (12.0 * float(n)))
            control_width = math.sqrt(variance)
            log_forward = log_asset_scale + mean + 0.5 * variance
            if 0.02 <= control_width <= 0.8 and abs(log_forward - log_strike) <= 2.0 * control_width:
                flags |= abi.C_AVERAGE_CONTROL
                c["control_log_strike"] = log_strike
                c["control_log_asset_scale"] = log_asset_scale
                c["control_first_weight"] = first_weight
                expected = _geometric_control_values(c_sign, log_discount, log_spot, log_forward,
                                                     log_strike, control_width)
                c["control_mean"] = expected[0]
    c["flags"] = flags
    return ContractPlan(c, np.zeros(dims, STEP_DTYPE), np.zeros(dims, np.uint8),
                        control_expected=expected)


def greek_output(plan, output: str):
    """A copy of `plan` whose paths report their native delta or gamma sample instead
    of the payoff (digital, barrier and average payoffs); an arithmetic average's control
    mean becomes the control's exact delta or gamma."""
    if isinstance(plan, Known):
        return plan
    index = {"delta": 1, "gamma": 2}[output]
    c = plan.contract.copy()
    c["flags"] = c["flags"] | (abi.C_OUTPUT_DELTA if index == 1 else abi.C_OUTPUT_GAMMA)
    if plan.control_expected is not None:
        c["control_mean"] = plan.control_expected[index]
    # An analytic addend's Greeks come from its own stencils, not from this sample.
    return replace(plan, contract=c, addend=None)


def path_vanilla(option: EuropeanOption, ctx: PricingContext, step_count: int):
    """Vanilla payoff after `step_count` uniform log-Euler steps (the reference's generic
    D-dimensional sampler path_samples, monte_carlo.rs:1498, with transition())."""
    if step_count < 1:
        raise InvalidInputError("step_count must be positive")
    times = _uniform_times(option.expiry, step_count)
    steps = _grid_steps(ctx, times)
    c = _new_contract(abi.PAYOFF_VANILLA_PATH, ctx.spot)
    c["strike"] = option.strike
    c["sign"] = option.sign
    c["step_count"] = step_count
    c["final_discount"] = math.exp(-ctx.rate * option.expiry)
    return ContractPlan(c, steps, np.zeros(step_count, np.uint8))


def asian(option: AsianOption, ctx: PricingContext, step_count: Optional[int] = None):
    """Arithmetic average of the spots at the fixing times.  The grid is the fixing
    times, refined to `step_count` uniform steps when given (each fixing must then lie on
    the uniform grid)."""
    fixings = list(option.fixings)
    if step_count is None:
        times = fixings
    else:
        times = _uniform_times(option.expiry, step_count)
    flags = np.zeros(len(times), np.uint8)
    index = {round(t, 12): i for i, t in enumerate(times)}
    for f in fixings:
        i = index.get(round(f, 12))
        if i is None:
            raise InvalidInputError("every fixing must lie on the simulation grid")
        flags[i] |= abi.STEP_FIXING
    c = _new_contract(abi.PAYOFF_ASIAN, ctx.spot)
    c["strike"] = option.strike
    c["sign"] = option.sign
    c["step_count"] = len(times)
    c["final_discount"] = math.exp(-ctx.rate * option.expiry)
    return ContractPlan(c, _grid_steps(ctx, times), flags)


_EVENT_GRID_CACHE: dict = {}
_EVENT_GRID_BY_ID: dict = {}


def refine_grid(times: List[float], time_steps: Optional[int]) -> List[float]:
    """Adds path steps between the dates of a grid (ascending, > 0) so that no step is
    much longer than times[-1] / time_steps: each interval between consecutive dates
    (from valuation) is cut into max(round(length / dt_max), 1) equal steps.  This is
    the rule of QuantLib's TimeGrid(mandatory times, steps), so a path discretised here
    visits the same times as QuantLib's path generators.  Exact BSM stepping does not
    need it; Euler schemes (local volatility, Heston) use it to bound the time step."""
    if not time_steps or not times:
        return list(times)
    if int(time_steps) < 1:
        raise InvalidInputError("time_steps must be positive")
    dt_max = times[-1] / int(time_steps)
    out = []
    begin = 0.0
    for end in times:
        n = max(int(math.floor((end - begin) / dt_max + 0.5)), 1)
        dt = (end - begin) / n
        out.extend(begin + k * dt for k in range(1, n))
        out.append(end)
        begin = end
    return out


def _event_grid(ctx: PricingContext, event_times, knock_in_times, expiry, time_steps=None):
    """future_event_times (instruments/autocallable/pricing.rs:70-106): the merged grid
    of event dates, daily knock-in dates (None when not monitored) and expiry, with its
    step records, knock-in flags and excursion (the sum over steps of |drift| + 20
    diffusion, added in step order).  `time_steps` refines the grid (refine_grid).
    Notes of one schedule share the result."""
    model = ctx.model
    bsm = isinstance(model, BlackScholesMertonParameters)
    # Notes of a book share their schedule objects: look the grid up by the schedule's
    # identity first (no hashing of a long tuple), then by its contents.
    fast = (type(model), model.rate, model.dividend, getattr(model, "volatility", None), event_times,
            id(knock_in_times), expiry, time_steps) if bsm else None
    if fast is not None:
        hit = _EVENT_GRID_BY_ID.get(fast)
        if hit is not None and hit[0] is knock_in_times:
            return hit[1]
    key = (type(model), model.rate, model.dividend, getattr(model, "volatility", None), event_times,
           knock_in_times, expiry, time_steps) if bsm else None
    hit = _EVENT_GRID_CACHE.get(key) if key is not None else None
    if hit is not None:
        if len(_EVENT_GRID_BY_ID) >= 256:
            _EVENT_GRID_BY_ID.clear()
        _EVENT_GRID_BY_ID[fast] = (knock_in_times, hit)
        return hit
    times = sorted(set(list(event_times) + (list(knock_in_times) if knock_in_times is not None else [])
                       + [expiry]))
    times = refine_grid([t for t in times if t > 0.0], time_steps)
    steps = _grid_steps(ctx, times)
    flags = np.zeros(len(times), np.uint8)
    if knock_in_times is not None:
        flags[np.isin(np.array(times), np.array(knock_in_times))] |= abi.STEP_KNOCK_IN
    excursion = (float(np.cumsum(np.abs(steps["drift"]) + 20.0 * steps["diffusion"])[-1])
                 if bsm else 0.0)
    grid = np.array(times)
    grid.flags.writeable = False
    out = (times, steps, flags, excursion, grid)
    if key is not None:
        if len(_EVENT_GRID_CACHE) >= 256:
            _EVENT_GRID_CACHE.clear()
        flags.flags.writeable = False
        _EVENT_GRID_CACHE[key] = out
    return out


_CASH_EVENT_CACHE: dict = {}


def cash_event(note: AutocallableNote, o, spot: float, rate: float, step: int):
    """CashEvent::new and discounted_payment (autocallable.rs:532-562): one observation's
    log-space knock-out and coupon thresholds and its four discounted payments, indexed
    coupon_due | knocked_out << 1, as an EVENT_DTYPE record at grid step `step`.  Notes
    of a book that share an observation and the terms its payments read share the
    record."""
    period_coupon = note.period_coupon if o.coupon_barrier_level is not None else 0.0
    key = (o, period_coupon, note.principal, note.rebate_rate, note.annual_rebate_rate,
           note.effective_time, spot, rate)
    record = _CASH_EVENT_CACHE.get(key)
    if record is None:
        if len(_CASH_EVENT_CACHE) >= 65536:
            _CASH_EVENT_CACHE.clear()
        record = _cash_event(note, o, spot, rate)
        _CASH_EVENT_CACHE[key] = record
    return record + (step,)


def _cash_event(note: AutocallableNote, o, spot: float, rate: float):
    has_ko = o.knock_out_level is not None
    ko = log_ratio(o.knock_out_level, spot) if has_ko else 0.0
    barrier = log_ratio(o.coupon_barrier_level if o.coupon_barrier_level is not None
                        else 0.0, spot)
    period_coupon = note.period_coupon if o.coupon_barrier_level is not None else 0.0
    redemption = note.knock_out_payment(o) if has_ko else 0.0
    log_discount = -rate * o.time
    # discounted_product(1, amount, log_discount), with the discount factor taken once
    discount = math.exp(log_discount) if log_discount < 709.0 else math.inf
    plain = math.isfinite(discount) and discount >= 2.2250738585072014e-308
    payments = []
    for outcome in range(4):
        coupon_due, knocked_out = outcome & 1, outcome >> 1
        coupon = period_coupon if coupon_due else 0.0
        amount = redemption + coupon if knocked_out else coupon
        if amount == 0.0:
            payments.append(0.0)
        elif plain and math.isfinite(amount) and abs(amount) >= 2.2250738585072014e-308:
            payments.append(amount * discount)
        else:
            payments.append(discounted_product(1.0, amount, log_discount))
    return (ko, barrier, tuple(payments), int(has_ko))


@dataclass(frozen=True)
class AutocallableInitial:
    """pricing::Initial (instruments/autocallable/pricing.rs:7-11): the knock-in state at
    valuation, a settlement that makes sampling unnecessary, and the coupon fixed at the
    valuation instant."""
    knocked_in: bool
    settlement: Optional[float]
    coupon: float


def _current_observation(note: AutocallableNote):
    """AutocallableNote::event_at(valuation) (instruments/autocallable.rs:1045-1051)."""
    for o in note.observations:
        if o.time == 0.0:
            return o
    return None


def autocallable_prior(note: AutocallableNote) -> bool:
    """AutocallableNote::prior (instruments/autocallable.rs:1320-1369): checks the
    recorded history against the schedule before valuation and returns whether the note
    knocked in before valuation."""
    ko = [o.time for o in note.observations if o.knock_out_level is not None]
    first_out = ko[0] if ko else (note.observations[0].time if note.observations else None)
    had_out = first_out is not None and first_out < 0.0
    had_in = (note.daily_knock_in and note.effective_time < 0.0
              and any(note.effective_time <= t < 0.0 for t in note.knock_in_times))
    state = note.barrier_state
    if state is None and (had_out or had_in):
        from .errors import MissingHistoryError
        raise MissingHistoryError("prior autocallable state is required")
    if state == "knocked_out" and not had_out:
        raise InvalidInputError("knock-out predates observations")
    if state == "knocked_in" and not had_in:
        raise InvalidInputError("knock-in predates monitoring")
    return state == "knocked_in"


def autocallable_expiry_payment(note: AutocallableNote, spot: float, knocked_in: bool, record) -> float:
    """pricing::expiry_payment (instruments/autocallable/pricing.rs:51-69)."""
    coupon = note.observation_coupon(record, spot)
    if record is not None and record.knock_out_level is not None and spot >= record.knock_out_level:
        return coupon + note.knock_out_payment(record)
    ki = knocked_in or (note.observes_knock_in(note.expiry) and note.below_knock_in(spot))
    return coupon + note.terminal(spot, ki)


def autocallable_initial(note: AutocallableNote, spot: float) -> AutocallableInitial:
    """pricing::initial (instruments/autocallable/pricing.rs:12-49) at the valuation
    instant (time 0): a knocked-out note settles at 0; a daily-monitored note whose
    valuation is a monitoring date knocks in when the spot is below the level (strict);
    an observation at valuation fixes its coupon, and settles the note when it knocks
    out (inclusive) or when valuation is expiry."""
    if note.barrier_state == "knocked_out":
        return AutocallableInitial(False, 0.0, 0.0)
    knocked_in = note.barrier_state == "knocked_in"
    if note.daily_knock_in and 0.0 in note.knock_in_times:
        knocked_in |= note.below_knock_in(spot)
    current = _current_observation(note)
    coupon = note.observation_coupon(current, spot)
    if note.expiry == 0.0:
        settlement = autocallable_expiry_payment(note, spot, knocked_in, current)
    elif (current is not None and current.knock_out_level is not None
          and spot >= current.knock_out_level):
        settlement = note.knock_out_payment(current) + coupon
    else:
        settlement = None
    return AutocallableInitial(knocked_in, settlement, coupon)


def _is_normal_float(x: float) -> bool:
    return math.isfinite(x) and abs(x) >= 2.2250738585072014e-308


def autocallable_fixed_value(note: AutocallableNote, ctx: PricingContext, knocked_in: bool):
    """pricing::fixed_value_at (instruments/autocallable/pricing.rs:137-193) at
    valuation: the note's value when no remaining path can change it (an exact
    comparison of terms and discounted payments), else None."""
    if note.daily_knock_in:
        pending = note.expiry > 0.0 and any(0.0 < t <= note.expiry for t in note.knock_in_times)
    else:
        pending = note.knock_in_level is not None and note.expiry > 0.0
    if knocked_in or pending:
        if note.fixed_knock_in_coupon is None and note.knock_in_level is not None:
            if note.lower_strike != note.upper_strike or (not knocked_in and note.maturity_coupon_rate != 0.0):
                return None
        elif not knocked_in and note.knock_in_affects_payoff():
            return None
    rate = ctx.rate

    def discount(t):
        return math.exp(-rate * t)
    value = note.terminal(ctx.spot, knocked_in) * discount(note.expiry)
    if not math.isfinite(value):
        return None
    coupons = 0.0
    for o in reversed(note.observations):
        if not o.time > 0.0:
            break
        d = discount(o.time)
        if not _is_normal_float(d) or (o.knock_out_level is not None
                                       and note.knock_out_payment(o) * d != value + coupons):
            return None
        if o.coupon_barrier_level is not None:
            if note.period_coupon != 0.0 and o.coupon_barrier_level != 0.0:
                return None
            coupons += note.period_coupon * d
            if not math.isfinite(coupons):
                return None
    return value + coupons if _is_normal_float(discount(note.expiry)) else None


def autocallable(note: AutocallableNote, ctx: PricingContext, allow_bridge: bool = True,
                 time_steps: Optional[int] = None):
    """prepare_sample_on_grid (autocallable.rs:293-430): the history check and
    `pricing::initial` at valuation (a settled or path-independent note is Known), then
    the merged event and daily knock-in grid of the future dates, log-space thresholds,
    discounted cash events, the coupon fixed at valuation as initial cash, and the
    Brownian-bridge plan when the reference would use one.  `time_steps` adds path
    steps between the dates (refine_grid) for Euler schemes."""
    model = ctx.model
    spot = ctx.spot
    rate, dividend = model.rate, model.dividend
    bsm = isinstance(model, BlackScholesMertonParameters)
    autocallable_prior(note)
    state = autocallable_initial(note, spot)
    value = state.settlement
    if value is None:
        fixed = autocallable_fixed_value(note, ctx, state.knocked_in)
        value = None if fixed is None else fixed + state.coupon
    if value is not None:
        if not math.isfinite(value):
            raise ComputationFailureError("Monte Carlo produced a non-finite parameter, path or result")
        return Known(value)
    knocked_in = state.knocked_in
    daily = note.daily_knock_in and not knocked_in and note.knock_in_affects_payoff()
    knock_in = log_ratio(note.knock_in_level, spot) if note.knock_in_level is not None else 0.0
    expiry_knock_in = note.knock_in_level is not None and (
        note.knock_in_times is None or (len(note.knock_in_times) > 0
                                        and note.knock_in_times[-1] == note.expiry))
    events = [o for o in note.observations if o.time > 0.0]
    times, steps, ki_flags, excursion, grid = _event_grid(ctx, tuple(o.time for o in events),
                                                          note.knock_in_times if daily else None,
                                                          note.expiry, time_steps)
    flags = ki_flags.copy()
    position = np.searchsorted(grid, [o.time for o in events]).tolist()
    flags[position] |= abi.STEP_EVENT
    ev = np.array([cash_event(note, o, spot, rate, i) for o, i in zip(events, position)], EVENT_DTYPE)
    c = _new_contract(abi.PAYOFF_AUTOCALLABLE, ctx.spot)
    flag = 0
    if note.knock_in_level is not None:
        flag |= abi.C_HAS_KNOCK_IN
    if knocked_in:
        flag |= abi.C_KNOCKED_IN
    if expiry_knock_in:
        flag |= abi.C_EXPIRY_KNOCK_IN
    if note.fixed_knock_in_coupon is None:
        flag |= abi.C_DOWNSIDE
    c["step_count"] = len(times)
    c["event_count"] = len(events)
    c["knock_in"] = knock_in
    c["initial_cash"] = state.coupon
    c["terminal_base"] = note.principal + note.rebate_payment(note.expiry)
    c["terminal_plain"] = note.terminal(0.0, False)
    c["terminal_fixed"] = note.terminal(0.0, True) if note.fixed_knock_in_coupon is not None else 0.0
    c["downside_lower"] = note.lower_strike
    c["downside_upper"] = note.upper_strike
    c["downside_initial"] = note.initial_spot
    c["final_discount"] = math.exp(-rate * times[-1])
    plan = ContractPlan(c, steps, flags, ev)
    low, high = safe_log_returns(spot)
    if (allow_bridge and bsm and daily and low <= excursion <= high and low <= -excursion <= high):
        bridge = _bridge_plan(times, steps, flags, model)
        if bridge is not None:
            plan.intervals, plan.daily = bridge
            c["flags"] = flag | abi.C_BRIDGE
            c["bridge_count"] = len(plan.intervals)
            return plan
    c["flags"] = flag
    return plan


def _bridge_plan(times, steps, flags, model):
    """BridgePlan::new (autocallable.rs:464-515)."""
    rate, dividend, sigma = model.rate, model.dividend, model.volatility
    intervals = []
    first = 0
    has_gap = False
    n = len(times)
    for end in range(n):
        if (flags[end] & abi.STEP_EVENT) or end + 1 == n:
            has_gap |= end - first >= 8
            start = 0.0 if first == 0 else times[first - 1]
            drift, diffusion, _ = transition(rate, dividend, sigma, times[end] - start, 0.0)
            intervals.append((end, 0, drift, diffusion))
            first = end + 1
    if not has_gap:
        return None
    daily = np.zeros(n, DAILY_DTYPE)
    first = 0
    previous = 0.0
    for end, _, _, _ in intervals:
        end_time = times[end]
        for i in range(first, end):
            dt = times[i] - previous
            fraction = dt / (end_time - previous)
            if not (0.0 < fraction < 1.0):
                return None
            daily[i] = (fraction, sigma * math.sqrt(dt * (1.0 - fraction)))
            previous = times[i]
        first = end + 1
        previous = end_time
    return np.array(intervals, INTERVAL_DTYPE), daily


def _accrues(option: Accumulator) -> bool:
    """Accumulator::accrues (instruments/accumulator.rs:456-470)."""
    if option.knock_out_settled or option.daily_quantity == 0.0 or option.expiry <= 0.0:
        return False
    ko = set(option.knock_out_times)
    return any(t > 0.0 and (option.acceleration != 0.0 or not option.is_knock_out(option.strike)
                            or t not in ko) for t in option.accumulation_times)


def accumulator_initial(option: Accumulator, ctx: PricingContext):
    """Accumulator::initial_with_accrual (instruments/accumulator.rs:528-567) at the
    valuation instant (time 0): (quantity held, settlement or None).  A knock-out
    observed now settles the held quantity; an accumulation date now adds its purchase
    at the current spot; a note that can no longer accrue, or is at expiry, settles."""
    spot = ctx.spot
    if option.knock_out_settled:
        return 0.0, 0.0
    quantity = option.quantity
    if 0.0 in option.knock_out_times and option.is_knock_out(spot):
        return quantity, quantity * option.unit_payoff(spot)
    if 0.0 in option.accumulation_times:
        quantity += option.purchase(spot)
    accrues = _accrues(option)
    if quantity == 0.0 and not accrues:
        return quantity, 0.0
    if option.expiry == 0.0 or (not accrues and ctx.rate == 0.0 and ctx.dividend == 0.0):
        return quantity, quantity * option.unit_payoff(spot)
    return quantity, None


def accumulator(option: Accumulator, ctx: PricingContext, time_steps: Optional[int] = None):
    """MonteCarloAccumulatorEngine::sample (accumulator.rs:91-160) without fixed purchase
    events: steps on the union of accumulation and knock-out dates, refined by
    `time_steps` (refine_grid) for Euler schemes."""
    spot = ctx.spot
    quantity, settlement = accumulator_initial(option, ctx)
    if settlement is not None:
        if not math.isfinite(settlement):
            raise ComputationFailureError("Monte Carlo produced a non-finite parameter, path or result")
        return Known(settlement)
    if not math.isfinite(quantity):
        raise ComputationFailureError("Monte Carlo produced a non-finite parameter, path or result")
    times = sorted(set(option.accumulation_times) | set(option.knock_out_times))
    times = refine_grid([t for t in times if t > 0.0], time_steps)
    if not times:
        raise InvalidInputError("an accumulator needs a future observation")
    acc = set(option.accumulation_times)
    ko = set(option.knock_out_times)
    flags = np.zeros(len(times), np.uint8)
    for i, t in enumerate(times):
        if t in ko:
            flags[i] |= abi.STEP_EVENT
        if t in acc:
            flags[i] |= abi.STEP_ACCUMULATE
    c = _new_contract(abi.PAYOFF_ACCUMULATOR, ctx.spot)
    c["strike"] = option.strike
    c["sign"] = option.sign
    c["step_count"] = len(times)
    c["knock_out"] = log_ratio(option.knock_out_level, spot)
    c["log_strike"] = log_ratio(option.strike, spot)
    c["quantity"] = quantity
    c["daily_quantity"] = option.daily_quantity
    c["acceleration"] = option.acceleration
    c["final_discount"] = math.exp(-ctx.rate * times[-1])
    return ContractPlan(c, _grid_steps(ctx, times), flags)


class BookBuilder:
    """Packs contract plans into the flat arrays of one kgpu_book."""

    def __init__(self):
        self.plans: List[ContractPlan] = []

    def add(self, plan: ContractPlan) -> int:
        self.plans.append(plan)
        return len(self.plans) - 1

    def build(self, path_counts=None):
        n = len(self.plans)
        contracts = np.zeros(n, CONTRACT_DTYPE)
        steps = np.concatenate([p.steps for p in self.plans]) if n else np.zeros(0, STEP_DTYPE)
        flags = np.concatenate([p.flags for p in self.plans]) if n else np.zeros(0, np.uint8)
        events = np.concatenate([p.events for p in self.plans]) if n else np.zeros(0, EVENT_DTYPE)
        intervals = (np.concatenate([p.intervals for p in self.plans]) if n
                     else np.zeros(0, INTERVAL_DTYPE))
        any_bridge = any(p.daily is not None for p in self.plans)
        daily = (np.concatenate([p.daily if p.daily is not None
                                 else np.zeros(len(p.steps), DAILY_DTYPE) for p in self.plans])
                 if any_bridge else None)
        so = eo = io = 0
        for i, p in enumerate(self.plans):
            contracts[i] = p.contract[0]
            contracts[i]["step_offset"] = so
            contracts[i]["event_offset"] = eo
            contracts[i]["bridge_offset"] = io
            if path_counts is not None:
                contracts[i]["path_count"] = int(path_counts[i])
            so += len(p.steps)
            eo += len(p.events)
            io += len(p.intervals)
        return PackedBook(contracts, steps, flags, events, intervals, daily)


class PackedBook:
    """Owns the numpy arrays behind a kgpu_book and exposes the struct."""

    def __init__(self, contracts, steps, flags, events, intervals, daily):
        self.contracts = np.ascontiguousarray(contracts)
        self.steps = np.ascontiguousarray(steps)
        self.flags = np.ascontiguousarray(flags)
        self.events = np.ascontiguousarray(events)
        self.intervals = np.ascontiguousarray(intervals)
        self.daily = None if daily is None else np.ascontiguousarray(daily)

    def struct(self) -> abi.Book:
        b = abi.Book()
        P = abi.C.POINTER
        b.contract_count = len(self.contracts)
        b.contracts = self.contracts.ctypes.data_as(P(abi.Contract))
        b.step_total = len(self.steps)
        b.steps = self.steps.ctypes.data_as(P(abi.Step))
        b.step_flags = self.flags.ctypes.data_as(P(abi.C.c_uint8))
        b.bridge_daily = (self.daily.ctypes.data_as(P(abi.BridgeDaily))
                          if self.daily is not None else None)
        b.event_total = len(self.events)
        b.interval_total = len(self.intervals)
        b.events = self.events.ctypes.data_as(P(abi.Event)) if len(self.events) else None
        b.intervals = (self.intervals.ctypes.data_as(P(abi.BridgeInterval))
                       if len(self.intervals) else None)
        return b
