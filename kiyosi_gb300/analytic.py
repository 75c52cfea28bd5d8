"""Closed-form BSM pieces the Monte Carlo engines resolve with before sampling.

The reference settles some contracts analytically instead of simulating them:
- a touched knock-in barrier is its vanilla option
  (engines/analytic/barrier.rs:20-78);
- an expiry reached prices at intrinsic value.

This module restates the lognormal pricing kernel those resolutions call
(engines/analytic/european.rs:317-403, with the normal-CDF helpers of numerics.rs:192-224
and 329-334). It is host-side arithmetic on a handful of scalars, not a path simulation.
"""
import math

from .errors import ComputationFailureError
from .market import BlackScholesMertonParameters, PricingContext, log_ratio

_FRAC_1_SQRT_2 = 0.7071067811865476
_LOG_2PI = math.log(2.0 * math.pi)


def normal_cdf(x: float) -> float:
    return 0.5 * math.erfc(-x * _FRAC_1_SQRT_2)


def log_normal_cdf(x: float) -> float:
    """numerics.rs:196-214: the erfc tail expansion below -10."""
    if x >= -10.0:
        return _ln(normal_cdf(x))
    inverse_square = (1.0 / x) / x
    term = 1.0
    total = 1.0
    for k in range(1, 21):
        term *= -float(2 * k - 1) * inverse_square
        total += term
    return -0.5 * x * x - _ln(-x) + _ln(total / math.sqrt(2.0 * math.pi))


def weighted_cdf(amount: float, exponent: float, argument: float) -> float:
    discount = math.exp(exponent)
    discounted = amount * discount
    if argument < -10.0 or not _is_normal(discount) or not math.isfinite(discounted):
        return math.exp(_ln(amount) + exponent + log_normal_cdf(argument))
    return discounted * normal_cdf(argument)


def discounted_product(scale: float, weight: float, log_discount: float) -> float:
    """numerics.rs:226-238."""
    value = scale * weight
    discount = math.exp(log_discount)
    if scale == 0.0 or weight == 0.0:
        return 0.0
    if _is_normal(discount) and _is_normal(value):
        return value * discount
    return math.copysign(math.exp(_ln(scale) + _ln(abs(weight)) + log_discount), weight)


def positive_difference(a: float, b: float) -> float:
    """exp(a) - exp(b) floored at zero (engines/monte_carlo/asian.rs:972-985)."""
    if a == math.inf:
        return a
    if b == -math.inf:
        return math.exp(a)
    difference = -math.expm1(b - a)
    if difference > 0.0:
        return math.exp(a + _ln(difference))
    return 0.0


def log_difference(high: float, low: float) -> float:
    if high == -math.inf:
        return -math.inf
    return high + _ln(-math.expm1(low - high))


def _is_normal(x: float) -> bool:
    return math.isfinite(x) and abs(x) >= 2.2250738585072014e-308


def _ln(x: float) -> float:
    """IEEE logarithm: -inf at zero, NaN below it (Python's math.log raises instead)."""
    if x > 0.0:
        return math.log(x)
    return -math.inf if x == 0.0 else math.nan


def _div(a: float, b: float) -> float:
    """IEEE division (Python raises on a zero divisor)."""
    if b != 0.0:
        return a / b
    if a == 0.0 or math.isnan(a):
        return math.nan
    return math.copysign(math.inf, a) * math.copysign(1.0, b)


def _standardize(value: float, volatility: float, root: float) -> float:
    width = volatility * root
    if width < 2.2250738585072014e-308:
        return _div(_div(value, volatility), root)
    return value / width


def lognormal_price(spot, strike, log_moneyness, asset_log, risk_log, volatility, root_time, sign):
    """lognormal_price (engines/analytic/european.rs:317-403), all three regimes:
    tiny width far from the strike, tiny width near it, and the regular formula with its
    log-space fallback."""
    try:
        return _lognormal_price(spot, strike, log_moneyness, asset_log, risk_log, volatility,
                                root_time, sign)
    except OverflowError:
        raise ComputationFailureError("analytic pricing produced a non-finite result") from None


def _lognormal_price(spot, strike, log_moneyness, asset_log, risk_log, volatility, root_time, sign):
    width = volatility * root_time
    if not math.isfinite(width):
        raise ComputationFailureError("unstable volatility limit")
    standardized = _standardize(log_moneyness, volatility, root_time)
    d1 = standardized + 0.5 * width
    d2 = standardized - 0.5 * width
    if width < 1e-5 and abs(standardized) >= 10.0:
        if sign * log_moneyness > 0.0:
            amount, discount = (spot, asset_log) if sign > 0.0 else (strike, risk_log)
            intrinsic = discounted_product(amount, -math.expm1(-sign * log_moneyness), discount)
        else:
            intrinsic = 0.0
        distance = abs(standardized)
        if math.isinf(distance):
            time_value = 0.0
        else:
            inverse_square = (1.0 / distance) / distance
            term, total, correction = 1.0, 1.0, -3.0
            for order in range(1, 21):
                term *= -float(2 * order + 1) * inverse_square
                total += term
                correction -= float(2 * order + 3) * term
            time_value = math.exp(
                _ln(spot) + asset_log - 0.5 * standardized * width + _ln(volatility)
                + _ln(root_time) - 0.5 * distance * distance - 0.5 * _LOG_2PI
                - 2.0 * _ln(distance) + _ln(total + width * width * correction / 24.0))
        value = intrinsic + time_value
    elif width < 1e-5:
        squared = standardized * standardized
        time_value = (_ln(volatility) + _ln(root_time) - 0.5 * squared - 0.5 * _LOG_2PI
                      + math.log1p((squared - 1.0) * width * width / 24.0))
        gap = abs(math.expm1(-log_moneyness))
        intrinsic = _ln(gap) + log_normal_cdf(sign * d2)
        scale = _ln(spot) + asset_log
        if sign * log_moneyness >= 0.0:
            value = math.exp(scale + time_value) + math.exp(scale + intrinsic)
        else:
            value = math.exp(scale + log_difference(time_value, intrinsic))
    else:
        asset = weighted_cdf(spot, asset_log, sign * d1)
        cash = weighted_cdf(strike, risk_log, sign * d2)
        direct = sign * (asset - cash)
        if math.isfinite(direct):
            value = direct
        else:
            a = log_moneyness + log_normal_cdf(sign * d1)
            c = log_normal_cdf(sign * d2)
            difference = log_difference(a, c) if sign > 0.0 else log_difference(c, a)
            value = math.exp(_ln(strike) + risk_log + difference)
    if not math.isfinite(value):
        raise ComputationFailureError("analytic pricing produced a non-finite result")
    return value


def european_price(option_type_sign: float, strike: float, expiry: float, ctx: PricingContext) -> float:
    """AnalyticEuropeanEngine::price (engines/analytic/european.rs:56-88) with flat rates."""
    model = ctx.model
    if not isinstance(model, BlackScholesMertonParameters):
        raise ComputationFailureError("the analytic European price needs BSM parameters")
    spot = ctx.spot
    if expiry == 0.0:
        return max(option_type_sign * (spot - strike), 0.0)
    risk_log = -model.rate * expiry
    dividend_log = -model.dividend * expiry
    return lognormal_price(spot, strike, log_ratio(spot, strike) + (dividend_log - risk_log),
                           dividend_log, risk_log, model.volatility, math.sqrt(expiry),
                           option_type_sign)


def european_delta_gamma(sign: float, strike: float, expiry: float, ctx: PricingContext):
    """Black-Scholes delta and gamma of a European option with flat rates (the analytic
    Greeks a settled knock-in barrier reports, engines/monte_carlo/barrier.rs:199-206)."""
    model = ctx.model
    spot, sigma = ctx.spot, model.volatility
    width = sigma * math.sqrt(expiry)
    d1 = (log_ratio(spot, strike) + (model.rate - model.dividend) * expiry) / width + 0.5 * width
    carry = math.exp(-model.dividend * expiry)
    delta = sign * carry * normal_cdf(sign * d1)
    gamma = carry * math.exp(-0.5 * d1 * d1) / math.sqrt(2.0 * math.pi) / (spot * width)
    return {"delta": delta, "gamma": gamma}


def scaled_cdf(amount: float, exponent: float, argument: float) -> float:
    """numerics.rs:168-174."""
    if amount == 0.0:
        return 0.0
    return math.exp(_ln(amount) + exponent + log_normal_cdf(argument))


def hit_value(amount: float, distance: float, upper: bool, drift: float, sigma: float, t: float,
              rate: float) -> float:
    """hit_value (engines/analytic/barrier.rs:361-425): the value of `amount` paid when a
    continuously monitored barrier `distance` (absolute log distance) away is first
    touched before `t`.  The closed form with both exponential terms is restated; the
    negative-discriminant quadrature and the reflection tail are not built."""
    from .errors import UnsupportedOperationError
    variance = sigma * sigma
    drift = -drift if upper else drift
    if variance == 0.0:
        raise UnsupportedOperationError("zero-volatility at-hit rebates are not sampled")
    discriminant = drift * drift + 2.0 * rate * variance
    scale = max(1.0, abs(drift * drift), abs(2.0 * rate * variance))
    if discriminant < 0.0 or (rate < 0.0 and discriminant <= 16.0 * 2.220446049250313e-16 * scale):
        raise UnsupportedOperationError("at-hit rebates with a non-positive discriminant are not sampled")
    root = math.sqrt(discriminant)
    width = sigma * math.sqrt(t)
    first_exponent = -2.0 * rate / (root - drift) if drift < 0.0 else (-drift - root) / variance
    second_exponent = 2.0 * rate / (root + drift) if drift > 0.0 else (-drift + root) / variance
    if not math.isfinite(second_exponent):
        raise UnsupportedOperationError("at-hit rebates needing the reflection tail are not sampled")
    first = scaled_cdf(amount, first_exponent * distance, (root * t - distance) / width)
    second = scaled_cdf(amount, second_exponent * distance, (-root * t - distance) / width)
    value = first + second
    if not math.isfinite(value):
        raise ComputationFailureError("analytic pricing produced a non-finite result")
    return value
