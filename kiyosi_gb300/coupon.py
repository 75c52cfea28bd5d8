"""Implied coupons of autocallable notes on the GPU engine (crates/kiyosi/src/risk/coupon.rs).

`implied_snowball_coupon` and `implied_phoenix_coupon` restate kiyosi's solver:
- validate the bounds;
- raise the lower bound to the minimum quotable coupon;
- price the two bound notes;
- interpolate;
- fall back to bisection on the residual.

The GB300 shape of the work: the two bound notes are one book, priced in one launch on
one pinned seed, which is kiyosi's `price_coupon_bounds` with its shared paths.
A note's value is affine in its coupon whenever knock-in affects the two bounds alike.
In that case kiyosi's `prepare_coupon_pricer` interpolates between the bound prices
(engines/monte_carlo/autocallable.rs:1039-1062), and so does this module. The
interpolated first guess then meets the tolerance, and no further launch is needed.
"""
import math
from dataclasses import dataclass, replace
from typing import Callable, Optional, Tuple

from . import plans
from .errors import (ComputationFailureError, InvalidInputError, KiyosiError,
                     RootNotBracketedError, UnsupportedOperationError)

SHIFT_MATURITY_COUPON = "shift_maturity_coupon"
PRESERVE_MATURITY_COUPON = "preserve_maturity_coupon"


class NonConvergenceError(KiyosiError):
    """The solver stopped without matching the observed price."""


@dataclass(frozen=True)
class ImpliedCouponSettings:
    """ImpliedCouponSettings (risk/coupon.rs:30-47)."""
    lower_bound: float = 0.0
    upper_bound: float = 2.0
    price_tolerance: float = 1e-8
    parameter_tolerance: float = 1e-8
    max_iterations: int = 100


def with_snowball_coupon(note, coupon: float, convention: str):
    """SnowballCoupon::with_coupon (instruments/autocallable.rs:647-660): every
    autocall observation's coupon moves by the same shift that sets the first one to
    `coupon`; the maturity coupon moves too under SHIFT_MATURITY_COUPON."""
    if convention not in (SHIFT_MATURITY_COUPON, PRESERVE_MATURITY_COUPON):
        raise InvalidInputError(f"unknown coupon quote convention {convention!r}")
    shift = coupon - (note.observations[0].coupon_rate if note.observations else 0.0)
    observations = [replace(o, coupon_rate=o.coupon_rate + shift) for o in note.observations]
    maturity = note.maturity_coupon_rate + shift if convention == SHIFT_MATURITY_COUPON else note.maturity_coupon_rate
    return replace(note, observations=observations, maturity_coupon_rate=maturity)


def with_phoenix_coupon(note, coupon: float):
    """PhoenixOption::with_coupon (instruments/autocallable.rs:1902-1907)."""
    return replace(note, period_coupon=coupon)


def minimum_quoted_coupon(note, convention: str) -> Optional[float]:
    """AutocallableNote::minimum_quoted_coupon (instruments/autocallable.rs:667-693): under
    SHIFT_MATURITY_COUPON a fixed knock-in coupon bounds the maturity coupon from below."""
    if convention != SHIFT_MATURITY_COUPON or note.knock_in_level is None or note.fixed_knock_in_coupon is None:
        return None
    minimum = note.fixed_knock_in_coupon
    anchor = note.observations[0].coupon_rate
    maturity = note.maturity_coupon_rate
    shift = minimum - maturity
    if maturity + shift < minimum:
        shift = math.nextafter(shift, math.inf)
    lower = anchor + shift
    return math.nextafter(lower, math.inf) if lower - anchor < shift else lower


def implied_snowball_coupon(engine, note, ctx, observed_price: float,
                            convention: str = PRESERVE_MATURITY_COUPON,
                            settings: ImpliedCouponSettings = ImpliedCouponSettings()) -> Tuple[float, str]:
    """implied_snowball_coupon (risk/coupon.rs:106-126): the first observation's coupon
    at which the note prices at `observed_price`, and the quote convention."""
    coupon = _solve(engine, note, ctx, observed_price, settings, minimum_quoted_coupon(note, convention),
                    lambda n, c: with_snowball_coupon(n, c, convention))
    return coupon, convention


def implied_phoenix_coupon(engine, note, ctx, observed_price: float,
                           settings: ImpliedCouponSettings = ImpliedCouponSettings()) -> float:
    """implied_phoenix_coupon (risk/coupon.rs:169-185)."""
    return _solve(engine, note, ctx, observed_price, settings, None, with_phoenix_coupon)


def _midpoint(a: float, b: float) -> float:
    """f64::midpoint: the halfway point without overflow or needless underflow."""
    lo_limit, hi_limit = 2.2250738585072014e-308 * 2.0, 1.7976931348623157e308 / 2.0
    if abs(a) <= hi_limit and abs(b) <= hi_limit:
        return (a + b) / 2.0
    if abs(a) < lo_limit:
        return a + b / 2.0
    if abs(b) < lo_limit:
        return a / 2.0 + b
    return a / 2.0 + b / 2.0


def _finite(name, value, allow_zero=True):
    if not math.isfinite(value) or (not allow_zero and value == 0.0):
        raise InvalidInputError(f"{name} must be finite")


def _solve(engine, option, ctx, observed: float, s: ImpliedCouponSettings, minimum: Optional[float],
           with_coupon: Callable):
    """solve (risk/coupon.rs:191-374)."""
    _finite("observed_price", observed)
    _finite("lower_bound", s.lower_bound)
    _finite("upper_bound", s.upper_bound)
    if not (math.isfinite(s.price_tolerance) and s.price_tolerance >= 0.0):
        raise InvalidInputError("price_tolerance must be finite and nonnegative")
    if not (math.isfinite(s.parameter_tolerance) and s.parameter_tolerance >= 0.0):
        raise InvalidInputError("parameter_tolerance must be finite and nonnegative")
    if s.lower_bound >= s.upper_bound:
        raise InvalidInputError("upper_bound must exceed lower_bound")
    if s.max_iterations <= 0:
        raise InvalidInputError("max_iterations must be positive")
    lower_bound = s.lower_bound
    if minimum is not None:
        lower_bound = max(lower_bound, minimum)
        if lower_bound >= s.upper_bound:
            raise RootNotBracketedError("coupon bounds exclude the contract's valid domain")
    if engine.seed is None:
        raise InvalidInputError("implied-parameter solvers require an explicit seed; "
                                "call with_resolved_seed() before solving")

    def checked(price):
        if not math.isfinite(price):
            raise ComputationFailureError("non-finite coupon price")
        return price

    def residual(value):
        r = value - observed
        if not math.isfinite(r):
            raise ComputationFailureError("non-finite coupon residual")
        return r

    def plan_of(note, ctx):
        build = getattr(engine, "_plan", None)
        return build(note, ctx) if build is not None else plans.autocallable(note, ctx)

    def scalar_price(note):
        return checked(engine._run(ctx, [plan_of(note, ctx)])[0].price)

    lo, hi = lower_bound, s.upper_bound
    lower_note, upper_note = with_coupon(option, lo), with_coupon(option, hi)
    original_lo, original_hi = lo, hi
    # price_coupon_bounds: both bound notes on shared paths, one launch.
    bounds = engine._run(ctx, [plan_of(lower_note, ctx), plan_of(upper_note, ctx)])
    lower, upper = checked(bounds[0].price), checked(bounds[1].price)
    curve = (s.price_tolerance >= 1e-10 * max(abs(observed), 1.0)
             and lower_note.knock_in_affects_payoff() == upper_note.knock_in_affects_payoff()
             and all(math.isfinite(v) and s.price_tolerance >= 1e-10 * max(abs(v), 1.0) for v in (lower, upper)))
    affected = lower_note.knock_in_affects_payoff()
    if lower == upper:
        raise UnsupportedOperationError("coupon does not affect remaining cashflows")
    flo, fhi = residual(lower), residual(upper)
    if abs(flo) <= s.price_tolerance:
        return lo
    if abs(fhi) <= s.price_tolerance:
        return hi
    if (flo < 0.0) == (fhi < 0.0):
        raise RootNotBracketedError("price is not bracketed by coupon bounds")

    def price(coupon):
        note = with_coupon(option, coupon)
        if curve and note.knock_in_affects_payoff() == affected:
            plan = plan_of(note, ctx)
            if isinstance(plan, plans.Known):
                return checked(plan.value)
            span = original_hi - original_lo
            fraction = ((coupon - original_lo) / span if math.isfinite(span)
                        else (0.5 * coupon - 0.5 * original_lo) / (0.5 * original_hi - 0.5 * original_lo))
            return checked(lower * (1.0 - fraction) + upper * fraction)
        return scalar_price(note)

    span = upper - lower
    fraction = ((observed - lower) / span if math.isfinite(span)
                else (0.5 * observed - 0.5 * lower) / (0.5 * upper - 0.5 * lower))

    def interpolate(f):
        return lo + (hi - lo) * f if (lo < 0.0) == (hi < 0.0) else lo * (1.0 - f) + hi * f

    coupon = interpolate(fraction)
    if lo < coupon < hi and abs(residual(price(coupon))) <= s.price_tolerance:
        return coupon
    for _ in range(s.max_iterations):
        mid = _midpoint(lo, hi)
        if mid == lo or mid == hi:
            raise NonConvergenceError("coupon bracket has no representable midpoint")
        value = residual(price(mid))
        if abs(value) <= s.price_tolerance:
            return mid
        if hi - lo <= s.parameter_tolerance:
            raise NonConvergenceError("coupon bracket converged without matching the observed price")
        if (flo < 0.0) == (value < 0.0):
            lo, flo = mid, value
        else:
            hi = mid
    raise NonConvergenceError("implied-coupon solver did not converge")
