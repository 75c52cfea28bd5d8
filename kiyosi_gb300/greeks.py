"""Numerical Greeks by bump-and-reprice, every scenario priced in one GPU launch.

This follows kiyosi's `numerical_greeks` and `complete_greeks_with_pair`
(crates/kiyosi/src/risk/numerical.rs:11-30, 33-132, 164-207, 275-702) for BSM
contexts:
- symmetric bumps whose legs share one representable distance;
- the default shifts: spot min(0.01, 1% of spot), volatility min(1e-4, half the
  volatility), and rates 1e-4 (risk/analytics.rs:403-421);
- the same difference formulas for delta, gamma, speed, vega, volga, vanna, zomma, rho
  and dividend rho;
- terminal-payoff stencils at expiry.

The reference prices each bumped context with a pinned seed, and its batched paths
(european_greek_prices, autocallable market_prices) drive every scenario with the same
normals. Here every scenario's plan goes into one book, and one `kgpu_price_book` call
prices them all. Each contract is sampled with the same seed and block streams, so the
scenarios share their random numbers exactly as the reference's do.

Time Greeks (theta, charm, color) need kiyosi's timestamp and calendar stencils, which
this package's year-fraction contexts do not model. They report `unsupported`.
"""
import math
from dataclasses import dataclass, field, replace
from typing import Callable, Dict, Iterable, List, Optional, Tuple

from .errors import GreekUnavailableError, InvalidInputError, UnsupportedOperationError
from .market import BlackScholesMertonParameters, PricingContext

GREEKS = ("delta", "gamma", "speed", "vega", "volga", "vanna", "zomma", "rho",
          "dividend_rho", "theta", "charm", "color")
SPOT_GREEKS = ("delta", "gamma", "speed", "vanna", "zomma", "charm", "color")
VOLATILITY_GREEKS = ("vega", "volga", "vanna", "zomma")
TIME_GREEKS = ("theta", "charm", "color")


@dataclass(frozen=True)
class NumericalShiftSettings:
    """NumericalShiftSettings (risk/analytics.rs:382-421): absolute bumps; None picks
    the automatic spot and volatility bumps."""
    spot_shift: Optional[float] = None
    volatility_shift: Optional[float] = None
    rate_shift: float = 1e-4

    def validate(self):
        for name in ("spot_shift", "volatility_shift"):
            v = getattr(self, name)
            if v is not None and not (math.isfinite(v) and v > 0.0):
                raise InvalidInputError(f"{name} must be positive and finite")
        if not (math.isfinite(self.rate_shift) and self.rate_shift > 0.0):
            raise InvalidInputError("rate_shift must be positive and finite")

    def spot_shift_at(self, spot: float) -> float:
        return self.spot_shift if self.spot_shift is not None else min(0.01, 0.01 * spot)

    def volatility_shift_at(self, volatility: float) -> float:
        return (self.volatility_shift if self.volatility_shift is not None
                else min(1e-4, volatility / 2.0))


@dataclass
class PricingResult:
    """PricingResult (risk/analytics.rs): a price and the requested Greeks.  `status`
    holds, per requested Greek without a value, why: 'stencil_unavailable',
    'undefined' or 'unsupported'."""
    price: float
    greeks: Dict[str, float] = field(default_factory=dict)
    status: Dict[str, str] = field(default_factory=dict)
    seed: Optional[int] = None

    def get(self, greek: str) -> Optional[float]:
        return self.greeks.get(greek)

    def require(self, greek: str) -> float:
        if greek in self.greeks:
            return self.greeks[greek]
        raise GreekUnavailableError(f"{greek}: {self.status.get(greek, 'not_requested')}")


def symmetric_shift(value: float, requested: float) -> float:
    """risk/numerical.rs:11-30: the bump both stencil legs can use exactly."""
    high = value + requested
    shift = high - value
    low = value - shift
    if (math.isfinite(high) and math.isfinite(shift) and shift > 0.0 and math.isfinite(low)
            and value - low == shift):
        return shift
    return 0.0


# A scenario is the BSM market (spot, volatility, rate, dividend).
Scenario = Tuple[float, float, float, float]


def scenario_context(key: Scenario) -> PricingContext:
    spot, vol, rate, dividend = key
    return PricingContext(BlackScholesMertonParameters(rate, dividend, vol), spot)


def _check_request(request: Iterable[str]) -> Tuple[str, ...]:
    request = tuple(request)
    for g in request:
        if g not in GREEKS:
            raise InvalidInputError(f"unknown Greek {g!r}")
    return request


def _stencils(ctx: PricingContext, expiry: float, request, shifts: NumericalShiftSettings,
              discontinuity: Callable[[float], bool], price: Callable[[Scenario], float],
              p0: float) -> PricingResult:
    """complete_greeks_with_pair without native spot Greeks (risk/numerical.rs:331-702)
    and expiry_greeks (33-132).  `price` maps a scenario to its price; with a recording
    `price` this enumerates the scenarios the stencils need."""
    model = ctx.model
    spot, vol, rate, dividend = ctx.spot, model.volatility, model.rate, model.dividend
    result = PricingResult(p0)
    want = lambda g: g in request and g not in result.greeks  # noqa: E731

    def put(g, value):
        if g in request:
            result.greeks[g] = value

    if expiry == 0.0:
        # Terminal payments are independent of volatility and discount rates.
        for g in ("vega", "volga", "rho", "dividend_rho"):
            put(g, 0.0)
        h = symmetric_shift(spot, shifts.spot_shift_at(spot))
        if not discontinuity(0.0) and h > 0.0 and spot > h and not discontinuity(h):
            put("vanna", 0.0)
            put("zomma", 0.0)
            if any(g in request for g in ("delta", "gamma", "speed")):
                up = price((spot + h, vol, rate, dividend))
                down = price((spot - h, vol, rate, dividend))
                put("delta", (up - down) / h / 2.0)
                put("gamma", ((up - p0) - (p0 - down)) / h / h)
                two_h = 2.0 * h
                if ("speed" in request and math.isfinite(two_h) and spot > two_h
                        and symmetric_shift(spot, two_h) == two_h and not discontinuity(two_h)):
                    up2 = price((spot + two_h, vol, rate, dividend))
                    down2 = price((spot - two_h, vol, rate, dividend))
                    put("speed", ((up2 - up) - (up - down) + (down - down2)) / h / h / two_h)
        for g in request:
            if g not in result.greeks:
                result.status[g] = "unsupported" if g in TIME_GREEKS else "stencil_unavailable"
        return result

    h = symmetric_shift(spot, shifts.spot_shift_at(spot))
    v = symmetric_shift(vol, shifts.volatility_shift_at(vol))
    spot_ok = (any(want(g) for g in SPOT_GREEKS) and h > 0.0 and spot > h and not discontinuity(h))
    two_h = 2.0 * h
    speed_ok = (want("speed") and spot_ok and math.isfinite(two_h) and spot > two_h
                and symmetric_shift(spot, two_h) == two_h and not discontinuity(two_h))

    def spot_derivatives(volatility, center):
        up = price((spot + h, volatility, rate, dividend))
        down = price((spot - h, volatility, rate, dividend))
        return (up - down) / h / 2.0, ((up - center) - (center - down)) / h / h

    if spot_ok and (want("delta") or want("gamma") or (want("speed") and speed_ok)):
        up = price((spot + h, vol, rate, dividend))
        down = price((spot - h, vol, rate, dividend))
        if want("delta"):
            put("delta", (up - down) / h / 2.0)
        if want("gamma"):
            put("gamma", ((up - p0) - (p0 - down)) / h / h)
        if want("speed") and speed_ok:
            up2 = price((spot + two_h, vol, rate, dividend))
            down2 = price((spot - two_h, vol, rate, dividend))
            put("speed", ((up2 - up) - (up - down) + (down - down2)) / h / h / two_h)
    if (v > 0.0 and vol > v and math.isfinite(2.0 * v)
            and (want("vega") or want("volga") or (spot_ok and (want("vanna") or want("zomma"))))):
        prices = None
        if want("vega") or want("volga"):
            prices = (price((spot, vol + v, rate, dividend)), price((spot, vol - v, rate, dividend)))
            put("vega", (prices[0] - prices[1]) / (2.0 * v))
            put("volga", ((prices[0] - p0) - (p0 - prices[1])) / v / v)
        if spot_ok and (want("vanna") or want("zomma")):
            if want("zomma"):
                first, last = prices if prices is not None else (
                    price((spot, vol + v, rate, dividend)), price((spot, vol - v, rate, dividend)))
            else:
                first, last = p0, p0
            high = spot_derivatives(vol + v, first)
            low = spot_derivatives(vol - v, last)
            put("vanna", (high[0] - low[0]) / (2.0 * v))
            put("zomma", (high[1] - low[1]) / (2.0 * v))
    if want("rho"):
        r = symmetric_shift(rate, shifts.rate_shift)
        if r > 0.0 and math.isfinite(2.0 * r):
            put("rho", (price((spot, vol, rate + r, dividend)) - price((spot, vol, rate + -r, dividend)))
                / (2.0 * r))
    if want("dividend_rho"):
        q = symmetric_shift(dividend, shifts.rate_shift)
        if q > 0.0 and math.isfinite(2.0 * q):
            put("dividend_rho", (price((spot, vol, rate, dividend + q))
                                 - price((spot, vol, rate, dividend + -q))) / (2.0 * q))
    spot_undefined = discontinuity(0.0)
    for g in request:
        if g in result.greeks:
            continue
        if g in TIME_GREEKS:
            result.status[g] = "unsupported"
        elif (g in SPOT_GREEKS and spot_undefined) or (g in VOLATILITY_GREEKS and vol == 0.0):
            result.status[g] = "undefined"
        else:
            result.status[g] = "stencil_unavailable"
    return result


def vanilla_discontinuity(option, ctx: PricingContext) -> Callable[[float], bool]:
    """EuropeanOption::at_spot_discontinuity (instruments/vanilla.rs): at expiry, a
    stencil reaching the strike; before expiry (positive volatility) none."""
    def check(radius: float) -> bool:
        return (option.expiry == 0.0 and ctx.spot - radius <= option.strike <= ctx.spot + radius)
    return check


def no_discontinuity(option, ctx: PricingContext) -> Callable[[float], bool]:
    """Contracts valued before their first observation: no stencil crosses an event;
    at expiry the terminal stencils are treated as unavailable."""
    def check(radius: float) -> bool:
        return option.expiry == 0.0
    return check


def numerical_greeks(engine, option, ctx: PricingContext, request: Iterable[str],
                     shifts: Optional[NumericalShiftSettings] = None,
                     discontinuity=None) -> PricingResult:
    """kiyosi's `numerical_greeks` (risk/numerical.rs:164-207) for BSM contexts, with a
    seed pinned for every scenario; engines exposing per-contract plans (`_plan`) price
    the base and all bumped scenarios in one book."""
    request = _check_request(request)
    shifts = shifts or NumericalShiftSettings()
    shifts.validate()
    if not isinstance(ctx.model, BlackScholesMertonParameters):
        raise UnsupportedOperationError("numerical Greeks need Black-Scholes-Merton parameters")
    if discontinuity is None:
        from .instruments import EuropeanOption
        discontinuity = (vanilla_discontinuity if type(option) is EuropeanOption
                         else no_discontinuity)(option, ctx)
    pinned = engine.with_resolved_seed()
    base: Scenario = (ctx.spot, ctx.model.volatility, ctx.model.rate, ctx.model.dividend)
    needed: List[Scenario] = [base]

    def record(key: Scenario) -> float:
        if key not in needed:
            needed.append(key)
        return 0.0

    _stencils(ctx, option.expiry, request, shifts, discontinuity, record, 0.0)
    prices = pinned._scenario_prices(option, [scenario_context(k) for k in needed])
    table = dict(zip(needed, prices))
    result = _stencils(ctx, option.expiry, request, shifts, discontinuity, table.__getitem__,
                       table[base])
    for g, value in result.greeks.items():
        if not math.isfinite(value):
            from .errors import ComputationFailureError
            raise ComputationFailureError(f"non-finite {g}")
    result.seed = pinned.seed
    return result


def barrier_discontinuity(option, ctx: PricingContext, radius: float) -> bool:
    """Monitoring::spot_discontinuity (instruments/monitoring.rs:430-444) before expiry:
    a spot stencil reaching a barrier that is monitored now."""
    from .instruments import DoubleBarrierOption
    monitored = option.continuous or option.observation_times[0] == 0.0
    levels = (option.lower, option.upper) if isinstance(option, DoubleBarrierOption) else (option.barrier,)
    return monitored and any(ctx.spot - radius <= level <= ctx.spot + radius for level in levels)


def native_greeks(engine, option, ctx: PricingContext, request, plan_for,
                  shifts: Optional[NumericalShiftSettings] = None, discontinuity=None,
                  resolved_greeks=None, redo_without_control=None) -> PricingResult:
    """The digital, barrier and Asian engines' Greeks (engines.rs:138-160 `greeks`,
    barrier.rs:180-214): delta and gamma from the price's own normals, as the means of
    the paths' likelihood-ratio or pathwise samples.  The price, delta and gamma
    contracts are priced in one book on one seed.  Other Greeks are not supported by
    these engines; at expiry delta and gamma come from terminal stencils."""
    request = _check_request(request)
    shifts = shifts or NumericalShiftSettings()
    shifts.validate()
    supported = [g for g in request if g in ("delta", "gamma")]
    pinned = engine.with_resolved_seed()
    if option.expiry == 0.0:
        def check(radius):
            return discontinuity(radius) if discontinuity is not None else True
        base = pinned._scenario_prices(option, [ctx])[0]
        needed, table = [], {}
        key0 = (ctx.spot, ctx.model.volatility, ctx.model.rate, ctx.model.dividend)

        def record(key):
            if key not in needed and key != key0:
                needed.append(key)
            return 0.0
        _stencils(ctx, 0.0, supported, shifts, check, record, base)
        if needed:
            table = dict(zip(needed, pinned._scenario_prices(option, [scenario_context(k) for k in needed])))
        table[key0] = base
        result = _stencils(ctx, 0.0, supported, shifts, check, table.__getitem__, base)
    else:
        h = symmetric_shift(ctx.spot, shifts.spot_shift_at(ctx.spot))
        blocked = discontinuity is not None and discontinuity(h)
        wanted = [] if blocked else supported
        plan = plan_for(option, ctx)
        from . import plans as _plans
        if isinstance(plan, _plans.Known):
            result = PricingResult(plan.value)
            greek_values = resolved_greeks(option, ctx) if resolved_greeks else {"delta": 0.0, "gamma": 0.0}
            for g in wanted:
                result.greeks[g] = greek_values[g]
        else:
            book = [plan] + [_plans.greek_output(plan, g) for g in wanted]
            estimates = pinned._run(ctx, book)
            if redo_without_control is not None and estimates[0].price < 0.0:
                alternative = redo_without_control(option, ctx)
                if alternative is not None:
                    book = [alternative] + [_plans.greek_output(alternative, g) for g in wanted]
                    estimates = pinned._run(ctx, book)
            result = PricingResult(estimates[0].price)
            for g, e in zip(wanted, estimates[1:]):
                result.greeks[g] = e.price
            if plan.addend is not None and wanted:
                # The analytic part's own spot stencils (barrier.rs:489-523).
                def addend_price(key):
                    return plan.addend(scenario_context(key))
                key0 = (ctx.spot, ctx.model.volatility, ctx.model.rate, ctx.model.dividend)
                extra = _stencils(ctx, option.expiry, wanted, shifts,
                                  discontinuity if discontinuity is not None else (lambda r: False),
                                  addend_price, addend_price(key0))
                for g in wanted:
                    if g in extra.greeks:
                        result.greeks[g] += extra.greeks[g]
                    else:
                        result.greeks.pop(g, None)
        for g in supported:
            if g not in result.greeks:
                result.status[g] = "stencil_unavailable"
    for g in request:
        if g not in supported:
            result.status[g] = "unsupported"
    for g, value in result.greeks.items():
        if not math.isfinite(value):
            from .errors import ComputationFailureError
            raise ComputationFailureError(f"non-finite {g}")
    result.seed = pinned.seed
    return result
