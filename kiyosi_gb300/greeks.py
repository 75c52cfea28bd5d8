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

Time Greeks (theta, charm, color; risk/numerical.rs:213-275, 594-630) move the valuation
instant: with flat rates and year-fraction times, pricing at valuation + t is pricing the
instrument with every time moved by -t.  The stencil is the reference's on whole
microseconds of Actual/365 Fixed time: one day (or the requested shift), capped at an
eighth of the remaining life and by the contract's start, halved until no observation
the instrument's rule names lies inside it.  Theta is the price's difference across the
stencil, charm and color those of the spot stencils' delta and gamma.  European and
American options, autocallable notes and accumulators have the rule; other instruments
report `unsupported`.
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


# Microseconds per Actual/365 Fixed year (time/date.rs:255-257).
YEAR_MICROS = 365 * 86_400 * 1_000_000


@dataclass(frozen=True)
class NumericalShiftSettings:
    """NumericalShiftSettings (risk/analytics.rs:382-464): absolute bumps; None picks
    the automatic spot, volatility and time bumps.  `time_shift` is in Actual/365 Fixed
    years and must be a whole number of microseconds (one day by default)."""
    spot_shift: Optional[float] = None
    volatility_shift: Optional[float] = None
    rate_shift: float = 1e-4
    time_shift: Optional[float] = None

    def validate(self):
        for name in ("spot_shift", "volatility_shift"):
            v = getattr(self, name)
            if v is not None and not (math.isfinite(v) and v > 0.0):
                raise InvalidInputError(f"{name} must be positive and finite")
        if not (math.isfinite(self.rate_shift) and self.rate_shift > 0.0):
            raise InvalidInputError("rate_shift must be positive and finite")
        self.time_shift_micros()

    def time_shift_micros(self) -> int:
        """NumericalShiftSettings::time_shift_micros (risk/analytics.rs:453-463)."""
        if self.time_shift is None:
            return 86_400 * 1_000_000
        micros = self.time_shift * YEAR_MICROS if math.isfinite(self.time_shift) else math.nan
        if not (micros >= 1.0 and abs(micros - round(micros)) <= 1e-6 * max(1.0, micros)):
            raise InvalidInputError("time_shift must be positive with whole-microsecond precision")
        return int(round(micros))

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


# A scenario is the BSM market (spot, volatility, rate, dividend), plus, for the time
# stencils, the valuation shift in years (a fifth entry; absent means no shift).
Scenario = Tuple[float, ...]


def scenario_context(key: Scenario) -> PricingContext:
    spot, vol, rate, dividend = key[:4]
    return PricingContext(BlackScholesMertonParameters(rate, dividend, vol), spot)


def _at(spot, vol, rate, dividend, shift: float) -> Scenario:
    """The scenario valued `shift` years later (the plain market when shift is 0)."""
    return (spot, vol, rate, dividend) if shift == 0.0 else (spot, vol, rate, dividend, shift)


# ---- time stencils (risk/numerical.rs:213-275) ----

@dataclass(frozen=True)
class TimeRule:
    """How an instrument moves in time: the start of its life (OptionContract::
    valuation_start; None for none), the instrument valued `t` years later, and whether a
    stencil [before, after] (years) keeps its history regime (time_stencil_available)."""
    start: Optional[float]
    valued_at: Callable[[float], object]
    available: Callable[[float, float], bool]


def _inside(times, before: float, after: float) -> bool:
    return any(before <= t <= after for t in times)


def time_rule(option) -> Optional[TimeRule]:
    """The TimeRule of the instruments whose engines take numerical Greeks."""
    from .instruments import Accumulator, AmericanOption, AutocallableNote, EuropeanOption
    if type(option) in (EuropeanOption, AmericanOption):
        # vanilla.rs:181-200, 375-377: no valuation start, every stencil available
        return TimeRule(None, lambda t: replace(option, expiry=option.expiry - t), lambda b, a: True)
    if isinstance(option, AutocallableNote):
        def shifted(t):
            times = None if option.knock_in_times is None else [x - t for x in option.knock_in_times]
            return replace(option, expiry=option.expiry - t, effective_time=option.effective_time - t,
                           observations=tuple(replace(o, time=o.time - t) for o in option.observations),
                           knock_in_times=times)

        def available(before, after):
            # AutocallableNote::time_stencil_available (instruments/autocallable.rs:1556-1582)
            from . import plans
            from .errors import KiyosiError
            try:
                plans.autocallable_prior(shifted(before))
            except KiyosiError:
                return False
            if option.barrier_state == "knocked_out":
                return True
            if _inside([o.time for o in option.observations], before, after):
                return False
            if (option.daily_knock_in and option.barrier_state != "knocked_in"
                    and option.knock_in_affects_payoff()
                    and _inside(option.knock_in_times, max(before, option.effective_time),
                                min(after, option.expiry))):
                return False
            return True
        return TimeRule(option.effective_time, shifted, available)
    if isinstance(option, Accumulator):
        # Accumulator::time_stencil_available (instruments/accumulator.rs:664-680).  This
        # package's accumulators list only dates after valuation and carry their history
        # as a quantity, so the valuation is the start of their life.
        def available(before, after):
            if option.knock_out_settled:
                return True
            return not (_inside(option.accumulation_times, before, after)
                        or _inside(option.knock_out_times, before, after))
        return TimeRule(0.0, lambda t: replace(
            option, expiry=option.expiry - t, accumulation_times=[x - t for x in option.accumulation_times],
            knock_out_times=[x - t for x in option.knock_out_times]), available)
    return None


def time_stencil(rule: TimeRule, expiry: float, shifts: NumericalShiftSettings) -> Optional[Tuple[int, int]]:
    """time_stencil (risk/numerical.rs:213-275) under flat curves: (before, after) in
    microseconds from valuation, or None.  The widths to the start of the contract's life
    and to expiry are whole microseconds (floored)."""
    before_width = math.inf if rule.start is None else math.floor(-rule.start * YEAR_MICROS)
    after_width = math.floor(expiry * YEAR_MICROS)
    radius = shifts.time_shift_micros()
    shift = min(radius, max(0, before_width + after_width))
    if shifts.time_shift is None:
        # Near expiry the price is far from linear in time: keep the stencil away from it.
        shift = min(shift, max(after_width // 8, 1))
    if before_width > 0 and after_width > 0:
        shift = min(shift, before_width, after_width)
    shift = int(shift)

    def legs(width):
        return -int(min(width, before_width)), int(min(width, after_width))

    def available(b, a):
        return rule.available(b / YEAR_MICROS, a / YEAR_MICROS)
    before, after = legs(shift)
    while shifts.time_shift is None and shift > 1 and not available(before, after):
        shift //= 2
        before, after = legs(shift)
    return (before, after) if before != after and available(before, after) else None


def _check_request(request: Iterable[str]) -> Tuple[str, ...]:
    request = tuple(request)
    for g in request:
        if g not in GREEKS:
            raise InvalidInputError(f"unknown Greek {g!r}")
    return request


def _stencils(ctx: PricingContext, expiry: float, request, shifts: NumericalShiftSettings,
              discontinuity: Callable[[float], bool], price: Callable[[Scenario], float],
              p0: float, stencil: Optional[Tuple[int, int]] = None,
              time_supported: bool = False) -> PricingResult:
    """complete_greeks_with_pair without native spot Greeks (risk/numerical.rs:331-702)
    and expiry_greeks (33-132).  `price` maps a scenario to its price; with a recording
    `price` this enumerates the scenarios the stencils need.  `stencil` is the time
    stencil in microseconds (None: unavailable); `time_supported` whether the instrument
    has time Greeks at all."""
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
                result.status[g] = ("unsupported" if g in TIME_GREEKS and not time_supported
                                    else "stencil_unavailable")
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
    if time_supported and stencil is not None and (want("theta") or want("charm") or want("color")):
        # risk/numerical.rs:594-630: prices at both ends of the stencil (the base price at
        # an end on valuation), then the spot stencils' delta and gamma at both ends.
        before, after = stencil[0] / YEAR_MICROS, stencil[1] / YEAR_MICROS
        years = (stencil[1] - stencil[0]) / YEAR_MICROS

        def at(shift, s=spot):
            return p0 if shift == 0.0 and s == spot else price(_at(s, vol, rate, dividend, shift))
        prices = None
        if want("theta"):
            prices = (at(after), at(before))
            put("theta", (prices[0] - prices[1]) / years)
        if spot_ok and (want("charm") or want("color")):
            if want("color"):
                first, last = (prices[1], prices[0]) if prices is not None else (at(before), at(after))
            else:
                first, last = p0, p0

            def derivatives(shift, center):
                up, down = at(shift, spot + h), at(shift, spot - h)
                return (up - down) / h / 2.0, ((up - center) - (center - down)) / h / h
            low, high = derivatives(before, first), derivatives(after, last)
            put("charm", (high[0] - low[0]) / years)
            put("color", (high[1] - low[1]) / years)
    spot_undefined = discontinuity(0.0)
    for g in request:
        if g in result.greeks:
            continue
        if g in TIME_GREEKS and not time_supported:
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
    rule = time_rule(option)
    stencil = None
    if rule is not None and option.expiry > 0.0 and any(g in request for g in TIME_GREEKS):
        stencil = time_stencil(rule, option.expiry, shifts)

    def record(key: Scenario) -> float:
        if key not in needed:
            needed.append(key)
        return 0.0

    _stencils(ctx, option.expiry, request, shifts, discontinuity, record, 0.0, stencil, rule is not None)
    prices = _scenario_prices(pinned, option, rule, needed)
    table = dict(zip(needed, prices))
    result = _stencils(ctx, option.expiry, request, shifts, discontinuity, table.__getitem__,
                       table[base], stencil, rule is not None)
    for g, value in result.greeks.items():
        if not math.isfinite(value):
            from .errors import ComputationFailureError
            raise ComputationFailureError(f"non-finite {g}")
    result.seed = pinned.seed
    return result


def _scenario_prices(pinned, option, rule: Optional[TimeRule], keys: List[Scenario]) -> List[float]:
    """Prices the scenarios on the pinned seed: the instrument valued at each scenario's
    shift, in one book when the engine prices (contract, context) pairs
    (`_scenario_prices_of`), else one call per shift."""
    def instrument(key):
        return option if len(key) == 4 else rule.valued_at(key[4])
    pairs_call = getattr(pinned, "_scenario_prices_of", None)
    if pairs_call is not None:
        return pairs_call([(instrument(k), scenario_context(k)) for k in keys])
    out: List[Optional[float]] = [None] * len(keys)
    groups: Dict[float, List[int]] = {}
    for i, k in enumerate(keys):
        groups.setdefault(0.0 if len(k) == 4 else k[4], []).append(i)
    for shift, members in groups.items():
        prices = pinned._scenario_prices(instrument(keys[members[0]]), [scenario_context(keys[i]) for i in members])
        for i, p in zip(members, prices):
            out[i] = p
    return out


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
