"""Numerical Greeks (risk/numerical.rs): bump-and-reprice with a pinned seed, the base
and every bumped scenario priced as one book.

CPU checks:
- the stencil logic on the oracle: the batched book reproduces scalar pricing of each
  bumped context bit for bit;
- European Monte Carlo Greeks near the Black-Scholes closed forms;
- the reference's default shifts and its symmetric-bump rule.

GPU checks: the engines' price_with_greeks against scalar prices of the bumped contexts,
and the European Greeks against the closed forms.
"""
import math

import pytest

from kiyosi_gb300 import greeks, plans
from kiyosi_gb300.errors import GreekUnavailableError, InvalidInputError
from kiyosi_gb300.instruments import EuropeanOption
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from oracle import loader

from helpers import c2_context, pack, settings, snowball_c2


def _ncdf(x):
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


def _npdf(x):
    return math.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def _bs_greeks(sign, s, k, t, r, q, v):
    sq = v * math.sqrt(t)
    d1 = (math.log(s / k) + (r - q + 0.5 * v * v) * t) / sq
    d2 = d1 - sq
    delta = sign * math.exp(-q * t) * _ncdf(sign * d1)
    gamma = math.exp(-q * t) * _npdf(d1) / (s * sq)
    vega = s * math.exp(-q * t) * _npdf(d1) * math.sqrt(t)
    rho = sign * k * t * math.exp(-r * t) * _ncdf(sign * d2)
    dividend_rho = -sign * s * t * math.exp(-q * t) * _ncdf(sign * d1)
    return dict(delta=delta, gamma=gamma, vega=vega, rho=rho, dividend_rho=dividend_rho)


class OracleEngine:
    """Stand-in for a GPU engine on the CPU: the same plan builder, priced by the oracle."""

    def __init__(self, plan, paths, seed, sobol=False):
        self.plan, self.paths, self.seed, self.sobol = plan, paths, seed, sobol

    def with_resolved_seed(self):
        return self

    def _scenario_prices(self, contract, contexts):
        plan_list = [self.plan(contract, c) for c in contexts]
        sampled = [p for p in plan_list if not isinstance(p, plans.Known)]
        out = iter(loader.price_book(contexts[0], pack(sampled),
                                     settings(self.paths, self.seed, sobol=self.sobol))
                   if sampled else [])
        return [p.value if isinstance(p, plans.Known) else next(out).price for p in plan_list]

    def price(self, contract, ctx):
        return self._scenario_prices(contract, [ctx])[0]


def _ctx(spot=100.0, vol=0.2, rate=0.05, dividend=0.02):
    return PricingContext(BlackScholesMertonParameters(rate, dividend, vol), spot)


def test_symmetric_shift_and_default_bumps():
    assert greeks.symmetric_shift(100.0, 0.01) == (100.0 + 0.01) - 100.0
    assert greeks.symmetric_shift(1e300, 1e-4) == 0.0  # collapses
    s = greeks.NumericalShiftSettings()
    assert s.spot_shift_at(100.0) == 0.01 and s.spot_shift_at(0.5) == 0.005
    assert s.volatility_shift_at(0.2) == 1e-4 and s.volatility_shift_at(1e-4) == 5e-5
    assert s.rate_shift == 1e-4
    with pytest.raises(InvalidInputError):
        greeks.NumericalShiftSettings(spot_shift=-1.0).validate()


def test_batched_scenarios_equal_scalar_bumped_prices():
    ctx = _ctx()
    option = EuropeanOption("call", 105.0, 1.0)
    engine = OracleEngine(plans.european, 1 << 14, 11)
    request = ("delta", "gamma", "speed", "vega", "volga", "vanna", "zomma", "rho",
               "dividend_rho", "theta")
    r = greeks.numerical_greeks(engine, option, ctx, request)
    price = lambda s, v, rr, q: engine.price(option, _ctx(s, v, rr, q))  # noqa: E731
    h = greeks.symmetric_shift(100.0, 0.01)
    v = greeks.symmetric_shift(0.2, 1e-4)
    p0 = price(100.0, 0.2, 0.05, 0.02)
    up, down = price(100.0 + h, 0.2, 0.05, 0.02), price(100.0 - h, 0.2, 0.05, 0.02)
    assert r.price == p0
    assert r.get("delta") == (up - down) / h / 2.0
    assert r.get("gamma") == ((up - p0) - (p0 - down)) / h / h
    vu, vd = price(100.0, 0.2 + v, 0.05, 0.02), price(100.0, 0.2 - v, 0.05, 0.02)
    assert r.get("vega") == (vu - vd) / (2.0 * v)
    assert r.get("volga") == ((vu - p0) - (p0 - vd)) / v / v
    dr = greeks.symmetric_shift(0.05, 1e-4)
    assert r.get("rho") == (price(100.0, 0.2, 0.05 + dr, 0.02) - price(100.0, 0.2, 0.05 - dr, 0.02)) / (2 * dr)
    # theta: the option valued one day later and one day earlier (a European option has
    # no start of life, so the stencil is central: one day, capped at an eighth of life)
    day = 86_400_000_000 / greeks.YEAR_MICROS
    later = engine.price(EuropeanOption("call", 105.0, 1.0 - day), ctx)
    earlier = engine.price(EuropeanOption("call", 105.0, 1.0 - -day), ctx)
    assert r.get("theta") == (later - earlier) / (2 * 86_400_000_000 / greeks.YEAR_MICROS)
    with pytest.raises(GreekUnavailableError):
        r.require("charm")


def test_european_monte_carlo_greeks_near_closed_forms():
    ctx = _ctx()
    for sign, kind in ((1.0, "call"), (-1.0, "put")):
        option = EuropeanOption(kind, 100.0, 1.0)
        engine = OracleEngine(plans.european, 1 << 18, 42)
        r = greeks.numerical_greeks(engine, option, ctx, ("delta", "vega", "rho", "dividend_rho"))
        exact = _bs_greeks(sign, 100.0, 100.0, 1.0, 0.05, 0.02, 0.2)
        assert abs(r.get("delta") - exact["delta"]) < 0.01, (kind, r.greeks, exact)
        assert abs(r.get("vega") - exact["vega"]) < 0.5
        assert abs(r.get("rho") - exact["rho"]) < 0.5
        assert abs(r.get("dividend_rho") - exact["dividend_rho"]) < 0.5


def test_expiry_greeks_use_terminal_stencils():
    ctx = _ctx()
    engine = OracleEngine(plans.european, 1 << 10, 3)
    itm = greeks.numerical_greeks(engine, EuropeanOption("call", 90.0, 0.0), ctx,
                                  ("delta", "gamma", "vega", "rho", "vanna"))
    assert itm.get("delta") == pytest.approx(1.0, abs=1e-9) and itm.get("gamma") == 0.0
    assert itm.get("vega") == 0.0 and itm.get("rho") == 0.0 and itm.get("vanna") == 0.0
    at = greeks.numerical_greeks(engine, EuropeanOption("call", 100.0, 0.0), ctx, ("delta", "vega"))
    assert at.get("delta") is None and at.status["delta"] == "stencil_unavailable"
    assert at.get("vega") == 0.0


@pytest.mark.gpu
def test_engine_greeks_equal_scalar_bumped_prices(native):
    from kiyosi_gb300.pricing import MonteCarloAutocallableEngine, MonteCarloVanillaEngine
    ctx = _ctx()
    option = EuropeanOption("put", 95.0, 1.0)
    engine = MonteCarloVanillaEngine(path_count=1 << 16, seed=5)
    r = engine.price_with_greeks(option, ctx, ("delta", "gamma", "vega", "rho", "dividend_rho"))
    h = greeks.symmetric_shift(100.0, 0.01)
    up = engine.price(option, _ctx(100.0 + h))
    down = engine.price(option, _ctx(100.0 - h))
    assert r.price == engine.price(option, ctx)
    assert r.get("delta") == (up - down) / h / 2.0
    exact = _bs_greeks(-1.0, 100.0, 95.0, 1.0, 0.05, 0.02, 0.2)
    assert abs(r.get("delta") - exact["delta"]) < 0.01
    assert abs(r.get("vega") - exact["vega"]) < 0.5
    # A snowball: every bumped note in one book with the base note.
    note_ctx = c2_context()
    note = snowball_c2()
    auto = MonteCarloAutocallableEngine(path_count=1 << 14, seed=9, sampling="sobol")
    g = auto.price_with_greeks(note, note_ctx, ("delta", "vega"))
    spot = note_ctx.spot
    h = greeks.symmetric_shift(spot, min(0.01, 0.01 * spot))
    bumped = lambda s: PricingContext(note_ctx.model, s)  # noqa: E731
    assert g.price == auto.price(note, note_ctx)
    assert g.get("delta") == (auto.price(note, bumped(spot + h)) - auto.price(note, bumped(spot - h))) / h / 2.0


def _bs_time_greeks(sign, s, k, t, r, q, v):
    """Closed-form theta (d price / d valuation time), charm (d delta / d valuation time)."""
    sq = v * math.sqrt(t)
    d1 = (math.log(s / k) + (r - q + 0.5 * v * v) * t) / sq
    d2 = d1 - sq
    theta = (-s * math.exp(-q * t) * _npdf(d1) * v / (2.0 * math.sqrt(t))
             - sign * r * k * math.exp(-r * t) * _ncdf(sign * d2)
             + sign * q * s * math.exp(-q * t) * _ncdf(sign * d1))
    charm = (sign * q * math.exp(-q * t) * _ncdf(sign * d1)
             - math.exp(-q * t) * _npdf(d1) * (2.0 * (r - q) * t - d2 * sq) / (2.0 * t * sq))
    return theta, charm


def test_european_time_greeks_near_closed_forms():
    ctx = _ctx()
    for sign, kind in ((1.0, "call"), (-1.0, "put")):
        option = EuropeanOption(kind, 100.0, 1.0)
        engine = OracleEngine(plans.european, 1 << 16, 3)
        r = greeks.numerical_greeks(engine, option, ctx, ("theta", "charm", "color"))
        theta, charm = _bs_time_greeks(sign, 100.0, 100.0, 1.0, 0.05, 0.02, 0.2)
        assert abs(r.get("theta") - theta) < 0.03 * abs(theta) + 0.02, (kind, r.get("theta"), theta)
        assert abs(r.get("charm") - charm) < 0.25 * abs(charm) + 0.02, (kind, r.get("charm"), charm)
        assert math.isfinite(r.get("color"))


def _note(effective=0.0, state=None, daily=True, first=21):
    from kiyosi_gb300.instruments import AutocallableNote, Observation
    dt = 1.0 / 252.0
    times = [effective + dt * (i + 1) for i in range(252)]
    past = [t for t in (effective + dt * k for k in range(0, 400)) if t < 0.0]
    obs = [Observation(times[first * (m + 1) - 1], knock_out_level=103.0, coupon_rate=0.1) for m in range(12)]
    return AutocallableNote(initial_spot=100.0, expiry=times[-1], observations=obs, knock_in_level=80.0,
                            knock_in_times=(past + [t for t in times if t >= 0.0]) if daily else None,
                            upper_strike=100.0, maturity_coupon_rate=0.1, effective_time=effective,
                            barrier_state=state)


def test_time_stencils():
    s = greeks.NumericalShiftSettings()
    day = 86_400_000_000
    # a European option: central, one day
    rule = greeks.time_rule(EuropeanOption("call", 100.0, 1.0))
    assert greeks.time_stencil(rule, 1.0, s) == (-day, day)
    # an eighth of the remaining life near expiry
    assert greeks.time_stencil(rule, 2.0 / 365.0, s) == (-day // 4, day // 4)
    # a note valued at its start: forward only; the first monitoring date is 1/252 year
    # away, beyond one day
    note = _note()
    assert greeks.time_stencil(greeks.time_rule(note), note.expiry, s) == (0, day)
    # a seasoned note between two monitoring dates: central, halved until the window
    # clears them
    seasoned = _note(effective=-0.5 / 252.0, state="no_event")
    before, after = greeks.time_stencil(greeks.time_rule(seasoned), seasoned.expiry, s)
    assert before == -after and 0 < after < 0.5 * greeks.YEAR_MICROS / 252.0
    assert not any(before / greeks.YEAR_MICROS <= t <= after / greeks.YEAR_MICROS
                   for t in seasoned.knock_in_times)
    # knock-in no longer matters once knocked in: monitoring dates do not block, and the
    # start of the note's life caps the stencil
    knocked = _note(effective=-0.5 / 252.0, state="knocked_in")
    width = math.floor(0.5 / 252.0 * greeks.YEAR_MICROS)
    assert greeks.time_stencil(greeks.time_rule(knocked), knocked.expiry, s) == (-width, width)
    # an explicit shift is not shortened for observations: none for a note seasoned ten
    # days whose window then holds monitoring dates
    explicit = greeks.NumericalShiftSettings(time_shift=2.0 / 252.0)
    older = _note(effective=-10.5 / 252.0, state="no_event")
    assert greeks.time_stencil(greeks.time_rule(older), older.expiry, explicit) is None
    assert greeks.time_stencil(greeks.time_rule(older), older.expiry, s) is not None
    with pytest.raises(InvalidInputError):
        greeks.NumericalShiftSettings(time_shift=0.3e-13).validate()


def test_autocallable_theta_is_the_shifted_prices_difference():
    ctx = c2_context()
    note = _note()
    engine = OracleEngine(plans.autocallable, 1 << 13, 9)
    r = greeks.numerical_greeks(engine, note, ctx, ("theta", "delta", "charm"))
    rule = greeks.time_rule(note)
    before, after = greeks.time_stencil(rule, note.expiry, greeks.NumericalShiftSettings())
    assert before == 0
    later = engine.price(rule.valued_at(after / greeks.YEAR_MICROS), ctx)
    assert r.get("theta") == (later - r.price) / ((after - before) / greeks.YEAR_MICROS)
    assert math.isfinite(r.get("charm"))


def test_observation_at_valuation_blocks_the_time_stencil():
    from kiyosi_gb300.instruments import AutocallableNote, Observation
    note = AutocallableNote(initial_spot=100.0, expiry=1.0, observations=[Observation(0.0, 110.0, None, 0.1),
                                                                         Observation(1.0, 103.0, None, 0.1)],
                            knock_in_level=80.0, upper_strike=100.0, maturity_coupon_rate=0.1,
                            barrier_state="no_event")
    assert greeks.time_stencil(greeks.time_rule(note), 1.0, greeks.NumericalShiftSettings()) is None
    engine = OracleEngine(plans.autocallable, 1 << 10, 9)
    r = greeks.numerical_greeks(engine, note, c2_context(), ("theta", "delta"))
    assert r.status["theta"] == "stencil_unavailable" and "delta" in r.greeks


@pytest.mark.gpu
def test_engine_time_greeks_on_the_gpu(native):
    """The engines' theta, charm and color on the GB300: the same stencils as the oracle
    engine's (FP64 to 1e-9), one book for every scenario, and theta near the closed form."""
    from kiyosi_gb300.pricing import MonteCarloAutocallableEngine, MonteCarloVanillaEngine
    ctx = _ctx()
    option = EuropeanOption("call", 100.0, 1.0)
    engine = MonteCarloVanillaEngine(path_count=1 << 16, seed=3)
    r = engine.price_with_greeks(option, ctx, ("theta", "charm", "color", "delta"))
    ref = greeks.numerical_greeks(OracleEngine(plans.european, 1 << 16, 3), option, ctx,
                                  ("theta", "charm", "color", "delta"))
    for g in ("theta", "charm", "color", "delta"):
        assert abs(r.get(g) - ref.get(g)) <= 1e-9 * max(1.0, abs(ref.get(g))), (g, r.get(g), ref.get(g))
    theta, charm = _bs_time_greeks(1.0, 100.0, 100.0, 1.0, 0.05, 0.02, 0.2)
    assert abs(r.get("theta") - theta) < 0.03 * abs(theta)
    # a note valued at its start (forward stencil), FP64 and FP32
    note_ctx = c2_context()
    note = _note()
    ref = greeks.numerical_greeks(OracleEngine(plans.autocallable, 1 << 13, 9), note, note_ctx, ("theta", "delta"))
    auto = MonteCarloAutocallableEngine(path_count=1 << 13, seed=9)
    got = auto.price_with_greeks(note, note_ctx, ("theta", "delta"))
    assert abs(got.get("theta") - ref.get("theta")) <= 1e-8 * max(1.0, abs(ref.get("theta")))
    fast = MonteCarloAutocallableEngine(path_count=1 << 13, seed=9, precision="fp32").price_with_greeks(
        note, note_ctx, ("theta",))
    # FP32 paths on the same normals: a path whose knock-out flips moves theta by about
    # a payment / paths / one day
    assert abs(fast.get("theta") - ref.get("theta")) < 0.2 * abs(ref.get("theta")) + 0.3, (
        fast.get("theta"), ref.get("theta"))
