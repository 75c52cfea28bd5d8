"""Autocallable books on a shared daily grid (engines/monte_carlo/autocallable/portfolio.rs).

CPU checks:
* The lane decomposition against the oracle's literal restatement of the reference's
  multi-lane path loop (SharedEvents::new, shared_payoffs, price_with_strips). Each lane
  is priced as its own bridged contract over the group's intervals, with the group's
  sampling dimensions. Lane prices are bit-identical to the loop's. The loop's
  knock-out and knock-in strip sums agree with lane prices to rounding.
* The reference's own portfolio tests, restated on the oracle:
  - coupon-family prices equal two-lane quotes within 2e-14, including a mixed book with
    an outlier (crates/kiyosi/tests/autocallable_monte_carlo.rs:130-210);
  - equal coupons give bit-equal prices;
  - singletons take the scalar quote;
  - without the shared grid, every quote is the scalar quote
    (autocallable_monte_carlo.rs:100-128);
  - the batch-size limit.

GPU checks: the CUDA lanes against the oracle's loop, and the engine's
price_many_on_shared_grid against the same book priced by the oracle.
"""
import datetime
import math

import pytest

from kiyosi_gb300 import portfolio, plans
from kiyosi_gb300.errors import InvalidInputError
from kiyosi_gb300.instruments import Observation, PhoenixOption, SnowballOption
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
from oracle import loader

from helpers import gpu_price, pack, settings

# multi_event_terms (crates/kiyosi/tests/support/autocallable.rs:3-70): a note from
# 2025-01-01 to 2025-04-01 observed on Feb 3, Mar 3 and Apr 1, knock-in monitored every
# weekday; times are ACT/365 year fractions from the valuation date.
_START = datetime.date(2025, 1, 1)


def _year(d):
    return (d - _START).days / 365.0


def _weekdays(last_day):
    days = [_START + datetime.timedelta(k) for k in range(1, last_day + 1)]
    return [_year(d) for d in days if d.weekday() < 5]


_DATES = [_year(datetime.date(2025, 2, 3)), _year(datetime.date(2025, 3, 3)),
          _year(datetime.date(2025, 4, 1))]
_EXPIRY = _DATES[-1]
_DAILY = _weekdays(90)


def snowball(coupon=0.06, knock_in=95.0, knock_out=(110.0, 108.0, 105.0), dates=None):
    dates = dates or _DATES
    return SnowballOption(coupon, 100.0, knock_in, 100.0, 60.0, dates[-1],
                          [Observation(t, k, None, 0.08) for t, k in zip(dates, knock_out)],
                          knock_in_times=[t for t in _DAILY if t <= dates[-1]])


def phoenix(coupon=0.08, knock_in=95.0):
    return PhoenixOption(coupon, 100.0, knock_in, 100.0, 60.0, _EXPIRY,
                         [Observation(t, k, 100.0, 0.0) for t, k in zip(_DATES, (110.0, 108.0, 105.0))],
                         knock_in_times=_DAILY)


def _ctx(vol=0.25):
    return PricingContext(BlackScholesMertonParameters(0.03, 0.01, vol), 100.0)


class OracleBookEngine:
    """The engine surface portfolio.price_many uses, priced by the oracle."""

    def __init__(self, paths, seed, sobol=False, antithetic=False):
        self.s = settings(paths, seed, sobol=sobol, antithetic=antithetic)

    def _run(self, ctx, batch):
        return loader.price_book(ctx, pack(batch), self.s)


def _lanes(notes, ctx):
    lanes = [portfolio.shared_lane(n, ctx, i) for i, n in enumerate(notes)]
    assert all(lane is not None for lane in lanes)
    return lanes


SAMPLINGS = [dict(sobol=False), dict(sobol=False, antithetic=True), dict(sobol=True)]


@pytest.mark.parametrize("sampling", SAMPLINGS)
def test_lanes_replay_the_group_path_loop(sampling):
    ctx = _ctx()
    # a coupon family, a lower knock-in, a lower knock-out and a shorter aligned grid
    notes = [snowball(c) for c in (0.02, 0.08, -0.01)] + [
        snowball(knock_in=85.0), snowball(knock_out=(104.0,) * 3),
        snowball(dates=[_DATES[0], _DATES[1]], knock_out=(110.0, 108.0)), phoenix()]
    lanes = _lanes(notes, ctx)
    assert [lane.maturity_on_grid for lane in lanes] == [True] * len(notes)
    packed = pack(portfolio.lane_plans(lanes, ctx.spot))
    s = settings(4096, 42, **sampling)
    lane_prices = [e.price for e in loader.price_book(ctx, packed, s)]
    loop, _ = loader.price_shared_group(ctx, packed, s)
    assert lane_prices == loop


def test_interval_plan_bridges_long_runs_only():
    ctx = _ctx()
    # Dates of the shorter note split the first run; a run of fewer than eight days
    # between two cash dates is stepped day by day.
    early = snowball(dates=[_DATES[0], _year(datetime.date(2025, 2, 10))], knock_out=(110.0, 108.0))
    lanes = _lanes([snowball(), early], ctx)
    base, intervals, daily = portfolio.interval_plan(lanes, ctx.spot)
    ends = [end for end, _, _ in intervals]
    assert ends == sorted(ends) and ends[-1] == len(base.steps) - 1
    first = ends.index(lanes[1].events[0][0])
    # the first cash date ends a bridged run; the three days after it step one by one
    assert ends[first + 1:first + 4] == [ends[first] + 1, ends[first] + 2, ends[first] + 3]
    bridged = [i for i in range(len(daily)) if daily["weight"][i] > 0.0]
    assert bridged and all(0.0 < daily["weight"][i] < 1.0 for i in bridged)
    s = settings(2048, 9)
    packed = pack(portfolio.lane_plans(lanes, ctx.spot))
    assert [e.price for e in loader.price_book(ctx, packed, s)] == \
        loader.price_shared_group(ctx, packed, s)[0]


@pytest.mark.parametrize("sampling", SAMPLINGS)
def test_threshold_strips_equal_lane_prices(sampling):
    """Knock-out and knock-in level families priced by the reference's bucket sums
    agree with the same notes priced as lanes."""
    ctx = _ctx()
    notes = ([snowball(knock_out=(k,) * 3) for k in (103.0, 106.0, 101.0, 109.0)]
             + [snowball(knock_in=k) for k in (90.0, 80.0, 95.0)] + [snowball(0.03)])
    lanes = _lanes(notes, ctx)
    s = settings(4096, 7, **sampling)
    by_index = {lane.index: p for lane, p in zip(
        lanes, (e.price for e in loader.price_book(ctx, pack(portfolio.lane_plans(lanes, ctx.spot)), s)))}
    order, strips = portfolio.threshold_strips(lanes, ctx.spot)
    kinds = sorted(strip[0] for strip in strips if strip is not None)
    assert kinds == [portfolio.KNOCK_OUT, portfolio.KNOCK_IN]
    ordered = [lanes[i] for i in order]
    packed = pack(portfolio.lane_plans(ordered, ctx.spot))
    loop, members = loader.price_shared_group(
        ctx, packed, s, [None if st is None else (st[0], st[1]) for st in strips])
    checked = 0
    for lane, price, strip, member in zip(ordered, loop, strips, members):
        if strip is None:
            assert price == by_index[lane.index]
            continue
        for index, value in zip(strip[2], member):
            assert abs(value - by_index[index]) <= 1e-13 * max(1.0, abs(value)), (index, value)
            checked += 1
    assert checked == 7


def _quotes(engine, notes, ctx):
    return portfolio.price_many(engine, notes, ctx, True)


@pytest.mark.parametrize("sampling", [dict(sobol=False, antithetic=True), dict(sobol=True)])
@pytest.mark.parametrize("make", [snowball, phoenix])
def test_coupon_families_match_two_lane_quotes(make, sampling):
    """shared_portfolio_coupon_strips_match_two_lane_quotes
    (autocallable_monte_carlo.rs:141-174)."""
    ctx = _ctx()
    engine = OracleBookEngine(4096, 42, **sampling)
    notes = [make(c) for c in (0.02, 0.08, -0.01, 0.02, 0.04)]
    book = portfolio.plan_book(notes, ctx, True)
    assert len(book.groups) == 1 and sum(book.groups[0].simulated) == 2
    prices = _quotes(engine, notes, ctx)
    for actual, note in zip(prices, notes):
        expected = _quotes(engine, [note, note], ctx)[0]
        assert abs(actual - expected) < 2e-14, (actual, expected)
    assert prices[0] == prices[3]
    assert abs(prices[1] - prices[2]) > 1e-4


def test_mixed_book_with_an_outlier():
    """autocallable_monte_carlo.rs:189-208: an outlier knock-in note in a coupon family
    is simulated; every quote matches its two-lane quote."""
    ctx = _ctx()
    engine = OracleBookEngine(2048, 42)
    snows = [snowball(c) for c in (0.02, 0.08, -0.01, 0.02, 0.04)]
    outlier = snowball(0.02, knock_in=85.0)
    notes = [snows[0], snows[1], outlier, snows[2], snows[4]]
    mixed = _quotes(engine, notes, ctx)
    for note, value in zip(notes, mixed):
        partner = snows[0] if note is outlier else outlier
        expected = _quotes(engine, [note, partner], ctx)[0]
        assert abs(value - expected) < 2e-14, (value, expected)


def test_singletons_and_unshared_books_take_scalar_quotes():
    ctx = _ctx()
    engine = OracleBookEngine(4096, 3)
    note = snowball()
    scalar = engine._run(ctx, [plans.autocallable(note, ctx)])[0].price
    assert _quotes(engine, [note], ctx) == [scalar]
    notes = [snowball(c) for c in (0.02, 0.05, 0.07)]
    assert portfolio.price_many(engine, notes, ctx, False) == [
        engine._run(ctx, [plans.autocallable(n, ctx)])[0].price for n in notes]
    # Notes whose knock-in no longer matters keep their scalar quote on the shared grid.
    flat = SnowballOption(0.0, 100.0, 95.0, 100.0, 100.0, _EXPIRY,
                          [Observation(t, 110.0, None, 0.08) for t in _DATES], knock_in_times=_DAILY)
    assert portfolio.shared_lane(flat, ctx, 0) is None


def test_shared_grid_quote_near_scalar_quote():
    """The shared grid drops the scalar bridge plan; both estimate the same value."""
    ctx = _ctx()
    engine = OracleBookEngine(1 << 16, 11)
    note = snowball()
    shared = _quotes(engine, [note, note], ctx)[0]
    e = engine._run(ctx, [plans.autocallable(note, ctx)])[0]
    assert abs(shared - e.price) < 4.0 * e.standard_error, (shared, e.price, e.standard_error)


def test_batch_size_limit():
    """autocallable_batches_reject_an_excessive_contract_count
    (autocallable_monte_carlo.rs:10-27), with and without the shared grid."""
    from kiyosi_gb300.pricing import MonteCarloAutocallableEngine
    note = snowball()
    with pytest.raises(InvalidInputError, match="1,048,576"):
        portfolio.plan_book([note] * ((1 << 20) + 1), _ctx(), True)
    engine = MonteCarloAutocallableEngine(path_count=1024, seed=1)
    for shared in (False, True):
        with pytest.raises(InvalidInputError, match="1,048,576"):
            engine.price_many([note] * ((1 << 20) + 1), _ctx(), shared_grid=shared)
    with pytest.raises(InvalidInputError):
        engine.price_many([note, note], _ctx(), path_counts=[1024, 2048], shared_grid=True)


@pytest.mark.gpu
@pytest.mark.parametrize("sampling", SAMPLINGS)
def test_gpu_lanes_match_group_loop(native, sampling):
    ctx = _ctx()
    notes = ([snowball(c) for c in (0.02, 0.08, -0.01)] + [snowball(knock_in=85.0),
             snowball(dates=[_DATES[0], _DATES[1]], knock_out=(110.0, 108.0)), phoenix()])
    lanes = _lanes(notes, ctx)
    packed = pack(portfolio.lane_plans(lanes, ctx.spot))
    s = settings(1 << 14, 5, **sampling)
    loop, _ = loader.price_shared_group(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for g, r in zip(got, loop):
        assert abs(g.price - r) <= 1e-11 * max(1.0, abs(r)), (g.price, r)
    if not sampling.get("antithetic"):
        got32 = gpu_price(native, ctx, packed, settings(1 << 14, 5, precision="fp32",
                                                        schedule="persistent", **sampling))
        ref = loader.price_book(ctx, packed, s)
        for g, r in zip(got32, ref):
            assert abs(g.price - r.price) <= 0.5 * max(r.sample_error, 1e-4), (g.price, r.price)


@pytest.mark.gpu
@pytest.mark.parametrize("sobol", [False, True])
def test_gpu_path_major_schedule_matches_lanes(native, sobol):
    """KGPU_SCHEDULE_SHARED_GRID (one path per sample settles every lane) against the
    per-lane plain schedule and the oracle's loop: FP64 to rounding, with and without
    antithetic pairs; FP32 within half a sample error."""
    from kiyosi_gb300 import abi
    from kiyosi_gb300.errors import KiyosiError
    ctx = _ctx()
    notes = ([snowball(c) for c in (0.02, 0.08, -0.01)] + [snowball(knock_in=85.0),
             snowball(knock_out=(103.0,) * 3), phoenix(), phoenix(0.03),
             snowball(dates=[_DATES[0], _DATES[1]], knock_out=(110.0, 108.0))] * 5)
    lanes = [portfolio.shared_lane(n, ctx, i) for i, n in enumerate(notes)]
    packed = pack(portfolio.lane_plans(lanes, ctx.spot))
    paths = 1 << 14 if sobol else (1 << 14) + 77  # a ragged last CTA for pseudo-random
    plain = gpu_price(native, ctx, packed, settings(paths, 13, sobol=sobol))
    fast = gpu_price(native, ctx, packed, settings(paths, 13, sobol=sobol, schedule="shared_grid"))
    loop, _ = loader.price_shared_group(ctx, packed, settings(paths, 13, sobol=sobol))
    for f, p, r in zip(fast, plain, loop):
        assert abs(f.price - p.price) <= 1e-12 * max(1.0, abs(p.price)), (f.price, p.price)
        assert abs(f.price - r) <= 1e-11 * max(1.0, abs(r)), (f.price, r)
        assert abs(f.sample_error - p.sample_error) <= 1e-6 * p.sample_error
    fast32 = gpu_price(native, ctx, packed, settings(paths, 13, sobol=sobol, precision="fp32",
                                                      schedule="shared_grid"))
    for f, p in zip(fast32, plain):
        assert abs(f.price - p.price) <= 0.5 * max(p.sample_error, 1e-4), (f.price, p.price)
    # antithetic pairs: both partners walked by one thread
    pairs_fast = gpu_price(native, ctx, packed, settings(paths, 13, sobol=sobol, antithetic=True,
                                                          schedule="shared_grid"))
    pairs_plain = gpu_price(native, ctx, packed, settings(paths, 13, sobol=sobol, antithetic=True))
    for f, p in zip(pairs_fast, pairs_plain):
        assert abs(f.price - p.price) <= 1e-12 * max(1.0, abs(p.price)), (f.price, p.price)
        assert f.uncertainty_status == p.uncertainty_status
        assert abs(f.standard_error - p.standard_error) <= 1e-6 * max(p.standard_error, 1e-300)
        assert abs(f.sample_error - p.sample_error) <= 1e-6 * p.sample_error
    # lanes of two different grids are refused
    other = portfolio.shared_lane(snowball(dates=[_DATES[0], _year(datetime.date(2025, 2, 10))],
                                           knock_out=(110.0, 108.0)), ctx, 0)
    bad = pack(portfolio.lane_plans([lanes[0]], ctx.spot) + portfolio.lane_plans([other], ctx.spot))
    with pytest.raises(KiyosiError):
        gpu_price(native, ctx, bad, settings(1024, 1, schedule="shared_grid"))


@pytest.mark.gpu
def test_gpu_engine_shared_grid_book(native):
    from kiyosi_gb300.pricing import MonteCarloAutocallableEngine
    ctx = _ctx()
    notes = [snowball(c) for c in (0.02, 0.08, -0.01, 0.02, 0.04)] + [
        snowball(knock_out=(k,) * 3) for k in (103.0, 106.0, 101.0)] + [phoenix(), phoenix(0.05)]
    for antithetic in (False, True):  # path-major schedule, single paths and pairs
        engine = MonteCarloAutocallableEngine(path_count=1 << 14, seed=21, antithetic=antithetic)
        got = engine.price_many_on_shared_grid(notes, ctx)
        expected = portfolio.price_many(OracleBookEngine(1 << 14, 21, antithetic=antithetic),
                                        notes, ctx, True)
        for g, r in zip(got, expected):
            assert abs(g - r) <= 1e-11 * max(1.0, abs(r)), (antithetic, g, r)
