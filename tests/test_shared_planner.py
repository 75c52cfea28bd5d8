"""The native planner of books on shared daily grids (kgpu_shared_plan_*, planner.cpp)
against this package's Python restatement (portfolio.plan_book / lane_plans), on the CPU.

* Every lane's plan is the same bit for bit: its contract (offsets aside), steps, flags,
  bridge weights, events and intervals, and whether FP32 can carry it.  The native book
  shares step segments between lanes of one maturity and event set; each lane's slice
  is compared.
* The same notes go to the scalar engine, in the same groups, with the same coupon
  families, and the interpolation gives the same prices and the same retries.
* price_many through both planners, priced by the oracle, returns identical quotes,
  including the retry of a member whose interpolation cancels.
Books: the benchmark's dealer book; seasoned notes (knocked-in, knocked-out, missing
history, observations and monitoring at valuation); events off the monitoring dates;
expiry-only knock-in; fixed knock-in coupons; rebates; singletons and pairs; several
grids; a vanishing volatility; a non-BSM model."""
import ctypes as C
import math

import numpy as np
import pytest

from kiyosi_gb300 import abi, plans, portfolio, workloads
from kiyosi_gb300.errors import InvalidInputError, MissingHistoryError
from kiyosi_gb300.instruments import AutocallableNote, Observation, PhoenixOption, SnowballOption
from kiyosi_gb300.market import BlackScholesMertonParameters, HestonParameters, PricingContext
from oracle import loader

from helpers import pack, settings

DT = 1.0 / 252.0
DAILY = [DT * (i + 1) for i in range(126)]
MONTHS = [DAILY[21 * (m + 1) - 1] for m in range(6)]


def ctx(vol=0.25, spot=100.0):
    return PricingContext(BlackScholesMertonParameters(0.03, 0.01, vol), spot)


def snowball(coupon=0.06, ki=80.0, ko=103.0, months=6, ko_coupon=0.08, lower=0.0, **kw):
    dates = MONTHS[:months]
    return SnowballOption(coupon, 100.0, ki, 100.0, lower, dates[-1],
                          [Observation(t, ko, None, ko_coupon) for t in dates],
                          knock_in_times=DAILY[:21 * months], **kw)


def phoenix(coupon=0.01, ki=75.0, ko=102.0, months=6, **kw):
    dates = MONTHS[:months]
    return PhoenixOption(coupon, 100.0, ki, 100.0, 0.0, dates[-1],
                         [Observation(t, ko, ki, 0.0) for t in dates],
                         knock_in_times=DAILY[:21 * months], **kw)


def mixed_book():
    notes = []
    notes += [snowball(c) for c in (0.02, 0.05, 0.11, 0.07)]            # a coupon family
    notes += [phoenix(c) for c in (0.004, 0.01, 0.02)]                   # a Phoenix family
    notes += [snowball(ki=70.0), snowball(ko=105.0, months=3)]           # other terms, shorter grid
    notes += [snowball(0.05, months=4, ki=85.0), snowball(0.05, months=4, ki=85.0)]  # equal notes
    notes.append(snowball(rebate_rate=0.01, annual_rebate_rate=0.02))    # rebates
    notes.append(snowball(fixed_knock_in_coupon=0.01))                   # fixed knock-in coupon
    # an event off the monitoring dates: the note keeps its own schedule
    notes.append(SnowballOption(0.06, 100.0, 80.0, 100.0, 0.0, MONTHS[5],
                                [Observation(MONTHS[2] + 0.5 * DT, 103.0, None, 0.08),
                                 Observation(MONTHS[5], 103.0, None, 0.08)],
                                knock_in_times=DAILY[:126]))
    notes.append(SnowballOption(0.06, 100.0, 80.0, 100.0, 0.0, MONTHS[5],   # expiry-only knock-in
                                [Observation(t, 103.0, None, 0.08) for t in MONTHS]))
    notes.append(snowball(lower=100.0, coupon=0.0))               # knock-in cannot matter
    # seasoned: monitoring and an observation before valuation, history given
    past = [-5 * DT + k * DT for k in range(5)]
    notes.append(SnowballOption(0.06, 100.0, 80.0, 100.0, 0.0, MONTHS[5],
                                [Observation(-3 * DT, 103.0, None, 0.08)]
                                + [Observation(t, 103.0, None, 0.08) for t in MONTHS],
                                knock_in_times=past + DAILY[:126], effective_time=-5 * DT,
                                barrier_state="no_event"))
    notes.append(SnowballOption(0.06, 100.0, 80.0, 100.0, 0.0, MONTHS[5],
                                [Observation(t, 103.0, None, 0.08) for t in MONTHS],
                                knock_in_times=past + DAILY[:126], effective_time=-5 * DT,
                                barrier_state="knocked_in"))
    notes.append(SnowballOption(0.06, 100.0, 80.0, 100.0, 0.0, MONTHS[5],
                                [Observation(-DT, 103.0, None, 0.08)]
                                + [Observation(t, 103.0, None, 0.08) for t in MONTHS],
                                knock_in_times=DAILY[:126], effective_time=-DT,
                                barrier_state="knocked_out"))
    # an observation and monitoring at valuation, with a coupon barrier
    notes.append(PhoenixOption(0.01, 100.0, 75.0, 100.0, 0.0, MONTHS[5],
                               [Observation(0.0, 110.0, 90.0, 0.0)]
                               + [Observation(t, 102.0, 75.0, 0.0) for t in MONTHS],
                               knock_in_times=[0.0] + DAILY[:126], barrier_state="no_event"))
    notes.append(snowball(ko=103.0, months=2))                           # a shorter aligned grid
    # other monitoring schedules: weekly (a group of three), every other day (a pair),
    # every third day (a singleton, quoted alone)
    for every, coupons in ((5, (0.03, 0.04, 0.06)), (2, (0.03, 0.05)), (3, (0.07,))):
        days = [t for k, t in enumerate(DAILY) if (k + 1) % every == 0 or t in MONTHS]
        for c in coupons:
            notes.append(SnowballOption(c, 100.0, 80.0, 100.0, 0.0, MONTHS[5],
                                        [Observation(t, 103.0, None, 0.08) for t in MONTHS],
                                        knock_in_times=days))
    return notes


def _array(ptr, ctype, dtype, n):
    if n == 0:
        return np.zeros(0, dtype)
    return np.frombuffer((ctype * n).from_address(C.cast(ptr, C.c_void_p).value), dtype)


def compare_planners(notes, context):
    """Asserts that the native plan equals the Python restatement's, lane by lane."""
    book = portfolio.plan_book(notes, context, True)
    plan = portfolio.SharedPlan(portfolio.note_tables(notes), context.kgpu_model())
    try:
        assert sorted(book.scalar) == np.flatnonzero(plan.note_group < 0).tolist()
        assert len(book.groups) == plan.group_count
        for g, group in enumerate(book.groups):
            lanes = group.simulated_lanes()
            assert [lane.index for lane in group.lanes] == np.flatnonzero(plan.note_group == g).tolist()
            assert [lane.index for lane in lanes] == plan.group_lanes(g).tolist()
            expected = portfolio.lane_plans(lanes, context.spot)
            b = plan.group_book(g)
            contracts = _array(b.contracts, abi.Contract, plans.CONTRACT_DTYPE, b.contract_count)
            steps = _array(b.steps, abi.Step, plans.STEP_DTYPE, b.step_total)
            flags = _array(b.step_flags, C.c_uint8, np.uint8, b.step_total)
            daily = _array(b.bridge_daily, abi.BridgeDaily, plans.DAILY_DTYPE, b.step_total)
            events = _array(b.events, abi.Event, plans.EVENT_DTYPE, b.event_total)
            intervals = _array(b.intervals, abi.BridgeInterval, plans.INTERVAL_DTYPE, b.interval_total)
            assert len(contracts) == len(expected)
            for k, p in enumerate(expected):
                got, want = contracts[k].copy(), p.contract[0].copy()
                so, eo, bo = int(got["step_offset"]), int(got["event_offset"]), int(got["bridge_offset"])
                for f in ("step_offset", "event_offset", "bridge_offset"):
                    got[f] = want[f] = 0
                assert got.tobytes() == want.tobytes(), [
                    f for f in plans.CONTRACT_DTYPE.names if got[f] != want[f]]
                m, e, q = int(got["step_count"]), int(got["event_count"]), int(got["bridge_count"])
                assert steps[so:so + m].tobytes() == p.steps.tobytes()
                assert flags[so:so + m].tobytes() == p.flags.tobytes()
                assert daily[so:so + m].tobytes() == p.daily.tobytes()
                assert events[eo:eo + e].tobytes() == p.events.tobytes()
                assert intervals[bo:bo + q].tobytes() == p.intervals.tobytes()
                assert bool(plan.group_fp32(g)[k]) == plans.fp32_representable(p, context)
        # the families' interpolation on arbitrary lane prices
        rng = np.random.default_rng(7)
        prices = np.full(len(notes), np.nan)
        mine = {}
        for group in book.groups:
            for lane in group.simulated_lanes():
                prices[lane.index] = mine[lane.index] = rng.normal()
        retry = plan.interpolate(prices)
        expected_retry = []
        for group in book.groups:
            expected_retry += [group.lanes[i].index for i in portfolio.interpolate(group, mine)]
        assert np.flatnonzero(retry).tolist() == sorted(expected_retry)
        for i, v in mine.items():
            assert prices[i] == v
        return book, plan
    finally:
        plan.close()


def test_benchmark_book_plans_equal():
    book, plan = compare_planners(workloads.shared_grid_book(coupons=6), workloads.c2_context())
    assert len(book.groups) == 1 and book.groups[0].strips


def test_mixed_book_plans_equal():
    book, _ = compare_planners(mixed_book(), ctx())
    assert len(book.scalar) >= 5 and [len(g.lanes) for g in book.groups][1:] == [3, 2]
    assert sum(len(g.strips) for g in book.groups) == 3


def test_shared_step_segments():
    """Lanes of one maturity and one set of event steps share their step segment."""
    notes = workloads.shared_grid_book(coupons=4)
    plan = portfolio.SharedPlan(portfolio.note_tables(notes), workloads.c2_context().kgpu_model())
    b = plan.group_book(0)
    offsets = {int(c.step_offset) for c in (b.contracts[k] for k in range(b.contract_count))}
    assert b.contract_count > 100 and len(offsets) == 4  # 6, 12, 18 and 24 monthly dates
    assert b.step_total == 126 + 252 + 378 + 504
    plan.close()


@pytest.mark.parametrize("vol", [1e-18, 1e-200])
def test_vanishing_volatility_plans_equal(vol):
    """Under sigma = 1e-200 the bridge weights are 0 / 0: both planners step forward."""
    book, _ = compare_planners([snowball(c) for c in (0.02, 0.05, 0.11)] + [phoenix()], ctx(vol))
    if vol == 1e-200:
        for group in book.groups:
            _, intervals, _ = portfolio.interval_plan(group.simulated_lanes(), 100.0)
            assert len(intervals) == len(group.lanes[0].steps)


def test_spot_moves_plans_equal():
    for spot in (75.0, 79.9, 103.0, 140.0):
        compare_planners(mixed_book(), ctx(spot=spot))


def test_other_models_quote_every_note_alone():
    heston = workloads.heston_context()
    plan = portfolio.SharedPlan(portfolio.note_tables(mixed_book()), heston.kgpu_model())
    assert (plan.note_group == -1).all() and plan.group_count == 0
    plan.close()


def test_invalid_tables_are_refused():
    notes = [snowball(c) for c in (0.02, 0.05, 0.11)]
    tables = portfolio.note_tables(notes)
    bad = portfolio.NoteTables(tables.notes.copy(), tables.observations, tables.monitoring)
    bad.notes["observation_offset"][1] = len(tables.observations)
    with pytest.raises(InvalidInputError):
        portfolio.SharedPlan(bad, ctx().kgpu_model())
    bad = portfolio.NoteTables(tables.notes.copy(), tables.observations, tables.monitoring)
    bad.notes["monitoring_count"][0] = len(tables.monitoring) + 1
    with pytest.raises(InvalidInputError):
        portfolio.SharedPlan(bad, ctx().kgpu_model())
    unsorted = tables.monitoring.copy()
    unsorted[[3, 4]] = unsorted[[4, 3]]
    with pytest.raises(InvalidInputError):
        portfolio.SharedPlan(portfolio.NoteTables(tables.notes, tables.observations, unsorted),
                             ctx().kgpu_model())


class OracleEngine:
    """The engine surface price_many uses, priced by the oracle (FP64 plain schedule);
    `shift` makes every price its note's terminal coupon term minus a constant, so that a
    family member's interpolation can be made to cancel."""

    def __init__(self, paths=256, seed=11, shift=None):
        self.s = settings(paths, seed)
        self.shift = shift

    def _estimates(self, context, packed):
        if self.shift is not None:
            return [type("E", (), {"price": float(c["terminal_plain"]) - self.shift})()
                    for c in packed.contracts]
        return loader.price_book(context, packed, self.s)

    def _run(self, context, batch):
        out = [type("E", (), {"price": p.value})() if isinstance(p, plans.Known) else None for p in batch]
        sampled = [p for p in batch if not isinstance(p, plans.Known)]
        estimates = iter(self._estimates(context, pack(sampled)) if sampled else [])
        return [e if e is not None else next(estimates) for e in out]

    def _run_group(self, context, lane_plans):
        return self._estimates(context, pack(lane_plans))

    def _run_shared_book(self, context, book, lane_fp32):
        return np.array([e.price for e in self._shared_estimates(context, book)])

    def _shared_estimates(self, context, book):
        n = book.contract_count
        b = plans.PackedBook(_array(book.contracts, abi.Contract, plans.CONTRACT_DTYPE, n).copy(),
                             _array(book.steps, abi.Step, plans.STEP_DTYPE, book.step_total).copy(),
                             _array(book.step_flags, C.c_uint8, np.uint8, book.step_total).copy(),
                             _array(book.events, abi.Event, plans.EVENT_DTYPE, book.event_total).copy(),
                             _array(book.intervals, abi.BridgeInterval, plans.INTERVAL_DTYPE,
                                    book.interval_total).copy(),
                             _array(book.bridge_daily, abi.BridgeDaily, plans.DAILY_DTYPE, book.step_total).copy())
        return self._estimates(context, b)


def test_price_many_quotes_equal_through_both_planners():
    notes = mixed_book()
    engine = OracleEngine()
    native = portfolio.price_many(engine, notes, ctx(), True, planner="native")
    python = portfolio.price_many(engine, notes, ctx(), True, planner="python")
    assert native == python
    assert all(math.isfinite(p) for p in native)


def test_cancelled_interpolation_is_simulated_through_both_planners():
    coupons = (0.02, 0.05, 0.08)
    notes = [snowball(c) for c in coupons]
    middle = portfolio.SharedPlan(portfolio.note_tables(notes), ctx().kgpu_model())
    b = middle.group_book(0)
    lows = {round(float(b.contracts[k].terminal_plain), 12) for k in range(b.contract_count)}
    middle.close()
    assert len(lows) == 2  # the family's bounds are simulated, the middle note is not
    shift = notes[1].terminal(0.0, False)  # the middle note's term: its interpolation cancels
    engine = OracleEngine(shift=shift)
    native = portfolio.price_many(engine, notes, ctx(), True, planner="native")
    python = portfolio.price_many(engine, notes, ctx(), True, planner="python")
    assert native == python and native[1] == 0.0


def test_missing_history_raises_through_both_planners():
    past = [-2 * DT, -DT] + DAILY[:126]
    bad = SnowballOption(0.06, 100.0, 80.0, 100.0, 0.0, MONTHS[5],
                         [Observation(t, 103.0, None, 0.08) for t in MONTHS],
                         knock_in_times=past, effective_time=-2 * DT)
    notes = [snowball(c) for c in (0.02, 0.05, 0.11)] + [bad]
    for planner in ("native", "python"):
        with pytest.raises(MissingHistoryError):
            portfolio.price_many(OracleEngine(), notes, ctx(), True, planner=planner)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_engine_prices_equal_through_both_planners(precision):
    """price_many_on_shared_grid on the GB300 with the native planner's book (shared step
    segments) and with the Python planner's (one copy per lane): identical quotes."""
    from kiyosi_gb300.pricing import MonteCarloAutocallableEngine
    engine = MonteCarloAutocallableEngine(path_count=1 << 13, seed=3, precision=precision)
    for notes, context in ((mixed_book(), ctx()), (workloads.shared_grid_book(coupons=3), workloads.c2_context())):
        native = portfolio.price_many(engine, notes, context, True, planner="native")
        python = portfolio.price_many(engine, notes, context, True, planner="python")
        assert native == python
        assert native == engine.price_many_on_shared_grid(notes, context)


def test_empty_book():
    plan = portfolio.SharedPlan(portfolio.note_tables([]), ctx().kgpu_model())
    assert plan.group_count == 0 and len(plan.note_group) == 0
    assert not plan.interpolate(np.zeros(0)).any()
    plan.close()
    assert portfolio.price_many(OracleEngine(), [], ctx(), True) == []
