"""Books of autocallable notes on shared paths (engines/monte_carlo/autocallable/portfolio.rs).

`price_many(engine, notes, ctx, shared_grid)` restates portfolio::price_many (187-318).

Without the shared grid, each note gets its scalar quote. The reference does group notes
of one grid onto shared paths, but every lane replays the scalar path, so the quote is
unchanged. Every note is therefore its own contract of one book.

With the shared grid:

* Daily grid (DailyGrids::prepare, 74-185). Eligible notes are those with daily knock-in
  monitoring that still matters, whose cash events fall on monitoring dates or expiry.
  Each is simulated on its daily grid, not on the scalar Brownian-bridge plan.
* Groups (same_daily_grid, 872-901). Notes of one daily grid form a group. Grids that end
  on their maturity may differ in length, and share their common dates.
* One path per group (SharedEvents::new, 903-1047; shared_payoffs, 1275-1439). A "date"
  here is one on which any note of the group pays or matures. When at least eight daily
  steps separate two such dates, those steps are drawn as a backward Brownian bridge;
  every other step is drawn forward.
* Coupon families (price_coupon_families, 570-667). Three or more notes that differ only
  in their coupon are priced from the lowest- and highest-coupon members. The rest are
  interpolated linearly in the coupon: on shared paths a note's value is affine in its
  coupon. A member is simulated after all when its interpolation cancels.
* Singletons (scalar, 504-515). A group of one note takes the scalar estimator, with its
  own bridge plan.

GB300 layout: the whole book is one launch. Each simulated note of a group is a lane
contract that carries:
* the group's intervals and bridge weights;
* the group's longest grid as its sampling dimensions (kgpu_contract.dimensions).

So lane k draws the same normals and walks the same path values that the reference's
multi-lane loop gives lane k. The loop's live-floor early exit skips only daily values
that can no longer change a live note.

The reference's threshold strips (price_shared, 702-760) cover families that differ only
in a knock-out or knock-in level. They save work on the CPU. Here every strip member is a
lane of the same launch. `threshold_strips` still describes them, for the oracle's
restatement of the strip sums.
"""
import ctypes as C
import math
import operator
import struct
from dataclasses import dataclass, field, fields, replace
from fractions import Fraction
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import abi, plans
from .errors import ComputationFailureError, InvalidInputError
from .instruments import AutocallableNote
from .market import BlackScholesMertonParameters, PricingContext, log_ratio, safe_log_returns

MAX_CONTRACTS = 1 << 20  # binding_support::validate_contract_batch_size (lib.rs:188-195)
_SMALLEST_NORMAL = 2.2250738585072014e-308


def _fma(a: float, b: float, c: float) -> float:
    """f64::mul_add: a * b + c with one rounding (exact rational arithmetic, then the
    correctly rounded conversion of int / int)."""
    if not (math.isfinite(a) and math.isfinite(b) and math.isfinite(c)):
        return a * b + c
    return float(Fraction(a) * Fraction(b) + Fraction(c))


@dataclass
class Lane:
    """One note on a shared daily grid (the PathPlan of a shared request)."""
    index: int                      # position in the caller's book
    note: AutocallableNote
    contract: np.ndarray            # scalar contract fields (thresholds, terminal terms)
    steps: np.ndarray               # STEP_DTYPE, the note's grid up to its maturity
    observe: np.ndarray             # uint8 STEP_KNOCK_IN per step
    events: List[Tuple[int, tuple]]  # (step, EVENT_DTYPE record)
    sparse: bool                    # grid from DailyGrids::prepare
    maturity_on_grid: bool

    @property
    def maturity(self) -> int:
        return len(self.steps) - 1


def _daily(note: AutocallableNote, spot: float) -> bool:
    """prepare_sample_on_grid's `daily` (autocallable.rs:335), with the knock-in state
    at valuation (pricing::initial)."""
    return (note.daily_knock_in and note.knock_in_affects_payoff()
            and not plans.autocallable_initial(note, spot).knocked_in)


def shared_lane(note: AutocallableNote, ctx: PricingContext, index: int) -> Optional[Lane]:
    """The note's plan when it joins a shared daily grid, else None (scalar quote).

    DailyGrids::prepare (portfolio.rs:74-185): the grid is every monitoring date, plus
    expiry when expiry is not one of them. A cash event off those dates keeps the
    ordinary schedule. That schedule still shares a grid when it monitors knock-in
    (PathPlan::shared_daily_grid, portfolio.rs:868-870)."""
    if not (_daily(note, ctx.spot) and isinstance(ctx.model, BlackScholesMertonParameters)):
        return None
    template = plans.autocallable(note, ctx, allow_bridge=False)
    if isinstance(template, plans.Known):
        return None
    contract = template.contract.copy()
    times, monitored = _future_monitoring(note.knock_in_times)
    events = [o for o in note.observations if o.time > 0.0]
    on_grid = bool(times) and all(o.time == note.expiry or o.time in monitored for o in events)
    records = template.events.tolist()
    cash = [(r[_EVENT_STEP], r) for r in records]
    if not on_grid:
        observe = template.flags & abi.STEP_KNOCK_IN
        if not observe.any():
            return None
        return Lane(index, note, contract, template.steps, observe.astype(np.uint8), cash, False, False)
    maturity_on_grid = times[-1] == note.expiry
    # With every event on a monitoring date or expiry, the scalar schedule (event dates,
    # monitoring dates and expiry) is this grid, step for step.
    observe = (template.flags & abi.STEP_KNOCK_IN).astype(np.uint8)
    return Lane(index, note, contract, template.steps, observe, cash, True, maturity_on_grid)


_EVENT_STEP = plans.EVENT_DTYPE.names.index("step")
_MONITORING: dict = {}


def _future_monitoring(knock_in_times):
    """The monitoring dates after valuation and their set, per schedule object (notes of
    a book share the object; see instruments._shared_times)."""
    hit = _MONITORING.get(id(knock_in_times))
    if hit is not None and hit[0] is knock_in_times:
        return hit[1], hit[2]
    times = [t for t in knock_in_times if t > 0.0]
    monitored = set(times)
    if len(_MONITORING) >= 4096:
        _MONITORING.clear()
    _MONITORING[id(knock_in_times)] = (knock_in_times, times, monitored)
    return times, monitored


def _grid_key(lane: Lane):
    """The grouping key (portfolio.rs:124-131, 438-458): aligned daily grids share one
    key; other grids hash their transitions and monitoring flags."""
    if lane.sparse and lane.maturity_on_grid:
        return ("daily",)
    s = lane.steps
    return ("grid", s["drift"].tobytes(), s["diffusion"].tobytes(), s["discount"].tobytes(),
            lane.observe.tobytes())


def same_daily_grid(a: Lane, b: Lane) -> bool:
    """PathPlan::same_daily_grid (portfolio.rs:872-901): equal transitions and monitoring
    flags on the common dates; grids of different lengths must both end on maturity."""
    if len(a.steps) != len(b.steps) and not (a.sparse and a.maturity_on_grid
                                             and b.sparse and b.maturity_on_grid):
        return False
    n = min(len(a.steps), len(b.steps))
    for f in ("drift", "diffusion", "discount"):
        if a.steps[f][:n].tobytes() != b.steps[f][:n].tobytes():
            return False
    return a.observe[:n].tobytes() == b.observe[:n].tobytes()


def _is_normal(x: float) -> bool:
    return math.isfinite(x) and abs(x) >= _SMALLEST_NORMAL


def interval_plan(lanes: Sequence[Lane], spot: float):
    """SharedEvents::new (portfolio.rs:903-1047) for the lanes of one group.

    Returns (base grid, [(end step, drift, diffusion)], DAILY_DTYPE weights).  A date on
    which any lane pays or matures ends an interval.  When the path cannot leave the
    finite range, runs of at least eight daily steps before such a date become one
    bridged interval: its end is drawn first with the summed drift and variance, then
    each day with the backward weights (variance share, conditional width)."""
    base = max(lanes, key=lambda lane: len(lane.steps))
    for lane in lanes:  # max_by_key keeps the last of equal maxima
        if len(lane.steps) == len(base.steps):
            base = lane
    steps = base.steps
    n = len(steps)
    actions = set()
    for lane in lanes:
        actions.update(step for step, _ in lane.events)
        actions.add(lane.maturity)
    drift = [float(v) for v in steps["drift"]]
    width = [float(v) for v in steps["diffusion"]]
    excursion = 0.0
    for i in range(n):
        excursion += abs(drift[i]) + 20.0 * width[i]
    low, high = safe_log_returns(spot)
    bridge = low <= excursion <= high and low <= -excursion <= high
    daily = np.zeros(n, plans.DAILY_DTYPE)
    intervals = []
    first = 0
    for step in range(n):
        if step not in actions and step + 1 < n:
            continue
        if bridge and step - first >= 8:
            total, variance = drift[step], width[step] * width[step]
            weights = []
            for i in range(step - 1, first - 1, -1):
                nxt = _fma(width[i], width[i], variance)
                if nxt == 0.0:
                    # 0 / 0 under a vanishing volatility: NaN weights refuse the bridge,
                    # as the reference's floating-point division does
                    weights.append((i, math.nan, math.nan))
                else:
                    weights.append((i, (width[i] * width[i]) / nxt, width[i] * math.sqrt(variance / nxt)))
                total += drift[i]
                variance = nxt
            diffusion = math.sqrt(variance)
            if (_is_normal(diffusion) and math.isfinite(total)
                    and all(w > 0.0 and d > 0.0 for _, w, d in weights)):
                for i, w, d in weights:
                    if not base.observe[i] & abi.STEP_KNOCK_IN:
                        # Bridged days always monitor knock-in: a day off the monitoring
                        # dates would be a cash or maturity date, which ends an interval.
                        raise ComputationFailureError("a bridged day does not monitor knock-in")
                    daily[i] = (w, d)
                intervals.append((step, total, diffusion))
                first = step + 1
                continue
        for i in range(first, step + 1):
            intervals.append((i, drift[i], width[i]))
        first = step + 1
    return base, intervals, daily


def lane_plans(lanes: Sequence[Lane], spot: float) -> List[plans.ContractPlan]:
    """One bridged contract per lane: the lane's steps and cash events, the group's
    intervals up to the lane's maturity, and the group's longest grid as sampling
    dimensions."""
    base, intervals, daily = interval_plan(lanes, spot)
    out = []
    for lane in lanes:
        m = lane.maturity
        # the lane's grid and monitoring flags are the longest grid's first m + 1 steps
        if lane.observe.tobytes() != base.observe[:m + 1].tobytes() or any(
                lane.steps[f].tobytes() != base.steps[f][:m + 1].tobytes()
                for f in ("drift", "diffusion", "discount")):
            raise InvalidInputError("the lanes do not share one daily grid")
        own = [(end, 0, d, w) for end, d, w in intervals if end <= m]
        if not own or own[-1][0] != m:
            raise ComputationFailureError("a lane's maturity does not end an interval")
        c = lane.contract.copy()
        flags = lane.observe.copy()
        for step, _ in lane.events:
            flags[step] |= abi.STEP_EVENT
        c["step_count"] = m + 1
        c["event_count"] = len(lane.events)
        c["flags"] = (int(c["flags"][0]) & ~abi.C_BRIDGE) | abi.C_BRIDGE
        c["bridge_count"] = len(own)
        c["final_discount"] = lane.steps["discount"][m]
        c["dimensions"] = len(base.steps)
        out.append(plans.ContractPlan(c, lane.steps.copy(), flags,
                                      np.array([e for _, e in lane.events], plans.EVENT_DTYPE),
                                      np.array(own, plans.INTERVAL_DTYPE), daily[:m + 1].copy()))
    return out


# ---- coupon families (price_coupon_families, portfolio.rs:570-667) ----

def _is_phoenix(note: AutocallableNote) -> bool:
    """A Phoenix note pays its period coupon on coupon-barrier observations."""
    return any(o.coupon_barrier_level is not None for o in note.observations)


def portfolio_coupon(note: AutocallableNote) -> float:
    """AutocallableNote::portfolio_coupon (instruments/autocallable.rs:1182-1186)."""
    return note.period_coupon if _is_phoenix(note) else note.maturity_coupon_rate


def _without_coupon(note: AutocallableNote):
    """Every term but the portfolio coupon, with whether knock-in changes the payoff
    (portfolio_family_key and shares_portfolio_terms, autocallable.rs:1188-1300)."""
    coupon = "period_coupon" if _is_phoenix(note) else "maturity_coupon_rate"
    return (tuple(getattr(note, f.name) for f in fields(note) if f.name != coupon),
            note.knock_in_affects_payoff())


@dataclass
class CouponStrip:
    members: List[int]  # positions in the group
    low: int
    high: int
    width: float


@dataclass
class GroupPlan:
    lanes: List[Lane]
    simulated: List[bool] = field(default_factory=list)
    strips: List[CouponStrip] = field(default_factory=list)

    def simulated_lanes(self) -> List[Lane]:
        return [lane for lane, s in zip(self.lanes, self.simulated) if s]


def coupon_families(lanes: Sequence[Lane]) -> GroupPlan:
    """Families of three or more notes differing only in their coupon, and the notes
    that must be simulated (their lowest- and highest-coupon members, and the rest)."""
    by_key: Dict[object, int] = {}
    families: List[List[int]] = []
    for i, lane in enumerate(lanes):
        key = _without_coupon(lane.note)
        if key not in by_key:
            by_key[key] = len(families)
            families.append([])
        families[by_key[key]].append(i)
    plan = GroupPlan(list(lanes), [True] * len(lanes))
    coupons = [portfolio_coupon(lane.note) for lane in lanes]
    coupon = coupons.__getitem__
    for family in families:
        if len(family) < 3:
            continue
        low, high = family[0], family[1]
        if coupon(low) > coupon(high):
            low, high = high, low
        for i in family[2:]:
            if coupon(i) < coupon(low):
                low = i
            if coupon(i) > coupon(high):
                high = i
        width = coupon(high) - coupon(low)
        if math.isfinite(width):
            plan.strips.append(CouponStrip(family, low, high, width))
            for i in family:
                plan.simulated[i] = i in (low, high)
    return plan


def interpolate(plan: GroupPlan, prices: Dict[int, float]) -> List[int]:
    """Fills the interpolated members' prices (keyed by book index) from their family's
    bound notes; returns the group positions whose interpolation cancels, which the
    reference then simulates."""
    retry = []
    for strip in plan.strips:
        lower = prices[plan.lanes[strip.low].index]
        upper = prices[plan.lanes[strip.high].index]
        c_low = portfolio_coupon(plan.lanes[strip.low].note)
        for i in strip.members:
            if plan.simulated[i]:
                continue
            fraction = ((portfolio_coupon(plan.lanes[i].note) - c_low) / strip.width
                        if strip.width > 0.0 else 0.0)
            value = (lower * (1.0 - fraction), upper * fraction)
            price = value[0] + value[1]
            magnitude = abs(value[0]) + abs(value[1])
            if not math.isfinite(price) or abs(price) < 1e-12 * magnitude:
                retry.append(i)
            else:
                prices[plan.lanes[i].index] = price
    return retry


# ---- threshold strips (price_shared and threshold_families, portfolio.rs:702-824) ----

KNOCK_OUT, KNOCK_IN = 1, 2


def _constant_knock_out(note: AutocallableNote) -> Optional[float]:
    """The one knock-out level of a note whose events are pure redemptions."""
    events = [o for o in note.observations if o.time > 0.0]
    if not events or events[0].knock_out_level is None:
        return None
    level = events[0].knock_out_level
    for o in events:
        coupon = note.period_coupon if o.coupon_barrier_level is not None else 0.0
        if o.knock_out_level != level or coupon != 0.0:
            return None
    return level


def _without_level(note: AutocallableNote, variation: int):
    if variation == KNOCK_IN:
        return replace(note, knock_in_level=0.0)
    obs = tuple(replace(o, knock_out_level=None if o.knock_out_level is None else 0.0)
                for o in note.observations)
    return replace(note, observations=obs)


def threshold_strips(lanes: Sequence[Lane], spot: float):
    """The reference's strips over the simulated lanes of a group of at least three:
    knock-out families first, then knock-in families among the rest.  Returns
    (lane order, per-lane (kind, ascending log levels, book indices))."""
    n = len(lanes)
    selected = [False] * n
    strips = []
    if n < 3:
        return list(range(n)), [None] * n
    for variation in (KNOCK_OUT, KNOCK_IN):
        by_key: Dict[object, int] = {}
        families: List[List[Tuple[float, int]]] = []
        for i, lane in enumerate(lanes):
            if selected[i] or not lane.sparse:
                continue
            if variation == KNOCK_OUT:
                level = _constant_knock_out(lane.note)
            else:
                level = None if lane.note.knocked_in else lane.note.knock_in_level
            if level is None:
                continue
            level = log_ratio(level, spot)
            if not math.isfinite(level):
                continue
            key = (_without_level(lane.note, variation), len(lane.steps))
            if key not in by_key:
                by_key[key] = len(families)
                families.append([])
            families[by_key[key]].append((level, i))
        for levels in families:
            if len(levels) < 3:
                continue
            levels.sort()
            for _, i in levels:
                selected[i] = True
            strips.append((levels[0][1], variation, [lv for lv, _ in levels],
                           [lanes[i].index for _, i in levels]))
    order = [rep for rep, _, _, _ in strips] + [i for i in range(n) if not selected[i]]
    described = [(kind, lv, idx) for _, kind, lv, idx in strips] + [None] * (len(order) - len(strips))
    return order, described


# ---- the book ----

@dataclass
class BookPlan:
    """What price_many samples: scalar plans by book index, and shared groups."""
    scalar: Dict[int, object]
    groups: List[GroupPlan]


def plan_book(notes: Sequence[AutocallableNote], ctx: PricingContext, shared_grid: bool) -> BookPlan:
    """Sorts the book into scalar quotes and shared groups (portfolio.rs:187-318,
    544-568)."""
    if len(notes) > MAX_CONTRACTS:
        raise InvalidInputError("contract batch exceeds 1,048,576 instruments")
    scalar: Dict[int, object] = {}
    groups: List[List[Lane]] = []
    by_key: Dict[object, List[int]] = {}
    for i, note in enumerate(notes):
        lane = shared_lane(note, ctx, i) if shared_grid else None
        if lane is None:
            scalar[i] = plans.autocallable(note, ctx)
            continue
        candidates = by_key.setdefault(_grid_key(lane), [])
        for g in candidates:
            if same_daily_grid(groups[g][0], lane):
                groups[g].append(lane)
                break
        else:
            candidates.append(len(groups))
            groups.append([lane])
    out = []
    for group in groups:
        if len(group) == 1:
            scalar[group[0].index] = plans.autocallable(group[0].note, ctx)
        elif len(group) == 2:
            out.append(GroupPlan(group, [True, True]))
        else:
            out.append(coupon_families(group))
    return BookPlan(scalar, out)


def price_many(engine, notes: Sequence[AutocallableNote], ctx: PricingContext,
               shared_grid: bool, planner: str = "native") -> List[float]:
    """Quotes of `notes` in input order.  Scalar quotes share one launch; each group's
    lanes go to the engine's path-major schedule when it has one (one path per sample
    settles every lane, kgpu's KGPU_SCHEDULE_SHARED_GRID), else into the same launch as
    per-lane contracts (identical estimates, each lane re-walking the path).

    With a shared grid under BSM the book is planned by the library's native planner
    (kgpu_shared_plan_create, `SharedPlan`); `planner="python"` plans it with this
    module's restatement instead (same lanes, same prices)."""
    if planner not in ("native", "python"):
        raise InvalidInputError("planner must be 'native' or 'python'")
    if (shared_grid and planner == "native" and isinstance(ctx.model, BlackScholesMertonParameters)
            and getattr(engine, "_run_shared_book", None) is not None):
        return _price_many_planned(engine, notes, ctx)
    book = plan_book(notes, ctx, shared_grid)
    prices: Dict[int, float] = {}
    pending = list(range(len(book.groups)))
    run_group = getattr(engine, "_run_group", None)
    first = True
    while first or pending:
        indices, batch = [], []
        if first:
            for i, p in book.scalar.items():
                indices.append(i)
                batch.append(p)
        for g in pending:
            lanes = book.groups[g].simulated_lanes()
            group_plans = lane_plans(lanes, ctx.spot)
            estimates = run_group(ctx, group_plans) if run_group is not None else None
            if estimates is not None:
                for lane, e in zip(lanes, estimates):
                    prices[lane.index] = e.price
                continue
            for lane, p in zip(lanes, group_plans):
                indices.append(lane.index)
                batch.append(p)
        if batch:
            for i, e in zip(indices, engine._run(ctx, batch)):
                prices[i] = e.price
        retry = []
        for g in pending:
            again = interpolate(book.groups[g], prices)
            if again:
                for i in again:
                    book.groups[g].simulated[i] = True
                retry.append(g)
        pending = retry
        first = False
    return [prices[i] for i in range(len(notes))]


# ---- the native planner (kgpu_shared_plan_* in include/kgpu.h) ----

NOTE_DTYPE = np.dtype(abi.Note)
NOTE_OBSERVATION_DTYPE = np.dtype(abi.NoteObservation)
_STATE_CODES = {None: abi.STATE_UNKNOWN, "no_event": abi.STATE_NO_EVENT,
                "knocked_in": abi.STATE_KNOCKED_IN, "knocked_out": abi.STATE_KNOCKED_OUT}
_NOTE_TERMS = operator.attrgetter(
    "initial_spot", "expiry", "knock_in_level", "upper_strike", "lower_strike",
    "maturity_coupon_rate", "period_coupon", "fixed_knock_in_coupon", "principal", "rebate_rate",
    "annual_rebate_rate", "effective_time", "barrier_state", "observations", "knock_in_times")


@dataclass
class NoteTables:
    """A book of notes as kgpu_shared_plan_create's flat tables."""
    notes: np.ndarray         # NOTE_DTYPE
    observations: np.ndarray  # NOTE_OBSERVATION_DTYPE
    monitoring: np.ndarray    # float64: every distinct monitoring schedule once


# kgpu_note: 12 doubles, then 6 int32; kgpu_note_observation: 4 doubles, then 2 int32
# (little-endian, no padding; test_abi checks both sizes against the header).
_NOTE_ROW = struct.Struct("<12d6i")
_OBSERVATION_ROW = struct.Struct("<4d2i")


def _note_encoding(note: AutocallableNote):
    """The note's flat terms (the bytes of a kgpu_note without its table ranges) and the
    bytes of its observation rows (None levels flagged absent).  Notes are frozen, so the
    encoding is computed once per note object and kept on it, as Observation keeps its
    hash."""
    encoding = note.__dict__.get("_kgpu_encoding")
    if encoding is None:
        (spot0, expiry, ki, upper, lower, maturity_coupon, period_coupon, fixed, principal,
         rebate, annual_rebate, effective, state, obs, times) = _NOTE_TERMS(note)
        flags = 0
        if ki is None:
            ki = 0.0
        else:
            flags |= abi.NOTE_KNOCK_IN
        if fixed is None:
            fixed = 0.0
        else:
            flags |= abi.NOTE_FIXED_COUPON
        if times is not None:
            flags |= abi.NOTE_MONITORING
        row = _NOTE_ROW.pack(spot0, expiry, ki, upper, lower, maturity_coupon, period_coupon, fixed,
                             principal, rebate, annual_rebate, effective, flags, _STATE_CODES[state],
                             0, len(obs), 0, 0)
        pack = _OBSERVATION_ROW.pack
        rows = []
        for o in obs:
            ko, cb = o.knock_out_level, o.coupon_barrier_level
            rows.append(pack(o.time, 0.0 if ko is None else ko, 0.0 if cb is None else cb, o.coupon_rate,
                             (0 if ko is None else abi.OBSERVATION_KNOCK_OUT)
                             | (0 if cb is None else abi.OBSERVATION_COUPON_BARRIER), 0))
        encoding = (row, b"".join(rows))
        object.__setattr__(note, "_kgpu_encoding", encoding)
    return encoding


def note_tables(notes: Sequence[AutocallableNote]) -> NoteTables:
    """Flattens the notes' terms into kgpu_shared_plan_create's tables: the notes'
    encodings stacked, their observation ranges, and each distinct monitoring schedule
    once (notes sharing a schedule object share its range)."""
    if not notes:
        return NoteTables(np.zeros(0, NOTE_DTYPE), np.zeros(0, NOTE_OBSERVATION_DTYPE), np.zeros(0, np.float64))
    encodings = [_note_encoding(n) for n in notes]
    table = np.frombuffer(b"".join([e[0] for e in encodings]), NOTE_DTYPE).copy()
    observations = np.frombuffer(b"".join([e[1] for e in encodings]), NOTE_OBSERVATION_DTYPE).copy()
    counts = table["observation_count"]
    table["observation_offset"] = np.cumsum(counts) - counts
    schedules: Dict[int, Tuple[int, int]] = {}
    monitoring = []
    total = 0
    first = np.zeros(len(notes), np.int32)
    count = np.zeros(len(notes), np.int32)
    for i, times in enumerate(map(operator.attrgetter("knock_in_times"), notes)):
        if times is None:
            continue
        hit = schedules.get(id(times))
        if hit is None:
            hit = schedules[id(times)] = (total, len(times))
            monitoring.append(times)
            total += len(times)
        first[i], count[i] = hit
    table["monitoring_offset"] = first
    table["monitoring_count"] = count
    mon = (np.concatenate([np.asarray(t, np.float64) for t in monitoring]) if monitoring
           else np.zeros(0, np.float64))
    return NoteTables(table, observations, mon)


class SharedPlan:
    """The native plan of a book on shared daily grids (kgpu_shared_plan_create): which
    notes are lanes of which group, each group's packed lane contracts, and the coupon
    families' interpolation.  Holds the library's plan until closed."""

    def __init__(self, tables: NoteTables, model: abi.Model, simulate: Optional[np.ndarray] = None):
        from . import _native
        from .errors import raise_for_status
        self.lib = lib = _native.library()
        self.tables = tables
        P = C.POINTER
        mask = None
        if simulate is not None:
            self._simulate = np.ascontiguousarray(simulate, np.uint8)
            mask = self._simulate.ctypes.data_as(P(C.c_uint8))
        handle = C.c_void_p()
        status = lib.kgpu_shared_plan_create(
            C.byref(model), tables.notes.ctypes.data_as(P(abi.Note)), len(tables.notes),
            tables.observations.ctypes.data_as(P(abi.NoteObservation)), len(tables.observations),
            tables.monitoring.ctypes.data_as(P(C.c_double)), len(tables.monitoring), mask,
            C.byref(handle))
        if status != 0:
            raise_for_status(status, lib.kgpu_last_error_message(None).decode())
        self.handle = handle
        view = abi.SharedPlanView()
        lib.kgpu_shared_plan_get(handle, C.byref(view))
        self.view = view
        n, g, k = view.note_count, view.group_count, view.lane_count
        self.note_group = np.ctypeslib.as_array(view.note_group, (n,)).copy() if n else np.zeros(0, np.int32)
        self.group_first_lane = np.ctypeslib.as_array(view.group_first_lane, (g + 1,)).copy()
        self.lane_note = np.ctypeslib.as_array(view.lane_note, (k,)).copy() if k else np.zeros(0, np.int32)
        self.lane_fp32 = (np.ctypeslib.as_array(view.lane_fp32, (k,)).astype(bool) if k
                          else np.zeros(0, bool))
        self.group_count = g

    def group_lanes(self, g: int) -> np.ndarray:
        """Book indices of group g's simulated lanes, in contract order."""
        return self.lane_note[self.group_first_lane[g]:self.group_first_lane[g + 1]]

    def group_fp32(self, g: int) -> np.ndarray:
        return self.lane_fp32[self.group_first_lane[g]:self.group_first_lane[g + 1]]

    def group_book(self, g: int) -> abi.Book:
        """Group g's kgpu_book (the library's arrays); raises the group's planning failure."""
        from .errors import raise_for_status
        status = self.view.group_status[g]
        if status != 0:
            raise_for_status(status, self.view.group_message[g].decode())
        return self.view.group_books[g]

    def group_packed(self, g: int) -> plans.PackedBook:
        """A numpy copy of group g's book (for the oracle and for device-resident runs)."""
        b = self.group_book(g)

        def take(ptr, ctype, dtype, n):
            if n == 0 or not ptr:
                return np.zeros(0, dtype)
            raw = (ctype * n).from_address(C.cast(ptr, C.c_void_p).value)
            return np.frombuffer(raw, dtype).copy()
        steps = int(b.step_total)
        return plans.PackedBook(take(b.contracts, abi.Contract, plans.CONTRACT_DTYPE, b.contract_count),
                                take(b.steps, abi.Step, plans.STEP_DTYPE, steps),
                                take(b.step_flags, C.c_uint8, np.uint8, steps),
                                take(b.events, abi.Event, plans.EVENT_DTYPE, b.event_total),
                                take(b.intervals, abi.BridgeInterval, plans.INTERVAL_DTYPE, b.interval_total),
                                take(b.bridge_daily, abi.BridgeDaily, plans.DAILY_DTYPE, steps))

    def interpolate(self, prices: np.ndarray) -> np.ndarray:
        """Fills the interpolated members of `prices` (float64, one per note, every
        simulated lane's price set); returns the mask of members to simulate instead."""
        retry = np.zeros(len(prices), np.uint8)
        self.lib.kgpu_shared_plan_interpolate(
            self.handle, prices.ctypes.data_as(C.POINTER(C.c_double)),
            retry.ctypes.data_as(C.POINTER(C.c_uint8)))
        return retry.astype(bool)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.kgpu_shared_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _price_many_planned(engine, notes: Sequence[AutocallableNote], ctx: PricingContext) -> List[float]:
    """price_many on a shared daily grid with the native planner.  The scalar quotes are
    planned first (their errors raise in book order, as plan_book's do), then every group
    runs on the path-major schedule, then the scalar quotes' launch, then the families'
    interpolation; members whose interpolation cancels are simulated after all."""
    if len(notes) > MAX_CONTRACTS:
        raise InvalidInputError("contract batch exceeds 1,048,576 instruments")
    tables = note_tables(notes)
    model = ctx.kgpu_model()
    plan = SharedPlan(tables, model)
    prices = np.full(len(notes), np.nan)
    scalar = np.flatnonzero(plan.note_group < 0)
    batch = [plans.autocallable(notes[i], ctx) for i in scalar]
    pending = range(plan.group_count)
    simulate = None
    try:
        while True:
            for g in pending:
                prices[plan.group_lanes(g)] = engine._run_shared_book(ctx, plan.group_book(g), plan.group_fp32(g))
            if batch:
                for i, e in zip(scalar, engine._run(ctx, batch)):
                    prices[i] = e.price
                batch = []
            retry = plan.interpolate(prices)
            if not retry.any():
                return prices.tolist()
            simulate = retry if simulate is None else (simulate | retry)
            plan.close()
            plan = SharedPlan(tables, model, simulate)
            pending = sorted(set(plan.note_group[retry].tolist()))
    finally:
        plan.close()
