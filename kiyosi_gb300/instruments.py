"""Contracts priced by the Monte Carlo engines.

These mirror the reference's instruments (crates/kiyosi/src/instruments/) for the fields
the Monte Carlo path reads.  Observation schedules are given as year fractions after the
valuation time (Actual/365 Fixed); calendar and schedule generation are host-side
inputs, so callers pass the resolved observation times.
"""
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

from .errors import InvalidInputError

CALL = "call"
PUT = "put"


def _sign(option_type: str) -> float:
    if option_type not in (CALL, PUT):
        raise InvalidInputError("option_type must be 'call' or 'put'")
    return 1.0 if option_type == CALL else -1.0


_SHARED_TIMES: dict = {}


def _shared_times(times: tuple) -> tuple:
    """One tuple object per distinct monitoring schedule, so that the notes of a book that
    share a schedule share the object (host planners key their caches on it)."""
    shared = _SHARED_TIMES.get(times)
    if shared is None:
        if len(_SHARED_TIMES) >= 4096:
            _SHARED_TIMES.clear()
        shared = _SHARED_TIMES[times] = times
    return shared


def _times(values: Sequence[float], expiry: float, name: str, start: float = 0.0) -> List[float]:
    out = [float(v) for v in values]
    if any(not math.isfinite(v) for v in out):
        raise InvalidInputError(f"{name} must be finite")
    if any(b <= a for a, b in zip(out, out[1:])):
        raise InvalidInputError(f"{name} must be strictly increasing")
    if out and (out[0] < start or out[-1] > expiry):
        raise InvalidInputError(f"{name} must lie within the contract's life")
    return out


@dataclass(frozen=True)
class EuropeanOption:
    option_type: str
    strike: float
    expiry: float  # years after valuation

    def __post_init__(self):
        _sign(self.option_type)
        if not (self.strike > 0.0 and self.expiry >= 0.0):
            raise InvalidInputError("strike must be positive and expiry nonnegative")

    @property
    def sign(self) -> float:
        return _sign(self.option_type)


@dataclass(frozen=True)
class AmericanOption(EuropeanOption):
    pass


@dataclass(frozen=True)
class DigitalOption(EuropeanOption):
    payout: Optional[float] = None  # cash amount; None pays the asset


BARRIER_TYPES = ("down_and_out", "down_and_in", "up_and_out", "up_and_in")


@dataclass(frozen=True)
class BarrierOption(EuropeanOption):
    """Single-barrier vanilla option (instruments/barrier.rs).  `observation_times`
    (years after valuation, strictly increasing, within the option's life) makes the
    monitoring scheduled; None monitors continuously (ObservationMode::Continuous).
    `rebate` is paid at expiry unless `rebate_timing` is 'at_hit', which only knock-outs
    may use (barrier.rs:198-202)."""
    barrier: float = 0.0
    barrier_type: str = "down_and_out"
    rebate: float = 0.0
    rebate_timing: str = "at_expiry"
    observation_times: Optional[Sequence[float]] = None

    def __post_init__(self):
        super().__post_init__()
        if self.barrier_type not in BARRIER_TYPES:
            raise InvalidInputError(f"barrier_type must be one of {BARRIER_TYPES}")
        if not (self.barrier > 0.0 and math.isfinite(self.barrier)):
            raise InvalidInputError("barrier must be positive and finite")
        if not (self.rebate >= 0.0 and math.isfinite(self.rebate)):
            raise InvalidInputError("rebate must be nonnegative and finite")
        if self.rebate_timing not in ("at_expiry", "at_hit"):
            raise InvalidInputError("rebate_timing must be 'at_expiry' or 'at_hit'")
        if self.is_knock_in and self.rebate_timing == "at_hit":
            raise InvalidInputError("knock-in rebates cannot pay at hit")
        if self.observation_times is not None:
            times = tuple(_times(self.observation_times, self.expiry, "observation_times"))
            if not times:
                raise InvalidInputError("a scheduled barrier needs at least one observation time")
            object.__setattr__(self, "observation_times", times)

    @property
    def continuous(self) -> bool:
        return self.observation_times is None

    @property
    def is_up(self) -> bool:
        return self.barrier_type.startswith("up")

    @property
    def is_knock_in(self) -> bool:
        return self.barrier_type.endswith("_in")


DOUBLE_BARRIER_TYPES = ("knock_out", "knock_in")


@dataclass(frozen=True)
class DoubleBarrierOption(EuropeanOption):
    """Double-barrier vanilla option (instruments/double_barrier.rs): knocked out (or in)
    when the spot reaches `lower` or `upper`.  Monitoring, rebate and its timing follow
    BarrierOption; kiyosi represents it as the lower down-barrier plus the upper level."""
    lower: float = 0.0
    upper: float = 0.0
    barrier_type: str = "knock_out"
    rebate: float = 0.0
    rebate_timing: str = "at_expiry"
    observation_times: Optional[Sequence[float]] = None

    def __post_init__(self):
        super().__post_init__()
        if self.barrier_type not in DOUBLE_BARRIER_TYPES:
            raise InvalidInputError(f"barrier_type must be one of {DOUBLE_BARRIER_TYPES}")
        if not (self.lower > 0.0 and math.isfinite(self.lower)):
            raise InvalidInputError("barrier must be positive and finite")
        if not math.isfinite(self.upper) or self.upper <= self.lower:
            raise InvalidInputError("double barriers require finite 0 < lower < upper")
        if not (self.rebate >= 0.0 and math.isfinite(self.rebate)):
            raise InvalidInputError("rebate must be nonnegative and finite")
        if self.rebate_timing not in ("at_expiry", "at_hit"):
            raise InvalidInputError("rebate_timing must be 'at_expiry' or 'at_hit'")
        if self.is_knock_in and self.rebate_timing == "at_hit":
            raise InvalidInputError("knock-in rebates cannot pay at hit")
        if self.observation_times is not None:
            times = tuple(_times(self.observation_times, self.expiry, "observation_times"))
            if not times:
                raise InvalidInputError("a scheduled barrier needs at least one observation time")
            object.__setattr__(self, "observation_times", times)

    @property
    def is_knock_in(self) -> bool:
        return self.barrier_type == "knock_in"

    @property
    def continuous(self) -> bool:
        return self.observation_times is None


@dataclass(frozen=True)
class AveragePriceOption:
    """Continuously averaged price option (instruments/asian.rs AverageTerms): the
    average of the spot over [averaging_start, expiry] (years after valuation) against
    `strike`.  Valuation is at the contract's effective time, so no realized average
    exists yet; averaging may start later (a forward start)."""
    option_type: str
    strike: float
    expiry: float
    averaging_start: float = 0.0

    def __post_init__(self):
        _sign(self.option_type)
        if not (self.strike > 0.0 and math.isfinite(self.strike)):
            raise InvalidInputError("strike must be positive and finite")
        if not (math.isfinite(self.expiry) and self.expiry >= 0.0):
            raise InvalidInputError("expiry must be finite and nonnegative")
        if not (0.0 <= self.averaging_start <= self.expiry):
            raise InvalidInputError("averaging must start within the contract's life")

    @property
    def sign(self) -> float:
        return _sign(self.option_type)

    @property
    def period(self) -> float:
        return self.expiry - self.averaging_start


@dataclass(frozen=True)
class ArithmeticAveragePriceOption(AveragePriceOption):
    """Arithmetic continuous average (ArithmeticAveragePriceOption)."""


@dataclass(frozen=True)
class GeometricAveragePriceOption(AveragePriceOption):
    """Geometric continuous average (GeometricAveragePriceOption)."""


@dataclass(frozen=True)
class AsianOption:
    """Arithmetic average-price option on the spots at `fixings` (years)."""
    option_type: str
    strike: float
    expiry: float
    fixings: Sequence[float]

    def __post_init__(self):
        _sign(self.option_type)
        object.__setattr__(self, "fixings", tuple(_times(self.fixings, self.expiry, "fixings")))
        if not self.fixings:
            raise InvalidInputError("an Asian option needs at least one fixing")

    @property
    def sign(self) -> float:
        return _sign(self.option_type)


@dataclass(frozen=True)
class Observation:
    """One observation date of an autocallable: knock-out level (absolute spot, or None),
    coupon barrier level (absolute spot, or None) and the annual coupon rate accrued on
    knock-out (snowball)."""
    time: float
    knock_out_level: Optional[float] = None
    coupon_barrier_level: Optional[float] = None
    coupon_rate: float = 0.0

    def __hash__(self):
        # The field hash, computed once: planners key their caches on observations.
        h = self.__dict__.get("_hash")
        if h is None:
            h = hash((self.time, self.knock_out_level, self.coupon_barrier_level, self.coupon_rate))
            object.__setattr__(self, "_hash", h)
        return h


BARRIER_STATES = (None, "no_event", "knocked_in", "knocked_out")


@dataclass(frozen=True)
class AutocallableNote:
    """Snowball, binary/ternary snowball or Phoenix note (instruments/autocallable.rs).

    knocked-in redemption is either the capped downside (`fixed_knock_in_coupon` None):
        principal + rebate + (clamp(S, lower, upper) - upper) / initial_spot
    or a fixed annual coupon.  Without knock-in the note pays principal + rebate +
    maturity_coupon_rate x accrual.  Phoenix notes pay `period_coupon` at each coupon
    observation whose barrier is met.

    Times are year fractions after the valuation instant, so a seasoned note has a
    negative `effective_time` and may list observation and monitoring times at or before
    zero; `expiry` 0 values the note at expiry.  `barrier_state` is the note's history
    strictly before valuation (AutocallableBarrierState: None when unknown, 'no_event',
    'knocked_in', 'knocked_out'); a note with past observations or past daily monitoring
    needs it (AutocallableNote::prior, instruments/autocallable.rs:1320-1369).
    """
    initial_spot: float
    expiry: float
    observations: Sequence[Observation]
    knock_in_level: Optional[float] = None
    knock_in_times: Optional[Sequence[float]] = None  # daily monitoring; None = expiry only
    upper_strike: float = 0.0
    lower_strike: float = 0.0
    maturity_coupon_rate: float = 0.0
    period_coupon: float = 0.0
    fixed_knock_in_coupon: Optional[float] = None
    principal: float = 1.0
    rebate_rate: float = 0.0
    annual_rebate_rate: float = 0.0
    effective_time: float = 0.0
    barrier_state: Optional[str] = None

    def __post_init__(self):
        if not (math.isfinite(self.effective_time) and math.isfinite(self.expiry)):
            raise InvalidInputError("effective and expiry times must be finite")
        if self.effective_time > 0.0 or self.expiry < 0.0:
            # validate_life (instruments/monitoring.rs:470-481)
            raise InvalidInputError("valuation outside contract life")
        if self.effective_time > self.expiry:
            raise InvalidInputError("the effective time must not follow expiry")
        if self.barrier_state not in BARRIER_STATES:
            raise InvalidInputError(f"barrier_state must be one of {BARRIER_STATES}")
        if self.barrier_state == "knocked_in" and self.knock_in_level is None:
            raise InvalidInputError("knock-in state requires a knock-in barrier")
        obs = tuple(self.observations)
        object.__setattr__(self, "observations", obs)
        _times([o.time for o in obs], self.expiry, "observations", self.effective_time)
        if self.knock_in_times is not None:
            object.__setattr__(self, "knock_in_times",
                               _shared_times(tuple(_times(self.knock_in_times, self.expiry, "knock_in_times",
                                                          self.effective_time))))
        if not self.initial_spot > 0.0:
            raise InvalidInputError("initial spot must be positive")
        if self.upper_strike == 0.0:
            object.__setattr__(self, "upper_strike", self.initial_spot)
        if self.lower_strike > self.upper_strike:
            raise InvalidInputError("lower strike must not exceed the upper strike")

    def rebate_payment(self, time: float) -> float:
        """AutocallableNote::rebate_payment (instruments/autocallable.rs:1415-1418)."""
        return self.rebate_rate + self.annual_rebate_rate * (time - self.effective_time)

    def knock_out_payment(self, obs: Observation) -> float:
        """AutocallableNote::knock_out_payment (instruments/autocallable.rs:1419-1424)."""
        return (self.principal + self.rebate_payment(obs.time)
                + obs.coupon_rate * (obs.time - self.effective_time))

    def terminal(self, spot: float, knocked_in: bool) -> float:
        """AutocallableNote::terminal (instruments/autocallable.rs:1396-1414)."""
        base = self.principal + self.rebate_payment(self.expiry)
        if knocked_in:
            if self.fixed_knock_in_coupon is None:
                clamped = min(max(spot, self.lower_strike), self.upper_strike)
                return base + (clamped - self.upper_strike) / self.initial_spot
            coupon = self.fixed_knock_in_coupon
        else:
            coupon = self.maturity_coupon_rate
        return base + coupon * (self.expiry - self.effective_time)

    @property
    def knocked_in(self) -> bool:
        """Knocked in before valuation (the recorded history)."""
        return self.barrier_state == "knocked_in"

    @property
    def daily_knock_in(self) -> bool:
        """Knock-in monitored on every listed date (KnockInObservation::EveryTradingDay)
        rather than at expiry only."""
        return self.knock_in_level is not None and self.knock_in_times is not None

    def observes_knock_in(self, time: float) -> bool:
        """AutocallableNote::observes_knock_in (instruments/autocallable.rs:1075-1080)."""
        if self.knock_in_level is None:
            return False
        if self.knock_in_times is not None:
            return time in self.knock_in_times
        return time == self.expiry

    def below_knock_in(self, spot: float) -> bool:
        """Terms::below_knock_in (instruments/autocallable.rs:1652-1654): strict."""
        return self.knock_in_level is not None and spot < self.knock_in_level

    def observation_coupon(self, obs: Optional["Observation"], spot: float) -> float:
        """AutocallableNote::observation_coupon (instruments/autocallable.rs:1164-1174)."""
        if obs is not None and obs.coupon_barrier_level is not None and spot >= obs.coupon_barrier_level:
            return self.period_coupon
        return 0.0

    def knock_in_affects_payoff(self) -> bool:
        """instruments/autocallable.rs:1323-1332."""
        if self.knock_in_level is None:
            return False
        if self.fixed_knock_in_coupon is not None:
            return self.fixed_knock_in_coupon != self.maturity_coupon_rate
        return self.lower_strike != self.upper_strike or self.maturity_coupon_rate != 0.0


def SnowballOption(maturity_coupon_rate: float, initial_spot: float, knock_in_level: float,
                   upper_strike: float, lower_strike: float, expiry: float,
                   autocall_observations: Sequence[Observation],
                   knock_in_times: Optional[Sequence[float]] = None, **kw) -> AutocallableNote:
    """Basic snowball: knock-out pays principal plus the accrued annual coupon; otherwise
    the maturity coupon if no knock-in occurred, or the capped downside after knock-in."""
    return AutocallableNote(initial_spot=initial_spot, expiry=expiry,
                            observations=autocall_observations, knock_in_level=knock_in_level,
                            knock_in_times=knock_in_times, upper_strike=upper_strike,
                            lower_strike=lower_strike, maturity_coupon_rate=maturity_coupon_rate,
                            **kw)


def PhoenixOption(coupon_per_period: float, initial_spot: float, knock_in_level: float,
                  upper_strike: float, lower_strike: float, expiry: float,
                  observations: Sequence[Observation],
                  knock_in_times: Optional[Sequence[float]] = None, **kw) -> AutocallableNote:
    """Phoenix: `coupon_per_period` at each observation whose coupon barrier is met."""
    return AutocallableNote(initial_spot=initial_spot, expiry=expiry, observations=observations,
                            knock_in_level=knock_in_level, knock_in_times=knock_in_times,
                            upper_strike=upper_strike, lower_strike=lower_strike,
                            period_coupon=coupon_per_period, **kw)


@dataclass(frozen=True)
class Accumulator:
    """Accumulator (instruments/accumulator.rs): buys `daily_quantity` at each
    accumulation date (times `acceleration` when the spot is beyond the strike), knocked
    out at observation dates; settles quantity x (S - K) for calls."""
    option_type: str
    strike: float
    knock_out_level: float
    expiry: float
    accumulation_times: Sequence[float]
    knock_out_times: Sequence[float]
    daily_quantity: float = 1.0
    acceleration: float = 2.0
    quantity: float = 0.0           # accumulated before valuation
    knock_out_settled: bool = False  # knocked out and settled before valuation

    def __post_init__(self):
        _sign(self.option_type)
        object.__setattr__(self, "accumulation_times",
                           tuple(_times(self.accumulation_times, self.expiry, "accumulation_times")))
        object.__setattr__(self, "knock_out_times",
                           tuple(_times(self.knock_out_times, self.expiry, "knock_out_times")))

    @property
    def sign(self) -> float:
        return _sign(self.option_type)

    def purchase(self, spot: float) -> float:
        """Accumulator::purchase (instruments/accumulator.rs:486-499): the daily quantity,
        times the acceleration when the spot is below (call) or above (put) the strike."""
        distance = spot - self.strike
        accelerated = distance < 0.0 if self.option_type == CALL else distance > 0.0
        return self.daily_quantity * self.acceleration if accelerated else self.daily_quantity

    def unit_payoff(self, spot: float) -> float:
        return spot - self.strike if self.option_type == CALL else self.strike - spot

    def is_knock_out(self, spot: float) -> bool:
        return spot >= self.knock_out_level if self.option_type == CALL else spot <= self.knock_out_level
