"""Market inputs of the Monte Carlo engines: flat-rate BSM, Heston and local volatility.

Mirrors the model types the reference's Monte Carlo engines read
(crates/kiyosi/src/market/parameters.rs:314-338 PricingContext,
market/heston.rs:58-227 HestonParameters, market/local_volatility.rs:93,322-359).
Times are year fractions from the valuation time on the Actual/365 Fixed clock
(time/date.rs:255-257); the engines need flat rates, as every reference MC engine does
(engines.rs:133-136).
"""
import math
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import abi
from .errors import InvalidInputError

MICROS_PER_YEAR = 365.0 * 86_400_000_000.0


def years_between(start_micros: int, end_micros: int) -> float:
    """Timestamp::years_until (time/date.rs:255-257) on integer microseconds."""
    return float(end_micros - start_micros) / MICROS_PER_YEAR


@dataclass(frozen=True)
class BlackScholesMertonParameters:
    rate: float
    dividend: float
    volatility: float

    def __post_init__(self):
        for name in ("rate", "dividend", "volatility"):
            if not math.isfinite(getattr(self, name)):
                raise InvalidInputError(f"{name} must be finite")
        if self.volatility < 0.0:
            raise InvalidInputError("volatility must be nonnegative")


@dataclass(frozen=True)
class HestonParameters:
    """Heston model with flat rates (market/heston.rs:58-227): initial variance v0,
    long-run variance theta, mean reversion kappa, vol of vol xi, correlation rho.
    The Feller condition is not required."""
    rate: float
    dividend: float
    v0: float
    kappa: float
    theta: float
    xi: float
    rho: float

    def __post_init__(self):
        if min(self.v0, self.theta, self.xi) < 0.0 or self.kappa < 0.0:
            raise InvalidInputError("Heston variances, speed and vol of vol must be nonnegative")
        if not -1.0 <= self.rho <= 1.0:
            raise InvalidInputError("correlation must be in [-1, 1]")


class LocalVolatilitySurface:
    """Bilinear local volatility in (years since times[0], absolute spot), clamped on both
    axes (local_volatility.rs:322-359); values[time][spot]."""

    def __init__(self, rate: float, dividend: float, times: Sequence[float],
                 spots: Sequence[float], values):
        self.rate = float(rate)
        self.dividend = float(dividend)
        self.times = np.ascontiguousarray(times, dtype=np.float64)
        self.spots = np.ascontiguousarray(spots, dtype=np.float64)
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        if self.times.size < 2 or self.spots.size < 2:
            raise InvalidInputError("a local volatility surface needs two nodes per axis")
        if self.values.shape != (self.times.size, self.spots.size):
            raise InvalidInputError("values must have shape (len(times), len(spots))")
        if np.any(np.diff(self.times) <= 0) or np.any(np.diff(self.spots) <= 0):
            raise InvalidInputError("surface nodes must be strictly increasing")
        if np.any(self.values < 0) or not np.all(np.isfinite(self.values)):
            raise InvalidInputError("local volatilities must be finite and nonnegative")

    def at_year(self, time: float, spot: float) -> float:
        def bracket(nodes, value):
            left = min(max(int(np.searchsorted(nodes, value, side="right")) - 1, 0),
                       nodes.size - 2)
            weight = (value - nodes[left]) / (nodes[left + 1] - nodes[left])
            return left, min(max(weight, 0.0), 1.0)

        def interpolate(low, high, weight):
            return low + weight * (high - low) if weight <= 0.5 else high + (1.0 - weight) * (low - high)

        years = self.times - self.times[0]
        row, tw = bracket(years, time)
        col, sw = bracket(self.spots, spot)
        v = self.values
        return interpolate(interpolate(v[row, col], v[row, col + 1], sw),
                           interpolate(v[row + 1, col], v[row + 1, col + 1], sw), tw)


class PricingContext:
    """Spot and model at the valuation time (parameters.rs:314-338)."""

    def __init__(self, model, spot: float):
        if not (spot > 0.0 and math.isfinite(spot)):
            raise InvalidInputError("spot must be positive and finite")
        self.model = model
        self.spot = float(spot)

    @property
    def rate(self) -> float:
        return self.model.rate

    @property
    def dividend(self) -> float:
        return self.model.dividend

    def kgpu_model(self):
        """The kgpu_model struct, keeping the surface arrays alive on the returned object."""
        m = abi.Model()
        m.spot = self.spot
        m.rate = self.model.rate
        m.dividend = self.model.dividend
        model = self.model
        if isinstance(model, BlackScholesMertonParameters):
            m.kind = abi.MODEL_BSM
            m.volatility = model.volatility
        elif isinstance(model, HestonParameters):
            m.kind = abi.MODEL_HESTON
            m.v0, m.kappa, m.theta, m.xi, m.rho = (model.v0, model.kappa, model.theta,
                                                   model.xi, model.rho)
        elif isinstance(model, LocalVolatilitySurface):
            m.kind = abi.MODEL_LOCAL_VOL
            m.lv_time_count = model.times.size
            m.lv_spot_count = model.spots.size
            P = abi.C.POINTER(abi.C.c_double)
            m.lv_times = model.times.ctypes.data_as(P)
            m.lv_spots = model.spots.ctypes.data_as(P)
            m.lv_values = model.values.ctypes.data_as(P)
            m._keep = (model.times, model.spots, model.values)
        else:
            raise InvalidInputError(f"unsupported model {type(model).__name__}")
        return m


def log_ratio(numerator: float, denominator: float) -> float:
    """numerics.rs:80-92."""
    relative = (numerator - denominator) / denominator
    if abs(relative) < 0.5:
        return math.log1p(relative)
    ratio = numerator / denominator
    if ratio != 0.0 and math.isfinite(ratio) and abs(ratio) >= 2.2250738585072014e-308:
        return math.log(ratio)
    return _safe_log(numerator) - _safe_log(denominator)


def _safe_log(x: float) -> float:
    return -math.inf if x == 0.0 else math.log(x)


def safe_log_returns(spot: float):
    """safe_log_returns (monte_carlo.rs:2139-2145)."""
    log_spot = math.log(spot)
    low = math.log(2.2250738585072014e-308) + 1.0
    high = math.log(1.7976931348623157e308) - 1.0
    return max(low, low - log_spot), min(high, high - log_spot)


def discounted_product(scale: float, weight: float, log_discount: float) -> float:
    """numerics.rs:226-238."""
    value = scale * weight
    discount = math.exp(log_discount) if log_discount < 709.0 else math.inf
    if scale == 0.0 or weight == 0.0:
        return 0.0
    if _is_normal(discount) and _is_normal(value):
        return value * discount
    return math.copysign(math.exp(math.log(scale) + math.log(abs(weight)) + log_discount), weight)


def _is_normal(x: float) -> bool:
    return math.isfinite(x) and abs(x) >= 2.2250738585072014e-308
