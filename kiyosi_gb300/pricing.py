"""Monte Carlo engines with kiyosi's Python surface, pricing on the GPU.

Class names, keyword arguments and MonteCarloEstimate fields mirror
`kiyosi.pricing` (crates/kiyosi-python/src/engines/monte_carlo.rs:90-344,476-510).
Added keywords select the GPU arithmetic (`precision`), the launch `schedule` and the
`device`.  Pricing calls go through the C ABI of include/kgpu.h; plans are built on the
host by kiyosi_gb300.plans.
"""
import ctypes as C
import math
import os
from dataclasses import dataclass, replace
from typing import Optional, Sequence, Tuple

import numpy as np

from . import abi, plans
from ._native import context
from .errors import InvalidInputError, UnsupportedOperationError
from .instruments import (Accumulator, AmericanOption, AsianOption, AutocallableNote,
                          AveragePriceOption, BarrierOption, DigitalOption, EuropeanOption)
from .market import PricingContext

PSEUDO_RANDOM = "pseudo_random"
SOBOL = "sobol"
_SAMPLING = {PSEUDO_RANDOM: abi.SAMPLING_PSEUDO_RANDOM, SOBOL: abi.SAMPLING_SOBOL}
_PRECISION = {"fp64": abi.PRECISION_FP64, "fp32": abi.PRECISION_FP32}
_SCHEDULE = {"plain": abi.SCHEDULE_PLAIN, "persistent": abi.SCHEDULE_PERSISTENT,
             "shared_grid": abi.SCHEDULE_SHARED_GRID, "lane_refill": abi.SCHEDULE_LANE_REFILL}
Z95 = 1.959963984540054


class MonteCarloSampling:
    PSEUDO_RANDOM = PSEUDO_RANDOM
    SOBOL = SOBOL


@dataclass(frozen=True)
class MonteCarloEstimate:
    """MonteCarloEstimate (engines/monte_carlo.rs:858-1001): price, optional standard
    error and 95% interval, uncertainty status and replay seed; plus the GPU's i.i.d.
    sample error (also for Sobol) and the path-step counts of the run."""
    price: float
    standard_error: Optional[float]
    uncertainty_status: str
    seed: Optional[int]
    sample_error: float = 0.0
    path_steps: float = 0.0
    executed_steps: float = 0.0

    @property
    def confidence_interval(self) -> Optional[Tuple[float, float]]:
        if self.standard_error is None:
            return None
        half = Z95 * self.standard_error
        return (self.price - half, self.price + half)

    @staticmethod
    def known(value: float) -> "MonteCarloEstimate":
        return MonteCarloEstimate(value, None, "insufficient_observations", None)

    @staticmethod
    def from_native(e: abi.Estimate) -> "MonteCarloEstimate":
        status = abi.UNCERTAINTY_NAMES[e.uncertainty_status]
        return MonteCarloEstimate(e.price, e.standard_error if e.uncertainty_status == 0 else None,
                                  status, int(e.seed), e.sample_error, e.path_steps,
                                  e.executed_steps)


def _resolve_seed(seed):
    if seed is not None:
        if not (0 <= int(seed) < 2 ** 64):
            raise InvalidInputError("seed must be an unsigned 64-bit integer")
        return int(seed)
    return int.from_bytes(os.urandom(8), "little")


class _MonteCarloEngine:
    _STATE_FIELDS = ("path_count", "seed", "max_active_workers", "sampling", "antithetic",
                     "precision", "schedule", "device", "tile_paths", "tuning")

    def __init__(self, *, path_count: int = 131_072, seed: Optional[int] = None,
                 max_active_workers: int = 0, sampling: str = PSEUDO_RANDOM,
                 antithetic: bool = False, precision: str = "fp64", schedule: str = "plain",
                 device: int = 0, tile_paths: int = 0, tuning: Optional[str] = None):
        if not (1 <= int(path_count) <= 2_147_483_647):
            raise InvalidInputError("path_count must be positive")
        if int(max_active_workers) < 0:
            raise InvalidInputError("max_active_workers must be nonnegative")
        if sampling not in _SAMPLING:
            raise InvalidInputError(f"unknown sampling {sampling!r}")
        if sampling == SOBOL and (int(path_count) & (int(path_count) - 1)) != 0:
            raise InvalidInputError("path_count must be a power of two for Sobol sampling")
        if precision not in _PRECISION:
            raise InvalidInputError(f"unknown precision {precision!r}")
        if schedule not in _SCHEDULE:
            raise InvalidInputError(f"unknown schedule {schedule!r}")
        if tuning not in (None, "auto"):
            raise InvalidInputError("tuning must be None or 'auto'")
        self.path_count = int(path_count)
        self.seed = None if seed is None else int(seed)
        self.max_active_workers = int(max_active_workers)
        self.sampling = sampling
        self.antithetic = bool(antithetic)
        self.precision = precision
        self.schedule = schedule
        self.device = int(device)
        self.tile_paths = int(tile_paths)
        # 'auto': the persistent schedule's launch shape is tuned per kind of book
        # (kiyosi_gb300.autotune); prices do not depend on it.
        self.tuning = tuning

    def _kwargs(self):
        return {k: getattr(self, k) for k in self._STATE_FIELDS if hasattr(self, k)}

    def replace(self, **changes):
        kw = self._kwargs()
        kw.update(changes)
        return type(self)(**kw)

    def with_resolved_seed(self):
        """An engine with a concrete seed (entropy when none is set), other controls kept."""
        return self.replace(seed=_resolve_seed(self.seed))

    def _settings(self, seed: int) -> abi.Settings:
        return abi.Settings(path_count=self.path_count, sampling=_SAMPLING[self.sampling],
                            antithetic=int(self.antithetic),
                            precision=_PRECISION[self.precision],
                            schedule=_SCHEDULE[self.schedule], tile_paths=self.tile_paths,
                            seed=seed)

    def _run_group(self, ctx: PricingContext, lane_plans):
        """Prices the lanes of one shared daily grid with the path-major schedule (one
        path per sample settles every lane)."""
        return self._run(ctx, lane_plans, schedule=abi.SCHEDULE_SHARED_GRID)

    def _run_shared_book(self, ctx: PricingContext, book: abi.Book, lane_fp32):
        """Prices the lanes of one shared daily grid from a packed group book (the native
        planner's, portfolio.SharedPlan) with the path-major schedule; returns the lanes'
        prices (float64, contract order).  As in _run, FP32 lanes whose plan FP32 cannot
        carry are priced by the FP64 kernels in a second launch."""
        seed = _resolve_seed(self.seed)
        settings = self._settings(seed)
        settings.schedule = abi.SCHEDULE_SHARED_GRID
        n = book.contract_count
        parts = [(settings, list(range(n)))]
        if settings.precision == abi.PRECISION_FP32:
            model_ok = plans.fp32_model_ok(ctx)
            wide = [j for j in range(n) if not (model_ok and lane_fp32[j])]
            if wide:
                fp64 = abi.Settings.from_buffer_copy(settings)
                fp64.precision = abi.PRECISION_FP64
                narrow = sorted(set(range(n)) - set(wide))
                parts = [(settings, narrow), (fp64, wide)]
        native = context(self.device)
        model = ctx.kgpu_model()
        prices = np.zeros(n, np.float64)
        for part_settings, members in parts:
            if not members:
                continue
            sub = book
            if len(members) != n:
                chosen = (abi.Contract * len(members))(*[book.contracts[j] for j in members])
                sub = abi.Book.from_buffer_copy(book)
                sub.contract_count = len(members)
                sub.contracts = C.cast(chosen, C.POINTER(abi.Contract))
            out = (abi.Estimate * len(members))()
            native.check(native.lib.kgpu_price_book(native.handle, C.byref(model), C.byref(sub),
                                                    C.byref(part_settings), out, None))
            prices[members] = np.frombuffer(out, np.dtype(abi.Estimate))["price"]
        return prices

    def _run(self, ctx: PricingContext, contract_plans, path_counts=None, cancel=None, schedule=None):
        """Prices plans (Known or ContractPlan) through kgpu_price_book."""
        seed = _resolve_seed(self.seed)
        results = [None] * len(contract_plans)
        builder = plans.BookBuilder()
        index = []
        counts = []
        for i, p in enumerate(contract_plans):
            if isinstance(p, plans.Known):
                if not math.isfinite(p.value):
                    from .errors import ComputationFailureError
                    raise ComputationFailureError("Monte Carlo produced a non-finite result")
                results[i] = MonteCarloEstimate(p.value, 0.0 if self.sampling == PSEUDO_RANDOM
                                                else None,
                                                "available" if self.sampling == PSEUDO_RANDOM
                                                else "unsupported_sampling", None)
            else:
                builder.add(p)
                index.append(i)
                counts.append(path_counts[i] if path_counts is not None else 0)
        if not index:
            return results
        settings = self._settings(seed)
        if schedule is not None:
            settings.schedule = schedule
        # FP32 kernels cannot carry every plan (plans.fp32_representable): those
        # contracts are priced by the FP64 kernels in a second launch.
        wide = []
        if settings.precision == abi.PRECISION_FP32:
            wide = [j for j, i in enumerate(index)
                    if not plans.fp32_representable(contract_plans[i], ctx)]
        narrow = set(wide)
        parts = [(settings, [j for j in range(len(index)) if j not in narrow])]
        if wide:
            fp64 = abi.Settings.from_buffer_copy(settings)
            fp64.precision = abi.PRECISION_FP64
            parts.append((fp64, wide))
        native = context(self.device)
        model = ctx.kgpu_model()
        flag = None if cancel is None else C.byref(cancel)
        for part_settings, members in parts:
            if not members:
                continue
            if len(parts) == 1:
                packed = builder.build(counts)
            else:
                sub = plans.BookBuilder()
                for j in members:
                    sub.add(builder.plans[j])
                packed = sub.build([counts[j] for j in members])
            out = (abi.Estimate * len(members))()
            book = packed.struct()
            if (schedule is None and self.tuning == "auto" and self.schedule == "persistent"
                    and part_settings.precision == settings.precision):
                from . import autotune
                shape, _ = autotune.tune(native, ctx, packed, part_settings)
                part_settings = autotune.apply(part_settings, shape)
            native.check(native.lib.kgpu_price_book(native.handle, C.byref(model), C.byref(book),
                                                    C.byref(part_settings), out, flag))
            for k, j in enumerate(members):
                i = index[j]
                results[i] = MonteCarloEstimate.from_native(out[k])
                addend = getattr(contract_plans[i], "addend", None)
                if addend is not None:
                    results[i] = replace(results[i], price=results[i].price + addend(ctx))
        return results

    def price(self, contract, ctx: PricingContext) -> float:
        return self.price_with_statistics(contract, ctx).price

    def price_with_seed(self, contract, ctx: PricingContext):
        e = self.price_with_statistics(contract, ctx)
        return e.price, e.seed

    def _scenario_prices(self, contract, contexts):
        """Prices `contract` in each context with this engine's seed.  Engines with a
        per-contract plan price every context in one book (one launch, shared random
        numbers); the others price them one by one."""
        return self._scenario_prices_of([(contract, c) for c in contexts])

    def _scenario_prices_of(self, pairs):
        """Prices (contract, context) pairs with this engine's seed, in one book when the
        engine has per-contract plans (the time stencils' scenarios are the contract
        valued at shifted instants)."""
        plan = getattr(self, "_plan", None)
        if plan is None:
            return [self.price(contract, c) for contract, c in pairs]
        return [e.price for e in self._run(pairs[0][1], [plan(contract, c) for contract, c in pairs])]


class MonteCarloVanillaEngine(_MonteCarloEngine):
    """European (exact terminal sampling) and American (LSMC) vanilla options.

    `terminal_sampling=False` steps `step_count` uniform log-Euler steps instead of the
    exact terminal draw (the reference's generic D-dimensional sampler).  American
    options use `step_count` exercise intervals; under Heston `substeps` Euler steps per
    interval and `basis` 'poly3' (default) or 'mlp'."""
    _STATE_FIELDS = _MonteCarloEngine._STATE_FIELDS + (
        "step_count", "terminal_sampling", "basis", "substeps", "mlp_epochs", "mlp_batch",
        "mlp_learning_rate", "mlp_seed")

    def __init__(self, *, step_count: int = 50, terminal_sampling: bool = True,
                 basis: Optional[str] = None, substeps: int = 5, mlp_epochs: int = 5,
                 mlp_batch: int = 8192, mlp_learning_rate: float = 1e-3, mlp_seed: int = 0,
                 **kw):
        if not (1 <= int(step_count) <= 10_000):
            raise InvalidInputError("step_count is outside the supported Monte Carlo range")
        super().__init__(**kw)
        self.step_count = int(step_count)
        self.terminal_sampling = bool(terminal_sampling)
        self.basis = basis
        self.substeps = int(substeps)
        self.mlp_epochs = int(mlp_epochs)
        self.mlp_batch = int(mlp_batch)
        self.mlp_learning_rate = float(mlp_learning_rate)
        self.mlp_seed = int(mlp_seed)

    def price_american_out_of_sample(self, option, ctx: PricingContext, fresh_seed: int):
        from .lsmc import price_american_out_of_sample
        return price_american_out_of_sample(self, option, ctx, fresh_seed)

    def _plan(self, option, ctx):
        if self.terminal_sampling:
            return plans.european(option, ctx)
        if option.expiry == 0.0:
            return plans.Known(max(option.sign * (ctx.spot - option.strike), 0.0))
        return plans.path_vanilla(option, ctx, self.step_count)

    def price_with_statistics(self, option, ctx: PricingContext) -> MonteCarloEstimate:
        if isinstance(option, AmericanOption):
            from .lsmc import price_american
            return price_american(self, option, ctx)
        return self._run(ctx, [self._plan(option, ctx)])[0]

    def price_with_greeks(self, option, ctx: PricingContext, request, shifts=None):
        """Greeks by bump-and-reprice with a pinned seed: European options with every
        scenario in one launch (monte_carlo.rs:1334-1409, european_greek_prices),
        American options with the bumped contexts in batched LSMC scenario calls
        (american.rs:820-946, 1487-1687)."""
        if isinstance(option, AmericanOption):
            from .lsmc import american_greeks
            return american_greeks(self, option, ctx, request, shifts)
        from .greeks import numerical_greeks
        return numerical_greeks(self, option, ctx, request, shifts)

    def price_strikes(self, option, ctx: PricingContext, strikes: Sequence[float]):
        opts = [replace(option, strike=float(k)) for k in strikes]
        return [e.price for e in self._run(ctx, [self._plan(o, ctx) for o in opts])]


class MonteCarloAsianEngine(_MonteCarloEngine):
    """kiyosi's MonteCarloAsianEngine (engines/monte_carlo/asian.rs) on continuously
    averaged ArithmeticAveragePriceOption / GeometricAveragePriceOption contracts under
    flat BSM rates:
    - geometric averages sample their exact law with one normal;
    - arithmetic averages integrate `step_count` trapezoid intervals (default 50, the
      reference's grid default), with the first interval integrated in closed form and
      a geometric control variate near the money.

    AsianOption (the arithmetic mean of the spots on discrete fixing dates, under any
    model) is priced on its fixing grid, refined to `step_count` uniform steps only
    when one is given."""
    _STATE_FIELDS = _MonteCarloEngine._STATE_FIELDS + ("step_count",)

    def __init__(self, *, step_count: Optional[int] = None, **kw):
        super().__init__(**kw)
        if step_count is not None and not (2 <= int(step_count) <= 10_000):
            raise InvalidInputError("step_count must be in 2..=10000")
        self.step_count = None if step_count is None else int(step_count)

    def _average(self, options, ctx: PricingContext):
        """Prices average-price options with one resolved seed; a controlled mean that
        comes out negative is priced again without the control on the same seed
        (ArithmeticGrid::sample, asian.rs:602-633)."""
        engine = self.with_resolved_seed()
        steps = self.step_count or 50
        first = [plans.average(o, ctx, steps) for o in options]
        out = engine._run(ctx, first)
        redo = [i for i, (p, e) in enumerate(zip(first, out))
                if isinstance(p, plans.ContractPlan) and p.record["flags"] & abi.C_AVERAGE_CONTROL
                and e.price < 0.0]
        if redo:
            again = engine._run(ctx, [plans.average(options[i], ctx, steps, control=False)
                                      for i in redo])
            for i, e in zip(redo, again):
                out[i] = e
        return out

    def price_with_statistics(self, option, ctx: PricingContext):
        if isinstance(option, AveragePriceOption):
            return self._average([option], ctx)[0]
        return self._run(ctx, [plans.asian(option, ctx, self.step_count)])[0]

    def price_with_greeks(self, option, ctx: PricingContext, request, shifts=None):
        """Native delta and gamma from the price's normals (asian.rs:740-784, 1087-1178,
        with the geometric control's exact delta and gamma added back)."""
        if not isinstance(option, AveragePriceOption):
            raise UnsupportedOperationError("Greeks of discrete-fixing Asian options are not built")
        from .greeks import native_greeks
        steps = self.step_count or 50

        def plan_for(option, ctx):
            return plans.average(option, ctx, steps)

        def without_control(option, ctx):
            return plans.average(option, ctx, steps, control=False)

        def discontinuity(radius):
            return option.expiry == 0.0 and ctx.spot - radius <= option.strike <= ctx.spot + radius
        return native_greeks(self, option, ctx, request, plan_for, shifts, discontinuity=discontinuity,
                             redo_without_control=without_control)

    def _scenario_prices(self, option, contexts):
        if isinstance(option, AveragePriceOption):
            return [self._average([option], c)[0].price for c in contexts]
        return super()._scenario_prices(option, contexts)

    def price_strikes(self, option: AveragePriceOption, ctx: PricingContext,
                      strikes: Sequence[float]):
        """Prices across strikes on common paths: every strike replays its scalar price
        (price_strikes, asian.rs:197-340), duplicates included."""
        if not isinstance(option, AveragePriceOption):
            raise InvalidInputError("price_strikes takes an average-price option")
        for k in strikes:
            if not (math.isfinite(k) and k > 0.0):
                raise InvalidInputError("strike must be positive and finite")
        unique = sorted(set(float(k) for k in strikes))
        prices = dict(zip(unique, (e.price for e in self._average(
            [replace(option, strike=k) for k in unique], ctx))))
        return [prices[float(k)] for k in strikes]


class _TimeStepsMixin:
    """`time_steps` (added keyword, default None): refines each contract's date grid so
    that no path step is much longer than its life / time_steps (plans.refine_grid,
    QuantLib's TimeGrid rule).  BSM steps are exact and need none; the Euler schemes of
    local volatility and Heston use it to bound the discretisation error."""

    def _init_time_steps(self, time_steps):
        if time_steps is not None and int(time_steps) < 1:
            raise InvalidInputError("time_steps must be positive")
        self.time_steps = None if time_steps is None else int(time_steps)


class MonteCarloAutocallableEngine(_MonteCarloEngine, _TimeStepsMixin):
    """Snowball / Phoenix notes (autocallable.rs), singly or as a batched book."""
    _STATE_FIELDS = _MonteCarloEngine._STATE_FIELDS + ("time_steps",)

    def __init__(self, *, time_steps: Optional[int] = None, **kw):
        super().__init__(**kw)
        self._init_time_steps(time_steps)

    def _plan(self, note: AutocallableNote, ctx: PricingContext):
        return plans.autocallable(note, ctx, time_steps=self.time_steps)

    def price_with_statistics(self, note: AutocallableNote, ctx: PricingContext):
        return self._run(ctx, [self._plan(note, ctx)])[0]

    def price_with_greeks(self, note: AutocallableNote, ctx: PricingContext, request, shifts=None):
        """Numerical Greeks with a pinned seed (autocallable.rs:174-283: the reference
        drives the base and bumped notes with shared paths); all scenarios in one
        launch."""
        from .greeks import numerical_greeks
        return numerical_greeks(self, note, ctx, request, shifts)

    def price_many(self, notes: Sequence[AutocallableNote], ctx: PricingContext,
                   path_counts: Optional[Sequence[int]] = None, shared_grid: bool = False):
        """Prices a book of notes in input order (autocallable.rs:119-152).  Unlike the
        reference's price_many, each note may carry its own path count.  With
        `shared_grid`, daily-knock-in notes of one daily grid share their paths and
        coupon families are interpolated (portfolio.rs); see `portfolio`."""
        if shared_grid:
            if path_counts is not None:
                raise InvalidInputError("a shared daily grid takes the engine's path count")
            from . import portfolio
            return portfolio.price_many(self, notes, ctx, True)
        if len(notes) > (1 << 20):
            raise InvalidInputError("contract batch exceeds 1,048,576 instruments")
        return [e.price for e in self.price_many_with_statistics(notes, ctx, path_counts)]

    def price_many_on_shared_grid(self, notes: Sequence[AutocallableNote], ctx: PricingContext):
        """MonteCarloAutocallableEngine::price_many_on_shared_grid (autocallable.rs:
        127-152)."""
        return self.price_many(notes, ctx, shared_grid=True)

    def price_many_with_statistics(self, notes, ctx: PricingContext, path_counts=None):
        return self._run(ctx, [self._plan(n, ctx) for n in notes], path_counts)


class MonteCarloAccumulatorEngine(_MonteCarloEngine, _TimeStepsMixin):
    _STATE_FIELDS = _MonteCarloEngine._STATE_FIELDS + ("time_steps",)

    def __init__(self, *, time_steps: Optional[int] = None, **kw):
        super().__init__(**kw)
        self._init_time_steps(time_steps)

    def _plan(self, option: Accumulator, ctx: PricingContext):
        return plans.accumulator(option, ctx, time_steps=self.time_steps)

    def price_with_statistics(self, option: Accumulator, ctx: PricingContext):
        return self._run(ctx, [self._plan(option, ctx)])[0]

    def price_with_greeks(self, option: Accumulator, ctx: PricingContext, request, shifts=None):
        from .greeks import numerical_greeks
        return numerical_greeks(self, option, ctx, request, shifts)


class MonteCarloDigitalEngine(_MonteCarloEngine):
    def _plan(self, option: DigitalOption, ctx: PricingContext):
        return plans.digital(option, ctx)

    def price_with_statistics(self, option: DigitalOption, ctx: PricingContext):
        return self._run(ctx, [plans.digital(option, ctx)])[0]

    def price_with_greeks(self, option: DigitalOption, ctx: PricingContext, request, shifts=None):
        """Delta and gamma as the means of the likelihood-ratio samples of the price's
        normals (digital.rs:110-150), priced with the price in one book."""
        from .greeks import native_greeks, vanilla_discontinuity
        return native_greeks(self, option, ctx, request, plans.digital, shifts,
                             discontinuity=vanilla_discontinuity(option, ctx))


class MonteCarloBarrierEngine(_MonteCarloEngine):
    """Single barriers (barrier.rs:231-452).  Continuous monitoring: one terminal draw
    per path, weighted by the Brownian-bridge survival or hit probability.  Scheduled
    monitoring: one draw per observation date (plus an unobserved expiry leg); knock-outs
    stop at the hit with their rebate (at expiry or at the hit), and dense knock-ins
    price the vanilla analytically from the hit."""

    def _plan(self, option, ctx: PricingContext):
        return plans.barrier(option, ctx)

    def price_with_statistics(self, option: BarrierOption, ctx: PricingContext):
        return self._run(ctx, [plans.barrier(option, ctx)])[0]

    def price_with_greeks(self, option, ctx: PricingContext, request, shifts=None):
        """Likelihood-ratio delta and gamma from the price's normals (barrier.rs:180-214,
        455-470): continuous barriers add the survival weight's spot derivatives.  They
        are absent when a spot stencil reaches a barrier monitored now; settled knock-ins
        report the vanilla's analytic delta and gamma, settled knock-outs zero."""
        from . import analytic
        from .greeks import NumericalShiftSettings, barrier_discontinuity, native_greeks

        def settled(option, ctx):
            if option.is_knock_in:
                return analytic.european_delta_gamma(option.sign, option.strike, option.expiry, ctx)
            return {"delta": 0.0, "gamma": 0.0}

        def discontinuity(radius):
            return option.expiry == 0.0 or barrier_discontinuity(option, ctx, radius)
        return native_greeks(self, option, ctx, request, plans.barrier, shifts,
                             discontinuity=discontinuity, resolved_greeks=settled)

    def price_strikes(self, option: BarrierOption, ctx: PricingContext, strikes: Sequence[float]):
        opts = [replace(option, strike=float(k)) for k in strikes]
        return [e.price for e in self._run(ctx, [plans.barrier(o, ctx) for o in opts])]
