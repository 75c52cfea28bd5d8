"""American options by least-squares Monte Carlo through kgpu_lsmc_price.

MonteCarloVanillaEngine prices AmericanOption here (american.rs:955-1455 in the
reference): `step_count` exercise intervals, the quadratic basis under BSM, the cubic
(S/K, v) basis or the MLP continuation model under Heston.
"""
import ctypes as C
import math
from dataclasses import replace

from . import abi
from ._native import context
from .errors import InvalidInputError
from .market import BlackScholesMertonParameters, HestonParameters

_BASIS = {"quadratic": abi.BASIS_QUADRATIC, "poly3": abi.BASIS_POLY3, "mlp": abi.BASIS_MLP,
          "mlp_standalone": abi.BASIS_MLP_STANDALONE}


def lsmc_settings(engine, model, basis=None, substeps=None, fresh_seed=None, seed=None):
    heston = isinstance(model, HestonParameters)
    if basis is None:
        basis = getattr(engine, "basis", None) or ("poly3" if heston else "quadratic")
    if basis not in _BASIS:
        raise InvalidInputError(f"unknown LSMC basis {basis!r}")
    s = abi.LsmcSettings()
    s.path_count = engine.path_count
    s.exercise_dates = engine.step_count
    s.substeps = substeps or getattr(engine, "substeps", 5) if heston else 1
    s.basis = _BASIS[basis]
    s.sampling = abi.SAMPLING_PSEUDO_RANDOM
    s.precision = abi.PRECISION_FP64 if engine.precision == "fp64" else abi.PRECISION_FP32
    s.mlp_epochs = getattr(engine, "mlp_epochs", 5)
    s.mlp_batch = getattr(engine, "mlp_batch", 8192)
    s.mlp_hidden = 64
    s.mlp_learning_rate = getattr(engine, "mlp_learning_rate", 1e-3)
    s.seed = seed if seed is not None else engine.seed
    s.mlp_seed = getattr(engine, "mlp_seed", 0) or 0
    return s


def _no_early_exercise(option, model) -> bool:
    """A call under BSM with no dividend yield and a nonnegative rate is never exercised
    early: its American price is the European one (american.rs:1047-1070)."""
    return (option.sign > 0.0 and isinstance(model, BlackScholesMertonParameters)
            and model.dividend <= 0.0 and model.rate >= 0.0)


def _european_shortcut(engine, option, ctx, seed):
    """The American price of a call that is never exercised early: the engine's European
    price of the same terms with the same seed, floored at the immediate payoff."""
    from .instruments import EuropeanOption
    est = engine.replace(seed=seed).price_with_statistics(EuropeanOption(option.option_type, option.strike, option.expiry), ctx)
    immediate = max(option.sign * (ctx.spot - option.strike), 0.0)
    return replace(est, price=max(immediate, est.price))


def price_american(engine, option, ctx, fresh_seed=None, shortcut=True):
    """MonteCarloEstimate of an American option (the in-sample LSMC price).  With
    `fresh_seed`, the out-of-sample lower bound is returned as well.  `shortcut` prices
    calls that are never exercised early as European options, as the reference's
    scalar price does; the rate Greeks of a call whose stencil crosses that boundary
    keep the exercise-grid estimator on both sides (american.rs:1606-1656)."""
    from .pricing import MonteCarloEstimate, _resolve_seed
    if engine.sampling != "pseudo_random":
        raise InvalidInputError("GPU LSMC samples pseudo-random paths")
    if engine.step_count < 2:
        raise InvalidInputError("American Monte Carlo requires at least two exercise intervals")
    model = ctx.model
    if not isinstance(model, (BlackScholesMertonParameters, HestonParameters)):
        raise InvalidInputError("American Monte Carlo requires BSM or Heston parameters")
    if option.expiry == 0.0:
        return MonteCarloEstimate(max(option.sign * (ctx.spot - option.strike), 0.0), None,
                                  "insufficient_observations", None)
    seed = _resolve_seed(engine.seed)
    if shortcut and fresh_seed is None and _no_early_exercise(option, model):
        return _european_shortcut(engine, option, ctx, seed)
    s = lsmc_settings(engine, model, seed=seed)
    native = context(engine.device)
    out = abi.LsmcResult()
    km = ctx.kgpu_model()
    fresh = seed if fresh_seed is None else int(fresh_seed)
    native.check(native.lib.kgpu_lsmc_price(native.handle, C.byref(km), option.strike,
                                            option.sign, option.expiry, C.byref(s), fresh,
                                            C.byref(out)))
    est = MonteCarloEstimate(out.price, out.standard_error if out.standard_error > 0 else None,
                             "available" if out.standard_error > 0 else "zero_observed_variance",
                             seed, out.standard_error,
                             float(engine.path_count) * engine.step_count,
                             float(engine.path_count) * engine.step_count)
    if fresh_seed is not None:
        return est, (out.out_of_sample, out.out_of_sample_error)
    return est


def price_american_out_of_sample(engine, option, ctx, fresh_seed):
    """price_american_out_of_sample (american.rs:574-637): the LSMC policy fitted on the
    engine's paths, applied forward to fresh paths drawn with `fresh_seed`."""
    est, (lower, lower_se) = price_american(engine, option, ctx, fresh_seed=fresh_seed)
    return lower, lower_se


# Default spot bump of the American Greeks: 8% of spot (american.rs:555-557).
AMERICAN_SPOT_SHIFT = 0.08


def price_american_scenarios(engine, option, contexts, seed, shortcut=True):
    """Prices of one American option in BSM `contexts` with one seed: the LSMC
    scenarios go through kgpu_lsmc_price_scenarios, 16 per call, sharing the paths
    (each equals its scalar kgpu_lsmc_price bit for bit); calls that are never exercised
    early are priced as European options when `shortcut` is set."""
    out = [None] * len(contexts)
    lsmc = []
    for i, c in enumerate(contexts):
        if shortcut and _no_early_exercise(option, c.model):
            out[i] = _european_shortcut(engine, option, c, seed).price
        else:
            lsmc.append(i)
    if lsmc:
        s = lsmc_settings(engine, contexts[lsmc[0]].model, seed=seed)
        native = context(engine.device)
        for first in range(0, len(lsmc), 16):
            chunk = lsmc[first:first + 16]
            models = (abi.Model * len(chunk))(*[contexts[i].kgpu_model() for i in chunk])
            results = (abi.LsmcResult * len(chunk))()
            native.check(native.lib.kgpu_lsmc_price_scenarios(
                native.handle, models, len(chunk), option.strike, option.sign, option.expiry, C.byref(s),
                seed, results))
            for i, r in zip(chunk, results):
                out[i] = r.price
    return out


def american_greeks(engine, option, ctx, request, shifts=None):
    """Numerical Greeks of an American option under BSM (price_with_greeks_with_settings,
    american.rs:1487-1687): the reference's stencils and formulas with its 8%-of-spot
    default spot bump, every bumped context priced on the same seed and paths in
    batched LSMC scenario calls (greek_prices / american_spots, american.rs:820-946).
    For a call, rho and dividend rho whose rate stencil crosses the no-early-exercise
    boundary use the exercise-grid estimator on both sides (american.rs:1606-1656).
    Theta, charm and color price the option valued at the time stencil's ends (its
    expiry moved; greeks.time_stencil), each instant's scenarios in one batched call."""
    from . import greeks as G
    from .errors import ComputationFailureError, UnsupportedOperationError
    from .pricing import _resolve_seed
    request = G._check_request(request)
    shifts = shifts or G.NumericalShiftSettings()
    shifts.validate()
    model = ctx.model
    if not isinstance(model, BlackScholesMertonParameters):
        raise UnsupportedOperationError("numerical Greeks need Black-Scholes-Merton parameters")
    if option.expiry > 0.0 and shifts.spot_shift is None:
        shifts = G.NumericalShiftSettings(AMERICAN_SPOT_SHIFT * ctx.spot, shifts.volatility_shift,
                                          shifts.rate_shift, shifts.time_shift)
    seed = _resolve_seed(engine.seed)
    discontinuity = G.vanilla_discontinuity(option, ctx)
    base = (ctx.spot, model.volatility, model.rate, model.dividend)
    needed = [base]
    rule = G.time_rule(option)
    stencil = None
    if option.expiry > 0.0 and any(g in request for g in G.TIME_GREEKS):
        stencil = G.time_stencil(rule, option.expiry, shifts)

    def record(key):
        if key not in needed:
            needed.append(key)
        return 0.0

    G._stencils(ctx, option.expiry, request, shifts, discontinuity, record, 0.0, stencil, True)
    prices = [None] * len(needed)
    instants = {}
    for i, k in enumerate(needed):
        instants.setdefault(0.0 if len(k) == 4 else k[4], []).append(i)
    for shift, members in instants.items():
        valued = option if shift == 0.0 else rule.valued_at(shift)
        if valued.expiry == 0.0:
            values = [max(valued.sign * (needed[i][0] - valued.strike), 0.0) for i in members]
        else:
            values = price_american_scenarios(engine, valued, [G.scenario_context(needed[i]) for i in members], seed)
        for i, v in zip(members, values):
            prices[i] = v
    table = dict(zip(needed, prices))
    result = G._stencils(ctx, option.expiry, request, shifts, discontinuity, table.__getitem__, table[base],
                         stencil, True)
    if option.expiry > 0.0 and option.sign > 0.0:
        spot, vol, rate, dividend = base
        for greek, value, can_switch in (("rho", rate, dividend <= 0.0), ("dividend_rho", dividend, rate >= 0.0)):
            if greek not in request or not can_switch:
                continue
            h = G.symmetric_shift(value, shifts.rate_shift)
            if not (h > 0.0 and math.isfinite(2.0 * h)):
                continue
            lo, hi = value - h, value + h
            crosses = (lo < 0.0 <= hi) if greek == "rho" else (lo <= 0.0 < hi)
            if not crosses:
                continue
            keys = ([(spot, vol, hi, dividend), (spot, vol, lo, dividend)] if greek == "rho"
                    else [(spot, vol, rate, hi), (spot, vol, rate, lo)])
            up, down = price_american_scenarios(engine, option, [G.scenario_context(k) for k in keys], seed,
                                                shortcut=False)
            result.greeks[greek] = (up - down) / (2.0 * h)
            result.status.pop(greek, None)
    for g, value in result.greeks.items():
        if not math.isfinite(value):
            raise ComputationFailureError(f"non-finite {g}")
    result.seed = seed
    return result
