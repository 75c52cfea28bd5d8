"""American options by least-squares Monte Carlo through kgpu_lsmc_price.

MonteCarloVanillaEngine prices AmericanOption here (american.rs:955-1455 in the
reference): `step_count` exercise intervals, the quadratic basis under BSM, the cubic
(S/K, v) basis or the MLP continuation model under Heston.
"""
import ctypes as C
import math

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


def price_american(engine, option, ctx, fresh_seed=None):
    """MonteCarloEstimate of an American option (the in-sample LSMC price).  With
    `fresh_seed`, the out-of-sample lower bound is returned as well."""
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
