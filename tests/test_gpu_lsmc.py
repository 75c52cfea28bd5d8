"""GPU least-squares Monte Carlo against the FP64 oracle on identical random numbers."""
import json
import os

import pytest

from kiyosi_gb300 import abi
from kiyosi_gb300.instruments import AmericanOption
from kiyosi_gb300.pricing import MonteCarloVanillaEngine

from helpers import bsm, gpu_lsmc, heston_context, lsmc_settings, oracle_lsmc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_bsm_lsmc_golden_on_gpu(native):
    """FP64 LSMC on the GPU reproduces kiyosi's recorded American put prices.  The normal
    equations are summed in a different order than the CPU blocks, so agreement is to
    1e-9 relative rather than bit for bit."""
    data = json.load(open(os.path.join(GOLDEN, "american_calibration.json")))
    ctx = bsm()
    for row in [r for r in data["samples"] if r["path_count"] == 65536][:6]:
        s = lsmc_settings(row["path_count"], row["step_count"], row["seed"], abi.BASIS_QUADRATIC)
        out = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s)
        assert abs(out.price - row["price"]) / row["price"] < 1e-9, (row, out.price)


@pytest.mark.parametrize("heston", [False, True])
def test_lsmc_fp32_and_fp64_match_oracle(native, heston):
    ctx = heston_context() if heston else bsm()
    basis = abi.BASIS_POLY3 if heston else abi.BASIS_QUADRATIC
    substeps = 3 if heston else 1
    s64 = lsmc_settings(1 << 15, 16, 11, basis, "fp64", substeps)
    ref = oracle_lsmc(ctx, 100.0, -1.0, 1.0, s64, fresh_seed=99)
    got = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s64, fresh_seed=99)
    assert abs(got.price - ref.price) <= 1e-8 * ref.price
    assert abs(got.out_of_sample - ref.out_of_sample) <= 1e-8 * ref.out_of_sample
    s32 = lsmc_settings(1 << 15, 16, 11, basis, "fp32", substeps)
    got32 = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, s32, fresh_seed=99)
    assert abs(got32.price - ref.price) <= 0.5 * ref.standard_error
    assert abs(got32.out_of_sample - ref.out_of_sample) <= 0.5 * ref.out_of_sample_error
    # In-sample LSMC is biased high, the fresh-path policy low.
    assert got.out_of_sample <= got.price + 3 * got.standard_error


def test_engine_prices_american_options():
    engine = MonteCarloVanillaEngine(path_count=1 << 16, step_count=50, seed=1009)
    est = engine.price_with_statistics(AmericanOption("put", 100.0, 1.0), bsm())
    assert abs(est.price - 6.6037595608588875) < 1e-9
    lower, lower_se = engine.price_american_out_of_sample(AmericanOption("put", 100.0, 1.0), bsm(),
                                                          fresh_seed=77)
    assert lower < est.price + 3 * est.standard_error


def test_graph_replay_and_update_give_the_same_prices(native):
    """The polynomial LSMC sequence is a CUDA graph: replaying it for an unchanged
    problem, updating it for a changed seed and going back all reproduce direct results."""
    ctx = heston_context()
    a = lsmc_settings(1 << 14, 8, 42, abi.BASIS_POLY3, precision="fp32", substeps=2)
    b = lsmc_settings(1 << 14, 8, 77, abi.BASIS_POLY3, precision="fp32", substeps=2)
    first = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, a, fresh_seed=5)
    again = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, a, fresh_seed=5)
    other = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, b, fresh_seed=5)
    back = gpu_lsmc(native, ctx, 100.0, -1.0, 1.0, a, fresh_seed=5)
    assert first.price == again.price == back.price
    assert first.out_of_sample == again.out_of_sample == back.out_of_sample
    assert other.price != first.price


def _scenarios():
    from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
    base = bsm()
    m = base.model
    keys = [(100.0, m.volatility, m.rate, m.dividend), (108.0, m.volatility, m.rate, m.dividend),
            (92.0, m.volatility, m.rate, m.dividend), (100.0, m.volatility + 1e-4, m.rate, m.dividend),
            (100.0, m.volatility - 1e-4, m.rate, m.dividend), (100.0, m.volatility, m.rate + 1e-4, m.dividend),
            (100.0, m.volatility, m.rate - 1e-4, m.dividend), (100.0, m.volatility, m.rate, m.dividend + 1e-4),
            (116.0, m.volatility, m.rate, m.dividend)]
    return [PricingContext(BlackScholesMertonParameters(r, q, v), s) for s, v, r, q in keys]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_scenario_batch_equals_scalar_prices(native, precision):
    """kgpu_lsmc_price_scenarios: each bumped BSM scenario, priced on the shared path
    store with its own regression, equals its scalar kgpu_lsmc_price bit for bit (price,
    standard error and the fresh-path lower bound); 9 scenarios, the reference's largest
    group, and a batch of 16 with repeats."""
    import ctypes as C
    ctxs = _scenarios()
    s = lsmc_settings(1 << 14, 20, 11, abi.BASIS_QUADRATIC, precision)
    for group in (ctxs, (ctxs * 2)[:16]):
        models = (abi.Model * len(group))(*[c.kgpu_model() for c in group])
        out = (abi.LsmcResult * len(group))()
        native.check(native.lib.kgpu_lsmc_price_scenarios(native.handle, models, len(group), 100.0, -1.0, 1.0,
                                                          C.byref(s), 99, out))
        for c, got in zip(group, out):
            ref = gpu_lsmc(native, c, 100.0, -1.0, 1.0, s, fresh_seed=99)
            assert got.price == ref.price and got.standard_error == ref.standard_error
            assert got.out_of_sample == ref.out_of_sample
    # The FP64 batch against the oracle, scenario by scenario.
    if precision == "fp64":
        for c, got in zip(ctxs, out):
            ref = oracle_lsmc(c, 100.0, -1.0, 1.0, s, fresh_seed=99)
            assert abs(got.price - ref.price) <= 1e-8 * ref.price


def test_scenario_batch_refusals(native):
    import ctypes as C
    s = lsmc_settings(1 << 10, 8, 1, abi.BASIS_QUADRATIC)
    models = (abi.Model * 17)(*[bsm().kgpu_model()] * 17)
    out = (abi.LsmcResult * 17)()
    for count in (0, 17):
        assert native.lib.kgpu_lsmc_price_scenarios(native.handle, models, count, 100.0, -1.0, 1.0,
                                                    C.byref(s), 1, out) == abi.KGPU_INVALID_INPUT
    heston = (abi.Model * 2)(bsm().kgpu_model(), heston_context().kgpu_model())
    assert native.lib.kgpu_lsmc_price_scenarios(native.handle, heston, 2, 100.0, -1.0, 1.0,
                                                C.byref(s), 1, out) != abi.KGPU_OK


def test_american_greeks_equal_scalar_bumped_prices():
    """The American put's Greeks from the batched scenarios equal the reference's
    difference formulas applied to scalar prices of the bumped contexts on the pinned
    seed (8%-of-spot default spot bump, 1e-4 volatility and rate bumps)."""
    from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
    engine = MonteCarloVanillaEngine(path_count=1 << 15, step_count=25, seed=1009)
    opt = AmericanOption("put", 100.0, 1.0)
    ctx = bsm()
    m = ctx.model
    res = engine.price_with_greeks(opt, ctx, ["delta", "gamma", "vega", "volga", "vanna", "rho", "dividend_rho",
                                              "theta"])
    from kiyosi_gb300.greeks import symmetric_shift

    def p(spot=100.0, vol=m.volatility, rate=m.rate, div=m.dividend):
        return engine.price(opt, PricingContext(BlackScholesMertonParameters(rate, div, vol), spot))
    p0 = p()
    h, v = symmetric_shift(100.0, 8.0), symmetric_shift(m.volatility, 1e-4)
    r, q = symmetric_shift(m.rate, 1e-4), symmetric_shift(m.dividend, 1e-4)
    up, down = p(spot=100.0 + h), p(spot=100.0 - h)
    assert res.price == p0
    assert res.greeks["delta"] == (up - down) / h / 2.0
    assert res.greeks["gamma"] == ((up - p0) - (p0 - down)) / h / h
    vu, vd = p(vol=m.volatility + v), p(vol=m.volatility - v)
    assert res.greeks["vega"] == (vu - vd) / (2.0 * v)
    assert res.greeks["volga"] == ((vu - p0) - (p0 - vd)) / v / v
    hi = ((p(spot=100.0 + h, vol=m.volatility + v) - p(spot=100.0 - h, vol=m.volatility + v)) / h / 2.0)
    lo = ((p(spot=100.0 + h, vol=m.volatility - v) - p(spot=100.0 - h, vol=m.volatility - v)) / h / 2.0)
    assert res.greeks["vanna"] == (hi - lo) / (2.0 * v)
    assert res.greeks["rho"] == (p(rate=m.rate + r) - p(rate=m.rate + -r)) / (2.0 * r)
    assert res.greeks["dividend_rho"] == (p(div=m.dividend + q) - p(div=m.dividend + -q)) / (2.0 * q)
    # A put's delta lies in [-1, 0], its gamma and vega are positive, its rho negative.
    assert -1.0 < res.greeks["delta"] < 0.0 and res.greeks["gamma"] > 0.0
    assert res.greeks["vega"] > 0.0 and res.greeks["rho"] < 0.0
    # theta: the option valued a day later and a day earlier (its expiry moved), each
    # priced on the pinned seed; a put loses value with time
    from kiyosi_gb300.greeks import YEAR_MICROS
    day = 86_400_000_000 / YEAR_MICROS
    later = engine.price(AmericanOption("put", 100.0, 1.0 - day), ctx)
    earlier = engine.price(AmericanOption("put", 100.0, 1.0 - -day), ctx)
    assert res.greeks["theta"] == (later - earlier) / (2 * 86_400_000_000 / YEAR_MICROS)
    assert res.greeks["theta"] < 0.0


def test_call_without_early_exercise_is_the_european_price():
    """A BSM call with no dividend yield and a nonnegative rate is priced as the
    European option on the same seed (american.rs:1047-1070)."""
    from kiyosi_gb300.instruments import EuropeanOption
    engine = MonteCarloVanillaEngine(path_count=1 << 15, step_count=25, seed=7)
    ctx = bsm()
    if ctx.model.dividend > 0.0:
        from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
        ctx = PricingContext(BlackScholesMertonParameters(ctx.model.rate, 0.0, ctx.model.volatility), ctx.spot)
    am = engine.price(AmericanOption("call", 100.0, 1.0), ctx)
    eu = engine.price(EuropeanOption("call", 100.0, 1.0), ctx)
    assert am == eu
