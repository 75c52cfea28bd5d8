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
