"""CPU: the LSMC oracle against kiyosi's recorded LSMC prices and its own invariants."""
import json
import math
import os

import pytest

from kiyosi_gb300 import abi

from helpers import bsm, heston_context, lsmc_settings, oracle_lsmc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_lsmc_golden_vectors():
    """kiyosi's recorded BSM American put prices (LSMC, quadratic basis; calibration of
    the 0.19.0 build: 65,536 paths x 50 dates and 131,072 paths x 25/50/100 dates) are
    reproduced by the oracle to within 1e-13 relative -- several bit for bit."""
    data = json.load(open(os.path.join(GOLDEN, "american_calibration.json")))
    ctx = bsm()
    rows = [r for r in data["samples"] if r["path_count"] == 65536][:16]
    rows += [r for r in data["samples"] if r["path_count"] == 131072][::8]
    exact = 0
    for row in rows:
        s = lsmc_settings(row["path_count"], row["step_count"], row["seed"], abi.BASIS_QUADRATIC)
        out = oracle_lsmc(ctx, 100.0, -1.0, 1.0, s)
        assert abs(out.price - row["price"]) / row["price"] < 1e-13, (row, out.price)
        exact += out.price == row["price"]
    assert exact > 0


def test_lsmc_known_answer_and_lower_bound():
    """In-sample LSMC is biased high, the out-of-sample policy low; both bracket the FD
    reference 6.660684545893456 (benchmarks/quantlib/references/american_monte_carlo.json)
    within a few standard errors."""
    known = json.load(open(os.path.join(GOLDEN, "known_answers.json")))["values"]
    ref = known["mc-american-put"]["value"]
    s = lsmc_settings(1 << 17, 50, 1009, abi.BASIS_QUADRATIC)
    out = oracle_lsmc(bsm(), 100.0, -1.0, 1.0, s, fresh_seed=4242)
    assert abs(out.price - ref) < 0.15
    assert out.out_of_sample < out.price + 3 * out.standard_error
    assert abs(out.out_of_sample - ref) < 0.15


def test_heston_poly3_runs_and_is_above_european():
    ctx = heston_context()
    s = lsmc_settings(1 << 13, 10, 7, abi.BASIS_POLY3, substeps=2)
    out = oracle_lsmc(ctx, 100.0, -1.0, 1.0, s)
    assert 5.0 < out.price < 9.0 and out.standard_error > 0
