"""CPU checks of the FP64 oracle against kiyosi's own golden vectors and invariants."""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.instruments import EuropeanOption
from oracle import loader

from helpers import bsm, pack, settings

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _golden(name):
    return json.load(open(os.path.join(GOLDEN, name)))


def test_european_golden_vectors():
    """Every per-seed European price kiyosi recorded (0.19.0 calibration, 198 rows:
    32 seeds x 3 path counts x call/put, plus timing seeds) is reproduced by the oracle's
    0.23.0 restatement to within 1e-13 relative.  The two builds evaluate the terminal
    payoff with different (algebraically equal) expressions, so agreement stops at
    rounding; any error in the PCG32 stream, the 256-sample block seeding or the
    block-ordered Welford merge would show at the 1e-2 level."""
    data = _golden("european_calibration.json")
    ctx = bsm()
    worst = 0.0
    for row in data["samples"]:
        opt = EuropeanOption("call" if row["id"].endswith("call") else "put", 100.0, 1.0)
        est = loader.price_book(ctx, pack([plans.european(opt, ctx)]),
                                settings(row["path_count"], row["seed"]))[0]
        rel = abs(est.price - row["price"]) / row["price"]
        worst = max(worst, rel)
        assert rel < 1e-13, (row, est.price)
    assert len(data["samples"]) == 198


def test_golden_with_v019_payoff_form(oracle):
    """With the 0.19.0 build's plain terminal payoff max(S_T - K, 0) e^{-rT}, several
    recorded prices are reproduced bit for bit."""
    data = _golden("european_calibration.json")
    exact = 0
    for row in data["samples"][:40]:
        call = row["id"].endswith("call")
        v = oracle.kor_golden_european_v019(row["seed"], row["path_count"], 100.0, 100.0, 0.05,
                                            0.02, 0.2, 1.0, int(call), 0)
        assert abs(v - row["price"]) / row["price"] < 1e-13
        exact += v == row["price"]
    assert exact > 0


def test_known_answer_european():
    """The oracle's price converges to the closed form within 4 standard errors."""
    known = _golden("known_answers.json")["values"]
    ctx = bsm()
    for kind in ("call", "put"):
        est = loader.price_book(ctx, pack([plans.european(EuropeanOption(kind, 100.0, 1.0), ctx)]),
                                settings(1 << 20, 42))[0]
        ref = known[f"mc-european-{kind}"]["value"]
        assert abs(est.price - ref) < 4 * est.standard_error


def test_sin_cos_turns_within_6_ulp(oracle):
    """monte_carlo.rs:1896-1912: sin_cos_turns agrees with sin/cos within 6 eps."""
    s, c = C.c_double(), C.c_double()
    for i in range(4097):
        t = i / 4096.0
        oracle.kor_sin_cos_turns(t, C.byref(s), C.byref(c))
        assert abs(s.value - math.sin(2 * math.pi * t)) <= 6 * 2.220446049250313e-16
        assert abs(c.value - math.cos(2 * math.pi * t)) <= 6 * 2.220446049250313e-16


def test_ndtri_inverts_normal_cdf(oracle):
    from math import erfc, sqrt
    for p in [1e-300, 1e-20, 1e-9, 0.01, 0.1353352832366127, 0.3, 0.5, 0.7, 0.95, 1 - 1e-12]:
        z = oracle.kor_ndtri(p)
        back = 0.5 * erfc(-z / sqrt(2.0))
        assert abs(back - p) <= 1e-12 * max(p, 1e-300) + 1e-15 or abs(back - p) / p < 1e-10


def test_pcg_stream_structure():
    """Words of Pcg32::new(seed, stream) after advance(n) equal the n-th words drawn
    sequentially; normals respect the Box-Muller spare across path boundaries."""
    w = loader.pcg_words(42, 7, 0, 64)
    for first in (1, 5, 31):
        assert np.array_equal(loader.pcg_words(42, 7, first, 16), w[first:first + 16])
    z = loader.pcg_normals(42, 3, 0, 21)
    for first in (1, 2, 7, 13):
        assert np.array_equal(loader.pcg_normals(42, 3, first, 21 - first), z[first:])


def test_sobol_first_dimension_is_van_der_corput_scrambled():
    """Sobol bits are 52-bit; each dimension's points are distinct within 2^k blocks."""
    bits, normals = loader.sobol_points(42, 8, 0, 0, 1024)
    assert np.all(bits < (1 << 52))
    top = bits >> np.uint64(42)
    assert len(set(top.tolist())) == 1024
    assert abs(np.mean(normals)) < 0.01


def test_welford_merge_matches_direct_statistics():
    """Block-merged moments give the ordinary mean and the unbiased standard error."""
    ctx = bsm()
    opt = EuropeanOption("put", 100.0, 1.0)
    est = loader.price_book(ctx, pack([plans.european(opt, ctx)]), settings(4096, 9))[0]
    assert est.uncertainty_status == 0 and est.standard_error > 0
    assert abs(est.standard_error - est.sample_error) < 1e-12 * est.sample_error


def test_uncertainty_statuses():
    ctx = bsm()
    p = [plans.european(EuropeanOption("call", 100.0, 1.0), ctx)]
    assert loader.price_book(ctx, pack(p), settings(1024, 1, sobol=True))[0].uncertainty_status == 1
    assert loader.price_book(ctx, pack(p), settings(1, 1))[0].uncertainty_status == 2
    assert loader.price_book(ctx, pack(p), settings(11, 1, antithetic=True))[0].uncertainty_status == 3
    assert loader.price_book(ctx, pack(p), settings(12, 1, antithetic=True))[0].uncertainty_status == 0


def test_threads_do_not_change_results():
    """Fixed seeds reproduce results across worker counts (monte_carlo.rs:1776)."""
    from helpers import c2_context, snowball_c2
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(steps=126, years=0.5, months=6), ctx)])
    a = loader.price_book(ctx, packed, settings(4096, 3), threads=1)[0]
    b = loader.price_book(ctx, packed, settings(4096, 3), threads=8)[0]
    assert a.price == b.price and a.standard_error == b.standard_error
