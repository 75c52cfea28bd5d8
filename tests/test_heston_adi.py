"""CPU: the Heston ADI judge of the LSMC workload against kiyosi's known answers.

kiyosi's own test (crates/kiyosi/tests/heston_finite_difference.rs:434-461) checks its
default 400 x 100 x 400 MCS-ADI grid against independent references -- QuantLib
European prices and a Haentjens/in 't Hout American put -- to 0.001 + 1e-4 x value,
and put-call parity to 2e-4.  The oracle's restatement of that solver is held to the
same bars, so it can stand in as the judge of Monte Carlo prices whose standard errors
are ten times larger.
"""
import ctypes as C
import json
import math
import os

import pytest

from kiyosi_gb300.market import HestonParameters, PricingContext

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _adi(lib, ctx, strike, sign, expiry, american, grid=(400, 100, 400)):
    model = ctx.kgpu_model()
    return lib.kor_heston_adi_american(C.byref(model), strike, sign, expiry, grid[0], grid[1],
                                       grid[2], int(american))


def _context(xi, rate=0.05, dividend=0.02, kappa=1.5):
    return PricingContext(HestonParameters(rate, dividend, 0.04, kappa, 0.04, xi, -0.7), 100.0)


def test_adi_matches_reference_known_answers(oracle):
    known = json.load(open(os.path.join(GOLDEN, "known_answers.json")))["values"]
    european = known["heston-fd-european-call"]["value"]
    american = known["heston-fd-american-put"]["value"]
    ctx = _context(0.3)
    call = _adi(oracle, ctx, 100.0, 1.0, 1.0, False)
    put = _adi(oracle, ctx, 100.0, -1.0, 1.0, False)
    am_put = _adi(oracle, ctx, 100.0, -1.0, 1.0, True)
    am_call = _adi(oracle, ctx, 100.0, 1.0, 1.0, True)
    assert abs(call - european) <= 0.001 + 1e-4 * european, call
    assert abs(call - put - 100.0 * (math.exp(-0.02) - math.exp(-0.05))) < 2e-4
    assert abs(am_put - american) < 0.001 + 1e-4 * american, am_put
    assert am_put >= put - 1e-8 and am_call >= call - 1e-8


def test_adi_high_vol_of_vol_european(oracle):
    """QuantLib's Gatheral/Lobatto price at xi = 0.9 (the same kiyosi test)."""
    reference = 7.783760588260141
    call = _adi(oracle, _context(0.9), 100.0, 1.0, 1.0, False)
    assert abs(call - reference) <= 0.001 + 1e-4 * reference, call


def test_adi_rejects_unusable_inputs(oracle):
    ctx = _context(0.3)
    assert math.isnan(_adi(oracle, ctx, 100.0, -1.0, 1.0, True, grid=(2, 100, 400)))
    assert math.isnan(_adi(oracle, ctx, -1.0, -1.0, 1.0, True))
