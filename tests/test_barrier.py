"""Continuously monitored single barriers (barrier.rs:231-452).

CPU: the oracle against kiyosi's recorded per-seed barrier prices (198 rows of the
0.19.0 calibration: down-and-out call at 90, up-and-in put at 120, 65,536 to 262,144
paths) and the host plan's resolution rules.  GPU: the CUDA path against the oracle on
the same random numbers, and the golden rows on the GPU."""
import json
import math
import os

import pytest

from kiyosi_gb300 import abi, analytic, plans
from kiyosi_gb300.errors import InvalidInputError, UnsupportedOperationError
from kiyosi_gb300.instruments import BarrierOption, EuropeanOption
from oracle import loader

from helpers import bsm, gpu_price, pack, settings

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = {"mc-barrier-down-out-call": BarrierOption("call", 100.0, 1.0, barrier=90.0,
                                                   barrier_type="down_and_out"),
         "mc-barrier-up-in-put": BarrierOption("put", 100.0, 1.0, barrier=120.0,
                                               barrier_type="up_and_in")}


def _rows():
    return json.load(open(os.path.join(GOLDEN, "barrier_calibration.json")))["samples"]


def _packs(ctx):
    return {k: pack([plans.barrier(o, ctx)]) for k, o in CASES.items()}


def test_barrier_golden_vectors():
    """Every recorded row within 1e-13 relative; most are bit-for-bit."""
    ctx = bsm()
    packs = _packs(ctx)
    exact = 0
    rows = _rows()
    for row in rows:
        e = loader.price_book(ctx, packs[row["id"]], settings(row["path_count"], row["seed"]))[0]
        assert abs(e.price - row["price"]) <= 1e-13 * row["price"], (row, e.price)
        exact += e.price == row["price"]
    assert exact >= len(rows) // 3


def test_barrier_known_answers_within_sampling_error():
    """The analytic prices (benchmarks/quantlib/references/monte_carlo.json) lie within
    four sample errors of a 2^18-path estimate."""
    known = json.load(open(os.path.join(GOLDEN, "known_answers.json")))["values"]
    ctx = bsm()
    for name, option in CASES.items():
        e = loader.price_book(ctx, pack([plans.barrier(option, ctx)]), settings(1 << 18, 1729))[0]
        assert abs(e.price - known[name]["value"]) < 4.0 * e.sample_error, (name, e.price)


def test_in_out_parity_and_resolution():
    """Knock-in + knock-out = vanilla on the same draws; touched barriers resolve on the
    host (a knock-out pays its rebate, a knock-in is the vanilla option)."""
    ctx = bsm()
    s = settings(1 << 14, 5)
    vanilla = loader.price_book(ctx, pack([plans.european(EuropeanOption("call", 100.0, 1.0), ctx)]), s)[0]
    for up, level in ((False, 85.0), (True, 125.0)):
        kind = "up" if up else "down"
        pair = [plans.barrier(BarrierOption("call", 100.0, 1.0, barrier=level,
                                            barrier_type=f"{kind}_and_{x}"), ctx) for x in ("in", "out")]
        est = loader.price_book(ctx, pack(pair), s)
        assert abs(est[0].price + est[1].price - vanilla.price) < 1e-9 * vanilla.price
    out = plans.barrier(BarrierOption("put", 100.0, 1.0, barrier=95.0, barrier_type="up_and_out",
                                      rebate=2.0), ctx)
    assert isinstance(out, plans.Known) and abs(out.value - 2.0 * math.exp(-0.05)) < 1e-15
    hit = plans.barrier(BarrierOption("put", 100.0, 1.0, barrier=95.0, barrier_type="up_and_out",
                                      rebate=2.0, rebate_timing="at_hit"), ctx)
    assert hit.value == 2.0
    # A touched knock-in is its vanilla option, priced analytically (analytic/barrier.rs:66-76).
    touched_in = plans.barrier(BarrierOption("put", 100.0, 1.0, barrier=100.0,
                                             barrier_type="down_and_in"), ctx)
    assert isinstance(touched_in, plans.Known)
    assert touched_in.value == analytic.european_price(-1.0, 100.0, 1.0, ctx)
    assert abs(touched_in.value - 6.330080627549918) < 1e-12  # Black-Scholes put, scipy
    # Payoffs that need the barrier crossed (analytic/barrier.rs:61-64): a knock-out is
    # worthless without a rebate, the knock-in is the vanilla.
    assert plans.barrier(BarrierOption("call", 130.0, 1.0, barrier=120.0,
                                       barrier_type="up_and_out"), ctx).value == 0.0
    assert plans.barrier(BarrierOption("call", 130.0, 1.0, barrier=120.0, barrier_type="up_and_in"),
                         ctx).value == analytic.european_price(1.0, 130.0, 1.0, ctx)
    at_hit = plans.barrier(BarrierOption("call", 100.0, 1.0, barrier=90.0, barrier_type="down_and_out",
                                         rebate=1.0, rebate_timing="at_hit"), ctx)
    assert at_hit.record["rebate"] == 0.0 and at_hit.addend is not None
    # The delta / gamma copies carry no addend: its Greeks come from its own stencils.
    assert plans.greek_output(at_hit, "delta").addend is None
    with pytest.raises(InvalidInputError):
        BarrierOption("call", 100.0, 1.0, barrier=90.0, barrier_type="sideways")


def test_expiry_rebate_is_paid_when_the_vanilla_leg_is_not():
    ctx = bsm()
    s = settings(1 << 14, 9)
    base = BarrierOption("call", 100.0, 1.0, barrier=90.0, barrier_type="down_and_out")
    with_rebate = BarrierOption("call", 100.0, 1.0, barrier=90.0, barrier_type="down_and_out",
                                rebate=3.0)
    a, b = loader.price_book(ctx, pack([plans.barrier(base, ctx), plans.barrier(with_rebate, ctx)]), s)
    assert 0.0 < b.price - a.price < 3.0 * math.exp(-0.05)


@pytest.mark.gpu
def test_barrier_golden_on_gpu(native):
    ctx = bsm()
    packs = _packs(ctx)
    for row in _rows()[::6]:
        g = gpu_price(native, ctx, packs[row["id"]], settings(row["path_count"], row["seed"]))[0]
        assert abs(g.price - row["price"]) <= 1e-12 * row["price"], (row, g.price)


@pytest.mark.gpu
@pytest.mark.parametrize("sobol", [False, True])
def test_barrier_gpu_parity(native, sobol):
    """FP64 plain within 1e-12 of the oracle; FP32 plain and persistent within 0.5 SE."""
    ctx = bsm(0.03, 0.01, 0.3)
    options = [BarrierOption("call", 100.0, 1.0, barrier=80.0, barrier_type="down_and_out", rebate=1.5),
               BarrierOption("put", 100.0, 0.5, barrier=115.0, barrier_type="up_and_in", rebate=0.5),
               BarrierOption("put", 95.0, 2.0, barrier=70.0, barrier_type="down_and_in"),
               BarrierOption("call", 90.0, 1.0, barrier=140.0, barrier_type="up_and_out")]
    packed = pack([plans.barrier(o, ctx) for o in options])
    s = settings(1 << 14, 21, sobol=sobol)
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= 1e-12 * max(1.0, abs(r.price)), (g.price, r.price)
    for schedule in ("plain", "persistent"):
        got32 = gpu_price(native, ctx, packed, settings(1 << 14, 21, sobol=sobol, precision="fp32",
                                                        schedule=schedule))
        for r, g in zip(ref, got32):
            assert abs(g.price - r.price) <= 0.5 * max(r.sample_error, 1e-12), (schedule, g.price, r.price)


def _reiner_rubinstein_out_call(s, k, h, t, r, q, v, rebate, up):
    """Textbook closed form of a continuously monitored knock-out call with a rebate
    paid at the hit (Reiner and Rubinstein 1991): an independent check."""
    from math import exp, log, sqrt
    n = lambda x: 0.5 * math.erfc(-x / sqrt(2.0))  # noqa: E731
    b = r - q
    sq = v * sqrt(t)
    mu = (b - 0.5 * v * v) / (v * v)
    lam = sqrt(mu * mu + 2.0 * r / (v * v))
    eta = -1.0 if up else 1.0
    x1 = log(s / k) / sq + (1 + mu) * sq
    x2 = log(s / h) / sq + (1 + mu) * sq
    y1 = log(h * h / (s * k)) / sq + (1 + mu) * sq
    y2 = log(h / s) / sq + (1 + mu) * sq
    z = log(h / s) / sq + lam * sq
    carry = s * exp((b - r) * t)
    cash = k * exp(-r * t)
    a_ = carry * n(x1) - cash * n(x1 - sq)
    b_ = carry * n(x2) - cash * n(x2 - sq)
    c_ = carry * (h / s) ** (2 * (mu + 1)) * n(eta * y1) - cash * (h / s) ** (2 * mu) * n(eta * y1 - eta * sq)
    d_ = carry * (h / s) ** (2 * (mu + 1)) * n(eta * y2) - cash * (h / s) ** (2 * mu) * n(eta * y2 - eta * sq)
    f_ = rebate * ((h / s) ** (mu + lam) * n(eta * z) + (h / s) ** (mu - lam) * n(eta * z - 2 * eta * lam * sq))
    if not up:
        return (a_ - c_ if k > h else b_ - d_) + f_
    return f_ if k > h else a_ - b_ + c_ - d_ + f_


@pytest.mark.parametrize("up,level", [(True, 120.0), (False, 80.0)])
@pytest.mark.parametrize("rate", [-0.02, 0.04])
def test_continuous_at_hit_rebate_matches_closed_form(up, level, rate):
    """barrier_monte_carlo.rs:422-467: rebate 10 at the hit, Sobol 65,536 paths, seed 17,
    within 0.015 of the analytic price (here the textbook closed form; the analytic
    rebate term itself agrees to 1e-10)."""
    ctx = bsm(rate, 0.01, 0.2)
    kind = "up_and_out" if up else "down_and_out"
    option = BarrierOption("call", 100.0, 1.0, barrier=level, barrier_type=kind, rebate=10.0,
                           rebate_timing="at_hit")
    plan = plans.barrier(option, ctx)
    e = loader.price_book(ctx, pack([plan]), settings(65536, 17, sobol=True))[0]
    price = e.price + plan.addend(ctx)
    expected = _reiner_rubinstein_out_call(100.0, 100.0, level, 1.0, rate, 0.01, 0.2, 10.0, up)
    assert abs(price - expected) < 0.015, (price, expected)
    rebate_only = _reiner_rubinstein_out_call(100.0, 1e9 if up else 1e-9, level, 1.0, rate, 0.01, 0.2,
                                              10.0, up) if up else None
    if up:
        assert abs(plan.addend(ctx) - rebate_only) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("up,level", [(True, 120.0), (False, 80.0)])
def test_at_hit_rebate_engine_greeks(native, up, level):
    """The engine's price, delta and gamma against the closed form's (the reference
    test's budgets: 0.015, 0.006, 0.003)."""
    from kiyosi_gb300.pricing import MonteCarloBarrierEngine
    ctx = bsm(0.04, 0.01, 0.2)
    option = BarrierOption("call", 100.0, 1.0, barrier=level, barrier_type="up_and_out" if up else "down_and_out",
                           rebate=10.0, rebate_timing="at_hit")
    engine = MonteCarloBarrierEngine(path_count=65536, seed=17, sampling="sobol")
    r = engine.price_with_greeks(option, ctx, ("delta", "gamma"))
    f = lambda s: _reiner_rubinstein_out_call(s, 100.0, level, 1.0, 0.04, 0.01, 0.2, 10.0, up)  # noqa: E731
    h = 0.01
    assert abs(r.price - f(100.0)) < 0.015
    assert abs(r.get("delta") - (f(100.0 + h) - f(100.0 - h)) / (2 * h)) < 0.006
    assert abs(r.get("gamma") - (f(100.0 + h) - 2 * f(100.0) + f(100.0 - h)) / (h * h)) < 0.003
