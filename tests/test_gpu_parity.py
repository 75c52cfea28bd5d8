"""GPU pricing against the FP64 oracle on identical random numbers.

FP64 kernels follow the reference's arithmetic (plain schedule, sequential block
Welford): prices agree with the oracle to 1e-12 relative (1e-10 where Heston or local
volatility adds state-dependent transcendental calls).  FP32 kernels start from the
same integer streams: prices agree within 0.5 standard errors."""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.instruments import Accumulator, DigitalOption, EuropeanOption
from kiyosi_gb300.market import PricingContext
from oracle import loader

from helpers import (bsm, c2_context, gpu_price, heston_asian_c3, heston_context, lv_book,
                     lv_surface, pack, settings, snowball_c2)

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FP64_REL = 1e-12
HALF_SE = 0.5


def _compare(native, ctx, packed, s, rel=FP64_REL, fp32_also=True, sobol=False):
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= rel * max(1.0, abs(r.price)), (g.price, r.price)
        assert g.uncertainty_status == r.uncertainty_status
        if r.uncertainty_status == 0:
            assert abs(g.standard_error - r.standard_error) <= 1e-9 * r.standard_error
    if fp32_also:
        for schedule in ("plain", "persistent"):
            s32 = settings(s.path_count, s.seed, sobol=bool(s.sampling), precision="fp32",
                           schedule=schedule)
            got32 = gpu_price(native, ctx, packed, s32)
            for r, g in zip(ref, got32):
                se = max(r.sample_error, 1e-12)
                assert abs(g.price - r.price) <= HALF_SE * se, (schedule, g.price, r.price, se)
    return ref, got


def test_european_golden_on_gpu(native):
    """The GPU reproduces kiyosi's recorded per-seed European prices (1e-13 relative)."""
    data = json.load(open(os.path.join(GOLDEN, "european_calibration.json")))
    ctx = bsm()
    packs = {k: pack([plans.european(EuropeanOption(k, 100.0, 1.0), ctx)]) for k in ("call", "put")}
    for row in data["samples"]:
        kind = "call" if row["id"].endswith("call") else "put"
        g = gpu_price(native, ctx, packs[kind], settings(row["path_count"], row["seed"]))[0]
        assert abs(g.price - row["price"]) / row["price"] < 1e-13, row


@pytest.mark.parametrize("paths", [1, 255, 256, 257, 4099])
@pytest.mark.parametrize("antithetic", [False, True])
def test_european_edge_sizes(native, paths, antithetic):
    ctx = bsm()
    packed = pack([plans.european(EuropeanOption("put", 95.0, 0.5), ctx)])
    _compare(native, ctx, packed, settings(paths, 11, antithetic=antithetic), fp32_also=False)


def test_log_euler_vanilla_252_steps(native):
    """European call under BSM with 252 log-Euler steps, 2^16 PCG32 paths, seed 42."""
    ctx = bsm()
    packed = pack([plans.path_vanilla(EuropeanOption("call", 100.0, 1.0), ctx, 252)])
    ref, got = _compare(native, ctx, packed, settings(1 << 16, 42))
    assert abs(ref[0].price - 9.227005508154047) < 4 * ref[0].standard_error


@pytest.mark.parametrize("dims", [3, 7])
def test_odd_dimensions_carry_the_box_muller_spare(native, dims):
    ctx = bsm()
    packed = pack([plans.path_vanilla(EuropeanOption("call", 100.0, 0.25), ctx, dims)])
    _compare(native, ctx, packed, settings(1000, 5))
    _compare(native, ctx, packed, settings(1001, 5, antithetic=True), fp32_also=False)


@pytest.mark.parametrize("sobol", [False, True])
@pytest.mark.parametrize("bridge", [True, False])
def test_snowball(native, sobol, bridge):
    """Snowball autocallable (daily knock-in, monthly knock-out) on the bridge and the
    forward plan, PCG32 and Sobol."""
    ctx = c2_context()
    note = snowball_c2(steps=252, years=1.0, months=12)
    packed = pack([plans.autocallable(note, ctx, allow_bridge=bridge)])
    assert bool(packed.contracts[0]["flags"] & abi.C_BRIDGE) == bridge
    _compare(native, ctx, packed, settings(1 << 14, 42, sobol=sobol))


def test_heston_asian(native):
    ctx = heston_context()
    packed = pack([plans.asian(heston_asian_c3(126), ctx, 126)])
    _compare(native, ctx, packed, settings(1 << 14, 42), rel=1e-10)
    _compare(native, ctx, packed, settings(1 << 13, 42, sobol=True), rel=1e-10, fp32_also=False)


def test_local_vol_book(native):
    notes, paths = lv_book(12, min_log2=9, max_log2=12, months_range=(3, 9))
    ctx = PricingContext(lv_surface(), 100.0)
    packed = pack([plans.autocallable(n, ctx) for n in notes], paths)
    _compare(native, ctx, packed, settings(256, 7), rel=1e-10)


def test_local_vol_book_every_contract(native):
    """The benchmark's whole 4096-note local-volatility book (every maturity, level and
    coupon it draws) with each note's paths capped at 2^10: GPU FP64 on both schedules
    within 1e-10 of the oracle, FP32 persistent within half a standard error, all on the
    same random numbers."""
    notes, paths = lv_book(4096)
    ctx = PricingContext(lv_surface(), 100.0)
    packed = pack([plans.autocallable(n, ctx) for n in notes], [min(p, 1 << 10) for p in paths])
    ref = loader.price_book(ctx, packed, settings(1 << 10, 7))
    for schedule in ("plain", "persistent"):
        got = gpu_price(native, ctx, packed, settings(1 << 10, 7, schedule=schedule))
        worst = max(abs(g.price - r.price) / max(1.0, abs(r.price)) for g, r in zip(got, ref))
        assert worst <= 1e-10, (schedule, worst)
    got32 = gpu_price(native, ctx, packed, settings(1 << 10, 7, precision="fp32", schedule="persistent"))
    worst = max(abs(g.price - r.price) / max(r.sample_error, 1e-12) for g, r in zip(got32, ref))
    assert worst <= HALF_SE, worst


def test_accumulator_and_digital(native):
    ctx = bsm(0.03, 0.01, 0.3)
    dt = 1.0 / 252
    acc = Accumulator("call", 95.0, 105.0, 0.5, [dt * (i + 1) for i in range(126)],
                      [dt * 5 * (i + 1) for i in range(25)], daily_quantity=1.0, acceleration=2.0)
    dig = DigitalOption("put", 100.0, 1.0, payout=10.0)
    asset = DigitalOption("call", 105.0, 1.0)
    packed = pack([plans.accumulator(acc, ctx), plans.digital(dig, ctx), plans.digital(asset, ctx)])
    _compare(native, ctx, packed, settings(1 << 13, 3))


def test_persistent_is_deterministic(native):
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(steps=252, years=1.0, months=12), ctx)])
    s = settings(1 << 14, 42, sobol=True, precision="fp32", schedule="persistent")
    a = gpu_price(native, ctx, packed, s)[0]
    b = gpu_price(native, ctx, packed, s)[0]
    assert a.price == b.price and a.executed_steps == b.executed_steps


def test_cancel_flag_interrupts(native):
    ctx = bsm()
    packed = pack([plans.european(EuropeanOption("call", 100.0, 1.0), ctx)])
    flag = C.c_int32(1)
    with pytest.raises(InterruptedError):
        gpu_price(native, ctx, packed, settings(1 << 12, 1), cancel=flag)
    with pytest.raises(InterruptedError):
        gpu_price(native, ctx, packed, settings(1 << 12, 1, precision="fp32",
                                                schedule="persistent"), cancel=flag)


@pytest.mark.parametrize("workload", ["heston_asian", "snowball"])
def test_cancel_during_a_pricing(native, workload):
    """Cancellation while the kernel runs (cancellation.rs:33-100): a host thread sets
    the caller's word about a quarter into a long FP32 pricing -- the Heston Asian
    option at 2^22 paths on the lane-refill kernel, which reads the word at every work
    item, or the snowball at 2^24 Sobol paths on the phase-major kernel, which reads it
    at every interval step.  The call raises InterruptedError and returns no estimate;
    the next call on the same context prices normally."""
    import threading
    import time
    if workload == "heston_asian":
        ctx = heston_context()
        packed = pack([plans.asian(heston_asian_c3(), ctx)])
        s = settings(1 << 22, 42, precision="fp32", schedule="persistent")
    else:
        ctx = c2_context()
        packed = pack([plans.autocallable(snowball_c2(), ctx)])
        s = settings(1 << 24, 42, sobol=True, precision="fp32", schedule="persistent")
    reference = gpu_price(native, ctx, packed, s)[0]
    t0 = time.perf_counter()
    gpu_price(native, ctx, packed, s)
    full = time.perf_counter() - t0
    flag = C.c_int32(0)

    def cancel():
        time.sleep(0.25 * full)
        flag.value = 1
    thread = threading.Thread(target=cancel)
    thread.start()
    t0 = time.perf_counter()
    with pytest.raises(InterruptedError):
        gpu_price(native, ctx, packed, s, cancel=flag)
    thread.join()
    assert time.perf_counter() - t0 < 5.0
    after = gpu_price(native, ctx, packed, s)[0]
    assert after.price == reference.price and after.executed_steps == reference.executed_steps


def test_invalid_inputs_are_rejected(native):
    from kiyosi_gb300.errors import InvalidInputError, UnsupportedOperationError
    ctx = bsm()
    packed = pack([plans.european(EuropeanOption("call", 100.0, 1.0), ctx)])
    with pytest.raises(InvalidInputError):
        gpu_price(native, ctx, packed, settings(1000, 1, sobol=True))
    with pytest.raises(UnsupportedOperationError):
        gpu_price(native, ctx, packed, settings(1000, 1, antithetic=True, schedule="persistent"))
