"""Shared builders for the parity tests: the benchmark workloads at test sizes and the
GPU / oracle pricing calls on one packed book."""
import ctypes as C
import math

import numpy as np

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.instruments import (Accumulator, AsianOption, AutocallableNote,
                                      EuropeanOption, Observation)
from kiyosi_gb300.market import (BlackScholesMertonParameters, HestonParameters,
                                 LocalVolatilitySurface, PricingContext)

PRECISION = {"fp64": abi.PRECISION_FP64, "fp32": abi.PRECISION_FP32}
SCHEDULE = {"plain": abi.SCHEDULE_PLAIN, "persistent": abi.SCHEDULE_PERSISTENT,
             "shared_grid": abi.SCHEDULE_SHARED_GRID, "lane_refill": abi.SCHEDULE_LANE_REFILL}


def settings(paths, seed, sobol=False, antithetic=False, precision="fp64", schedule="plain",
             tile_paths=0):
    return abi.Settings(path_count=int(paths), sampling=int(sobol), antithetic=int(antithetic),
                        precision=PRECISION[precision], schedule=SCHEDULE[schedule],
                        tile_paths=tile_paths, seed=seed)


def pack(plan_list, path_counts=None):
    b = plans.BookBuilder()
    for p in plan_list:
        b.add(p)
    return b.build(path_counts)


def gpu_price(native, ctx, packed, s, cancel=None):
    n = len(packed.contracts)
    out = (abi.Estimate * n)()
    model = ctx.kgpu_model()
    book = packed.struct()
    flag = None if cancel is None else C.byref(cancel)
    native.check(native.lib.kgpu_price_book(native.handle, C.byref(model), C.byref(book),
                                            C.byref(s), out, flag))
    return list(out)


from kiyosi_gb300.workloads import (bsm, c2_context, heston_asian_c3, heston_context,  # noqa: F401
                                   lv_book, lv_surface, snowball_c2)


def lsmc_settings(paths, dates, seed, basis, precision="fp64", substeps=1):
    return abi.LsmcSettings(path_count=paths, exercise_dates=dates, substeps=substeps,
                            basis=basis, sampling=0, precision=PRECISION[precision],
                            mlp_epochs=5, mlp_batch=8192, mlp_hidden=64, mlp_learning_rate=1e-3,
                            seed=seed, mlp_seed=1)


def oracle_lsmc(ctx, strike, sign, expiry, s, fresh_seed=None, threads=0):
    import ctypes as C
    from oracle import loader
    lib = loader.load()
    out = abi.LsmcResult()
    model = ctx.kgpu_model()
    st = lib.kor_lsmc_price(C.byref(model), strike, sign, expiry, C.byref(s),
                            s.seed if fresh_seed is None else fresh_seed, C.byref(out), threads)
    assert st == 0, st
    return out


def gpu_lsmc(native, ctx, strike, sign, expiry, s, fresh_seed=None):
    import ctypes as C
    out = abi.LsmcResult()
    model = ctx.kgpu_model()
    native.check(native.lib.kgpu_lsmc_price(native.handle, C.byref(model), strike, sign, expiry,
                                            C.byref(s), s.seed if fresh_seed is None else fresh_seed,
                                            C.byref(out)))
    return out


FP64_REL = 1e-12
HALF_SE = 0.5


def compare_gpu_oracle(native, ctx, packed, s, rel=FP64_REL, fp32_also=True):
    """GPU prices of `packed` against the FP64 oracle on the same random numbers: FP64
    (plain schedule) within `rel` relative with equal standard errors and statuses, and
    FP32 (plain and persistent schedules) within half a sample standard error."""
    from oracle import loader
    ref = loader.price_book(ctx, packed, s)
    got = gpu_price(native, ctx, packed, s)
    for r, g in zip(ref, got):
        assert abs(g.price - r.price) <= rel * max(1.0, abs(r.price)), (g.price, r.price)
        assert g.uncertainty_status == r.uncertainty_status
        if r.uncertainty_status == 0:
            assert abs(g.standard_error - r.standard_error) <= 1e-9 * r.standard_error
    if fp32_also:
        for schedule in ("plain", "persistent"):
            if schedule == "persistent" and s.antithetic:
                continue
            s32 = settings(s.path_count, s.seed, sobol=bool(s.sampling), precision="fp32",
                           schedule=schedule, antithetic=bool(s.antithetic))
            got32 = gpu_price(native, ctx, packed, s32)
            for r, g in zip(ref, got32):
                se = max(r.sample_error, 1e-12)
                assert abs(g.price - r.price) <= HALF_SE * se, (schedule, g.price, r.price, se)
    return ref, got
