"""Throughput benchmark of the GB300 Monte Carlo engine.

Workload (one "step" = one full pricing): a single snowball autocallable under BSM,
S0=100, sigma=0.25, r=0.03, q=0, T=2y, 504 daily steps, 24 monthly knock-out
observations at 103%, daily knock-in at 80%, 15% p.a. coupon, 2^20 Sobol paths, seed 42.
The metric is path-steps/s = paths x grid steps / time.

Arms:
  ours (default)    FP32 persistent lane-refill kernel.  `value` times the kernels with
                    the plan resident in HBM (kgpu_price_book_device, CUDA events on the
                    library's stream); `e2e` times kgpu_price_book from host buffers
                    (plan upload, kernels, estimate download) with the host clock.
                    Also measured: the FP64 plain one-contract-per-launch path on the
                    same random numbers, the oracle (FP64 CPU) price and a timed CPU
                    baseline sample.
  --impl reference  the FP64 CPU oracle (restatement of kiyosi's Rust engine, which
                    cannot be built here) on all host cores, same workload.

Prints one JSON line.
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PATHS = 1 << 20
STEPS = 504
SEED = 42
# The phase-major kernel on this workload, from one ncu capture of a 2^19-path pricing
# (41,683,020 executed path positions): warp instructions issued and DRAM bytes moved
# per launch.  The kernel is neither HBM- nor tensor-bound; its roofline is the op model
# of kiyosi_gb300/roofline_ops.json against the measured pipe rates, with the SM issue
# rate (4 warp-instructions per cycle per SM) beside it.
PHASED_WARP_INST = 140338724
PHASED_POSITIONS = 41683020
PHASED_DRAM_BYTES = 4312576
PHASED_CAPTURE_PATHS = 1 << 19


def snowball():
    from kiyosi_gb300.instruments import AutocallableNote, Observation
    from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext
    ctx = PricingContext(BlackScholesMertonParameters(0.03, 0.0, 0.25), 100.0)
    dt = 2.0 / STEPS
    times = [dt * (i + 1) for i in range(STEPS)]
    obs = [Observation(times[21 * (m + 1) - 1], knock_out_level=103.0, coupon_rate=0.15)
           for m in range(24)]
    note = AutocallableNote(initial_spot=100.0, expiry=times[-1], observations=obs,
                            knock_in_level=80.0, knock_in_times=times, upper_strike=100.0,
                            lower_strike=0.0, maturity_coupon_rate=0.15)
    return ctx, note


def packed_plan():
    from kiyosi_gb300 import plans
    ctx, note = snowball()
    b = plans.BookBuilder()
    b.add(plans.autocallable(note, ctx))
    return ctx, b.build()


TUNING = {"tile_paths": 0, "ctas_per_sm": 0, "refill": 0}


def settings(precision, schedule, paths=PATHS):
    from kiyosi_gb300 import abi
    return abi.Settings(path_count=paths, sampling=abi.SAMPLING_SOBOL, antithetic=0,
                        precision=precision, schedule=schedule, seed=SEED, **TUNING)


class Cuda:
    """Minimal CUDA runtime access for device-resident plans and L2 flushing."""

    def __init__(self):
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        self.rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.rt.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
        self.rt.cudaDeviceSynchronize.argtypes = []
        self.rt.cudaFree.argtypes = [C.c_void_p]
        self.ptrs = []

    def to_device(self, array):
        p = C.c_void_p()
        n = max(int(array.nbytes), 16)
        assert self.rt.cudaMalloc(C.byref(p), n) == 0
        if array.nbytes:
            assert self.rt.cudaMemcpy(p, array.ctypes.data, array.nbytes, 1) == 0
        self.ptrs.append(p)
        return p

    def flush_l2(self, nbytes=512 << 20):
        if not hasattr(self, "scratch"):
            self.scratch = C.c_void_p()
            assert self.rt.cudaMalloc(C.byref(self.scratch), nbytes) == 0
            self.scratch_bytes = nbytes
        self.rt.cudaMemset(self.scratch, 1, self.scratch_bytes)
        self.rt.cudaDeviceSynchronize()


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix=f"kiyosi_clocks{self.device}_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device),
                                          f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
        self.summary()

    def summary(self):
        if getattr(self, "_summary", None) is not None:
            return self._summary
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9 or not f[1].replace(".", "").isdigit():
                    continue
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
                for name, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        except OSError:
            pass
        try:
            os.remove(self.path)
        except OSError:
            pass
        self._summary = {"sm_mhz": statistics.median(sm) if sm else None,
                         "sm_max_mhz": mx or None, "reasons": sorted(reasons),
                         "samples": len(sm)}
        return self._summary


class Ranks:
    """Replicas under torchrun: one process per GPU, each pricing the full workload on
    its own device (the pricing shards by reference block, but no cross-GPU merge is
    built), a host barrier around the timed region and the maximum time over ranks."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.device = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, value):
        if not self.dist:
            return value
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def run_ours(args):
    from kiyosi_gb300 import _native, abi
    from oracle import loader
    ranks = Ranks()
    native = _native.context(ranks.device)
    lib = native.lib
    ctx, packed = packed_plan()
    model = ctx.kgpu_model()
    host_book = packed.struct()
    cuda = Cuda()
    cuda.rt.cudaSetDevice(ranks.device)
    # Device-resident plan for the kernel-only measurement.
    dev = abi.Book()
    dev.contract_count = 1
    dev.contracts = host_book.contracts  # the contract table is read on the host
    dev.step_total = host_book.step_total
    dev.steps = C.cast(cuda.to_device(packed.steps), C.POINTER(abi.Step))
    dev.step_flags = C.cast(cuda.to_device(packed.flags), C.POINTER(C.c_uint8))
    dev.bridge_daily = C.cast(cuda.to_device(packed.daily), C.POINTER(abi.BridgeDaily))
    dev.event_total = host_book.event_total
    dev.interval_total = host_book.interval_total
    dev.events = C.cast(cuda.to_device(packed.events), C.POINTER(abi.Event))
    dev.intervals = C.cast(cuda.to_device(packed.intervals), C.POINTER(abi.BridgeInterval))
    out = (abi.Estimate * 1)()

    def device_call(s):
        native.check(lib.kgpu_price_book_device(native.handle, C.byref(model), C.byref(dev),
                                                C.byref(s), out))
        # Copy: `out` is reused by the next call.
        return (abi.Estimate.from_buffer_copy(out[0]), native.last_kernel_ms, native.last_launches,
                native.last_path_kernel_ms)

    def host_call(s):
        native.check(lib.kgpu_price_book(native.handle, C.byref(model), C.byref(host_book),
                                         C.byref(s), out, None))
        return abi.Estimate.from_buffer_copy(out[0])

    s32 = settings(abi.PRECISION_FP32, abi.SCHEDULE_PERSISTENT)
    s64 = settings(abi.PRECISION_FP64, abi.SCHEDULE_PLAIN)
    shape = None
    if args.autotune and not any(TUNING.values()):
        # The project's autotuner picks the persistent launch shape (outside the timed
        # region; prices do not depend on it).
        from kiyosi_gb300 import autotune
        shape, _ = autotune.tune(native, ctx, packed, s32)
        s32 = autotune.apply(s32, shape)
    for _ in range(args.warmup):
        device_call(s32)
    kernel_ms, path_ms, launches = [], [], 0
    graph_modes = []
    est32 = None
    with Clocks(ranks.device) as clocks:
        ranks.barrier()
        for _ in range(args.steps):
            cuda.flush_l2()
            est32, ms, nl, pk = device_call(s32)
            kernel_ms.append(ms)
            path_ms.append(pk)
            launches += nl
            graph_modes.append(native.last_graph)
        ranks.barrier()
    clock = clocks.summary()
    total_ms = ranks.max(sum(kernel_ms))
    path_steps = est32.path_steps
    value = ranks.world * path_steps * args.steps / (total_ms / 1e3)
    # End to end through the host-buffer C ABI call.
    h2d = (packed.steps.nbytes + packed.flags.nbytes + packed.events.nbytes
           + packed.intervals.nbytes + (packed.daily.nbytes if packed.daily is not None else 0)
           + packed.contracts.nbytes)
    d2h = C.sizeof(abi.Estimate)
    for _ in range(max(1, args.warmup // 2)):
        host_call(s32)
    ranks.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_call(s32)
    e2e_s = ranks.max(time.perf_counter() - t0)
    e2e = ranks.world * path_steps * args.steps / e2e_s
    if ranks.rank != 0:
        ranks.close()
        return
    # FP64 plain one-contract-per-launch path on the same random numbers.
    device_call(s64)
    f64_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        cuda.flush_l2()
        est64, ms, _, _ = device_call(s64)
        f64_ms.append(ms)
    fp64_rate = path_steps / (statistics.median(f64_ms) / 1e3)
    # FP64 CPU oracle at full size (parity) and timed as the CPU baseline, on all host
    # cores and on one.
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = loader.price_book(ctx, packed, s64, threads=threads)[0]
    cpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    loader.price_book(ctx, packed, settings(abi.PRECISION_FP64, abi.SCHEDULE_PLAIN, 1 << 18),
                      threads=1)
    cpu1_rate = (1 << 18) * STEPS / (time.perf_counter() - t0)
    se = ref.sample_error
    executed = est32.executed_steps
    kernel_s = sum(path_ms) / len(path_ms) / 1e3
    roofline = op_roofline(native, executed, kernel_s, clock)
    # The lane-refill kernel on the same book (one pricing, flushed L2), for comparison.
    lanes = settings(abi.PRECISION_FP32, abi.SCHEDULE_LANE_REFILL)
    device_call(lanes)
    cuda.flush_l2()
    lane_est, _, _, lane_ms = device_call(lanes)
    line = {
        "metric": "path-steps/s (FP32 batched vs FP64 plain) at <=0.5 SE",
        "value": value,
        "unit": "path-steps/s",
        "n_gpus": ranks.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Sobol draws; benchmark contract parameters)",
        "config": {"workload": "snowball autocallable, BSM, 2^20 Sobol paths x 504 daily "
                               "steps, 24 monthly KO 103%, daily KI 80%, 15% p.a. coupon",
                   "paths": PATHS, "grid_steps": STEPS, "sampling": "sobol", "seed": SEED,
                   "precision": "fp32", "schedule": "persistent",
                   "l2": "flushed between timed iterations (512 MiB memset)",
                   "launch_shape": ({"tile_paths": shape.tile_paths, "ctas_per_sm": shape.ctas_per_sm,
                                     "refill": shape.refill, "source": "autotune"} if shape else
                                    {**TUNING, "source": "flags or kernel defaults"})},
        "e2e": {"value": e2e, "unit": "path-steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "launch_sequence": {"cuda_graph_replays": graph_modes.count(2), "captures": graph_modes.count(1),
                            "direct": graph_modes.count(0),
                            "note": "timed calls: the persistent schedule's sequence (plan compile, path "
                                    "kernel, fixed-order reduction) replayed as one CUDA graph"},
        "clocks": clock,
        "roofline": roofline,
        "executed_path_steps_per_s": executed * args.steps / (total_ms / 1e3) * ranks.world,
        "lane_refill": {"path_kernel_ms": lane_ms, "identical_estimate": lane_est.price == est32.price,
                        "note": "the same book on the lane-refill persistent kernel"},
        "fp64_plain": {"value": fp64_rate, "unit": "path-steps/s",
                       "speedup_fp32_persistent": value / fp64_rate,
                       "price": est64.price},
        "parity": {"fp32_price": est32.price, "oracle_fp64_price": ref.price,
                   "sample_se": se, "fp32_error_in_se": abs(est32.price - ref.price) / se,
                   "fp64_gpu_rel_error": abs(est64.price - ref.price) / abs(ref.price)},
        "executed_steps_per_path": executed / PATHS,
        "fp64_executed_steps_per_path": est64.executed_steps / PATHS,
        "cpu_baseline": {"value": path_steps / cpu_s, "unit": "path-steps/s", "cores": threads,
                         "kind": "port", "sample": "full workload (2^20 paths x 504 steps), "
                                                   "one pricing, FP64 oracle",
                         "single_core_value": cpu1_rate,
                         "single_core_sample": "2^18 paths x 504 steps, one thread"},
    }
    if ranks.world > 1:
        line["config"]["parallelism"] = f"replicas x{ranks.world} (one full pricing per GPU)"
    print(json.dumps(line))
    ranks.close()


def op_roofline(native, executed, kernel_s, clock):
    """The path kernel against its op model: algorithmic operations per executed position
    by pipe (kiyosi_gb300/roofline_ops.json) over the pipe rates measured on this device
    (kgpu_pipe_rates); the bound is the pipe that allows the fewest positions per second.
    Beside it, the issued warp instructions against the SM issue rate."""
    from kiyosi_gb300 import abi
    model = json.load(open(os.path.join(ROOT, "kiyosi_gb300", "roofline_ops.json")))
    ops = model["per_executed_position"]
    r = (C.c_double * 5)()
    native.check(native.lib.kgpu_pipe_rates(native.handle, r, 5))
    rates = {"fp32": max(r[0], r[1]), "logic": r[2], "mufu": r[3], "l1_loads": r[4]}
    ceilings = {pipe: rates[pipe] / ops[pipe] for pipe in ops}
    bound = min(ceilings, key=ceilings.get)
    achieved = ops[bound] * executed / kernel_s
    sms = native_sm_count(native)
    issue_peak = 4.0 * sms * (clock["sm_mhz"] or 2070.0) * 1e6
    issued = PHASED_WARP_INST / PHASED_POSITIONS * executed / kernel_s
    return {"bound": bound, "achieved": achieved / 1e9, "peak": rates[bound] / 1e9,
            "unit": "Gop/s", "frac": achieved / rates[bound],
            "traffic": PHASED_DRAM_BYTES * PATHS / PHASED_CAPTURE_PATHS,
            "kernel": "phased_kernel<float, Sobol> (one cooperative launch)",
            "kernel_ms": kernel_s * 1e3,
            "positions_per_s": executed / kernel_s,
            "position_ceiling_per_s": ceilings[bound],
            "ops_per_position": ops, "pipe_rates_gops": {k: v / 1e9 for k, v in rates.items()},
            "issue": {"warp_inst_per_position": PHASED_WARP_INST / PHASED_POSITIONS,
                      "achieved_gwarp_inst_s": issued / 1e9, "peak_gwarp_inst_s": issue_peak / 1e9,
                      "frac": issued / issue_peak},
            "note": "peak = the bound pipe's rate measured by kgpu_pipe_rates in this run; "
                    "traffic = DRAM bytes per launch (ncu, 2^19-path capture scaled by paths)"}


def native_sm_count(native):
    """Multiprocessor count of device 0 (cudaDevAttrMultiProcessorCount)."""
    rt = Cuda().rt
    v = C.c_int(0)
    rt.cudaDeviceGetAttribute(C.byref(v), 16, 0)
    return v.value


def run_kernel_only(args):
    """Device-resident pricings of one arm only, for ncu captures of the kernels."""
    from kiyosi_gb300 import _native, abi
    native = _native.context(0)
    if args.kernel_only == "lv-book":
        # The local-volatility book of `--notes` notes, FP32 persistent.
        _, ctx, packed, paths, sampling = _workload("lv-book", args.notes)
        s = abi.Settings(path_count=paths[0], sampling=sampling, antithetic=0, precision=abi.PRECISION_FP32,
                         schedule=abi.SCHEDULE_PERSISTENT, seed=7)
        model = ctx.kgpu_model()
        book = packed.struct()
        out = (abi.Estimate * len(packed.contracts))()
        for _ in range(args.warmup + args.steps):
            native.check(native.lib.kgpu_price_book(native.handle, C.byref(model), C.byref(book), C.byref(s),
                                                    out, None))
        print(json.dumps({"arm": "lv-book", "notes": args.notes, "path_kernel_ms": native.last_path_kernel_ms,
                          "executed_steps": sum(e.executed_steps for e in out)}))
        return
    if args.kernel_only == "mlp-train-grid":
        # The grid-barrier trainer alone: 40 Adam steps of batch 8192 over 65,536
        # synthetic samples per call.
        rng = np.random.default_rng(5)
        x = rng.normal(size=(65536, 4)).astype(np.float32)
        x[:, 3] = np.abs(x[:, 3]) * 0.1
        p0 = rng.uniform(-0.3, 0.3, abi.MLP_PARAMS).astype(np.float32)
        fp = C.POINTER(C.c_float)
        for _ in range(args.warmup + args.steps):
            q = p0.copy()
            t0 = time.perf_counter()
            native.check(native.lib.kgpu_mlp_train(native.handle, q.ctypes.data_as(fp), x.ctypes.data_as(fp),
                                                   len(x), 8192, 40, 1e-3, abi.TRAINER_GRID))
        print(json.dumps({"arm": "mlp-train-grid", "steps_per_call": 40,
                          "us_per_step_host": (time.perf_counter() - t0) / 40 * 1e6}))
        return
    if args.kernel_only.startswith("lsmc"):
        from kiyosi_gb300 import workloads
        ctx = workloads.heston_context()
        model = ctx.kgpu_model()
        basis = abi.BASIS_MLP if args.kernel_only == "lsmc-mlp" else abi.BASIS_POLY3
        s = abi.LsmcSettings(path_count=args.paths, exercise_dates=args.dates, substeps=5,
                             basis=basis, sampling=0, precision=abi.PRECISION_FP32, mlp_epochs=5,
                             mlp_batch=8192, mlp_hidden=64, mlp_learning_rate=1e-3, seed=42,
                             mlp_seed=7, mlp_samples=args.mlp_samples)
        out = abi.LsmcResult()
        for _ in range(args.warmup + args.steps):
            native.check(native.lib.kgpu_lsmc_price(native.handle, C.byref(model), 100.0, -1.0,
                                                    1.0, C.byref(s), 43, C.byref(out)))
        print(json.dumps({"arm": args.kernel_only, "paths": args.paths, "dates": args.dates,
                          "price": out.price, "out_of_sample": out.out_of_sample,
                          "wall_ms": out.wall_ms, "path_store_ms": out.path_store_ms,
                          "regression_ms": out.regression_ms, "launches": native.last_launches}))
        return
    if args.kernel_only == "shared-grid":
        # the shared-grid book's lanes (native planner) on the path-major FP32 schedule
        from kiyosi_gb300 import portfolio, workloads
        ctx = workloads.c2_context()
        shared = portfolio.SharedPlan(portfolio.note_tables(workloads.shared_grid_book()), ctx.kgpu_model())
        packed = shared.group_packed(0)
        lanes = packed.contracts
        s = abi.Settings(path_count=args.paths, sampling=abi.SAMPLING_PSEUDO_RANDOM, antithetic=0,
                         precision=abi.PRECISION_FP32, schedule=abi.SCHEDULE_SHARED_GRID, seed=42)
        for _ in range(args.warmup + args.steps):
            est, k, pk, _ = _host_pricing(native, ctx, packed, s)
        print(json.dumps({"arm": args.kernel_only, "paths": args.paths, "lanes": len(lanes),
                          "first_price": est[0].price, "kernel_ms": k, "path_kernel_ms": pk}))
        return
    ctx, packed = packed_plan()
    model = ctx.kgpu_model()
    book = packed.struct()
    s = (settings(abi.PRECISION_FP32, abi.SCHEDULE_PERSISTENT, args.paths)
         if args.kernel_only == "fp32" else
         settings(abi.PRECISION_FP32, abi.SCHEDULE_LANE_REFILL, args.paths)
         if args.kernel_only == "fp32-lanes" else
         settings(abi.PRECISION_FP64, abi.SCHEDULE_PLAIN, args.paths))
    out = (abi.Estimate * 1)()
    for _ in range(args.warmup + args.steps):
        native.check(native.lib.kgpu_price_book(native.handle, C.byref(model), C.byref(book),
                                                C.byref(s), out, None))
    print(json.dumps({"arm": args.kernel_only, "paths": args.paths, "price": out[0].price,
                      "executed_steps": out[0].executed_steps, "kernel_ms": native.last_kernel_ms,
                      "path_kernel_ms": native.last_path_kernel_ms}))


def _host_pricing(native, ctx, packed, s):
    """kgpu_price_book from host buffers: estimates, device time of the call's kernels,
    of its path kernels alone, and the host wall time."""
    from kiyosi_gb300 import abi
    n = len(packed.contracts)
    out = (abi.Estimate * n)()
    model = ctx.kgpu_model()
    book = packed.struct()
    t0 = time.perf_counter()
    native.check(native.lib.kgpu_price_book(native.handle, C.byref(model), C.byref(book),
                                            C.byref(s), out, None))
    wall = time.perf_counter() - t0
    return ([abi.Estimate.from_buffer_copy(e) for e in out], native.last_kernel_ms,
            native.last_path_kernel_ms, wall)


def _first(packed, n):
    """The first n contracts of a packed book (the arrays they index stay shared)."""
    return type(packed)(packed.contracts[:n].copy(), packed.steps, packed.flags, packed.events,
                        packed.intervals, packed.daily)


def _workload(name, notes=4096):
    """(description, context, packed book, per-contract paths, sampling) of a named
    benchmark configuration."""
    from kiyosi_gb300 import plans, workloads
    from kiyosi_gb300.market import PricingContext
    b = plans.BookBuilder()
    if name == "european":
        ctx, opt = workloads.european()
        b.add(plans.path_vanilla(opt, ctx, 252))
        return ("European call, BSM, 2^16 PCG32 paths x 252 daily log-Euler steps", ctx,
                b.build(), [1 << 16], 0)
    if name == "heston-asian":
        ctx = workloads.heston_context()
        b.add(plans.asian(workloads.heston_asian_c3(), ctx))
        return ("Heston arithmetic-average Asian call, 2^22 PCG32 paths x 252 full-truncation "
                "Euler steps", ctx, b.build(), [1 << 22], 0)
    if name == "lv-book":
        ctx = PricingContext(workloads.lv_surface(), 100.0)
        notes, paths = workloads.lv_book(notes)
        for n in notes:
            b.add(plans.autocallable(n, ctx))
        return ("book of 4096 snowball/phoenix notes under local volatility (50x20 surface), "
                "3-36 monthly observations, daily steps, 2^14-2^18 paths per note", ctx,
                b.build(paths), paths, 0)
    raise ValueError(name)


def run_workload(args, name):
    """One of the other benchmark configurations: FP32 persistent (one launch for the
    whole book) against the FP64 plain path, with parity in standard errors."""
    from kiyosi_gb300 import _native, abi
    from oracle import loader
    native = _native.context(0)
    desc, ctx, packed, paths, sampling = _workload(name)
    seed = 42 if name != "lv-book" else 7
    s32 = abi.Settings(path_count=paths[0], sampling=sampling, antithetic=0,
                       precision=abi.PRECISION_FP32, schedule=abi.SCHEDULE_PERSISTENT, seed=seed,
                       **TUNING)
    s64 = abi.Settings(path_count=paths[0], sampling=sampling, antithetic=0,
                       precision=abi.PRECISION_FP64, schedule=abi.SCHEDULE_PLAIN, seed=seed)
    for _ in range(args.warmup):
        _host_pricing(native, ctx, packed, s32)
    kernel, path, walls, launches = [], [], [], 0
    with Clocks() as clocks:
        for _ in range(args.steps):
            est32, k, pk, w = _host_pricing(native, ctx, packed, s32)
            kernel.append(k)
            path.append(pk)
            walls.append(w)
            launches += native.last_launches
    path_steps = sum(e.path_steps for e in est32)
    # FP64 plain, one launch per contract (the speed comparator): the whole book, or its
    # first 128 notes for the local-volatility book (one launch per note would take
    # minutes on all 4096).
    fp64_n = min(len(est32), 128)
    _host_pricing(native, ctx, _first(packed, min(fp64_n, 2)), s64)  # loads the FP64 kernels
    est64, k64, _, _ = _host_pricing(native, ctx, _first(packed, fp64_n), s64)
    fp64_path_steps = sum(e.path_steps for e in est64)
    # Parity over every contract at full size: FP32 against FP64 on the same random
    # numbers, the FP64 side on the persistent schedule (one launch for the book).
    s64_all = abi.Settings.from_buffer_copy(s64)
    s64_all.schedule = abi.SCHEDULE_PERSISTENT
    est64_all = _host_pricing(native, ctx, packed, s64_all)[0]
    worst = max(abs(a.price - b.price) / max(b.sample_error, 1e-300) for a, b in zip(est32, est64_all))
    # Against the CPU oracle: every contract, at full size (C1, C3) or with each note's
    # paths capped at 2^12 (the local-volatility book), GPU FP64 and FP32 on the same
    # random numbers as the oracle.
    cap = 1 << 12 if name == "lv-book" else None
    sub = _first(packed, len(est32))
    if cap:
        sub.contracts["path_count"] = np.minimum(np.where(sub.contracts["path_count"] > 0,
                                                          sub.contracts["path_count"], paths[0]), cap)
    s_cpu = abi.Settings.from_buffer_copy(s64)
    if cap:
        s_cpu.path_count = min(paths[0], cap)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    cpu = loader.price_book(ctx, sub, s_cpu, threads=threads)
    cpu_s = time.perf_counter() - t0
    s64_sub = abi.Settings.from_buffer_copy(s_cpu)
    s64_sub.schedule = abi.SCHEDULE_PERSISTENT
    g64 = _host_pricing(native, ctx, sub, s64_sub)[0]
    s32_sub = abi.Settings.from_buffer_copy(s32)
    s32_sub.path_count = s_cpu.path_count
    g32 = _host_pricing(native, ctx, sub, s32_sub)[0]
    oracle_fp64_rel = max(abs(a.price - b.price) / max(abs(b.price), 1.0) for a, b in zip(g64, cpu))
    oracle_fp32_se = max(abs(a.price - b.price) / max(b.sample_error, 1e-300) for a, b in zip(g32, cpu))
    ms = statistics.median(kernel)
    line = {
        "metric": "path-steps/s (FP32 batched vs FP64 plain) at <=0.5 SE",
        "value": path_steps / (ms / 1e3), "unit": "path-steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded draws; benchmark contract parameters)",
        "config": {"workload": desc, "contracts": len(est32), "sampling": "pcg32",
                   "precision": "fp32", "schedule": "persistent",
                   "l2": "inputs and per-path values exceed L2 (no flush)"},
        "e2e": {"value": path_steps / statistics.median(walls), "unit": "path-steps/s",
                "h2d_bytes_per_step": int(packed.steps.nbytes + packed.flags.nbytes
                                          + packed.events.nbytes + packed.contracts.nbytes),
                "d2h_bytes_per_step": int(len(est32) * C.sizeof(abi.Estimate))},
        "gpu_launches": launches, "clocks": clocks.summary(),
        "path_kernel_ms": statistics.median(path),
        "fp64_plain": {"value": fp64_path_steps / (k64 / 1e3), "unit": "path-steps/s",
                       "ms": k64, "contracts": fp64_n,
                       "speedup_fp32_persistent": (path_steps / (ms / 1e3)) / (fp64_path_steps / (k64 / 1e3))},
        "parity": {"contracts": len(est32),
                   "max_fp32_vs_fp64_in_se": worst,
                   "fp64_schedule": "persistent (one launch, every contract, full paths)",
                   "oracle": {"paths": f"each note capped at {cap}" if cap else "full",
                              "max_err_in_se": oracle_fp32_se,
                              "max_fp64_gpu_rel_err": oracle_fp64_rel,
                              "note": "GPU FP32 (persistent) and FP64 against the FP64 CPU oracle "
                                      "on the same random numbers, every contract"}},
        "executed_steps_per_path_step": sum(e.executed_steps for e in est32) / path_steps,
        "executed_path_steps_per_s": sum(e.executed_steps for e in est32) / (ms / 1e3),
        "cpu_baseline": {"value": sum(e.path_steps for e in cpu) / cpu_s,
                         "unit": "path-steps/s", "cores": threads, "kind": "port",
                         "sample": (f"all {len(est32)} contracts at up to {cap} paths" if cap else
                                    "the full workload") + ", FP64 oracle"},
    }
    print(json.dumps(line), flush=True)


def run_shared_grid(args):
    """price_many on a shared daily grid (autocallable/portfolio.rs): a 4096-note book of
    snowball and Phoenix notes on one 504-step daily grid under BSM, 2^16 PCG32 paths.
    The group's lanes go through the path-major schedule: one thread per path walks the
    grid once and settles every lane from its per-date records.  Beside it:
    * the per-lane layout (each lane re-walks the path; FP32 persistent);
    * FP64 parity;
    * the whole engine call from host notes;
    * the reference's multi-lane CPU algorithm (coupon families and threshold strips,
      restated in the FP64 oracle) on a bounded sample of paths."""
    from kiyosi_gb300 import _native, abi, plans, portfolio, workloads
    from kiyosi_gb300.pricing import MonteCarloAutocallableEngine
    from oracle import loader
    native = _native.context(0)
    ctx = workloads.c2_context()
    notes = workloads.shared_grid_book()
    paths, seed = 1 << 16, 42
    # The book's plan: the library's native planner (what the engine call runs), and the
    # Python restatement beside it (the oracle's lanes below).
    t0 = time.perf_counter()
    tables = portfolio.note_tables(notes)
    t1 = time.perf_counter()
    shared = portfolio.SharedPlan(tables, ctx.kgpu_model())
    packed = shared.group_packed(0)
    plan_s = time.perf_counter() - t0
    tables_s = t1 - t0
    assert shared.group_count == 1 and (shared.note_group >= 0).all()
    t0 = time.perf_counter()
    book = portfolio.plan_book(notes, ctx, True)
    lanes = [lane for g in book.groups for lane in g.simulated_lanes()]
    python_book = plans.BookBuilder()
    for p in portfolio.lane_plans(lanes, ctx.spot):
        python_book.add(p)
    python_packed = python_book.build()
    python_plan_s = time.perf_counter() - t0
    assert len(book.groups) == 1 and not book.scalar

    def cfg(precision, schedule):
        return abi.Settings(path_count=paths, sampling=abi.SAMPLING_PSEUDO_RANDOM, antithetic=0,
                            precision=precision, schedule=schedule, seed=seed, **TUNING)

    fast32 = cfg(abi.PRECISION_FP32, abi.SCHEDULE_SHARED_GRID)
    for _ in range(args.warmup):
        _host_pricing(native, ctx, packed, fast32)
    kernel, path, walls, launches = [], [], [], 0
    with Clocks() as clocks:
        for _ in range(args.steps):
            est32, k, pk, w = _host_pricing(native, ctx, packed, fast32)
            kernel.append(k)
            path.append(pk)
            walls.append(w)
            launches += native.last_launches
    ms = statistics.median(kernel)
    est64, k64, _, _ = _host_pricing(native, ctx, packed, cfg(abi.PRECISION_FP64, abi.SCHEDULE_SHARED_GRID))
    # the first 64 lanes on the per-lane FP64 plain schedule
    first = type(packed)(packed.contracts[:64].copy(), packed.steps, packed.flags, packed.events,
                         packed.intervals, packed.daily)
    lanes64, _, _, _ = _host_pricing(native, ctx, first, cfg(abi.PRECISION_FP64, abi.SCHEDULE_PLAIN))
    per_lane = [_host_pricing(native, ctx, packed, cfg(abi.PRECISION_FP32, abi.SCHEDULE_PERSISTENT))[1]
                for _ in range(2)]
    worst_fp64 = max(abs(a.price - b.price) / max(abs(b.price), 1.0) for a, b in zip(est64, lanes64))
    worst_se = max(abs(a.price - b.price) / max(b.sample_error, 1e-300) for a, b in zip(est32, est64))
    # The whole engine call from host notes (planning, staging, launch, results).
    engine = MonteCarloAutocallableEngine(path_count=paths, seed=seed, precision="fp32")
    engine.price_many_on_shared_grid(notes, ctx)
    # The first call on note objects never priced before: it also flattens their terms,
    # which later calls on the same (frozen) notes reuse.
    fresh = workloads.shared_grid_book()
    t0 = time.perf_counter()
    engine.price_many_on_shared_grid(fresh, ctx)
    e2e_first = time.perf_counter() - t0
    e2e = []
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        engine.price_many_on_shared_grid(notes, ctx)
        e2e.append(time.perf_counter() - t0)
    # CPU: the reference's multi-lane loop with its threshold strips, all 2^16 paths.
    order, strips = portfolio.threshold_strips(lanes, ctx.spot)
    cpu_book = plans.BookBuilder()
    for p in portfolio.lane_plans([lanes[i] for i in order], ctx.spot):
        cpu_book.add(p)
    cpu_paths = paths
    threads = os.cpu_count() or 1
    s_cpu = abi.Settings(path_count=cpu_paths, sampling=abi.SAMPLING_PSEUDO_RANDOM, antithetic=0,
                         precision=abi.PRECISION_FP64, schedule=abi.SCHEDULE_PLAIN, seed=seed)
    t0 = time.perf_counter()
    loader.price_shared_group(ctx, cpu_book.build(), s_cpu,
                              [None if st is None else (st[0], st[1]) for st in strips], threads=threads)
    cpu_s = (time.perf_counter() - t0) * (paths / cpu_paths)
    lane_path_steps = sum(e.path_steps for e in est32)
    line = {
        "metric": "notes priced per second (price_many on a shared daily grid)",
        "value": len(notes) / (ms / 1e3), "unit": "notes/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded draws; benchmark contract parameters)",
        "config": {"workload": "book of 4096 snowball/Phoenix notes on one 504-step daily grid, BSM, "
                               "2^16 PCG32 paths, coupon families interpolated",
                   "notes": len(notes), "simulated_lanes": len(lanes), "group_steps": int(packed.contracts["step_count"].max()),
                   "precision": "fp32", "schedule": "shared_grid (path-major)",
                   "l2": "per-path records live in shared memory (no flush)"},
        "e2e": {"value": len(notes) / statistics.median(e2e), "unit": "notes/s",
                "h2d_bytes_per_step": int(packed.steps.nbytes + packed.flags.nbytes + packed.events.nbytes
                                          + packed.contracts.nbytes + packed.intervals.nbytes
                                          + (packed.daily.nbytes if packed.daily is not None else 0)),
                "d2h_bytes_per_step": int(len(lanes) * C.sizeof(abi.Estimate)),
                "includes": "the engine call from host notes: note tables (Python), native planning, "
                            "staging, launch, interpolation, results",
                "first_call_on_new_notes_s": e2e_first},
        "host_planning": {"native_s": plan_s, "note_tables_s": tables_s, "python_planner_s": python_plan_s,
                          "note": "first planning of the book's note objects (their terms flattened)",
                          "step_records": {"native": int(len(packed.steps)), "python": int(len(python_packed.steps))}},
        "gpu_launches": launches, "clocks": clocks.summary(),
        "path_kernel_ms": statistics.median(path),
        "lane_equivalent_path_steps_per_s": lane_path_steps / (ms / 1e3),
        "per_lane_layout": {"ms": statistics.median(per_lane), "schedule": "persistent fp32, each lane re-walks the path",
                            "speedup_path_major": statistics.median(per_lane) / ms},
        "fp64_path_major_ms": k64,
        "parity": {"fp64_path_major_vs_fp64_lanes_max_rel": worst_fp64, "lanes_checked": 64,
                   "fp32_vs_fp64_max_in_se": worst_se},
        "cpu_baseline": {"value": len(notes) / cpu_s, "unit": "notes/s", "cores": threads, "kind": "port",
                         "sample": "the reference's multi-lane path loop with coupon families and threshold "
                                   f"strips (FP64 oracle), {cpu_paths} of {paths} paths"},
    }
    print(json.dumps(line), flush=True)


def lsmc_roofline(poly, us_per_step):
    """The two bounds of the LSMC configuration against the measured peaks of
    MEASURED_PEAKS.json: the polynomial pricing's path-store traffic over HBM (per path
    and date an 8-byte state write and read plus an 8-byte cash read and write:
    2^20 x 50 x 24 B = 1.26 GB) over its whole wall time, and the trainer's tensor work
    (fwd + bwd of every layer, 3 x 2 x (3*64 + 64*64 + 64) = 26,112 FLOP per sample) per
    Adam step of 8,192 samples over its time per step."""
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    bf16 = peaks.get("bf16_tflops_sustained", 1700.0)
    source = "of measured" if peaks else "of fallback"
    store_bytes = poly["paths"] * 50 * 24
    store_gbs = store_bytes / (poly["wall_ms"] * 1e-3) / 1e9
    train_tflops = 26112 * 8192 / (us_per_step * 1e-6) / 1e12
    return {
        "path_store": {"bound": "hbm", "achieved": store_gbs, "peak": hbm, "unit": "GB/s",
                       "frac": store_gbs / hbm, "algorithmic_bytes": store_bytes, "peak_source": source,
                       "note": "poly3 FP32 at 2^20 paths over the whole pricing: 150 dependent launches of "
                               "per-date passes, latency-bound"},
        "trainer": {"bound": "tensor", "achieved": train_tflops, "peak": bf16, "unit": "TFLOP/s",
                    "frac": train_tflops / bf16, "peak_source": source + " (sustained)",
                    "note": "one Adam step is a dependent chain of phases across SMs"},
    }


def run_lsmc(args):
    """American put under Heston, 50 exercise dates x 5 Euler substeps, judged by the
    Heston ADI price.  Two comparisons of the polynomial LSMC (the reference's method)
    with the polynomial plus the fitted network and with the network alone (no
    polynomial): at the configuration's 2^20 paths (network: 5 epochs per date over every
    in-the-money path, batch 8192), and at equal wall time (networks at 2^22 paths
    training on 131,072 samples per date, against the polynomial at the path count whose
    wall time is closest).  Also the trainer's time per Adam step."""
    from kiyosi_gb300 import _native, abi, workloads
    from oracle import loader
    native = _native.context(0)
    ctx = workloads.heston_context()
    model = ctx.kgpu_model()
    t0 = time.perf_counter()
    adi = loader.load().kor_heston_adi_american(C.byref(model), 100.0, -1.0, 1.0, 400, 100, 400, 1)
    adi_s = time.perf_counter() - t0

    def price(basis, log2_paths, samples=0, precision=abi.PRECISION_FP32):
        s = abi.LsmcSettings(path_count=1 << log2_paths, exercise_dates=50, substeps=5, basis=basis,
                             sampling=0, precision=precision, mlp_epochs=5, mlp_batch=8192,
                             mlp_hidden=64, mlp_samples=samples, mlp_learning_rate=1e-3, seed=42,
                             mlp_seed=7)
        out = abi.LsmcResult()
        for _ in range(1 + max(0, args.warmup // 3)):
            native.check(native.lib.kgpu_lsmc_price(native.handle, C.byref(model), 100.0, -1.0,
                                                    1.0, C.byref(s), 43, C.byref(out)))

        def num(x):
            return None if x != x else x
        return {"paths": 1 << log2_paths, "training_samples_per_date": samples or "all",
                "price": out.price, "standard_error": out.standard_error,
                "out_of_sample": out.out_of_sample,
                "out_of_sample_error": out.out_of_sample_error,
                "error_vs_adi": out.price - adi, "out_of_sample_error_vs_adi": out.out_of_sample - adi,
                "wall_ms": out.wall_ms, "path_store_ms": num(out.path_store_ms),
                "regression_ms": num(out.regression_ms)}

    poly = price(abi.BASIS_POLY3, 20)
    poly64 = price(abi.BASIS_POLY3, 20, precision=abi.PRECISION_FP64)
    # The configuration at full size on the FP64 CPU oracle (same random numbers):
    # 2^20 paths x 50 dates x 5 substeps, polynomial basis, fresh-path pass included.
    s_or = abi.LsmcSettings(path_count=1 << 20, exercise_dates=50, substeps=5, basis=abi.BASIS_POLY3,
                            sampling=0, precision=abi.PRECISION_FP64, mlp_epochs=5, mlp_batch=8192,
                            mlp_hidden=64, mlp_samples=0, mlp_learning_rate=1e-3, seed=42, mlp_seed=7)
    oracle = abi.LsmcResult()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    st = loader.load().kor_lsmc_price(C.byref(model), 100.0, -1.0, 1.0, C.byref(s_or), 43,
                                      C.byref(oracle), threads)
    oracle_s = time.perf_counter() - t0
    assert st == 0, st
    oracle_parity = {
        "paths": 1 << 20, "dates": 50, "substeps": 5, "basis": "poly3",
        "oracle_price": oracle.price, "oracle_out_of_sample": oracle.out_of_sample,
        "fp64_gpu_rel_err": abs(poly64["price"] - oracle.price) / oracle.price,
        "fp64_gpu_out_of_sample_rel_err": abs(poly64["out_of_sample"] - oracle.out_of_sample) / oracle.out_of_sample,
        "fp32_err_in_se": abs(poly["price"] - oracle.price) / oracle.standard_error,
        "fp32_out_of_sample_err_in_se": abs(poly["out_of_sample"] - oracle.out_of_sample) / oracle.out_of_sample_error,
        "max_err_in_se": max(abs(poly["price"] - oracle.price) / oracle.standard_error,
                             abs(poly["out_of_sample"] - oracle.out_of_sample) / oracle.out_of_sample_error),
        "oracle_cpu_s": oracle_s, "oracle_threads": threads}
    mlp = price(abi.BASIS_MLP, 20)
    alone = price(abi.BASIS_MLP_STANDALONE, 20)
    mlp_eq = price(abi.BASIS_MLP, 22, samples=131072)
    alone_eq = price(abi.BASIS_MLP_STANDALONE, 22, samples=131072)
    polys = [price(abi.BASIS_POLY3, k) for k in range(21, 27)]
    equal = min(polys, key=lambda r: abs(r["wall_ms"] - mlp_eq["wall_ms"]))
    # Context for the fixed comparison above: other path and sample counts of the
    # network, each beside the polynomial run whose wall time is closest.
    sweep = []
    for log2_paths, samples in ((21, 131072), (22, 262144), (23, 131072)):
        r = price(abi.BASIS_MLP, log2_paths, samples=samples)
        near = min(polys, key=lambda q: abs(q["wall_ms"] - r["wall_ms"]))
        sweep.append({"poly3_plus_network": r, "poly3_nearest_wall": near})
    # The trainer alone: Adam steps of batch 8192 over 65,536 samples, one launch.
    rng = np.random.default_rng(5)
    tsamples = rng.normal(size=(65536, 4)).astype(np.float32)
    tsamples[:, 3] = np.abs(tsamples[:, 3]) * 0.1
    tparams = (rng.uniform(-0.3, 0.3, abi.MLP_PARAMS)).astype(np.float32)
    fp = C.POINTER(C.c_float)
    trainer = {}
    for kind in (abi.TRAINER_CLUSTER, abi.TRAINER_GRID):
        for steps in (8, 1008):
            q = tparams.copy()
            t0 = time.perf_counter()
            native.check(native.lib.kgpu_mlp_train(native.handle, q.ctypes.data_as(fp),
                                                   tsamples.ctypes.data_as(fp), len(tsamples), 8192, steps,
                                                   1e-3, kind))
            trainer[kind, steps] = time.perf_counter() - t0
    us_per_step = {k: (trainer[k, 1008] - trainer[k, 8]) / 1000 * 1e6 for k in (abi.TRAINER_CLUSTER, abi.TRAINER_GRID)}
    line = {
        "metric": "LSMC |price - ADI| at equal wall time: polynomial + fitted network vs polynomial",
        "value": abs(mlp_eq["error_vs_adi"]), "unit": "price units",
        "higher_is_better": False, "n_gpus": 1, "dtype": "f32 paths, bf16 network, f64 solve",
        "data": "synthetic (seeded PCG32 draws; benchmark model parameters)",
        "config": {"workload": "American put under Heston (S0=K=100, v0=theta=0.04, kappa=2, "
                               "xi=0.5, rho=-0.7, r=0.03, T=1), 50 exercise dates x 5 Euler "
                               "substeps; network 3-64-64-1 on the polynomial's residual, 5 "
                               "epochs/date, batch 8192", "fresh_paths_seed": 43},
        "adi": {"price": adi, "grid": "400 x 100 x 400 (MCS, Ikonen-Toivanen)", "cpu_s": adi_s},
        "at_2^20_paths": {"poly3_fp32": poly, "poly3_fp64": poly64, "poly3_plus_network": mlp,
                          "network_alone": alone},
        "parity": {"oracle": oracle_parity},
        "at_equal_wall_time": {"poly3_plus_network": mlp_eq, "network_alone": alone_eq, "poly3": equal},
        "trainer": {"us_per_adam_step": us_per_step[abi.TRAINER_CLUSTER],
                    "us_per_adam_step_grid_barrier_trainer": us_per_step[abi.TRAINER_GRID],
                    "batch": 8192, "network": "3-64-64-1",
                    "timing": "host clock around kgpu_mlp_train, 1008 minus 8 steps"},
        "poly3_by_paths": polys,
        "network_sweep": sweep,
        "roofline": lsmc_roofline(poly, us_per_step[abi.TRAINER_CLUSTER]),
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    """The FP64 CPU restatement of kiyosi's engine on all host threads (the Rust reference
    cannot be compiled here), same workload and metric."""
    from kiyosi_gb300 import abi
    from oracle import loader
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    ctx, packed = packed_plan()
    threads = os.cpu_count() or 1
    s = settings(abi.PRECISION_FP64, abi.SCHEDULE_PLAIN)
    for _ in range(args.warmup):
        loader.price_book(ctx, packed, settings(abi.PRECISION_FP64, abi.SCHEDULE_PLAIN, 1 << 14),
                          threads=threads)
    t0 = time.perf_counter()
    est = None
    for _ in range(args.steps):
        est = loader.price_book(ctx, packed, s, threads=threads)[0]
    elapsed = time.perf_counter() - t0
    value = est.path_steps * args.steps / elapsed
    line = {
        "impl": "reference",
        "metric": "path-steps/s (FP32 batched vs FP64 plain) at <=0.5 SE",
        "value": value, "unit": "path-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Sobol draws; benchmark contract parameters)",
        "config": {"workload": "snowball autocallable, BSM, 2^20 Sobol paths x 504 daily "
                               "steps, 24 monthly KO 103%, daily KI 80%, 15% p.a. coupon",
                   "paths": PATHS, "grid_steps": STEPS, "sampling": "sobol", "seed": SEED},
        "cpu_baseline": {"value": value, "unit": "path-steps/s", "cores": threads,
                         "kind": "port", "sample": f"{args.steps} full pricings"},
        "e2e": {"value": value, "unit": "path-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "price": est.price,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--paths", type=int, default=PATHS,
                    help="path count (profiling runs use smaller cases)")
    ap.add_argument("--dates", type=int, default=50, help="LSMC exercise dates (profiling runs)")
    ap.add_argument("--notes", type=int, default=4096, help="local-volatility book size (profiling runs)")
    ap.add_argument("--mlp-samples", type=int, default=0,
                    help="LSMC network: in-the-money samples trained on per date (0: all)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="use the kernel's default launch shape instead of the autotuner's")
    ap.add_argument("--kernel-only", choices=["fp32", "fp32-lanes", "fp64", "lsmc-poly", "lsmc-mlp", "shared-grid",
                                              "mlp-train-grid", "lv-book"],
                    help="run only the device-resident pricing of one arm (for profilers)")
    ap.add_argument("--tile", type=int, default=0, help="persistent tile paths (0 = default)")
    ap.add_argument("--ctas-per-sm", type=int, default=0, help="persistent CTAs per SM (0 = max)")
    ap.add_argument("--refill", type=int, default=0, help="units between lane refills (0 = 16)")
    ap.add_argument("--workload", default="snowball",
                    choices=["snowball", "european", "heston-asian", "lv-book", "lsmc", "shared-grid",
                             "all"],
                    help="benchmark configuration (default: the snowball headline)")
    args = ap.parse_args()
    TUNING.update(tile_paths=args.tile, ctas_per_sm=args.ctas_per_sm, refill=args.refill)
    if args.workload != "snowball" and args.impl == "ours" and not args.kernel_only:
        names = (["european", "heston-asian", "lv-book", "shared-grid", "lsmc"] if args.workload == "all"
                 else [args.workload])
        for name in names:
            if name == "lsmc":
                run_lsmc(args)
            elif name == "shared-grid":
                run_shared_grid(args)
            else:
                run_workload(args, name)
        return
    if args.kernel_only:
        run_kernel_only(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    run_ours(args)


if __name__ == "__main__":
    main()
