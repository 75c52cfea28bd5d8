"""kgpu_price_contract_noalloc: pricing without device allocation.

Callers that cannot call cudaMalloc (a host that hands out slices of a device-memory
budget it reserved up front, a plugin inside such a host, a loop that must never
allocate) price through this entry point, whose scratch is a fixed array in device
memory.  This file is collected last; it checks the entry point through the C ABI
against the FP64 oracle and kgpu_price_book on the same plan and settings, on two calls
in a row, and that it refuses bad device plans and settings before any launch.
"""
import ctypes as C

import numpy as np
import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.errors import InvalidInputError, UnsupportedOperationError, raise_for_status
from kiyosi_gb300.instruments import EuropeanOption

from helpers import (c2_context, gpu_price, heston_asian_c3, heston_context, lv_surface, pack,
                     settings, snowball_c2)
from kiyosi_gb300.market import PricingContext


def lv_context(surface):
    return PricingContext(surface, 100.0)

pytestmark = pytest.mark.gpu
FP64_REL = 1e-12


class DeviceArrays:
    """Device copies of a packed book, made by the test (the caller here can allocate)."""

    def __init__(self):
        self.rt = None
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        assert self.rt is not None, "libcudart not found"
        self.rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.rt.cudaFree.argtypes = [C.c_void_p]
        self.ptrs = []

    def put(self, array):
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), max(int(array.nbytes), 16)) == 0
        if array.nbytes:
            assert self.rt.cudaMemcpy(p, array.ctypes.data, array.nbytes, 1) == 0
        self.ptrs.append(p)
        return p

    def book(self, packed):
        b = abi.Book()
        b.contract_count = len(packed.contracts)
        b.contracts = C.cast(self.put(packed.contracts), C.POINTER(abi.Contract))
        b.step_total = len(packed.steps)
        b.steps = C.cast(self.put(packed.steps), C.POINTER(abi.Step))
        b.step_flags = C.cast(self.put(packed.flags), C.POINTER(C.c_uint8))
        if packed.daily is not None:
            b.bridge_daily = C.cast(self.put(packed.daily), C.POINTER(abi.BridgeDaily))
        b.event_total = len(packed.events)
        b.interval_total = len(packed.intervals)
        b.events = C.cast(self.put(packed.events), C.POINTER(abi.Event))
        b.intervals = C.cast(self.put(packed.intervals), C.POINTER(abi.BridgeInterval))
        return b

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)


def _noalloc(lib, ctx, book, index, s):
    out = abi.Estimate()
    model = ctx.kgpu_model()
    status = lib.kgpu_price_contract_noalloc(C.byref(model), C.byref(book), index, C.byref(s),
                                             C.byref(out), None)
    raise_for_status(status, lib.kgpu_last_error_message(None).decode())
    return out


def _same(got, ref):
    assert abs(got.price - ref.price) <= FP64_REL * abs(ref.price), (got.price, ref.price)
    if ref.uncertainty_status == 0:
        assert abs(got.standard_error - ref.standard_error) <= FP64_REL * ref.standard_error
    assert got.uncertainty_status == ref.uncertainty_status


def test_noalloc_matches_oracle_and_price_book_on_consecutive_calls(native):
    from oracle import loader
    ctx = c2_context()
    packed = pack([plans.european(EuropeanOption("put", 95.0, 0.5), ctx),
                   plans.path_vanilla(EuropeanOption("call", 100.0, 1.0), ctx, 63),
                   plans.autocallable(snowball_c2(steps=126, years=0.5, months=6), ctx)])
    s = settings(20000, 5)
    expected = gpu_price(native, ctx, packed, s)
    oracle = loader.price_book(ctx, packed, s)
    arrays = DeviceArrays()
    try:
        book = arrays.book(packed)
        lib = native.lib
        # Two calls in a row on the same contract, then the others: the shared scratch
        # keeps the previous call's contents and must not leak into the next result.
        for index in (2, 2, 0, 1):
            got = _noalloc(lib, ctx, book, index, s)
            _same(got, oracle[index])
            _same(got, expected[index])
            assert got.executed_steps == expected[index].executed_steps
        # Beyond the fixed scratch: rejected with a clear error, nothing launched.
        with pytest.raises(InvalidInputError, match="4,194,304"):
            _noalloc(lib, ctx, book, 0, settings(5_000_000, 5))
    finally:
        arrays.free()


def test_noalloc_heston_and_odd_antithetic_match_the_oracle(native):
    from oracle import loader
    hctx = heston_context()
    hpacked = pack([plans.asian(heston_asian_c3(steps=48), hctx, None)])
    bctx = c2_context()
    bpacked = pack([plans.autocallable(snowball_c2(steps=126, years=0.5, months=6), bctx)])
    arrays = DeviceArrays()
    try:
        lib = native.lib
        for ctx, packed, s in ((hctx, hpacked, settings(12345, 9)),
                               (bctx, bpacked, settings(4097, 11, antithetic=True))):
            book = arrays.book(packed)
            ref = loader.price_book(ctx, packed, s)[0]
            for _ in range(2):
                _same(_noalloc(lib, ctx, book, 0, s), ref)
    finally:
        arrays.free()


def test_noalloc_refuses_what_it_does_not_run(native):
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(steps=126, years=0.5, months=6), ctx)])
    arrays = DeviceArrays()
    try:
        book = arrays.book(packed)
        lib = native.lib
        for s in (settings(4096, 5, sobol=True), settings(4096, 5, precision="fp32"),
                  settings(4096, 5, schedule="persistent")):
            with pytest.raises(UnsupportedOperationError):
                _noalloc(lib, ctx, book, 0, s)
        s = settings(4096, 5)
        s.precision = 7
        with pytest.raises(InvalidInputError, match="precision"):
            _noalloc(lib, ctx, book, 0, s)
        lv = lv_surface(7)
        with pytest.raises(UnsupportedOperationError):
            _noalloc(lib, lv_context(lv), book, 0, settings(4096, 5))
    finally:
        arrays.free()


def _bad(packed, **changes):
    contracts = packed.contracts.copy()
    for k, v in changes.items():
        contracts[0][k] = v
    return plans.PackedBook(contracts, packed.steps, packed.flags, packed.events,
                            packed.intervals, packed.daily)


def test_noalloc_rejects_bad_device_plans_before_any_launch(native):
    ctx = c2_context()
    note = snowball_c2(steps=126, years=0.5, months=6)
    bridged = pack([plans.autocallable(note, ctx)])
    assert bridged.contracts[0]["flags"] & abi.C_BRIDGE
    terminal = pack([plans.european(EuropeanOption("put", 95.0, 0.5), ctx)])
    c = bridged.contracts[0]
    cases = [
        (bridged, dict(event_offset=1)),
        (bridged, dict(event_count=int(c["event_count"]) + 1)),
        (bridged, dict(event_count=int(c["event_count"]) - 1)),
        (bridged, dict(bridge_offset=1)),
        (bridged, dict(bridge_count=0)),
        (bridged, dict(bridge_count=int(c["bridge_count"]) - 1)),
        (bridged, dict(step_offset=1)),
        (terminal, dict(dimensions=4)),
    ]
    arrays = DeviceArrays()
    try:
        lib = native.lib
        for packed, change in cases:
            book = arrays.book(_bad(packed, **change))
            with pytest.raises(InvalidInputError):
                _noalloc(lib, ctx, book, 0, settings(4096, 5))
        # A bridged contract whose book has no interval or daily arrays.
        book = arrays.book(bridged)
        book.intervals = None
        with pytest.raises(InvalidInputError, match="bridge"):
            _noalloc(lib, ctx, book, 0, settings(4096, 5))
        book = arrays.book(bridged)
        book.bridge_daily = None
        with pytest.raises(InvalidInputError, match="bridge"):
            _noalloc(lib, ctx, book, 0, settings(4096, 5))
        # The intact book still prices after the refusals.
        from oracle import loader
        ref = loader.price_book(ctx, bridged, settings(4096, 5))[0]
        _same(_noalloc(lib, ctx, arrays.book(bridged), 0, settings(4096, 5)), ref)
    finally:
        arrays.free()
