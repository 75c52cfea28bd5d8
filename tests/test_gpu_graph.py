"""The persistent schedules' launch sequence as a CUDA graph (kgpu_price_book).

The first call with a key runs directly, the second captures the sequence into a graph
and launches it, later ones replay it; a different call in between drops the graph.
Every call's estimates are identical bit for bit, whichever way it ran: the phase-major
snowball (Sobol and PCG32, host and device-resident books), the lane-refill kernel on a
Heston Asian book, a changed book content under the same arrays (read at every replay),
and cancellation of a replayed call."""
import ctypes as C

import numpy as np
import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.errors import KiyosiError

from helpers import (c2_context, gpu_price, heston_asian_c3, heston_context, pack, settings,
                     snowball_c2)

pytestmark = pytest.mark.gpu


def _same(a, b):
    for x, y in zip(a, b):
        assert x.price == y.price and x.sample_error == y.sample_error, (x.price, y.price)
        assert x.standard_error == y.standard_error or (x.standard_error != x.standard_error)
        assert x.executed_steps == y.executed_steps and x.uncertainty_status == y.uncertainty_status


def _calls(native, ctx, packed, s, count=5):
    """Prices `count` times; returns the estimates and each call's graph mode."""
    out, modes = [], []
    for _ in range(count):
        out.append(gpu_price(native, ctx, packed, s))
        modes.append(native.last_graph)
    return out, modes


@pytest.mark.parametrize("sobol", [True, False])
def test_phase_major_replay_is_identical(native, sobol):
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(), ctx)])
    s = settings(1 << 18, 42, sobol=sobol, precision="fp32", schedule="persistent")
    runs, modes = _calls(native, ctx, packed, s)
    _captured_then_replayed(modes)
    for r in runs[1:]:
        _same(r, runs[0])
    assert native.last_launches >= 3
    # another book in between drops the graph; the first book captures again
    other = pack([plans.autocallable(snowball_c2(steps=252, years=1.0, months=12), ctx)])
    gpu_price(native, ctx, other, s)
    assert native.last_graph == 0
    again, modes = _calls(native, ctx, packed, s)
    _captured_then_replayed(modes)
    for r in again:
        _same(r, runs[0])


def _captured_then_replayed(modes):
    """Direct calls until the key repeats, one capture, then replays."""
    assert modes.count(1) == 1 and modes[-1] == 2, modes
    first = modes.index(1)
    assert set(modes[:first]) == {0} and set(modes[first + 1:]) == {2}, modes


def test_lane_refill_heston_replay_is_identical(native):
    hctx = heston_context()
    packed = pack([plans.asian(heston_asian_c3(steps=64), hctx, None)] * 3, [1 << 14, 5000, 1 << 12])
    s = settings(1 << 14, 9, precision="fp32", schedule="persistent")
    runs, modes = _calls(native, hctx, packed, s)
    _captured_then_replayed(modes)
    for r in runs[1:]:
        _same(r, runs[0])


def test_device_book_contents_are_read_at_every_replay(native):
    """A replayed graph reads the caller's device arrays at launch: changing a step record
    in place changes the price exactly as a direct call would see it."""
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(), ctx)])
    torch = pytest.importorskip("torch")
    dev = {}
    for name in ("steps", "flags", "events", "intervals", "daily"):
        arr = getattr(packed, name)
        t = torch.from_numpy(arr.view(np.uint8).copy()).cuda()
        dev[name] = t
    book = abi.Book()
    host = packed.struct()
    book.contract_count = 1
    book.contracts = host.contracts
    book.step_total = host.step_total
    book.steps = C.cast(dev["steps"].data_ptr(), C.POINTER(abi.Step))
    book.step_flags = C.cast(dev["flags"].data_ptr(), C.POINTER(C.c_uint8))
    book.events = C.cast(dev["events"].data_ptr(), C.POINTER(abi.Event))
    book.event_total = host.event_total
    book.intervals = C.cast(dev["intervals"].data_ptr(), C.POINTER(abi.BridgeInterval))
    book.interval_total = host.interval_total
    book.bridge_daily = C.cast(dev["daily"].data_ptr(), C.POINTER(abi.BridgeDaily))
    model = ctx.kgpu_model()
    s = settings(1 << 16, 42, sobol=True, precision="fp32", schedule="persistent")
    out = (abi.Estimate * 1)()

    def price():
        torch.cuda.synchronize()
        native.check(native.lib.kgpu_price_book_device(native.handle, C.byref(model), C.byref(book),
                                                       C.byref(s), out))
        return abi.Estimate.from_buffer_copy(out[0]), native.last_graph
    base = [price() for _ in range(5)]
    _captured_then_replayed([m for _, m in base])
    for e, _ in base[1:]:
        _same([e], [base[0][0]])
    # lower every knock-out payment in place: the replay sees the new events
    events = packed.events.copy()
    events["payment"] *= 0.5
    dev["events"].copy_(torch.from_numpy(events.view(np.uint8).copy()).cuda())
    changed, mode = price()
    assert mode == 2 and changed.price < base[0][0].price
    direct = gpu_price(native, ctx, plans.PackedBook(packed.contracts, packed.steps, packed.flags, events,
                                                     packed.intervals, packed.daily),
                       s)[0]
    assert changed.price == direct.price


def test_cancelled_replay(native):
    """A replayed call whose cancellation word is set ends with InterruptedError and no
    result; the next call replays cleanly."""
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(), ctx)])
    s = settings(1 << 18, 42, sobol=True, precision="fp32", schedule="persistent")
    flag = C.c_int32(0)
    runs = []
    for _ in range(5):
        runs.append(gpu_price(native, ctx, packed, s, cancel=flag))
    assert native.last_graph == 2
    flag.value = 1
    with pytest.raises(InterruptedError):
        gpu_price(native, ctx, packed, s, cancel=flag)
    flag.value = 0
    again = gpu_price(native, ctx, packed, s, cancel=flag)
    assert native.last_graph == 2
    _same(again, runs[0])


def test_other_entry_points_in_between(native):
    """A Sobol sequence of another seed and size built in between (kgpu_sobol_points
    rebuilds the context's cached tables) is not read by a replay: the next call runs
    directly and its estimate is unchanged."""
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(), ctx)])
    s = settings(1 << 18, 42, sobol=True, precision="fp32", schedule="persistent")
    runs, modes = _calls(native, ctx, packed, s)
    _captured_then_replayed(modes)
    bits = np.zeros(64, np.uint64)
    native.check(native.lib.kgpu_sobol_points(native.handle, 7, 33, 5, 0, 64,
                                              bits.ctypes.data_as(C.POINTER(C.c_uint64)), None, 0))
    after = gpu_price(native, ctx, packed, s)
    assert native.last_graph == 0
    _same(after, runs[0])


def test_host_book_contents_change_under_one_contract_table(native):
    """A host book whose step records change while its contract table stays: every call
    uploads the book, and the replayed sequence prices the new records."""
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(), ctx)])
    s = settings(1 << 16, 42, sobol=True, precision="fp32", schedule="persistent")
    runs, modes = _calls(native, ctx, packed, s, 4)
    _captured_then_replayed(modes)
    changed = plans.PackedBook(packed.contracts, packed.steps.copy(), packed.flags, packed.events.copy(),
                               packed.intervals, packed.daily)
    changed.events["payment"] *= 0.5
    replayed = gpu_price(native, ctx, changed, s)
    assert native.last_graph == 2 and replayed[0].price < runs[0][0].price
    gpu_price(native, ctx, pack([plans.autocallable(snowball_c2(steps=252, years=1.0, months=12), ctx)]), s)
    direct = gpu_price(native, ctx, changed, s)
    assert native.last_graph == 0
    _same(replayed, direct)
