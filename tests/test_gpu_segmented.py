"""The segmented kernel of BSM vanilla-path books (FP32, PCG32; kSegments lanes per path,
each from its own position of the path's stream) against the lane-refill kernel on the
same normals, and against the FP64 oracle.

Only the order of the FP32 additions of a path's log return differs from the sequential
walk, so prices agree to 1e-5 relative and the simulated step counts exactly; a segment
that started on the wrong normal would move a price by about a standard error.  Cases:
step counts not divisible by the segment count, odd dimension counts (a sample's first
normal is a Box-Muller spare for every other sample), one-step paths, several contracts
of different path counts in one book, ragged last reference blocks."""
import pytest

from kiyosi_gb300 import plans
from kiyosi_gb300.instruments import EuropeanOption

from helpers import bsm, gpu_price, pack, settings

pytestmark = pytest.mark.gpu


def _book(ctx):
    contracts = [plans.path_vanilla(EuropeanOption("call", 100.0, 1.0), ctx, 252),
                 plans.path_vanilla(EuropeanOption("put", 95.0, 0.5), ctx, 7),
                 plans.path_vanilla(EuropeanOption("call", 105.0, 0.25), ctx, 3),
                 plans.path_vanilla(EuropeanOption("put", 100.0, 1.0), ctx, 251),
                 plans.path_vanilla(EuropeanOption("call", 90.0, 0.1), ctx, 1),
                 plans.path_vanilla(EuropeanOption("call", 100.0, 2.0), ctx, 17)]
    return pack(contracts, [1 << 14, 1000, 4097, 300, 257, 5000])


def test_segmented_equals_lane_refill(native):
    ctx = bsm()
    packed = _book(ctx)
    seg = gpu_price(native, ctx, packed, settings(1 << 14, 17, precision="fp32", schedule="persistent"))
    lanes = gpu_price(native, ctx, packed, settings(1 << 14, 17, precision="fp32", schedule="lane_refill"))
    for a, b in zip(seg, lanes):
        assert abs(a.price - b.price) <= 1e-5 * max(1.0, abs(b.price)), (a.price, b.price)
        assert a.executed_steps == b.executed_steps and a.path_steps == b.path_steps


def test_segmented_against_the_oracle(native):
    from oracle import loader
    ctx = bsm()
    packed = _book(ctx)
    ref = loader.price_book(ctx, packed, settings(1 << 14, 23))
    got = gpu_price(native, ctx, packed, settings(1 << 14, 23, precision="fp32", schedule="persistent"))
    for g, r in zip(got, ref):
        assert abs(g.price - r.price) <= 0.5 * r.sample_error, (g.price, r.price, r.sample_error)


def test_segmented_is_deterministic_and_replays(native):
    ctx = bsm()
    packed = _book(ctx)
    s = settings(1 << 14, 5, precision="fp32", schedule="persistent")
    runs = [gpu_price(native, ctx, packed, s) for _ in range(4)]
    assert native.last_graph == 2
    for r in runs[1:]:
        assert [e.price for e in r] == [e.price for e in runs[0]]
