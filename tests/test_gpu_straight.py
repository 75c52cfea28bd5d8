"""The straight kernel (one thread per path) of books whose paths take every grid step --
arithmetic Asians on fixings and vanilla paths -- under Heston, local volatility and BSM
(FP32, PCG32), against the lane-refill kernel, which runs the same grid_step on the same
normals, and against the FP64 oracle.  Cases: several contracts of different step counts
and path counts in one book, ragged last reference blocks, odd normal counts per sample
(a Box-Muller spare carried into the next sample), a local-volatility surface staged in
shared memory, and the launch sequence replayed as a CUDA graph."""
import pytest

from kiyosi_gb300 import plans
from kiyosi_gb300.instruments import AsianOption, EuropeanOption
from kiyosi_gb300.market import PricingContext

from helpers import bsm, gpu_price, heston_asian_c3, heston_context, lv_surface, pack, settings

pytestmark = pytest.mark.gpu


def _books():
    h = heston_context()
    heston = pack([plans.asian(heston_asian_c3(steps=64), h, None),
                   plans.asian(AsianOption("put", 95.0, 0.5, [(i + 1) / 50 for i in range(25)]), h, None),
                   plans.path_vanilla(EuropeanOption("call", 100.0, 1.0), h, 33)],
                  [1 << 14, 3001, 5000])
    lv = PricingContext(lv_surface(), 100.0)
    local = pack([plans.asian(heston_asian_c3(steps=48), lv, None),
                  plans.path_vanilla(EuropeanOption("put", 100.0, 0.75), lv, 37)],
                 [4097, 2048])
    b = bsm()
    black = pack([plans.asian(heston_asian_c3(steps=31), b, None),
                  plans.path_vanilla(EuropeanOption("call", 105.0, 1.0), b, 12)],
                 [2000, 3000])
    return [(h, heston), (lv, local), (b, black)]


def test_straight_equals_lane_refill(native):
    for ctx, packed in _books():
        straight = gpu_price(native, ctx, packed, settings(1 << 12, 31, precision="fp32", schedule="persistent"))
        lanes = gpu_price(native, ctx, packed, settings(1 << 12, 31, precision="fp32", schedule="lane_refill"))
        for a, b in zip(straight, lanes):
            assert abs(a.price - b.price) <= 1e-6 * max(1.0, abs(b.price)), (a.price, b.price)
            assert a.executed_steps == b.executed_steps


def test_straight_against_the_oracle(native):
    from oracle import loader
    for ctx, packed in _books():
        ref = loader.price_book(ctx, packed, settings(1 << 12, 17))
        got = gpu_price(native, ctx, packed, settings(1 << 12, 17, precision="fp32", schedule="persistent"))
        for g, r in zip(got, ref):
            assert abs(g.price - r.price) <= 0.5 * r.sample_error, (g.price, r.price, r.sample_error)


def test_straight_replays(native):
    ctx, packed = _books()[0]
    s = settings(1 << 12, 5, precision="fp32", schedule="persistent")
    runs = [gpu_price(native, ctx, packed, s) for _ in range(4)]
    assert native.last_graph == 2
    for r in runs[1:]:
        assert [e.price for e in r] == [e.price for e in runs[0]]
