"""The phase-major schedule of bridged autocallable books against the lane-refill kernel
and the FP64 oracle.

Both persistent kernels run the same FP32 arithmetic on the same normals in the same
order per path and sum the per-path payoffs in a fixed order, so their estimates and
simulated-position counts must be identical; both land within half a standard error of
the oracle.  Cases: the headline snowball shape (Sobol and PCG32), notes of different
maturities and levels in one book (uneven interval counts, paths of different contracts
in one warp, paths that finish in the phase launches, in the in-launch completion and in
the knocked-in drain), and an odd dimension count (PCG32's Box-Muller spare carried
across the lists)."""
import pytest

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.instruments import AutocallableNote, Observation

from helpers import c2_context, gpu_price, pack, settings, snowball_c2

pytestmark = pytest.mark.gpu
HALF_SE = 0.5


def _book(ctx):
    notes = [snowball_c2(steps=252, years=1.0, months=12),
             snowball_c2(steps=126, years=0.5, months=6, ko=101.0, ki=85.0, coupon=0.2),
             snowball_c2(steps=63, years=0.25, months=3, ko=105.0, ki=90.0, coupon=0.1)]
    dt = 1.0 / 252
    times = [dt * (i + 1) for i in range(189)]
    phoenix = AutocallableNote(initial_spot=100.0, expiry=times[-1], period_coupon=0.02,
                               observations=[Observation(times[21 * (m + 1) - 1], knock_out_level=104.0,
                                                         coupon_barrier_level=90.0) for m in range(9)],
                               knock_in_level=75.0, knock_in_times=times, upper_strike=100.0)
    notes.append(phoenix)
    packed = pack([plans.autocallable(n, ctx) for n in notes], [1 << 18, 300000, 1 << 17, 5000])
    assert all(packed.contracts["flags"] & abi.C_BRIDGE)
    return packed


def _same(a, b):
    for x, y in zip(a, b):
        assert x.price == y.price, (x.price, y.price)
        assert x.executed_steps == y.executed_steps
        assert x.sample_error == y.sample_error


@pytest.mark.parametrize("sobol", [True, False])
def test_phased_equals_lane_refill_on_the_headline_shape(native, sobol):
    from oracle import loader
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(), ctx)])
    for n in (1 << 16, 1 << 20):
        phased = gpu_price(native, ctx, packed, settings(n, 42, sobol=sobol, precision="fp32", schedule="persistent"))
        lanes = gpu_price(native, ctx, packed, settings(n, 42, sobol=sobol, precision="fp32", schedule="lane_refill"))
        _same(phased, lanes)
    ref = loader.price_book(ctx, packed, settings(1 << 16, 42, sobol=sobol))[0]
    small = gpu_price(native, ctx, packed, settings(1 << 16, 42, sobol=sobol, precision="fp32", schedule="persistent"))
    assert abs(small[0].price - ref.price) <= HALF_SE * ref.sample_error


def test_phased_mixed_book(native):
    from oracle import loader
    ctx = c2_context()
    packed = _book(ctx)
    s = settings(1 << 12, 7, precision="fp32", schedule="persistent")
    phased = gpu_price(native, ctx, packed, s)
    lanes = gpu_price(native, ctx, packed, settings(1 << 12, 7, precision="fp32", schedule="lane_refill"))
    _same(phased, lanes)
    small = pack([plans.autocallable(snowball_c2(steps=126, years=0.5, months=6, ko=101.0, ki=85.0,
                                                 coupon=0.2), ctx)])
    ref = loader.price_book(ctx, small, settings(1 << 14, 7))[0]
    got = gpu_price(native, ctx, small, settings(1 << 14, 7, precision="fp32", schedule="persistent"))[0]
    assert abs(got.price - ref.price) <= HALF_SE * ref.sample_error
    # The same book again: results do not depend on the order atomics hand out slots.
    _same(phased, gpu_price(native, ctx, packed, s))


def test_phased_odd_dimensions_pcg(native):
    """Two intervals (9 and 10 days) over 19 grid steps: odd normal counts per sample put
    the Box-Muller spare at different parities across samples and intervals."""
    ctx = c2_context()
    dt = 1.0 / 252
    times = [dt * (i + 1) for i in range(19)]
    note = AutocallableNote(initial_spot=100.0, expiry=times[-1], knock_in_level=97.0, knock_in_times=times,
                            observations=[Observation(times[i], knock_out_level=101.0, coupon_rate=0.1)
                                          for i in (8, 18)],
                            upper_strike=100.0, maturity_coupon_rate=0.1)
    packed = pack([plans.autocallable(note, ctx)])
    assert packed.contracts[0]["flags"] & abi.C_BRIDGE
    for n in (4097, 400001):
        phased = gpu_price(native, ctx, packed, settings(n, 3, precision="fp32", schedule="persistent"))
        lanes = gpu_price(native, ctx, packed, settings(n, 3, precision="fp32", schedule="lane_refill"))
        _same(phased, lanes)
