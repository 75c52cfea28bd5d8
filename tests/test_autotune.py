"""The persistent schedule's autotuner: signatures and the cache on the CPU; on the GPU,
that the tuned shape is the fastest it timed and that prices do not depend on shape."""
import os

import pytest

from kiyosi_gb300 import abi, autotune, plans
from kiyosi_gb300.instruments import EuropeanOption

from helpers import bsm, c2_context, gpu_price, pack, settings, snowball_c2


def test_signature_and_cache_roundtrip(tmp_path):
    ctx = bsm()
    packed = pack([plans.european(EuropeanOption("call", 100.0, 1.0), ctx)] * 3, [256, 1024, 4096])
    s = settings(1 << 12, 1, precision="fp32", schedule="persistent")
    key = autotune.signature(ctx.kgpu_model().kind, packed, s)
    assert key[3] == 3 and key[4] == 12  # three contracts, 5376 samples -> 2^12
    path = os.path.join(str(tmp_path), "shapes.json")
    cache = autotune.Cache(path)
    cache.put(key, autotune.Shape(64, 3, 8))
    assert autotune.Cache(path).get(key) == autotune.Shape(64, 3, 8)
    assert len(list(autotune.candidates())) == 36 and len(list(autotune.candidates(True))) == 8


@pytest.mark.gpu
def test_tuned_shape_is_fastest_timed_and_price_invariant(native):
    ctx = c2_context()
    packed = pack([plans.autocallable(snowball_c2(steps=252, years=1.0, months=12), ctx)])
    s = settings(1 << 16, 42, sobol=True, precision="fp32", schedule="persistent")
    best, timings = autotune.tune(native, ctx, packed, s, cache=autotune.Cache())
    assert timings[best] == min(timings.values())
    prices = {gpu_price(native, ctx, packed, autotune.apply(s, shape))[0].price
              for shape in list(timings)[:6] + [best]}
    assert len(prices) == 1
