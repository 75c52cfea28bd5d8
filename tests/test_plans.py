"""Host plan builders (no GPU): grids, events and the bridge decision."""
import math

import numpy as np

from kiyosi_gb300 import abi, plans
from kiyosi_gb300.instruments import EuropeanOption

from helpers import bsm, c2_context, heston_asian_c3, heston_context, lv_book, snowball_c2


def test_snowball_plan_matches_reference_grid():
    ctx = c2_context()
    p = plans.autocallable(snowball_c2(), ctx)
    c = p.record
    assert c["step_count"] == 504 and c["event_count"] == 24
    assert int(np.sum(p.flags & abi.STEP_EVENT != 0)) == 24
    assert int(np.sum(p.flags & abi.STEP_KNOCK_IN != 0)) == 504
    # Daily knock-in with 21-step gaps between events selects the Brownian bridge.
    assert c["flags"] & abi.C_BRIDGE
    assert len(p.intervals) == 24 and p.intervals[-1]["end"] == 503
    assert math.isclose(c["knock_in"], math.log(0.8), rel_tol=1e-15)
    # Knock-out pays principal plus the accrued coupon, discounted on the host.
    e0 = p.events[0]
    t = 21 * 2.0 / 504
    assert math.isclose(e0["payment"][2], (1.0 + 0.15 * t) * math.exp(-0.03 * t), rel_tol=1e-14)


def test_transition_is_reference_formula():
    ctx = bsm()
    p = plans.path_vanilla(EuropeanOption("call", 100.0, 1.0), ctx, 252)
    dt = 1.0 / 252
    assert p.steps["drift"][0] == (0.05 - 0.02 - 0.5 * 0.2 * 0.2) * dt
    assert p.steps["diffusion"][0] == 0.2 * math.sqrt(dt)


def test_heston_asian_plan_has_fixings_on_every_step():
    p = plans.asian(heston_asian_c3(), heston_context(), 252)
    assert int(np.sum(p.flags & abi.STEP_FIXING != 0)) == 252


def test_book_packs_offsets():
    from helpers import lv_surface
    from kiyosi_gb300.market import PricingContext
    notes, paths = lv_book(6, min_log2=8, max_log2=10)
    ctx = PricingContext(lv_surface(), 100.0)
    b = plans.BookBuilder()
    for n in notes:
        b.add(plans.autocallable(n, ctx))
    packed = b.build(paths)
    offs = packed.contracts["step_offset"]
    counts = packed.contracts["step_count"]
    assert np.all(offs[1:] == np.cumsum(counts)[:-1])
    assert len(packed.steps) == int(np.sum(counts))
    assert np.all(packed.contracts["flags"] & abi.C_BRIDGE == 0)  # no bridge off BSM
