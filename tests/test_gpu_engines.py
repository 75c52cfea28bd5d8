"""The Python engine surface (kiyosi.pricing names and keywords) on the GPU."""
import pytest

from kiyosi_gb300.instruments import EuropeanOption
from kiyosi_gb300.pricing import (MonteCarloAutocallableEngine, MonteCarloVanillaEngine,
                                  MonteCarloEstimate)

from helpers import bsm, c2_context, snowball_c2

pytestmark = pytest.mark.gpu


def test_vanilla_engine_replays_with_seed():
    ctx = bsm()
    opt = EuropeanOption("call", 100.0, 1.0)
    engine = MonteCarloVanillaEngine(path_count=1 << 15, seed=None).with_resolved_seed()
    a = engine.price_with_statistics(opt, ctx)
    b = MonteCarloVanillaEngine(path_count=1 << 15, seed=a.seed).price_with_statistics(opt, ctx)
    assert a == b and a.standard_error > 0 and a.confidence_interval[0] < a.price
    assert abs(a.price - 9.227005508154047) < 5 * a.standard_error


def test_autocallable_price_many_matches_single_prices():
    ctx = c2_context()
    notes = [snowball_c2(steps=126, years=0.5, months=6, ko=k) for k in (100.0, 103.0, 106.0)]
    engine = MonteCarloAutocallableEngine(path_count=1 << 12, seed=5)
    many = engine.price_many(notes, ctx)
    single = [engine.price(n, ctx) for n in notes]
    assert many == single
