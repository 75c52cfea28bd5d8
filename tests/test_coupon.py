"""Implied coupons (risk/coupon.rs) on the pricing engine: the two bound notes are
priced in one book on one seed, and the affine coupon curve between them is
interpolated, as kiyosi's prepare_coupon_pricer does.

CPU: the solver on the oracle (an engine stand-in that prices books with the oracle):
round trips through a seeded price, both quote conventions, Phoenix coupons, the
minimum quotable coupon and the error cases.
GPU: the same round trip through MonteCarloAutocallableEngine."""
import math
from dataclasses import replace

import pytest

from kiyosi_gb300 import coupon, plans
from kiyosi_gb300.errors import InvalidInputError, RootNotBracketedError
from kiyosi_gb300.instruments import AutocallableNote, Observation
from oracle import loader

from helpers import c2_context, pack, settings, snowball_c2


class OracleEngine:
    def __init__(self, paths, seed, sobol=True):
        self.paths, self.seed, self.sobol = paths, seed, sobol

    def _run(self, ctx, plan_list):
        out = []
        sampled = [p for p in plan_list if not isinstance(p, plans.Known)]
        est = iter(loader.price_book(ctx, pack(sampled), settings(self.paths, self.seed, sobol=self.sobol))
                   if sampled else [])
        for p in plan_list:
            out.append(type("E", (), {"price": p.value})() if isinstance(p, plans.Known) else next(est))
        return out

    def price(self, note, ctx):
        return self._run(ctx, [plans.autocallable(note, ctx)])[0].price


def _note(steps=126, years=0.5):
    return snowball_c2(steps=steps, years=years, months=6)


@pytest.mark.parametrize("convention", [coupon.PRESERVE_MATURITY_COUPON, coupon.SHIFT_MATURITY_COUPON])
def test_snowball_coupon_round_trip(convention):
    ctx = c2_context()
    engine = OracleEngine(1 << 14, 42)
    note = _note()
    target = coupon.with_snowball_coupon(note, 0.11, convention)
    observed = engine.price(target, ctx)
    solved, used = coupon.implied_snowball_coupon(engine, note, ctx, observed, convention)
    assert used == convention
    assert abs(solved - 0.11) < 1e-6, solved
    assert abs(engine.price(coupon.with_snowball_coupon(note, solved, convention), ctx) - observed) < 1e-7


def test_with_coupon_shifts_every_observation():
    note = _note()
    shifted = coupon.with_snowball_coupon(note, 0.2, coupon.SHIFT_MATURITY_COUPON)
    shift = 0.2 - note.observations[0].coupon_rate
    assert all(abs(b.coupon_rate - (a.coupon_rate + shift)) < 1e-15
               for a, b in zip(note.observations, shifted.observations))
    assert shifted.maturity_coupon_rate == note.maturity_coupon_rate + shift
    kept = coupon.with_snowball_coupon(note, 0.2, coupon.PRESERVE_MATURITY_COUPON)
    assert kept.maturity_coupon_rate == note.maturity_coupon_rate


def test_minimum_quoted_coupon_and_errors():
    ctx = c2_context()
    engine = OracleEngine(1 << 12, 7)
    note = replace(_note(), fixed_knock_in_coupon=0.03)
    minimum = coupon.minimum_quoted_coupon(note, coupon.SHIFT_MATURITY_COUPON)
    shifted = coupon.with_snowball_coupon(note, minimum, coupon.SHIFT_MATURITY_COUPON)
    assert shifted.maturity_coupon_rate >= 0.03
    assert coupon.minimum_quoted_coupon(note, coupon.PRESERVE_MATURITY_COUPON) is None
    with pytest.raises(RootNotBracketedError):
        coupon.implied_snowball_coupon(engine, _note(), ctx, 5.0)
    with pytest.raises(InvalidInputError):
        coupon.implied_snowball_coupon(engine, _note(), ctx, 1.0,
                                       settings=coupon.ImpliedCouponSettings(lower_bound=1.0, upper_bound=0.5))
    unseeded = OracleEngine(1 << 12, None)
    with pytest.raises(InvalidInputError):
        coupon.implied_snowball_coupon(unseeded, _note(), ctx, 1.0)


def test_phoenix_coupon_round_trip():
    ctx = c2_context()
    engine = OracleEngine(1 << 14, 11)
    obs = [Observation(t / 12, knock_out_level=103.0, coupon_barrier_level=85.0) for t in range(1, 7)]
    note = AutocallableNote(initial_spot=100.0, expiry=0.5, observations=obs, knock_in_level=80.0,
                            upper_strike=100.0, period_coupon=0.01)
    observed = engine.price(coupon.with_phoenix_coupon(note, 0.017), ctx)
    solved = coupon.implied_phoenix_coupon(engine, note, ctx, observed)
    assert abs(solved - 0.017) < 1e-6, solved


@pytest.mark.gpu
def test_implied_coupon_on_the_gpu_engine(native):
    from kiyosi_gb300.pricing import MonteCarloAutocallableEngine
    ctx = c2_context()
    engine = MonteCarloAutocallableEngine(path_count=1 << 16, seed=42, sampling="sobol")
    note = snowball_c2()
    observed = engine.price(coupon.with_snowball_coupon(note, 0.12, coupon.PRESERVE_MATURITY_COUPON), ctx)
    solved, _ = coupon.implied_snowball_coupon(engine, note, ctx, observed)
    assert abs(solved - 0.12) < 1e-6, solved
