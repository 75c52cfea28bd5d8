"""The benchmark configurations of the GPU Monte Carlo engines as builders: seeded
synthetic contracts and models with the configurations' parameters (no dataset is
involved).  Tests build reduced-size versions with the same code.

* european(): plain MC European call under BSM, 252 daily log-Euler steps.
* snowball_c2() / c2_context(): single snowball autocallable under BSM, 504 daily steps.
* heston_asian_c3() / heston_context(): Heston arithmetic-average Asian call, 252 steps.
* lv_surface() / lv_book(): book of snowball/phoenix notes under local volatility.
* heston_context() with an American put for least-squares Monte Carlo.
* shared_grid_book() / c2_context(): a book of snowball and Phoenix notes on one daily
  grid under BSM, priced with price_many on the shared grid.
"""
import math

import numpy as np

from .instruments import AsianOption, AutocallableNote, EuropeanOption, Observation
from .market import (BlackScholesMertonParameters, HestonParameters, LocalVolatilitySurface,
                     PricingContext)


def bsm(rate=0.05, dividend=0.02, sigma=0.2, spot=100.0):
    return PricingContext(BlackScholesMertonParameters(rate, dividend, sigma), spot)


def heston_context(spot=100.0):
    """The Heston model of the Asian and American benchmark workloads."""
    return PricingContext(HestonParameters(rate=0.03, dividend=0.0, v0=0.04, kappa=2.0,
                                           theta=0.04, xi=0.5, rho=-0.7), spot)


def snowball_c2(steps=504, years=2.0, months=24, ko=103.0, ki=80.0, coupon=0.15):
    """Single snowball under BSM: daily steps, monthly knock-out observations (every
    steps/months steps), daily knock-in, annual coupon accrued A/365F."""
    dt = years / steps
    per = steps // months
    times = [dt * (i + 1) for i in range(steps)]
    obs = [Observation(times[per * (m + 1) - 1], knock_out_level=ko, coupon_rate=coupon)
           for m in range(months)]
    return AutocallableNote(initial_spot=100.0, expiry=times[-1], observations=obs,
                            knock_in_level=ki, knock_in_times=times, upper_strike=100.0,
                            lower_strike=0.0, maturity_coupon_rate=coupon)


def c2_context():
    return PricingContext(BlackScholesMertonParameters(0.03, 0.0, 0.25), 100.0)


def lv_surface(seed=7, n_spot=50, n_time=20, rate=0.03, dividend=0.0):
    """Local-vol grid: spots log-spaced on [50, 200], times over (0, 3y], vols U[0.15, 0.45]."""
    rng = np.random.default_rng(seed)
    spots = np.exp(np.linspace(math.log(50.0), math.log(200.0), n_spot))
    times = np.linspace(3.0 / n_time, 3.0, n_time)
    vols = rng.uniform(0.15, 0.45, size=(n_time, n_spot))
    return LocalVolatilitySurface(rate, dividend, times, spots, vols)


def lv_book(count, seed=7, min_log2=14, max_log2=18, months_range=(3, 36)):
    """A book of snowball/phoenix notes (1:1) under local volatility: monthly observations
    (21 daily steps per month), KO U[1.00, 1.05] S0, KI U[0.70, 0.85] S0, coupons
    U[0.05, 0.25] p.a., paths 2^U[min,max] rounded to a multiple of 256."""
    rng = np.random.default_rng(seed)
    notes, paths = [], []
    dt = 1.0 / 252.0
    for i in range(count):
        months = int(rng.integers(months_range[0], months_range[1] + 1))
        steps = 21 * months
        times = [dt * (k + 1) for k in range(steps)]
        ko = 100.0 * rng.uniform(1.00, 1.05)
        ki = 100.0 * rng.uniform(0.70, 0.85)
        coupon = rng.uniform(0.05, 0.25)
        if i % 2 == 0:
            obs = [Observation(times[21 * (m + 1) - 1], knock_out_level=ko, coupon_rate=coupon)
                   for m in range(months)]
            note = AutocallableNote(initial_spot=100.0, expiry=times[-1], observations=obs,
                                    knock_in_level=ki, knock_in_times=times, upper_strike=100.0,
                                    lower_strike=0.0, maturity_coupon_rate=coupon)
        else:
            obs = [Observation(times[21 * (m + 1) - 1], knock_out_level=ko,
                               coupon_barrier_level=ki) for m in range(months)]
            note = AutocallableNote(initial_spot=100.0, expiry=times[-1], observations=obs,
                                    knock_in_level=ki, knock_in_times=times, upper_strike=100.0,
                                    lower_strike=0.0, period_coupon=coupon / 12.0)
        notes.append(note)
        p = 2.0 ** rng.uniform(min_log2, max_log2)
        paths.append(max(256, int(round(p / 256.0)) * 256))
    return notes, paths


def heston_asian_c3(steps=252):
    times = [(i + 1) / steps for i in range(steps)]
    return AsianOption("call", 100.0, 1.0, times)


def european():
    """S0 = K = 100, r = 0.05, q = 0.02, sigma = 0.2, T = 1y (the reference's
    calibration inputs)."""
    return bsm(), EuropeanOption("call", 100.0, 1.0)


def shared_grid_book(coupons=32, steps=504, years=2.0, months=24):
    """A dealer book on one underlying and one daily grid: 128 term sets (snowball or
    Phoenix; 6, 12, 18 or 24 monthly observations, each maturity a monitoring date;
    knock-out 100/102/103/105%; knock-in 70/75/80/85%) with `coupons` coupons each,
    from 5% to 25%.  A snowball's coupon is both its knock-out accrual and its maturity
    coupon, so every snowball is simulated; Phoenix notes of one term set differ only in
    their period coupon and form coupon families."""
    dt = years / steps
    per = steps // months
    times = [dt * (i + 1) for i in range(steps)]
    notes = []
    for phoenix in (False, True):
        for count in (6, 12, 18, 24):
            dates = [times[per * (m + 1) - 1] for m in range(count)]
            daily = times[:per * count]
            for ko in (100.0, 102.0, 103.0, 105.0):
                for ki in (70.0, 75.0, 80.0, 85.0):
                    for j in range(coupons):
                        coupon = 0.05 + 0.20 * j / max(coupons - 1, 1)
                        if phoenix:
                            obs = [Observation(t, ko, ki, 0.0) for t in dates]
                            note = AutocallableNote(
                                initial_spot=100.0, expiry=dates[-1], observations=obs,
                                knock_in_level=ki, knock_in_times=daily, upper_strike=100.0,
                                lower_strike=0.0, period_coupon=coupon / 12.0)
                        else:
                            obs = [Observation(t, ko, None, coupon) for t in dates]
                            note = AutocallableNote(
                                initial_spot=100.0, expiry=dates[-1], observations=obs,
                                knock_in_level=ki, knock_in_times=daily, upper_strike=100.0,
                                lower_strike=0.0, maturity_coupon_rate=coupon)
                        notes.append(note)
    return notes
