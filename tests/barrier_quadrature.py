"""Independent values of discretely monitored barriers for the tests: the surviving
density of x = log(S / S0) is propagated across the observation dates on a grid with
the trapezoid rule. The vanilla from the last observation is priced with the analytic
BSM formula. Knock-ins are valued by in/out parity."""
import math

import numpy as np

from kiyosi_gb300 import analytic
from kiyosi_gb300.market import BlackScholesMertonParameters, PricingContext


def scheduled_barrier_value(ctx, sign, strike, expiry, dates, lower=None, upper=None,
                            knock_in=False, rebate=0.0, at_hit=False, nodes=2001):
    """Price of a barrier observed on `dates` (years, > 0), knocked out (or in) when the
    spot is at or below `lower` or at or above `upper` on a date; the rebate is paid at
    the hit date (`at_hit`) or at expiry."""
    m = ctx.model
    r, q, sigma, spot = m.rate, m.dividend, m.volatility, ctx.spot
    drift = r - q - 0.5 * sigma * sigma
    span = 8.0 * sigma * math.sqrt(expiry) + abs(drift) * expiry
    lo = math.log(lower / spot) if lower is not None else -span
    hi = math.log(upper / spot) if upper is not None else span
    x = np.linspace(lo, hi, nodes)
    w = np.full(nodes, x[1] - x[0])
    w[0] = w[-1] = 0.5 * (x[1] - x[0])
    density = None
    previous, survive, hit_value = 0.0, 1.0, 0.0
    for t in dates:
        dt = t - previous
        s = sigma * math.sqrt(dt)
        if density is None:
            density = np.exp(-0.5 * ((x - drift * dt) / s) ** 2) / (s * math.sqrt(2 * math.pi))
        else:
            kernel = np.exp(-0.5 * ((x[:, None] - x[None, :] - drift * dt) / s) ** 2) / (
                s * math.sqrt(2 * math.pi))
            density = kernel @ (density * w)
        now = float(np.sum(density * w))
        hit_value += rebate * math.exp(-r * t) * (survive - now)
        survive = now
        previous = t
    last = dates[-1]
    tau = expiry - last
    if tau > 0.0:
        unit = PricingContext(BlackScholesMertonParameters(r, q, sigma), 1.0)
        inner = np.array([analytic.european_price(sign, strike / (spot * math.exp(v)), tau, unit)
                          * spot * math.exp(v) for v in x])
    else:
        inner = np.maximum(sign * (spot * np.exp(x) - strike), 0.0)
    knock_out = math.exp(-r * last) * float(np.sum(density * w * inner))
    if not knock_in:
        return knock_out + (hit_value if at_hit else rebate * math.exp(-r * expiry) * (1.0 - survive))
    vanilla = analytic.european_price(sign, strike, expiry, ctx)
    return vanilla - knock_out + rebate * math.exp(-r * expiry) * survive
