"""Fits the polynomials of the FP32 normal quantile used by the FP32 Sobol path.

For a lower-tail probability t in (0, 1/2], with x = 1 - 2t and w = -ln(4 t (1 - t)),
Phi^{-1}(t) = -sqrt(2) erfinv(x) = -sqrt(2) x p(w).  p is smooth in w; this script
fits p by least squares in two pieces (w < 5 in w - 2.5, w >= 5 in sqrt(w) - 3; the
change of variable follows M. Giles, "Approximating the erfinv function", GPU Computing
Gems Jade, 2011) against scipy.special.erfinv in float64, then checks the maximum
absolute error of the float32 evaluation over the whole 52-bit Sobol probability range.
Prints the coefficients (highest degree first) for device_rng.cuh.
"""
import numpy as np
from scipy.special import erfinv, ndtri

DEGREE = 8


def fit(lo, hi, transform, n=200000):
    w = np.concatenate([np.linspace(lo, hi, n), np.geomspace(max(lo, 1e-12), hi, n)])
    w = w[(w >= max(lo, 1e-12)) & (w <= hi)]
    # Truth from the lower-tail probability t, solved stably from 4 t (1 - t) = exp(-w).
    t = np.exp(-w) / (2.0 * (1.0 + np.sqrt(-np.expm1(-w))))
    x = 1.0 - 2.0 * t
    p = -ndtri(t) / (np.sqrt(2.0) * x)
    keep = np.isfinite(p) & (x > 0)
    w, p = w[keep], p[keep]
    v = transform(w)
    # least squares on relative error
    A = np.vander(v, DEGREE + 1)
    coef, *_ = np.linalg.lstsq(A / p[:, None], np.ones_like(p), rcond=None)
    return coef


def evaluate32(t, c1, c2):
    t = t.astype(np.float32)
    x = np.float32(1) - np.float32(2) * t
    w = -np.log(np.float32(4) * t * (np.float32(1) - t)).astype(np.float32)
    v1 = w - np.float32(2.5)
    v2 = np.sqrt(w) - np.float32(3.0)
    p1 = np.zeros_like(w)
    p2 = np.zeros_like(w)
    for a in c1:
        p1 = p1 * v1 + np.float32(a)
    for a in c2:
        p2 = p2 * v2 + np.float32(a)
    p = np.where(w < np.float32(5.0), p1, p2)
    return -np.float32(np.sqrt(2.0)) * x * p


def main():
    c1 = fit(0.0, 5.0, lambda w: w - 2.5)
    c2 = fit(5.0, 37.0, lambda w: np.sqrt(w) - 3.0)
    k = np.concatenate([np.arange(0, 4096), (2.0 ** np.linspace(12, 51, 200000)).astype(np.int64)])
    t = (k.astype(np.float64) + 0.5) / 2.0 ** 52
    t = t[t <= 0.5]
    ref = ndtri(t)
    got = evaluate32(t, c1, c2).astype(np.float64)
    err = np.abs(got - ref)
    print("max abs error", err.max(), "max rel error", (err / np.maximum(np.abs(ref), 1e-3)).max())
    for name, c in (("central", c1), ("tail", c2)):
        print(name, ", ".join(f"{float(a):.9e}f" for a in c))


if __name__ == "__main__":
    main()
