"""Derivation of the FP32 arccos coefficients used for the bending angle (acosBend in
genesis_tissue_simulation_gb300/csrc/tissue_device.cuh and oracle/xpbd_oracle.cpp).

asin x = x + x z P(z), z = x^2, on |x| <= 1/2 (the half-angle reduction covers the rest of [-1, 1]);
P of degree 5 is the weighted least-squares fit of (asin x - x)/(x z) on 4000 Chebyshev nodes of
[0, 1/4] (weight z: the error of x z P relative to asin x), rounded to FP32.  Running this script
prints the coefficients and the largest error of the FP32 evaluation against the float64 arccos over
a dense sample of [-1, 1] (the kernels' sequence of correctly rounded FP32 operations, evaluated with
numpy float32 arithmetic).
"""
import numpy as np

f32 = np.float32


def fit(degree=5, nodes=4000):
    k = np.arange(nodes)
    z = 0.125 * (1 - np.cos(np.pi * (k + 0.5) / nodes))
    x = np.sqrt(z)
    f = (np.arcsin(x) - x) / (x * z)
    w = np.maximum(z, 1e-3)
    coef, *_ = np.linalg.lstsq(np.vander(z, degree + 1, increasing=True) * w[:, None], f * w, rcond=None)
    return coef.astype(np.float32)


def acos_bend(c, coef):
    c = np.asarray(c, dtype=np.float32)
    a = np.abs(c)
    mid = a <= f32(0.5)
    z = np.where(mid, c * c, (f32(1) - a) * f32(0.5)).astype(np.float32)
    x = np.where(mid, c, np.sqrt(z)).astype(np.float32)
    p = coef[-1]
    for q in coef[-2::-1]:
        p = (p * z + q).astype(np.float32)
    asinx = (x + x * (z * p)).astype(np.float32)
    pio2_hi, pio2_lo = f32(np.pi / 2), f32(np.pi / 2 - float(f32(np.pi / 2)))
    pi_hi, pi_lo = f32(np.pi), f32(np.pi - float(f32(np.pi)))
    return np.where(mid, pio2_hi - (asinx - pio2_lo),
                    np.where(c > 0, f32(2) * asinx, pi_hi - (f32(2) * asinx - pi_lo))).astype(np.float32)


def max_ulp(coef, samples=4_000_000, seed=0):
    rng = np.random.default_rng(seed)
    xs = np.concatenate([rng.uniform(-1, 1, samples), 1 - rng.uniform(0, 1e-3, samples // 4),
                         -1 + rng.uniform(0, 1e-3, samples // 4), 0.5 + rng.uniform(-1e-3, 1e-3, samples // 4),
                         -0.5 + rng.uniform(-1e-3, 1e-3, samples // 4)]).astype(np.float32)
    exact = np.arccos(xs.astype(np.float64))
    got = acos_bend(xs, coef).astype(np.float64)
    return float((np.abs(got - exact) / np.spacing(np.abs(exact.astype(np.float32))).astype(np.float64)).max())


if __name__ == "__main__":
    coef = fit()
    print("P coefficients (z^0 .. z^5):", [repr(float(c)) for c in coef])
    print("max error: %.3f ulp" % max_ulp(coef))
