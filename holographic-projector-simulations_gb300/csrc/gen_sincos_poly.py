"""Fit the polynomials of the FMA-pipe sin/cos used by the split kernels.

Full turns (poly_sincos, poly_sincos2): for f in [-1/2, 1/2] turns
(theta = 2 pi f in [-pi, pi]),
    sin(2 pi f) ~ f * P(f^2),  P of degree 5  (odd terms f^1 .. f^11),
    cos(2 pi f) ~ Q(f^2),      Q of degree 6  (even terms f^0 .. f^12).
Half turns (poly_sincos2_half): for g in [-1/2, 1/2] half turns
(theta = pi g in [-pi/2, pi/2]; the caller applies (-1)^n),
    sin(pi g) ~ g * P(g^2),    P of degree 4  (odd terms g^1 .. g^9),
    cos(pi g) ~ Q(g^2),        Q of degree 4  (even terms g^0 .. g^8).
Each is fitted by iteratively reweighted least squares on Chebyshev nodes
(Lawson's algorithm, which converges to the minimax fit), in float64, then
rounded to float32.  Prints the coefficients (highest degree first, for Horner)
and the maximum absolute error of a float32 Horner evaluation over 2e6 points.
Run:  python gen_sincos_poly.py
"""
import numpy as np


def lawson(fun, basis, x, iters=200):
    w = np.ones_like(x) / x.size
    A = np.stack([b(x) for b in basis], axis=1)
    y = fun(x)
    for _ in range(iters):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(A * sw[:, None], y * sw, rcond=None)
        err = np.abs(A @ c - y)
        w = w * err
        w /= w.sum()
    return c, np.max(np.abs(A @ c - y))


def fit(scale, n_sin, n_cos, name):
    k = np.arange(1, 20001)
    f = 0.5 * np.cos((2 * k - 1) * np.pi / (2 * k.size))  # Chebyshev nodes on [-1/2, 1/2]
    f = f[f > 0]
    sin_basis = [lambda x, p=p: x ** (2 * p + 1) for p in range(n_sin)]
    cos_basis = [lambda x, p=p: x ** (2 * p) for p in range(n_cos)]
    cs, es = lawson(lambda x: np.sin(scale * x), sin_basis, f)
    cc, ec = lawson(lambda x: np.cos(scale * x), cos_basis, f)
    cs32 = cs.astype(np.float32)
    cc32 = cc.astype(np.float32)
    t = np.linspace(-0.5, 0.5, 2_000_001).astype(np.float32)
    t2 = (t * t).astype(np.float32)
    s = np.float32(cs32[-1])
    for c in cs32[-2::-1]:
        s = (s * t2 + c).astype(np.float32)
    s = (s * t).astype(np.float32)
    c_ = np.float32(cc32[-1])
    for c in cc32[-2::-1]:
        c_ = (c_ * t2 + c).astype(np.float32)
    td = t.astype(np.float64)
    print(f"{name}:")
    print(f"  sin coefficients x^{2 * n_sin - 1}..x^1:", ", ".join(f"{x:.9e}f" for x in cs32[::-1]))
    print(f"  cos coefficients x^{2 * n_cos - 2}..x^0:", ", ".join(f"{x:.9e}f" for x in cc32[::-1]))
    print(f"  fit error (float64): sin {es:.2e}, cos {ec:.2e}")
    print(f"  float32 Horner max abs error: sin {np.max(np.abs(s - np.sin(scale * td))):.2e}, "
          f"cos {np.max(np.abs(c_ - np.cos(scale * td))):.2e}")


def main():
    fit(2 * np.pi, 6, 7, "full turns (poly_sincos, poly_sincos2)")
    fit(np.pi, 5, 5, "half turns (poly_sincos2_half)")


if __name__ == "__main__":
    main()
