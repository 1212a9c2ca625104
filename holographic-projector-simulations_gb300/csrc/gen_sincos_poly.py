"""Fit the polynomials of the FMA-pipe sin/cos used by the split kernel.

Method: for f in [-1/2, 1/2] turns (theta = 2 pi f in [-pi, pi]),
    sin(2 pi f) ~ f * P(f^2),  P of degree 5  (odd terms f^1 .. f^11),
    cos(2 pi f) ~ Q(f^2),      Q of degree 6  (even terms f^0 .. f^12),
fitted by iteratively reweighted least squares on Chebyshev nodes (Lawson's
algorithm, which converges to the minimax fit), in float64, then rounded to
float32.  Prints the coefficients (highest degree first, for Horner) and the
maximum absolute error of a float32 Horner evaluation over 2e6 points.
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


def main():
    k = np.arange(1, 20001)
    f = 0.5 * np.cos((2 * k - 1) * np.pi / (2 * k.size))  # Chebyshev nodes on [-1/2, 1/2]
    f = f[f > 0]
    sin_basis = [lambda x, p=p: x ** (2 * p + 1) for p in range(6)]
    cos_basis = [lambda x, p=p: x ** (2 * p) for p in range(7)]
    cs, es = lawson(lambda x: np.sin(2 * np.pi * x), sin_basis, f)
    cc, ec = lawson(lambda x: np.cos(2 * np.pi * x), cos_basis, f)
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
    print("sin coefficients f^11..f^1:", ", ".join(f"{x:.9e}f" for x in cs32[::-1]))
    print("cos coefficients f^12..f^0:", ", ".join(f"{x:.9e}f" for x in cc32[::-1]))
    print(f"fit error (float64): sin {es:.2e}, cos {ec:.2e}")
    print(f"float32 Horner max abs error: sin {np.max(np.abs(s - np.sin(2*np.pi*td))):.2e}, "
          f"cos {np.max(np.abs(c_ - np.cos(2*np.pi*td))):.2e}")


if __name__ == "__main__":
    main()
