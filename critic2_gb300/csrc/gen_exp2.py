"""Coefficients of exp2_poly in k_tc.cu: 2^r = 1 + r q(r) on |r| <= 0.501.

q (degree 6) is a weighted least-squares fit of (2^r - 1)/r on 400
Chebyshev nodes, weights 2^-r so that the fit minimises the relative error
of 1 + r q(r).  Prints the FP32 coefficients (constant term first) and the
relative error of the FP32-coefficient polynomial in exact arithmetic.
"""
import numpy as np


def main(deg: int = 6, half: float = 0.501, nodes: int = 400):
    k = np.arange(nodes)
    r = half * np.cos(np.pi * (k + 0.5) / nodes)
    V = np.vander(r, deg + 1, increasing=True) * r[:, None]
    w = np.exp2(-r)
    c, *_ = np.linalg.lstsq(V * w[:, None], (np.exp2(r) - 1) * w, rcond=None)
    c32 = c.astype(np.float32)
    rr = np.linspace(-half, half, 200001)
    err = np.abs((1 + rr * np.polyval(c32.astype(np.float64)[::-1], rr)) / np.exp2(rr) - 1).max()
    for v in c32:
        print(repr(float(v)))
    print(f"max relative error {err:.3e}")


if __name__ == "__main__":
    main()
