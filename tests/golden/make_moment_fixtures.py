"""Known answers for moments of spherical Bessel functions at orders above
the reference's tests: I_m(x) = int_0^x t^m j_n(t) dt from its Maclaurin
series, sum_k (-1)^k x^(n+m+2k+1) / ((n+m+2k+1) 2^k k! (2n+2k+1)!!), summed
by mpmath in enough digits to absorb the alternating terms' cancellation.
Writes tests/golden/sph_moment_mpmath.npz.

    python tests/golden/make_moment_fixtures.py
"""
import os

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def moment(n, m, x):
    """The Maclaurin series of the moment summed exactly: working precision
    40 digits plus the ~0.44 x digits its alternating terms cancel."""
    mp.mp.dps = 40 + int(0.5 * float(x))
    n, m, x = int(n), mp.mpf(m), mp.mpf(x)
    a = n + m
    term = x ** (a + 1) / ((a + 1) * mp.fac2(2 * n + 1))
    s = term
    k = 0
    while True:
        k += 1
        term *= -x * x * (a + 2 * k - 1) / (2 * k * (a + 2 * k + 1) * (2 * n + 2 * k + 1))
        s += term
        if k > x and abs(term) < mp.mpf(10) ** (-45) * abs(s):
            return s


def main():
    cases = []
    for n in (7, 20, 60, 150):
        for m in (0, 1, 2, 3):
            for x in (0.5, 3.0, 0.6 * n, 1.0 * n, 1.7 * n, 4.5 * n + 10):
                cases.append((n, m, x))
    vals = []
    for n, m, x in cases:
        v = moment(n, m, x)
        vals.append(float(v) if abs(v) > mp.mpf("1e-300") else 0.0)
    c = np.array(cases, dtype=float)
    np.savez_compressed(os.path.join(HERE, "sph_moment_mpmath.npz"), n=c[:, 0].astype(int), m=c[:, 1], x=c[:, 2],
                        moment=np.array(vals))


if __name__ == "__main__":
    main()
