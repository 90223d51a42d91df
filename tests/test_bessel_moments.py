"""Moments of spherical Bessel functions, their interpolation table and the
Filon-type integrator (Bolt.jl src/bessel/): the oracle against the
reference's own known answers (test/testbessel.jl, read into
tests/golden/bessel_moment_refs.json by tests/golden/make_golden.py), at the
reference's tolerances: TOL = 1e-13 relative for moments (1e-15 where
testbessel.jl asks it), 1e-12 for table values, TOL on Filon integrals;
and, at orders 7-150 above the reference's tests, against the moments'
Maclaurin series summed exactly by mpmath
(tests/golden/make_moment_fixtures.py), 1e-12 relative.

Cylindrical moments int_0^x t^alpha J_nu(t) dt with nu = n + 1/2 (the
reference's J_moment_* tests) are sqrt(2/pi) times the spherical moment of
order alpha + 1/2.  Every method that the reference tests separately
(series, Lommel asymptotic, Weniger 1F2) is checked where the reference
checks it: "quad" stands where the reference uses the Weniger transform.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN

TOL = 1e-13  # testbessel.jl:4

with open(os.path.join(GOLDEN, "bessel_moment_refs.json")) as fh:
    REFS = {k: [float(v) for v in vs] for k, vs in json.load(fh).items()}


def rel(a, b):
    return abs(1.0 - a / b)


def test_bessel_J_moderate_argument():
    # testbessel.jl:8-33: x = 200, nu = 2.5, alpha = 0, 1, 2
    for alpha, ref in zip((0, 1, 2), REFS["moments: Bessel J, moderate argument"]):
        for meth in ("asymp", "quad", "auto"):
            assert rel(O.J_moment(200.0, 2.5, alpha, meth), ref) < TOL, (alpha, meth)


def test_bessel_J_small_argument():
    # testbessel.jl:36-48
    r = REFS["moments: Bessel J, small argument"]
    assert rel(O.J_moment(10.0, 2.5, 1.5, "quad"), r[0]) < 1e-15
    assert rel(O.J_moment(0.1, 2.5, -0.5, "quad"), r[1]) < TOL
    assert rel(O.J_moment(0.1, 2.5, -0.5, "maclaurin"), r[1]) < TOL


@pytest.mark.parametrize("nu,name", [(2, "quadrupole"), (3, "octupole")])
def test_spherical_large_argument(nu, name):
    # testbessel.jl:51-75 (quadrupole), 99-121 (octupole): x = 200, m = 0, 1, 2
    for m, ref in zip((0, 1, 2), REFS[f"moments: spherical Bessel J, large argument {name}"]):
        for meth in ("asymp", "quad", "auto"):
            assert rel(O.sph_j_moment(200.0, nu, m, meth), ref) < TOL, (m, meth)


def test_spherical_small_argument_quadrupole():
    # testbessel.jl:78-96
    r = REFS["moments: spherical Bessel J, small argument quadrupole"]
    for (x, m), ref in zip(((0.1, 1), (0.1, 0), (0.01, 2)), r):
        for meth in ("quad", "maclaurin", "auto"):
            assert rel(O.sph_j_moment(x, 2, m, meth), ref) < TOL, (x, m, meth)


def test_maclaurin_vanishing_argument_octupole():
    # testbessel.jl:124-151
    r = REFS["moments: maclaurin series vanishing argument octupole"]
    for i, (x, m) in enumerate([(0.01, 0), (0.01, 1), (0.01, 2), (0.001, 0), (0.001, 1), (0.001, 2)]):
        assert rel(O.sph_j_moment(x, 3, m, "maclaurin"), r[i]) < TOL, (x, m)


@pytest.fixture(scope="module")
def big_tables():
    # sph_bessel_interpolator(nu, order, 0.0, 1.6e4, 2_000_000), the reference's test tables
    return {(nu, order): O.MomentTable(nu, order, 0.0, 1.6e4, 2_000_000) for nu, order in ((2, 3), (3, 3), (3, 4))}


@pytest.mark.parametrize("nu,name", [(2, "quadrupole"), (3, "octupole")])
def test_interpolator_large_argument(big_tables, nu, name):
    # testbessel.jl:156-186
    moms = big_tables[(nu, 3)](200.0)
    for i, ref in enumerate(REFS[f"interpolator: spherical Bessel J, large argument {name}"]):
        assert rel(moms[i], ref) < 1e-12, i


def test_interpolator_small_argument_octupole(big_tables):
    # testbessel.jl:188-199
    moms = big_tables[(3, 3)](0.1)
    for i, ref in enumerate(REFS["interpolator: spherical Bessel J, small argument octupole"]):
        assert abs(moms[i] - ref) < 1e-12, i


def test_interpolator_fourth_order(big_tables):
    # testbessel.jl:202-245
    r = REFS["interpolator: spherical Bessel J, 4th order, moderate arg"]
    moms = big_tables[(3, 4)](1.0)
    assert np.max(np.abs(moms - r)) < 1e-12
    moms = O.MomentTable(3, 4, 2.0, 1.6e4, 20)(1.0)  # below the table: the series
    assert np.max(np.abs(moms - r)) < 1e-12
    r = REFS["interpolator: spherical Bessel J, 4th order, asymptotic arg"]
    moms = big_tables[(3, 4)](1000.0)
    assert np.max(np.abs(moms / r - 1)) < 1e-12
    moms = O.MomentTable(3, 4, 0.0, 500.0, 20)(1000.0)  # above the table: the Lommel form
    assert np.max(np.abs(moms / r - 1)) < 1e-12


def test_interpolator_maclaurin_vanishing_argument():
    # testbessel.jl:248-271: a table starting at 1.0 evaluated below it
    r = REFS["interpolator: maclaurin series vanishing argument octupole"]
    itp = O.MomentTable(3, 3, 1.0, 1.6e4, 2_000)
    assert np.max(np.abs(itp(0.01) / r[:3] - 1)) < TOL
    assert np.max(np.abs(itp(0.001) / r[3:] - 1)) < TOL


def test_filon(big_tables):
    # testbessel.jl:274-304
    r = REFS["3rd order filon integration using the interpolator"]
    itp = big_tables[(3, 3)]
    cases = [(4.0, -0.2, 6.0, 10.0, 0.0, 2.0), (4.0, -0.2, 6.0, 10.0, 0.0, 1.0), (6.8, 5.8, 6.0, 10.0, 1.0, 2.0),
             (15.6, 11.8, 6.0, 10.0, 2.0, 4.0)]
    for c, ref in zip(cases, r[:4]):
        assert abs(itp.filon(*c) - ref) < TOL, c
    # the piecewise form over [1, 2] alone
    assert abs(itp.filon_piecewise([1.0, 2.0], [6.8, 0.0], [5.8, 0.0], [6.0, 0.0], 10.0)[0] - r[2]) < TOL
    itp = O.MomentTable(3, 3, 2.0, 50.0, 20)  # series below, Lommel form above
    cases = [(3.9983, -0.14, 6.0, 10.0, 0.01, 0.02), (3999803 / 1000000, -(97 / 500), 6.0, 10.0, 0.001, 0.002),
             (7494.0, 299.8, 6.0, 10.0, 50.0, 100.0), (119964.0, 1199.8, 6.0, 10.0, 200.0, 201.0),
             (74999004.0, 149999 / 5, 6.0, 10.0, 5000.0, 5100.0)]
    for c, ref in zip(cases, r[4:]):
        assert rel(itp.filon(*c), ref) < TOL, c


def test_filon_piecewise_converges_to_the_integral():
    """The piecewise Filon sum of a smooth f(t) j_3(k t), with the local
    quadratic's derivatives exact, against a direct quadrature."""
    mp = pytest.importorskip("mpmath")
    itp = O.MomentTable(3, 3, 0.0, 400.0, 50_001)
    t = np.linspace(0.0, 20.0, 401)
    f = np.exp(-t / 7.0) * (1 + t)
    fp = np.exp(-t / 7.0) * (1 - (1 + t) / 7.0)
    fpp = np.exp(-t / 7.0) * (-2.0 / 7.0 + (1 + t) / 49.0)
    ks = np.array([0.5, 3.0, 17.0])
    got = itp.filon_piecewise(t, f, fp, fpp, ks)
    mp.mp.dps = 30
    for k, g in zip(ks, got):
        ref = mp.quad(lambda s: mp.exp(-s / 7) * (1 + s) * mp.sqrt(mp.pi / (2 * k * s)) *
                      mp.besselj(3.5, k * s), mp.linspace(0, 20, 60))
        # a quadratic per segment of width 0.05: error ~ h^3 f''' / 24 per unit length
        assert abs(g - float(ref)) < 2e-6 * 20, (k, g, float(ref))


def test_high_order_moments_vs_exact_series():
    d = np.load(os.path.join(GOLDEN, "sph_moment_mpmath.npz"))
    got = np.array([O.sph_j_moment(x, int(n), m) for n, m, x in zip(d["n"], d["m"], d["x"])])
    ref = d["moment"]
    big = ref != 0.0
    assert np.max(np.abs(got[big] / ref[big] - 1)) < 1e-12
