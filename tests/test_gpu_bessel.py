"""GPU parity of the Bessel-moment path (Bolt.jl src/bessel/) through the C
ABI: the device moments, tables and Filon integrals against the reference's
known answers (test/testbessel.jl via tests/golden/bessel_moment_refs.json)
at the reference's tolerances, and against the CPU oracle on seeded random
arguments (1e-12 relative where the values are not cancellation-limited),
including orders far above the reference's tests, tables whose nodes
straddle the switch from quadrature to the Lommel form, short tables (the
end-sweep-only prefilter) and the error paths.
"""
import json
import os

import numpy as np
import pytest

import bolt_gb300 as B
import oracle as O
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-13  # testbessel.jl:4

with open(os.path.join(GOLDEN, "bessel_moment_refs.json")) as fh:
    REFS = {k: [float(v) for v in vs] for k, vs in json.load(fh).items()}


def rel(a, b):
    return np.abs(1.0 - np.asarray(a) / np.asarray(b))


@pytest.fixture(scope="module")
def big():
    # sph_bessel_interpolator(nu, order, 0.0, 1.6e4, 2_000_000), the reference's test tables
    return {k: B.MomentTable(k[0], k[1], 0.0, 1.6e4, 2_000_000) for k in ((2, 3), (3, 3), (3, 4))}


def test_direct_moments_known_answers():
    for alpha, ref in zip((0, 1, 2), REFS["moments: Bessel J, moderate argument"]):
        assert rel(B.J_moment(200.0, 2.5, alpha), ref) < TOL  # testbessel.jl:8-33
    r = REFS["moments: Bessel J, small argument"]  # testbessel.jl:36-48
    assert rel(B.J_moment(10.0, 2.5, 1.5), r[0]) < 1e-15
    assert rel(B.J_moment(0.1, 2.5, -0.5), r[1]) < TOL
    for nu, name in ((2, "quadrupole"), (3, "octupole")):  # testbessel.jl:51-75, 99-121
        got = np.array([B.sph_j_moment(200.0, nu, m) for m in (0, 1, 2)])
        assert np.all(rel(got, REFS[f"moments: spherical Bessel J, large argument {name}"]) < TOL)
    r = REFS["moments: spherical Bessel J, small argument quadrupole"]  # testbessel.jl:78-96
    for (x, m), ref in zip(((0.1, 1), (0.1, 0), (0.01, 2)), r):
        assert rel(B.sph_j_moment(x, 2, m), ref) < TOL
    r = REFS["moments: maclaurin series vanishing argument octupole"]  # testbessel.jl:124-151
    got = [B.sph_j_moment(x, 3, m) for x in (0.01, 0.001) for m in (0, 1, 2)]
    assert np.all(rel(got, r) < TOL)


def test_high_order_moments_vs_exact_series():
    """Orders 7-150 against the Maclaurin series summed exactly (fixture),
    1e-12 relative, through the series, quadrature and Lommel ranges."""
    d = np.load(os.path.join(GOLDEN, "sph_moment_mpmath.npz"))
    for n in np.unique(d["n"]):
        for m in np.unique(d["m"]):
            sel = (d["n"] == n) & (d["m"] == m)
            got = B.sph_j_moment(d["x"][sel], int(n), float(m))
            ref = d["moment"][sel]
            big = ref != 0.0
            assert np.max(np.abs(got[big] / ref[big] - 1)) < 1e-12, (n, m)


def test_direct_moments_vs_oracle():
    rng = np.random.default_rng(7)
    for nu in (0, 1, 2, 5, 40, 300):
        for m in (0.0, 1.0, 2.0, 3.0, 0.5, 2.5):
            x = np.concatenate([rng.uniform(0, 3, 6), rng.uniform(3, 60, 6), rng.uniform(60, 5 * nu + 400, 6)])
            got = B.sph_j_moment(x, nu, m)
            ref = np.array([O.sph_j_moment(v, nu, m) for v in x])
            big = np.abs(ref) > 1e-280
            assert np.max(rel(got[big], ref[big])) < 1e-12, (nu, m)


@pytest.mark.parametrize("nu,name", [(2, "quadrupole"), (3, "octupole")])
def test_table_known_answers_large_argument(big, nu, name):
    assert np.all(rel(big[(nu, 3)](200.0), REFS[f"interpolator: spherical Bessel J, large argument {name}"]) < 1e-12)


def test_table_known_answers(big):
    r = REFS["interpolator: spherical Bessel J, small argument octupole"]  # testbessel.jl:188-199
    assert np.max(np.abs(big[(3, 3)](0.1) - r)) < 1e-12
    r = REFS["interpolator: spherical Bessel J, 4th order, moderate arg"]  # testbessel.jl:202-223
    assert np.max(np.abs(big[(3, 4)](1.0) - r)) < 1e-12
    assert np.max(np.abs(B.MomentTable(3, 4, 2.0, 1.6e4, 20)(1.0) - r)) < 1e-12
    r = REFS["interpolator: spherical Bessel J, 4th order, asymptotic arg"]  # testbessel.jl:226-245
    assert np.max(rel(big[(3, 4)](1000.0), r)) < 1e-12
    assert np.max(rel(B.MomentTable(3, 4, 0.0, 500.0, 20)(1000.0), r)) < 1e-12
    r = REFS["interpolator: maclaurin series vanishing argument octupole"]  # testbessel.jl:248-271
    itp = B.MomentTable(3, 3, 1.0, 1.6e4, 2_000)
    assert np.max(rel(itp(0.01), r[:3])) < TOL
    assert np.max(rel(itp(0.001), r[3:])) < TOL


def test_filon_known_answers(big):
    r = REFS["3rd order filon integration using the interpolator"]  # testbessel.jl:274-304
    itp = big[(3, 3)]
    cases = np.array([(4.0, -0.2, 6.0, 10.0, 0.0, 2.0), (4.0, -0.2, 6.0, 10.0, 0.0, 1.0),
                      (6.8, 5.8, 6.0, 10.0, 1.0, 2.0), (15.6, 11.8, 6.0, 10.0, 2.0, 4.0)])
    got = B.integrate_sph_bessel_filon(*cases.T, itp)
    assert np.max(np.abs(got - r[:4])) < TOL
    pw = B.integrate_sph_bessel_filon_piecewise([1.0, 2.0], [6.8, 0.0], [5.8, 0.0], [6.0, 0.0], 10.0, itp)
    assert abs(pw - r[2]) < TOL
    itp = B.MomentTable(3, 3, 2.0, 50.0, 20)
    cases = np.array([(3.9983, -0.14, 6.0, 10.0, 0.01, 0.02), (3999803 / 1000000, -(97 / 500), 6.0, 10.0, 0.001, 0.002),
                      (7494.0, 299.8, 6.0, 10.0, 50.0, 100.0), (119964.0, 1199.8, 6.0, 10.0, 200.0, 201.0),
                      (74999004.0, 149999 / 5, 6.0, 10.0, 5000.0, 5100.0)])
    got = B.integrate_sph_bessel_filon(*cases.T, itp)
    assert np.max(rel(got, r[4:])) < TOL


@pytest.mark.parametrize("nu,order,kmin,kmax,N", [(3, 3, 0.0, 1.6e4, 2_000_000), (40, 4, 0.0, 2000.0, 200_001),
                                                  (300, 3, 0.0, 3000.0, 300_001), (2, 3, 5.0, 60.0, 67),
                                                  (2, 2, 5.0, 60.0, 68), (7, 1, 0.5, 9.0, 2), (3, 4, 45.0, 55.0, 1001)])
def test_table_vs_oracle(nu, order, kmin, kmax, N):
    """Nodes below the cut (compensated prefix sums of interval integrals),
    above it (Lommel form) and across it; short tables (N < 68) solve the
    whole prefilter by the end sweep."""
    d = B.MomentTable(nu, order, kmin, kmax, N)
    o = O.MomentTable(nu, order, kmin, kmax, N)
    rng = np.random.default_rng(nu * 1000 + N % 997)
    # above the table the Lommel form holds where the expansion converges (x >= max(50, 4 nu))
    above = rng.uniform(kmax, 3 * kmax, 20) if kmax >= max(50.0, 4.0 * nu) else []
    x = np.concatenate([rng.uniform(kmin, kmax, 4000), np.linspace(kmin, kmax, 50), [kmin, kmax],
                        rng.uniform(0, kmin, 20) if kmin > 0 else [], above])
    a, b = d(x), o(x)
    # 1e-12 relative, or 1e-14 of the order's largest value where the moment is a
    # cancellation of larger terms (x^m j_nu(x) against the constant)
    assert np.all(np.abs(a - b) <= 1e-12 * np.abs(b) + 1e-14 * np.max(np.abs(b), axis=0))
    d.close()


def test_filon_piecewise_vs_oracle():
    itp = B.MomentTable(3, 3, 0.0, 400.0, 50_001)
    oitp = O.MomentTable(3, 3, 0.0, 400.0, 50_001)
    t = np.linspace(0.0, 20.0, 4001)
    f = np.exp(-t / 7.0) * (1 + t)
    fp = np.exp(-t / 7.0) * (1 - (1 + t) / 7.0)
    fpp = np.exp(-t / 7.0) * (-2.0 / 7.0 + (1 + t) / 49.0)
    ks = np.geomspace(0.05, 19.0, 300)
    got = B.integrate_sph_bessel_filon_piecewise(t, f, fp, fpp, ks, itp)
    ref = oitp.filon_piecewise(t, f, fp, fpp, ks)
    assert np.max(np.abs(got - ref)) < 1e-11 * np.max(np.abs(ref))
    # per segment, the same sum
    seg = B.integrate_sph_bessel_filon(f[:-1], fp[:-1], fpp[:-1], ks[17], t[:-1], t[1:], itp)
    assert abs(np.sum(seg) - got[17]) < 1e-11 * np.max(np.abs(ref))
    # beyond the table (k t > 400): the Lommel form takes over
    got2 = B.integrate_sph_bessel_filon_piecewise(t, f, fp, fpp, [30.0, 45.0], itp)
    assert np.max(np.abs(got2 - oitp.filon_piecewise(t, f, fp, fpp, [30.0, 45.0]))) < 1e-11 * np.max(np.abs(ref))


def test_filon_batched_vs_oracle():
    """One integrand per k (the line-of-sight shape) against the oracle's
    piecewise sum with that k's integrand; a k whose integrand is the shared
    one reproduces the piecewise entry point."""
    itp = B.MomentTable(3, 3, 0.0, 400.0, 50_001)
    oitp = O.MomentTable(3, 3, 0.0, 400.0, 50_001)
    t = np.linspace(0.0, 20.0, 801)
    ks = np.geomspace(0.05, 19.0, 64)
    rng = np.random.default_rng(11)
    w = rng.uniform(3.0, 9.0, ks.size)[:, None]
    ph = rng.uniform(0.0, 1.0, ks.size)[:, None]
    e = np.exp(-t / w)
    f = e * (1 + t + ph)
    fp = e * (1 - (1 + t + ph) / w)
    fpp = e * (-2.0 / w + (1 + t + ph) / w ** 2)
    got = B.integrate_sph_bessel_filon_batched(t, f, fp, fpp, ks, itp)
    ref = np.array([oitp.filon_piecewise(t, f[j], fp[j], fpp[j], [ks[j]])[0] for j in range(ks.size)])
    assert np.max(np.abs(got - ref)) < 1e-11 * np.max(np.abs(ref))
    one = B.integrate_sph_bessel_filon_batched(t, f[5], fp[5], fpp[5], ks, itp)
    pw = B.integrate_sph_bessel_filon_piecewise(t, f[5], fp[5], fpp[5], ks, itp)
    assert np.max(np.abs(one - pw)) < 1e-12 * np.max(np.abs(pw))


def test_errors():
    with pytest.raises(B.BoltError):
        B.MomentTable(3, 5, 0.0, 10.0, 100)
    with pytest.raises(B.BoltError):
        B.MomentTable(3, 3, 0.0, 10.0, 1)
    with pytest.raises(B.BoltError):
        B.MomentTable(3, 3, 10.0, 10.0, 100)
    with pytest.raises(B.BoltError):
        B.MomentTable(-1, 3, 0.0, 10.0, 100)
    with pytest.raises(B.BoltError):
        B.sph_j_moment(-1.0, 2, 0)
    with pytest.raises(B.BoltError):
        B.sph_j_moment(1.0, 2, -3.5)
    itp = B.MomentTable(3, 2, 0.0, 10.0, 100)
    with pytest.raises(B.BoltError):
        B.integrate_sph_bessel_filon(1.0, 0.0, 0.0, 1.0, 0.0, 1.0, itp)  # order 2 < 3
    itp3 = B.MomentTable(3, 3, 0.0, 10.0, 100)
    with pytest.raises(B.BoltError):
        B.integrate_sph_bessel_filon(1.0, 0.0, 0.0, 0.0, 0.0, 1.0, itp3)  # k = 0
    itp.close()
    with pytest.raises(B.BoltError):
        itp(1.0)  # freed
    assert B.integrate_sph_bessel_filon_piecewise([1.0], [1.0], [0.0], [0.0], [2.0], itp3)[0] == 0.0
