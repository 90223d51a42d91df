"""The gradient oracle (oracle/oracle_grad.hpp): the CPU oracle instantiated
on dual numbers with six partials, which restates the reference's
ForwardDiff gradient (every quantity carries d/dtheta; the k grids, the
Bessel grid's upper end and RECFAST's switch redshifts carry none, as
assume_nondual makes them in spectra.jl:46-66 and recfast.jl:451,456).

* The reference's own FD-vs-AD tests (test/runtests.jl:54-80):
  bg_fwddiff, d eta(-5) / d Omega_b on the x grid -20:0.1:0, and
  ih_fwddiff, d c_s^2(0) / d Omega_b through RECFAST at tol 1e-10, with the
  reference's assertion (central difference minus ForwardDiff, steps 1e-3,
  below 1e-5) and a sharper one: eta's central differences converge to the
  dual derivative (1e-8 relative at step 1e-5); c_s^2's stay 6e-4 away,
  because they move RECFAST's switch redshifts, which the dual derivative
  (like ForwardDiff's) holds fixed -- within 1e-3 relative.
* The dual values are the plain oracle's, bit for bit.
* P_lin and C_l^TT partials against central differences of the plain
  oracle at tight tolerances (relative steps 1e-5; frozen grids).
* At the differentiation configuration's sizes, the committed dual-oracle
  Jacobians (tests/golden/oracle_jac_*_dual.npz) against the committed
  central-difference Jacobians: every element above 1e-3 of its
  parameter's peak within 1e-3 relative.
"""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN

THETA0 = np.array([0.68, 0.0224, 0.119, 0.965, 2.1e-9, 0.1])


def _params(t):
    h = t[0]
    return O.Params(h=h, Omega_b=t[1] / h ** 2, Omega_c=t[2] / h ** 2, n=t[3], A=t[4], Sigma_m_nu_eV=t[5])


def _tight(t):
    return O.Cosmo(_params(t), recfast_tol=1e-11, recfast_atol=1e-12)


def test_bg_fwddiff():
    grid = (-20.0, 0.1, 0.0)
    d = O.DualCosmo(params=O.Params(), x_grid=grid, omega_b_only=True)
    ad = d.table("eta", [-5.0])[1][0, 0]

    def fbg(ob):
        return O.Cosmo(O.Params(Omega_b=ob), x_grid=grid).table("eta", np.array([-5.0]))[0]
    fd3 = (fbg(0.046 + 1e-3) - fbg(0.046 - 1e-3)) / 2e-3
    assert fd3 - ad < 1e-5  # runtests.jl:66
    fd5 = (fbg(0.046 + 1e-5) - fbg(0.046 - 1e-5)) / 2e-5
    assert abs(fd5 - ad) < 1e-8 * abs(ad)


def test_ih_fwddiff():
    grid = (-20.0, 0.1, 0.0)
    d = O.DualCosmo(params=O.Params(), x_grid=grid, omega_b_only=True, recfast_tol=1e-10)
    ad = d.table("csb2", [0.0])[1][0, 0]

    def fih(ob):
        return O.Cosmo(O.Params(Omega_b=ob), x_grid=grid, recfast_tol=1e-10).table("csb2", np.array([0.0]))[0]
    fd3 = (fih(0.046 + 1e-3) - fih(0.046 - 1e-3)) / 2e-3
    assert fd3 - ad < 1e-5  # runtests.jl:79
    fd5 = (fih(0.046 + 1e-5) - fih(0.046 - 1e-5)) / 2e-5
    assert abs(fd5 - ad) < 1e-3 * abs(ad)


@pytest.fixture(scope="module")
def pair():
    return O.DualCosmo(theta=THETA0, recfast_tol=1e-11, recfast_atol=1e-12), _tight(THETA0)


def test_dual_values_are_the_plain_oracle(pair):
    d, c = pair
    for nm in ("H", "eta", "taup", "g", "csb2", "Xe", "rho0M"):
        assert np.array_equal(d.table(nm, c.x)[0], c.table(nm)), nm
    assert d.eta0()[0] == c.eta0
    P, _ = d.plin(0.05, 15, 8, 8, 10, 0.0, 1e-8, 1e-8)
    assert P == c.plin(0.05, 15, 8, 8, 10, 0.0, 1e-8, 1e-8)


def _fd(f, j, step=1e-5):
    vals = []
    for sgn in (1.0, -1.0):
        t = THETA0.copy()
        t[j] += sgn * step * abs(THETA0[j])
        vals.append(f(t))
    return (vals[0] - vals[1]) / (2 * step * abs(THETA0[j]))


def test_dual_plin_partials_vs_central_differences(pair):
    d, _ = pair
    for k in (0.01, 0.2):
        _, dP = d.plin(k, 15, 8, 8, 10, 0.0, 1e-10, 1e-10)
        for j in range(6):
            fd = _fd(lambda t: _tight(t).plin(k, 15, 8, 8, 10, 0.0, 1e-10, 1e-10), j)
            assert abs(dP[j] - fd) < 1e-5 * abs(fd), (k, O.THETA_NAMES[j], dP[j], fd)


def test_dual_cltt_partials_vs_central_differences(pair):
    d, c0 = pair
    H0 = c0.H0
    ks = O.log10_k(0.1 * H0, 100 * H0, 8)
    ells = np.array([2, 20, 100], dtype=np.int32)
    kd = (0.01 * H0, 1000 * H0, 5000)
    am = kd[1] * c0.eta0
    tt, dtt = d.cltt(ks, ells, 8, 8, 10, 15, 1e-10, 1e-10, kd=kd, bessel_argmax=am)
    ST0, SE0, _ = c0.source_grid(ks, 8, 8, 10, 15, reltol=1e-10, abstol=1e-10)
    assert np.array_equal(tt, c0.cl(ST0, SE0, ks, ells, kd=kd, bessel_argmax=am)[0])

    def cl_of(t, j):
        c = _tight(t)
        S1, S2 = (ST0, SE0) if j in (3, 4) else c.source_grid(ks, 8, 8, 10, 15, reltol=1e-10, abstol=1e-10)[:2]
        return c.cl(S1, S2, ks, ells, kd=kd, bessel_argmax=am)[0]
    for j in range(6):
        fd = _fd(lambda t: cl_of(t, j), j)
        assert np.max(np.abs(dtt[j] - fd) / np.abs(fd)) < 1e-4, (O.THETA_NAMES[j], dtt[j], fd)


@pytest.mark.parametrize("name", ["oracle_jac_cltt", "oracle_jac_plin"])
def test_dual_jacobian_fixture_vs_central_difference_fixture(name):
    f = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = np.load(os.path.join(GOLDEN, name + "_dual.npz"))
    assert np.array_equal(f["theta"], g["theta"]) and np.array_equal(f["ks"], g["ks"])
    J, Jfd = g["J"], f["J_0.0001"]
    for j in range(6):
        big = np.abs(Jfd[j]) > 1e-3 * np.max(np.abs(Jfd[j]))
        rel = np.abs(J[j][big] - Jfd[j][big]) / np.abs(Jfd[j][big])
        assert np.max(rel) < 1e-3, (name, O.THETA_NAMES[j], np.max(rel))
