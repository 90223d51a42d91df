"""Pins the CPU oracle against the reference's own fixtures and known answers.

Reference tests restated (Bolt.jl test/runtests.jl):
  RECFAST Xe(z) vs Fortran RECFAST, 1e-4 absolute          (runtests.jl:38-48)
  Phi, delta_b at k = 0.03 h/Mpc vs CLASS, 1e-3 relative   (runtests.jl:83-147)
  C_l^TT, C_l^EE vs CAMB, 1.1e-1 relative                   (runtests.jl:149-185)
plus j_l(x) against mpmath, the exactness of the Jacobian split, and P_lin at
z = 0 against the CAMB linear P(k) in the reference's test data
(test/data/camb_pk_x0.dat, made by test/camb_v_class_2022.ipynb; the
reference compares the two by eye in scripts/first_plin.jl), 3e-3 relative.
"""
import os

import numpy as np
import pytest
from scipy.interpolate import CubicSpline

import oracle as O
from conftest import GOLDEN


@pytest.fixture(scope="module")
def nonu():
    return O.Cosmo(O.Params(Sigma_m_nu_eV=0.0))


def test_recfast_vs_fortran():
    g = np.load(os.path.join(GOLDEN, "recfast_fortran.npz"))
    p = O.Params(Sigma_m_nu_eV=0.0, N_nu=3.0, Omega_r=5.042e-5)
    xe = O.recfast_xe(p, g["z"], OmegaG=p.Omega_r, Tnow=2.725)
    assert np.all(np.abs(xe - g["xe"]) < 1e-4)


def test_sph_bessel_vs_mpmath():
    g = np.load(os.path.join(GOLDEN, "sph_bessel_mpmath.npz"))
    L = int(g["ell"].max())
    for j, x in enumerate(g["x"]):
        allj = O.sph_bessel_all(L, float(x))
        ref = g["j"][:, j]
        got = allj[g["ell"]]
        scale = np.maximum(np.abs(ref), 1e-280)
        big = np.abs(ref) > 1e-200
        assert np.all(np.abs(got - ref)[big] / scale[big] < 1e-11), (x, got, ref)


@pytest.mark.parametrize("k,x", [(1e-3, -15.0), (0.1, -7.0), (0.3, -1.0)])
def test_jacobian_split_is_exact(nonu, k, x):
    lg, lnu, lmnu, nq = 8, 8, 10, 15
    J = nonu.jacobian(k, x, lg, lnu, lmnu, nq)
    u = np.random.default_rng(0).standard_normal(J.shape[0])
    du, _ = nonu.rhs(k, u, x, lg, lnu, lmnu, nq)
    assert np.max(np.abs(J @ u - du)) <= 1e-13 * np.max(np.abs(du))


def test_rhs_x_derivative(nonu):
    lg, lnu, lmnu, nq = 8, 8, 10, 15
    u = np.random.default_rng(1).standard_normal(O.state_len(lg, lnu, lmnu, nq))
    k, x, h = 0.05, -7.3, 1e-6
    _, dx = nonu.rhs(k, u, x, lg, lnu, lmnu, nq)
    dp, _ = nonu.rhs(k, u, x + h, lg, lnu, lmnu, nq)
    dm, _ = nonu.rhs(k, u, x - h, lg, lnu, lmnu, nq)
    assert np.max(np.abs((dp - dm) / (2 * h) - dx)) < 1e-8 * np.max(np.abs(dx))


@pytest.mark.parametrize("kc,tol", [("p03", 1e-3), ("p01", 1e-4), ("p001", 1e-4)])
def test_perturbations_vs_class(nonu, kc, tol):
    g = np.load(os.path.join(GOLDEN, "class_nonu.npz"))
    k = 0.7 * float(g[f"{kc}_k_hMpc"][0])
    u, _ = nonu.boltsolve(k, nonu.x, 50, 50, 20, 15, reltol=1e-9, abstol=1e-9)
    iphi = u.shape[1] - 5
    cx = g[f"{kc}_x"][::-1]
    phib = CubicSpline(nonu.x, u[:, iphi], bc_type="natural")(cx)
    phic = CubicSpline(cx, g[f"{kc}_phi"][::-1], bc_type="natural")(cx)
    dbb = CubicSpline(nonu.x, u[:, iphi + 3], bc_type="natural")(cx)
    dbc = CubicSpline(cx, g[f"{kc}_d_b"][::-1], bc_type="natural")(cx)
    assert np.all(np.abs(phib / phic - 1) < tol)
    assert np.all(np.abs(-dbb / dbc - 1) < tol)


def test_cl_vs_camb():
    c = O.Cosmo(O.Params())
    kg = O.quadratic_k(0.1 * c.H0, 1000 * c.H0, 100)
    ST, SE, _ = c.source_grid(kg, 8, 8, 10, 15, reltol=1e-8, abstol=1e-6)
    ells = np.arange(10, 2501, 10)
    tt, te, ee = c.cl(ST, SE, kg, ells)
    g = np.load(os.path.join(GOLDEN, "camb_rough.npz"))
    fac = ells * (ells + 1) / (2 * np.pi)
    assert np.all(np.abs(fac * tt / np.interp(ells, g["ell"], g["tt"]) - 1) < 1.1e-1)
    assert np.all(np.abs(fac * ee / np.interp(ells, g["ell"], g["ee"]) - 1) < 1.1e-1)


def test_plin_vs_camb():
    """P_lin(k) at z = 0 against CAMB for the notebook's cosmology (Bolt's
    defaults with Omega_r 5.042e-5, n_s 1, ln(1e10 A_s) 3.043): within 0.1 %
    from 1e-3 to 0.5 h/Mpc, pinned at 3e-3."""
    from concurrent.futures import ThreadPoolExecutor
    g = np.load(os.path.join(GOLDEN, "camb_pk_x0.npz"))
    p = O.Params(Omega_r=5.042e-5, A=1e-10 * np.exp(3.043), n=1.0)
    c = O.Cosmo(p)
    # fixture nodes near 1e-3, 1e-2, 0.05, 0.2 and 0.5 h/Mpc (no interpolation across the BAO wiggles)
    idx = [int(np.argmin(np.abs(np.log(g["k_hMpc"] / t)))) for t in (1e-3, 1e-2, 0.05, 0.2, 0.5)]
    khs, camb = g["k_hMpc"][idx], g["pk"][idx]
    with ThreadPoolExecutor(len(khs)) as ex:
        P = np.array(list(ex.map(lambda kh: c.plin(kh * p.h, lg=50, lnu=50, lmnu=20, reltol=1e-8, abstol=1e-8),
                                 khs)))
    assert np.all(np.abs(P * p.h ** 3 / camb - 1) < 3e-3), P * p.h ** 3 / camb
