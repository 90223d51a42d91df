"""The discrete adjoint (bolt.jl_gb300/csrc/adjoint.cuh) on the GPU.

Its building blocks, through bolt_adjoint_check, on hierarchies from the
smallest to the reference plin default (N = 473) and nq = 27:
* the column form of hierarchy! (A^T, and dA/dx transposed) against the row
  form by the dot-product identity lam.(A u) = (A^T lam).u at the five
  stage abscissae of a step, 1e-13 relative, at every step tried (deep in
  the tightly coupled era, at recombination, late);
* the transposed solve against the forward solve by the same identity,
  lam.(M^-1 u) = (M^-T lam).u, 1e-13 at every step tried: the reverse sweep
  inverts exactly the matrix the forward step factorised;
* both solves against the step matrix M = I/(h gamma) - A itself, residual
  1e-10 of the right-hand side on moderately conditioned steps (the
  residual of a very stiff step with a large h, e.g. x = -18, h = 0.05,
  loses digits to cancellation in forming M x, whatever the solve);
* the source and P_lin gradients against the functions at nodes the line of
  sight reads: S_T is linear in (u, du), 1e-13; P_lin is quadratic in u, a
  central difference, 1e-9;
* the parameter cotangent from the coefficients' cotangents (one reverse
  pass over hierarchy!'s coefficients) against tangent-number arithmetic
  on pseudo-random coefficient tangents, 1e-12 of the terms' magnitude.
"""
import numpy as np
import pytest

import bolt_gb300 as B

pytestmark = pytest.mark.gpu

HIERS = [(3, 3, 3, 4), (8, 8, 10, 15), (20, 20, 10, 15), (50, 50, 20, 15), (20, 20, 10, 27)]


@pytest.fixture(scope="module")
def ih():
    par = B.CosmoParams(h=0.68, Omega_b=0.0224 / 0.68 ** 2, Omega_c=0.119 / 0.68 ** 2, n=0.965, A=2.1e-9,
                        Sigma_m_nu=0.1 * B.mass_natural())
    bg = B.Background(par)
    return B.IonizationHistory(B.RECFAST(bg, Yp=par.Y_p, OmegaB=par.Omega_b, OmegaG=par.Omega_r), par, bg)


@pytest.mark.parametrize("hier", HIERS)
@pytest.mark.parametrize("k,x,hs", [(0.002, -18.0, 0.05), (0.002, -18.0, 1e-4), (1.0, -1.0, 0.05)])
def test_adjoint_transposes_everywhere(ih, hier, k, x, hs):
    r = B.adjoint_check(ih, k, x, hs, *hier)
    assert r[10] == 0.0
    assert np.all(r[:6] < 1e-13), r[:6]
    assert r[11] < 1e-13, r[11]


@pytest.mark.parametrize("hier", HIERS)
@pytest.mark.parametrize("k,x,hs", [(0.05, -7.0, 0.01), (0.3, -6.9, 2e-3), (0.1, -3.0, 0.01), (1.0, -1.0, 1e-4)])
def test_adjoint_building_blocks(ih, hier, k, x, hs):
    r = B.adjoint_check(ih, k, x, hs, *hier)
    assert r[10] == 0.0
    assert np.all(r[:6] < 1e-13), r[:6]
    assert r[11] < 1e-13, r[11]
    assert r[6] < 1e-10 and r[7] < 1e-10, r[6:8]
    assert r[8] < 1e-13, r[8]
    assert r[9] < 1e-9, r[9]
    assert r[12] < 1e-12 and r[13] < 1e-12, r[12:14]


def _par(h=0.69, wb=0.02254, wc=0.10976, n=0.96, A=2.1e-9, mnu=0.11):
    return B.params_of(B.CosmoParams(), [h, wb, wc, n, A, mnu])


def test_adjoint_vjp_equals_tangent_jacobian_contraction():
    """The pullbacks by the discrete adjoint (engine grad_scheme "adjoint":
    a checkpointed forward solve, the adjoint of the line of sight, a
    reverse sweep) equal the cotangent contracted with the tangent-linear
    Jacobian: both differentiate the discrete pipeline with the same
    coefficient tangents, each on its own solve's steps (both land on every
    node; the checkpointed solve takes its step as the difference of the
    recorded abscissae, so its step sequence can part from the tangent
    solve's at rounding level: their C_l agree to 1e-9), so they agree to
    1e-7 of the largest term ybar_l |dC_l/dtheta_j| (measured: 3e-8 and
    below; n_s and A_s, which need no solve, to 1e-14)."""
    rng = np.random.default_rng(11)
    hier = (20, 20, 10, 15)
    par = _par()
    H0 = par.h * B.km_s_Mpc_100()
    ks = B.log10_k(0.1 * H0, 300 * H0, 40)
    ells = np.arange(2, 600, 13, dtype=np.int32)
    kp = B.log10_k(1e-3 * par.h, 0.5 * par.h, 16)
    ybc = rng.standard_normal(ells.size)
    ybp = rng.standard_normal(kp.size)
    with B.Engine(lanes=1, grad_scheme="tangent") as eng:
        c = eng.run(B.Request("cl", par, ks, hier=hier, ells=ells, cl=("tt",), grad=True))
        p = eng.run(B.Request("plin", par, kp, hier=hier, grad=True))
    assert c.rc == 0 and p.rc == 0, (c.err, p.err)
    with B.Engine(lanes=1, grad_scheme="adjoint") as eng:
        rc_, gc = eng.vjp(B.Request("cl", par, ks, hier=hier, ells=ells, cl=("tt",)), {"tt": ybc})
        rp_, gp = eng.vjp(B.Request("plin", par, kp, hier=hier), ybp)
    assert rc_.rc == 0 and rp_.rc == 0, (rc_.err, rp_.err)
    assert np.max(np.abs(rc_.cl["tt"] / c.cl["tt"] - 1)) < 1e-9
    assert np.max(np.abs(rp_.plin / p.plin - 1)) < 1e-9
    bad = []
    for what, g, J, yb in (("C_l^TT", gc, c.dcl["tt"], ybc), ("P_lin", gp, p.dplin, ybp)):
        want = J @ yb
        scale = np.max(np.abs(J * yb[None, :]), axis=1)
        err = np.abs(g - want) / scale
        if not np.all(err < 1e-7):
            bad.append((what, err.tolist(), g.tolist(), want.tolist()))
    assert not bad, bad
