"""The batching / serving engine (bolt_engine_*) against the drop-in entry
points and the oracle.

* A C_l request and a P_lin request give the drop-in results
  (bolt_cl_pipeline, bolt_plin on the same host-built tables).
* Requests give the same result alone (one request per batch) and in a mix
  submitted together (batched, several lanes in flight).
* Gradients (forward differences of the frozen-step pipeline; the C_l^TT
  part from the tangent of the LOS integral) agree with
  central finite differences of the oracle (tight tolerances, the k grids and
  the Bessel grid of the unperturbed cosmology held fixed as the reference's
  assume_nondual does) within 1e-3.
"""
import numpy as np
import pytest

import bolt_gb300 as B

pytestmark = pytest.mark.gpu

HIER = (20, 20, 10, 15)


def _par(h=0.7, wb=0.02254, wc=0.10976, n=0.96, A=2.1e-9, mnu=0.06):
    return B.params_of(B.CosmoParams(), [h, wb, wc, n, A, mnu])


def _ks(par, nk=60, kmax_h0=600.0):
    H0 = par.h * B.km_s_Mpc_100()
    return B.log10_k(0.1 * H0, kmax_h0 * H0, nk)


def _dropin_cl(par, ks, ells):
    bg = B.Background(par)
    ih = B.IonizationHistory(B.RECFAST(bg, Yp=par.Y_p, OmegaB=par.Omega_b, OmegaG=par.Omega_r), par, bg)
    tt, te, ee, st = B.cl_all(ells, ih, ks, *HIER, reltol=1e-8, abstol=3e-7)
    ih.close()
    return tt, te, ee


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b))


def test_cl_request_matches_dropin():
    par = _par()
    ks = _ks(par)
    ells = np.arange(2, 801, 7, dtype=np.int32)
    with B.Engine(lanes=1) as eng:
        r = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt", "te", "ee")))
    assert r.rc == 0, r.err
    tt, te, ee = _dropin_cl(par, ks, ells)
    assert _rel(r.cl["tt"], tt) < 1e-9
    assert _rel(r.cl["te"], te) < 1e-9
    assert _rel(r.cl["ee"], ee) < 1e-9


def test_plin_request_matches_dropin():
    par = _par(h=0.68, mnu=0.1)
    H0 = par.h * B.km_s_Mpc_100()
    ks = B.log10_k(1e-4 * par.h, 1.0 * par.h, 40)
    with B.Engine(lanes=1) as eng:
        r = eng.run(B.Request("plin", par, ks, hier=HIER))
    assert r.rc == 0, r.err
    bg = B.Background(par)
    ih = B.IonizationHistory(B.RECFAST(bg, Yp=par.Y_p, OmegaB=par.Omega_b, OmegaG=par.Omega_r), par, bg)
    P = B.plin(ks, par, bg, ih, n_q=15, lg=HIER[0], lnu=HIER[1], lmnu=HIER[2], reltol=1e-8, abstol=3e-7)
    ih.close()
    assert _rel(r.plin, P) < 1e-9
    del H0


def _mix():
    rng = np.random.default_rng(7)
    reqs = []
    for i in range(6):
        par = _par(h=rng.uniform(0.62, 0.78), wb=rng.uniform(0.019, 0.025), wc=rng.uniform(0.10, 0.14),
                   n=rng.uniform(0.92, 1.0), A=np.exp(rng.uniform(2.9, 3.2)) / 1e10, mnu=rng.uniform(0.0, 0.3))
        if i % 2 == 0:
            ells = np.arange(2, 400, 11, dtype=np.int32)
            reqs.append(B.Request("cl", par, _ks(par, nk=int(rng.integers(40, 80))), hier=HIER, ells=ells,
                                  cl=("tt", "ee")))
        else:
            ks = B.log10_k(1e-4 * par.h, par.h, int(rng.integers(20, 50)))
            reqs.append(B.Request("plin", par, ks, hier=HIER))
    return reqs


def test_alone_equals_mixed():
    reqs = _mix()
    with B.Engine(lanes=1, max_batch=1) as eng:
        alone = [eng.run(q) for q in reqs]
    with B.Engine(lanes=3) as eng:
        tickets = [eng.submit(q) for q in reqs]
        mixed = [eng.wait(t) for t in tickets]
        st = eng.stats()
    assert st["requests"] == len(reqs)
    for q, a, m in zip(reqs, alone, mixed):
        assert a.rc == 0 and m.rc == 0, (a.err, m.err)
        if q.kind == "plin":
            assert _rel(m.plin, a.plin) < 1e-9
        else:
            for c in q.cl:
                assert _rel(m.cl[c], a.cl[c]) < 1e-9


def _oracle_cl_fd(par, ks, ells, rel_step, j):
    """Central difference of the oracle's C_l^TT in theta_j, frozen grids."""
    import oracle as O
    th = B.theta_of(par)
    H0 = par.h * B.km_s_Mpc_100()
    kd = (0.01 * H0, 1000.0 * H0, 5000)
    c0 = O.Cosmo(O.Params(h=par.h, Omega_b=par.Omega_b, Omega_c=par.Omega_c, n=par.n, A=par.A,
                          Sigma_m_nu_eV=th[5]))
    argmax = kd[1] * c0.eta0
    out = []
    for sgn in (1.0, -1.0):
        t = th.copy()
        t[j] += sgn * rel_step * abs(th[j])
        p = B.params_of(par, t)
        c = O.Cosmo(O.Params(h=p.h, Omega_b=p.Omega_b, Omega_c=p.Omega_c, n=p.n, A=p.A, Sigma_m_nu_eV=t[5]),
                    recfast_tol=1e-11, recfast_atol=1e-12)
        ST, SE, _ = c.source_grid(ks, *HIER, reltol=1e-10, abstol=1e-10)
        tt, _, _ = c.cl(ST, SE, ks, ells, kd=kd, bessel_argmax=argmax)
        out.append(tt)
    return (out[0] - out[1]) / (2 * rel_step * abs(th[j]))


@pytest.mark.slow
def test_cl_gradient_vs_oracle_fd():
    par = _par()
    ks = _ks(par, nk=40, kmax_h0=300.0)
    ells = np.array([2, 10, 40, 120, 250], dtype=np.int32)
    with B.Engine(lanes=1) as eng:
        r = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt",), grad=True))
    assert r.rc == 0, r.err
    d = r.dcl["tt"]
    # A enters linearly: dC/dA = C/A
    assert _rel(d[4], r.cl["tt"] / par.A) < 1e-7
    for j in range(6):
        fd3 = _oracle_cl_fd(par, ks, ells, 1e-3, j)
        fd4 = _oracle_cl_fd(par, ks, ells, 1e-4, j)
        scale = np.max(np.abs(fd3))
        assert np.max(np.abs(fd3 - fd4)) < 1e-3 * scale, (B.THETA_NAMES[j], fd3, fd4)  # oracle FD converged
        assert np.max(np.abs(d[j] - fd4)) < 1e-3 * scale, (B.THETA_NAMES[j], d[j], fd4)


@pytest.mark.slow
def test_plin_gradient_vs_oracle_fd():
    import oracle as O
    par = _par(mnu=0.12)
    ks = B.log10_k(1e-3 * par.h, 0.5 * par.h, 6)
    with B.Engine(lanes=1) as eng:
        r = eng.run(B.Request("plin", par, ks, hier=HIER, grad=True))
    assert r.rc == 0, r.err
    th = B.theta_of(par)
    for j in range(6):
        vals = []
        for sgn in (1.0, -1.0):
            t = th.copy()
            t[j] += sgn * 1e-4 * abs(th[j])
            p = B.params_of(par, t)
            c = O.Cosmo(O.Params(h=p.h, Omega_b=p.Omega_b, Omega_c=p.Omega_c, n=p.n, A=p.A, Sigma_m_nu_eV=t[5]),
                        recfast_tol=1e-11, recfast_atol=1e-12)
            vals.append(np.array([c.plin(k, lg=HIER[0], lnu=HIER[1], lmnu=HIER[2], reltol=1e-10, abstol=1e-10)
                                  for k in ks]))
        fd = (vals[0] - vals[1]) / (2e-4 * abs(th[j]))
        assert np.max(np.abs(r.dplin[j] - fd)) < 1e-3 * np.max(np.abs(fd)), (B.THETA_NAMES[j], r.dplin[j], fd)


def test_tangent_los_matches_difference_los():
    """C_l^TT gradients from the tangent of the LOS integral (TT-only
    requests) against forward differences of the full LOS (TT + EE
    requests), both on the same frozen-step source grids."""
    par = _par(h=0.66, mnu=0.09)
    ks = _ks(par, nk=50, kmax_h0=400.0)
    ells = np.array([2, 30, 150, 400, 900], dtype=np.int32)
    with B.Engine(lanes=1) as eng:
        a = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt",), grad=True))
        b = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt", "ee"), grad=True))
    assert a.rc == 0 and b.rc == 0, (a.err, b.err)
    assert _rel(a.cl["tt"], b.cl["tt"]) < 1e-12
    for j in range(6):
        scale = np.max(np.abs(b.dcl["tt"][j]))
        assert np.max(np.abs(a.dcl["tt"][j] - b.dcl["tt"][j])) < 1e-4 * scale, (B.THETA_NAMES[j], a.dcl["tt"][j],
                                                                                 b.dcl["tt"][j])


def test_request_validation_errors():
    par = _par()
    ks = _ks(par, nk=20)
    with B.Engine(lanes=1) as eng:
        with pytest.raises(ValueError, match="ascending"):
            eng.submit(B.Request("plin", par, ks[::-1].copy(), hier=HIER))
        with pytest.raises(ValueError, match="truncations"):
            eng.submit(B.Request("plin", par, ks, hier=(2, 20, 10, 15)))
        with pytest.raises(ValueError, match="multipoles"):
            eng.submit(B.Request("cl", par, ks, hier=HIER, ells=np.array([1, 5], dtype=np.int32)))
        with pytest.raises(ValueError, match="plin_x"):
            eng.submit(B.Request("plin", par, ks, hier=HIER, plin_x=0.5))
        # the engine still serves after rejected submissions
        r = eng.run(B.Request("plin", par, ks[:4], hier=HIER))
        assert r.rc == 0, r.err


def test_budget_rejects_oversized_request():
    par = _par()
    with B.Engine(lanes=1, mem_budget_gb=1e-4) as eng:  # 100 kB
        r = eng.run(B.Request("cl", par, _ks(par, nk=64), hier=HIER, ells=np.arange(2, 100, dtype=np.int32)))
    assert r.rc == -5 and "budget" in r.err


def test_failing_request_does_not_affect_others():
    """A request that exhausts the step cap (tight tolerances) reports its
    status; a request submitted with it completes normally."""
    par = _par()
    ks = _ks(par, nk=16)
    with B.Engine(lanes=2, max_steps=5000) as eng:
        bad = eng.submit(B.Request("plin", par, ks, hier=HIER, reltol=1e-13, abstol=1e-15))
        good = eng.submit(B.Request("plin", par, ks, hier=HIER))
        rb, rg = eng.wait(bad), eng.wait(good)
    assert rb.rc == -4 and "status" in rb.err
    assert np.any((rb.status & 0xFF) == 1)  # max iterations
    assert rg.rc == 0, rg.err
    with B.Engine(lanes=1) as eng:
        ref = eng.run(B.Request("plin", par, ks, hier=HIER))
    assert _rel(rg.plin, ref.plin) < 1e-12


def test_vjp_matches_jacobian_contraction():
    """bolt_cl_vjp / bolt_plin_vjp equal the cotangent contracted with the
    Jacobian of the same request."""
    rng = np.random.default_rng(3)
    par = _par(h=0.69, mnu=0.08)
    ks = _ks(par, nk=40, kmax_h0=300.0)
    ells = np.arange(2, 500, 9, dtype=np.int32)
    with B.Engine(lanes=1) as eng:
        full = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt", "ee"), grad=True))
        yb = {"tt": rng.standard_normal(ells.size), "ee": rng.standard_normal(ells.size)}
        res, g = eng.vjp(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt", "ee")), yb)
        kp = B.log10_k(1e-3 * par.h, 0.5 * par.h, 12)
        pf = eng.run(B.Request("plin", par, kp, hier=HIER, grad=True))
        ybp = rng.standard_normal(kp.size)
        rp, gp = eng.vjp(B.Request("plin", par, kp, hier=HIER), ybp)
    assert full.rc == 0 and res.rc == 0 and pf.rc == 0 and rp.rc == 0, (full.err, res.err, pf.err, rp.err)
    want = full.dcl["tt"] @ yb["tt"] + full.dcl["ee"] @ yb["ee"]
    assert np.max(np.abs(g - want)) <= 1e-12 * np.max(np.abs(want))
    assert _rel(res.cl["tt"], full.cl["tt"]) < 1e-12
    wantp = pf.dplin @ ybp
    assert np.max(np.abs(gp - wantp)) <= 1e-12 * np.max(np.abs(wantp))
    assert _rel(rp.plin, pf.plin) < 1e-12


def test_cl_request_with_plin():
    """A C_l request with with_plin also returns P_lin(k) at the end of the x
    grid from the same modes: it matches a P_lin request on the same k and
    hierarchy (another step sequence, so to the solver tolerance), its C_l
    are those of the request without it, and its Jacobian keeps
    dP/dA = P/A."""
    par = _par(h=0.71, mnu=0.07)
    ks = _ks(par, nk=32, kmax_h0=300.0)
    ells = np.arange(2, 300, 7, dtype=np.int32)
    with B.Engine(lanes=1) as eng:
        a = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt",), with_plin=True, grad=True))
        b = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt",), grad=True))
        p = eng.run(B.Request("plin", par, ks, hier=HIER))
    assert a.rc == 0 and b.rc == 0 and p.rc == 0, (a.err, b.err, p.err)
    assert _rel(a.cl["tt"], b.cl["tt"]) < 1e-12
    assert _rel(a.dcl["tt"], b.dcl["tt"]) < 1e-12
    # two solves with different step sequences at abstol 3e-7: ~1e-5 apart at the lowest k
    assert np.max(np.abs(a.plin / p.plin - 1)) < 1e-4
    assert np.max(np.abs(a.dplin[4] * par.A / a.plin - 1)) < 1e-12


def test_land_stride_changes_cl_by_the_interpolation_error_only():
    """land_stride = 2 (every other x node at x >= -8.5 from dense output):
    fewer steps, C_l within the cubic interpolation error of landing on
    every node."""
    par = _par(h=0.67)
    ks = _ks(par, nk=48, kmax_h0=400.0)
    ells = np.arange(2, 1200, 11, dtype=np.int32)
    out = {}
    for stride in (1, 2):
        with B.Engine(lanes=1, land_stride=stride) as eng:
            out[stride] = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt", "ee")))
        assert out[stride].rc == 0, out[stride].err
    assert out[2].steps < out[1].steps
    for c in ("tt", "ee"):
        assert _rel(out[2].cl[c], out[1].cl[c]) < 1e-5
    with pytest.raises(RuntimeError):
        B.Engine(land_stride=65)


def test_tangent_equals_replay_jacobians():
    """The tangent-linear solver (one solve carries the state and its four
    derivatives, sharing each step's factorisation) and the frozen-step
    replays (forward differences of four perturbed solves on the recorded
    steps) differentiate the same discrete pipeline: C_l^TT and P_lin agree
    to 1e-6 and their Jacobians to 2e-4 of each parameter's peak (the
    replays' forward differences carry ~1e-6 truncation; the two schemes run
    the base solve in different kernels)."""
    par = _par(h=0.69, mnu=0.11)
    ks = _ks(par, nk=40, kmax_h0=300.0)
    ells = np.arange(2, 600, 13, dtype=np.int32)
    kp = B.log10_k(1e-3 * par.h, 0.5 * par.h, 16)
    out = {}
    for scheme in ("tangent", "replay"):
        with B.Engine(lanes=1, grad_scheme=scheme) as eng:
            c = eng.run(B.Request("cl", par, ks, hier=HIER, ells=ells, cl=("tt",), grad=True))
            p = eng.run(B.Request("plin", par, kp, hier=HIER, grad=True))
        assert c.rc == 0 and p.rc == 0, (scheme, c.err, p.err)
        out[scheme] = (c, p)
    (ct, pt), (cr, pr) = out["tangent"], out["replay"]
    assert _rel(ct.cl["tt"], cr.cl["tt"]) < 1e-6
    assert _rel(pt.plin, pr.plin) < 1e-6
    bad = []
    for j in range(6):
        for what, a, b in (("C_l^TT", ct.dcl["tt"][j], cr.dcl["tt"][j]), ("P_lin", pt.dplin[j], pr.dplin[j])):
            err = np.max(np.abs(a - b)) / np.max(np.abs(b))
            if not err < 2e-4:
                bad.append((what, B.THETA_NAMES[j], float(err)))
    assert not bad, bad
