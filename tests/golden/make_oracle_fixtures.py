"""Converged CPU-oracle results at the configurations' own sizes, for the GPU
parity tests (tests/test_gpu_config_sizes.py).

The oracle (oracle/, the C++ FP64 restatement of Bolt.jl's CPU path) needs
minutes on many cores for these cases, longer than a GPU test should wait, so
its outputs are computed once here and stored as small .npz files.  Run from
the repository root after building the oracle (make -C oracle):

    python tests/golden/make_oracle_fixtures.py [name ...]

Fixtures (all FP64; k in Mpc^-1):
  oracle_cl_l50_1024k   C_l^TT/TE/EE, l = 2..2500, of the hardest C_l request
                        of the serving stream: 1024 log k in [0.1, 1000] H0,
                        l_gamma = l_nu = 50, l_mnu = 10, nq = 15 (N = 323),
                        fiducial LCDM, oracle at reltol = abstol = 1e-11.
  oracle_plin_n473      P_lin(k) at z = 0 on 200 log k in [1e-4, 1] h/Mpc at
                        the reference plin defaults l 50/50/20, nq 15
                        (N = 473), fiducial LCDM, reltol = abstol = 1e-10.
  oracle_jac_cltt       d C_l^TT / d theta, l = 2..2000, theta = (h, omega_b,
                        omega_c, n_s, A_s, Sigma m_nu [eV]) by central
                        differences with relative steps 1e-3 and 1e-4 (the
                        k grids and the Bessel grid of the unperturbed
                        cosmology held fixed, as the reference's ForwardDiff
                        gradient holds them), 200 log k in [0.1, 1000] H0,
                        l_gamma = l_nu = 35, l_mnu = 10 (N = 278).
  oracle_jac_plin       d P_lin / d theta on 200 log k in [1e-4, 1] h/Mpc,
                        l 50/50/20 (N = 473), central differences as above.
Both Jacobians at theta0 below, oracle at reltol = abstol = 1e-10 with
RECFAST at tol 1e-11 / atol 1e-12 (so the differences are smooth).
  oracle_jac_cltt_dual, oracle_jac_plin_dual
                        the same two Jacobians from the gradient oracle
                        (dual numbers with six partials, the reference's
                        ForwardDiff gradient restated; oracle_grad.hpp).
"""
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

CORES = os.cpu_count() or 1
FID = dict(h=0.7, Omega_b=0.046, Omega_c=0.224, n=0.96, A=2.1e-9, Sigma_m_nu_eV=0.06)
THETA0 = np.array([0.68, 0.0224, 0.119, 0.965, 2.1e-9, 0.1])  # h, omega_b, omega_c, n_s, A_s, Sigma m_nu [eV]
STEPS = (1e-3, 1e-4)


def params_of(th):
    h = th[0]
    return O.Params(h=h, Omega_b=th[1] / h ** 2, Omega_c=th[2] / h ** 2, n=th[3], A=th[4], Sigma_m_nu_eV=th[5])


def plin_many(c, ks, hier, tol):
    lg, lnu, lmnu, nq = hier
    with ThreadPoolExecutor(CORES) as ex:
        return np.array(list(ex.map(lambda k: c.plin(k, nq, lg, lnu, lmnu, 0.0, tol, tol), ks)))


def cl_l50_1024k():
    c = O.Cosmo(O.Params(**FID))
    ks = O.log10_k(0.1 * c.H0, 1000.0 * c.H0, 1024)
    ells = np.arange(2, 2501, dtype=np.int32)
    ST, SE, _ = c.source_grid(ks, 50, 50, 10, 15, reltol=1e-11, abstol=1e-11, nthreads=CORES)
    tt, te, ee = c.cl(ST, SE, ks, ells, nthreads=CORES)
    return dict(ks=ks, ells=ells, tt=tt, te=te, ee=ee, hier=np.array([50, 50, 10, 15]), tol=1e-11)


def plin_n473():
    c = O.Cosmo(O.Params(**FID))
    h = FID["h"]
    ks = O.log10_k(1e-4 * h, 1.0 * h, 200)
    P = plin_many(c, ks, (50, 50, 20, 15), 1e-10)
    return dict(ks=ks, plin=P, hier=np.array([50, 50, 20, 15]), tol=1e-10)


def _cosmo(th):
    return O.Cosmo(params_of(th), recfast_tol=1e-11, recfast_atol=1e-12)


def jac_cltt():
    hier = (35, 35, 10, 15)
    c0 = _cosmo(THETA0)
    H0 = c0.H0
    ks = O.log10_k(0.1 * H0, 1000.0 * H0, 200)
    ells = np.arange(2, 2001, dtype=np.int32)
    kd = (0.01 * H0, 1000.0 * H0, 5000)
    argmax = kd[1] * c0.eta0
    ST0, SE0, _ = c0.source_grid(ks, *hier, reltol=1e-10, abstol=1e-10, nthreads=CORES)
    tt0, _, _ = c0.cl(ST0, SE0, ks, ells, kd=kd, bessel_argmax=argmax, nthreads=CORES)
    out = dict(theta=THETA0, ks=ks, ells=ells, tt=tt0, hier=np.array(hier))
    for step in STEPS:
        J = np.zeros((6, ells.size))
        for j in range(6):
            vals = []
            for sgn in (1.0, -1.0):
                th = THETA0.copy()
                th[j] += sgn * step * abs(THETA0[j])
                c = _cosmo(th)
                if j in (3, 4):  # n_s, A_s: primordial spectrum only, same sources
                    ST, SE = ST0, SE0
                else:
                    ST, SE, _ = c.source_grid(ks, *hier, reltol=1e-10, abstol=1e-10, nthreads=CORES)
                tt, _, _ = c.cl(ST, SE, ks, ells, kd=kd, bessel_argmax=argmax, nthreads=CORES)
                vals.append(tt)
            J[j] = (vals[0] - vals[1]) / (2 * step * abs(THETA0[j]))
            print(f"  cltt step {step:g} theta_{j} done", flush=True)
        out[f"J_{step:g}"] = J
    return out


def jac_plin():
    hier = (50, 50, 20, 15)
    h = THETA0[0]
    ks = O.log10_k(1e-4 * h, 1.0 * h, 200)
    P0 = plin_many(_cosmo(THETA0), ks, hier, 1e-10)
    out = dict(theta=THETA0, ks=ks, plin=P0, hier=np.array(hier))
    for step in STEPS:
        J = np.zeros((6, ks.size))
        for j in range(6):
            vals = []
            for sgn in (1.0, -1.0):
                th = THETA0.copy()
                th[j] += sgn * step * abs(THETA0[j])
                vals.append(plin_many(_cosmo(th), ks, hier, 1e-10))
            J[j] = (vals[0] - vals[1]) / (2 * step * abs(THETA0[j]))
            print(f"  plin step {step:g} theta_{j} done", flush=True)
        out[f"J_{step:g}"] = J
    return out


def jac_cltt_dual():
    f = np.load(os.path.join(HERE, "oracle_jac_cltt.npz"))
    hier = tuple(int(v) for v in f["hier"])
    d = O.DualCosmo(theta=THETA0, recfast_tol=1e-11, recfast_atol=1e-12)
    c0 = _cosmo(THETA0)
    H0 = c0.H0
    kd = (0.01 * H0, 1000.0 * H0, 5000)
    tt, J = d.cltt(f["ks"], f["ells"], *hier, reltol=1e-10, abstol=1e-10, kd=kd, bessel_argmax=kd[1] * c0.eta0,
                   nthreads=CORES)
    return dict(theta=THETA0, ks=f["ks"], ells=f["ells"], tt=tt, J=J, hier=f["hier"])


def jac_plin_dual():
    f = np.load(os.path.join(HERE, "oracle_jac_plin.npz"))
    lg, lnu, lmnu, nq = (int(v) for v in f["hier"])
    d = O.DualCosmo(theta=THETA0, recfast_tol=1e-11, recfast_atol=1e-12)
    with ThreadPoolExecutor(CORES) as ex:
        res = list(ex.map(lambda k: d.plin(k, nq, lg, lnu, lmnu, 0.0, 1e-10, 1e-10), f["ks"]))
    return dict(theta=THETA0, ks=f["ks"], plin=np.array([r[0] for r in res]), J=np.array([r[1] for r in res]).T,
                hier=f["hier"])


MAKERS = {"oracle_cl_l50_1024k": cl_l50_1024k, "oracle_plin_n473": plin_n473, "oracle_jac_cltt": jac_cltt,
          "oracle_jac_plin": jac_plin, "oracle_jac_cltt_dual": jac_cltt_dual, "oracle_jac_plin_dual": jac_plin_dual}


def main(names):
    for name in names or list(MAKERS):
        t0 = time.perf_counter()
        d = MAKERS[name]()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(f"{name}: {time.perf_counter() - t0:.0f} s on {CORES} threads", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
