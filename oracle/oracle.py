"""CPU oracle (test infrastructure only).

ctypes wrapper over ``oracle/_build/liboracle.so``, the C++ FP64
restatement of Bolt.jl's algorithm for the perturbation solve, source
grid, line-of-sight spectra and P_lin.  Only the test suite, the smoke
check and the CPU-baseline leg of ``bench.py`` import this module; the
product library never does.

Reference correspondence (paths within Bolt.jl):
  CosmoParams                  src/Bolt.jl:56-66
  Background                   src/background.jl:104-128
  RECFAST / IonizationHistory  src/ionization/recfast.jl:22-121, 446-536, 674-726
  boltsolve / hierarchy!       src/perturbations.jl:25-33, 161-271
  source_grid(_P)              src/spectra.jl:6-42
  cltt / clte / clee           src/spectra.jl:49-160
  plin                         src/spectra.jl:163-198
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)


class _Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("h", "Omega_r", "Omega_b", "Omega_c", "A", "n", "Y_p", "N_nu", "Sigma_m_nu")]


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.oracle_mass_natural.restype = C.c_double
        L.oracle_km_s_Mpc_100.restype = C.c_double
        L.oracle_cosmo_new.restype = C.c_void_p
        L.oracle_cosmo_new.argtypes = [C.POINTER(_Params), C.c_double, C.c_double, C.c_double, C.c_int,
                                       C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
        L.oracle_cosmo_free.argtypes = [C.c_void_p]
        L.oracle_cosmo_ngrid.argtypes = [C.c_void_p]
        L.oracle_grid_nodes.argtypes = [C.c_void_p, _dp]
        L.oracle_cosmo_scalars.argtypes = [C.c_void_p, _dp]
        L.oracle_table_eval.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _dp]
        L.oracle_table_coefs.argtypes = [C.c_void_p, C.c_int, _dp]
        L.oracle_recfast_xe.argtypes = [C.POINTER(_Params), C.c_double, C.c_double, C.c_double, C.c_int,
                                        C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                        _dp, C.c_int, _dp]
        L.oracle_dual_cosmo_theta.restype = C.c_void_p
        L.oracle_dual_cosmo_theta.argtypes = [_dp, C.POINTER(_Params), C.c_double, C.c_double, C.c_double, C.c_int,
                                              C.c_double, C.c_double]
        L.oracle_dual_cosmo_omega_b.restype = C.c_void_p
        L.oracle_dual_cosmo_omega_b.argtypes = [C.POINTER(_Params), C.c_double, C.c_double, C.c_double, C.c_int,
                                                C.c_double]
        L.oracle_dual_free.argtypes = [C.c_void_p]
        L.oracle_dual_table.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _dp]
        L.oracle_dual_eta0.argtypes = [C.c_void_p, _dp]
        L.oracle_dual_plin.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                       C.c_double, C.c_double, _dp]
        L.oracle_dual_cltt.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                       C.c_double, _ip, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, _dp,
                                       C.c_int]
        L.oracle_rhs.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                 _dp, _dp, _dp]
        L.oracle_jacobian.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_double, _dp]
        L.oracle_initial_conditions.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int,
                                                C.c_int, _dp]
        L.oracle_boltsolve.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_double, C.c_double, _dp, C.c_int, _dp, _lp]
        L.oracle_source_grid.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_double, C.c_double, _dp, _dp, _lp, C.c_int]
        L.oracle_quadratic_k.argtypes = [C.c_double, C.c_double, C.c_int, _dp]
        L.oracle_log10_k.argtypes = [C.c_double, C.c_double, C.c_int, _dp]
        L.oracle_sph_bessel.argtypes = [C.c_int, C.c_double, _dp]
        L.oracle_cl.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double,
                                C.c_int, _dp, _dp, _dp, C.c_int]
        L.oracle_cl_frozen.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, _ip, C.c_int, C.c_double,
                                       C.c_double, C.c_int, C.c_double, _dp, _dp, _dp, C.c_int]
        L.oracle_cosmo_new_peebles.restype = C.c_void_p
        L.oracle_cosmo_new_peebles.argtypes = [C.POINTER(_Params), C.c_double, C.c_double, C.c_double, C.c_int,
                                               C.c_double, C.c_double, C.c_double]
        L.oracle_cosmo_new_atol.restype = C.c_void_p
        L.oracle_cosmo_new_atol.argtypes = [C.POINTER(_Params), C.c_double, C.c_double, C.c_double, C.c_int,
                                            C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                            C.c_double]
        L.oracle_rsa_perts.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp]
        L.oracle_plin.restype = C.c_double
        L.oracle_plin.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_double, C.c_double, _ip]
        L.oracle_sphj.restype = C.c_double
        L.oracle_sphj.argtypes = [C.c_int, C.c_double]
        L.oracle_sphj_moment.restype = C.c_double
        L.oracle_sphj_moment.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int]
        L.oracle_moment_table_new.restype = C.c_void_p
        L.oracle_moment_table_new.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.oracle_moment_table_free.argtypes = [C.c_void_p]
        L.oracle_moment_table_eval.argtypes = [C.c_void_p, _dp, C.c_int, _dp]
        L.oracle_filon.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.oracle_filon_piecewise.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def mass_natural() -> float:
    return lib().oracle_mass_natural()


def km_s_Mpc_100() -> float:
    return lib().oracle_km_s_Mpc_100()


@dataclass
class Params:
    """CosmoParams (Bolt.jl:56-66); Sigma_m_nu in eV here, converted on use."""
    h: float = 0.7
    Omega_r: float = 5.0469e-5
    Omega_b: float = 0.046
    Omega_c: float = 0.224
    A: float = 2.097e-9
    n: float = 1.0
    Y_p: float = 0.24
    N_nu: float = 3.046
    Sigma_m_nu_eV: float = 0.06

    def c(self) -> _Params:
        return _Params(self.h, self.Omega_r, self.Omega_b, self.Omega_c, self.A, self.n, self.Y_p,
                       self.N_nu, self.Sigma_m_nu_eV * mass_natural())


TABLES = ["H", "Hp", "Hpp", "eta", "etap", "etapp", "rho0M", "Xe", "tau", "taup", "taupp",
          "g", "gp", "gpp", "Tmat", "csb2"]


def state_len(lg, lnu, lmnu, nq):
    return 2 * (lg + 1) + (lnu + 1) + (lmnu + 1) * nq + 5


class Cosmo:
    """Background + IonizationHistory (RECFAST, or with ionization="peebles"
    the Saha-Peebles history through customion) for one parameter set."""

    def __init__(self, p: Params, x_grid=(-20.0, 0.01, 0.0), nq=15, OmegaG=None, Tnow=-1.0,
                 recfast_tol=1e-8, recfast_atol=None, ionization="recfast"):
        self.p = p
        self._pc = p.c()
        og = p.Omega_r if OmegaG is None else OmegaG
        if ionization == "peebles":
            self.h = lib().oracle_cosmo_new_peebles(C.byref(self._pc), x_grid[0], x_grid[1], x_grid[2], nq,
                                                    p.Y_p, p.Omega_b, og)
        elif recfast_atol is None:
            self.h = lib().oracle_cosmo_new(C.byref(self._pc), x_grid[0], x_grid[1], x_grid[2], nq,
                                            p.Y_p, p.Omega_b, og, Tnow, recfast_tol)
        else:
            self.h = lib().oracle_cosmo_new_atol(C.byref(self._pc), x_grid[0], x_grid[1], x_grid[2], nq,
                                                 p.Y_p, p.Omega_b, og, Tnow, recfast_tol, recfast_atol)
        if not self.h:
            raise RuntimeError("oracle_cosmo_new failed")
        self.nx = lib().oracle_cosmo_ngrid(self.h)
        self.x = np.zeros(self.nx)
        lib().oracle_grid_nodes(self.h, _d(self.x))
        s = np.zeros(8)
        lib().oracle_cosmo_scalars(self.h, _d(s))
        (self.H0, self.eta0, self.rho_crit, self.Omega_Lambda, self.z_He_evo_start,
         self.z_H_He_evo_start, self.tau0, self.Tnow) = s

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().oracle_cosmo_free(self.h)
        except Exception:
            pass

    def table(self, name, x=None):
        x = self.x if x is None else np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(len(x))
        lib().oracle_table_eval(self.h, TABLES.index(name), _d(x), len(x), _d(out))
        return out

    def coefs(self, name):
        out = np.zeros(self.nx + 2)
        lib().oracle_table_coefs(self.h, TABLES.index(name), _d(out))
        return out

    def rhs(self, k, u, x, lg=8, lnu=8, lmnu=10, nq=15):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.zeros_like(u)
        dx = np.zeros_like(u)
        lib().oracle_rhs(self.h, k, lg, lnu, lmnu, nq, x, _d(u), _d(du), _d(dx))
        return du, dx

    def jacobian(self, k, x, lg=8, lnu=8, lmnu=10, nq=15):
        N = state_len(lg, lnu, lmnu, nq)
        J = np.zeros((N, N))
        lib().oracle_jacobian(self.h, k, lg, lnu, lmnu, nq, x, _d(J))
        return J

    def initial_conditions(self, k, lg=8, lnu=8, lmnu=10, nq=15):
        u = np.zeros(state_len(lg, lnu, lmnu, nq))
        lib().oracle_initial_conditions(self.h, k, lg, lnu, lmnu, nq, _d(u))
        return u

    def boltsolve(self, k, xout, lg=8, lnu=8, lmnu=10, nq=15, reltol=1e-6, abstol=1e-6):
        xout = np.ascontiguousarray(xout, dtype=np.float64)
        N = state_len(lg, lnu, lmnu, nq)
        u = np.zeros((len(xout), N))
        st = np.zeros(3, dtype=np.int64)
        rc = lib().oracle_boltsolve(self.h, k, lg, lnu, lmnu, nq, reltol, abstol, _d(xout), len(xout),
                                    _d(u), st.ctypes.data_as(_lp))
        if rc != 0:
            raise RuntimeError(f"oracle_boltsolve status {rc}")
        return u, st

    def source_grid(self, k_grid, lg=8, lnu=8, lmnu=10, nq=15, reltol=1e-11, abstol=1e-6, nthreads=0):
        k_grid = np.ascontiguousarray(k_grid, dtype=np.float64)
        nk = len(k_grid)
        ST = np.zeros((nk, self.nx))
        SE = np.zeros((nk, self.nx))
        steps = np.zeros(nk, dtype=np.int64)
        rc = lib().oracle_source_grid(self.h, _d(k_grid), nk, lg, lnu, lmnu, nq, reltol, abstol, _d(ST),
                                      _d(SE), steps.ctypes.data_as(_lp), nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle_source_grid status {rc}")
        return ST, SE, steps

    def cl(self, ST, SE, k_grid, ells, kd=None, nthreads=0, bessel_argmax=None):
        ells = np.ascontiguousarray(ells, dtype=np.int32)
        k_grid = np.ascontiguousarray(k_grid, dtype=np.float64)
        ST = np.ascontiguousarray(ST, dtype=np.float64)
        SE = np.ascontiguousarray(SE, dtype=np.float64)
        if kd is None:
            kd = (0.01 * self.H0, 1000.0 * self.H0, 5000)
        tt, te, ee = (np.zeros(len(ells)) for _ in range(3))
        lib().oracle_cl_frozen(self.h, _d(ST), _d(SE), _d(k_grid), len(k_grid), ells.ctypes.data_as(_ip),
                               len(ells), kd[0], kd[1], kd[2], -1.0 if bessel_argmax is None else bessel_argmax,
                               _d(tt), _d(te), _d(ee), nthreads)
        return tt, te, ee

    def rsa_perts(self, k, x, u, lg=8, lnu=8, lmnu=10, nq=15):
        """rsa_perts! (perturbations.jl:35-88) on a copy of the state u at x."""
        out = np.ascontiguousarray(u, dtype=np.float64).copy()
        lib().oracle_rsa_perts(self.h, k, lg, lnu, lmnu, nq, x, _d(out))
        return out

    def plin(self, k, nq=15, lg=50, lnu=50, lmnu=20, x=0.0, reltol=1e-5, abstol=1e-6):
        st = C.c_int(0)
        v = lib().oracle_plin(self.h, k, nq, lg, lnu, lmnu, x, reltol, abstol, C.byref(st))
        if st.value != 0:
            raise RuntimeError(f"oracle_plin status {st.value}")
        return v


THETA_NAMES = ("h", "omega_b", "omega_c", "n_s", "A_s", "Sigma_m_nu_eV")


class DualCosmo:
    """The gradient oracle: Background + RECFAST + IonizationHistory whose
    every quantity carries its partial derivatives (oracle/oracle_grad.hpp),
    the reference's ForwardDiff gradient restated.  Build it from theta =
    (h, omega_b, omega_c, n_s, A_s, Sigma m_nu [eV]) (partials along theta),
    or with ``omega_b_only`` from a Params with the single partial along
    Omega_b (the reference's bg_fwddiff / ih_fwddiff tests).  Results come
    as (value, partials)."""

    def __init__(self, theta=None, params: Params | None = None, x_grid=(-20.0, 0.01, 0.0), nq=15,
                 recfast_tol=1e-8, recfast_atol=None, omega_b_only=False):
        base = params or Params()
        self._pc = base.c()
        if omega_b_only:
            self.h = lib().oracle_dual_cosmo_omega_b(C.byref(self._pc), x_grid[0], x_grid[1], x_grid[2], nq,
                                                     recfast_tol)
        else:
            th = np.ascontiguousarray(theta, dtype=np.float64)
            self.h = lib().oracle_dual_cosmo_theta(_d(th), C.byref(self._pc), x_grid[0], x_grid[1], x_grid[2], nq,
                                                   recfast_tol, -1.0 if recfast_atol is None else recfast_atol)
        if not self.h:
            raise RuntimeError("gradient oracle construction failed")

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().oracle_dual_free(self.h)
        except Exception:
            pass

    def table(self, name, x):
        x = np.ascontiguousarray(np.atleast_1d(x), dtype=np.float64)
        out = np.zeros((x.size, 7))
        if lib().oracle_dual_table(self.h, TABLES.index(name), _d(x), x.size, _d(out)) != 0:
            raise ValueError(f"table {name} not available in the gradient oracle")
        return out[:, 0], out[:, 1:]

    def eta0(self):
        out = np.zeros(7)
        lib().oracle_dual_eta0(self.h, _d(out))
        return out[0], out[1:]

    def plin(self, k, nq=15, lg=50, lnu=50, lmnu=20, x=0.0, reltol=1e-5, abstol=1e-6):
        out = np.zeros(7)
        st = lib().oracle_dual_plin(self.h, k, nq, lg, lnu, lmnu, x, reltol, abstol, _d(out))
        if st != 0:
            raise RuntimeError(f"oracle_dual_plin status {st}")
        return out[0], out[1:]

    def cltt(self, k_grid, ells, lg=8, lnu=8, lmnu=10, nq=15, reltol=1e-8, abstol=1e-8, kd=None, bessel_argmax=None,
             nthreads=0):
        """C_l^TT and its partials on the source-grid k (frozen), the dense k
        grid kd = (kmin, kmax, n) (frozen) and the Bessel grid's upper end
        (frozen).  Returns (tt[nell], dtt[6][nell])."""
        kg = np.ascontiguousarray(k_grid, dtype=np.float64)
        ells = np.ascontiguousarray(ells, dtype=np.int32)
        out = np.zeros((ells.size, 7))
        st = lib().oracle_dual_cltt(self.h, _d(kg), kg.size, lg, lnu, lmnu, nq, reltol, abstol,
                                    ells.ctypes.data_as(_ip), ells.size, kd[0], kd[1], kd[2], bessel_argmax,
                                    _d(out), nthreads)
        if st != 0:
            raise RuntimeError(f"oracle_dual_cltt status {st}")
        return out[:, 0], out[:, 1:].T.copy()


def recfast_xe(p: Params, z, x_grid=(-20.0, 0.01, 0.0), nq=15, OmegaG=None, Tnow=-1.0, tol=1e-8):
    z = np.ascontiguousarray(z, dtype=np.float64)
    out = np.zeros(len(z))
    pc = p.c()
    og = p.Omega_r if OmegaG is None else OmegaG
    rc = lib().oracle_recfast_xe(C.byref(pc), x_grid[0], x_grid[1], x_grid[2], nq, p.Y_p, p.Omega_b, og,
                                 Tnow, tol, _d(z), len(z), _d(out))
    if rc != 0:
        raise RuntimeError("oracle_recfast_xe failed")
    return out


def quadratic_k(kmin, kmax, nk):
    out = np.zeros(nk)
    lib().oracle_quadratic_k(kmin, kmax, nk, _d(out))
    return out


def log10_k(kmin, kmax, nk):
    out = np.zeros(nk)
    lib().oracle_log10_k(kmin, kmax, nk, _d(out))
    return out


def sph_bessel_all(L, x):
    out = np.zeros(L + 1)
    lib().oracle_sph_bessel(L, x, _d(out))
    return out


# ------------------------------------------------- Bessel moments, Filon ---
_MOMENT_METHODS = {"auto": 0, "maclaurin": 1, "asymp": 2, "quad": 3}


def sphj(n, t):
    """j_n(t) of one order (n = -1: cos t / t)."""
    return lib().oracle_sphj(int(n), float(t))


def sph_j_moment(x, nu, m, method="auto"):
    """int_0^x t^m j_nu(t) dt (moments.jl: sph_j_moment_asymp /
    sph_j_moment_weniger_1F2 / sph_j_moment_maclaurin_1F2 all return this)."""
    return lib().oracle_sphj_moment(int(nu), float(m), float(x), _MOMENT_METHODS[method])


def J_moment(x, nu, alpha, method="auto"):
    """int_0^x t^alpha J_nu(t) dt for half-integer nu = n + 1/2 (moments.jl:
    J_moment_asymp / J_moment_weniger_1F2): sqrt(2/pi) times the spherical
    moment of order alpha + 1/2."""
    n = int(round(nu - 0.5))
    assert abs(n + 0.5 - nu) < 1e-12, "half-integer orders only"
    return np.sqrt(2.0 / np.pi) * sph_j_moment(x, n, alpha + 0.5, method)


class MomentTable:
    """sph_bessel_interpolator(nu, order, kmin, kmax, N) (interpolator.jl:81-94);
    calling it evaluates the moments m = 0..order-1 (interpolator.jl:67-75)."""

    def __init__(self, nu, order, kmin, kmax, N):
        self.nu, self.order = int(nu), int(order)
        self.h = lib().oracle_moment_table_new(self.nu, self.order, float(kmin), float(kmax), int(N))
        if not self.h:
            raise ValueError("bad moment table arguments")

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_moment_table_free(self.h)
            self.h = None

    def __call__(self, x):
        xa = np.ascontiguousarray(np.atleast_1d(np.asarray(x, dtype=np.float64)))
        out = np.zeros((xa.size, self.order))
        lib().oracle_moment_table_eval(self.h, _d(xa), xa.size, _d(out))
        return out[0] if np.ndim(x) == 0 else out

    def filon(self, f, fp, fpp, k, a, b):
        """integrate_sph_bessel_filon (integrator.jl:7-19), elementwise."""
        arr = [np.ascontiguousarray(np.atleast_1d(np.asarray(v, dtype=np.float64))) for v in (f, fp, fpp, k, a, b)]
        n = max(v.size for v in arr)
        arr = [np.ascontiguousarray(np.broadcast_to(v, (n,))) for v in arr]
        out = np.zeros(n)
        lib().oracle_filon(self.h, n, *[_d(v) for v in arr], _d(out))
        return out[0] if all(np.ndim(v) == 0 for v in (f, fp, fpp, k, a, b)) else out

    def filon_piecewise(self, t, f, fp, fpp, k, nthreads=0):
        """sum over segments [t_i, t_{i+1}] of the Filon integral of the
        quadratic at t_i (integrator.jl:25-38), for every k."""
        t, f, fp, fpp = (np.ascontiguousarray(v, dtype=np.float64) for v in (t, f, fp, fpp))
        k = np.ascontiguousarray(np.atleast_1d(k), dtype=np.float64)
        out = np.zeros(k.size)
        lib().oracle_filon_piecewise(self.h, t.size, _d(t), _d(f), _d(fp), _d(fpp), k.size, _d(k), _d(out),
                                     int(nthreads))
        return out
