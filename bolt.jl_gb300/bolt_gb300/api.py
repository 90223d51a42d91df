"""Python mirror of Bolt.jl's public API for the Boltzmann hot path.

Names, argument meaning and defaults follow the reference (paths within
Bolt.jl):

    CosmoParams                      src/Bolt.jl:56-66
    Background(par; x_grid, nq)      src/background.jl:104-128
    RECFAST(bg; Yp, OmegaB, ...)     src/ionization/recfast.jl:22-124
    IonizationHistory(rf, par, bg)   src/ionization/recfast.jl:674-726
    Hierarchy(integrator, ...)       src/perturbations.jl:7-21
    boltsolve(hierarchy; ...)        src/perturbations.jl:25-33
    boltsolve_rsa(hierarchy; ...)    src/perturbations.jl:35-111
    source_grid / source_grid_P      src/spectra.jl:6-42
    quadratic_k / log10_k            src/spectra.jl:60-68
    cltt / clte / clee               src/spectra.jl:84-160
    plin                             src/spectra.jl:163-198

Every solve and projection runs in libbolt_gb300.so on the GPU; Background
and the ionization history are built by the library's host C++ code and kept
resident in HBM.  As in the reference, per-mode solver return codes do not
raise: they are exposed as ``.status`` and reported with a warning.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings
from dataclasses import dataclass, field, replace

import numpy as np

from . import _lib as L

# ------------------------------------------------------------------ units --


def mass_natural() -> float:
    """1 eV in Mpc^-1 (src/Bolt.jl:51)."""
    return L.load().bolt_mass_natural()


def km_s_Mpc_100() -> float:
    """100 km/s/Mpc in Mpc^-1 (src/Bolt.jl:49)."""
    return L.load().bolt_km_s_Mpc_100()


class BoltError(RuntimeError):
    pass


STATUS_NAMES = {0: "ok", 1: "max iterations", 2: "step underflow", 3: "non-finite state",
                4: "singular step matrix", 5: "bad input", 6: "replay ran past the recorded steps"}


def _check_status(status, what):
    st = np.asarray(status)
    hard = st & 0xFF
    if np.any(hard != 0):
        bad = np.unique(hard[hard != 0])
        warnings.warn(f"{what}: {np.count_nonzero(hard)} mode(s) returned "
                      + ", ".join(STATUS_NAMES.get(int(b), str(b)) for b in bad), RuntimeWarning)


# ---------------------------------------------------------------- context --
class Context:
    """One GPU context (device memory, stream, cosmology registry)."""

    def __init__(self, device: int = 0, warps_per_block: int = 0, max_steps: int = 0, land_stride: int = 1):
        self.lib = L.load()
        opts = L.BoltOpts(device, warps_per_block, max_steps)
        h = C.c_void_p()
        rc = self.lib.bolt_ctx_create(C.byref(opts), C.byref(h))
        if rc != 0 or not h.value:
            raise BoltError(f"bolt_ctx_create failed ({rc}): no usable CUDA device {device}")
        self.h = h
        if land_stride != 1:
            self.check(self.lib.bolt_set_land_stride(self.h, int(land_stride)), "bolt_set_land_stride")

    def check(self, rc, what):
        if rc != 0:
            msg = self.lib.bolt_last_error(self.h)
            raise BoltError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def stats(self):
        out = np.zeros(8, dtype=np.int64)
        self.lib.bolt_last_stats(self.h, out.ctypes.data_as(C.POINTER(C.c_int64)))
        keys = ["accepted_steps", "rejected_steps", "solver_us", "los_us", "modes", "solver_launches",
                "kernel_launches", "los_terms"]
        return dict(zip(keys, (int(v) for v in out)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.bolt_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context()
    return _default_ctx


# ---------------------------------------------------------------- params ---
@dataclass
class CosmoParams:
    """CosmoParams{T} (src/Bolt.jl:56-66).  Sigma_m_nu is in Mpc^-1 like the
    reference; ``CosmoParams.from_eV`` converts a neutrino mass sum in eV."""
    h: float = 0.7
    Omega_r: float = 5.0469e-5
    Omega_b: float = 0.046
    Omega_c: float = 0.224
    A: float = 2.097e-9
    n: float = 1.0
    Y_p: float = 0.24
    N_nu: float = 3.046
    Sigma_m_nu: float = field(default_factory=lambda: 0.06 * mass_natural())

    @classmethod
    def from_eV(cls, Sigma_m_nu_eV: float = 0.06, **kw):
        return cls(Sigma_m_nu=Sigma_m_nu_eV * mass_natural(), **kw)

    def c(self) -> L.BoltParams:
        return L.BoltParams(self.h, self.Omega_r, self.Omega_b, self.Omega_c, self.A, self.n, self.Y_p,
                            self.N_nu, self.Sigma_m_nu)


TABLE_NAMES = ["H", "Hp", "Hpp", "eta", "etap", "etapp", "rho0M", "Xe", "tau", "taup", "taupp",
               "g", "gp", "gpp", "Tmat", "csb2"]


def _grid_nodes(x_grid):
    start, step, stop = x_grid
    n = int(math.floor((stop - start) / step + 1e-9)) + 1
    inv = 1.0 / step
    M = round(inv)
    if abs(inv - M) < 1e-9 * M and abs(start * M - round(start * M)) < 1e-6:
        i0 = round(start * M)
        return np.array([(i0 + j) / M for j in range(n)])
    return start + step * np.arange(n)


def _natural_spline_eval(nodes, x0, h, x):
    """Evaluates the library's node tables with the same cubic B-spline
    (natural ends) the reference's `spline` builds (util.jl:11)."""
    from scipy.interpolate import CubicSpline
    xs = x0 + h * np.arange(len(nodes))
    return CubicSpline(xs, nodes, bc_type="natural")(x)


class _Tables:
    def __init__(self, nodes, x, step):
        self.nodes = nodes
        self.x = x
        self.step = step

    def fn(self, name):
        y = self.nodes[TABLE_NAMES.index(name)]
        x0, h = self.x[0], self.step

        def f(x):
            return _natural_spline_eval(y, x0, h, x)
        return f


class Background:
    """Background(par; x_grid=-20.0:0.01:0.0, nq=15) (background.jl:104-128).

    Scalars H0, eta0, rho_crit, Omega_Lambda and the spline tables (as
    callables H, Hp, Hpp, eta, etap, etapp, rho0M of x) come from the
    library's host construction."""

    def __init__(self, par: CosmoParams, x_grid=(-20.0, 0.01, 0.0), nq: int = 15):
        self.par = par
        self.x_grid_spec = tuple(float(v) for v in x_grid)
        self.nq = int(nq)
        self.x_grid = _grid_nodes(self.x_grid_spec)
        rf = L.BoltRecfast(par.Y_p, par.Omega_b, par.Omega_r, -1.0, 1e-8)
        nodes, sc = _host_tables(par, self.x_grid_spec, self.nq, rf)
        self.H0, self.eta0, self.rho_crit, self.Omega_Lambda = sc[0], sc[1], sc[2], sc[3]
        self._t = _Tables(nodes, self.x_grid, self.x_grid_spec[1])
        for nm in ("H", "Hp", "Hpp", "eta", "etap", "etapp", "rho0M"):
            setattr(self, nm, self._t.fn(nm))


def _host_tables(par, x_grid, nq, rf):
    lib = L.load()
    n = len(_grid_nodes(x_grid))
    nodes = np.zeros((16, n))
    sc = np.zeros(10)
    err = C.create_string_buffer(512)
    g = L.BoltGrid(*x_grid)
    rc = lib.bolt_host_tables(C.byref(par.c()), C.byref(g), nq, C.byref(rf), L.dptr(nodes), L.dptr(sc), err, 512)
    if rc != 0:
        raise BoltError(f"bolt_host_tables failed ({rc}): {err.value.decode()}")
    return nodes, sc


def host_tables(par: CosmoParams, x_grid=(-20.0, 0.01, 0.0), nq: int = 15, Yp=None, OmegaB=None, OmegaG=None,
                Tnow=-1.0, tol=1e-8, ionization: str = "recfast"):
    """Node values of all 16 background/ionization tables, host-built
    (ionization "recfast", or "peebles" for Saha-Peebles, see Peebles)."""
    rf = L.BoltRecfast(par.Y_p if Yp is None else Yp, par.Omega_b if OmegaB is None else OmegaB,
                       par.Omega_r if OmegaG is None else OmegaG, -1.0 if Tnow is None else Tnow, tol,
                       _ION[ionization])
    return _host_tables(par, tuple(x_grid), nq, rf)


_ION = {"recfast": 0, "peebles": 1}


@dataclass
class Peebles:
    """Peebles() -- exported by Bolt.jl (Bolt.jl:6) but never defined there.
    Here: the reference's Saha-Peebles X_e (saha_peebles_recombination,
    ionization.jl:83-93: Saha until z = 1587.4, then the Peebles equation by
    Tsit5 at 1e-11) made an IonizationHistory as customion does
    (ionization.jl:141-164), with T_mat = 2.725 K (1 + z) (the T_b of its
    Saha and Peebles equations) and RECFAST's sound-speed formula on it
    (recfast.jl:709-712) for the two functions customion takes from its
    caller."""
    Yp: float = 0.24
    OmegaB: float = 0.046
    OmegaG: float = 5.0469e-5


@dataclass
class RECFAST:
    """RECFAST(bg; Yp, OmegaB, OmegaG, Tnow, tol) (recfast.jl:22-124).  OmegaG
    defaults to 5.0469e-5 and Tnow to the temperature implied by OmegaG."""
    bg: Background
    Yp: float = 0.24
    OmegaB: float = 0.046
    OmegaG: float = 5.0469e-5
    Tnow: float | None = None
    tol: float = 1e-8


class IonizationHistory:
    """IonizationHistory(RECFAST, par, bg) (recfast.jl:674-726), or from
    ``Peebles()`` (the Saha-Peebles history, ionization.jl:83-93,141-164):
    host-built, then resident in HBM for the solver; ``cosmo_id`` names it
    there."""

    def __init__(self, rf, par: CosmoParams, bg: Background, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.par, self.bg, self.rf = par, bg, rf
        if isinstance(rf, Peebles):
            r = L.BoltRecfast(rf.Yp, rf.OmegaB, rf.OmegaG, -1.0, 1e-8, _ION["peebles"])
        else:
            r = L.BoltRecfast(rf.Yp, rf.OmegaB, rf.OmegaG, -1.0 if rf.Tnow is None else rf.Tnow, rf.tol,
                              _ION["recfast"])
        cid = C.c_int(-1)
        g = L.BoltGrid(*bg.x_grid_spec)
        self.ctx.check(self.ctx.lib.bolt_cosmo_build(self.ctx.h, C.byref(par.c()), C.byref(g), bg.nq, C.byref(r),
                                                     C.byref(cid)), "bolt_cosmo_build")
        self.cosmo_id = cid.value
        sc = np.zeros(10)
        self.ctx.check(self.ctx.lib.bolt_cosmo_info(self.ctx.h, self.cosmo_id, L.dptr(sc)), "bolt_cosmo_info")
        self.scalars = sc
        self.z_He_evo_start, self.z_H_He_evo_start = sc[4], sc[5]
        self.tau0 = 0.0
        self._cache = {}
        nodes = np.zeros((16, bg.x_grid.size))
        for t in range(16):
            self.ctx.check(self.ctx.lib.bolt_cosmo_table(self.ctx.h, self.cosmo_id, t, L.dptr(nodes[t])),
                           "bolt_cosmo_table")
        self.nodes = nodes
        tb = _Tables(nodes, bg.x_grid, bg.x_grid_spec[1])
        for nm in ("Xe", "tau", "taup", "taupp", "g", "gp", "gpp", "Tmat", "csb2"):
            setattr(self, nm, tb.fn(nm))

    def close(self):
        if self.cosmo_id >= 0:
            self.ctx.lib.bolt_cosmo_free(self.ctx.h, self.cosmo_id)
            self.cosmo_id = -1


# ----------------------------------------------------------- integrators ---
class PerturbationIntegrator:
    pass


class BasicNewtonian(PerturbationIntegrator):
    """The reference's Newtonian-gauge integrator tag (perturbations.jl:4)."""


class GPUNewtonian(BasicNewtonian):
    """Same equations, integrated by the GB300 Rodas4 kernel."""


@dataclass
class Hierarchy:
    """Hierarchy(integrator, par, bg, ih, k, lg=8, lnu=8, lmnu=10, nq=15)."""
    integrator: PerturbationIntegrator
    par: CosmoParams
    bg: Background
    ih: IonizationHistory
    k: float
    lg: int = 8
    lnu: int = 8
    lmnu: int = 10
    nq: int = 15

    @property
    def N(self):
        return 2 * (self.lg + 1) + (self.lnu + 1) + (self.lmnu + 1) * self.nq + 5


def _hier(lg, lnu, lmnu, nq):
    return L.BoltHier(int(lg), int(lnu), int(lmnu), int(nq))


def state_len(lg, lnu, lmnu, nq):
    return 2 * (lg + 1) + (lnu + 1) + (lmnu + 1) * nq + 5


def boltsolve_batch(ih: IonizationHistory, k, x_out, lg=8, lnu=8, lmnu=10, nq=15, reltol=1e-6, abstol=1e-6):
    """Solves every k and samples u at the ascending x_out: u[ik, ix, :]."""
    k = np.ascontiguousarray(np.atleast_1d(k), dtype=np.float64)
    x_out = np.ascontiguousarray(np.atleast_1d(x_out), dtype=np.float64)
    N = state_len(lg, lnu, lmnu, nq)
    u = np.zeros((k.size, x_out.size, N))
    st = np.zeros(k.size, dtype=np.int32)
    c = ih.ctx
    c.check(c.lib.bolt_boltsolve(c.h, ih.cosmo_id, L.dptr(k), k.size, C.byref(_hier(lg, lnu, lmnu, nq)), reltol,
                                 abstol, L.dptr(x_out), x_out.size, L.dptr(u), L.i32ptr(st)), "bolt_boltsolve")
    _check_status(st, "boltsolve")
    return u, st


class Perturbation:
    """Callable solution of boltsolve: perturb(x) -> u(x) (x scalar or an
    ascending array).  Each call integrates from the first grid node and
    lands on the requested points."""

    def __init__(self, hierarchy: Hierarchy, reltol, abstol):
        self.h = hierarchy
        self.reltol, self.abstol = reltol, abstol
        self.status = None

    def __call__(self, x):
        xs = np.atleast_1d(np.asarray(x, dtype=np.float64))
        order = np.argsort(xs)
        xu, inv = np.unique(xs[order], return_inverse=True)
        h = self.h
        u, st = boltsolve_batch(h.ih, [h.k], xu, h.lg, h.lnu, h.lmnu, h.nq, self.reltol, self.abstol)
        self.status = int(st[0])
        out = np.empty((xs.size, u.shape[2]))
        out[order] = u[0][inv]
        return out[0] if np.ndim(x) == 0 else out


def boltsolve_rsa_batch(ih: IonizationHistory, k, lg=8, lnu=8, lmnu=10, nq=15, reltol=1e-6, abstol=1e-6):
    """boltsolve_rsa (perturbations.jl:90-111) for many k: states on every
    x-grid node with the radiation-streaming values past the switch,
    u[ik][ix][N], and the per-mode status."""
    k = np.ascontiguousarray(np.atleast_1d(k), dtype=np.float64)
    N = state_len(lg, lnu, lmnu, nq)
    u = np.zeros((k.size, ih.bg.x_grid.size, N))
    st = np.zeros(k.size, dtype=np.int32)
    c = ih.ctx
    c.check(c.lib.bolt_boltsolve_rsa(c.h, ih.cosmo_id, L.dptr(k), k.size, C.byref(_hier(lg, lnu, lmnu, nq)), reltol,
                                     abstol, L.dptr(u), L.i32ptr(st)), "bolt_boltsolve_rsa")
    _check_status(st, "boltsolve_rsa")
    return u, st


def boltsolve_rsa(hierarchy: Hierarchy, ode_alg=None, reltol=1e-6, abstol=1e-6) -> np.ndarray:
    """boltsolve_rsa(hierarchy; reltol, abstol): the (pertlen, length(x_grid))
    matrix of states, as the reference returns it."""
    h = hierarchy
    u, _ = boltsolve_rsa_batch(h.ih, [h.k], h.lg, h.lnu, h.lmnu, h.nq, reltol, abstol)
    return u[0].T.copy()


def boltsolve(hierarchy: Hierarchy, ode_alg=None, reltol=1e-6, abstol=1e-6) -> Perturbation:
    """boltsolve(hierarchy, ode_alg=KenCarp4(); reltol=1e-6, abstol=1e-6)."""
    return Perturbation(hierarchy, reltol, abstol)


# ----------------------------------------------------------- source grid ---
class SourceGrid:
    """The interpolant source_grid returns (spectra.jl:21):
    LinearInterpolation((x_grid, k_grid), S, extrapolation_bc=Line()).
    ``S[ik, ix]``; evaluation is exact in x at the grid nodes."""

    def __init__(self, x_grid, k_grid, S, status):
        self.x_grid = x_grid
        self.k_grid = k_grid
        self.S = S
        self.status = status

    def __call__(self, x, k):
        xg, kg, S = self.x_grid, self.k_grid, self.S
        x = float(x)
        k = float(k)
        i = int(np.clip(np.searchsorted(xg, x, side="right") - 1, 0, xg.size - 2))
        j = int(np.clip(np.searchsorted(kg, k, side="right") - 1, 0, kg.size - 2))
        wx = (x - xg[i]) / (xg[i + 1] - xg[i])
        wk = (k - kg[j]) / (kg[j + 1] - kg[j])
        if wx == 0.0:
            return (1 - wk) * S[j, i] + wk * S[j + 1, i]
        if wx == 1.0:
            return (1 - wk) * S[j, i + 1] + wk * S[j + 1, i + 1]
        return ((1 - wx) * ((1 - wk) * S[j, i] + wk * S[j + 1, i]) +
                wx * ((1 - wk) * S[j, i + 1] + wk * S[j + 1, i + 1]))


def _source_pair(par, bg, ih, k_grid, lg, lnu, lmnu, nq, reltol, abstol):
    k_grid = np.ascontiguousarray(k_grid, dtype=np.float64)
    key = (k_grid.tobytes(), lg, lnu, lmnu, nq, reltol, abstol)
    if key in ih._cache:
        return ih._cache[key]
    nx = bg.x_grid.size
    ST = np.zeros((k_grid.size, nx))
    SE = np.zeros((k_grid.size, nx))
    st = np.zeros(k_grid.size, dtype=np.int32)
    c = ih.ctx
    c.check(c.lib.bolt_source_grid(c.h, ih.cosmo_id, L.dptr(k_grid), k_grid.size, C.byref(_hier(lg, lnu, lmnu, nq)),
                                   reltol, abstol, L.dptr(ST), L.dptr(SE), L.i32ptr(st)), "bolt_source_grid")
    _check_status(st, "source_grid")
    res = (SourceGrid(bg.x_grid, k_grid, ST, st), SourceGrid(bg.x_grid, k_grid, SE, st))
    ih._cache = {key: res}
    return res


def source_grid(par, bg, ih, k_grid, integrator=None, lg=8, reltol=1e-11, abstol=1e-6, lnu=None, lmnu=10, nq=None):
    """source_grid(par, bg, ih, k_grid, integrator; ℓᵧ=8, reltol=1e-11)
    (spectra.jl:6-23).  As in the reference the hierarchy is
    Hierarchy(..., k, ℓᵧ) with ℓ_ν = ℓᵧ's default 8, ℓ_mν = 10, nq = 15."""
    lnu = 8 if lnu is None else lnu
    nq = bg.nq if nq is None else nq
    return _source_pair(par, bg, ih, k_grid, lg, lnu, lmnu, nq, reltol, abstol)[0]


def source_grid_P(par, bg, ih, k_grid, integrator=None, lg=8, reltol=1e-11, abstol=1e-6, lnu=None, lmnu=10, nq=None):
    """source_grid_P (spectra.jl:25-42): the polarization source."""
    lnu = 8 if lnu is None else lnu
    nq = bg.nq if nq is None else nq
    return _source_pair(par, bg, ih, k_grid, lg, lnu, lmnu, nq, reltol, abstol)[1]


def quadratic_k(kmin, kmax, nk):
    """quadratic_k (spectra.jl:60-63): kmin + (kmax-kmin)(i/nk)^2, i = 1..nk."""
    i = np.arange(1, nk + 1, dtype=np.float64)
    return kmin + (kmax - kmin) * (i / nk) ** 2


def log10_k(kmin, kmax, nk):
    """log10_k (spectra.jl:65-68)."""
    i = np.arange(1, nk + 1, dtype=np.float64)
    return 10.0 ** (math.log10(kmin) + math.log10(kmax / kmin) * (i - 1) / (nk - 1))


def _cl(ells, ih, sf_t, sf_e, want):
    ells_a = np.ascontiguousarray(np.atleast_1d(ells), dtype=np.int32)
    src = sf_t if sf_t is not None else sf_e
    kg = np.ascontiguousarray(src.k_grid, dtype=np.float64)
    ST = np.ascontiguousarray((sf_t if sf_t is not None else sf_e).S)
    SE = np.ascontiguousarray(sf_e.S) if sf_e is not None else None
    out = {w: np.zeros(ells_a.size) for w in want}
    c = ih.ctx
    c.check(c.lib.bolt_cl(c.h, ih.cosmo_id, L.dptr(ST), L.dptr(SE), L.dptr(kg), kg.size, L.iptr(ells_a), ells_a.size,
                          L.dptr(out.get("tt")), L.dptr(out.get("te")), L.dptr(out.get("ee"))), "bolt_cl")
    return out


def cltt(ells, par, bg, ih, sf):
    """cltt(ℓs, par, bg, ih, sf) (spectra.jl:132-150)."""
    r = _cl(ells, ih, sf, None, ["tt"])["tt"]
    return r if np.ndim(ells) else r[0]


def clte(ells, par, bg, ih, sf, sf_P):
    """clte(ℓs, par, bg, ih, sf, sf_P) (spectra.jl:137-155)."""
    r = _cl(ells, ih, sf, sf_P, ["te"])["te"]
    return r if np.ndim(ells) else r[0]


def clee(ells, par, bg, ih, sf_P):
    """clee(ℓs, par, bg, ih, sf_P) (spectra.jl:142-160).  The E source is
    passed as the polarization grid."""
    ells_a = np.atleast_1d(ells)
    r = _cl(ells_a, ih, sf_P, sf_P, ["ee"])["ee"]
    return r if np.ndim(ells) else r[0]


def cl_all(ells, ih, k_grid, lg=8, lnu=8, lmnu=10, nq=None, reltol=1e-11, abstol=1e-6, spectra=("tt", "te", "ee")):
    """Fused source grid + C_l^TT/TE/EE; the source grids never leave HBM.
    Spectra not named in ``spectra`` come back as None (TT alone skips the
    polarization source)."""
    ells_a = np.ascontiguousarray(np.atleast_1d(ells), dtype=np.int32)
    kg = np.ascontiguousarray(k_grid, dtype=np.float64)
    nq = ih.bg.nq if nq is None else nq
    tt, te, ee = (np.zeros(ells_a.size) if w in spectra else None for w in ("tt", "te", "ee"))
    st = np.zeros(kg.size, dtype=np.int32)
    c = ih.ctx
    c.check(c.lib.bolt_cl_pipeline(c.h, ih.cosmo_id, L.dptr(kg), kg.size, C.byref(_hier(lg, lnu, lmnu, nq)), reltol,
                                   abstol, L.iptr(ells_a), ells_a.size, L.dptr(tt), L.dptr(te), L.dptr(ee),
                                   L.i32ptr(st)), "bolt_cl_pipeline")
    _check_status(st, "cl_all")
    return tt, te, ee, st


def adjoint_check(ih: IonizationHistory, k: float, x: float, hstep: float, lg=8, lnu=8, lmnu=10, nq=15) -> np.ndarray:
    """Residuals of the discrete adjoint's building blocks at one Rosenbrock
    step (bolt_adjoint_check): [0..4] A^T at the stage abscissae, [5] dA/dx
    transposed, [6] the transposed solve, [7] the forward solve, [8] the
    source gradient, [9] the P_lin gradient, [10] the streaming switch,
    [11] the two solves as each other's transposes, [12] the coefficient
    cotangents against tangent arithmetic, [13] the same for d/dx."""
    out = np.zeros(14)
    c = ih.ctx
    c.check(c.lib.bolt_adjoint_check(c.h, ih.cosmo_id, float(k), C.byref(_hier(lg, lnu, lmnu, nq)), float(x),
                                     float(hstep), L.dptr(out)), "bolt_adjoint_check")
    return out


def plin(k, par, bg, ih, n_q=15, lg=50, lnu=50, lmnu=20, x=0.0, reltol=1e-5, abstol=1e-6):
    """plin(k, par, bg, ih, n_q=15, ℓᵧ=50, ℓ_ν=50, ℓ_mν=20, x=0, reltol=1e-5)
    (spectra.jl:163-198); vectorised over k."""
    ks = np.ascontiguousarray(np.atleast_1d(k), dtype=np.float64)
    P = np.zeros(ks.size)
    st = np.zeros(ks.size, dtype=np.int32)
    c = ih.ctx
    c.check(c.lib.bolt_plin(c.h, ih.cosmo_id, L.dptr(ks), ks.size, C.byref(_hier(lg, lnu, lmnu, n_q)), float(x),
                            reltol, abstol, L.dptr(P), L.i32ptr(st)), "bolt_plin")
    _check_status(st, "plin")
    return P if np.ndim(k) else P[0]
