"""Batched and served requests through the library's native engine.

A request is one cosmology with its own k grid, hierarchy and outputs:
``plin`` (src/spectra.jl:163-198) or ``cl`` (source_grid + cltt / clte / clee,
src/spectra.jl:6-160), optionally with the Jacobian with respect to
theta = (h, omega_b, omega_c, n_s, A_s, Sigma m_nu [eV]) (``grad=True``; the
rrule of the Julia binding).  ``Engine.submit`` returns at once; the engine's
scheduler thread batches the requests whose tables are ready (continuous
batching on several streams, admission by a device-memory budget) and
``Engine.wait`` returns the result.  ``Engine.run`` is the one-request-per-call
path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .api import CosmoParams, mass_natural

THETA_NAMES = ("h", "omega_b", "omega_c", "n_s", "A_s", "Sigma_m_nu_eV")
# Engine grad_scheme values (bolt_engine_cfg.grad_scheme): frozen-step
# replays, the tangent-linear solver, the discrete adjoint for pullbacks.
GRAD_SCHEMES = ("replay", "tangent", "adjoint")
_CL_BITS = {"tt": 1, "te": 2, "ee": 4}


def theta_of(par: CosmoParams) -> np.ndarray:
    """theta = (h, Omega_b h^2, Omega_c h^2, n, A, Sigma m_nu in eV)."""
    return np.array([par.h, par.Omega_b * par.h ** 2, par.Omega_c * par.h ** 2, par.n, par.A,
                     par.Sigma_m_nu / mass_natural()])


def params_of(base: CosmoParams, theta) -> CosmoParams:
    """CosmoParams at theta, Omega_r / Y_p / N_nu taken from base."""
    h, wb, wc, n, A, mnu = (float(v) for v in theta)
    return CosmoParams(h=h, Omega_r=base.Omega_r, Omega_b=wb / h ** 2, Omega_c=wc / h ** 2, A=A, n=n,
                       Y_p=base.Y_p, N_nu=base.N_nu, Sigma_m_nu=mnu * mass_natural())


@dataclass
class Request:
    kind: str                      # "plin" or "cl"
    par: CosmoParams
    k: np.ndarray                  # Mpc^-1, ascending
    grad: bool = False
    hier: tuple = (50, 50, 20, 15)  # (l_gamma, l_nu, l_mnu, nq)
    x_grid: tuple = (-20.0, 0.01, 0.0)
    reltol: float = 1e-8
    abstol: float = 3e-7
    plin_x: float = 0.0
    ells: np.ndarray | None = None
    cl: tuple = ("tt",)             # any of "tt", "te", "ee"
    with_plin: bool = False         # "cl": also P_lin(k) at the end of the x grid from the same solve


@dataclass
class Result:
    rc: int
    err: str
    times: np.ndarray               # submitted, tables ready, launched, completed (s since engine start), steps
    status: np.ndarray
    plin: np.ndarray | None = None
    dplin: np.ndarray | None = None  # [6][nk]
    cl: dict = field(default_factory=dict)   # "tt" -> [nell]
    dcl: dict = field(default_factory=dict)  # "tt" -> [6][nell]

    @property
    def latency(self) -> float:
        return float(self.times[3] - self.times[0])

    @property
    def steps(self) -> int:
        return int(self.times[4])


class _Pending:
    def __init__(self, req: Request):
        self.req = req
        k = np.ascontiguousarray(req.k, dtype=np.float64)
        self.k = k
        lg, lnu, lmnu, nq = req.hier
        c = L.BoltRequest()
        c.kind = 1 if req.kind == "plin" else 2
        c.grad = 1 if req.grad else 0
        c.par = req.par.c()
        c.grid = L.BoltGrid(*req.x_grid)
        c.nq = nq
        c.hier = L.BoltHier(lg, lnu, lmnu, nq)
        c.reltol, c.abstol = req.reltol, req.abstol
        c.k = L.dptr(k)
        c.nk = k.size
        c.plin_x = req.plin_x
        self.status = np.zeros(k.size, dtype=np.int32)
        c.status = L.i32ptr(self.status)
        self.out = {}
        if req.kind == "plin" or req.with_plin:
            self.out["plin"] = np.zeros(k.size)
            c.plin = L.dptr(self.out["plin"])
            if req.grad:
                self.out["dplin"] = np.zeros((6, k.size))
                c.dplin = L.dptr(self.out["dplin"])
        if req.kind != "plin":
            ells = np.ascontiguousarray(req.ells, dtype=np.int32)
            self.ells = ells
            c.ells = L.iptr(ells)
            c.nell = ells.size
            want = 0
            for q in req.cl:
                want |= _CL_BITS[q]
                self.out[q] = np.zeros(ells.size)
                setattr(c, q, L.dptr(self.out[q]))
                if req.grad:
                    self.out["d" + q] = np.zeros((6, ells.size))
                    setattr(c, "d" + q, L.dptr(self.out["d" + q]))
            c.cl_want = want
        self.c = c

    def result(self, rc, err, times) -> Result:
        r = Result(rc=rc, err=err, times=times, status=self.status)
        r.plin = self.out.get("plin")
        r.dplin = self.out.get("dplin")
        if self.req.kind != "plin":
            for q in self.req.cl:
                r.cl[q] = self.out[q]
                if self.req.grad:
                    r.dcl[q] = self.out["d" + q]
        return r


class Engine:
    """Native batching / serving engine on one GPU (bolt_engine_*)."""

    def __init__(self, device: int = 0, lanes: int = 6, host_threads: int = 0, max_batch: int = 0,
                 mem_budget_gb: float = 150.0, warps_per_mode: int = 0, max_steps: int = 0,
                 batch_window_s: float = 0.0, objective: str = "latency", land_stride: int = 1,
                 grad_scheme: str = "replay"):
        if objective not in ("latency", "throughput"):
            raise ValueError("objective is 'latency' or 'throughput'")
        if grad_scheme not in GRAD_SCHEMES:
            raise ValueError("grad_scheme is one of " + ", ".join(GRAD_SCHEMES))
        self.lib = L.load()
        cfg = L.BoltEngineCfg(device, lanes, host_threads, max_batch, mem_budget_gb, warps_per_mode, max_steps,
                              batch_window_s, 1 if objective == "throughput" else 0, land_stride,
                              GRAD_SCHEMES.index(grad_scheme))
        h = C.c_void_p()
        rc = self.lib.bolt_engine_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"bolt_engine_create failed ({rc})")
        self.h = h
        self._pending = {}

    def submit(self, req: Request) -> int:
        p = _Pending(req)
        t = C.c_int64(0)
        rc = self.lib.bolt_engine_submit(self.h, C.byref(p.c), C.byref(t))
        if rc != 0:
            raise ValueError(f"bolt_engine_submit: {self.lib.bolt_engine_last_error(self.h).decode()} ({rc})")
        self._pending[t.value] = p
        return t.value

    def wait(self, ticket: int, timeout: float | None = None) -> Result | None:
        p = self._pending[ticket]
        rc = C.c_int(0)
        times = np.zeros(5)
        err = C.create_string_buffer(512)
        done = self.lib.bolt_engine_wait(self.h, ticket, -1.0 if timeout is None else float(timeout), C.byref(rc),
                                         L.dptr(times), err, 512)
        if done == 0:
            return None
        if done < 0:
            raise KeyError(f"unknown ticket {ticket}")
        del self._pending[ticket]
        return p.result(rc.value, err.value.decode(), times)

    def run(self, req: Request) -> Result:
        """One request alone (submit + wait)."""
        return self.wait(self.submit(req))

    def vjp(self, req: Request, ybar) -> tuple[Result, np.ndarray]:
        """Pullback of the rrule (bolt_cl_vjp / bolt_plin_vjp): the request
        alone with its Jacobian, contracted with the cotangents ``ybar`` --
        for C_l a dict spectrum -> [nell] (missing spectra count as zero), for
        P_lin an array [nk].  Returns (result with the primal outputs, grad[6]
        with respect to theta)."""
        q = Request(**{**req.__dict__, "grad": False})
        p = _Pending(q)
        grad = np.zeros(6)
        err = C.create_string_buffer(512)
        if req.kind == "plin":
            yb = np.ascontiguousarray(ybar, dtype=np.float64)
            if yb.shape != (p.k.size,):
                raise ValueError("ybar needs one entry per wavenumber")
            rc = self.lib.bolt_plin_vjp(self.h, C.byref(p.c), L.dptr(yb), L.dptr(grad), err, 512)
        else:
            yb = {}
            for c, v in dict(ybar).items():
                if c not in req.cl:
                    raise ValueError(f"cotangent for {c!r}, which the request does not compute")
                yb[c] = np.ascontiguousarray(v, dtype=np.float64)
                if yb[c].shape != (p.ells.size,):
                    raise ValueError("ybar needs one entry per multipole")
            rc = self.lib.bolt_cl_vjp(self.h, C.byref(p.c), L.dptr(yb.get("tt")), L.dptr(yb.get("te")),
                                      L.dptr(yb.get("ee")), L.dptr(grad), err, 512)
        return p.result(rc, err.value.decode(), np.zeros(5)), grad

    def stats(self) -> dict:
        out = np.zeros(12, dtype=np.int64)
        self.lib.bolt_engine_stats(self.h, out.ctypes.data_as(C.POINTER(C.c_int64)))
        keys = ["batches", "requests", "modes", "solver_us", "los_us", "steps", "kernel_launches",
                "graph_launches", "batches_wpm1", "batches_wpm2", "batches_wpm4", "peak_inflight_bytes"]
        return dict(zip(keys, (int(v) for v in out)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.bolt_engine_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
