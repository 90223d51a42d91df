"""Moments of spherical Bessel functions, their interpolation table and the
Filon-type integrator (Bolt.jl src/bessel/), computed on the GPU through the
C ABI (bolt_sph_j_moment, bolt_moment_table_*, bolt_filon*).

    sph_j_moment_asymp / _weniger_1F2 / _maclaurin_1F2  moments.jl:56-92  -> sph_j_moment
    J_moment_asymp / J_moment_weniger_1F2              moments.jl:23-36  -> J_moment (half-integer orders)
    sph_bessel_interpolator(nu, order, kmin, kmax, N)  interpolator.jl:81-94 -> MomentTable
    integrate_sph_bessel_filon(f, f', f'', k, a, b, itp)  integrator.jl:7-19 -> integrate_sph_bessel_filon
    _loop_integrate_sph_bessel_filon (summed)          integrator.jl:25-38 -> integrate_sph_bessel_filon_piecewise
    (one integrand per k on shared nodes, the line-of-sight shape)          -> integrate_sph_bessel_filon_batched
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .api import Context, default_context


def _arr(v):
    return np.ascontiguousarray(np.atleast_1d(np.asarray(v, dtype=np.float64)))


def sph_j_moment(x, nu: int, m: float, ctx: Context | None = None):
    """int_0^x t^m j_nu(t) dt, elementwise over x (a scalar for a scalar)."""
    ctx = ctx or default_context()
    xa = _arr(x)
    out = np.zeros(xa.size)
    ctx.check(ctx.lib.bolt_sph_j_moment(ctx.h, int(nu), float(m), L.dptr(xa), xa.size, L.dptr(out)),
              "bolt_sph_j_moment")
    return float(out[0]) if np.ndim(x) == 0 else out


def J_moment(x, nu: float, alpha: float, ctx: Context | None = None):
    """int_0^x t^alpha J_nu(t) dt for half-integer nu = n + 1/2: sqrt(2/pi)
    times the spherical moment of order alpha + 1/2."""
    n = int(round(nu - 0.5))
    if abs(n + 0.5 - nu) > 1e-12:
        raise ValueError("J_moment: half-integer orders only")
    v = sph_j_moment(x, n, alpha + 0.5, ctx)
    return np.sqrt(2.0 / np.pi) * v


class MomentTable:
    """sph_bessel_interpolator(nu, order, kmin, kmax, N): the moments
    m = 0..order-1 on N uniform nodes of [kmin, kmax], cubic B-splines,
    resident on the GPU.  ``table(x)`` evaluates them (interpolator.jl:67-75):
    the splines inside the range, the Lommel form above, the series below."""

    def __init__(self, nu: int, order: int, kmin: float, kmax: float, N: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.nu, self.order, self.kmin, self.kmax, self.N = int(nu), int(order), float(kmin), float(kmax), int(N)
        tid = C.c_int(-1)
        self.ctx.check(self.ctx.lib.bolt_moment_table_build(self.ctx.h, self.nu, self.order, self.kmin, self.kmax,
                                                            self.N, C.byref(tid)), "bolt_moment_table_build")
        self.id = tid.value

    def __call__(self, x):
        xa = _arr(x)
        out = np.zeros((xa.size, self.order))
        self.ctx.check(self.ctx.lib.bolt_moment_table_eval(self.ctx.h, self.id, L.dptr(xa), xa.size, L.dptr(out)),
                       "bolt_moment_table_eval")
        return out[0] if np.ndim(x) == 0 else out

    def close(self):
        if getattr(self, "id", -1) >= 0 and getattr(self.ctx, "h", None) and self.ctx.h.value:
            self.ctx.lib.bolt_moment_table_free(self.ctx.h, self.id)
        self.id = -1

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sph_bessel_interpolator(nu: int, order: int, kmin: float, kmax: float, N: int,
                            ctx: Context | None = None) -> MomentTable:
    return MomentTable(nu, order, kmin, kmax, N, ctx)


def integrate_sph_bessel_filon(f, fp, fpp, k, a, b, itp: MomentTable):
    """int_a^b p(t) j_nu(k t) dt for the quadratic p with p(a) = f,
    p'(a) = fp, p'' = fpp; elementwise over broadcast arguments."""
    args = np.broadcast_arrays(*[np.asarray(v, dtype=np.float64) for v in (f, fp, fpp, k, a, b)])
    flat = [np.ascontiguousarray(v.ravel()) for v in args]
    n = flat[0].size
    out = np.zeros(n)
    c = itp.ctx
    c.check(c.lib.bolt_filon(c.h, itp.id, n, *[L.dptr(v) for v in flat], L.dptr(out)), "bolt_filon")
    return float(out[0]) if args[0].ndim == 0 else out.reshape(args[0].shape)


def integrate_sph_bessel_filon_piecewise(t, f, fp, fpp, k, itp: MomentTable):
    """For every k: the sum over consecutive segments [t_i, t_{i+1}] of the
    Filon integral of the quadratic at t_i (f, fp, fpp sampled on t)."""
    t, f, fp, fpp = (np.ascontiguousarray(v, dtype=np.float64) for v in (t, f, fp, fpp))
    if not (t.shape == f.shape == fp.shape == fpp.shape):
        raise ValueError("t, f, fp, fpp must have one shape")
    ka = _arr(k)
    out = np.zeros(ka.size)
    c = itp.ctx
    c.check(c.lib.bolt_filon_piecewise(c.h, itp.id, t.size, L.dptr(t), L.dptr(f), L.dptr(fp), L.dptr(fpp), ka.size,
                                       L.dptr(ka), L.dptr(out)), "bolt_filon_piecewise")
    return float(out[0]) if np.ndim(k) == 0 else out


def integrate_sph_bessel_filon_batched(t, f, fp, fpp, k, itp: MomentTable):
    """One integrand per k: f, fp, fpp of shape (nk, nt) on the shared nodes
    t; returns, for every k, the sum over segments of the Filon integral of
    that k's quadratic at t_i."""
    t = np.ascontiguousarray(t, dtype=np.float64)
    ka = _arr(k)
    f, fp, fpp = (np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (ka.size, t.size)))
                  for v in (f, fp, fpp))
    out = np.zeros(ka.size)
    c = itp.ctx
    c.check(c.lib.bolt_filon_batched(c.h, itp.id, t.size, L.dptr(t), L.dptr(f), L.dptr(fp), L.dptr(fpp), ka.size,
                                     L.dptr(ka), L.dptr(out)), "bolt_filon_batched")
    return out
