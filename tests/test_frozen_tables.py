"""Host tables on a frozen RECFAST discretisation (bolt_host_tables_frozen),
the building block of the engine's gradients: identical to the regular
build at the base point, and a smooth function of the parameters around it
(central differences with steps 1e-4 and 1e-5 agree), which the regular,
re-discretised build is not at this resolution."""
import ctypes as C

import numpy as np

import bolt_gb300 as B
from bolt_gb300 import _lib as L

GRID = (-20.0, 0.01, 0.0)
NAMES = B.api.TABLE_NAMES


def _rf(par):
    return L.BoltRecfast(par.Y_p, par.Omega_b, par.Omega_r, -1.0, 1e-8)


def _frozen(base, par):
    lib = L.load()
    n = int(round((GRID[2] - GRID[0]) / GRID[1])) + 1
    out = np.zeros((16, n))
    err = C.create_string_buffer(256)
    rc = lib.bolt_host_tables_frozen(C.byref(base.c()), C.byref(par.c()), C.byref(L.BoltGrid(*GRID)), 15,
                                     C.byref(_rf(base)), C.byref(_rf(par)), L.dptr(out), err, 256)
    assert rc == 0, err.value
    return out


def _theta_par(base, j, d):
    th = B.theta_of(base)
    th[j] += d
    return B.params_of(base, th)


def test_frozen_equals_regular_at_base():
    base = B.params_of(B.CosmoParams(), [0.7, 0.0224, 0.12, 0.96, 2.1e-9, 0.06])
    nodes, _ = B.host_tables(base, GRID, 15)
    assert np.array_equal(_frozen(base, base), nodes)


def test_frozen_tables_are_smooth_in_theta():
    base = B.params_of(B.CosmoParams(), [0.7, 0.0224, 0.12, 0.96, 2.1e-9, 0.06])
    th = B.theta_of(base)
    xe, g = NAMES.index("Xe"), NAMES.index("g")
    for j in (0, 1, 2, 5):  # h, omega_b, omega_c, Sigma m_nu
        ds = []
        for rel in (1e-4, 1e-5):
            d = rel * abs(th[j])
            ds.append((_frozen(base, _theta_par(base, j, d)) - _frozen(base, _theta_par(base, j, -d))) / (2 * d))
        for t in (xe, g):
            scale = np.max(np.abs(ds[0][t]))
            assert np.max(np.abs(ds[0][t] - ds[1][t])) < 1e-4 * scale, (B.THETA_NAMES[j], NAMES[t])
