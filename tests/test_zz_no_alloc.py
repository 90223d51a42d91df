"""The allocation-free source grid (bolt_source_grid_static) against the
regular entry point (bolt_cosmo_upload + bolt_source_grid).

bolt_source_grid_static serves callers that cannot allocate device memory
themselves (code running under another framework's allocator, or hosts that
forbid cudaMalloc after start-up): it takes host inputs and caller-owned
device outputs, and keeps every other buffer in one fixed device array.
Here the caller's device buffers come from torch.  Two calls in a row must
both reproduce the regular entry point's source grid (same kernel, same
tables) within 1e-10 of the grid's peak, also at the array's largest
momentum-bin count (nq = 27) with a state length near its limit (N = 509,
where the grid is clamped to the array's 320 solver slabs); calls beyond the
array's limits (N > 512, more than 2048 wavenumbers, more than 4097 x nodes)
must be rejected.
"""
import ctypes as C

import numpy as np
import pytest

import bolt_gb300 as B
from bolt_gb300 import _lib as L

pytestmark = pytest.mark.gpu

PRIMARY = [0, 3, 6, 7, 8, 11, 14, 15]  # H, eta, rho0M, Xe, tau, g, Tmat, csb2


def _inputs(nq=15, grid=(-20.0, 0.01, 0.0)):
    par = B.CosmoParams(n=0.96, A=2.1e-9)
    nodes16, sc = B.host_tables(par, grid, nq)
    nodes = np.ascontiguousarray(nodes16[PRIMARY])
    scal = np.ascontiguousarray(sc[:3])
    return par, grid, nodes, scal


def _reference(par, grid, nodes, scal, ks, hier):
    ctx = B.Context()
    cid = C.c_int(-1)
    g = L.BoltGrid(*grid)
    ctx.check(ctx.lib.bolt_cosmo_upload(ctx.h, C.byref(par.c()), C.byref(g), hier.nq, L.dptr(nodes), L.dptr(scal),
                                        C.byref(cid)), "bolt_cosmo_upload")
    n = nodes.shape[1]
    ST = np.zeros((ks.size, n))
    SE = np.zeros((ks.size, n))
    st = np.zeros(ks.size, dtype=np.int32)
    ctx.check(ctx.lib.bolt_source_grid(ctx.h, cid.value, L.dptr(ks), ks.size, C.byref(hier), 1e-8, 1e-6, L.dptr(ST),
                                       L.dptr(SE), L.i32ptr(st)), "bolt_source_grid")
    ctx.close()
    return ST, SE, st


def _static_call(lib, par, grid, nodes, scal, ks, hier, dST, dSE, dst):
    import torch
    err = C.create_string_buffer(256)
    rc = lib.bolt_source_grid_static(C.byref(par.c()), C.byref(L.BoltGrid(*grid)), hier.nq, L.dptr(nodes), L.dptr(scal),
                                     L.dptr(ks), ks.size, C.byref(hier), 1e-8, 1e-6, C.c_void_p(dST.data_ptr()),
                                     C.c_void_p(dSE.data_ptr()), C.c_void_p(dst.data_ptr()), None, err, 256)
    torch.cuda.synchronize()
    return rc, err.value.decode()


@pytest.mark.parametrize("hier_t,nk,kmax", [((8, 8, 10, 15), 16, 1000.0), ((68, 68, 10, 27), 8, 100.0)],
                         ids=["N101_nq15", "N509_nq27"])
def test_static_source_grid_matches_regular_entry_point(hier_t, nk, kmax):
    torch = pytest.importorskip("torch")
    lib = L.load()
    par, grid, nodes, scal = _inputs(nq=hier_t[3])
    ks = B.log10_k(0.1 * 2.33e-4, kmax * 2.33e-4, nk)
    hier = L.BoltHier(*hier_t)
    assert B.state_len(*hier_t) <= 512
    ST, SE, st = _reference(par, grid, nodes, scal, ks, hier)
    assert np.all((st & 0xFF) == 0)
    n = nodes.shape[1]
    dST = torch.empty((ks.size, n), dtype=torch.float64, device="cuda")
    dSE = torch.empty((ks.size, n), dtype=torch.float64, device="cuda")
    dst = torch.empty(ks.size, dtype=torch.int32, device="cuda")
    fin = np.isfinite(SE)
    for call in range(2):
        dST.fill_(np.nan)
        dSE.fill_(np.nan)
        rc, msg = _static_call(lib, par, grid, nodes, scal, ks, hier, dST, dSE, dst)
        assert rc == 0, msg
        gT, gE, gs = dST.cpu().numpy(), dSE.cpu().numpy(), dst.cpu().numpy()
        assert np.array_equal(gs, st), call
        assert np.max(np.abs(gT - ST)) <= 1e-10 * np.max(np.abs(ST)), call
        assert np.array_equal(np.isfinite(gE), fin), call
        assert np.max(np.abs(gE[fin] - SE[fin])) <= 1e-10 * np.max(np.abs(SE[fin])), call


def test_static_source_grid_rejects_oversized_state():
    torch = pytest.importorskip("torch")
    lib = L.load()
    par, grid, nodes, scal = _inputs()
    ks = np.array([0.01])
    hier = L.BoltHier(120, 120, 10, 15)  # N = 533 > 512
    n = nodes.shape[1]
    dST = torch.empty((1, n), dtype=torch.float64, device="cuda")
    dSE = torch.empty((1, n), dtype=torch.float64, device="cuda")
    dst = torch.empty(1, dtype=torch.int32, device="cuda")
    rc, msg = _static_call(lib, par, grid, nodes, scal, ks, hier, dST, dSE, dst)
    assert rc != 0 and "512" in msg


@pytest.mark.parametrize("what", ["modes", "grid"])
def test_static_source_grid_rejects_too_many_modes_or_nodes(what):
    torch = pytest.importorskip("torch")
    lib = L.load()
    if what == "modes":
        par, grid, nodes, scal = _inputs()
        ks = B.log10_k(1e-4, 1e-1, 2049)
    else:  # 4098 nodes: one past the array's x-grid limit
        par, grid, nodes, scal = _inputs(grid=(-20.0, 20.0 / 4097, 0.0))
        assert nodes.shape[1] == 4098
        ks = np.array([0.01])
    hier = L.BoltHier(8, 8, 10, 15)
    n = nodes.shape[1]
    dST = torch.empty((ks.size, n), dtype=torch.float64, device="cuda")
    dSE = torch.empty((ks.size, n), dtype=torch.float64, device="cuda")
    dst = torch.empty(ks.size, dtype=torch.int32, device="cuda")
    rc, msg = _static_call(lib, par, grid, nodes, scal, ks, hier, dST, dSE, dst)
    assert rc != 0 and ("2048" if what == "modes" else "4097") in msg
