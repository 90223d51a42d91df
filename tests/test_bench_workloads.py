"""The benchmark's synthetic workloads (no GPU): seeded and reproducible,
the serving mix in its stated proportions and parameter box, the batch and
gradient workloads' request structure, and the per-request transfer sizes
the e2e figures are quoted with."""
import importlib.util
import math
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
bench = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(bench)


def _in_box(th):
    h, wb, wc, n, A, mnu = th
    return (0.6 <= h <= 0.8 and 0.019 <= wb <= 0.025 and 0.10 <= wc <= 0.14 and 0.92 <= n <= 1.0
            and 2.9 <= math.log(1e10 * A) <= 3.2 and 0.0 <= mnu <= 0.3)


def test_serving_stream_is_seeded_and_in_proportion():
    a, b = bench.make_stream(40), bench.make_stream(40)
    assert all(x["kind"] == y["kind"] and np.array_equal(x["theta"], y["theta"]) and x["nk"] == y["nk"]
               for x, y in zip(a, b))
    kinds = [d["kind"] for d in a]
    assert kinds.count("plin") == 20 and kinds.count("cl") == 16 and kinds.count("grad") == 4  # 5 : 4 : 1
    for d in a:
        assert _in_box(d["theta"])
        if d["kind"] == "plin":
            assert 100 <= d["nk"] <= 400 and d["hier"] == (50, 50, 20, 15)
        else:
            assert 64 <= d["nk"] <= 1024 and d["hier"][0] in (20, 35, 50) and d["hier"][2] == 10
            assert d["lmax"] == 2000 if d["kind"] == "grad" else d["lmax"] in (1000, 2500)
    # another offset is another draw (warm-up and ranks do not reuse the timed requests)
    c = bench.make_stream(40, offset=1000)
    assert not all(np.array_equal(x["theta"], y["theta"]) for x, y in zip(a, c))


def test_batch_and_gradient_workloads():
    batch = bench.cosmology_requests("batch", 8, 3000)
    assert len(batch) == 8 and all(d["kind"] == "cltt_plin" and d["lmax"] == 2000 for d in batch)
    grad = bench.cosmology_requests("grad", 5, 4000)
    assert len(grad) == 10
    for cl, pl in zip(grad[0::2], grad[1::2]):
        assert cl["kind"] == "grad" and pl["kind"] == "plin_grad"
        assert np.array_equal(cl["theta"], pl["theta"])  # both Jacobians of one cosmology
        assert pl["nk"] == 200 and pl["hier"] == (50, 50, 20, 15)
    assert all(_in_box(d["theta"]) for d in batch + grad)


def test_transfer_sizes_grow_with_the_request():
    small = {"kind": "cl", "nk": 64, "lmax": 1000, "hier": (20, 20, 10, 15)}
    large = {"kind": "cl", "nk": 1024, "lmax": 2500, "hier": (20, 20, 10, 15)}
    grad = {"kind": "grad", "nk": 64, "lmax": 1000, "hier": (20, 20, 10, 15)}
    for a, b in ((small, large), (small, grad)):
        ha, da = bench.io_bytes(a)
        hb, db = bench.io_bytes(b)
        assert 0 < ha < hb and 0 < da < db


def test_solver_flop_count_and_state_length():
    # N = 2(l_gamma + 1) + (l_nu + 1) + (l_mnu + 1) nq + 5 (perturbations.jl:281)
    assert bench.state_len(20, 20, 10, 15) == 233
    assert bench.state_len(50, 50, 20, 15) == 473
    assert bench.solver_flops_per_step(473, 15) == 159 * 473 + 560 * 20 + 66 * 15 + 650


def test_cpu_arm_runs_whole_requests():
    """The CPU oracle runs each request of the stream in full (no sampling or
    scaling model); tiny versions of the three request types here."""
    O = bench._oracle()
    s = bench.make_stream(10)
    for kind in ("plin", "cl", "grad"):
        d = next(x for x in s if x["kind"] == kind)
        d = {**d, "nk": 4, "lmax": 20, "hier": (8, 8, 10, 15) if kind != "plin" else (8, 8, 10, 15)}
        assert bench.oracle_request(O, d, 2) > 0.0
    v, cores, sample = bench.cpu_prefix([{**s[0], "nk": 4, "hier": (8, 8, 10, 15)}], budget_s=0.0)
    assert v > 0 and cores >= 1 and "first 1 requests" in sample


def test_los_flops_from_terms():
    assert bench.los_flops(1000) == 27000.0
    assert bench.los_flops(1000, with_e=False) == 25000.0
    assert bench.SWEEP_RATES == (1.0, 10.0, 100.0, 500.0, 2000.0)


def test_filon_workload():
    """The Filon workload's integrand carries its exact derivatives, and its
    (k, t) products stay inside the moment table's range [0, 1.6e4]."""
    t, f, fp, fpp, k = bench.filon_workload()
    assert t.size == 2001 and k.size == 5000
    assert np.max(k) * np.max(t) <= 1.6e4
    h = 1e-4
    z = lambda s: np.exp(-((s - 1400.0) / 80.0) ** 2) * (1.0 + 0.3 * np.sin(s / 50.0))
    np.testing.assert_allclose(f, z(t), rtol=0, atol=1e-15)
    np.testing.assert_allclose(fp, (z(t + h) - z(t - h)) / (2 * h), rtol=0, atol=1e-9)
    np.testing.assert_allclose(fpp, (z(t + h) - 2 * z(t) + z(t - h)) / h ** 2, rtol=0, atol=1e-6)
