"""Regenerate the golden fixtures in tests/golden/ from the reference's own
test data (Bolt.jl test/data/*.dat, the known answers of test/testbessel.jl)
and from mpmath.

Run in a checkout that has the reference mounted:
    python tests/golden/make_golden.py /path/to/Bolt.jl
The outputs are small .npz files; the tests read only these.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    data = os.path.join(ref, "test", "data")
    # RECFAST Xe(z) from Fortran RECFAST (runtests.jl:38-48 uses rows 1:end-5)
    d = np.loadtxt(os.path.join(data, "test_recfast_1.dat"), delimiter=",", skiprows=1)
    d = d[:-5]
    np.savez_compressed(os.path.join(HERE, "recfast_fortran.npz"), z=d[::4, 0], xe=d[::4, 1])
    # CLASS perturbations, no massive neutrinos (runtests.jl:83-147)
    out = {}
    for kc in ["p001", "p01", "p03"]:
        rows = [np.array(l.split(), dtype=float)
                for l in open(os.path.join(data, f"zack_N_class_px_k{kc}_nofluid_nonu.dat"))]
        k_hMpc = rows[1][0]
        cls = [r for i, r in enumerate(rows) if i != 1]
        out[f"{kc}_k_hMpc"] = np.array([k_hMpc])
        out[f"{kc}_x"] = cls[0]
        out[f"{kc}_phi"] = cls[6]
        out[f"{kc}_d_b"] = cls[2]
    np.savez_compressed(os.path.join(HERE, "class_nonu.npz"), **out)
    # CAMB unlensed C_l, ell(ell+1)C_l/2pi (runtests.jl:149-185)
    camb = np.loadtxt(os.path.join(data, "camb_rough_ttteee_unlensed.dat"))
    np.savez_compressed(os.path.join(HERE, "camb_rough.npz"), ell=camb[0][:2600], tt=camb[1][:2600],
                        te=camb[2][:2600], ee=camb[3][:2600])
    camb_pk(data)
    bessel_moment_refs(ref)
    # spherical Bessel j_l(x) known answers from mpmath (50 digits)
    import mpmath as mp
    mp.mp.dps = 50
    rng = np.random.default_rng(1234)
    ls = np.array([0, 1, 2, 3, 7, 20, 99, 250, 640, 1000, 1499, 2000, 2500])
    xs = np.concatenate([[0.37, 0.65, 1.0, 2.5, 9.9, 31.4], rng.uniform(0, 3400, 24)])
    vals = np.zeros((len(ls), len(xs)))
    for i, l in enumerate(ls):
        for j, x in enumerate(xs):
            v = mp.sqrt(mp.pi / (2 * mp.mpf(x))) * mp.besselj(int(l) + mp.mpf(1) / 2, mp.mpf(x))
            vals[i, j] = float(v) if abs(v) > mp.mpf("1e-300") else 0.0
    np.savez_compressed(os.path.join(HERE, "sph_bessel_mpmath.npz"), ell=ls, x=xs, j=vals)


def bessel_moment_refs(ref):
    """Known answers of the Bessel-moment and Filon tests (test/testbessel.jl):
    every testset's reference values, in the order they appear, as decimal
    strings (the big"..." literals keep their 30+ digits)."""
    import json
    import re
    src = open(os.path.join(ref, "test", "testbessel.jl")).read()
    parts = re.split(r'@testset\s+"([^"]+)"', src)
    out = {}
    num = r'[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?'
    for name, body in zip(parts[1::2], parts[2::2]):
        vals = []
        for m in re.finditer(r'big"(' + num + r')"|refs\s*=\s*\(([^)]*)\)', body):
            if m.group(1) is not None:
                vals.append(m.group(1))
            elif "big" in m.group(2):
                vals.extend(re.findall(r'big"(' + num + r')"', m.group(2)))
            else:
                vals.extend(v.strip() for v in m.group(2).split(",") if v.strip())
        out[name] = vals
    with open(os.path.join(HERE, "bessel_moment_refs.json"), "w") as fh:
        json.dump(out, fh, indent=1)


def camb_pk(data):
    """CAMB linear P(k) at z = 0 (test/data/camb_pk_x0.dat: k in h/Mpc, P in
    (Mpc/h)^3), made by test/camb_v_class_2022.ipynb for h 0.7, Omega_r
    5.042e-5, Omega_b 0.046, Omega_c 0.224, n_s 1.0, Y_p 0.24, N_eff 3.046,
    Sigma m_nu 0.06 eV, A_s = exp(3.043) 1e-10; every 10th of its 1000 k."""
    d = np.loadtxt(os.path.join(data, "camb_pk_x0.dat"))
    np.savez_compressed(os.path.join(HERE, "camb_pk_x0.npz"), k_hMpc=d[0][::10], pk=d[1][::10])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/Bolt.jl")
    main(sys.argv[1])
