"""The Saha-Peebles ionization history (no GPU).

The reference exports `Peebles` but never defines it (Bolt.jl:6); its
Peebles code is `saha_peebles_recombination` (ionization.jl:83-93: the Saha
equation for hydrogen until z = 1587.4, then the Peebles equation by Tsit5 at
1e-11) and `customion` (ionization.jl:141-164), which makes an
IonizationHistory from X_e, T_mat and c_s^2 functions of the caller.  The
library's `ionization = 1` (Python: `B.Peebles()`) takes T_mat = 2.725 K
(1 + z), the T_b of the Saha and Peebles equations, and RECFAST's
sound-speed formula on it.  Checked here: every host-built ionization table
against the oracle's independent restatement (1e-10 of each table's scale;
the background's 1e-9, as for RECFAST histories); X_e is 1 in
the Saha era, continuous at the switch, and within the few per cent of
RECFAST that separate the two physics around recombination; no
reionization, so tau_0 is that of the recombination era alone.
"""
import numpy as np

import bolt_gb300 as B
import oracle as O


def test_host_tables_match_oracle_peebles():
    for par, op in ((B.CosmoParams(), O.Params()),
                    (B.CosmoParams(h=0.68, Omega_b=0.049, Omega_c=0.26, Sigma_m_nu=0.1 * B.mass_natural()),
                     O.Params(h=0.68, Omega_b=0.049, Omega_c=0.26, Sigma_m_nu_eV=0.1))):
        nodes, sc = B.host_tables(par, ionization="peebles")
        o = O.Cosmo(op, ionization="peebles")
        for i, nm in enumerate(O.TABLES):
            ref = o.table(nm)
            tol = 1e-10 if i >= 7 else 1e-9  # ionization tables; the background's re-splined derivatives
            assert np.max(np.abs(nodes[i] - ref)) <= tol * np.max(np.abs(ref)), nm


def test_saha_peebles_physics():
    o = O.Cosmo(O.Params(), ionization="peebles")
    r = O.Cosmo(O.Params())
    x = o.x
    z = 1.0 / np.exp(x) - 1.0
    xe = o.table("Xe")
    assert np.all(np.abs(xe[z > 3000] - 1.0) < 1e-6)  # fully ionized hydrogen (no helium in Saha)
    ztr = 1587.4
    i = np.searchsorted(-z, -ztr)  # first node past the switch
    assert abs(xe[i] - xe[i - 1]) < 0.01  # continuous through the switch
    win = (z > 800) & (z < 1500)
    xr = r.table("Xe")
    assert np.max(np.abs(xe[win] / xr[win] - 1)) < 0.05  # within 5 % of RECFAST
    assert np.all(np.diff(xe[z < 1500]) <= 1e-12)  # recombination only: X_e falls
    assert xe[-1] < 1e-3  # no reionization
    tm = o.table("Tmat")
    np.testing.assert_allclose(tm, 2.725 * (1 + z), rtol=1e-14)
