"""The radiation-streaming branch of hierarchy! (perturbations.jl:216-233)
driven on, in the oracle (CPU).

The switch k eta > 240 and -tau' H / eta > 100 holds only for k above
~24 Mpc^-1 at x < -10.75 in the fiducial cosmology, far beyond the
configurations' wavenumbers; k = 30 Mpc^-1 with the solve stopped at
x = -10.7 crosses it.  While it is on, the reference zeroes the photon and
massless-neutrino derivatives and overwrites Theta_0..2 and N_0..2 of the
state (perturbations.jl:217-227); the restatement applies the overwrite to
every accepted state.  Checked: the switch fired; at every output node where
it is on, Theta_2 = N_2 = 0, Theta_0 = Phi - H tau' v_b / k and N_0 = Phi
exactly; between two such nodes inside one switched interval the untouched
radiation multipoles (Theta_3.., Theta^P, N_3..) do not move.
"""
import numpy as np

import oracle as O

K = 30.0
HIER = (8, 8, 10, 15)


def rsa_case(c):
    xo = np.concatenate([np.linspace(-20.0, -11.0, 10), np.linspace(-10.94, -10.76, 10), [-10.7]])
    u, st = c.boltsolve(K, xo, *HIER, reltol=1e-6, abstol=1e-6)
    eta, tp, H = c.table("eta", xo), c.table("taup", xo), c.table("H", xo)
    on = (K * eta > 240.0) & (-tp * H / eta > 100.0)
    return xo, u, st, on, H, tp


def test_rsa_overwrite_in_oracle():
    c = O.Cosmo(O.Params())
    xo, u, st, on, H, tp = rsa_case(c)
    lg, lnu, lmnu, nq = HIER
    iTp, iN = lg + 1, 2 * (lg + 1)
    iPhi = iN + lnu + 1 + (lmnu + 1) * nq
    assert st[2] > 0 and on.sum() >= 3 and not on[-1]
    i = np.where(on)[0]
    assert np.all(u[i, 2] == 0.0) and np.all(u[i, iN + 2] == 0.0)
    np.testing.assert_array_equal(u[i, 0], u[i, iPhi] - H[i] / K * tp[i] * u[i, iPhi + 4])
    np.testing.assert_array_equal(u[i, iN], u[i, iPhi])
    frozen = np.r_[3:lg + 1, iTp:iTp + lg + 1, iN + 3:iN + lnu + 1]
    run = i[np.diff(np.r_[i, -5]) == 1]  # consecutive switched nodes
    assert run.size >= 2
    for j in run:
        np.testing.assert_array_equal(u[j + 1, frozen], u[j, frozen])
    # after the switch turns off the hierarchy evolves again
    assert np.any(u[-1, frozen] != u[i[-1], frozen])
