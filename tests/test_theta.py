"""theta = (h, omega_b, omega_c, n_s, A_s, Sigma m_nu [eV]) <-> CosmoParams."""
import numpy as np

import bolt_gb300 as B


def test_theta_round_trip():
    par = B.CosmoParams(h=0.68, Omega_b=0.049, Omega_c=0.26, n=0.965, A=2.2e-9,
                        Sigma_m_nu=0.1 * B.mass_natural())
    th = B.theta_of(par)
    assert np.allclose(th, [0.68, 0.049 * 0.68 ** 2, 0.26 * 0.68 ** 2, 0.965, 2.2e-9, 0.1], rtol=1e-14)
    back = B.params_of(par, th)
    for f in ("h", "Omega_b", "Omega_c", "n", "A", "Sigma_m_nu", "Omega_r", "Y_p", "N_nu"):
        assert abs(getattr(back, f) - getattr(par, f)) <= 1e-14 * abs(getattr(par, f)), f
