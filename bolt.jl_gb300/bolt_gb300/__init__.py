"""GB300-native Boltzmann hot path with Bolt.jl's API (see api.py; batched and
served requests in serve.py)."""
from .api import (BasicNewtonian, Background, BoltError, Context, CosmoParams, GPUNewtonian, Hierarchy,
                  adjoint_check,
                  IonizationHistory, Peebles, Perturbation, RECFAST, SourceGrid, boltsolve, boltsolve_batch, boltsolve_rsa,
                  boltsolve_rsa_batch, cl_all, clee,
                  clte, cltt, default_context, host_tables, km_s_Mpc_100, log10_k, mass_natural, plin,
                  quadratic_k, source_grid, source_grid_P, state_len)
from .bessel import (J_moment, MomentTable, integrate_sph_bessel_filon, integrate_sph_bessel_filon_batched,
                     integrate_sph_bessel_filon_piecewise, sph_bessel_interpolator, sph_j_moment)
from .serve import GRAD_SCHEMES, THETA_NAMES, Engine, Request, Result, params_of, theta_of

__all__ = ["BasicNewtonian", "Background", "BoltError", "Context", "CosmoParams", "Engine", "GPUNewtonian",
           "GRAD_SCHEMES", "J_moment", "MomentTable", "adjoint_check", "integrate_sph_bessel_filon",
           "integrate_sph_bessel_filon_batched", "integrate_sph_bessel_filon_piecewise", "sph_bessel_interpolator", "sph_j_moment",
           "Hierarchy", "IonizationHistory", "Peebles", "Perturbation", "RECFAST", "Request", "Result", "SourceGrid",
           "THETA_NAMES", "boltsolve", "boltsolve_batch", "boltsolve_rsa", "boltsolve_rsa_batch", "cl_all", "clee", "clte", "cltt", "default_context",
           "host_tables", "km_s_Mpc_100", "log10_k", "mass_natural", "params_of", "plin", "quadratic_k",
           "source_grid", "source_grid_P", "state_len", "theta_of"]
