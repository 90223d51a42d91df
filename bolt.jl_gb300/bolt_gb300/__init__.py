"""GB300-native Boltzmann hot path with Bolt.jl's API (see api.py)."""
from .api import (BasicNewtonian, Background, BoltError, Context, CosmoParams, GPUNewtonian, Hierarchy,
                  IonizationHistory, Perturbation, RECFAST, SourceGrid, boltsolve, boltsolve_batch, cl_all, clee,
                  clte, cltt, default_context, host_tables, km_s_Mpc_100, log10_k, mass_natural, plin,
                  quadratic_k, source_grid, source_grid_P, state_len)

__all__ = ["BasicNewtonian", "Background", "BoltError", "Context", "CosmoParams", "GPUNewtonian", "Hierarchy",
           "IonizationHistory", "Perturbation", "RECFAST", "SourceGrid", "boltsolve", "boltsolve_batch", "cl_all",
           "clee", "clte", "cltt", "default_context", "host_tables", "km_s_Mpc_100", "log10_k", "mass_natural",
           "plin", "quadratic_k", "source_grid", "source_grid_P", "state_len"]
