"""imexlbm_gb300: GB300-native IMEXLBM time step (D3Q27 BGK collide + pull
stream on a periodic Taylor-Green lattice), hand-written CUDA for sm_103a
behind a C ABI (include/imexlbm.h).

Python surface:
    System(path="input.in")          deck, as the reference's class System
    LBM(sx, sy, sz, tau, rho0, u0)   one resident lattice, as struct LBM
    Batch(max_members)               many lattices stepped in one launch
    Server(budget_bytes, ...)        continuous-batching request server
    Domain(sx, sy, sz, nranks, ...)  a lattice split into the reference's rank
                                     blocks, with a pruned halo exchange
"""
from ._lib import (IMEX_ENGINE_AUTO, IMEX_ENGINE_FIXED, IMEX_ENGINE_NATIVE, IMEX_ERR_ARG, IMEX_ERR_CUDA,
                   IMEX_ERR_DECK, IMEX_ERR_IO, IMEX_ERR_MEMORY, IMEX_ERR_NONFINITE, IMEX_ERR_STATE, IMEX_F16DEV,
                   IMEX_F32, IMEX_F64, IMEX_OK, IMEX_POLICY_ARRIVAL, IMEX_POLICY_LEAST_WORK, IMEX_ROUND_NEAREST,
                   IMEX_ROUND_STOCHASTIC, IMEX_TEST_FAULT_BATCH_TABLE, IMEX_TEST_FAULT_NONE,
                   IMEX_TEST_FAULT_STARVE_STAGE, ImexError, load)
from .lbm import LBM, Batch, Domain, Q, Server, System, decomp_block, decomp_grid, decomp_halo

__all__ = ["System", "LBM", "Batch", "Server", "Domain", "decomp_grid", "decomp_block", "decomp_halo", "ImexError", "Q", "load", "IMEX_F64", "IMEX_F32", "IMEX_F16DEV",
           "IMEX_ENGINE_AUTO", "IMEX_ENGINE_NATIVE", "IMEX_ENGINE_FIXED",
           "IMEX_ROUND_NEAREST", "IMEX_ROUND_STOCHASTIC", "IMEX_OK", "IMEX_ERR_ARG", "IMEX_ERR_CUDA",
           "IMEX_ERR_MEMORY", "IMEX_ERR_DECK", "IMEX_ERR_NONFINITE", "IMEX_ERR_STATE", "IMEX_ERR_IO",
           "IMEX_POLICY_ARRIVAL", "IMEX_POLICY_LEAST_WORK", "IMEX_TEST_FAULT_NONE", "IMEX_TEST_FAULT_STARVE_STAGE",
           "IMEX_TEST_FAULT_BATCH_TABLE"]
