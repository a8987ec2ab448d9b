"""imexlbm_gb300: GB300-native IMEXLBM time step (D3Q27 BGK collide + pull
stream on a periodic Taylor-Green lattice), hand-written CUDA for sm_103a
behind a C ABI (include/imexlbm.h).

Python surface:
    System(path="input.in")          deck, as the reference's class System
    LBM(sx, sy, sz, tau, rho0, u0)   one resident lattice, as struct LBM
"""
from ._lib import (IMEX_ROUND_NEAREST, IMEX_ROUND_STOCHASTIC, IMEX_ENGINE_AUTO, IMEX_ENGINE_FIXED, IMEX_ENGINE_NATIVE, IMEX_F16DEV, IMEX_F32, IMEX_F64,
                   ImexError, load)
from .lbm import LBM, Batch, Q, System

__all__ = ["System", "LBM", "Batch", "ImexError", "Q", "load", "IMEX_F64", "IMEX_F32", "IMEX_F16DEV",
           "IMEX_ENGINE_AUTO", "IMEX_ENGINE_NATIVE", "IMEX_ENGINE_FIXED",
           "IMEX_ROUND_NEAREST", "IMEX_ROUND_STOCHASTIC"]
