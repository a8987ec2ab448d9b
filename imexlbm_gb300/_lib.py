"""ctypes binding of libimexlbm.so (the C ABI in include/imexlbm.h).

The library is built in-tree by ``imexlbm_gb300.build``.  There is no
fallback: if the shared library is missing, loading raises ``ImportError``
with the build command, and every compute call goes to the CUDA kernels.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

IMEX_OK = 0
IMEX_ERR_ARG = 1
IMEX_ERR_CUDA = 2
IMEX_ERR_MEMORY = 3
IMEX_ERR_DECK = 4
IMEX_ERR_NONFINITE = 5
IMEX_ERR_STATE = 6
IMEX_ERR_IO = 7

IMEX_F64 = 0
IMEX_F32 = 1
IMEX_F16DEV = 2

IMEX_ROUND_NEAREST = 0
IMEX_ROUND_STOCHASTIC = 1

IMEX_ENGINE_AUTO = 0
IMEX_ENGINE_NATIVE = 1
IMEX_ENGINE_FIXED = 2

IMEX_TEST_FAULT_NONE = 0
IMEX_TEST_FAULT_STARVE_STAGE = 1
IMEX_TEST_FAULT_BATCH_TABLE = 2

# Every symbol include/imexlbm.h declares, with (restype, argtypes).
_dp = ctypes.POINTER(ctypes.c_double)
_h = ctypes.c_void_p


IMEX_POLICY_ARRIVAL = 0
IMEX_POLICY_LEAST_WORK = 1

IMEX_PHASE_COLLISION = 0
IMEX_PHASE_STREAM = 1
IMEX_PHASE_MACRO = 2
IMEX_PHASE_CONSERVED = 3
IMEX_NPHASE = 4


class PhaseStats(ctypes.Structure):
    _fields_ = [("calls", ctypes.c_int64), ("total_ms", ctypes.c_double), ("min_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double)]


class Deck(ctypes.Structure):
    """struct imex_deck (include/imexlbm.h)."""

    _fields_ = [
        ("rho0", ctypes.c_double), ("R", ctypes.c_double), ("u0", ctypes.c_double),
        ("Re", ctypes.c_int), ("Time", ctypes.c_int), ("inter", ctypes.c_int),
        ("sx", ctypes.c_int), ("sy", ctypes.c_int), ("sz", ctypes.c_int),
        ("cs2", ctypes.c_double), ("cs", ctypes.c_double), ("Ma", ctypes.c_double),
        ("miu", ctypes.c_double), ("tau", ctypes.c_double),
    ]


class Request(ctypes.Structure):
    """struct imex_request (include/imexlbm.h)."""

    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("precision", ctypes.c_int), ("rounding", ctypes.c_int), ("pad", ctypes.c_int),
                ("tau", ctypes.c_double), ("rho0", ctypes.c_double), ("u0", ctypes.c_double),
                ("phase", ctypes.c_double * 3), ("steps", ctypes.c_int64), ("tag", ctypes.c_int64),
                ("resume_path", ctypes.c_char * 256), ("save_path", ctypes.c_char * 256)]


class Result(ctypes.Structure):
    """struct imex_result (include/imexlbm.h)."""

    _fields_ = [("id", ctypes.c_int64), ("tag", ctypes.c_int64), ("status", ctypes.c_int), ("pad", ctypes.c_int),
                ("conserved", ctypes.c_double * 5), ("steps", ctypes.c_int64), ("cells", ctypes.c_int64),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    """struct imex_server_stats (include/imexlbm.h)."""

    _fields_ = [("queued", ctypes.c_int64), ("active", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("bytes_in_use", ctypes.c_int64), ("cell_updates", ctypes.c_int64), ("ticks", ctypes.c_int64),
                ("busy_seconds", ctypes.c_double), ("now", ctypes.c_double), ("failed", ctypes.c_int64)]


class Block(ctypes.Structure):
    """struct imex_block (include/imexlbm.h)."""

    _fields_ = [("rank", ctypes.c_int), ("coord", ctypes.c_int * 3), ("lo", ctypes.c_int * 3),
                ("len", ctypes.c_int * 3)]


class HaloMsg(ctypes.Structure):
    """struct imex_halo_msg (include/imexlbm.h)."""

    _fields_ = [("channel", ctypes.c_int), ("offset", ctypes.c_int * 3), ("send_to", ctypes.c_int),
                ("recv_from", ctypes.c_int), ("send_lo", ctypes.c_int * 3), ("recv_lo", ctypes.c_int * 3),
                ("ext", ctypes.c_int * 3), ("ndir", ctypes.c_int), ("dirs", ctypes.c_int * 9)]


class DomainStats(ctypes.Structure):
    """struct imex_domain_stats (include/imexlbm.h)."""

    _fields_ = [("nranks", ctypes.c_int), ("grid", ctypes.c_int * 3), ("steps", ctypes.c_int64),
                ("launches", ctypes.c_int64), ("halo_values_per_step", ctypes.c_int64),
                ("device_bytes", ctypes.c_int64)]


SIGNATURES = {
    "imex_deck_parse": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Deck)]),
    "imex_deck_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Deck)]),
    "imex_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "imex_destroy": (None, [_h]),
    "imex_initialize": (ctypes.c_int, [_h]),
    "imex_collision": (ctypes.c_int, [_h]),
    "imex_streaming": (ctypes.c_int, [_h]),
    "imex_step": (ctypes.c_int, [_h, ctypes.c_int]),
    "imex_conserved": (ctypes.c_int, [_h, _dp]),
    "imex_macroscopic": (ctypes.c_int, [_h, _dp, _dp, _dp, _dp]),
    "imex_velocity_max_diff": (ctypes.c_int, [_h, _h, _dp]),
    "imex_minmax_uvwp": (ctypes.c_int, [_h, _dp]),
    "imex_profile_enable": (ctypes.c_int, [_h, ctypes.c_int]),
    "imex_profile_read": (ctypes.c_int, [_h, ctypes.c_void_p, ctypes.c_int]),
    "imex_write_tecplot": (ctypes.c_int, [_h, ctypes.c_char_p, ctypes.c_int]),
    "imex_write_output": (ctypes.c_int, [_h, ctypes.c_char_p, ctypes.c_int]),
    "imex_checkpoint_save": (ctypes.c_int, [_h, ctypes.c_char_p]),
    "imex_checkpoint_load": (ctypes.c_int, [_h, ctypes.c_char_p]),
    "imex_get_f": (ctypes.c_int, [_h, _dp, ctypes.c_size_t]),
    "imex_set_f": (ctypes.c_int, [_h, _dp, ctypes.c_size_t]),
    "imex_get_f_device": (ctypes.c_int, [_h, ctypes.c_void_p, ctypes.c_size_t]),
    "imex_set_f_device": (ctypes.c_int, [_h, ctypes.c_void_p, ctypes.c_size_t]),
    "imex_conserved_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p]),
    "imex_set_launch": (ctypes.c_int, [_h, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "imex_get_launch": (ctypes.c_int, [_h, ctypes.POINTER(ctypes.c_int)]),
    "imex_set_engine": (ctypes.c_int, [_h, ctypes.c_int]),
    "imex_set_rounding": (ctypes.c_int, [_h, ctypes.c_int]),
    "imex_set_stream": (ctypes.c_int, [_h, ctypes.c_void_p]),
    "imex_synchronize": (ctypes.c_int, [_h]),
    "imex_steps_done": (ctypes.c_int64, [_h]),
    "imex_kernel_launches": (ctypes.c_int64, [_h]),
    "imex_fallback_cells": (ctypes.c_int, [_h, ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "imex_device_bytes": (ctypes.c_size_t, [_h]),
    "imex_last_error": (ctypes.c_char_p, [_h]),
    "imex_version": (ctypes.c_char_p, []),
    "imex_initialize_phase": (ctypes.c_int, [_h, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "imex_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "imex_batch_destroy": (None, [ctypes.c_void_p]),
    "imex_batch_add": (ctypes.c_int, [ctypes.c_void_p, _h, ctypes.c_int64]),
    "imex_batch_remove": (ctypes.c_int, [ctypes.c_void_p, _h]),
    "imex_batch_size": (ctypes.c_int, [ctypes.c_void_p]),
    "imex_batch_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "imex_batch_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "imex_batch_set_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "imex_batch_get_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "imex_batch_set_row_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int]),
    "imex_batch_get_row_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "imex_batch_set_graph": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "imex_batch_kernel_launches": (ctypes.c_int64, [ctypes.c_void_p]),
    "imex_batch_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "imex_server_create": (ctypes.c_int, [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "imex_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_int64)]),
    "imex_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Result), ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_int)]),
    "imex_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerStats)]),
    "imex_server_set_policy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "imex_server_now": (ctypes.c_double, [ctypes.c_void_p]),
    "imex_server_destroy": (None, [ctypes.c_void_p]),
    "imex_test_set_fault": (ctypes.c_int, [ctypes.c_int, ctypes.c_longlong]),
    "imex_decomp_grid": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_int)]),
    "imex_decomp_block": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(Block)]),
    "imex_decomp_halo": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.POINTER(HaloMsg)]),
    "imex_domain_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]),
    "imex_domain_destroy": (None, [ctypes.c_void_p]),
    "imex_domain_initialize": (ctypes.c_int, [ctypes.c_void_p]),
    "imex_domain_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "imex_domain_conserved": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "imex_domain_conserved_blocks": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "imex_domain_get_f": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_size_t]),
    "imex_domain_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(DomainStats)]),
    "imex_domain_fallback_cells": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "imex_domain_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "imex_domain_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
}

_lib = None


class ImexError(RuntimeError):
    """A non-zero status from the C ABI, with the library's message."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def load(path: str | None = None):
    """Load the shared library (once) and declare every signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with `python -m imexlbm_gb300.build` "
                          "(or __graft_entry__.build()); imexlbm_gb300 has no CPU fallback")
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def check(rc: int, handle=None) -> None:
    if rc != IMEX_OK:
        msg = load().imex_last_error(handle)
        raise ImexError(rc, msg.decode() if msg else "")
