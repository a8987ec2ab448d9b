"""Python mirror of the reference's System / LBM call surface.

``System`` follows class System (src/System.hpp, src/System.cpp: the nine
numbers of input.in and the derived tau), and ``LBM`` follows struct LBM
(src/lbm.hpp:113-211): ``Initialize``, ``Collision``, ``Streaming``,
``Conserved``, ``ComputeMacroscopic``.  Both are thin wrappers over the C
ABI (include/imexlbm.h); every compute call runs the CUDA kernels.

Errors: where the reference aborts (missing deck) or continues silently,
these raise ``ImexError`` with the library's status code and message.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import IMEX_ENGINE_AUTO, IMEX_F64, ImexError, check

Q = 27


class System:
    """Input deck: ``rho0 R Re / u0 Time inter / sx sy sz`` (src/System.cpp:22-24)."""

    def __init__(self, path: str = "input.in", text: str | None = None):
        L = _lib.load()
        d = _lib.Deck()
        rc = L.imex_deck_parse(text.encode(), ctypes.byref(d)) if text is not None else \
            L.imex_deck_read(path.encode(), ctypes.byref(d))
        check(rc)
        for name, _ in _lib.Deck._fields_:
            setattr(self, name, getattr(d, name))

    def Monitor(self) -> str:
        """The reference's banner (src/System.cpp:31-44), returned as text."""
        lines = ["============================", "3D Taylor-Green Vortex",
                 f"Re    = {self.Re}", f"Ma    = {self.Ma:g}", f"rho   = {self.rho0:g}",
                 f"miu   = {self.miu:g}", f"tau   = {self.tau:g}", f"Time  = {self.Time}",
                 f"inter = {self.inter}", f"nx,ny,nz = {self.sx} {self.sy} {self.sz}",
                 "============================"]
        return "\n".join(lines)


class LBM:
    """One periodic D3Q27 lattice resident on the current GPU."""

    def __init__(self, sx: int, sy: int, sz: int, tau: float, rho0: float, u0: float,
                 precision: int = IMEX_F64, engine: int = IMEX_ENGINE_AUTO):
        self._L = _lib.load()
        self.glx, self.gly, self.glz = int(sx), int(sy), int(sz)
        self.tau0, self.rho0, self.u0 = float(tau), float(rho0), float(u0)
        self.cs2 = 1.0 / 3.0
        self.me, self.nranks = 0, 1
        h = ctypes.c_void_p()
        check(self._L.imex_create(self.glx, self.gly, self.glz, self.tau0, self.rho0, self.u0,
                                  int(precision), ctypes.byref(h)))
        self._h = h
        if engine != IMEX_ENGINE_AUTO:
            self._check(self._L.imex_set_engine(self._h, int(engine)))

    # -- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.imex_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> None:
        check(rc, self._h)

    @property
    def shape(self):
        return (Q, self.glx, self.gly, self.glz)

    @property
    def handle(self):
        return self._h

    # -- the reference's methods ------------------------------------------
    def Initialize(self) -> None:
        self._check(self._L.imex_initialize(self._h))

    def initialize_phase(self, phx: float, phy: float, phz: float) -> None:
        """Taylor-Green init with coordinates shifted by (phx, phy, phz)."""
        self._check(self._L.imex_initialize_phase(self._h, float(phx), float(phy), float(phz)))

    def Collision(self) -> None:
        self._check(self._L.imex_collision(self._h))

    def Streaming(self) -> None:
        self._check(self._L.imex_streaming(self._h))

    def step(self, n: int = 1) -> None:
        self._check(self._L.imex_step(self._h, int(n)))

    def Conserved(self, allow_nonfinite: bool = False):
        """(mass, px, py, pz, ke) of the current distributions."""
        out = np.zeros(5)
        rc = self._L.imex_conserved(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if not (allow_nonfinite and rc == _lib.IMEX_ERR_NONFINITE):
            self._check(rc)
        return tuple(float(x) for x in out)

    def ComputeMacroscopic(self):
        """(p, u, v, w) arrays of shape (nx, ny, nz)."""
        arrs = [np.empty((self.glx, self.gly, self.glz)) for _ in range(4)]
        ptr = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrs]
        self._check(self._L.imex_macroscopic(self._h, *ptr))
        return tuple(arrs)

    def velocity_max_diff(self, ref: "LBM"):
        """(max |u_self - u_ref|, max |u_ref|) over all cells and components."""
        out = np.zeros(2)
        self._check(self._L.imex_velocity_max_diff(self._h, ref._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return float(out[0]), float(out[1])

    def profile_enable(self, on: bool = True) -> None:
        self._check(self._L.imex_profile_enable(self._h, int(bool(on))))

    def profile_read(self, reset: bool = False) -> dict:
        """{phase: {calls, total_ms, min_ms, max_ms}} of the timed launches."""
        buf = (_lib.PhaseStats * _lib.IMEX_NPHASE)()
        self._check(self._L.imex_profile_read(self._h, buf, int(bool(reset))))
        names = ("collision", "stream", "macro", "conserved")
        return {names[q]: {k: getattr(buf[q], k) for k, _ in _lib.PhaseStats._fields_} for q in range(_lib.IMEX_NPHASE)}

    def minmax_uvwp(self):
        """(umax, vmax, wmax, pmax, umin, vmin, wmin, pmin), the reducer
        order of the reference's "minmax_uvwp" (src/lbm.cpp:351-372)."""
        out = np.zeros(8)
        self._check(self._L.imex_minmax_uvwp(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return tuple(float(x) for x in out)

    def MPIoutput(self, n: int, path: str | None = None) -> str:
        """Write the reference's Tecplot file output<n>.plt (src/lbm.cpp:307)
        or ``path``; returns the file name."""
        name = path if path is not None else f"output{int(n)}.plt"
        self._check(self._L.imex_write_tecplot(self._h, name.encode(), int(n)))
        return name

    def Output(self, n: int, path: str | None = None) -> str:
        """Write the reference's ASCII dump of f(0), output<n>0.dat
        (src/lbm.cpp:606-636), or ``path``; returns the file name."""
        name = path if path is not None else f"output{int(n)}0.dat"
        self._check(self._L.imex_write_output(self._h, name.encode(), int(n)))
        return name

    def checkpoint_save(self, path: str) -> None:
        self._check(self._L.imex_checkpoint_save(self._h, str(path).encode()))

    def checkpoint_load(self, path: str) -> None:
        self._check(self._L.imex_checkpoint_load(self._h, str(path).encode()))

    # -- data access --------------------------------------------------------
    def get_f(self, out: np.ndarray | None = None) -> np.ndarray:
        f = np.empty(self.shape) if out is None else out
        if f.dtype != np.float64 or not f.flags["C_CONTIGUOUS"]:
            raise ValueError("get_f needs a C-contiguous float64 array")
        self._check(self._L.imex_get_f(self._h, f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), f.size))
        return f

    def set_f(self, f: np.ndarray) -> None:
        f = np.ascontiguousarray(f, dtype=np.float64)
        self._check(self._L.imex_set_f(self._h, f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), f.size))

    def get_f_device(self, ptr: int, n: int) -> None:
        self._check(self._L.imex_get_f_device(self._h, ctypes.c_void_p(ptr), n))

    def set_f_device(self, ptr: int, n: int) -> None:
        self._check(self._L.imex_set_f_device(self._h, ctypes.c_void_p(ptr), n))

    def set_engine(self, engine: int) -> None:
        self._check(self._L.imex_set_engine(self._h, int(engine)))

    def set_launch(self, stages: int, rows_per_stage: int = 1, ctas_per_sm: int = 1) -> None:
        """Pin the fused step's launch shape (stages 0: one thread per cell;
        1: two steps per launch through a ring of rows_per_stage + 2 x-planes,
        ctas_per_sm resident CTAs - float64 fixed point only, never chosen
        automatically; >= 2: row-staged ring depth, with rows_per_stage
        y-rows per item and ctas_per_sm resident CTAs; < 0: automatic)."""
        self._check(self._L.imex_set_launch(self._h, int(stages), int(rows_per_stage), int(ctas_per_sm)))

    def get_launch(self):
        """(stages, rows_per_stage, ctas_per_sm, threads) of the fused step,
        tuning first if needed."""
        out = (ctypes.c_int * 4)()
        self._check(self._L.imex_get_launch(self._h, out))
        return tuple(out)

    def set_rounding(self, mode: int) -> None:
        """IMEX_ROUND_NEAREST or IMEX_ROUND_STOCHASTIC (float16-deviation storage)."""
        self._check(self._L.imex_set_rounding(self._h, int(mode)))

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(self._L.imex_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def fence(self) -> None:
        self._check(self._L.imex_synchronize(self._h))

    def steps_done(self) -> int:
        return int(self._L.imex_steps_done(self._h))

    def kernel_launches(self) -> int:
        return int(self._L.imex_kernel_launches(self._h))

    def fallback_cells(self, reset: bool = False) -> int:
        v = ctypes.c_int64()
        self._check(self._L.imex_fallback_cells(self._h, ctypes.byref(v), int(reset)))
        return int(v.value)

    def device_bytes(self) -> int:
        return int(self._L.imex_device_bytes(self._h))


class Batch:
    """Float32 / float16-deviation lattices advanced together by one
    persistent launch per step (include/imexlbm.h, imex_batch_*)."""

    def __init__(self, max_members: int = 256):
        self._L = _lib.load()
        b = ctypes.c_void_p()
        check(self._L.imex_batch_create(int(max_members), ctypes.byref(b)))
        self._b = b
        self.members = []

    def _check(self, rc: int) -> None:
        if rc != _lib.IMEX_OK:
            msg = self._L.imex_batch_last_error(self._b)
            raise ImexError(rc, msg.decode() if msg else "")

    def add(self, lat: LBM, max_steps: int = -1) -> None:
        self._check(self._L.imex_batch_add(self._b, lat.handle, int(max_steps)))
        self.members.append(lat)

    def remove(self, lat: LBM) -> None:
        self._check(self._L.imex_batch_remove(self._b, lat.handle))
        self.members.remove(lat)

    def step(self, n: int) -> None:
        self._check(self._L.imex_batch_step(self._b, int(n)))

    def synchronize(self) -> None:
        self._check(self._L.imex_batch_synchronize(self._b))

    def set_launch(self, threads: int, cells_per_thread: int = 1, ctas_per_sm: int = 4) -> None:
        self._check(self._L.imex_batch_set_launch(self._b, int(threads), int(cells_per_thread), int(ctas_per_sm)))

    def get_launch(self):
        out = (ctypes.c_int * 3)()
        self._check(self._L.imex_batch_get_launch(self._b, out))
        return tuple(out)

    def set_row_launch(self, stages: int, dir_kb: int = 2, ctas_per_sm: int = 1, float32_members: bool = True) -> None:
        """Row-staged kernel shape (stages, KiB per direction in a stage,
        CTAs per SM, float32 members in it); stages 0 autotunes, -1 turns
        the row kernel off."""
        self._check(self._L.imex_batch_set_row_launch(self._b, int(stages), int(dir_kb), int(ctas_per_sm),
                                                      int(bool(float32_members))))

    def get_row_launch(self):
        out = (ctypes.c_int * 4)()
        self._check(self._L.imex_batch_get_row_launch(self._b, out))
        return tuple(out)

    def set_graph(self, steps: int) -> None:
        self._check(self._L.imex_batch_set_graph(self._b, int(steps)))

    def kernel_launches(self) -> int:
        return int(self._L.imex_batch_kernel_launches(self._b))

    def close(self) -> None:
        if getattr(self, "_b", None):
            self._L.imex_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def decomp_grid(nranks: int, nx: int, ny: int, nz: int):
    """The reference's rank grid (rx, ry, rz) for nranks ranks
    (setup_Cartesian, src/mpi_view_transfer.cpp:53-95)."""
    L = _lib.load()
    out = (ctypes.c_int * 3)()
    check(L.imex_decomp_grid(int(nranks), int(nx), int(ny), int(nz), out))
    return tuple(out)


def decomp_block(nranks: int, nx: int, ny: int, nz: int, rank: int) -> dict:
    """Rank `rank`'s block: coord (px, py, pz), lo and len per axis."""
    L = _lib.load()
    b = _lib.Block()
    check(L.imex_decomp_block(int(nranks), int(nx), int(ny), int(nz), int(rank), ctypes.byref(b)))
    return {"rank": b.rank, "coord": tuple(b.coord), "lo": tuple(b.lo), "len": tuple(b.len)}


def decomp_halo(nranks: int, nx: int, ny: int, nz: int, rank: int, channel: int) -> dict:
    """Halo channel `channel` (0..25) of rank `rank`: peers, boxes in padded
    block coordinates and the directions it carries."""
    L = _lib.load()
    m = _lib.HaloMsg()
    check(L.imex_decomp_halo(int(nranks), int(nx), int(ny), int(nz), int(rank), int(channel), ctypes.byref(m)))
    return {"channel": m.channel, "offset": tuple(m.offset), "send_to": m.send_to, "recv_from": m.recv_from,
            "send_lo": tuple(m.send_lo), "recv_lo": tuple(m.recv_lo), "ext": tuple(m.ext),
            "dirs": tuple(m.dirs[:m.ndir])}


class Domain:
    """A lattice decomposed into `nranks` blocks on this GPU, stepped as the
    reference's ranks step theirs (include/imexlbm.h, imex_domain_*)."""

    def __init__(self, sx: int, sy: int, sz: int, nranks: int, tau: float, rho0: float, u0: float):
        self._L = _lib.load()
        d = ctypes.c_void_p()
        check(self._L.imex_domain_create(int(sx), int(sy), int(sz), int(nranks), float(tau), float(rho0), float(u0),
                                         ctypes.byref(d)))
        self._d = d
        self.glx, self.gly, self.glz = int(sx), int(sy), int(sz)
        self.nranks = int(nranks)

    def _check(self, rc: int) -> None:
        if rc != _lib.IMEX_OK:
            msg = self._L.imex_domain_last_error(self._d)
            raise ImexError(rc, msg.decode() if msg else "")

    @property
    def shape(self):
        return (Q, self.glx, self.gly, self.glz)

    def Initialize(self) -> None:
        self._check(self._L.imex_domain_initialize(self._d))

    def step(self, n: int = 1) -> None:
        self._check(self._L.imex_domain_step(self._d, int(n)))

    def Conserved(self):
        out = (ctypes.c_double * 5)()
        self._check(self._L.imex_domain_conserved(self._d, out))
        return tuple(out)

    def conserved_blocks(self) -> np.ndarray:
        out = np.zeros((self.nranks, 5))
        self._check(self._L.imex_domain_conserved_blocks(self._d, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def get_f(self) -> np.ndarray:
        f = np.empty(self.shape)
        self._check(self._L.imex_domain_get_f(self._d, f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), f.size))
        return f

    def info(self) -> dict:
        st = _lib.DomainStats()
        self._check(self._L.imex_domain_info(self._d, ctypes.byref(st)))
        return {"nranks": st.nranks, "grid": tuple(st.grid), "steps": st.steps, "launches": st.launches,
                "halo_values_per_step": st.halo_values_per_step, "device_bytes": st.device_bytes}

    def fallback_cells(self) -> int:
        v = ctypes.c_int64()
        self._check(self._L.imex_domain_fallback_cells(self._d, ctypes.byref(v)))
        return int(v.value)

    def fence(self) -> None:
        self._check(self._L.imex_domain_synchronize(self._d))

    def close(self) -> None:
        if getattr(self, "_d", None):
            self._L.imex_domain_destroy(self._d)
            self._d = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """Request server with continuous batching (include/imexlbm.h,
    imex_server_*): submit solves from any thread, poll finished results."""

    def __init__(self, budget_bytes: float = 120e9, max_active: int = 256, steps_per_tick: int = 25):
        self._L = _lib.load()
        s = ctypes.c_void_p()
        check(self._L.imex_server_create(int(budget_bytes), int(max_active), int(steps_per_tick), ctypes.byref(s)))
        self._s = s

    def submit(self, nx: int, ny: int, nz: int, tau: float, u0: float, steps: int, precision: int = _lib.IMEX_F32,
               rho0: float = 1.0, phase=(0.0, 0.0, 0.0), rounding: int | None = None, tag: int = 0,
               resume_path: str = "", save_path: str = "") -> int:
        """Queue a solve; returns its id.  resume_path starts it from a
        checkpoint (its step count included), save_path keeps its final
        state: a solve can be paused and resumed across requests."""
        r = _lib.Request()
        r.nx, r.ny, r.nz = int(nx), int(ny), int(nz)
        r.precision = int(precision)
        if rounding is None:
            rounding = _lib.IMEX_ROUND_STOCHASTIC if precision == _lib.IMEX_F16DEV else _lib.IMEX_ROUND_NEAREST
        r.rounding = int(rounding)
        r.tau, r.rho0, r.u0 = float(tau), float(rho0), float(u0)
        for i in range(3):
            r.phase[i] = float(phase[i])
        r.steps, r.tag = int(steps), int(tag)
        for name, val in (("resume_path", resume_path), ("save_path", save_path)):
            b = str(val).encode()
            if len(b) >= 256:
                raise ValueError(f"{name} longer than 255 bytes")
            setattr(r, name, b)
        rid = ctypes.c_int64()
        check(self._L.imex_server_submit(self._s, ctypes.byref(r), ctypes.byref(rid)))
        return int(rid.value)

    def poll(self, max_results: int = 4096):
        buf = (_lib.Result * max_results)()
        n = ctypes.c_int()
        check(self._L.imex_server_poll(self._s, buf, max_results, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            r = buf[i]
            out.append({"id": r.id, "tag": r.tag, "status": r.status, "conserved": tuple(r.conserved),
                        "steps": r.steps, "cells": r.cells, "t_submit": r.t_submit, "t_admit": r.t_admit,
                        "t_done": r.t_done})
        return out

    def stats(self) -> dict:
        st = _lib.ServerStats()
        check(self._L.imex_server_get_stats(self._s, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in _lib.ServerStats._fields_}

    def now(self) -> float:
        return float(self._L.imex_server_now(self._s))

    def set_policy(self, policy: int) -> None:
        """IMEX_POLICY_ARRIVAL (default) or IMEX_POLICY_LEAST_WORK admission."""
        check(self._L.imex_server_set_policy(self._s, int(policy)))

    def close(self) -> None:
        if getattr(self, "_s", None):
            self._L.imex_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


__all__ = ["System", "LBM", "Batch", "Server", "ImexError", "Q"]
