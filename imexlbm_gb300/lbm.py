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
        >= 2: row-staged ring depth, with rows_per_stage y-rows per item and
        ctas_per_sm resident CTAs; < 0: automatic)."""
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


__all__ = ["System", "LBM", "Batch", "ImexError", "Q"]
