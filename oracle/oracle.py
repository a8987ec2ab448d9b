"""ctypes wrapper around the CPU oracle (test infrastructure only).

The oracle is what the CUDA library is checked against: tests, the smoke check
and the benchmark's CPU-baseline leg may call it; the product path never does.  It
restates the reference's single-rank IMEXLBM step in plain C (see the header
of ``lbm_oracle.c`` for the reference file:line of every function).

Arrays are numpy float64 in the layout ``f[27][nx][ny][nz]`` (z fastest).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
Q = 27

_lib = None


class Deck(ctypes.Structure):
    _fields_ = [
        ("rho0", ctypes.c_double), ("R", ctypes.c_double), ("u0", ctypes.c_double),
        ("Re", ctypes.c_int), ("Time", ctypes.c_int), ("inter", ctypes.c_int),
        ("sx", ctypes.c_int), ("sy", ctypes.c_int), ("sz", ctypes.c_int),
        ("cs2", ctypes.c_double), ("cs", ctypes.c_double), ("Ma", ctypes.c_double),
        ("miu", ctypes.c_double), ("tau", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP) if needed."""
    src = os.path.join(HERE, "lbm_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        i = ctypes.c_int
        L.oracle_set_threads.argtypes = [i]
        L.oracle_max_threads.restype = i
        L.oracle_weight.argtypes = [i]
        L.oracle_weight.restype = ctypes.c_double
        L.oracle_velocity.argtypes = [i, i]
        L.oracle_velocity.restype = i
        L.oracle_deck_parse.argtypes = [ctypes.c_char_p, ctypes.POINTER(Deck)]
        L.oracle_deck_parse.restype = i
        L.oracle_init.argtypes = [i, i, i, ctypes.c_double, ctypes.c_double, dp]
        L.oracle_collide.argtypes = [i, i, i, ctypes.c_double, dp]
        L.oracle_stream.argtypes = [i, i, i, dp, dp]
        L.oracle_step.argtypes = [i, i, i, ctypes.c_double, dp, dp, i]
        L.oracle_step_pingpong.argtypes = [i, i, i, ctypes.c_double, dp, dp]
        L.oracle_conserved.argtypes = [i, i, i, dp, dp]
        L.oracle_macroscopic.argtypes = [i, i, i, dp, dp, dp, dp, dp]
        L.oracle_minmax_uvwp.argtypes = [i, i, i, dp, dp]
        L.oracle_write_tecplot.argtypes = [i, i, i, dp, i, ctypes.c_char_p]
        L.oracle_write_tecplot.restype = i
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def weights() -> np.ndarray:
    return np.array([lib().oracle_weight(a) for a in range(Q)])


def velocities() -> np.ndarray:
    return np.array([[lib().oracle_velocity(a, d) for d in range(3)] for a in range(Q)], dtype=np.int64)


def parse_deck(text: str) -> Deck:
    d = Deck()
    if lib().oracle_deck_parse(text.encode(), ctypes.byref(d)) != 0:
        raise ValueError("malformed deck")
    return d


def init(nx: int, ny: int, nz: int, rho0: float, u0: float) -> np.ndarray:
    f = np.empty((Q, nx, ny, nz), dtype=np.float64)
    lib().oracle_init(nx, ny, nz, rho0, u0, _p(f))
    return f


def collide(f: np.ndarray, tau0: float) -> None:
    _, nx, ny, nz = f.shape
    lib().oracle_collide(nx, ny, nz, tau0, _p(f))


def stream(f: np.ndarray) -> np.ndarray:
    _, nx, ny, nz = f.shape
    ft = np.empty_like(f)
    lib().oracle_stream(nx, ny, nz, _p(f), _p(ft))
    return ft


def step(f: np.ndarray, tau0: float, nsteps: int = 1, scratch: np.ndarray | None = None) -> None:
    """Advance f in place by nsteps reference steps (collide, stream, swap)."""
    _, nx, ny, nz = f.shape
    ft = np.empty_like(f) if scratch is None else scratch
    lib().oracle_step(nx, ny, nz, tau0, _p(f), _p(ft), int(nsteps))


def step_pingpong(f: np.ndarray, ft: np.ndarray, tau0: float) -> None:
    """One step, collide f in place then stream into ft (no copy back)."""
    _, nx, ny, nz = f.shape
    lib().oracle_step_pingpong(nx, ny, nz, tau0, _p(f), _p(ft))


def conserved(f: np.ndarray) -> np.ndarray:
    _, nx, ny, nz = f.shape
    out = np.zeros(5)
    lib().oracle_conserved(nx, ny, nz, _p(f), _p(out))
    return out


def macroscopic(f: np.ndarray):
    _, nx, ny, nz = f.shape
    p, u, v, w = (np.empty((nx, ny, nz)) for _ in range(4))
    lib().oracle_macroscopic(nx, ny, nz, _p(f), _p(p), _p(u), _p(v), _p(w))
    return p, u, v, w


def minmax_uvwp(f: np.ndarray) -> np.ndarray:
    """(umax, vmax, wmax, pmax, umin, vmin, wmin, pmin) of f's macroscopic fields."""
    _, nx, ny, nz = f.shape
    out = np.zeros(8)
    lib().oracle_minmax_uvwp(nx, ny, nz, _p(f), _p(out))
    return out


def write_tecplot(f: np.ndarray, n: int, path: str) -> None:
    """The reference's one-rank output<n>.plt of f, written to path."""
    _, nx, ny, nz = f.shape
    if lib().oracle_write_tecplot(nx, ny, nz, _p(f), int(n), str(path).encode()) != 0:
        raise OSError(f"cannot write {path}")


# ---------------------------------------------------------------------------
# The reference's own code (oracle/_ref/imexref): its unmodified src/*.cpp
# built against the single-process Kokkos / MPI stand-ins of oracle/refshim
# by `make -C oracle ref` (see oracle/Makefile).  Test infrastructure, like
# the rest of this module.

REF_EXE = os.path.join(HERE, "_ref", os.uname().machine, "imexref")
REF_SRC_DEFAULT = "/root/reference/src"


def build_ref(refsrc: str | None = None) -> str | None:
    """Build oracle/_ref/imexref from the reference's sources (REFSRC, or the
    copy staged in oracle/_ref/src).  Returns its path, or None when neither
    source is present."""
    src = refsrc or os.environ.get("IMEXREF_SRC", REF_SRC_DEFAULT)
    staged = os.path.join(HERE, "_ref", "src", "lbm.cpp")
    if not os.path.isdir(src) and not os.path.exists(staged):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFSRC={src}", "-j", str(min(8, os.cpu_count() or 1))],
                   check=True, stdout=subprocess.DEVNULL)
    return REF_EXE if os.path.exists(REF_EXE) else None


def run_ref(deck: str, cwd: str, ranks: int = 1, threads: int | None = None, mode: str = "main",
            args: tuple = (), timeout: float = 600.0, bind: bool = False) -> str:
    """Run the reference's code on `ranks` rank threads in directory cwd
    (which gets the deck as input.in); returns its standard output.  bind:
    OpenMP threads spread over the hardware threads and pinned there
    (OMP_PROC_BIND=spread, OMP_PLACES=threads unless the environment sets
    them), as the reference's job scripts run it (machines/polaris/env.sh:67-68)."""
    with open(os.path.join(cwd, "input.in"), "w") as fp:
        fp.write(deck)
    cmd = [REF_EXE, "--ranks", str(ranks)]
    if threads:
        cmd += ["--threads", str(threads)]
    cmd += [mode, *map(str, args)]
    env = dict(os.environ)
    if bind:
        env.setdefault("OMP_PROC_BIND", "spread")
        env.setdefault("OMP_PLACES", "threads")
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True, timeout=timeout, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"imexref failed ({r.returncode}): {r.stderr[-2000:]}")
    return r.stdout


def parse_cons(text: str) -> list:
    """The `cons` lines of src/main.cpp:88-93: [(step, mass, px, py, pz, ke)]."""
    out = []
    for ln in text.splitlines():
        if ln.startswith("cons"):
            parts = [p for p in ln.replace("|", " ").split() if p]
            out.append((int(parts[2]), float(parts[4]), float(parts[6]), float(parts[8]), float(parts[10]),
                        float(parts[12])))
    return out


def parse_mlups(text: str) -> list:
    """The MLUPS figures of the `step` lines of src/main.cpp:75-80."""
    out = []
    for ln in text.splitlines():
        if ln.startswith("step") and ln.rstrip().endswith("MLUPS"):
            out.append(float(ln.split("|")[-1].split()[0]))
    return out
