"""Build the CUDA library and the driver executable in-tree.

Outputs (git-ignored) go to ``imexlbm_gb300/_build/``:
  libimexlbm.so   the C-ABI library (include/imexlbm.h), sm_103a only
  imexlbm         the drop-in driver (reads ./input.in, prints the
                  reference's ``step`` / ``cos`` lines)

Every translation unit is compiled by nvcc in parallel, then linked once.
A unit is rebuilt when its source or any header under csrc/ or include/ is
newer than its object.

Usage: ``python -m imexlbm_gb300.build [--force] [--jobs N]``
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(CSRC, "host")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libimexlbm.so")
EXE = os.path.join(OUT, "imexlbm")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", INCLUDE, "-I", CSRC]
# Sources of the shared library.
LIB_SOURCES = ["lattice.cu", "kernels_f64.cu", "kernels_fx.cu", "kernels_lowp.cu", "fx_params.cpp", "deck.cpp",
               "conserved_noalloc.cu", "batch.cu", "server.cu", "fields.cu", "decomp.cu"]
# Sources of the driver executable (host C++ facade + main).
EXE_SOURCES = ["lbm.cpp", "main.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build imexlbm_gb300")


def _headers() -> list[str]:
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp"))
    hs += glob.glob(os.path.join(HOST, "*.hpp")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    """Compile libimexlbm.so and the imexlbm driver; return the library path."""
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    headers = _headers()
    objs, work = [], []
    for name in LIB_SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(OUT, name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            work.append([cc, *ARCH, *COMMON, "-c", src, "-o", obj])
    exe_objs = []
    for name in EXE_SOURCES:
        src = os.path.join(HOST, name)
        obj = os.path.join(OUT, "host_" + name + ".o")
        exe_objs.append(obj)
        if force or _stale(obj, [src] + headers):
            work.append([cc, *COMMON, "-I", HOST, "-c", src, "-o", obj])
    if work:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(work), os.cpu_count() or 4)) as ex:
            for cmd, fut in [(c, ex.submit(_run, c)) for c in work]:
                fut.result()
                if verbose:
                    print(" ".join(cmd))
    if force or work or _stale(LIB, objs):
        _run([cc, *ARCH, "-shared", "-o", LIB, *objs, "-cudart=static"])
    if force or work or _stale(EXE, exe_objs + [LIB]):
        _run([cc, "-o", EXE, *exe_objs, "-L", OUT, "-limexlbm", "-Xlinker", "-rpath,$ORIGIN"])
    return LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, jobs=a.jobs, verbose=a.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
