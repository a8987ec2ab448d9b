"""Generate tests/golden/reference_runs.json by running the reference's own code.

The reference's unmodified src/*.cpp are compiled against the single-process
Kokkos / MPI stand-ins of oracle/refshim (``make -C oracle ref``) into
oracle/_ref/imexref, whose ranks are threads of one process.  This script
runs it on small decks and records what the tests compare against:

  cons       the `cons` lines of src/main.cpp:88-93 (mass, momentum, ke), per
             deck and rank count
  f_sha256   SHA-256 of the interior f of the whole lattice after the run
             (float64, the reference's order f[a][x][y][z], little endian):
             the bitwise pin of the oracle and of the decomposed GPU runs
  layout     the rx, ry, rz the reference's setup_Cartesian prints per rank
             count (src/mpi_view_transfer.cpp:53-95)
  files      SHA-256 and size of the Tecplot file of LBM::MPIoutput and of the
             ASCII dump of LBM::Output after a short run, plus the ASCII
             dump's first lines

Usage: python tests/golden/make_ref_golden.py /path/to/reference
(the reference checkout is read here only; the tests read the JSON).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as o  # noqa: E402

# (name, deck text, steps of the dump run, rank counts)
DECKS = [
    # tests/regression.sh:58 - 32^3, 20 steps, report every step
    ("regression", "1.0  0.1  1600\n0.05  20  1\n32  32  32\n", 20, [1, 2, 4, 8]),
    # the 32^3 parity deck: 100 steps, report every 10
    ("parity32", "1.0  0.1  1600\n0.05  100  10\n32  32  32\n", 100, [1, 2, 4, 8]),
    # a ragged lattice whose blocks do not divide evenly
    ("ragged", "1.0  0.1  400\n0.06  24  6\n18  20  22\n", 24, [1, 2, 3, 4, 6, 8]),
]


def sha(path: str) -> str:
    with open(path, "rb") as fp:
        return hashlib.sha256(fp.read()).hexdigest()


def main(ref: str) -> None:
    exe = o.build_ref(os.path.join(ref, "src"))
    if not exe:
        raise SystemExit(f"no reference sources under {ref}/src")
    out = {"source": "Maccchiatooo/IMEXLBM src/*.cpp, unmodified, built with oracle/refshim "
                     "(single-process Kokkos / MPI stand-ins; ranks are threads)",
           "generator": "tests/golden/make_ref_golden.py", "decks": {}}
    for name, deck, steps, ranks in DECKS:
        rec = {"deck": deck, "steps": steps, "runs": {}}
        for n in ranks:
            with tempfile.TemporaryDirectory() as d:
                text = o.run_ref(deck, d, ranks=n, threads=1, mode="main")
                layout = [ln for ln in text.splitlines() if ln.startswith("rx=")]
                dump = o.run_ref(deck, d, ranks=n, threads=1, mode="dump", args=(steps, "f.bin"))
                rec["runs"][str(n)] = {"cons": o.parse_cons(text), "layout": layout[0] if layout else "",
                                       "f_sha256": sha(os.path.join(d, "f.bin")),
                                       "dump_cons_last": o.parse_cons(dump)[-1]}
        out["decks"][name] = rec
    # output files after 10 steps of the 32^3 deck, one rank
    deck = "1.0  0.1  1600\n0.05  10  10\n32  32  32\n"
    with tempfile.TemporaryDirectory() as d:
        o.run_ref(deck, d, ranks=1, threads=1, mode="dump", args=(10, "f.bin", "--tecplot", 1, "--ascii", 1))
        plt, dat = os.path.join(d, "output1.plt"), os.path.join(d, "output10.dat")
        with open(dat) as fp:
            head = [next(fp).rstrip("\n") for _ in range(6)]
        out["files"] = {"deck": deck, "steps": 10,
                        "tecplot": {"name": "output1.plt", "sha256": sha(plt), "bytes": os.path.getsize(plt)},
                        "ascii": {"name": "output10.dat", "sha256": sha(dat), "bytes": os.path.getsize(dat),
                                  "head": head},
                        "f_sha256": sha(os.path.join(d, "f.bin"))}
    with open(os.path.join(HERE, "reference_runs.json"), "w") as fp:
        json.dump(out, fp, indent=1)
        fp.write("\n")
    print("wrote", os.path.join(HERE, "reference_runs.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])
