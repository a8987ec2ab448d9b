"""The oracle pinned bit for bit to the reference's own code.

tests/golden/reference_runs.json holds what the reference's unmodified
src/*.cpp computed when built against the single-process Kokkos / MPI
stand-ins of oracle/refshim (tests/golden/make_ref_golden.py): SHA-256 of
the whole lattice's f after each deck's run on 1 to 8 ranks, the `cons`
lines of src/main.cpp:88-93, and the Tecplot and ASCII files of
LBM::MPIoutput / LBM::Output.  The oracle must reproduce f bit for bit, the
reductions to the rounding of their summation order, and the Tecplot file
byte for byte.  Where the reference's code can be built here (its sources or
the staged copy of oracle/_ref/src are present), it is also run live and
must agree with the committed record.
"""
import hashlib
import json
import os
import shutil
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN

with open(os.path.join(GOLDEN, "reference_runs.json")) as _fp:
    RUNS = json.load(_fp)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def oracle_run(oracle, deck_text, steps):
    d = oracle.parse_deck(deck_text)
    f = oracle.init(d.sx, d.sy, d.sz, d.rho0, d.u0)
    cons = []
    for it in range(1, steps + 1):
        oracle.step(f, d.tau, 1)
        if it % d.inter == 0:
            cons.append((it, *oracle.conserved(f)))
    return f, cons


@pytest.mark.parametrize("name", sorted(RUNS["decks"]))
def test_oracle_f_is_the_references_bit_for_bit(oracle, name):
    rec = RUNS["decks"][name]
    f, _ = oracle_run(oracle, rec["deck"], rec["steps"])
    digests = {r["f_sha256"] for r in rec["runs"].values()}
    # the reference's field does not depend on its decomposition
    assert len(digests) == 1, rec["runs"].keys()
    assert sha(f) == digests.pop()


@pytest.mark.parametrize("name", sorted(RUNS["decks"]))
def test_oracle_cons_lines_match_the_references(oracle, name):
    """Mass and ke to 1e-13 relative (only the summation order differs),
    momentum to 1e-13 absolute; every rank count of the reference agrees
    with the oracle, hence with each other (regression.sh check 3)."""
    rec = RUNS["decks"][name]
    _, cons = oracle_run(oracle, rec["deck"], rec["steps"])
    for n, run in rec["runs"].items():
        ref = run["cons"]
        assert [c[0] for c in ref] == [c[0] for c in cons], n
        for r, c in zip(ref, cons):
            assert abs(r[1] - c[1]) <= 1e-13 * abs(c[1]), (n, r, c)
            assert abs(r[5] - c[5]) <= 1e-13 * abs(c[5]), (n, r, c)
            assert max(abs(r[k] - c[k]) for k in (2, 3, 4)) <= 1e-13, (n, r, c)


def test_reference_layouts_follow_setup_cartesian():
    """The rank grids the reference chose (setup_Cartesian's least-spread
    factorisation, src/mpi_view_transfer.cpp:53-95)."""
    lay = {n: r["layout"] for n, r in RUNS["decks"]["ragged"]["runs"].items()}
    assert lay == {"1": "rx=1,ry=1,rz=1", "2": "rx=1,ry=1,rz=2", "3": "rx=1,ry=1,rz=3", "4": "rx=1,ry=2,rz=2",
                   "6": "rx=1,ry=2,rz=3", "8": "rx=2,ry=2,rz=2"}


def test_oracle_tecplot_writer_is_the_references(oracle, tmp_path):
    rec = RUNS["files"]
    f, _ = oracle_run(oracle, rec["deck"], rec["steps"])
    assert sha(f) == rec["f_sha256"]
    path = tmp_path / "out.plt"
    oracle.write_tecplot(f, 1, str(path))
    data = path.read_bytes()
    assert len(data) == rec["tecplot"]["bytes"]
    assert hashlib.sha256(data).hexdigest() == rec["tecplot"]["sha256"]


@pytest.fixture(scope="module")
def ref_exe():
    from oracle import oracle as o
    try:
        exe = o.build_ref()
    except Exception as e:  # a compiler problem is a failure, absent sources a skip
        pytest.fail(f"the reference's code did not build: {e}")
    if not exe:
        pytest.skip("the reference's sources are not present on this machine")
    return o


def test_live_reference_run_matches_the_record(ref_exe):
    """Rerun the reference's code (2 ranks, ragged deck) and compare with the
    committed record, so that the record cannot drift from the sources."""
    o = ref_exe
    rec = RUNS["decks"]["ragged"]
    with tempfile.TemporaryDirectory() as d:
        text = o.run_ref(rec["deck"], d, ranks=2, threads=1, mode="dump", args=(rec["steps"], "f.bin"))
        got = hashlib.sha256(open(os.path.join(d, "f.bin"), "rb").read()).hexdigest()
        assert got == rec["runs"]["2"]["f_sha256"]
        assert o.parse_cons(text)[-1] == tuple(rec["runs"]["2"]["dump_cons_last"])


def ascii_dump(f: np.ndarray) -> bytes:
    """LBM::Output's text (src/lbm.cpp:606-627) of f on one rank: a header,
    then "x y z f(0)" per cell, x fastest, f in fixed notation, 8 decimals."""
    _, nx, ny, nz = f.shape
    lines = ["variables=x,y,z,f", f"zone I={nx},J={ny},K={nz}"]
    f0 = f[0]
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                lines.append(f"{i} {j} {k} {f0[i, j, k]:.8f}")
    return ("\n".join(lines) + "\n").encode()


def test_ascii_dump_format_is_the_references(oracle):
    rec = RUNS["files"]
    f, _ = oracle_run(oracle, rec["deck"], rec["steps"])
    data = ascii_dump(f)
    assert data.decode().splitlines()[:6] == rec["ascii"]["head"]
    assert len(data) == rec["ascii"]["bytes"]
    assert hashlib.sha256(data).hexdigest() == rec["ascii"]["sha256"]
