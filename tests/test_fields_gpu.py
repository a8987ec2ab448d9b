"""Field output and restart: the min/max report reduction, the Tecplot file
of LBM::MPIoutput, and checkpoint save / load.

The library's file must equal, byte for byte, the oracle's restatement of
the reference writer applied to the lattice's own distributions (read back
with get_f) - whatever the storage precision and whether a streaming is
pending.  A run restored from a checkpoint must continue bit for bit as the
saved run does.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRECS = ["f64", "f32", "f16dev"]


def prec_id(imex, name):
    return {"f64": imex.IMEX_F64, "f32": imex.IMEX_F32, "f16dev": imex.IMEX_F16DEV}[name]


@pytest.mark.parametrize("name", PRECS)
@pytest.mark.parametrize("shape", [(12, 10, 16), (33, 5, 40), (1, 3, 70)])
def test_minmax_equals_oracle(imex, oracle, name, shape):
    with imex.LBM(*shape, 0.01, 1.0, 0.05, precision=prec_id(imex, name)) as lat:
        lat.initialize_phase(0.3, 1.2, 2.0)
        lat.step(3)                      # a streaming is pending: read through it
        got = lat.minmax_uvwp()
        f = lat.get_f()
    assert np.array_equal(np.array(got), oracle.minmax_uvwp(f))


@pytest.mark.parametrize("name", PRECS)
@pytest.mark.parametrize("shape", [(16, 12, 20), (35, 3, 33)])
def test_tecplot_bytes_equal_oracle(imex, oracle, tmp_path, name, shape):
    with imex.LBM(*shape, 0.02, 1.0, 0.06, precision=prec_id(imex, name)) as lat:
        lat.Initialize()
        lat.step(4)
        got = lat.MPIoutput(4, str(tmp_path / "lib.plt"))
        f = lat.get_f()
    oracle.write_tecplot(f, 4, str(tmp_path / "oracle.plt"))
    a = open(got, "rb").read()
    b = (tmp_path / "oracle.plt").read_bytes()
    assert len(a) == 332 + 7 * 8 * int(np.prod(shape))
    assert a == b


def test_tecplot_after_set_f_and_default_name(imex, oracle, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    shape = (8, 9, 10)
    f = oracle.init(*shape, 1.0, 0.05)
    oracle.step(f, 0.05, 2)
    with imex.LBM(*shape, 0.05, 1.0, 0.05) as lat:
        lat.set_f(f)
        assert lat.MPIoutput(12) == "output12.plt"
    oracle.write_tecplot(f, 12, str(tmp_path / "want.plt"))
    assert (tmp_path / "output12.plt").read_bytes() == (tmp_path / "want.plt").read_bytes()


def test_tecplot_unwritable_path(imex):
    with imex.LBM(4, 4, 4, 0.1, 1.0, 0.05) as lat:
        lat.Initialize()
        with pytest.raises(imex.ImexError) as ei:
            lat.MPIoutput(1, "/nonexistent-dir/x.plt")
        assert ei.value.code == imex.IMEX_ERR_IO


@pytest.mark.parametrize("name,engine", [("f64", "fixed"), ("f64", "native"), ("f32", None), ("f16dev", None)])
def test_checkpoint_resume_is_bit_identical(imex, tmp_path, name, engine):
    shape = (20, 16, 24)
    prec = prec_id(imex, name)
    eng = {None: imex.IMEX_ENGINE_AUTO, "fixed": imex.IMEX_ENGINE_FIXED, "native": imex.IMEX_ENGINE_NATIVE}[engine]
    path = str(tmp_path / "ck.bin")
    with imex.LBM(*shape, 0.004, 1.0, 0.05, precision=prec, engine=eng) as lat:
        lat.Initialize()
        lat.step(7)                      # pending streaming at the save
        lat.checkpoint_save(path)
        lat.step(9)
        want = lat.get_f()
        want_c = lat.Conserved()
    with imex.LBM(*shape, 0.004, 1.0, 0.05, precision=prec, engine=eng) as lat:
        lat.checkpoint_load(path)
        assert lat.steps_done() == 7
        lat.step(9)
        assert lat.steps_done() == 16
        assert np.array_equal(lat.get_f(), want)
        assert lat.Conserved() == want_c


def test_checkpoint_restores_rounding_mode(imex, tmp_path):
    shape = (12, 12, 12)
    path = str(tmp_path / "ck.bin")
    with imex.LBM(*shape, 0.01, 1.0, 0.05, precision=imex.IMEX_F16DEV) as lat:
        lat.set_rounding(imex.IMEX_ROUND_NEAREST)
        lat.Initialize()
        lat.step(3)
        lat.checkpoint_save(path)
        lat.step(5)
        want = lat.get_f()
    with imex.LBM(*shape, 0.01, 1.0, 0.05, precision=imex.IMEX_F16DEV) as lat:   # default: stochastic
        lat.checkpoint_load(path)
        lat.step(5)
        assert np.array_equal(lat.get_f(), want)


def test_checkpoint_errors(imex, tmp_path):
    path = str(tmp_path / "ck.bin")
    with imex.LBM(8, 8, 8, 0.01, 1.0, 0.05) as lat:
        lat.Initialize()
        lat.checkpoint_save(path)
    with imex.LBM(8, 8, 9, 0.01, 1.0, 0.05) as other:
        with pytest.raises(imex.ImexError) as ei:
            other.checkpoint_load(path)          # other size
        assert ei.value.code == imex.IMEX_ERR_ARG
    with imex.LBM(8, 8, 8, 0.01, 1.0, 0.05, precision=imex.IMEX_F32) as other:
        with pytest.raises(imex.ImexError):
            other.checkpoint_load(path)          # other precision
    with imex.LBM(8, 8, 8, 0.01, 1.0, 0.05) as other:
        with pytest.raises(imex.ImexError) as ei:
            other.checkpoint_load(str(tmp_path / "missing.bin"))
        assert ei.value.code == imex.IMEX_ERR_IO
        data = open(path, "rb").read()
        trunc = tmp_path / "trunc.bin"
        trunc.write_bytes(data[: len(data) - 100])
        with pytest.raises(imex.ImexError) as ei:
            other.checkpoint_load(str(trunc))
        assert ei.value.code == imex.IMEX_ERR_IO
        with pytest.raises(imex.ImexError):
            other.step(1)                        # a failed load leaves the lattice uninitialised
        other.checkpoint_load(path)
        other.step(1)


@pytest.mark.parametrize("name", PRECS)
def test_ascii_output_equals_the_reference_format(imex, tmp_path, name):
    """LBM::Output's ASCII dump of f(0) (src/lbm.cpp:606-636): the file equals
    the reference's format (pinned against the reference's own file in
    tests/test_reference_pin.py) applied to the lattice's own f, which a
    pending streaming does not change."""
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from test_reference_pin import RUNS, ascii_dump
    deck = imex.System(text=RUNS["files"]["deck"])
    with imex.LBM(deck.sx, deck.sy, deck.sz, deck.tau, deck.rho0, deck.u0, precision=prec_id(imex, name)) as lat:
        lat.Initialize()
        lat.step(RUNS["files"]["steps"])
        path = lat.Output(1, str(tmp_path / "o.dat"))
        f = lat.get_f()
    data = open(path, "rb").read()
    assert data == ascii_dump(f)
    assert data.decode().splitlines()[:2] == RUNS["files"]["ascii"]["head"][:2]
    if name == "f64":
        # within the reference's printed precision of the reference's own file
        ref = [float(ln.split()[3]) for ln in RUNS["files"]["ascii"]["head"][2:]]
        got = [float(ln.split()[3]) for ln in data.decode().splitlines()[2:6]]
        assert np.allclose(got, ref, rtol=0, atol=1e-8)
