"""CPU tests of the C ABI: the library loads, exports every declared symbol,
and its host-side logic (deck parsing, argument checks) behaves like the
reference's System class.  No compute call runs here."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "imexlbm.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(imex_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_expected_surface():
    names = declared_functions()
    for must in ("imex_create", "imex_initialize", "imex_collision", "imex_streaming", "imex_conserved",
                 "imex_get_f", "imex_destroy", "imex_deck_parse", "imex_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(imex):
    L = imex.load()
    from imexlbm_gb300._lib import SIGNATURES
    for name in declared_functions():
        assert hasattr(L, name), name
        assert name in SIGNATURES, f"{name} has no ctypes signature"


def test_deck_parse_matches_oracle(imex, oracle, known_answers, shipped_deck):
    texts = [known_answers["deck"], shipped_deck["text"], "2.5 0 100\n0.08 5 2\n17 19 23\n",
             "  1e0\t0.1 3200 5e-2 1000 100 256 256 256 trailing words"]
    for t in texts:
        s = imex.System(text=t)
        d = oracle.parse_deck(t)
        for name in ("rho0", "R", "u0", "Re", "Time", "inter", "sx", "sy", "sz", "cs2", "cs", "Ma", "miu", "tau"):
            assert getattr(s, name) == getattr(d, name), (t, name)


def test_deck_int_field_stops_at_dot(imex):
    # operator>>(int&) stops at '.', so "1600.0" gives Re = 1600 and the rest
    # of the token (".0") is read as u0 - the stream semantics of System.cpp:22.
    s = imex.System(text="1.0 0.1 1600.0 20 1 32 32 32 32")
    assert s.Re == 1600 and s.u0 == 0.0 and s.Time == 20 and s.inter == 1


def test_deck_errors(imex, tmp_path):
    with pytest.raises(imex.ImexError) as e:
        imex.System(text="1.0 0.1")
    assert e.value.code == 4
    with pytest.raises(imex.ImexError) as e:
        imex.System(path=str(tmp_path / "no_such_input.in"))
    assert e.value.code == 4 and "cannot open" in str(e.value)


def test_deck_read_file(imex, tmp_path, shipped_deck):
    p = tmp_path / "input.in"
    p.write_text(shipped_deck["text"])
    s = imex.System(path=str(p))
    assert (s.sx, s.sy, s.sz, s.Time, s.inter) == (256, 256, 256, 20, 1)


def test_create_argument_checks(imex):
    L = imex.load()
    h = ctypes.c_void_p()
    assert L.imex_create(0, 4, 4, 0.1, 1.0, 0.05, 0, ctypes.byref(h)) == 1
    assert b"sizes" in L.imex_last_error(None)
    assert L.imex_create(4, 4, 4, -0.6, 1.0, 0.05, 0, ctypes.byref(h)) == 1
    assert L.imex_create(4, 4, 4, 0.1, 1.0, 0.05, 0, None) == 1
    assert L.imex_initialize(None) == 1
    assert L.imex_collision(None) == 1
    L.imex_destroy(None)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_cleanly(imex):
    L = imex.load()
    h = ctypes.c_void_p()
    rc = L.imex_create(8, 8, 8, 0.1, 1.0, 0.05, 0, ctypes.byref(h))
    assert rc == 2 and not h.value
    assert L.imex_last_error(None)
