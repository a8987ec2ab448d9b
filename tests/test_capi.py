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


def test_null_and_range_checks_of_every_entry_point(imex):
    """Host-side argument checks that run before any CUDA call."""
    L = imex.load()
    out = (ctypes.c_double * 8)()
    assert L.imex_conserved(None, out) == 1
    assert L.imex_minmax_uvwp(None, out) == 1
    assert L.imex_write_tecplot(None, b"x.plt", 1) == 1
    assert L.imex_checkpoint_save(None, b"x") == 1
    assert L.imex_checkpoint_load(None, b"x") == 1
    assert L.imex_profile_enable(None, 1) == 1
    assert L.imex_set_launch(None, 2, 1, 1) == 1
    assert L.imex_set_rounding(None, 0) == 1
    assert L.imex_steps_done(None) == -1
    b = ctypes.c_void_p()
    assert L.imex_batch_create(0, ctypes.byref(b)) == 1
    assert L.imex_batch_create(4096, ctypes.byref(b)) == 1
    assert L.imex_batch_add(None, None, -1) == 1
    assert L.imex_batch_step(None, 1) == 1
    assert L.imex_batch_set_row_launch(None, 2, 1, 1, 1) == 1
    s = ctypes.c_void_p()
    assert L.imex_server_create(0, 4, 5, ctypes.byref(s)) == 1
    assert L.imex_server_create(10**9, 0, 5, ctypes.byref(s)) == 1
    assert L.imex_server_create(10**9, 4, 0, ctypes.byref(s)) == 1
    assert L.imex_server_submit(None, None, None) == 1
    n = ctypes.c_int()
    assert L.imex_server_poll(None, None, 0, ctypes.byref(n)) == 1
    assert L.imex_server_now(None) == -1.0
    L.imex_server_destroy(None)
    L.imex_batch_destroy(None)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_batch_and_server_without_gpu_fail_cleanly(imex):
    L = imex.load()
    b = ctypes.c_void_p()
    assert L.imex_batch_create(4, ctypes.byref(b)) == 2 and not b.value
    s = ctypes.c_void_p()
    assert L.imex_server_create(10**9, 4, 5, ctypes.byref(s)) == 2 and not s.value
    assert L.imex_last_error(None)


def test_struct_layouts_match_header(imex, tmp_path):
    """The ctypes mirrors of the ABI's structs have the header's sizes and
    field offsets (compiled here from include/imexlbm.h with the C compiler) -
    what a cgo / JNI binding must also lay out."""
    import shutil
    import subprocess
    from imexlbm_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    checks = {"imex_request": (_lib.Request, ["nx", "precision", "tau", "phase", "steps", "tag", "resume_path",
                                              "save_path"]),
              "imex_result": (_lib.Result, ["id", "status", "conserved", "steps", "t_done"]),
              "imex_server_stats": (_lib.ServerStats, ["queued", "busy_seconds", "failed"]),
              "imex_phase_stats": (_lib.PhaseStats, ["calls", "max_ms"]),
              "imex_deck": (_lib.Deck, ["rho0", "Re", "sz", "tau"])}
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "imexlbm.h"', "int main(void) {"]
    for st, (_, fields) in checks.items():
        src.append(f'printf("{st} %zu\\n", sizeof({st}));')
        for f in fields:
            src.append(f'printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    src.append("return 0; }")
    (tmp_path / "layout.c").write_text("\n".join(src))
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I", inc, str(tmp_path / "layout.c"), "-o", str(tmp_path / "layout")], check=True)
    out = dict(line.split() for line in subprocess.run([str(tmp_path / "layout")], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for st, (py, fields) in checks.items():
        assert int(out[st]) == ctypes.sizeof(py), st
        for f in fields:
            assert int(out[f"{st}.{f}"]) == getattr(py, f).offset, (st, f)
