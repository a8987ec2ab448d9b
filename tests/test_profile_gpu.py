"""Per-phase device-time accounting (imex_profile_*) and the driver's
--profile report in the reference's per-phase table format."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_phase_counts_and_reset(imex):
    with imex.LBM(32, 16, 24, 0.01, 1.0, 0.05) as lat:
        lat.Initialize()
        lat.step(2)                       # before profiling: not counted
        lat.profile_enable(True)
        lat.step(10)
        lat.Conserved()
        lat.ComputeMacroscopic()
        lat.minmax_uvwp()
        lat.get_f()                       # materialises the pending streaming
        st = lat.profile_read()
        assert st["collision"]["calls"] == 10
        assert st["conserved"]["calls"] == 1
        assert st["macro"]["calls"] == 2
        assert st["stream"]["calls"] == 1
        for ph in st.values():
            if ph["calls"]:
                assert 0 < ph["min_ms"] <= ph["total_ms"] / ph["calls"] <= ph["max_ms"]
        lat.profile_read(reset=True)
        assert lat.profile_read()["collision"]["calls"] == 0
        lat.profile_enable(False)
        lat.step(3)
        assert lat.profile_read()["collision"]["calls"] == 0


def test_profile_survives_many_launches(imex):
    """More launches than the pending-event window: folded in as it fills."""
    with imex.LBM(16, 16, 16, 0.01, 1.0, 0.05, precision=imex.IMEX_F32) as lat:
        lat.Initialize()
        lat.profile_enable(True)
        lat.step(1200)
        assert lat.profile_read()["collision"]["calls"] == 1200


def test_driver_profile_report(imex, tmp_path):
    from imexlbm_gb300 import build
    exe = build.EXE
    (tmp_path / "input.in").write_text("1.0 0.1 1600\n0.05 20 10\n32 32 32\n")
    r = subprocess.run([exe, "--no-perstep-timing", "--profile"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert "=== per-phase profile: 1 ranks, 19 timed steps ===" in out
    assert any(ln.startswith("STEP TOTAL") for ln in out.splitlines())
    coll = [ln for ln in out.splitlines() if ln.startswith("  collision (kernel)")]
    assert len(coll) == 1 and float(coll[0].split()[2]) > 0
    assert any(ln.startswith("collision ") and "GB/s" not in ln for ln in out.splitlines())
    assert "workload/rank: 32768 interior cells" in out


def test_driver_output_files(imex, oracle, tmp_path):
    from imexlbm_gb300 import build
    (tmp_path / "input.in").write_text("1.0 0.1 1600\n0.05 20 10\n16 16 16\n")
    r = subprocess.run([build.EXE, "--no-perstep-timing", "--output"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    for n in (1, 2):
        assert os.path.getsize(tmp_path / f"output{n}.plt") == 332 + 7 * 8 * 16 ** 3
    # the file of report 2 is the oracle's writer on the oracle's state after 20 steps
    d = oracle.parse_deck("1.0 0.1 1600\n0.05 20 10\n16 16 16\n")
    f = oracle.init(16, 16, 16, d.rho0, d.u0)
    oracle.step(f, d.tau, 20)
    oracle.write_tecplot(f, 2, str(tmp_path / "want.plt"))
    got = (tmp_path / "output2.plt").read_bytes()
    want = (tmp_path / "want.plt").read_bytes()
    assert got[:332 - 8 * 8] == want[:332 - 8 * 8]      # header up to the field ranges
    import numpy as np
    a = np.frombuffer(got, dtype="<f8", offset=220)
    b = np.frombuffer(want, dtype="<f8", offset=220)
    assert np.max(np.abs(a - b)) <= 1e-12                 # ranges and fields: float64 parity
