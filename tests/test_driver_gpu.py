"""The imexlbm driver executable, checked the way the reference's
tests/regression.sh checks its binary: run the 32^3 deck for 20 steps
reporting every step, parse the ``cons`` lines with the regression's field
layout, and assert (1) mass drift <= 1e-12 relative, (2) |momentum| <=
1e-10, (3) agreement with an independent run - here the CPU oracle in place
of the regression's 2- and 4-rank runs - to 1e-12 relative, and no NaN/Inf.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "imexlbm_gb300", "_build", "imexlbm")


def run_driver(tmp_path, deck, *args):
    (tmp_path / "input.in").write_text(deck)
    r = subprocess.run([EXE, *args], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def cons_lines(out):
    rows = []
    for ln in out.splitlines():
        if ln.startswith("cons"):
            fld = re.split(r"[ |]+", ln)
            # regression.sh:87-89 field layout (1-based): 3 it, 5 mass, 7 px, 9 py, 11 pz, 13 ke
            rows.append([float(fld[i - 1]) for i in (3, 5, 7, 9, 11, 13)])
    return np.array(rows)


@pytest.mark.parametrize("engine", ["", "--engine=native"])
def test_regression_checks(imex, oracle, known_answers, tmp_path, engine):
    deck = known_answers["deck"]
    tol = known_answers["tolerances"]
    out = run_driver(tmp_path, deck, *([engine] if engine else []))
    assert "rx=1,ry=1,rz=1" in out and "3D Taylor-Green Vortex" in out
    assert len([l for l in out.splitlines() if l.startswith("collision |")]) == 20
    assert len([l for l in out.splitlines() if "MLUPS" in l]) == 20
    c = cons_lines(out)
    assert c.shape == (20, 6)
    assert not re.search(r"nan|inf", "\n".join(l for l in out.splitlines() if l.startswith("cons")), re.I)
    mass = c[:, 1]
    assert np.abs((mass - mass[0]) / mass[0]).max() <= tol["mass_drift_rel"]
    assert np.abs(c[:, 2:5]).max() <= tol["momentum_abs"]
    d = oracle.parse_deck(deck)
    f = oracle.init(d.sx, d.sy, d.sz, d.rho0, d.u0)
    for row in c:
        oracle.step(f, d.tau, 1)
        w = oracle.conserved(f)
        assert abs(row[1] - w[0]) <= tol["rank_agreement_rel"] * abs(w[0])
        assert abs(row[5] - w[4]) <= tol["rank_agreement_rel"] * abs(w[4])
    # known answers of regression.sh:29
    for got, want in zip(c[:3, 5], known_answers["ke_after_steps_1_2_3"]):
        assert f"{got:.3f}" == want


def test_scaling_build_flag_same_answers(imex, known_answers, tmp_path):
    a = cons_lines(run_driver(tmp_path, known_answers["deck"]))
    out = run_driver(tmp_path, known_answers["deck"], "--no-perstep-timing")
    assert "collision |" not in out
    assert np.array_equal(a, cons_lines(out))


def test_runs_between_reports_same_answers(imex, tmp_path):
    """Without per-step timing the driver runs the steps between report steps
    as one call (fixed-point runs on the float64 engine): the report lines
    carry the same numbers as one Collision()/Streaming() pair per step."""
    deck = "1.0 0.1 1600\n0.05 47 10\n32 32 32\n"
    a = cons_lines(run_driver(tmp_path, deck))
    b = cons_lines(run_driver(tmp_path, deck, "--no-perstep-timing"))
    assert len(a) == 4 and np.array_equal(a, b)


def test_missing_deck_fails(imex, tmp_path):
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr
