"""Generate tests/golden/*.json from the reference's own test and deck files.

The reference (Maccchiatooo/IMEXLBM) ships no field dumps; its known answers
for the time step live as text in tests/regression.sh and input.in.  This
script reads those files (it runs where the reference's checkout is present;
the tests read only the fixtures it writes) and writes:

  regression_known_answers.json   deck, tolerances, ke trajectory and the
                                  measured residual scale of tests/regression.sh
  shipped_deck.json               the shipped input.in text and its nine fields

Usage: python tests/golden/make_golden.py /path/to/reference
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def line_of(text: str, needle: str) -> int:
    for i, ln in enumerate(text.splitlines(), 1):
        if needle in ln:
            return i
    raise ValueError(f"{needle!r} not found")


def main(ref: str) -> None:
    reg_path = os.path.join(ref, "tests", "regression.sh")
    reg = open(reg_path).read()
    deck_m = re.search(r"printf '([^']*)' > input\.in", reg)
    deck = deck_m.group(1).encode().decode("unicode_escape")
    tol = {k: float(v) for k, v in re.findall(r"^(TOL_[A-Z_]+)=([0-9.eE+-]+)", reg, re.M)}
    ranks = re.search(r'^RANKS="([^"]*)"', reg, re.M).group(1).split()
    traj_m = re.search(r"oscillates \(([0-9.]+) -> ([0-9.]+) -> ([0-9.]+) at (\d+)\^3\)", reg)
    ke = [traj_m.group(i) for i in (1, 2, 3)]
    resid = {}
    for label, key in (("mass drift within a run", "mass_drift"), ("mass across rank counts", "mass_across_ranks"),
                       ("kinetic energy across ranks", "ke_across_ranks")):
        m = re.search(re.escape(label) + r"\s+([0-9.eE+-]+)", reg)
        resid[key] = float(m.group(1))
    out = {
        "source": "tests/regression.sh of Maccchiatooo/IMEXLBM",
        "deck": deck,
        "deck_line": line_of(reg, "printf '"),
        "tolerances": {"mass_drift_rel": tol["TOL_MASS_DRIFT"], "momentum_abs": tol["TOL_MOMENTUM"],
                       "rank_agreement_rel": tol["TOL_RANK_AGREE"]},
        "tolerance_lines": [line_of(reg, "TOL_MASS_DRIFT="), line_of(reg, "TOL_MOMENTUM="),
                            line_of(reg, "TOL_RANK_AGREE=")],
        "ranks": ranks,
        "ke_after_steps_1_2_3": ke,
        "ke_digits_after_point": [len(x.split(".")[1]) for x in ke],
        "ke_line": line_of(reg, "oscillates ("),
        "measured_residuals": resid,
        "measured_residuals_lines": [line_of(reg, "mass drift within a run"), line_of(reg, "kinetic energy across ranks")],
    }
    with open(os.path.join(HERE, "regression_known_answers.json"), "w") as fp:
        json.dump(out, fp, indent=1)
        fp.write("\n")

    deck_text = open(os.path.join(ref, "input.in")).read()
    nums = deck_text.split()[:9]
    with open(os.path.join(HERE, "shipped_deck.json"), "w") as fp:
        json.dump({"source": "input.in of Maccchiatooo/IMEXLBM", "text": deck_text,
                   "fields": dict(zip(["rho0", "R", "Re", "u0", "Time", "inter", "sx", "sy", "sz"], nums))},
                  fp, indent=1)
        fp.write("\n")
    print("wrote", os.path.join(HERE, "regression_known_answers.json"), "and shipped_deck.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])
