"""CPU tests of the oracle against the reference's own known answers.

The reference's only known answers for this path are in tests/regression.sh
(committed as tests/golden/regression_known_answers.json by
tests/golden/make_golden.py): the 32^3 kinetic-energy trajectory after
steps 1-3, the mass-drift and momentum tolerances, and the residual scale.
"""
import numpy as np
import pytest


def _deck(oracle, known_answers):
    return oracle.parse_deck(known_answers["deck"])


def test_known_ke_trajectory(oracle, known_answers):
    """ke after steps 1, 2, 3 of the regression deck matches regression.sh:29."""
    d = _deck(oracle, known_answers)
    f = oracle.init(d.sx, d.sy, d.sz, d.rho0, d.u0)
    got = []
    for _ in range(3):
        oracle.step(f, d.tau, 1)
        got.append(oracle.conserved(f)[4])
    for g, want, nd in zip(got, known_answers["ke_after_steps_1_2_3"], known_answers["ke_digits_after_point"]):
        assert f"{g:.{nd}f}" == want, (g, want)


def test_regression_invariants(oracle, known_answers):
    """The three checks of regression.sh on the 20-step, report-every-step deck."""
    d = _deck(oracle, known_answers)
    tol = known_answers["tolerances"]
    f = oracle.init(d.sx, d.sy, d.sz, d.rho0, d.u0)
    cons = []
    for it in range(1, d.Time + 1):
        oracle.step(f, d.tau, 1)
        if it % d.inter == 0:
            cons.append(oracle.conserved(f))
    cons = np.array(cons)
    assert np.isfinite(cons).all()
    drift = np.abs((cons[:, 0] - cons[0, 0]) / cons[0, 0]).max()
    assert drift <= tol["mass_drift_rel"], drift
    assert np.abs(cons[:, 1:4]).max() <= tol["momentum_abs"]
    # residual scale of the reference's own run (regression.sh:32-36), with 10x room
    assert drift <= 10 * known_answers["measured_residuals"]["mass_drift"]


def test_deck_tau_matches_system_cpp(oracle, known_answers):
    d = _deck(oracle, known_answers)
    # System.cpp:28, left to right with Re an int
    want = 0.05 * 32 / 1600 / (1.0 / 3.0) / 2.0 / 3.1415926
    assert d.tau == want
    assert (d.Re, d.Time, d.inter, d.sx, d.sy, d.sz) == (1600, 20, 1, 32, 32, 32)


def test_stream_is_periodic_permutation(oracle):
    rng = np.random.default_rng(5)
    f = rng.random((27, 5, 4, 3))
    ft = oracle.stream(f)
    e = oracle.velocities()
    for a in range(27):
        want = np.roll(f[a], shift=tuple(e[a]), axis=(0, 1, 2))
        assert np.array_equal(ft[a], want)


def test_collision_conserves_moments(oracle):
    rng = np.random.default_rng(7)
    w = oracle.weights()
    f = w[:, None, None, None] * (1.0 + 0.05 * rng.standard_normal((27, 6, 5, 4)))
    e = oracle.velocities().astype(float)
    m0 = f.sum(0)
    p0 = np.einsum("a...,ad->d...", f, e)
    oracle.collide(f, 0.01)
    assert np.abs(f.sum(0) - m0).max() < 1e-15
    assert np.abs(np.einsum("a...,ad->d...", f, e) - p0).max() < 1e-15


def test_equilibrium_is_fixed_point(oracle):
    """Init builds feq of its own moments, so collision leaves it (nearly) unchanged."""
    f = oracle.init(8, 8, 8, 1.0, 0.05)
    g = f.copy()
    oracle.collide(g, 0.3)
    assert np.abs(g - f).max() < 1e-15


def test_threads_bitwise(oracle):
    f1 = oracle.init(12, 10, 14, 1.0, 0.05)
    f2 = f1.copy()
    oracle.set_threads(1)
    oracle.step(f1, 0.01, 3)
    oracle.set_threads(max(2, oracle.max_threads()))
    oracle.step(f2, 0.01, 3)
    oracle.set_threads(1)
    assert np.array_equal(f1, f2)


def test_weights_and_velocities(oracle):
    w = oracle.weights()
    e = oracle.velocities()
    assert abs(w.sum() - 1.0) < 1e-15
    assert np.abs(w @ e).max() < 1e-15
    assert np.allclose(np.einsum("a,ai,aj->ij", w, e, e), np.eye(3) / 3)
    opp = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17, 20, 19, 22, 21, 24, 23, 26, 25]
    assert np.array_equal(e[opp], -e)


def test_minmax_uvwp(oracle):
    f = oracle.init(9, 7, 5, 1.0, 0.05)
    oracle.step(f, 0.01, 3)
    p, u, v, w = oracle.macroscopic(f)
    got = oracle.minmax_uvwp(f)
    want = [u.max(), v.max(), w.max(), p.max(), u.min(), v.min(), w.min(), p.min()]
    assert list(got) == want


def test_tecplot_layout(oracle, tmp_path):
    """The oracle's output<n>.plt follows the byte layout LBM::MPIoutput
    writes (src/lbm.cpp:397-591): section ends at bytes 20, 80, 120, 172,
    220 and 332 as the reference's own comments count them, then seven
    x-fastest float64 blocks."""
    import struct
    nx, ny, nz = 6, 5, 4
    f = oracle.init(nx, ny, nz, 1.0, 0.05)
    path = tmp_path / "output7.plt"
    oracle.write_tecplot(f, 7, str(path))
    b = path.read_bytes()
    n = nx * ny * nz
    assert len(b) == 332 + 7 * n * 8
    assert b[:8] == b"#!TDV112"
    assert struct.unpack_from("<3i", b, 8) == (1, 0, 0)
    assert struct.unpack_from("<15i", b, 20) == (7, 120, 0, 121, 0, 122, 0, 117, 0, 118, 0, 119, 0, 112, 0)
    assert struct.unpack_from("<f9i", b, 80) == (299.0, 90, 79, 78, 69, 32, 48, 48, 49, 0)
    assert struct.unpack_from("<i", b, 120)[0] == -1
    assert struct.unpack_from("<d", b, 124)[0] == 7.0
    assert struct.unpack_from("<10i", b, 132) == (0, -1, 0, 0, 0, 0, nx, ny, nz, 0)
    assert struct.unpack_from("<ff7i3i", b, 172) == (357.0, 299.0, 2, 2, 2, 2, 2, 2, 2, 0, 0, -1)
    rng = struct.unpack_from("<14d", b, 220)
    mm = oracle.minmax_uvwp(f)
    assert rng == (0.0, 1.0, 0.0, 1.0, 0.0, 1.0, mm[4], mm[0], mm[5], mm[1], mm[6], mm[2], mm[7], mm[3])
    blocks = np.frombuffer(b, dtype="<f8", offset=332).reshape(7, nz, ny, nx)
    i = np.arange(nx)
    assert np.array_equal(blocks[0][2, 3], i / (nx - 1))
    assert np.array_equal(blocks[2][:, 0, 0], np.arange(nz) / (nz - 1))
    p, u, v, w = oracle.macroscopic(f)
    for blk, fld in zip(blocks[3:], (u, v, w, p)):
        assert np.array_equal(blk, fld.transpose(2, 1, 0))
