"""Reduced-precision storage (float32 f, float16 (f - w) 2^12) against the float64
oracle, through the C ABI.

Tolerances come from the error these formats carry, not from parity:
float32 storage rounds f to 2^-24 relative, float16 rounds f - w to 2^-11
relative.  On the 32^3 Re = 1600 deck over 100 steps the kinetic energy
stays within 2e-5 (float32) and 2e-4 (float16 deviations) of the oracle,
the velocity field within 1e-4 u0 and 5e-3 u0, mass within 1e-8 and 1e-6
relative, and momentum stays zero to 1e-6 of the mass.  Streaming alone
moves stored bits and must be exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W = None


def weights(oracle):
    global W
    if W is None:
        W = oracle.weights()[:, None, None, None]
    return W


def stored(oracle, prec, imex, f):
    """What the storage format keeps of a float64 f, as float64."""
    if prec == imex.IMEX_F32:
        return f.astype(np.float32).astype(np.float64)
    w = weights(oracle)
    return w + ((f - w) * 4096.0).astype(np.float16).astype(np.float64) / 4096.0


PRECS = [("f32", 2e-5, 1e-4, 1e-8), ("f16dev", 2e-4, 5e-3, 1e-6)]


def prec_id(imex, name):
    return {"f32": imex.IMEX_F32, "f16dev": imex.IMEX_F16DEV}[name]


@pytest.mark.parametrize("name", ["f32", "f16dev"])
def test_init_is_rounded_oracle(imex, oracle, name):
    prec = prec_id(imex, name)
    shape = (12, 10, 14)
    with imex.LBM(*shape, 0.01, 1.0, 0.05, precision=prec) as lat:
        lat.Initialize()
        got = lat.get_f()
    want = stored(oracle, prec, imex, oracle.init(*shape, 1.0, 0.05))
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["f32", "f16dev"])
def test_streaming_alone_is_exact(imex, oracle, name):
    prec = prec_id(imex, name)
    shape = (9, 7, 12)
    rng = np.random.default_rng(11)
    w = weights(oracle)
    f = stored(oracle, prec, imex, w * (1.0 + 0.2 * rng.standard_normal((27,) + shape)))
    with imex.LBM(*shape, 0.05, 1.0, 0.05, precision=prec) as lat:
        lat.set_f(f)
        assert np.array_equal(lat.get_f(), f)
        lat.Streaming()
        lat.Streaming()
        got = lat.get_f()
    assert np.array_equal(got, oracle.stream(oracle.stream(f)))


@pytest.mark.parametrize("name,ke_tol,u_tol,mass_tol", PRECS)
def test_deck_32cubed_against_float64(imex, oracle, name, ke_tol, u_tol, mass_tol):
    prec = prec_id(imex, name)
    d = oracle.parse_deck("1.0 0.1 1600\n0.05 100 10\n32 32 32\n")
    f = oracle.init(32, 32, 32, d.rho0, d.u0)
    m0 = oracle.conserved(f)[0]
    with imex.LBM(32, 32, 32, d.tau, d.rho0, d.u0, precision=prec) as lat, \
            imex.LBM(32, 32, 32, d.tau, d.rho0, d.u0) as ref:
        lat.Initialize()
        ref.Initialize()
        for it in range(10, 101, 10):
            lat.step(10)
            ref.step(10)
            oracle.step(f, d.tau, 10)
            c = np.array(lat.Conserved())
            w = oracle.conserved(f)
            assert abs(c[4] - w[4]) <= ke_tol * w[4], (it, c[4], w[4])
            assert abs(c[0] - m0) <= mass_tol * m0
            assert np.abs(c[1:4]).max() <= 1e-6 * m0
            du, umax = lat.velocity_max_diff(ref)
            assert du <= u_tol * d.u0, (it, du)
            assert 0.5 * d.u0 < umax < 1.5 * d.u0


@pytest.mark.parametrize("name", ["f32", "f16dev"])
def test_call_sequences_and_macroscopic(imex, oracle, name):
    prec = prec_id(imex, name)
    shape = (10, 12, 14)
    tau = 0.05
    with imex.LBM(*shape, tau, 1.0, 0.05, precision=prec) as lat:
        lat.Initialize()
        f = stored(oracle, prec, imex, oracle.init(*shape, 1.0, 0.05))
        for op in "CSCSSCCSCS":
            if op == "C":
                lat.Collision()
                oracle.collide(f, tau)
            else:
                lat.Streaming()
                f = oracle.stream(f)
        got = lat.get_f()
        p, u, v, w = lat.ComputeMacroscopic()
    wts = weights(oracle)
    if prec == imex.IMEX_F32:
        assert np.max(np.abs(got - f) / wts) <= 1e-6
    else:
        # every population within 2e-4 of its weight; the corner populations,
        # which take up the other populations' momentum rounding errors,
        # within 2e-4 of the axis weight
        corner = np.abs(oracle.velocities()).sum(1) == 3
        scale = np.where(corner[:, None, None, None], wts[1], wts)
        assert np.max(np.abs(got - f) / scale) <= 2e-4
    for a, b in zip((u, v, w), oracle.macroscopic(got)[1:]):
        assert np.max(np.abs(a - b)) <= 1e-12


def test_fixed_engine_refuses_low_precision(imex):
    with imex.LBM(4, 4, 4, 0.1, 1.0, 0.05, precision=imex.IMEX_F32) as lat:
        with pytest.raises(imex.ImexError):
            lat.set_engine(imex.IMEX_ENGINE_FIXED)


def test_stochastic_rounding_is_deterministic_and_kernel_independent(imex):
    """Stochastic rounding draws its bits from (cell, step): two runs agree
    bit for bit, and so do the one-thread-per-cell and row-staged kernels."""
    shape = (16, 12, 32)
    runs = []
    for stages, rows in [(0, 1), (0, 1), (2, 4)]:
        with imex.LBM(*shape, 0.002, 1.0, 0.05, precision=imex.IMEX_F16DEV) as lat:
            lat.set_rounding(imex.IMEX_ROUND_STOCHASTIC)
            lat.set_launch(stages, rows, 1)
            lat.Initialize()
            lat.step(21)
            runs.append(lat.get_f())
    assert np.array_equal(runs[0], runs[1])
    assert np.array_equal(runs[0], runs[2])
    with imex.LBM(*shape, 0.002, 1.0, 0.05, precision=imex.IMEX_F16DEV) as lat:
        lat.Initialize()
        lat.step(21)
        assert np.array_equal(lat.get_f(), runs[0])       # stochastic rounding is the default
    with imex.LBM(*shape, 0.002, 1.0, 0.05, precision=imex.IMEX_F16DEV) as lat:
        lat.set_rounding(imex.IMEX_ROUND_NEAREST)
        lat.Initialize()
        lat.step(21)
        assert not np.array_equal(lat.get_f(), runs[0])   # nearest rounding differs


def test_stochastic_rounding_keeps_ke_on_the_deck(imex, oracle):
    d = oracle.parse_deck("1.0 0.1 1600\n0.05 100 10\n32 32 32\n")
    f = oracle.init(32, 32, 32, d.rho0, d.u0)
    with imex.LBM(32, 32, 32, d.tau, d.rho0, d.u0, precision=imex.IMEX_F16DEV) as lat:
        lat.set_rounding(imex.IMEX_ROUND_STOCHASTIC)
        lat.Initialize()
        m0 = lat.Conserved()[0]
        lat.step(100)
        oracle.step(f, d.tau, 100)
        c = lat.Conserved()
    w = oracle.conserved(f)
    assert abs(c[4] - w[4]) <= 1e-4 * w[4]
    assert abs(c[0] - m0) <= 1e-6 * m0


def f16_step(x):
    """Spacing of float16 numbers at |x| (normal range)."""
    return 2.0 ** (np.floor(np.log2(np.maximum(np.abs(x), 2.0 ** -14))) - 10)


@pytest.mark.parametrize("rounding", ["nearest", "stochastic"])
def test_float16_rounding_keeps_cell_momentum(imex, oracle, rounding):
    """The float16 rounding moves the momentum of the rounding errors of the
    rest, axis and face-diagonal populations into the eight corner
    populations: after one collision each cell's momentum equals the float64
    collision's to the corners' own rounding, far below one float16 step of
    an axis population (what rounding every value on its own leaves)."""
    shape = (8, 10, 12)
    tau = 0.01
    rng = np.random.default_rng(5)
    w = weights(oracle)
    f = oracle.init(*shape, 1.0, 0.08)
    f = stored(oracle, imex.IMEX_F16DEV, imex, f + 1e-3 * w * rng.standard_normal(f.shape))
    with imex.LBM(*shape, tau, 1.0, 0.08, precision=imex.IMEX_F16DEV) as lat:
        lat.set_rounding(imex.IMEX_ROUND_NEAREST if rounding == "nearest" else imex.IMEX_ROUND_STOCHASTIC)
        lat.set_f(f)
        lat.Collision()
        got = lat.get_f()
    want = f.copy()
    oracle.collide(want, tau)
    e = oracle.velocities().astype(np.float64)
    du = np.tensordot(e.T, got - want, axes=1)
    H = (want - w) * 4096.0
    corner = np.abs(e).sum(1) == 3
    axis = np.abs(e).sum(1) == 1
    corner_step = f16_step(np.abs(H[corner]).max(0)) / 4096.0
    axis_step = f16_step(np.abs(H[axis]).max(0)) / 4096.0
    # each corner rounds once (one step at most); the float32 collision's own
    # error is far below
    assert np.all(np.abs(du) <= (8 * corner_step + 1e-9)[None])
    rms = np.sqrt(np.mean(du ** 2))
    assert rms <= 0.2 * np.sqrt(np.mean(axis_step ** 2)), rms


def test_stochastic_rounding_needs_float16(imex):
    with imex.LBM(4, 4, 4, 0.1, 1.0, 0.05, precision=imex.IMEX_F32) as lat:
        with pytest.raises(imex.ImexError):
            lat.set_rounding(imex.IMEX_ROUND_STOCHASTIC)
