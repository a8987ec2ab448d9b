"""GPU parity of the CUDA path against the CPU oracle, through the C ABI.

Tolerance: every f_a of every cell within 1e-12 relative of the oracle
(|gpu - oracle| <= 1e-12 * |oracle|), the bound the reference's single-rank
run must meet; reductions within 1e-12 relative (mass, ke) and momentum
within the regression's absolute 1e-10.  Streaming alone is a permutation
and must be bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
ENGINES = ["native", "fixed"]


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


def engine_id(imex, name):
    return {"native": imex.IMEX_ENGINE_NATIVE, "fixed": imex.IMEX_ENGINE_FIXED}[name]


def make(imex, shape, tau, rho0=1.0, u0=0.05, engine="native"):
    lat = imex.LBM(*shape, tau, rho0, u0)
    try:
        lat.set_engine(engine_id(imex, engine))
    except imex.ImexError:
        lat.close()
        pytest.skip(f"{engine} engine not available")
    return lat


def test_init_matches_oracle(imex, oracle):
    for shape in [(16, 16, 16), (17, 19, 23), (1, 1, 8), (3, 2, 1)]:
        with imex.LBM(*shape, 0.01, 1.0, 0.05) as lat:
            lat.Initialize()
            got = lat.get_f()
        want = oracle.init(*shape, 1.0, 0.05)
        assert np.array_equal(got, want), shape


@pytest.mark.parametrize("engine", ENGINES)
def test_regression_deck_32cubed_100_steps(imex, oracle, engine):
    """The 32^3 deck rho0=1, Re=1600, u0=0.05: 100 steps, report every 10.
    Conserved at every report step (steady-state fused path, no
    materialisation), all f_a at step 100."""
    d = oracle.parse_deck("1.0 0.1 1600\n0.05 100 10\n32 32 32\n")
    lat = make(imex, (32, 32, 32), d.tau, engine=engine)
    lat.Initialize()
    f = oracle.init(32, 32, 32, d.rho0, d.u0)
    for it in range(1, 101):
        lat.Collision()
        lat.Streaming()
        oracle.step(f, d.tau, 1)
        if it % 10 == 0:
            c = np.array(lat.Conserved())
            w = oracle.conserved(f)
            assert abs(c[0] - w[0]) <= RTOL * abs(w[0])
            assert abs(c[4] - w[4]) <= RTOL * abs(w[4])
            assert np.abs(c[1:4]).max() <= 1e-10
    got = lat.get_f()
    assert rel_err(got, f) <= RTOL
    assert lat.steps_done() == 100
    lat.close()


@pytest.mark.parametrize("engine", ENGINES)
def test_every_f_at_every_report_step(imex, oracle, engine):
    """get_f at each report step (materialises the pending streaming)."""
    d = oracle.parse_deck("1.0 0.1 1600\n0.05 100 10\n32 32 32\n")
    lat = make(imex, (32, 32, 32), d.tau, engine=engine)
    lat.Initialize()
    f = oracle.init(32, 32, 32, d.rho0, d.u0)
    worst = 0.0
    for it in range(10, 101, 10):
        lat.step(10)
        oracle.step(f, d.tau, 10)
        worst = max(worst, rel_err(lat.get_f(), f))
    assert worst <= RTOL, worst
    lat.close()


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("shape", [(17, 19, 23), (8, 8, 8), (1, 1, 16), (2, 3, 5), (40, 1, 33), (5, 64, 2)])
def test_ragged_shapes(imex, oracle, shape, engine):
    tau = 0.02
    lat = make(imex, shape, tau, u0=0.06, engine=engine)
    lat.Initialize()
    f = oracle.init(*shape, 1.0, 0.06)
    lat.step(7)
    oracle.step(f, tau, 7)
    assert rel_err(lat.get_f(), f) <= RTOL
    c = np.array(lat.Conserved())
    w = oracle.conserved(f)
    assert abs(c[0] - w[0]) <= RTOL * abs(w[0])
    # ke of a degenerate lattice (e.g. 1x1xN, where only acoustic motion
    # survives) is itself a cancellation residue: floor of 1e-18 per cell
    assert abs(c[4] - w[4]) <= RTOL * abs(w[4]) + 1e-18 * np.prod(shape)
    lat.close()


def test_streaming_alone_is_bitwise(imex, oracle):
    rng = np.random.default_rng(3)
    shape = (9, 7, 12)
    f = rng.random((27,) + shape)
    with imex.LBM(*shape, 0.05, 1.0, 0.05) as lat:
        lat.set_f(f)
        lat.Streaming()
        lat.Streaming()
        got = lat.get_f()
    assert np.array_equal(got, oracle.stream(oracle.stream(f)))


@pytest.mark.parametrize("engine", ENGINES)
def test_call_sequences(imex, oracle, engine):
    """Any order of Collision/Streaming keeps the reference's meaning."""
    shape = (10, 12, 14)
    tau = 0.05
    seq = "CSCSSCCSCSCCSS"
    lat = make(imex, shape, tau, engine=engine)
    lat.Initialize()
    f = oracle.init(*shape, 1.0, 0.05)
    for op in seq:
        if op == "C":
            lat.Collision()
            oracle.collide(f, tau)
        else:
            lat.Streaming()
            f = oracle.stream(f)
    assert rel_err(lat.get_f(), f) <= RTOL
    lat.close()


def test_macroscopic(imex, oracle):
    shape = (12, 10, 16)
    tau = 0.01
    with imex.LBM(*shape, tau, 1.0, 0.05) as lat:
        lat.Initialize()
        lat.step(5)
        p, u, v, w = lat.ComputeMacroscopic()
    f = oracle.init(*shape, 1.0, 0.05)
    oracle.step(f, tau, 5)
    for got, want in zip((p, u, v, w), oracle.macroscopic(f)):
        assert np.max(np.abs(got - want)) <= 1e-13


def test_set_get_roundtrip_and_restart(imex, oracle):
    """Checkpoint f, continue, restore, continue again: same answer."""
    shape = (16, 8, 12)
    tau = 0.02
    with imex.LBM(*shape, tau, 1.0, 0.05) as lat:
        lat.Initialize()
        lat.step(4)
        ck = lat.get_f()
        lat.step(6)
        a = lat.get_f()
        lat.set_f(ck)
        lat.step(6)
        b = lat.get_f()
    assert np.array_equal(a, b)


def test_fixed_point_run_equals_single_steps(imex):
    """imex_step(n) on the fixed-point engine keeps the state as 64-bit fixed
    point between its launches; single steps go through float64 every step.
    Both hold the same numbers, so the results are bit-identical."""
    with imex.LBM(24, 20, 32, 0.003, 1.0, 0.05, engine=imex.IMEX_ENGINE_FIXED) as a, \
            imex.LBM(24, 20, 32, 0.003, 1.0, 0.05, engine=imex.IMEX_ENGINE_FIXED) as b:
        for lat in (a, b):
            lat.set_launch(0, 1, 1)
            lat.Initialize()
        a.step(50)
        for _ in range(50):
            b.step(1)
        assert np.array_equal(a.get_f(), b.get_f())
        assert a.Conserved() == b.Conserved()


def test_fixed_point_run_redone_from_failing_step(imex, oracle):
    """A run whose cells leave the exact range partway (an under-resolved
    Mach-0.3 deck: the first value leaves [2^-9, 1/8) after ~30 steps) is
    redone from the last complete step with the per-cell float64 fallback:
    the result equals stepping one step at a time, bit for bit."""
    shape, tau, u0, n = (16, 16, 16), 1e-4, 0.18, 40
    with imex.LBM(*shape, tau, 1.0, u0, engine=imex.IMEX_ENGINE_FIXED) as a, \
            imex.LBM(*shape, tau, 1.0, u0, engine=imex.IMEX_ENGINE_FIXED) as b:
        for lat in (a, b):
            lat.set_launch(0, 1, 1)
            lat.Initialize()
        a.step(n)
        first = None
        for s in range(1, n + 1):
            b.step(1)
            if first is None and b.fallback_cells() > 0:
                first = s
        assert first is not None and first >= 3   # the run fails after its first launch
        assert a.fallback_cells() > 0
        assert np.array_equal(a.get_f(), b.get_f(), equal_nan=True)
        # the failure is remembered: the next call steps one at a time (10
        # launches) instead of a run that fails again and is redone
        before = a.kernel_launches()
        a.step(10)
        assert a.kernel_launches() - before == 10
        for _ in range(10):
            b.step(1)
        assert np.array_equal(a.get_f(), b.get_f(), equal_nan=True)


def test_nonfinite_is_reported(imex):
    """A diverging request (Mach ~1.7) is reported by status, not a crash."""
    with imex.LBM(16, 16, 16, 1e-4, 1.0, 1.0) as lat:
        lat.Initialize()
        status = None
        for _ in range(60):
            lat.step(10)
            try:
                lat.Conserved()
            except imex.ImexError as e:
                status = e.code
                break
        assert status == 5
        vals = lat.Conserved(allow_nonfinite=True)
        assert not all(np.isfinite(vals))


def test_state_errors(imex):
    with imex.LBM(4, 4, 4, 0.1, 1.0, 0.05) as lat:
        with pytest.raises(imex.ImexError) as e:
            lat.Collision()
        assert e.value.code == 6
        with pytest.raises(imex.ImexError):
            lat.get_f(np.empty(10))


def test_benchmarked_fixed_point_run_against_oracle(imex, oracle):
    """The kernel bench.py times: the one-thread-per-cell shape pinned, so
    that every imex_step(10) of the 32^3 regression deck is a fixed-point
    run of k_step_fxs (one in-place collision opens the first), checked in
    every f against the oracle at each report step of src/main.cpp:69-93
    (every 10 steps, 100 steps)."""
    d = oracle.parse_deck("1.0 0.1 1600\n0.05 100 10\n32 32 32\n")
    f = oracle.init(32, 32, 32, d.rho0, d.u0)
    with imex.LBM(32, 32, 32, d.tau, d.rho0, d.u0, engine=imex.IMEX_ENGINE_FIXED) as lat:
        lat.set_launch(0, 1, 1)
        lat.Initialize()
        assert lat.get_launch()[0] == 0
        for report in range(1, 11):
            before = lat.kernel_launches()
            lat.step(10)
            # a run of 10 launches: reading f leaves the streaming pending,
            # so only the first run opens with the in-place collision
            assert lat.kernel_launches() - before == 10
            oracle.step(f, d.tau, 10)
            got = lat.get_f()
            assert rel_err(got, f) <= RTOL, report
            c, w = np.array(lat.Conserved()), oracle.conserved(f)
            assert abs(c[0] - w[0]) <= RTOL * abs(w[0]) and abs(c[4] - w[4]) <= RTOL * abs(w[4])
        assert lat.fallback_cells() == 0
        assert lat.steps_done() == 100


def test_get_f_leaves_the_streaming_pending(imex):
    """Reading f pulls through the pending streaming into the destination
    (pinned host, pageable host or device) without changing the handle:
    the next step is one fused launch, and the three reads agree."""
    torch = pytest.importorskip("torch")
    with imex.LBM(16, 12, 20, 0.01, 1.0, 0.05, engine=imex.IMEX_ENGINE_FIXED) as lat:
        lat.set_launch(0, 1, 1)
        lat.Initialize()
        lat.step(3)
        n = 27 * 16 * 12 * 20
        pageable = lat.get_f()
        pinned = torch.empty(n, dtype=torch.float64, pin_memory=True)
        lat.get_f(pinned.numpy().reshape(lat.shape))
        dev = torch.empty(n, dtype=torch.float64, device="cuda")
        lat.get_f_device(dev.data_ptr(), n)
        torch.cuda.synchronize()
        assert np.array_equal(pageable.ravel(), pinned.numpy())
        assert np.array_equal(pageable.ravel(), dev.cpu().numpy())
        before = lat.kernel_launches()
        lat.step(1)
        assert lat.kernel_launches() - before == 1


@pytest.mark.parametrize("shape,ring,ctas", [((32, 32, 32), 4, 5), ((32, 32, 32), 16, 6), ((9, 5, 7), 4, 1),
                                             ((8, 4, 16), 6, 2), ((17, 19, 23), 12, 5), ((12, 40, 33), 8, 6)])
def test_two_steps_per_launch_equal_single_steps(imex, oracle, shape, ring, ctas):
    """Runs of two fused steps per launch (launch shape stages 1: the first
    step's values through the ring of x-planes, rows ordered by tickets and
    flags) give the one-step run's numbers bit for bit, odd and even step
    counts, for ring depths 4..16 and both CTA residencies, and stay within
    1e-12 of the oracle."""
    tau = 0.004
    with imex.LBM(*shape, tau, 1.0, 0.05, engine=imex.IMEX_ENGINE_FIXED) as a, \
            imex.LBM(*shape, tau, 1.0, 0.05, engine=imex.IMEX_ENGINE_FIXED) as b:
        a.set_launch(1, ring, ctas)
        assert a.get_launch()[:3] == (1, ring, ctas)
        b.set_launch(0, 1, 1)
        for lat in (a, b):
            lat.Initialize()
        for n in (9, 4, 13, 3):
            a.step(n)
            b.step(n)
            assert np.array_equal(a.get_f(), b.get_f()), n
        assert a.fallback_cells() == 0
        got = a.get_f()
        assert a.Conserved() == b.Conserved()
    f = oracle.init(*shape, 1.0, 0.05)
    oracle.step(f, tau, 29)
    assert rel_err(got, f) <= RTOL


def test_two_steps_per_launch_redone_from_failing_launch(imex):
    """A run in two-step launches whose cells leave the exact range partway is
    redone from the failing launch's source state; the result equals single
    steps bit for bit."""
    shape, tau, u0, n = (16, 16, 16), 1e-4, 0.18, 40
    with imex.LBM(*shape, tau, 1.0, u0, engine=imex.IMEX_ENGINE_FIXED) as a, \
            imex.LBM(*shape, tau, 1.0, u0, engine=imex.IMEX_ENGINE_FIXED) as b:
        a.set_launch(1, 1, 1)
        b.set_launch(0, 1, 1)
        for lat in (a, b):
            lat.Initialize()
        a.step(n)
        for _ in range(n):
            b.step(1)
        assert a.fallback_cells() > 0
        assert np.array_equal(a.get_f(), b.get_f(), equal_nan=True)


def test_two_step_shape_is_refused_where_it_does_not_apply(imex):
    with imex.LBM(6, 8, 8, 0.01, 1.0, 0.05) as lat:        # nx < 8
        with pytest.raises(imex.ImexError):
            lat.set_launch(1, 1, 1)
    with imex.LBM(8, 4, 8, 0.01, 1.0, 0.05) as lat:        # the lag of a 16-plane ring exceeds nx * ny
        lat.set_launch(1, 4, 5)
        for bad in ((1, 16, 5), (1, 17, 5), (1, 4, 7)):
            with pytest.raises(imex.ImexError):
                lat.set_launch(*bad)
    with imex.LBM(16, 16, 16, 0.01, 1.0, 0.05, precision=imex.IMEX_F32) as lat:
        with pytest.raises(imex.ImexError):
            lat.set_launch(1, 1, 1)
