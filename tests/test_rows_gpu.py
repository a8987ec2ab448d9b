"""The row-staged fused kernel (bulk copies into a shared-memory ring) and
the launch-shape autotuner.

The row kernel runs the same per-cell arithmetic as the one-thread-per-cell
kernel, so for every precision, lattice shape and ring configuration the two
must produce bit-identical distributions.  Cells outside the fixed-point
engine's exact range must take the native float64 path in both kernels.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(32, 32, 32), (17, 19, 24), (3, 1, 16), (8, 8, 64), (40, 3, 48)]
RING = [(2, 1, 1), (3, 2, 1), (2, 4, 2), (4, 1, 2), (2, 8, 1), (3, 3, 1)]


def prec_ids(imex):
    return {"f64": imex.IMEX_F64, "f32": imex.IMEX_F32, "f16dev": imex.IMEX_F16DEV}


def run(imex, shape, prec, stages, rows, ctas, steps=9, tau=0.003):
    with imex.LBM(*shape, tau, 1.0, 0.06, precision=prec) as lat:
        lat.set_launch(stages, rows, ctas)
        lat.Initialize()
        lat.step(steps)
        got = lat.get_f()
        assert lat.fallback_cells() == 0
        return got, lat.Conserved()


@pytest.mark.parametrize("pname", ["f64", "f32", "f16dev"])
@pytest.mark.parametrize("shape", SHAPES)
def test_rows_bitwise_equal_classic(imex, shape, pname):
    prec = prec_ids(imex)[pname]
    ref, cref = run(imex, shape, prec, 0, 1, 1)
    for stages, rows, ctas in RING:
        try:
            got, c = run(imex, shape, prec, stages, rows, ctas)
        except imex.ImexError as e:  # ring does not fit, or rows do not divide / exceed ny
            assert "shared memory" in str(e) or "divide" in str(e) or "exceed" in str(e)
            continue
        assert np.array_equal(got, ref), (shape, pname, stages, rows, ctas)
        assert c == cref


def test_rows_match_oracle_on_the_deck(imex, oracle):
    d = oracle.parse_deck("1.0 0.1 1600\n0.05 100 10\n32 32 32\n")
    f = oracle.init(32, 32, 32, d.rho0, d.u0)
    with imex.LBM(32, 32, 32, d.tau, d.rho0, d.u0) as lat:
        lat.set_launch(3, 2, 1)
        lat.Initialize()
        lat.step(100)
        oracle.step(f, d.tau, 100)
        got = lat.get_f()
    assert np.max(np.abs(got - f) / f) <= 1e-12


def test_odd_rows_refuse_ring(imex):
    with imex.LBM(4, 4, 17, 0.01, 1.0, 0.05) as lat:
        with pytest.raises(imex.ImexError):
            lat.set_launch(3, 1, 1)


def test_autotuner_picks_a_valid_shape(imex, oracle):
    shape = (24, 16, 32)
    with imex.LBM(*shape, 0.003, 1.0, 0.05) as lat:
        lat.Initialize()
        stages, rows, ctas, threads = lat.get_launch()
        assert stages == 0 or (stages >= 2 and rows >= 1 and 16 % rows == 0 and ctas >= 1 and threads >= 32)
        lat.step(5)
        got = lat.get_f()
    f = oracle.init(*shape, 1.0, 0.05)
    oracle.step(f, 0.003, 5)
    assert np.max(np.abs(got - f) / f) <= 1e-12


@pytest.mark.parametrize("stages,rows", [(0, 1), (3, 1), (2, 3)])
def test_out_of_range_cells_fall_back_to_float64(imex, oracle, stages, rows):
    """A few cells with negative or huge distributions leave the fixed-point
    range; they must be computed in native float64 and counted."""
    shape = (8, 6, 16)
    tau = 0.01
    f = oracle.init(*shape, 1.0, 0.05)
    f[3, 2, 1, 5] = -0.02      # negative
    f[0, 5, 4, 9] = 1.7        # rest population above 1
    f[19, 7, 0, 15] = 1e-6     # below 2^-9
    with imex.LBM(*shape, tau, 1.0, 0.05, engine=imex.IMEX_ENGINE_FIXED) as lat:
        lat.set_launch(stages, rows, 1)
        lat.set_f(f)
        lat.Collision()        # in place (native), then fused steps
        lat.Streaming()
        lat.step(3)
        got = lat.get_f()
        assert lat.fallback_cells() > 0
    g = f.copy()
    oracle.step(g, tau, 4)
    assert np.all(np.abs(got - g) <= 1e-12 * np.maximum(np.abs(g), 1e-2))
