"""Device-side failure paths, made to fire without faulting the GPU.

The row-staged kernels wait on mbarriers for their asynchronous copies, and
every wait is bounded.  The test hook imex_test_set_fault makes CTA 0 arm the
first stage of its ring without issuing that stage's copies, with a short
wait limit: the wait runs out, the CTA records the failure, waits (bounded)
for the copies it still has in flight and returns.  Nothing is in flight and
nothing spins forever.  The next synchronising call must report
IMEX_ERR_CUDA, and the handle must work again once the hook is cleared.
The reference has no such path: it aborts (src/System.cpp:17-21)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# 4e6 SM clocks (about 2 ms): far above the time any legitimate copy of
# these small lattices takes, so only the starved stage runs out.
WAIT = 4_000_000
TAU, RHO0, U0 = 0.003, 1.0, 0.05


@pytest.fixture
def fault(imex):
    L = imex.load()

    def set_fault(kind, value=0):
        assert L.imex_test_set_fault(kind, value) == 0

    yield set_fault
    L.imex_test_set_fault(0, 0)


def test_fault_hook_rejects_bad_arguments(imex):
    L = imex.load()
    assert L.imex_test_set_fault(1, 10) == imex.IMEX_ERR_ARG
    assert L.imex_test_set_fault(7, 0) == imex.IMEX_ERR_ARG
    assert L.imex_test_set_fault(0, 0) == 0


@pytest.mark.parametrize("precision,launch", [(0, (2, 1, 1)), (2, (2, 4, 1)), (1, (3, 2, 1))])
def test_starved_copy_is_reported_and_the_handle_recovers(imex, oracle, fault, precision, launch):
    shape = (32, 32, 32)
    with imex.LBM(*shape, TAU, RHO0, U0, precision=precision) as lat:
        lat.set_launch(*launch)
        lat.Initialize()
        lat.step(1)                      # in-place collision: the next steps are fused row launches
        fault(imex.IMEX_TEST_FAULT_STARVE_STAGE, WAIT)
        lat.step(2)
        with pytest.raises(imex.ImexError) as e:
            lat.Conserved()
        assert e.value.code == imex.IMEX_ERR_CUDA
        assert "did not complete in time" in str(e.value)
        fault(imex.IMEX_TEST_FAULT_NONE)
        # the error was reported once; a fresh run on the same handle is clean
        lat.Initialize()
        lat.step(6)
        cons = lat.Conserved()
        got = lat.get_f()
    f = oracle.init(*shape, RHO0, U0)
    oracle.step(f, TAU, 6)
    want = oracle.conserved(f)
    tol = 1e-12 if precision == 0 else 2e-4
    assert abs(cons[0] - want[0]) <= tol * abs(want[0])
    assert abs(cons[4] - want[4]) <= tol * abs(want[4])
    if precision == 0:
        assert np.max(np.abs(got - f) / f) <= 1e-12


def test_starved_copy_in_the_batch_row_kernel(imex, fault):
    with imex.LBM(32, 32, 32, TAU, RHO0, U0, precision=imex.IMEX_F16DEV) as a, \
            imex.LBM(48, 16, 64, TAU, RHO0, U0, precision=imex.IMEX_F32) as b, imex.Batch(4) as batch:
        for lat in (a, b):
            lat.Initialize()
            batch.add(lat)
        batch.set_graph(0)               # direct launches: each reads the hook
        batch.set_row_launch(2, 4, 1, True)
        batch.step(2)
        batch.synchronize()
        fault(imex.IMEX_TEST_FAULT_STARVE_STAGE, WAIT)
        batch.step(2)
        with pytest.raises(imex.ImexError) as e:
            batch.synchronize()
        assert e.value.code == imex.IMEX_ERR_CUDA
        assert "did not complete in time" in str(e.value)
        fault(imex.IMEX_TEST_FAULT_NONE)
        batch.step(2)
        batch.synchronize()


def test_batch_table_refusal_is_reported(imex, fault):
    """The batch row kernel refuses a member table larger than the shared
    memory its launch was given; the refusal reaches the host."""
    with imex.LBM(32, 32, 32, TAU, RHO0, U0, precision=imex.IMEX_F16DEV) as a, \
            imex.LBM(32, 16, 32, TAU, RHO0, U0, precision=imex.IMEX_F16DEV) as b, imex.Batch(4) as batch:
        for lat in (a, b):
            lat.Initialize()
            batch.add(lat)
        batch.set_graph(0)
        batch.set_row_launch(2, 2, 1, True)
        batch.step(1)                    # first collisions run alone, in place
        fault(imex.IMEX_TEST_FAULT_BATCH_TABLE)
        batch.step(2)
        with pytest.raises(imex.ImexError) as e:
            batch.synchronize()
        assert e.value.code == imex.IMEX_ERR_CUDA
        assert "member table" in str(e.value)
        fault(imex.IMEX_TEST_FAULT_NONE)
        batch.step(3)
        batch.synchronize()
        assert np.all(np.isfinite(a.Conserved(allow_nonfinite=True)))
