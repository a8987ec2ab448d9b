"""Batched step: many uneven reduced-precision lattices in one persistent
launch per step.  The batched kernel runs the per-cell arithmetic of the
one-lattice kernels, so every member must end bit-identical to the same
lattice stepped alone - whatever the batch's size mix, launch shape, graph
length, or the members joining, leaving and finishing in between."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [  # shape, precision name, tau, u0, phase
    ((16, 16, 16), "f32", 0.004, 0.05, (0.0, 0.0, 0.0)),
    ((24, 20, 12), "f16dev", 0.02, 0.06, (0.3, 1.1, 2.0)),
    ((32, 32, 32), "f32", 0.0007, 0.04, (1.0, 0.5, 0.25)),
    ((17, 9, 13), "f16dev", 0.01, 0.07, (2.5, 0.1, 4.0)),
    ((8, 8, 8), "f32", 0.1, 0.03, (0.0, 3.0, 1.0)),
    ((1, 5, 40), "f32", 0.05, 0.05, (0.7, 0.7, 0.7)),
]


def prec(imex, name):
    return {"f32": imex.IMEX_F32, "f16dev": imex.IMEX_F16DEV}[name]


def make(imex, spec):
    shape, pname, tau, u0, ph = spec
    lat = imex.LBM(*shape, tau, 1.0, u0, precision=prec(imex, pname))
    lat.initialize_phase(*ph)
    return lat


def alone(imex, spec, steps):
    with make(imex, spec) as lat:
        lat.step(steps)
        return lat.get_f()


def test_batch_equals_alone(imex):
    steps = 23
    want = [alone(imex, s, steps) for s in SPECS]
    lats = [make(imex, s) for s in SPECS]
    with imex.Batch(16) as b:
        for lat in lats:
            b.add(lat)
        b.step(10)
        b.step(13)
        for lat, w in zip(lats, want):
            assert lat.steps_done() == steps
            assert np.array_equal(lat.get_f(), w)
        assert b.kernel_launches() >= steps - 1
    for lat in lats:
        lat.close()


@pytest.mark.parametrize("shape", [(128, 1, 1), (256, 2, 4), (128, 4, 8), (256, 1, 2), (128, 1, 9), (128, 0, 0)])
@pytest.mark.parametrize("graph", [0, 5])
def test_batch_launch_shapes_and_graphs(imex, shape, graph):
    steps = 12
    want = [alone(imex, s, steps) for s in SPECS[:4]]
    lats = [make(imex, s) for s in SPECS[:4]]
    with imex.Batch(8) as b:
        b.set_launch(*shape)
        b.set_graph(graph)
        for lat in lats:
            b.add(lat)
        b.step(steps)
        for lat, w in zip(lats, want):
            assert np.array_equal(lat.get_f(), w)
    for lat in lats:
        lat.close()


ROW_SPECS = SPECS + [  # rows of a multiple of 16 bytes: the row-staged kernel takes these
    ((24, 20, 48), "f16dev", 0.003, 0.05, (0.2, 0.4, 0.6)),
    ((32, 32, 32), "f16dev", 0.001, 0.07, (1.5, 2.5, 0.5)),
    ((16, 12, 64), "f32", 0.02, 0.04, (0.0, 1.0, 2.0)),
    ((9, 7, 8), "f16dev", 0.05, 0.06, (0.3, 0.3, 0.3)),
]


@pytest.mark.parametrize("row_shape", [(-1, 0, 0, 1), (2, 1, 2, 1), (2, 2, 2, 1), (2, 2, 2, 0), (3, 1, 1, 1),
                                       (2, 4, 1, 0), (4, 2, 1, 1)])
@pytest.mark.parametrize("graph", [0, 6])
def test_row_kernel_equals_alone(imex, row_shape, graph):
    """The row-staged batch kernel (and the cell kernel beside it for the
    members it does not take) ends every member where it would alone."""
    steps = 13
    want = [alone(imex, s, steps) for s in ROW_SPECS]
    lats = [make(imex, s) for s in ROW_SPECS]
    with imex.Batch(16) as b:
        b.set_row_launch(*row_shape)
        b.set_graph(graph)
        for lat in lats:
            b.add(lat)
        b.step(steps)
        assert b.get_row_launch() == tuple(row_shape)
        for i, (lat, w) in enumerate(zip(lats, want)):
            assert np.array_equal(lat.get_f(), w), i
    for lat in lats:
        lat.close()


def test_row_kernel_member_limits(imex):
    """Members stop mid-tick at their step limits inside the row kernel."""
    specs = ROW_SPECS[6:]
    limits = [3, 11, -1, 7]
    lats = [make(imex, s) for s in specs]
    with imex.Batch(8) as b:
        b.set_row_launch(2, 1, 2)
        b.set_graph(5)
        for lat, lim in zip(lats, limits):
            b.add(lat, lim)
        b.step(12)
    for lat, spec, lim in zip(lats, specs, limits):
        n = 12 if lim < 0 else lim
        assert lat.steps_done() == n
        assert np.array_equal(lat.get_f(), alone(imex, spec, n))
        lat.close()


def test_row_kernel_graph_while_members_join(imex):
    """A captured graph stays in use while row-kernel members join: the
    member table must fit the launch's shared memory whatever the count."""
    specs = ROW_SPECS[6:] + [SPECS[0], SPECS[2], SPECS[4]]
    lats = [make(imex, s) for s in specs]
    joined_at = [0, 0, 4, 8, 8, 12, 16]
    with imex.Batch(16) as b:
        b.set_row_launch(2, 2, 2)
        b.set_graph(4)
        for t in range(0, 20, 4):
            for lat, j in zip(lats, joined_at):
                if j == t:
                    b.add(lat)
            b.step(4)
        b.synchronize()
    for lat, spec, j in zip(lats, specs, joined_at):
        assert lat.steps_done() == 20 - j
        assert np.array_equal(lat.get_f(), alone(imex, spec, 20 - j))
        lat.close()


def test_row_launch_checks(imex):
    with imex.Batch(2) as b:
        with pytest.raises(imex.ImexError):
            b.set_row_launch(3, 2, 2)         # two CTAs' rings exceed an SM
        with pytest.raises(imex.ImexError):
            b.set_row_launch(2, 3, 1)         # 1 or 2 KiB per direction
        with pytest.raises(imex.ImexError):
            b.set_row_launch(1, 1, 1)         # one stage cannot overlap


def test_members_join_leave_and_finish(imex):
    """Continuous batching: members admitted and retired between steps, with
    per-member step limits, each ending where it would alone."""
    limits = {0: 7, 1: 30, 2: -1, 3: 18}
    lats = [make(imex, s) for s in SPECS[:5]]
    with imex.Batch(8) as b:
        b.set_graph(4)
        b.add(lats[0], limits[0])
        b.add(lats[1], limits[1])
        b.step(5)                     # 0 and 1 at 5
        b.add(lats[2], limits[2])     # joins at step 0
        b.add(lats[3], limits[3])
        b.step(6)                     # 0 stops at 7; 1 at 11; 2, 3 at 6
        b.remove(lats[2])
        lats[2].step(3)               # leaves and continues alone: 9
        b.add(lats[4])                # joins
        b.step(20)                    # 1 at 30 (limit), 3 at 18 (limit), 4 at 20
        b.add(lats[2])
        b.step(4)                     # 2 at 13, 4 at 24
    expect = [7, 30, 13, 18, 24]
    for i, lat in enumerate(lats):
        assert lat.steps_done() == expect[i], (i, lat.steps_done())
        assert np.array_equal(lat.get_f(), alone(imex, SPECS[i], expect[i])), i
        lat.close()


def test_batch_member_diagnostics_match_alone(imex):
    spec = SPECS[2]
    with make(imex, spec) as ref:
        ref.step(15)
        want = ref.Conserved()
    with make(imex, spec) as lat, imex.Batch(2) as b:
        b.add(lat)
        b.step(15)
        assert lat.Conserved() == want


def test_batch_stochastic_rounding_equals_alone(imex):
    spec = SPECS[1]
    with make(imex, spec) as ref:
        ref.set_rounding(imex.IMEX_ROUND_STOCHASTIC)
        ref.step(17)
        want = ref.get_f()
    with make(imex, spec) as lat, make(imex, SPECS[0]) as other, imex.Batch(4) as b:
        lat.set_rounding(imex.IMEX_ROUND_STOCHASTIC)
        b.set_graph(5)
        b.add(other)
        b.add(lat)
        b.step(17)
        assert np.array_equal(lat.get_f(), want)


def test_batch_rejects_float64(imex):
    with imex.LBM(8, 8, 8, 0.1, 1.0, 0.05) as lat, imex.Batch(2) as b:
        lat.Initialize()
        with pytest.raises(imex.ImexError):
            b.add(lat)


def test_segment_kernel_graph_follows_the_members(imex):
    """One CTA per row segment (cells_per_thread 0): the launch covers the
    members' segments, so a member joining or leaving between ticks changes
    the grid; the captured graph must follow, and every member still ends
    where it ends alone."""
    specs = SPECS[:4]
    lats = [make(imex, s) for s in specs]
    with imex.Batch(8) as b:
        b.set_launch(128, 0, 0)
        b.set_row_launch(-1)
        b.set_graph(4)
        for lat in lats[:2]:
            b.add(lat)
        b.step(8)                      # two members
        for lat in lats[2:]:
            b.add(lat)
        b.step(8)                      # four: more segments
        b.remove(lats[0])
        b.step(8)                      # three
        for lat, s in zip(lats, specs):
            assert np.array_equal(lat.get_f(), alone(imex, s, lat.steps_done()))
        assert b.get_launch() == (128, 0, 0)
    for lat in lats:
        lat.close()


def test_segment_kernel_graph_after_a_retune_moves_its_group_table(imex):
    """A re-tune times the row kernel switched off, which puts every member
    in the segment kernel; when that outgrows the segment kernel's group
    table, the table moves.  A graph captured before reads the table through
    a pointer baked into it, so it must be captured again even when the
    tuner settles on the same shapes and the segment count is the one it
    was captured with; every member still ends where it ends alone."""
    specs = [((16, 16, 16), "f32", 0.004, 0.05, (0.0, 0.0, 0.0)),
             ((64, 64, 16), "f16dev", 0.02, 0.06, (0.3, 1.1, 2.0)),
             ((96, 96, 16), "f16dev", 0.01, 0.07, (2.5, 0.1, 4.0))]
    lats = [make(imex, s) for s in specs]
    with imex.Batch(4) as b:
        b.set_graph(4)
        for lat in lats[:2]:
            b.add(lat)
        b.step(8)                      # tuned with the float32 member in the segment kernel, graph captured
        b.add(lats[2])
        b.step(4)                      # a larger float16 member joins the row kernel
        b.set_launch(0, 0, 0)          # re-tune both kernels: a row-kernel-off candidate
        b.set_row_launch(0, 0, 0, 1)   # needs more groups than the table holds
        b.step(8)
        for lat, s in zip(lats, specs):
            assert np.array_equal(lat.get_f(), alone(imex, s, lat.steps_done()))
    for lat in lats:
        lat.close()


@pytest.mark.parametrize("row_shape", [(2, 4, 1), (2, 2, 2), (3, 1, 2)])
def test_row_kernel_many_members_stopping_mid_tick(imex, row_shape):
    """Many float16 members reaching their step limits at staggered steps
    inside the row kernel's ticks: every tick mixes items with bytes and
    items without (a stopped member's), which complete their stage's phase
    on arrival.  Every member ends where it ends alone, at its limit."""
    rng = np.random.default_rng(5)
    specs, limits = [], []
    for q in range(12):
        edge = int(rng.choice([16, 24, 32]))
        specs.append(((edge, edge, edge), "f16dev", 0.01, 0.05, (0.1 * q, 0.2 * q, 0.3 * q)))
        limits.append(int(rng.integers(1, 60)))
    lats = [make(imex, s) for s in specs]
    with imex.Batch(16) as b:
        b.set_row_launch(*row_shape)
        b.set_graph(25)
        for lat, lim in zip(lats, limits):
            b.add(lat, lim)
        b.step(75)
        b.synchronize()
    for lat, spec, lim in zip(lats, specs, limits):
        assert lat.steps_done() == lim
        assert np.array_equal(lat.get_f(), alone(imex, spec, lim))
        lat.close()
