"""The decomposed lattice on the GPU (imex_domain_*) against the undivided one.

The reference's regression calls this its most valuable check
(tests/regression.sh:17-24, 107-126): collision is per cell and streaming a
permutation, so the field must not depend on how the domain is split; only
the order of the final reductions may.  Here every f of a lattice split into
1, 2, 4 and 8 blocks (the reference's own rank grids) must equal the
undivided lattice's bit for bit at every report step, and the conserved mass
and kinetic energy - each block's sums added in rank order - must agree with
the undivided lattice's and with the reference's own `cons` lines on the same
rank count (tests/golden/reference_runs.json) to 1e-12 relative.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RTOL = 1e-12
with open(os.path.join(GOLDEN, "reference_runs.json")) as _fp:
    RUNS = json.load(_fp)


def _deck(imex, name):
    return imex.System(text=RUNS["decks"][name]["deck"])


def _close(a, b, tol=RTOL):
    return abs(a - b) <= tol * abs(b)


@pytest.mark.parametrize("nranks", [1, 2, 4, 8])
def test_decomposed_parity_deck_is_the_undivided_lattice(imex, oracle, nranks):
    """32^3, Re 1600, 100 steps, reporting every 10 (src/main.cpp:69-93)."""
    d = _deck(imex, "parity32")
    ref = {c[0]: c for c in RUNS["decks"]["parity32"]["runs"][str(nranks)]["cons"]}
    f = oracle.init(d.sx, d.sy, d.sz, d.rho0, d.u0)
    with imex.LBM(d.sx, d.sy, d.sz, d.tau, d.rho0, d.u0) as lat, \
            imex.Domain(d.sx, d.sy, d.sz, nranks, d.tau, d.rho0, d.u0) as dom:
        lat.Initialize()
        dom.Initialize()
        assert "rx=%d,ry=%d,rz=%d" % dom.info()["grid"] == RUNS["decks"]["parity32"]["runs"][str(nranks)]["layout"]
        for it in range(d.inter, d.Time + 1, d.inter):
            lat.step(d.inter)
            dom.step(d.inter)
            oracle.step(f, d.tau, d.inter)
            got = dom.get_f()
            assert np.array_equal(got, lat.get_f()), it
            assert np.max(np.abs(got - f) / np.abs(f)) <= RTOL
            c, w, r = dom.Conserved(), lat.Conserved(), ref[it]
            assert _close(c[0], w[0]) and _close(c[4], w[4]), (it, c, w)
            assert _close(c[0], r[1]) and _close(c[4], r[5]), (it, c, r)
            assert max(abs(v) for v in c[1:4]) <= 1e-10
        assert dom.fallback_cells() == 0
        assert dom.info()["steps"] == d.Time


@pytest.mark.parametrize("nranks", [1, 2, 3, 4, 6, 8])
def test_decomposed_ragged_lattice(imex, oracle, nranks):
    """18x20x22: blocks of unequal sizes (the remainder cells go to the low
    coordinates), on the reference's grids for 1-8 ranks."""
    d = _deck(imex, "ragged")
    rec = RUNS["decks"]["ragged"]
    f = oracle.init(d.sx, d.sy, d.sz, d.rho0, d.u0)
    oracle.step(f, d.tau, rec["steps"])
    with imex.LBM(d.sx, d.sy, d.sz, d.tau, d.rho0, d.u0) as lat, \
            imex.Domain(d.sx, d.sy, d.sz, nranks, d.tau, d.rho0, d.u0) as dom:
        lat.Initialize()
        dom.Initialize()
        lat.step(rec["steps"])
        dom.step(rec["steps"])
        got = dom.get_f()
        assert np.array_equal(got, lat.get_f())
        assert np.max(np.abs(got - f) / np.abs(f)) <= RTOL
        c, r = dom.Conserved(), rec["runs"][str(nranks)]["dump_cons_last"]
        assert _close(c[0], r[1]) and _close(c[4], r[5])
        # per-block sums add up to the whole
        blocks = dom.conserved_blocks()
        assert blocks.shape == (nranks, 5)
        assert _close(float(np.sum(blocks[:, 0])), c[0])


def test_halo_is_pruned(imex):
    """A step moves 9 values per face ghost cell, 3 per edge and 1 per corner."""
    n, nranks = (24, 20, 28), 8
    want = 0
    for r in range(nranks):
        L = imex.decomp_block(nranks, *n, r)["len"]
        faces = 2 * (L[1] * L[2] + L[0] * L[2] + L[0] * L[1])
        edges = 4 * (L[0] + L[1] + L[2])
        want += 9 * faces + 3 * edges + 8
    with imex.Domain(*n, nranks, 0.01, 1.0, 0.05) as dom:
        assert dom.info()["halo_values_per_step"] == want


def test_domain_state_and_argument_errors(imex):
    with imex.Domain(8, 8, 8, 2, 0.01, 1.0, 0.05) as dom:
        with pytest.raises(imex.ImexError) as e:
            dom.step(1)
        assert e.value.code == imex.IMEX_ERR_STATE
    with pytest.raises(imex.ImexError):
        imex.Domain(4, 4, 4, 5, 0.01, 1.0, 0.05)   # the grid puts 5 blocks along 4 cells
    with pytest.raises(imex.ImexError):
        imex.Domain(8, 8, 8, 2, 0.01, 2.0, 0.05)   # density outside the fixed-point range


def test_run_leaving_the_fixed_point_range_is_redone(imex):
    """A decomposed run whose cells leave the fixed-point engine's exact range
    partway (a deck that diverges) is redone from the last complete step in
    native float64: every f equals the undivided lattice stepped one step at
    a time, NaNs included, and later calls keep agreeing."""
    shape, tau, u0 = (16, 16, 16), 1e-4, 0.18
    with imex.LBM(*shape, tau, 1.0, u0, engine=imex.IMEX_ENGINE_FIXED) as lat, \
            imex.Domain(*shape, 4, tau, 1.0, u0) as dom:
        lat.Initialize()
        dom.Initialize()
        for n in (40, 3, 7):
            for _ in range(n):
                lat.step(1)
            dom.step(n)
            assert np.array_equal(dom.get_f(), lat.get_f(), equal_nan=True), n
        assert dom.fallback_cells() > 0
        assert dom.info()["steps"] == 50


@pytest.mark.parametrize("nranks,n", [(8, (2, 2, 2)), (27, (3, 3, 3)), (16, (4, 4, 4)), (6, (3, 2, 6)), (9, (3, 3, 9))])
def test_blocks_one_cell_thick(imex, nranks, n):
    """Blocks one cell thick along an axis: a cell on both faces of that axis
    stores its values into both neighbours' ghost shells (and, on a 1x1x1
    block, into every neighbour's); every f still equals the undivided
    lattice's, over runs of odd and even length."""
    tau, u0 = 0.01, 0.05
    with imex.LBM(*n, tau, 1.0, u0) as lat, imex.Domain(*n, nranks, tau, 1.0, u0) as dom:
        assert min(min(imex.decomp_block(nranks, *n, r)["len"]) for r in range(nranks)) == 1
        lat.Initialize()
        dom.Initialize()
        for k in (1, 4, 7, 2):
            lat.step(k)
            dom.step(k)
            assert np.array_equal(dom.get_f(), lat.get_f()), k
        assert dom.fallback_cells() == 0
