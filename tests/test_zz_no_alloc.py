"""imex_conserved_noalloc: the diagnostics entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (a host code whose device
memory belongs to its own pool allocator, or a latency-critical loop that
cannot afford cudaMalloc's implicit device synchronisation).  Its scratch is
a static device array inside the library, so this test checks that calls in
a row - on different lattices - each give what the handle-based
imex_conserved gives, to the tolerances of the parity tests (mass and ke
1e-12 relative, momentum 1e-10 absolute), that a larger lattice's partial
sums left in the shared scratch do not change a later smaller call's result,
and that a call takes no device memory.

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _device_f(torch, lat):
    """A test-owned device copy of lat's f (reference order)."""
    n = 27 * lat.glx * lat.gly * lat.glz
    f_dev = torch.empty(n, dtype=torch.float64, device="cuda")
    lat.get_f_device(f_dev.data_ptr(), n)
    return f_dev


def _noalloc(imex, torch, lat, f_dev, out):
    """Reduce f_dev (lat's shape) into the device buffer out with the
    no-alloc entry point; returns the 5 diagnostics."""
    out.fill_(float("nan"))
    torch.cuda.synchronize()
    L = imex.load()
    rc = L.imex_conserved_noalloc(ctypes.c_void_p(f_dev.data_ptr()), lat.glx, lat.gly, lat.glz,
                                  ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0, L.imex_last_error(None)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _check(got, want):
    assert abs(got[0] - want[0]) <= RTOL * abs(want[0])
    assert abs(got[4] - want[4]) <= RTOL * abs(want[4])
    assert np.abs(np.asarray(got[1:4]) - np.asarray(want[1:4])).max() <= 1e-10


def test_noalloc_matches_conserved_twice(imex):
    """Calls in a row on a small lattice, a larger one (which leaves more
    partial sums in the shared scratch than the small one writes), and the
    small one again: each matches imex_conserved, the two small results are
    bit-identical, and the repeated call takes no device memory."""
    torch = pytest.importorskip("torch")
    d_tau = 0.05 * 48 / 1600 / (1.0 / 3.0) / 2.0 / 3.1415926
    with imex.LBM(48, 40, 36, d_tau, 1.0, 0.05) as big, imex.LBM(17, 19, 23, 0.02, 1.0, 0.06) as small:
        big.Initialize()
        big.step(12)
        small.Initialize()
        small.step(5)
        f_big, f_small = _device_f(torch, big), _device_f(torch, small)
        out = torch.empty(5, dtype=torch.float64, device="cuda")
        first = _noalloc(imex, torch, small, f_small, out)
        _check(first, small.Conserved())
        second = _noalloc(imex, torch, big, f_big, out)
        _check(second, big.Conserved())
        free_before = torch.cuda.mem_get_info()[0]
        held_before = torch.cuda.memory_allocated()
        third = _noalloc(imex, torch, small, f_small, out)
        assert torch.cuda.mem_get_info()[0] == free_before
        assert torch.cuda.memory_allocated() == held_before
        # the larger lattice's partial sums left in the scratch do not leak in
        assert np.array_equal(first, third)


def test_noalloc_rejects_oversize(imex):
    L = imex.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.imex_conserved_noalloc(dummy, 512, 512, 512, dummy, None)
    assert rc == 1
    assert b"131072" in L.imex_last_error(None)
    assert L.imex_conserved_noalloc(None, 8, 8, 8, dummy, None) == 1
