"""imex_conserved_noalloc: the diagnostics entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (a host code whose device
memory belongs to its own pool allocator, or a latency-critical loop that
cannot afford cudaMalloc's implicit device synchronisation).  Its scratch is
a static device array inside the library, so this test checks that two
calls in a row - on different lattices, the larger first - both give what
the handle-based imex_conserved gives, to the tolerances of the parity tests
(mass and ke 1e-12 relative, momentum 1e-10 absolute).

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _noalloc(imex, torch, lat):
    """Copy lat's f into a test-owned device buffer and reduce it with the
    no-alloc entry point; returns the 5 diagnostics."""
    n = 27 * lat.glx * lat.gly * lat.glz
    f_dev = torch.empty(n, dtype=torch.float64, device="cuda")
    lat.get_f_device(f_dev.data_ptr(), n)
    out = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
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
    torch = pytest.importorskip("torch")
    d_tau = 0.05 * 48 / 1600 / (1.0 / 3.0) / 2.0 / 3.1415926
    with imex.LBM(48, 40, 36, d_tau, 1.0, 0.05) as big, imex.LBM(17, 19, 23, 0.02, 1.0, 0.06) as small:
        big.Initialize()
        big.step(12)
        small.Initialize()
        small.step(5)
        first = _noalloc(imex, torch, big)
        _check(first, big.Conserved())
        second = _noalloc(imex, torch, small)
        _check(second, small.Conserved())
        # the shared scratch keeps the first call's partial sums; the second
        # call's answer must not depend on them
        assert not np.allclose(first[0], second[0])


def test_noalloc_rejects_oversize(imex):
    L = imex.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.imex_conserved_noalloc(dummy, 512, 512, 512, dummy, None)
    assert rc == 1
    assert b"131072" in L.imex_last_error(None)
    assert L.imex_conserved_noalloc(None, 8, 8, 8, dummy, None) == 1
