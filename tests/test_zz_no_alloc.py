"""cpfft_green_apply_noalloc: the Green-operator apply for callers that cannot allocate
device memory (programs whose device memory all belongs to their own pool allocator, or
that run under a fixed device-memory budget).  It keeps its scratch in a static device
array and works on the caller's device buffers.  Checked through the C-ABI against the
allocating entry point cpfft_green_apply on two calls in a row, within the tolerance of
the other Green parity tests (1e-11 relative).  Collected last so that a run stopping at
the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from cpfft_gb300 import rve

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("N,gmap", [(32, 1), (16, 1), (7, 0)])
def test_noalloc_matches_allocating_green_apply(gpulib, N, gmap):
    """The allocation-free calls come first, with no library context in this test (the
    documented use: no cpfft_init at all); the allocating entry point then evaluates the
    same operator on the same tangent.  N = 32 fills the static scratch exactly."""
    import torch
    L = gpulib.load_library()
    N3 = N ** 3
    rng = np.random.default_rng(N)
    x = rng.standard_normal((9, N3))
    # a tangent field near a stiff elastic one, different in every voxel
    K4 = np.zeros((81, N3))
    for i in range(9):
        K4[10 * i] = 1.0e5
    K4 += 2.0e4 * rng.standard_normal((81, N3))
    dev = torch.device("cuda:0")
    xd = torch.from_numpy(x).to(dev)
    kd = torch.from_numpy(K4).to(dev)
    yd = torch.zeros_like(xd)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    got = {}
    for flgK in (True, True, False, False):  # two calls in a row per mode
        yd.fill_(float("nan"))
        rc = L.cpfft_green_apply_noalloc(N, gmap, ctypes.c_void_p(xd.data_ptr()),
                                         ctypes.c_void_p(kd.data_ptr()), int(flgK),
                                         ctypes.c_void_p(yd.data_ptr()), stream)
        assert rc == 0, L.cpfft_last_error()
        torch.cuda.synchronize(dev)
        got.setdefault(flgK, []).append(yd.cpu().numpy())
    r = rve.make_rve(N, 3, 5)
    solver = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gmap)
    try:
        solver.set_K4(K4)
        refs = {True: solver.G_K_dF(x, True), False: solver.G_K_dF(x, False)}
    finally:
        solver.close()
    for flgK, ys in got.items():
        for y in ys:
            assert _rel(y, refs[flgK]) < 1e-11


def test_noalloc_rejects_grids_beyond_its_scratch(gpulib):
    L = gpulib.load_library()
    rc = L.cpfft_green_apply_noalloc(33, 1, ctypes.c_void_p(1), ctypes.c_void_p(1), 1,
                                     ctypes.c_void_p(1), None)
    assert rc == -5
    assert b"outside [2, 32]" in L.cpfft_last_error()
