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


@pytest.mark.parametrize("N,gmap", [(16, 1), (7, 0)])
def test_noalloc_matches_allocating_green_apply(gpulib, N, gmap):
    import torch
    L = gpulib.load_library()
    r = rve.make_rve(N, 3, 5)
    N3 = N ** 3
    rng = np.random.default_rng(N)
    Fn = np.zeros((9, N3))
    Fn[[0, 4, 8]] = 1.0
    Fn1 = Fn + 1e-3 * rng.standard_normal((9, N3))
    x = rng.standard_normal((9, N3))
    solver = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gmap)
    try:
        _, K4, _ = solver.drive_eps_sig(1, 0, Fn, Fn1, want_P=False, want_K4=True)
        refs = {True: solver.G_K_dF(x, True), False: solver.G_K_dF(x, False)}
    finally:
        solver.close()
    dev = torch.device("cuda:0")
    xd = torch.from_numpy(x).to(dev)
    kd = torch.from_numpy(K4).to(dev)
    yd = torch.zeros_like(xd)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for flgK in (True, True, False, False):  # two calls in a row per mode
        yd.fill_(float("nan"))
        rc = L.cpfft_green_apply_noalloc(N, gmap, ctypes.c_void_p(xd.data_ptr()),
                                         ctypes.c_void_p(kd.data_ptr()), int(flgK),
                                         ctypes.c_void_p(yd.data_ptr()), stream)
        assert rc == 0, L.cpfft_last_error()
        torch.cuda.synchronize(dev)
        assert _rel(yd.cpu().numpy(), refs[flgK]) < 1e-11


def test_noalloc_rejects_grids_beyond_its_scratch(gpulib):
    L = gpulib.load_library()
    rc = L.cpfft_green_apply_noalloc(33, 1, ctypes.c_void_p(1), ctypes.c_void_p(1), 1,
                                     ctypes.c_void_p(1), None)
    assert rc == -5
    assert b"outside [2, 32]" in L.cpfft_last_error()
