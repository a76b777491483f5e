"""The allocation-free entry point, teufel_cuda_integrate_screen_noalloc.

It is meant for callers that cannot let the library call cudaMalloc (their
device memory belongs to another allocator, or they must not allocate while
running because cudaMalloc/cudaFree can synchronize the device).  It keeps its
partial traces in a fixed device array shared by all calls, so the test calls
it twice in a row and checks both results against the allocating entry point
(teufel_cuda_integrate_screen_ex with device pointers), within the FP32-split
tolerance the other GPU tests use.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from teufel_gb300 import abi, harness as H

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def noalloc(ts, pos, t0, dt, nots, n_pix, out, stream=0):
    return abi.lib().teufel_cuda_integrate_screen_noalloc(
        ts.handle, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(t0.data_ptr()), dt, nots,
        n_pix, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))


def test_noalloc_matches_allocating_entry_twice():
    import torch
    dev = torch.device("cuda", 0)
    w = H.config1()
    pos = torch.from_numpy(w.pix_pos).to(dev)
    t0 = torch.from_numpy(w.pix_t0).to(dev)
    shape = (w.n_pix, w.nots, 6)
    assert w.n_pix * w.nots * 6 * 4 <= abi.NOALLOC_SCRATCH_BYTES
    with abi.TrajSet(w.traj) as ts:
        ref = torch.zeros(shape, dtype=torch.float64, device=dev)
        ts.integrate_screen_device(pos.data_ptr(), t0.data_ptr(), w.dt, w.nots, w.n_pix,
                                   ref.data_ptr())
        torch.cuda.synchronize(dev)
        ref = ref.cpu().numpy()
        assert np.abs(ref).max() > 0
        results = []
        for _ in range(2):
            out = torch.zeros(shape, dtype=torch.float64, device=dev)
            st = noalloc(ts, pos, t0, w.dt, w.nots, w.n_pix, out)
            assert st == abi.TEUFEL_OK, abi.status_string(st)
            results.append(out.cpu().numpy())
    for r in results:
        assert rel_l2(r, ref) < TOL_FP32
    # the second call starts from a cleared array: same result as the first
    assert np.array_equal(results[0], results[1])


def test_noalloc_rejects_observers_beyond_the_array():
    import torch
    dev = torch.device("cuda", 0)
    w = H.config1()
    nots = 8192  # 441 pixels x 8192 samples x 24 B = 86.7 MB > 64 MiB
    assert w.n_pix * nots * 6 * 4 > abi.NOALLOC_SCRATCH_BYTES
    pos = torch.from_numpy(w.pix_pos).to(dev)
    t0 = torch.from_numpy(w.pix_t0).to(dev)
    out = torch.zeros((w.n_pix, nots, 6), dtype=torch.float64, device=dev)
    with abi.TrajSet(w.traj) as ts:
        st = noalloc(ts, pos, t0, w.dt, nots, w.n_pix, out)
        # the warp kernel needs dt > 0 (a negative dt reverses the window)
        st_neg = noalloc(ts, pos, t0, -w.dt, 16, w.n_pix, out)
    assert st == abi.TEUFEL_ERR_ARG
    assert st_neg == abi.TEUFEL_ERR_ARG
    assert float(out.abs().max()) == 0.0
