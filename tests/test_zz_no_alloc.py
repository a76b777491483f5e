"""The allocation-free entry point, teufel_cuda_integrate_screen_noalloc.

It is meant for callers that cannot let the library call cudaMalloc (their
device memory belongs to another allocator, or they must not allocate while
running because cudaMalloc/cudaFree can synchronize the device).  It keeps its
partial traces in a fixed device array shared by all calls, so the tests call
it twice in a row and check both results against the CPU oracle and against
the allocating entry point (teufel_cuda_integrate_screen_ex with device
pointers), within the FP32-split tolerance the other GPU tests use; they check
that the device's free memory does not change across a call; and one case is
large enough to need two passes through the array.  This file is collected
last on purpose.
"""
import ctypes

import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import abi, harness as H

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def noalloc(ts, pos, t0, dt, nots, n_pix, out, stream=0):
    return abi.lib().teufel_cuda_integrate_screen_noalloc(
        ts.handle, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(t0.data_ptr()), dt, nots,
        n_pix, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))


def run_twice(w, dev):
    """Two allocation-free calls in a row (each into a fresh zeroed buffer),
    the device's free memory around the second, and the allocating entry's
    result on the same inputs."""
    import torch
    pos = torch.from_numpy(np.ascontiguousarray(w.pix_pos)).to(dev)
    t0 = torch.from_numpy(np.ascontiguousarray(w.pix_t0)).to(dev)
    shape = (w.n_pix, w.nots, 6)
    assert w.n_pix * w.nots * 6 * 4 <= abi.NOALLOC_SCRATCH_BYTES
    outs = [torch.zeros(shape, dtype=torch.float64, device=dev) for _ in range(2)]
    ref = torch.zeros(shape, dtype=torch.float64, device=dev)
    with abi.TrajSet(w.traj) as ts:
        st = noalloc(ts, pos, t0, w.dt, w.nots, w.n_pix, outs[0])
        assert st == abi.TEUFEL_OK, abi.status_string(st)
        torch.cuda.synchronize(dev)
        free_before, _ = torch.cuda.mem_get_info(dev)
        st = noalloc(ts, pos, t0, w.dt, w.nots, w.n_pix, outs[1])
        torch.cuda.synchronize(dev)
        free_after, _ = torch.cuda.mem_get_info(dev)
        assert st == abi.TEUFEL_OK, abi.status_string(st)
        ts.integrate_screen_device(pos.data_ptr(), t0.data_ptr(), w.dt, w.nots, w.n_pix,
                                   ref.data_ptr())
        torch.cuda.synchronize(dev)
    return [o.cpu().numpy() for o in outs], ref.cpu().numpy(), free_before, free_after


def test_noalloc_matches_oracle_and_allocating_entry_twice():
    import torch
    dev = torch.device("cuda", 0)
    w = H.config1()
    results, ref, free_before, free_after = run_twice(w, dev)
    # a call makes no device allocation: the free memory is unchanged
    assert free_after == free_before, (free_before, free_after)
    oracle, rc = lw.integrate_screen(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
    assert rc == 0 and np.abs(oracle).max() > 0
    for r in results:
        assert rel_l2(r, oracle) < TOL_FP32
        assert rel_l2(r, ref) < TOL_FP32
    # the second call starts from a cleared array: same result as the first
    assert np.array_equal(results[0], results[1])


def test_noalloc_two_passes():
    """1024 pixels x 2048 samples x 24 B = 50 MB: one slot fills the array,
    and 2100 particles need two slots (2048 particles per slot at most), so
    the call runs two passes, each clearing the array and adding its slot
    into the output."""
    import torch
    dev = torch.device("cuda", 0)
    w = H.config2(count=2100)
    w = w.pixel_subset(np.arange(0, w.n_pix, 4))
    slot_bytes = w.n_pix * w.nots * 6 * 4
    assert 2 * slot_bytes > abi.NOALLOC_SCRATCH_BYTES >= slot_bytes
    assert w.traj.n_particles > 2048
    results, ref, free_before, free_after = run_twice(w, dev)
    assert free_after == free_before, (free_before, free_after)
    for r in results:
        assert rel_l2(r, ref) < TOL_FP32
    assert np.array_equal(results[0], results[1])
    # against the oracle on every 16th of these pixels
    sel = np.arange(0, w.n_pix, 16)
    sub = w.pixel_subset(sel)
    oracle, rc = lw.integrate_screen(sub.traj, sub.pix_pos, sub.pix_t0, sub.dt, sub.nots)
    assert rc == 0
    assert rel_l2(results[1][sel], oracle) < TOL_FP32


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
        # the warp kernel needs a finite dt > 0 (a negative dt reverses the window)
        st_neg = noalloc(ts, pos, t0, -w.dt, 16, w.n_pix, out)
        st_inf = noalloc(ts, pos, t0, float("inf"), 16, w.n_pix, out)
        st_nan = noalloc(ts, pos, t0, float("nan"), 16, w.n_pix, out)
    assert st == abi.TEUFEL_ERR_ARG
    assert st_neg == abi.TEUFEL_ERR_ARG
    assert st_inf == abi.TEUFEL_ERR_ARG
    assert st_nan == abi.TEUFEL_ERR_ARG
    assert float(out.abs().max()) == 0.0
