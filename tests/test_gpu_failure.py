"""Failure paths made on the host: an allocation failure injected through the
caller's device-memory bound (teufel_options.max_device_mib).

A call that cannot run within the bound returns TEUFEL_ERR_NOMEM (the status
a failed cudaMalloc gives) before it touches the caller's trace buffer; a
bound that holds only some of the slots runs them as successive passes, each
reduced into the traces, with the result of the unbounded call.
"""
import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import abi, harness as H

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def c1():
    return H.config1()


@pytest.mark.parametrize("precision", [abi.PREC_FP32_SPLIT, abi.PREC_FP64])
def test_bound_too_small_returns_nomem_and_leaves_out_untouched(c1, precision):
    base = np.random.default_rng(5).normal(size=(c1.n_pix, c1.nots, 6))
    out = base.copy()
    with abi.TrajSet(c1.traj) as ts:
        with pytest.raises(abi.TeufelError) as ei:
            ts.integrate_screen(c1.pix_pos, c1.pix_t0, c1.dt, c1.nots, out=out,
                                precision=precision, max_device_mib=8)
        assert ei.value.status == abi.TEUFEL_ERR_NOMEM
        # the handle stays usable: the same call without the bound runs
        g = ts.integrate_screen(c1.pix_pos, c1.pix_t0, c1.dt, c1.nots, precision=precision)
    assert np.array_equal(out, base)
    assert np.abs(g).max() > 0


def test_bound_holding_two_slots_runs_passes(c1):
    """441 pixels x 2048 samples: a slot's FP32 partial traces are 21.7 MB,
    the staged pixel and trace buffers 43.4 MB.  A bound of both plus two
    slots runs six slots as three passes."""
    slot = c1.n_pix * c1.nots * 6 * 4
    staged = 8 * (4 * c1.n_pix + c1.n_pix * c1.nots * 6)
    mib = (staged + 2 * slot) // (1 << 20) + 1
    with abi.TrajSet(c1.traj) as ts:
        bounded = ts.integrate_screen(c1.pix_pos, c1.pix_t0, c1.dt, c1.nots, n_slots=6,
                                      variant=4, max_device_mib=mib)
        _, _, launches, _, _ = ts.last_timing()
        free = ts.integrate_screen(c1.pix_pos, c1.pix_t0, c1.dt, c1.nots, n_slots=6, variant=4)
        _, _, launches_free, _, _ = ts.last_timing()
    # two launches (integration, reduction) per pass
    assert launches == 6 and launches_free == 2
    assert rel_l2(bounded, free) < 1e-6
    ref, rc = lw.integrate_screen(c1.traj, c1.pix_pos, c1.pix_t0, c1.dt, c1.nots)
    assert rc == 0
    assert rel_l2(bounded, ref) < TOL_FP32
