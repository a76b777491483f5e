"""teufel_cuda_autotune: picks one of the FP32 configurations by timing them
on the observer, leaves no trace anywhere, and the automatic path then uses
its choice with results still within the FP32 bar of the oracle."""
import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import abi, harness as H

pytestmark = pytest.mark.gpu


def test_autotune_choice_and_parity():
    w = H.config2(count=40)
    w = w.pixel_subset(np.arange(0, w.n_pix, 5))
    ref, rc = lw.integrate_screen(w.traj, w.pix_pos, w.pix_t0, w.dt, w.nots)
    assert rc == 0
    with abi.TrajSet(w.traj) as ts:
        variant, slots, ms = ts.autotune(w.pix_pos, w.pix_t0, w.dt, w.nots)
        assert variant in (1, 4, 5, 6, 7, 8, 10, 11) and slots >= 1 and ms > 0.0
        g = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots)  # automatic: the tuned choice
        g2 = ts.integrate_screen(w.pix_pos, w.pix_t0, w.dt, w.nots, variant=variant,
                                 n_slots=slots)
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < 1e-5
    assert np.array_equal(g, g2)
