"""RetardedField(t, X) on the device (teufel_cuda_retarded_field, the
SnapshotObserver computation) against the reference's compiled
ChargedParticle::RetardedField(double, Vector) (fixture) and the oracle, and
the reference's electrostatic test run through the device."""
import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import abi, harness as H

from retarded_field_cases import check_electrostatic, load

pytestmark = pytest.mark.gpu


def device_field(tr, t, pos):
    with abi.TrajSet(tr) as ts:
        return ts.retarded_field(t, pos)


def test_device_matches_reference_fixture():
    cases, _ = load()
    for name, (tr, tobs, pos, ref) in cases.items():
        g = device_field(tr, tobs, pos)
        scale = np.abs(ref).max()
        if scale == 0.0:
            assert np.all(g == 0.0), name
        else:
            # the same IEEE operations in the same order; pow() may differ by an ulp
            np.testing.assert_allclose(g, ref, rtol=1e-13, atol=1e-13 * scale, err_msg=name)


def test_device_passes_the_electrostatic_test():
    check_electrostatic(device_field)


def test_device_bunch_matches_oracle():
    w = H.config2(count=64)
    pos = w.pix_pos[::97]
    for tobs in (w.pix_t0[0], w.pix_t0[0] + 1.0e-12, w.pix_t0[0] + 4.0e-12):
        ref, rc = lw.retarded_field_at(w.traj, tobs, pos)
        assert rc == 0
        g = device_field(w.traj, tobs, pos)
        scale = np.abs(ref).max()
        np.testing.assert_allclose(g, ref, rtol=1e-12, atol=1e-12 * max(scale, 1e-300))


def test_particle_without_points_raises():
    tr = load()[0]["rest"][0]
    two = H.Trajectories(tr.t, tr.x, tr.p, tr.a, np.array([1, 0], np.int32),
                         np.array([1.0, 1.0]), np.array([1.0, 1.0]))
    with abi.TrajSet(two) as ts:
        with pytest.raises(abi.TeufelError) as ei:
            ts.retarded_field(0.0, np.zeros((2, 3)))
    assert ei.value.status == abi.TEUFEL_ERR_RANGE
