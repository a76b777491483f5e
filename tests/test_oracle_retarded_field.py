"""The oracle's RetardedField(t, X) against the reference's compiled
ChargedParticle::RetardedField(double, Vector) (fixture), and against the
reference's electrostatic test.  Bit-exact on x86-64 (no FMA)."""
import platform

import numpy as np

from oracle import lw

from retarded_field_cases import check_electrostatic, load

EXACT = platform.machine() == "x86_64"


def test_oracle_matches_reference_fixture():
    cases, _ = load()
    assert len(cases) == 9
    for name, (tr, tobs, pos, ref) in cases.items():
        out, rc = lw.retarded_field_at(tr, tobs, pos)
        assert rc == 0
        if EXACT:
            assert np.array_equal(out, ref), name
        else:
            np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-300)
    # the undulator sets cover no signal yet, back-extrapolation and the
    # interpolation inside the trajectory
    assert np.all(cases["undulator_5"][3] == 0.0)
    assert np.abs(cases["undulator_4"][3]).max() > 0.0


def test_oracle_passes_the_electrostatic_test():
    check_electrostatic(lambda tr, t, pos: lw.retarded_field_at(tr, t, pos)[0])


def test_particle_without_points_is_an_error():
    cases, _ = load()
    tr = cases["rest"][0]
    from teufel_gb300 import harness as H
    empty = H.Trajectories(tr.t, tr.x, tr.p, tr.a, np.array([1, 0], np.int32),
                           np.array([1.0, 1.0]), np.array([1.0, 1.0]))
    _, rc = lw.retarded_field_at(empty, 0.0, np.zeros((1, 3)))
    assert rc == 4
