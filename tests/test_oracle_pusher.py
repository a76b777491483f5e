"""The reference's pusher known-answer tests (tests/teufel.undulator.cpp,
tests/teufel.magnet.cpp, tests/teufel.EcrossB.cpp; restated in
tests/pusher_cases.py) on the harness's Vay pusher, and on the reference's
own InitVay/StepVay (src/particle.cpp:407-512) where its build is present;
the two agree bit for bit on x86-64 and within a few ulp elsewhere."""
import platform

import numpy as np
import pytest

from oracle import lw
from pusher_cases import CASES
from teufel_gb300 import harness as H

EXACT = platform.machine() == "x86_64"


def harness_lattice(setup):
    u = setup["undulator"] or {}
    return H.Lattice(b_peak=u.get("b_peak", 0.0), lambda_u=u.get("lambda_u", 1.0),
                     n_periods=u.get("n_periods", 0), origin=u.get("origin", (0.0, 0.0, 0.0)),
                     hom_e=setup["E"], hom_b=setup["B"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_harness_pusher_passes_the_reference_test(name):
    setup, check = CASES[name]()
    tr = H.track(setup["init"], harness_lattice(setup), setup["tstep"], setup["n_steps"], -1.0,
                 1.0)
    assert check(tr.t, tr.x, tr.p) == []
    if lw.reference_available():
        t, x, p, a = lw.track_reference(setup["init"], harness_lattice(setup).packed(),
                                        setup["tstep"], setup["n_steps"], -1.0, 1.0)
        assert check(t, x, p) == []
        for got, ref in ((tr.t, t), (tr.x, x), (tr.p, p), (tr.a, a)):
            if EXACT:
                assert np.array_equal(got, ref)
            else:
                np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300)
