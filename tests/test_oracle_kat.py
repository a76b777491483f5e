"""The reference's known-answer test of the deposit algorithm,
tests/teufel.integrate_field.cpp:98-189 (four scenarios, 28 bin values to
1e-6), run through the CPU oracle and, where it was built, through the
reference's own compiled integrateFieldTrace (oracle/_ref)."""
import numpy as np
import pytest

from oracle import lw

# (particles as (t1, t2, Ex1, Ex2), trace t0, dt, N, expected Ex per bin)
KAT = [
    ([(0.0, 1.0, 1.5, 0.5)], 0.0, 0.2, 8, [0.725, 1.3, 1.1, 0.9, 0.7, 0.275, 0.0, 0.0]),
    ([(0.0, 1.0, 1.5, 0.5)], -0.1, 0.2, 8, [0.0, 1.4, 1.2, 1.0, 0.8, 0.6, 0.0, 0.0]),
    ([(0.05, 0.15, 1.5, 0.5)], -0.2, 0.2, 4, [0.0, 0.3125, 0.1875, 0.0]),
    ([(0.05, 0.15, 1.5, 0.5)], -0.1, 0.2, 4, [0.0, 0.5, 0.0, 0.0]),
    ([(1.0, 2.0, 1.0, 0.0), (1.0, 2.0, 0.0, 1.0), (2.0, 2.2, 1.0, 1.0), (2.2, 2.4, 1.0, 0.0),
      (2.4, 3.0, 0.0, 1.0)], 0.0, 0.5, 8,
     [0.0, 0.0, 0.5, 1.0, 0.9875, 0.316667, 0.395833, 0.0]),
]


def kat_inputs(parts):
    ts = [[p[0], p[1]] for p in parts]
    fs = [[[p[2], 0, 0, 0, 0, 0], [p[3], 0, 0, 0, 0, 0]] for p in parts]
    return ts, fs


@pytest.mark.parametrize("case", range(len(KAT)))
def test_oracle_kat(case):
    parts, t0, dt, n, expect = KAT[case]
    ts, fs = kat_inputs(parts)
    tr, rc = lw.deposit_injected(ts, fs, t0, dt, n)
    assert rc == 0
    np.testing.assert_allclose(tr[:, 0], expect, atol=1e-6, rtol=0)
    assert np.all(tr[:, 1:] == 0.0)


@pytest.mark.parametrize("case", range(len(KAT)))
def test_oracle_equals_reference_kat(case):
    if not lw.reference_available():
        pytest.skip("the reference build oracle/_ref is not present on this machine")
    parts, t0, dt, n, _ = KAT[case]
    ts, fs = kat_inputs(parts)
    a, rc1 = lw.deposit_injected(ts, fs, t0, dt, n)
    b, rc2 = lw.deposit_injected(ts, fs, t0, dt, n, impl="reference")
    assert rc1 == rc2 == 0
    assert np.array_equal(a, b)
