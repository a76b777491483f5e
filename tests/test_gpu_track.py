"""The device pusher (teufel_cuda_traj_track) against the reference's Vay
pusher (fixtures of InitVay/StepVay from tests/golden/make_golden.py), and the
reference's circular-loop test (tests/teufel.loop.cpp:70-187) run entirely on
the device: tracking, the field snapshot and the point observer."""
import os

import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import abi, harness as H

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
C = 2.99792458e8
E_CHARGE = 1.6021766208e-19
MEC2 = 0.5109989461e6
MU0 = 4 * np.pi * 1e-7


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_undulator_tracking_matches_the_reference_pusher():
    d = np.load(os.path.join(GOLD, "traj_undulator.npz"))
    lat = abi.lattice(b_peak=float(d["lattice"][1]), lambda_u=float(d["lattice"][2]),
                      n_periods=int(d["lattice"][3]))
    tstep, n = float(d["tstep"]), int(d["n_steps"])
    with abi.TrajSet.track(d["init1"], -1.0, 1.0, lat, tstep, n) as ts:
        t, x, p, a = ts.download()
    assert np.array_equal(t, d["t1"])  # time steps: the same IEEE additions
    # sin/cos/sinh/cosh may differ from the host libm by an ulp
    assert rel(x, d["x1"]) < 1e-12 and rel(p, d["p1"]) < 1e-12 and rel(a, d["a1"]) < 1e-11
    with abi.TrajSet.track(d["init4"], float(d["charge4"]), float(d["mass4"]), lat, tstep,
                           n) as ts:
        t4, x4, p4, a4 = ts.download()
    assert np.array_equal(t4, d["t4"])
    assert rel(x4, d["x4"]) < 1e-12 and rel(p4, d["p4"]) < 1e-12 and rel(a4, d["a4"]) < 1e-11


def test_homogeneous_field_tracking_is_bit_exact():
    d = np.load(os.path.join(GOLD, "traj_loop.npz"))
    lat = abi.lattice(B=tuple(d["lattice"][11:14]))
    with abi.TrajSet.track(d["init"], float(d["charge"]), float(d["mass"]), lat,
                           float(d["tstep"]), int(d["n_steps"])) as ts:
        t, x, p, a = ts.download()
    # no transcendental functions on this path: every operation is the reference's
    for got, ref in ((t, d["t"]), (x, d["x"]), (p, d["p"]), (a, d["a"])):
        assert np.array_equal(got, ref)


def test_loop_radiation_on_the_device():
    """tests/teufel.loop.cpp: a 1 nC electron macro-particle on a circle in
    0.5 T; the field at the circle's centre equals mu0 I / (2R)."""
    B, gamma = 0.5, 10.0
    bg = np.sqrt(gamma * gamma - 1.0)
    ang = B / (gamma * MEC2) * C * C
    radius = bg * 0.511e6 / (B * C)
    tau = 2 * np.pi / ang
    charge = 1.0e-9
    ne = charge / E_CHARGE
    rad_b = MU0 * charge / tau / (2.0 * radius)
    init = np.array([[0.0, 0.0, 0.0, 0.0, 0.0, 0.0, bg]])
    with abi.TrajSet.track(init, ne, ne, abi.lattice(B=(0.0, B, 0.0)), 0.5 * tau / 100,
                           200) as ts:
        t, x, p, a = ts.download()
        assert np.linalg.norm(x[100] - np.array([-2.0 * radius, 0.0, 0.0])) < 1e-3
        assert np.linalg.norm(x[200]) < 1e-4
        assert abs(np.linalg.norm(p[200]) - bg) < 1e-3
        snap = ts.retarded_field(tau, np.array([[-radius, 0.0, 0.0]]))
        assert abs(np.linalg.norm(snap[0, 3:]) - rad_b) / rad_b < 1e-3
        trace = ts.integrate_point(np.array([-radius, 0.0, 0.0]), tau - 1.0e-15, 2.0e-15, 2)
        assert abs(np.linalg.norm(trace[0, 3:]) - rad_b) / rad_b < 1e-3


def test_device_tracked_screen_matches_host_tracked():
    w = H.config1()
    tr = w.traj
    init = np.array([[tr.t[0], *tr.x[0], *tr.p[0]]])
    lat = abi.lattice(b_peak=w.info["lattice"].b_peak, lambda_u=w.info["lattice"].lambda_u,
                      n_periods=w.info["lattice"].n_periods)
    sel = np.arange(0, w.n_pix, 9)
    ref, rc = lw.integrate_screen(tr, w.pix_pos[sel], w.pix_t0[sel], w.dt, w.nots)
    assert rc == 0
    with abi.TrajSet.track(init, tr.charge[0], tr.mass[0], lat, w.info["tstep"],
                           w.info["n_steps"]) as ts:
        g = ts.integrate_screen(w.pix_pos[sel], w.pix_t0[sel], w.dt, w.nots)
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < 1e-5


def test_bad_tracking_arguments():
    init = np.zeros((1, 7))
    with pytest.raises(abi.TeufelError):
        abi.TrajSet.track(init, 1.0, 0.0, abi.lattice(), 1e-12, 10)   # zero mass
    with pytest.raises(abi.TeufelError):
        abi.TrajSet.track(init, 1.0, 1.0, abi.lattice(), -1e-12, 10)  # negative step


@pytest.mark.parametrize("name", ["undulator", "magnet", "ecrossb"])
def test_device_pusher_passes_the_reference_tests(name):
    """tests/teufel.undulator.cpp, teufel.magnet.cpp and teufel.EcrossB.cpp
    (restated in tests/pusher_cases.py) on the device pusher, which also
    matches the host pusher: bit for bit in homogeneous fields, within 1e-12
    in the undulator (the device's sin/cos/sinh/cosh)."""
    from pusher_cases import CASES
    setup, check = CASES[name]()
    u = setup["undulator"] or {}
    lat = abi.lattice(b_peak=u.get("b_peak", 0.0), lambda_u=u.get("lambda_u", 1.0),
                      n_periods=u.get("n_periods", 0), origin=u.get("origin", (0.0, 0.0, 0.0)),
                      E=setup["E"], B=setup["B"])
    with abi.TrajSet.track(setup["init"], -1.0, 1.0, lat, setup["tstep"], setup["n_steps"]) as ts:
        t, x, p, a = ts.download()
    assert check(t, x, p) == []
    hl = H.Lattice(b_peak=u.get("b_peak", 0.0), lambda_u=u.get("lambda_u", 1.0),
                   n_periods=u.get("n_periods", 0), origin=u.get("origin", (0.0, 0.0, 0.0)),
                   hom_e=setup["E"], hom_b=setup["B"])
    ref = H.track(setup["init"], hl, setup["tstep"], setup["n_steps"], -1.0, 1.0)
    assert np.array_equal(t, ref.t)
    if name == "undulator":
        assert rel(x, ref.x) < 1e-12 and rel(p, ref.p) < 1e-12 and rel(a, ref.a) < 1e-11
    else:
        for got, want in ((x, ref.x), (p, ref.p), (a, ref.a)):
            assert np.array_equal(got, want)
