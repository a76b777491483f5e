"""The CPU oracle against fixtures produced by the reference's own compiled
code (tests/golden/make_golden.py): trajectories of the Vay pusher, traces of
ChargedParticle::integrateFieldTrace, and the range-error cases of
FieldTrace::add.  Bit-exact on the machine the fixtures were made on
(x86-64, no FMA); elsewhere within a few ulp."""
import os
import platform

import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import harness as H

GOLD = os.path.join(os.path.dirname(__file__), "golden")
EXACT = platform.machine() == "x86_64"


def load(name):
    return np.load(os.path.join(GOLD, name))


def same(a, b, rtol=1e-12):
    if EXACT:
        assert np.array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=0)


def test_harness_pusher_matches_reference_pusher():
    d = load("traj_undulator.npz")
    lat = H.Lattice(b_peak=float(d["lattice"][1]), lambda_u=float(d["lattice"][2]),
                    n_periods=int(d["lattice"][3]))
    tr = H.track(d["init1"], lat, float(d["tstep"]), int(d["n_steps"]), -1.0, 1.0)
    same(tr.t, d["t1"])
    same(tr.x, d["x1"])
    same(tr.p, d["p1"])
    same(tr.a, d["a1"])
    tr4 = H.track(d["init4"], lat, float(d["tstep"]), int(d["n_steps"]), float(d["charge4"]),
                  float(d["mass4"]))
    same(tr4.t, d["t4"])
    same(tr4.x, d["x4"])
    same(tr4.p, d["p4"])
    same(tr4.a, d["a4"])


def test_harness_loop_matches_reference():
    d = load("traj_loop.npz")
    lat = H.Lattice(hom_b=(0.0, 0.5, 0.0))
    tr = H.track(d["init"], lat, float(d["tstep"]), int(d["n_steps"]), float(d["charge"]),
                 float(d["mass"]))
    same(tr.x, d["x"])
    same(tr.a, d["a"])


def _traj(d, key, n, charge, mass):
    t, x, p, a = d["t" + key], d["x" + key], d["p" + key], d["a" + key]
    npnt = len(t) // n
    return H.Trajectories(t, x, p, a, np.full(n, npnt, np.int32), np.full(n, charge),
                          np.full(n, mass))


def test_oracle_single_electron_traces():
    d = load("traj_undulator.npz")
    s = load("screen_single.npz")
    tr = _traj(d, "1", 1, -1.0, 1.0)
    out, rc = lw.integrate_screen(tr, s["pix_pos"], s["pix_t0"], float(s["dt"]), int(s["nots"]))
    assert rc == 0
    assert np.abs(s["traces"]).max() > 0
    same(out, s["traces"])


def test_oracle_bunch_traces():
    d = load("traj_undulator.npz")
    s = load("screen_bunch.npz")
    tr = _traj(d, "4", 4, float(d["charge4"]), float(d["mass4"]))
    out, rc = lw.integrate_screen(tr, s["pix_pos"], s["pix_t0"], float(s["dt"]), int(s["nots"]))
    assert rc == 0
    same(out, s["traces"])


def test_oracle_range_errors_like_reference():
    g = load("range_error.npz")
    nots = int(g["nots"])
    f = [[[1.0, 2.0, 3.0, 4.0, 5.0, 6.0], [2.0, 3.0, 4.0, 5.0, 6.0, 7.0]]]
    assert 4 in set(g["status"].tolist())
    for (t0, dt, a, b), st, ref in zip(g["cases"], g["status"], g["traces"]):
        tr, rc = lw.deposit_injected([[a, b]], f, t0, dt, nots)
        assert rc == st
        same(tr, ref)


def test_oracle_equals_reference_on_config1_subset():
    if not lw.reference_available():
        pytest.skip("the reference build oracle/_ref is not present on this machine")
    w = H.config1()
    sel = np.arange(3, w.n_pix, 11)
    a, rc1 = lw.integrate_screen(w.traj, w.pix_pos[sel], w.pix_t0[sel], w.dt, w.nots)
    b, rc2 = lw.integrate_screen(w.traj, w.pix_pos[sel], w.pix_t0[sel], w.dt, w.nots,
                                 impl="reference")
    assert rc1 == rc2 == 0
    assert np.array_equal(a, b)


def test_diffraction_screen_kat():
    """tests/teufel.DiffractionScreen.cpp:67-153 with the harness pusher and the
    oracle: a 100 pC macro-particle at gamma = 20 from z = -10 m to +10 m in
    20000 steps; the energy through the annular mesh is 0.463 +- 0.020 uJ,
    and trajectory, per-cell energies and traces equal the reference's."""
    d = load("diffraction_screen.npz")
    tr = H.track(d["init"], H.Lattice(), float(d["tstep"]), int(d["n_steps"]),
                 float(d["charge"]), float(d["mass"]))
    idx = d["check_idx"]
    same(tr.t[idx], d["check_t"])
    same(tr.x[idx], d["check_x"])
    same(tr.p[idx], d["check_p"])
    beta = np.sqrt(1.0 - 1.0 / 400.0)
    assert abs(tr.t[0] + 10.0 / (beta * 2.99792458e8)) < 1e-6
    assert abs(tr.x[-1, 2] - 10.0) < 1e-6
    dt, nt = float(d["dt"]), int(d["nt"])
    traces, rc = lw.integrate_screen(tr, d["pos"], d["t0"], dt, nt)
    assert rc == 0
    energy, flux = lw.mesh_energy(d["corner"], d["tri"].astype(np.int64), traces, dt)
    assert abs(energy * 1e6 - 0.463) <= 0.020
    same(traces[d["pix"]], d["traces"])
    np.testing.assert_allclose(flux, d["flux"], rtol=0, atol=1e-12 * np.abs(d["flux"]).max())
    np.testing.assert_allclose(energy, float(d["energy"]), rtol=1e-12)


def test_oracle_equals_reference_on_unusual_inputs():
    """The inputs the device routes to its FP64 kernel, pinned here: a
    negative dt (a reversed window: a range error where a step straddles it,
    nothing otherwise) and trajectories whose arrival times fall along the
    points (the electron's points reversed; its positions doubled, chords
    faster than light).  Same status as the reference's compiled
    integrateFieldTrace, and the same traces where it raises nothing."""
    if not lw.reference_available():
        pytest.skip("the reference build oracle/_ref is not present on this machine")
    w = H.config1()
    tr = w.traj
    sel = np.arange(0, w.n_pix, 20)
    pos = w.pix_pos[sel]
    C = 2.99792458e8
    mid = tr.t.shape[0] // 2

    def arrival(k):
        return tr.t[k] + np.linalg.norm(pos - tr.x[k], axis=1) / C

    reversed_ = H.Trajectories(tr.t[::-1].copy(), tr.x[::-1].copy(), tr.p[::-1].copy(),
                               tr.a[::-1].copy(), tr.n_points, tr.charge, tr.mass)
    doubled = H.Trajectories(tr.t.copy(), 2.0 * tr.x, tr.p.copy(), tr.a.copy(), tr.n_points,
                             tr.charge, tr.mass)
    cases = [(tr, 0.5 * (arrival(mid) + arrival(mid + 1)), -1e-17, 2),
             (tr, arrival(mid), -1e-17, 2),
             (tr, w.pix_t0[sel] + 2048 * 5e-15, -5e-15, 2048),
             (reversed_, w.pix_t0[sel], w.dt, w.nots),
             (doubled, w.pix_t0[sel], w.dt, w.nots)]
    statuses = []
    for t, t0, dt, nt in cases:
        a, rc1 = lw.integrate_screen(t, pos, t0, dt, nt)
        b, rc2 = lw.integrate_screen(t, pos, t0, dt, nt, impl="reference")
        assert rc1 == rc2
        statuses.append(rc1)
        if rc1 == 0:
            same(a, b)
    assert statuses == [4, 0, 0, 0, 0]
