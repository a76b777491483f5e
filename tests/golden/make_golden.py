"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs only where the reference tree is present (it builds oracle/_ref from the
reference's src/{vector,fields,fieldtrace,particle,global}.cpp):

    python tests/golden/make_golden.py

Fixtures (numpy .npz, compressed):
  traj_undulator.npz  initial conditions, lattice and the trajectories that
                      the reference's InitVay/StepVay (src/particle.cpp:407-512)
                      produce for the single-electron undulator run and for
                      four particles of the 1e4-particle bunch
  traj_loop.npz       the circular-loop run of tests/teufel.loop.cpp:70-110
  screen_single.npz   ChargedParticle::integrateFieldTrace traces of the
                      single electron on 16 pixels of the 21x21 screen
  screen_bunch.npz    the same for the four-particle bunch on 8 pixels
  range_error.npz     injected arrival times for which FieldTrace::add throws
                      (src/fieldtrace.cpp:185-190) inside the reference
  retarded_field.npz  ChargedParticle::RetardedField(double, Vector)
                      (src/particle.cpp:612-769) of the reference's
                      electrostatic test (tests/teufel.electrostatic.cpp:60-233:
                      a 1 pC charge at rest, and moving at gamma = 10 through a
                      field-free region) and of the single-electron undulator run
  diffraction_screen.npz  the mesh of tests/DiffractionScreen.h5 and the
                      reference's tracking and traces of its known-answer
                      test (tests/teufel.DiffractionScreen.cpp:67-153): energy,
                      per-cell energy and 8 pixels' traces
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import lw  # noqa: E402
from teufel_gb300 import harness as H  # noqa: E402

E_CHARGE = 1.6021766208e-19
C = 2.99792458e8


def undulator_runs():
    w = H.config1()
    lat = H.undulator(1.0, 0.1, 8)
    tstep, n_steps = w.info["tstep"], w.info["n_steps"]
    init1 = np.array([[0.0, 0.0, 0.0, float(w.traj.x[0, 2]), 0.0, 0.0, float(w.traj.p[0, 2])]])
    t1, x1, p1, a1 = lw.track_reference(init1, lat.packed(), tstep, n_steps, -1.0, 1.0)
    # four particles of the 1e4-particle, 100 pC bunch
    w2 = H.config2(count=4)
    ne = 100e-12 / E_CHARGE / 1e4
    init4 = H.gaussian_bunch(4, 20240602, 0.5e-3, 0.5e-3, 300e-6, 0.02, 0.02, 50.0, 0.05,
                             float(w.traj.x[0, 2]))
    t4, x4, p4, a4 = lw.track_reference(init4, lat.packed(), tstep, n_steps, -ne, ne)
    np.savez_compressed(os.path.join(HERE, "traj_undulator.npz"), lattice=lat.packed(),
                        tstep=tstep, n_steps=n_steps, init1=init1, t1=t1, x1=x1, p1=p1, a1=a1,
                        init4=init4, charge4=-ne, mass4=ne, t4=t4, x4=x4, p4=p4, a4=a4)
    return w, w2, (t1, x1, p1, a1), (t4, x4, p4, a4), ne


def loop_run():
    # tests/teufel.loop.cpp:70-110: B = 0.5 T along y, gamma = 10, 1 nC as one
    # macro-particle, 2 x 100 steps over a full turn
    B = 0.5
    gamma = 10.0
    bg = np.sqrt(gamma * gamma - 1.0)
    mec2 = 0.5109989461e6
    ang = B / (gamma * mec2) * C * C
    tau = 2 * np.pi / ang
    ne = 1.0e-9 / E_CHARGE
    lat = H.Lattice(hom_b=(0.0, B, 0.0))
    init = np.array([[0.0, 0.0, 0.0, 0.0, 0.0, 0.0, bg]])
    n_steps = 200
    t, x, p, a = lw.track_reference(init, lat.packed(), 0.5 * tau / 100, n_steps, ne, ne)
    np.savez_compressed(os.path.join(HERE, "traj_loop.npz"), lattice=lat.packed(),
                        tstep=0.5 * tau / 100, n_steps=n_steps, init=init, charge=ne, mass=ne,
                        t=t, x=x, p=p, a=a, tau=tau)


def screens(w, w2, tr1, tr4, ne):
    traj1 = H.Trajectories(tr1[0], tr1[1], tr1[2], tr1[3], np.array([len(tr1[0])], np.int32),
                           np.array([-1.0]), np.array([1.0]))
    sel = np.array([0, 10, 110, 200, 210, 220, 221, 230, 231, 240, 300, 320, 330, 400, 430, 440])
    pos, t0 = w.pix_pos[sel], w.pix_t0[sel]
    out, rc = lw.integrate_screen(traj1, pos, t0, w.dt, w.nots, impl="reference")
    assert rc == 0
    np.savez_compressed(os.path.join(HERE, "screen_single.npz"), pix=sel, pix_pos=pos,
                        pix_t0=t0, dt=w.dt, nots=w.nots, traces=out)
    n = len(tr4[0]) // 4
    traj4 = H.Trajectories(tr4[0], tr4[1], tr4[2], tr4[3], np.full(4, n, np.int32),
                           np.full(4, -ne), np.full(4, ne))
    sel2 = np.array([0, 100, 1000, 2015, 2080, 2500, 3000, 4095])
    pos2, t02 = w2.pix_pos[sel2], w2.pix_t0[sel2]
    out2, rc = lw.integrate_screen(traj4, pos2, t02, w2.dt, w2.nots, impl="reference")
    assert rc == 0
    np.savez_compressed(os.path.join(HERE, "screen_bunch.npz"), pix=sel2, pix_pos=pos2,
                        pix_t0=t02, dt=w2.dt, nots=w2.nots, traces=out2)


def cround(x):
    """C's round(): halfway cases away from zero (Python's round() is not)."""
    return int(np.sign(x) * np.floor(abs(x) + 0.5))


def range_errors():
    """Arrival times just above tmin for which (ts - t0)/dt rounds to -0.5,
    so round() gives -1 and FieldTrace::add(-1) throws; and times just below
    tmax whose index rounds to N."""
    # Such times exist only where the bin width is comparable to t0 itself,
    # so the search draws t0 and dt of similar size; it is bounded.
    rng = np.random.default_rng(7)
    found_lo, found_hi = [], []
    nots = 4
    for _ in range(200000):
        if len(found_lo) >= 3 and len(found_hi) >= 3:
            break
        t0 = float(rng.uniform(0.5, 2.0))
        dt = float(rng.uniform(0.3, 3.0))
        tmin = t0 - dt * 0.5
        tmax = t0 + dt * (nots - 0.5)
        ts = tmin
        for _k in range(3):
            ts = float(np.nextafter(ts, np.inf))
            if len(found_lo) < 3 and ts > tmin and cround((ts - t0) / dt) == -1:
                found_lo.append((t0, dt, ts))
                break
        te = tmax
        for _k in range(3):
            te = float(np.nextafter(te, -np.inf))
            if len(found_hi) < 3 and te < tmax and cround((te - t0) / dt) == nots:
                found_hi.append((t0, dt, te))
                break
    assert found_lo and found_hi, "no range-error inputs found"
    cases = []
    for t0, dt, ts in found_lo:
        # one step ending at ts, starting well before the window (case A)
        cases.append((t0, dt, ts - 3 * dt, ts))
    for t0, dt, ts in found_hi:
        # a step starting at ts, inside the window by a hair (case B)
        cases.append((t0, dt, ts, ts + 0.25 * dt))
    cases = np.array(cases)
    status, traces = [], []
    for t0, dt, a, b in cases:
        f = [[[1.0, 2.0, 3.0, 4.0, 5.0, 6.0], [2.0, 3.0, 4.0, 5.0, 6.0, 7.0]]]
        tr, rc = lw.deposit_injected([[a, b]], f, t0, dt, nots, impl="reference")
        status.append(rc)
        traces.append(tr)
    np.savez_compressed(os.path.join(HERE, "range_error.npz"), cases=cases, nots=nots,
                        status=np.array(status), traces=np.array(traces))


def electrostatic_cases():
    """The scenario of tests/teufel.electrostatic.cpp:60-233: trajectories
    and observation (time, points) sets."""
    q = -1.0e-12 / E_CHARGE
    rest = H.Trajectories(np.zeros(1), np.zeros((1, 3)), np.zeros((1, 3)), np.zeros((1, 3)),
                          np.array([1], np.int32), np.array([q]), np.array([1.0]))
    gamma = 10.0
    bg = np.sqrt(gamma * gamma - 1.0)
    d = np.array([2.0, 3.0, 5.0])
    d = d / np.sqrt(np.sum(d * d))
    perp = np.cross(d, [1.0, 0.0, 0.0])
    perp = perp / np.sqrt(np.sum(perp * perp))
    n_steps, tau = 2000, 4.0e-9
    init = np.array([[0.0, 0.0, 0.0, 0.0, bg * d[0], bg * d[1], bg * d[2]]])
    lat = H.Lattice(hom_b=(0.0, 0.0, 0.0))
    t, x, p, a = lw.track_reference(init, lat.packed(), tau / n_steps, n_steps, q, 1.0)
    moving = H.Trajectories(t, x, p, a, np.array([n_steps + 1], np.int32), np.array([q]),
                            np.array([1.0]))
    beta = np.sqrt(1.0 - 1.0 / (gamma * gamma))
    ls = -0.005 + 0.001 * np.arange(11)
    p0 = perp * 0.001
    p1 = d * 3.0e-9 * beta * C + perp * 0.001
    sets = [
        ("rest", rest, 0.0, np.array([[0.001, 0.0, 0.0], [-0.001, 0.0, 0.0], [0.0, 0.0, 0.001]])),
        ("moving_t0", moving, 0.0, np.vstack([p0] + [p0 + d * l for l in ls])),
        ("moving_t3ns", moving, 3.0e-9, np.vstack([p1] + [p1 + d * l for l in ls])),
    ]
    return sets, dict(d=d, perp=perp, gamma=gamma, beta=beta)


def retarded_fields(tr1):
    sets, geo = electrostatic_cases()
    w = H.config1()
    traj1 = H.Trajectories(tr1[0], tr1[1], tr1[2], tr1[3], np.array([len(tr1[0])], np.int32),
                           np.array([-1.0]), np.array([1.0]))
    pos = w.pix_pos[::29]
    for k, tobs in enumerate((0.0, 2.0e-8, 3.34e-8, 3.4e-8, 3.5e-8, 1.0e-6)):
        sets.append((f"undulator_{k}", traj1, tobs, pos))
    rec, trajs = {}, {}
    for name, tr, tobs, p in sets:
        out, rc = lw.retarded_field_at(tr, tobs, p, impl="reference")
        assert rc == 0
        key = name.split("_")[0]
        trajs[key] = tr
        rec[name] = dict(traj=key, obs_time=tobs, pos=p, fields=out)
    flat = {f"{n}__{k}": v for n, d in rec.items() for k, v in d.items()}
    for key, tr in trajs.items():
        for f in ("t", "x", "p", "a", "n_points", "charge", "mass"):
            flat[f"traj_{key}__{f}"] = getattr(tr, f)
    np.savez_compressed(os.path.join(HERE, "retarded_field.npz"), names=np.array(list(rec)),
                        **flat, **{f"geo__{k}": v for k, v in geo.items()})


def diffraction_screen():
    """tests/teufel.DiffractionScreen.cpp:67-153: a 100 pC macro-particle at
    gamma = 20 tracked from z = -10 m through an empty lattice for 20000 Vay
    steps, recorded on the annular mesh of tests/DiffractionScreen.h5 (read
    here with the numpy HDF5 reader tests/h5min.py)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from h5min import H5Min
    f = H5Min(str(lw.reference_file("tests/DiffractionScreen.h5")))
    corner, ca, _ = f.dataset("MeshCornerPoints")
    tri, ta, _ = f.dataset("MeshTriangles")
    pos, pa, _ = f.dataset("ObservationPosition")
    t0, oa, _ = f.dataset("ObservationTime")
    nt, dt = int(oa["Nt"]), float(oa["dt"])
    gamma, charge, nots = 20.0, 100e-12, 20000
    beta = np.sqrt(1.0 - 1.0 / (gamma * gamma))
    init = np.array([[-10.0 / (beta * C), 0.0, 0.0, -10.0, 0.0, 0.0, np.sqrt(gamma * gamma - 1.0)]])
    tstep = 20.0 / (beta * C) / nots
    q = charge / E_CHARGE
    t, x, p, a = lw.track_reference(init, np.zeros(16), tstep, nots, -q, q)
    traj = H.Trajectories(t, x, p, a, np.array([nots + 1], np.int32), np.array([-q]),
                          np.array([q]))
    traces, rc = lw.integrate_screen(traj, pos, t0, dt, nt, impl="reference")
    assert rc == 0, rc
    energy, flux = lw.mesh_energy(corner, tri.astype(np.int64), traces, dt)
    print(f"DiffractionScreen: reference energy {energy * 1e6:.6f} uJ")
    sel = np.argsort(flux)[::-1][:4].tolist() + [0, 300, 900, 1461]
    check = np.arange(0, nots + 1, 1000)
    np.savez_compressed(os.path.join(HERE, "diffraction_screen.npz"), corner=corner,
                        tri=tri.astype(np.int32), pos=pos, t0=t0, nt=nt, dt=dt,
                        attrs=np.array([int(ca["Ncp"]), int(ta["Ntri"]), int(pa["Np"])]),
                        init=init, tstep=tstep, n_steps=nots, charge=-q, mass=q,
                        check_idx=check, check_t=t[check], check_x=x[check], check_p=p[check],
                        energy=energy, flux=flux, pix=np.array(sel), traces=traces[sel])


def main():
    lw.build(with_reference=True)
    if not lw.reference_available():
        raise SystemExit("the reference tree is needed to generate the fixtures")
    w, w2, tr1, tr4, ne = undulator_runs()
    retarded_fields(tr1)
    loop_run()
    screens(w, w2, tr1, tr4, ne)
    range_errors()
    diffraction_screen()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
