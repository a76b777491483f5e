"""The RetardedField(t, X) fixture (tests/golden/retarded_field.npz, made by
tests/golden/make_golden.py from the reference's compiled particle.cpp) and
the checks of the reference's electrostatic test
(tests/teufel.electrostatic.cpp:60-233), shared by the oracle and device
tests."""
import os

import numpy as np

from teufel_gb300 import harness as H

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "retarded_field.npz")
E_CHARGE = 1.6021766208e-19
C = 2.99792458e8
EPS0 = 8.854187817e-12
MU0 = 4.0e-7 * np.pi  # src/global.h


def load():
    """{name: (Trajectories, obs_time, pos[n,3], reference fields[n,6])}, geometry."""
    d = np.load(GOLD)
    trajs = {}
    out = {}
    for name in d["names"]:
        name = str(name)
        key = str(d[f"{name}__traj"])
        if key not in trajs:
            g = lambda f: d[f"traj_{key}__{f}"]  # noqa: E731
            trajs[key] = H.Trajectories(g("t"), g("x"), g("p"), g("a"), g("n_points"),
                                        g("charge"), g("mass"))
        out[name] = (trajs[key], float(d[f"{name}__obs_time"]), d[f"{name}__pos"],
                     d[f"{name}__fields"])
    geo = {k[5:]: d[k] for k in d.files if k.startswith("geo__")}
    return out, geo


def check_electrostatic(field_fn):
    """The assertions of tests/teufel.electrostatic.cpp on field_fn(traj,
    obs_time, pos) -> [n,6]."""
    cases, geo = load()
    eref = 1e-12 / (4.0 * np.pi * EPS0 * 1.0e-3 * 1.0e-3)
    tr, tobs, pos, _ = cases["rest"]
    f = field_fn(tr, tobs, pos)
    assert np.linalg.norm(np.array([-1.0, 0, 0]) * eref - f[0, :3]) < 1e-3
    assert np.linalg.norm(np.array([1.0, 0, 0]) * eref - f[1, :3]) < 1e-3
    assert np.linalg.norm(np.array([0, 0, -1.0]) * eref - f[2, :3]) / eref < 1e-6
    d, perp, gamma, beta = geo["d"], geo["perp"], float(geo["gamma"]), float(geo["beta"])
    erefv = perp * eref * -1.0 * gamma
    brefv = np.cross(d * beta * C, perp) * -1.0e-12 * MU0 / (4 * np.pi) / (0.001 * 0.001) * gamma
    lists = []
    for name, tol in (("moving_t0", 1e-5), ("moving_t3ns", 1e-3)):
        tr, tobs, pos, _ = cases[name]
        f = field_fn(tr, tobs, pos)
        assert np.linalg.norm(erefv - f[0, :3]) / np.linalg.norm(erefv) < tol
        assert np.linalg.norm(brefv - f[0, 3:]) / np.linalg.norm(brefv) < tol
        lists.append(f[1:, :3] @ perp)
    assert np.all((lists[1] - lists[0]) / lists[0] <= 1e-5)
