"""The C++ observer layer (include/teufel_observers.hpp) driven on the GPU:
ScreenObserver, MeshedScreen and PointObserver integrate() through the C-ABI,
compared with the CPU oracle on the single-electron screen."""
import os
import subprocess

import numpy as np
import pytest

from oracle import lw
from teufel_gb300 import _build, harness as H

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def build_driver(tmpdir):
    lib = _build.build_cuda()
    exe = os.path.join(tmpdir, "observer_driver")
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{_build.INCLUDE}",
                    os.path.join(HERE, "cpp", "observer_driver.cpp"), "-o", exe,
                    str(lib), f"-Wl,-rpath,{lib.parent}"], check=True)
    return exe


def test_cpp_observers_match_oracle(tmp_path):
    w = H.config1()
    s = w.info["screen"]
    tr = w.traj
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([tr.n_particles], np.int32).tofile(f)
        tr.n_points.astype(np.int32).tofile(f)
        (tr.charge * 1.6021766208e-19).tofile(f)
        for v in (tr.t, tr.x, tr.p, tr.a):
            np.ascontiguousarray(v).tofile(f)
        np.array(s.origin + s.dx + s.dy).tofile(f)
        np.array([s.nx, s.ny], np.int32).tofile(f)
        np.array([s.t0, s.dt, s.dtx, s.dty]).tofile(f)
        np.array([s.nots], np.int32).tofile(f)
    exe = build_driver(str(tmp_path))
    outp = tmp_path / "out.bin"
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    data = np.fromfile(outp)
    n = w.n_pix * w.nots * 6
    screen = data[:n].reshape(w.n_pix, w.nots, 6)
    mesh = data[n:2 * n].reshape(w.n_pix, w.nots, 6)
    point = data[2 * n:2 * n + w.nots * 6].reshape(w.nots, 6)
    m = 2 * n + w.nots * 6
    snap = data[m:m + s.nx * s.ny * 6].reshape(s.nx * s.ny, 6)
    m += s.nx * s.ny * 6
    mesh_twice = data[m:m + n].reshape(w.n_pix, w.nots, 6)
    mesh_again = data[m + n:].reshape(w.n_pix, w.nots, 6)
    # the first integrate() after construction or zero() stores the traces
    # (overwrite_out), a later one adds them: twice the traces, then the same
    # traces again, bit for bit
    assert mesh_again.shape == mesh.shape
    assert np.array_equal(mesh_twice, 2.0 * mesh)
    assert np.array_equal(mesh_again, mesh)
    ref, rc = lw.integrate_screen(tr, w.pix_pos, w.pix_t0, w.dt, w.nots)
    assert rc == 0
    nrm = np.linalg.norm(ref)
    assert np.linalg.norm(screen - ref) / nrm < 1e-5
    assert np.array_equal(screen, mesh)
    c = (s.nx // 2) * s.ny + s.ny // 2
    assert np.linalg.norm(point - ref[c]) / np.linalg.norm(ref[c]) < 1e-5
    # SnapshotObserver: cell (ix, iy) at O + dX (ix - (Nx-1)/2) + dY (iy - (Ny-1)/2)
    ix, iy = np.meshgrid(np.arange(s.nx), np.arange(s.ny), indexing="ij")
    cells = (np.asarray(s.origin)[None, :] + np.asarray(s.dx)[None, :] * (ix.reshape(-1, 1) - 0.5 * (s.nx - 1))
             + np.asarray(s.dy)[None, :] * (iy.reshape(-1, 1) - 0.5 * (s.ny - 1)))
    sref, rc = lw.retarded_field_at(tr, s.t0 + 0.5 * s.nots * s.dt, cells)
    assert rc == 0 and np.abs(sref).max() > 0
    np.testing.assert_allclose(snap, sref, rtol=1e-12, atol=1e-12 * np.abs(sref).max())
