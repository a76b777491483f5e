"""HDF5 input and output of the meshed and rectangular screens, without the
HDF5 library: the C++ reader (include/teufel_hdf5_read.hpp) behind
MeshedScreen(filename) (src/mesh.cpp:31-218) and init() (src/mesh.cpp:227-278),
the C++ writer (include/teufel_hdf5_write.hpp) behind MeshedScreen::writeFile
(src/mesh.cpp:428-736) and ScreenObserver::WriteTimeDomainFieldHDF5
(src/screen.cpp:298-560), each checked against the independent numpy reader
tests/h5min.py and the DiffractionScreen mesh fixture."""
import os
import struct
import subprocess

import numpy as np
import pytest

from h5min import H5Min
from oracle import lw
from teufel_gb300 import _build

HERE = os.path.dirname(os.path.abspath(__file__))
MESH = os.path.join(HERE, "golden", "diffraction_screen.npz")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = _build.build_cuda()
    exe = tmp_path_factory.mktemp("mesh") / "mesh_driver"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{_build.INCLUDE}",
                    os.path.join(HERE, "cpp", "mesh_driver.cpp"), "-o", str(exe), str(lib),
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    return str(exe)


@pytest.fixture(scope="module")
def mesh():
    return dict(np.load(MESH))


def write_mesh_bin(path, g, nt, dt, field):
    with open(path, "wb") as fh:
        np.array([g["corner"].shape[0], g["pos"].shape[0], nt], np.int32).tofile(fh)
        np.array([dt]).tofile(fh)
        np.ascontiguousarray(g["corner"], np.float64).tofile(fh)
        np.ascontiguousarray(g["tri"], np.int32).tofile(fh)
        np.ascontiguousarray(g["pos"], np.float64).tofile(fh)
        np.ascontiguousarray(g["t0"], np.float64).tofile(fh)
        np.ascontiguousarray(field, np.float64).tofile(fh)


def read_driver_dump(path):
    b = open(path, "rb").read()
    np_, nt = struct.unpack_from("<ii", b, 0)
    dt, area = struct.unpack_from("<dd", b, 8)
    rec = np.frombuffer(b, np.float64, offset=24).reshape(np_, 14)
    return dict(np=np_, nt=nt, dt=dt, total_area=area, t0=rec[:, 0], pos=rec[:, 1:4],
                area=rec[:, 4], normal=rec[:, 5:8], xi=rec[:, 8:11], eta=rec[:, 11:14])


def numpy_init(g):
    """Areas, normals and (xi, eta) frames as src/mesh.cpp:227-278 sets them up."""
    area, normal = lw.mesh_cells(g["corner"], g["tri"].astype(np.int64))
    avg = normal.sum(axis=0)
    avg /= np.linalg.norm(avg)
    unit = lambda v: v / np.linalg.norm(v, axis=1)[:, None]  # noqa: E731
    if avg[1] < 0.7:
        xi = unit(np.cross(np.array([0.0, 1.0, 0.0]), normal))
        eta = unit(np.cross(normal, xi))
    else:
        eta = unit(np.cross(normal, np.array([1.0, 0.0, 0.0])))
        xi = unit(np.cross(eta, normal))
    return area, normal, xi, eta


def test_fixture_matches_reference_mesh_file(mesh):
    path = lw.reference_file("tests/DiffractionScreen.h5")
    if path is None:
        pytest.skip("the reference tree is absent")
    f = H5Min(str(path))
    assert sorted(f.links) == ["MeshCornerPoints", "MeshTriangles", "ObservationPosition",
                               "ObservationTime"]
    for name, key in [("MeshCornerPoints", "corner"), ("MeshTriangles", "tri"),
                      ("ObservationPosition", "pos"), ("ObservationTime", "t0")]:
        a, _, _ = f.dataset(name)
        assert np.array_equal(a, mesh[key]), name
    _, attrs, _ = f.dataset("ObservationTime")
    assert int(attrs["Nt"]) == int(mesh["nt"]) and float(attrs["dt"]) == float(mesh["dt"])


def test_cpp_reader_on_reference_file(driver, mesh, tmp_path):
    path = lw.reference_file("tests/DiffractionScreen.h5")
    if path is None:
        pytest.skip("the reference tree is absent")
    out = tmp_path / "dump.bin"
    r = subprocess.run([driver, "read", str(path), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = read_driver_dump(out)
    assert (d["np"], d["nt"], d["dt"]) == (1462, int(mesh["nt"]), float(mesh["dt"]))
    assert np.array_equal(d["t0"], mesh["t0"]) and np.array_equal(d["pos"], mesh["pos"])
    area, normal, xi, eta = numpy_init(mesh)
    np.testing.assert_allclose(d["area"], area, rtol=1e-13)
    np.testing.assert_allclose(d["total_area"], area.sum(), rtol=1e-13)
    for k, v in [("normal", normal), ("xi", xi), ("eta", eta)]:
        np.testing.assert_allclose(d[k], v, rtol=0, atol=1e-14)


@pytest.mark.parametrize("nt", [7, 0])
def test_mesh_writer_layout_and_roundtrip(driver, mesh, tmp_path, nt):
    rng = np.random.default_rng(11 + nt)
    np_ = mesh["pos"].shape[0]
    field = rng.standard_normal((np_, nt, 6)) * np.array([1e3, 1e3, 1e3, 1e-5, 1e-5, 1e-5])
    inp, out = tmp_path / "mesh.bin", tmp_path / "mesh.h5"
    dt = float(mesh["dt"])
    write_mesh_bin(inp, mesh, nt, dt, field)
    r = subprocess.run([driver, "write", str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    e1, e2 = (float(v) for v in r.stdout.split()[1:3])
    assert e1 == e2 and "buffer same" in r.stdout
    if nt:
        ref, _ = lw.mesh_energy(mesh["corner"], mesh["tri"].astype(np.int64), field, dt)
        np.testing.assert_allclose(e1, ref, rtol=1e-12)

    f = H5Min(str(out))
    # file structure: superblock 0, symbol-table root group of the library's defaults
    assert (f.leaf_k, f.internal_k, f.root_cache_type) == (4, 16, 1)
    assert f.eof == os.path.getsize(out)
    assert f.heap["free"] == 1 and f.btree["level"] == 0 and f.btree["used"] == 1
    assert f.btree_last_key == "ObservationTime"
    assert sorted(f.links) == ["ElMagField", "MeshCornerPoints", "MeshTriangles",
                               "ObservationPosition", "ObservationTime"]
    expect = {"MeshCornerPoints": (mesh["corner"], {"Ncp": mesh["corner"].shape[0]}),
              "ObservationPosition": (mesh["pos"], {"Np": np_}),
              "MeshTriangles": (mesh["tri"], {"Ntri": np_}),
              "ObservationTime": (mesh["t0"], {"Nt": nt, "dt": dt}),
              "ElMagField": (field, {})}
    for name, (data, attrs) in expect.items():
        a, at, info = f.dataset(name)
        assert a.dtype == (np.int32 if name == "MeshTriangles" else np.float64), name
        assert a.shape == data.shape and np.array_equal(a, data), name
        assert set(at) == set(attrs), name
        for k, v in attrs.items():
            assert at[k] == v, (name, k)
            assert at[k].dtype == (np.float64 if k == "dt" else np.int32), (name, k)
        if a.size:
            assert info["addr"] % 8 == 0 and info["size"] == a.nbytes
        else:
            assert info["addr"] == 2**64 - 1 and info["size"] == 0


def test_screen_writer(driver, tmp_path):
    out = tmp_path / "screen.h5"
    r = subprocess.run([driver, "screen", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    f = H5Min(str(out))
    assert sorted(f.links) == ["ElMagField", "ObservationPosition", "Screen"]
    origin, dx, dy = np.array([0.001, -0.002, 2.5]), np.array([0.01, 0, 0]), np.array([0, 0.02, 0])
    nx, ny, nots = 3, 2, 4
    pos, at, _ = f.dataset("ObservationPosition")
    ix, iy = np.meshgrid(np.arange(nx) - nx // 2, np.arange(ny) - ny // 2, indexing="ij")
    want = origin + dx * ix[..., None] + dy * iy[..., None]
    np.testing.assert_array_equal(pos, want)
    assert {k: int(v) for k, v in at.items()} == {"Nx": nx, "Ny": ny}
    scr, at, _ = f.dataset("Screen")
    normal = -np.cross(dx, dy)
    normal /= np.linalg.norm(normal)
    np.testing.assert_array_equal(scr, np.array([origin, normal, dx, dy]))
    assert {k: float(v) for k, v in at.items()} == {"Nx": 3, "Ny": 2, "NOTS": 4, "t0": 8.3e-9,
                                                   "dt": 1e-13, "dtx": 2e-14, "dty": -3e-14}
    fld, at, _ = f.dataset("ElMagField")
    np.testing.assert_array_equal(fld, (0.25 * np.arange(nx * ny * nots * 6) - 7.0)
                                  .reshape(nx, ny, nots, 6))
    assert {k: float(v) for k, v in at.items()} == {"t0": 8.3e-9, "dt": 1e-13, "NOTS": 4}


def test_reader_rejects_bad_files(driver, mesh, tmp_path):
    inp, good = tmp_path / "mesh.bin", tmp_path / "mesh.h5"
    write_mesh_bin(inp, mesh, 2, 1e-13, np.zeros((mesh["pos"].shape[0], 2, 6)))
    assert subprocess.run([driver, "write", str(inp), str(good)], capture_output=True).returncode == 0
    data = good.read_bytes()
    cases = {"truncated": data[:len(data) // 2], "not_hdf5": b"\0" * 256,
             "superblock_v2": data[:8] + b"\x02" + data[9:]}
    for name, blob in cases.items():
        bad = tmp_path / f"{name}.h5"
        bad.write_bytes(blob)
        r = subprocess.run([driver, "read", str(bad), str(tmp_path / "x.bin")], capture_output=True,
                           text=True)
        assert r.returncode == 3 and "MeshedScreen - HDF5 reader" in r.stderr, (name, r.stderr)


def test_snapshot_writer_with_particle_coordinates(driver, tmp_path):
    """SnapshotObserver::WriteFieldHDF5 (src/snapshot.cpp:226-396) after
    storeParticlePositions (src/snapshot.cpp:114-149): ParticleCoordinates
    from CoordinatesAtTime (src/particle.cpp:514-558), pinned to the
    reference's own function where its build is present."""
    from teufel_gb300 import harness as H
    rng = np.random.default_rng(5)
    lens = [40, 1, 25]
    t_snap = 2.2e-10
    parts = tmp_path / "parts.bin"
    ts, xs, ps = [], [], []
    with open(parts, "wb") as fh:
        np.array([len(lens)], np.int32).tofile(fh)
        for m, n in enumerate(lens):
            t = np.cumsum(rng.uniform(5e-12, 2e-11, n)) + 1e-10 * m
            x, p, a = (rng.standard_normal((n, 3)) for _ in range(3))
            np.array([n], np.int32).tofile(fh)
            np.array([-1.6e-19]).tofile(fh)
            for v in (t, x, p, a):
                v.tofile(fh)
            ts.append(t), xs.append(x), ps.append(p)
    out = tmp_path / "snap.h5"
    r = subprocess.run([driver, "snapshot", str(parts), repr(t_snap), str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    f = H5Min(str(out))
    assert sorted(f.links) == ["ElMagField", "ObservationPosition", "ParticleCoordinates"]
    pos, at, _ = f.dataset("ObservationPosition")
    ix, iy = np.meshgrid(np.arange(4) - 1.5, np.arange(3) - 1.0, indexing="ij")
    want = (np.array([0.0, 0.1, 3.0]) + np.array([0.002, 0, 0]) * ix[..., None] +
            np.array([0, 0.003, 0]) * iy[..., None])
    np.testing.assert_array_equal(pos, want)
    assert {k: int(v) for k, v in at.items()} == {"Nx": 4, "Ny": 3}
    fld, at, _ = f.dataset("ElMagField")
    np.testing.assert_array_equal(fld, (1.5 * np.arange(72) + 0.25).reshape(4, 3, 6))
    assert float(at["t0"]) == t_snap
    pc, at, _ = f.dataset("ParticleCoordinates")
    assert int(at["N_particles"]) == 3 and pc.shape == (3, 6)
    for m in range(3):  # restated: linear interpolation inside, zero outside
        t, x, p = ts[m], xs[m], ps[m]
        if t[0] <= t_snap <= t[-1]:
            i2 = max(int(np.searchsorted(t, t_snap)), 1)
            fr = (t_snap - t[i2 - 1]) / (t[i2] - t[i2 - 1])
            expect = np.concatenate([x[i2 - 1] * (1 - fr) + x[i2] * fr,
                                     p[i2 - 1] * (1 - fr) + p[i2] * fr])
        else:
            expect = np.zeros(6)
        np.testing.assert_allclose(pc[m], expect, rtol=1e-15, atol=0)
    if lw.reference_available():
        traj = H.Trajectories(np.concatenate(ts), np.concatenate(xs), np.concatenate(ps),
                              np.zeros((sum(lens), 3)), np.array(lens, np.int32),
                              np.full(3, -1.0), np.ones(3))
        assert np.array_equal(pc, lw.coordinates_at_time(traj, t_snap))
