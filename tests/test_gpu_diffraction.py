"""The reference's DiffractionScreen known-answer test
(tests/teufel.DiffractionScreen.cpp:67-153) on the device: a 100 pC
macro-particle at gamma = 20 tracked from z = -10 m through an empty lattice
for 20000 steps and recorded on the annular mesh of 1462 triangles x 500
samples; the energy through the screen is 0.463 +- 0.020 uJ.

Two routes: the C++ observer layer exactly as the reference's test body runs
(the mesh written to HDF5 and read back by MeshedScreen(filename), init,
integrate, totalEnergy, writeFile), and the Python C-ABI binding with the
device pusher.  Both are also held to the reference's own traces and energy
(tests/golden/diffraction_screen.npz) within the FP32 path's 1e-5 bound."""
import os
import subprocess

import numpy as np
import pytest

from h5min import H5Min
from oracle import lw
from teufel_gb300 import _build, abi, harness as H

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
E_CHARGE = 1.6021766208e-19
RTOL = 1e-5


@pytest.fixture(scope="module")
def fixture():
    return dict(np.load(os.path.join(HERE, "golden", "diffraction_screen.npz")))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = _build.build_cuda()
    exe = tmp_path_factory.mktemp("mesh") / "mesh_driver"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{_build.INCLUDE}",
                    os.path.join(HERE, "cpp", "mesh_driver.cpp"), "-o", str(exe), str(lib),
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    return str(exe)


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def check_against_reference(fx, traces, energy):
    dt = float(fx["dt"])
    assert abs(energy * 1e6 - 0.463) <= 0.020, energy
    assert abs(energy - float(fx["energy"])) <= RTOL * float(fx["energy"])
    _, flux = lw.mesh_energy(fx["corner"], fx["tri"].astype(np.int64), traces, dt)
    assert rel_l2(flux, fx["flux"]) <= RTOL
    assert rel_l2(traces[fx["pix"]], fx["traces"]) <= RTOL


def test_diffraction_screen_through_the_observer_layer(driver, fixture, tmp_path):
    fx = fixture
    tr = H.track(fx["init"], H.Lattice(), float(fx["tstep"]), int(fx["n_steps"]),
                 float(fx["charge"]), float(fx["mass"]))
    mesh_bin, traj_bin = tmp_path / "mesh.bin", tmp_path / "traj.bin"
    with open(mesh_bin, "wb") as fh:
        np.array([fx["corner"].shape[0], fx["pos"].shape[0], int(fx["nt"])], np.int32).tofile(fh)
        np.array([float(fx["dt"])]).tofile(fh)
        for k, t in (("corner", np.float64), ("tri", np.int32), ("pos", np.float64),
                     ("t0", np.float64)):
            np.ascontiguousarray(fx[k], t).tofile(fh)
        np.zeros((fx["pos"].shape[0], int(fx["nt"]), 6)).tofile(fh)
    with open(traj_bin, "wb") as fh:
        np.array([tr.t.shape[0]], np.int32).tofile(fh)
        np.array([float(fx["charge"]) * E_CHARGE]).tofile(fh)
        for a in (tr.t, tr.x, tr.p, tr.a):
            np.ascontiguousarray(a).tofile(fh)
    h5_in, h5_out = tmp_path / "DiffractionScreen.h5", tmp_path / "DiffractionScreenWithFields.h5"
    r = subprocess.run([driver, "kat", str(mesh_bin), str(traj_bin), str(h5_in), str(h5_out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    energy_uJ = float(r.stdout.split()[1])
    f = H5Min(str(h5_out))
    traces, _, _ = f.dataset("ElMagField")
    assert traces.shape == (1462, 500, 6)
    check_against_reference(fx, traces, energy_uJ * 1e-6)
    np.testing.assert_allclose(
        energy_uJ * 1e-6,
        lw.mesh_energy(fx["corner"], fx["tri"].astype(np.int64), traces, float(fx["dt"]))[0],
        rtol=1e-12)


@pytest.mark.parametrize("precision,variant", [(abi.PREC_FP32_SPLIT, 4), (abi.PREC_FP32_SPLIT, 8),
                                               (abi.PREC_FP32_SPLIT, 1), (abi.PREC_FP32_SPLIT, 2),
                                               (abi.PREC_FP64, 0)])
def test_diffraction_screen_with_the_device_pusher(fixture, precision, variant):
    """Variants: 4 the pair kernel (default), 8 the pair kernel with packed
    multi-bin deposits, 1 the warp-uniform kernel, 2 the lane-divergent
    kernel; all use the exact arrival increment of steps that
    pass close to the observation point."""
    fx = fixture
    with abi.TrajSet.track(fx["init"], float(fx["charge"]), float(fx["mass"]), abi.lattice(),
                           float(fx["tstep"]), int(fx["n_steps"])) as ts:
        t, x, p, _ = ts.download()
        idx = fx["check_idx"]
        assert np.array_equal(t[idx], fx["check_t"])
        np.testing.assert_allclose(x[idx], fx["check_x"], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(p[idx], fx["check_p"], rtol=1e-13)
        traces = ts.integrate_screen(fx["pos"], fx["t0"], float(fx["dt"]), int(fx["nt"]),
                                     precision=precision, variant=variant)
    energy, _ = lw.mesh_energy(fx["corner"], fx["tri"].astype(np.int64), traces,
                               float(fx["dt"]))
    check_against_reference(fx, traces, energy)
