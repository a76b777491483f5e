"""CPU-only checks of the boundary and of the host logic: the C-ABI library
builds, loads and exports every function include/teufel_cuda.h declares; the
status codes and options struct match the header; the screen geometry and
buffer layout follow the reference's ScreenObserver; calls without a GPU
report TEUFEL_ERR_NODEVICE instead of falling back to the CPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from teufel_gb300 import abi, harness as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "teufel_cuda.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(teufel_cuda_\w+)\s*\(", src)))


def test_library_exports_every_declared_function():
    L = abi.lib()
    declared = header_functions()
    assert len(declared) >= 12
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(abi.EXPORTED) == declared


def test_status_codes_match_header():
    src = open(HEADER).read()
    codes = dict((k, int(v)) for k, v in re.findall(r"#define (TEUFEL_\w+) (\d+)", src))
    assert codes["TEUFEL_OK"] == abi.TEUFEL_OK
    assert codes["TEUFEL_ERR_ARG"] == abi.TEUFEL_ERR_ARG
    assert codes["TEUFEL_ERR_RANGE"] == abi.TEUFEL_ERR_RANGE
    assert codes["TEUFEL_ERR_NODEVICE"] == abi.TEUFEL_ERR_NODEVICE
    assert codes["TEUFEL_PREC_FP64"] == abi.PREC_FP64
    assert abi.status_string(abi.TEUFEL_ERR_RANGE) == "FieldTrace::add - index out of range."


def test_options_struct_matches_header():
    src = open(HEADER).read()
    body = re.search(r"typedef struct teufel_options \{(.*?)\} teufel_options;", src, re.S)
    fields = re.findall(r"int (\w+);", body.group(1))
    assert fields == [f for f, _ in abi.Options._fields_]
    o = abi.options(abi.PREC_FP64, True, 3, True)
    assert (o.precision, o.device_pointers, o.n_slots, o.timing) == (1, 1, 3, 1)


def test_no_device_means_an_error_not_a_fallback():
    """Without an sm_103 device the C-ABI refuses the work."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    tr = H.Trajectories(np.zeros(2), np.zeros((2, 3)), np.zeros((2, 3)), np.zeros((2, 3)),
                        np.array([2], np.int32), np.array([-1.0]), np.array([1.0]))
    with pytest.raises(abi.TeufelError) as ei:
        abi.TrajSet(tr)
    assert ei.value.status == abi.TEUFEL_ERR_NODEVICE
    _, st = abi.deposit_injected([[0.0, 1.0]], [[[1, 0, 0, 0, 0, 0], [0, 0, 0, 0, 0, 0]]],
                                 0.0, 0.2, 8)
    assert st == abi.TEUFEL_ERR_NODEVICE


def test_screen_geometry_follows_screen_observer():
    """CellPosition/CellTimeZero (src/screen.cpp:97-110) with the integer
    division Nx/2 and the ix-major order of getBuffer (src/screen.cpp:249-272)."""
    s = H.Screen((0.1, -0.2, 10.0), (0.01, 0.0, 0.001), (0.0, 0.02, 0.0), 5, 4, 3e-8, 1e-15,
                 16, dtx=1e-14, dty=-2e-14)
    pos = s.pixel_positions()
    t0 = s.pixel_t0()
    assert pos.shape == (20, 3) and t0.shape == (20,)
    for ix in range(5):
        for iy in range(4):
            p = ix * 4 + iy
            a = ix - 5 // 2
            b = iy - 4 // 2
            exp = [0.1 + 0.01 * a + 0.0 * b, -0.2 + 0.0 * a + 0.02 * b, 10.0 + 0.001 * a + 0.0 * b]
            assert np.array_equal(pos[p], np.array(exp))
            assert t0[p] == 3e-8 + 1e-14 * a + -2e-14 * b


def test_workload_shapes():
    w = H.config1()
    assert w.n_pix == 441 and w.nots == 2048 and w.dt == 5e-15
    assert int(w.traj.n_points[0]) == 3802
    w4 = H.config4(count=2)
    assert w4.n_pix == 40000 and w4.nots == 4096
    w5 = H.config5(count=1)
    assert w5.n_pix == 10000 and w5.nots == 8192 and w5.dt == 1e-18
    specs = H.config3_specs()
    assert len(specs) == 16
    for s in specs:
        assert 1000 <= s["n_particles"] <= 100000
        assert 20 <= s["gamma0"] <= 100 and 4 <= s["n_periods"] <= 40
        assert 16 <= s["npix"] <= 128 and 512 <= s["nots"] <= 8192
        assert 2e-15 <= s["dt"] <= 2e-14 * 1.0000001


def test_bunch_subsets_are_consistent():
    """Particle m of a bunch is the same whether drawn alone or with others."""
    a = H.gaussian_bunch(10, 5, 1e-3, 1e-3, 1e-4, 0.01, 0.01, 300.0, 0.15, -3.0)
    b = H.gaussian_bunch(4, 5, 1e-3, 1e-3, 1e-4, 0.01, 0.01, 300.0, 0.15, -3.0, first=6)
    assert np.array_equal(a[6:], b)
