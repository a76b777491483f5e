"""PointObserver's SDDS output (the layout of
PointObserver::WriteTimeDomainFieldSDDS, src/point_observer.cpp:120-181)
written by the C++ observer layer, read back with a minimal reader of the
SDDS ASCII format: parameters, columns, units, types and every value."""
import os
import re
import subprocess

import numpy as np
import pytest

from teufel_gb300 import _build

HERE = os.path.dirname(os.path.abspath(__file__))


def read_sdds_ascii(path):
    """(parameters, columns, data) of a one-page SDDS1 ASCII file."""
    with open(path) as f:
        lines = f.read().split("\n")
    assert lines[0] == "SDDS1"
    params, cols, i = [], [], 1
    while not lines[i].startswith("&data"):
        m = re.match(r"&(parameter|column) (.*)&end", lines[i])
        assert m, lines[i]
        fields = dict(re.findall(r'(\w+)=("[^"]*"|[^,]*),', m.group(2)))
        fields = {k: v.strip('"') for k, v in fields.items()}
        (params if m.group(1) == "parameter" else cols).append(fields)
        i += 1
    assert "mode=ascii" in lines[i]
    body = [ln for ln in lines[i + 1:] if ln and not ln.startswith("!")]
    pvals = body[:len(params)]
    nrows = int(body[len(params)])
    rows = np.array([[float(v) for v in ln.split()] for ln in body[len(params) + 1:]])
    assert rows.shape == (nrows, len(cols))
    return params, pvals, cols, rows


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = _build.build_cuda()
    exe = tmp_path_factory.mktemp("sdds") / "sdds_driver"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{_build.INCLUDE}",
                    os.path.join(HERE, "cpp", "sdds_driver.cpp"), "-o", str(exe), str(lib),
                    f"-Wl,-rpath,{lib.parent}"], check=True)
    return str(exe)


def test_point_observer_sdds_layout_and_values(driver, tmp_path):
    rng = np.random.default_rng(7)
    n, t0, dt = 257, 3.3356409519815205e-08, 5e-15
    f = rng.standard_normal((n, 6)) * np.array([1e3, 1e3, 1e1, 1e-5, 1e-5, 1e-7])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        np.array([t0, dt]).tofile(fh)
        np.array([n], np.int32).tofile(fh)
        f.tofile(fh)
    out = tmp_path / "trace.sdds"
    r = subprocess.run([driver, str(inp), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    params, pvals, cols, rows = read_sdds_ascii(out)
    assert [(p["name"], p["type"]) for p in params] == [
        ("NumberTimeSteps", "long"), ("t0", "double"), ("dt", "double")]
    assert int(pvals[0]) == n and float(pvals[1]) == t0 and float(pvals[2]) == dt
    assert [(c["name"], c["units"], c["type"]) for c in cols] == [
        ("t", "s", "double"), ("Ex", "V/m", "double"), ("Ey", "V/m", "double"),
        ("Ez", "V/m", "double"), ("Bx", "T", "double"), ("By", "T", "double"),
        ("Bz", "T", "double")]
    assert [c["description"] for c in cols] == ["time"] + ["electric field"] * 3 + \
        ["magnetic field"] * 3
    assert np.array_equal(rows[:, 0], t0 + np.arange(n) * dt)
    assert np.array_equal(rows[:, 1:], f)


def test_point_observer_sdds_unwritable_path_raises(driver, tmp_path):
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        np.array([0.0, 1e-15]).tofile(fh)
        np.array([2], np.int32).tofile(fh)
        np.zeros((2, 6)).tofile(fh)
    r = subprocess.run([driver, str(inp), str(tmp_path / "no" / "such" / "dir" / "x.sdds")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "WriteTimeDomainFieldSDDS" in r.stderr
