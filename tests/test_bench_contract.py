"""The JSON line of bench.py's reference arm, which the benchmark's callers
parse: its keys and their meaning, with the timed oracle sample replaced by
a stub so that the test takes seconds (the oracle's timing itself is what
the arm measures on the benchmark machine)."""
import io
import json
from contextlib import redirect_stdout
from types import SimpleNamespace

import pytest

import bench  # the repository root is on sys.path (conftest.py)


def test_reference_arm_line(monkeypatch):
    calls = []

    def fake_rate(w, target_s, nthreads):
        calls.append(target_s)
        return 2.5e8, "4 random pixels x 4 particles x 2434 steps", 0.5

    monkeypatch.setattr(bench, "cpu_rate", fake_rate)
    monkeypatch.setattr(bench, "make_batches", lambda n, batch, **kw: [small_workload()])
    args = SimpleNamespace(gpus=1, steps=3, warmup=2, batch=1024, impl="reference")
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(args) == 0
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] == pytest.approx(2.5e8)
    assert line["higher_is_better"] is True
    assert line["steps"] == 3 and line["warmup"] == 2 and line["n_gpus"] == 1
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["value"] == pytest.approx(2.5e8) and cb["unit"] == bench.UNIT
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == pytest.approx(2.5e8) and e2e["unit"] == bench.UNIT
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert len(calls) == 5  # warm-up and timed samples


def small_workload():
    """Two particles of the benchmark's bunch on its screen."""
    from teufel_gb300 import harness as H
    return H.config4(count=2)
