"""benchmark_scene_lifecycle (utils/benchmark_gpu_scene_lifecycle.cpp over the C ABI).

CPU: argument validation. GPU: a short run checks every lifecycle kind and
writes the reference's JSON layout (schema 1).
"""
from __future__ import annotations

import json
import subprocess

import pytest

from ray_tracing_gb300 import build as _build


@pytest.fixture(scope="module")
def tool():
    if not _build.LIFECYCLE.exists():
        _build.build_all()
    return _build.LIFECYCLE


@pytest.mark.parametrize("args,message", [
    ([], "usage: benchmark_scene_lifecycle"),
    (["out.json", "--primitives", "1"], "--primitives is out of range"),
    (["out.json", "--iterations", "0"], "--iterations is out of range"),
    (["out.json", "--bogus", "1"], "unknown argument"),
    (["out.json", "--iterations"], "needs a value"),
])
def test_argument_validation(tool, tmp_path, args, message):
    res = subprocess.run([str(tool), *args], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert res.returncode != 0
    assert message in res.stderr


@pytest.mark.gpu
def test_lifecycle_kinds_and_report(tool, tmp_path):
    out = tmp_path / "lifecycle" / "gpu_scene_lifecycle.json"
    res = subprocess.run([str(tool), str(out), "--iterations", "3"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    rep = json.loads(out.read_text())
    assert rep["schema_version"] == 1 and rep["iterations"] == 3 and rep["primitive_count"] == 1024
    assert rep["acceleration"]["node_count"] == 1023
    assert rep["acceleration"]["primitive_reference_count"] == 1024
    # warm-up and every iteration: rebuild, reuse, update, refit, rebuild = 4 generations each
    assert rep["acceleration"]["generation"] == 4 + 4 * 3
    for kind in ("rebuild", "update", "refit", "reuse"):
        t = rep["timings"][kind]
        assert 0.0 <= t["avg_ms"] <= t["max_ms"] and t["p95_ms"] <= t["max_ms"]
    assert rep["device_timings"]["reuse"]["max_ms"] == 0.0
    assert rep["device_timings"]["refit"]["avg_ms"] > 0.0
