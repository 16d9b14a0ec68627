"""SceneIR v2 input (include/rtgb_scene_ir_v2.hpp; src/scene/scene_ir_v2.cpp,
realtime_scene_adapter.cpp, openpbr_core_adapter.cpp and
analytic_light_compiler.cpp of the reference).

CPU: tests/scene_ir_v2_harness.cpp, compiled against the headers and linked
to librtgb.so, runs the reference's adapter and light-compiler expectations
(tests/test_realtime_scene_adapter.cpp, tests/test_analytic_light_compiler.cpp;
for SceneIR v1 also the Cornell box built through the IR, byte for byte equal
to the builtin scene)
and cases of its own (validator codes, time samples, reset transforms,
visibility and purpose, winding, normals, spheres, the scene file), then
writes a parity scene lowered from SceneIR v2 to a scene file.
GPU: that scene (meshes, n-gons, instances, subsets, checker / image /
constant textures on OpenPBR inputs, all six analytic light types) renders
through the wavefront path and matches the oracle along identical paths, and
render_realtime renders it from the scene file into its usual artifacts.
"""
from __future__ import annotations

import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import compare_paths, equi, look_at, pinhole, render_both, rig_of
from ray_tracing_gb300 import build as _build
from ray_tracing_gb300 import scenes

ROOT = Path(__file__).resolve().parent.parent
HARNESS = Path(__file__).resolve().parent / "scene_ir_v2_harness.cpp"


@pytest.fixture(scope="module")
def parity_scene_file(tmp_path_factory):
    if not _build.LIB.exists():
        _build.build_all()
    d = tmp_path_factory.mktemp("scene_ir_v2")
    exe = d / "harness"
    subprocess.run(["g++", "-std=c++23", "-O1", "-Wall", "-Wextra", "-I", str(ROOT / "include"),
                    "-I", str(_build.CSRC), "-I", str(_build._cuda_home() / "include"), str(HARNESS),
                    "-L", str(_build.LIB_DIR), "-lrtgb", f"-Wl,-rpath,{_build.LIB_DIR}", "-o", str(exe)], check=True)
    out = d / "parity.rtgbscene"
    res = subprocess.run([str(exe), str(d), "--write-scene", str(out)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "failures=0" in res.stdout
    return out


@pytest.mark.gpu
def test_instanced_lowering_flattens_on_the_device_like_the_host(parity_scene_file):
    # rtgb_prepare_scene_instanced (mesh_flatten.cu) against rtgb_prepare_scene
    # of the flat lowering: triangles, light table and a frame, bit for bit
    exe = parity_scene_file.parent / "harness"
    res = subprocess.run([str(exe), str(parity_scene_file.parent), "--instanced-gpu"], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "failures=0" in res.stdout
    assert res.stdout.count("instanced variant") == 3


def test_harness_cases_pass_and_the_scene_file_loads(parity_scene_file):
    sc = scenes.HostScene.load(parity_scene_file)
    c = sc.counts()
    assert c == {"spheres": 2, "quads": 0, "triangles": 53, "media": 0, "analytic_lights": 6, "materials": 6,
                 "textures": 4}
    lights = np.ctypeslib.as_array(sc.view.analytic_lights, (6,))
    assert [int(x["type"]) for x in lights] == [0, 2, 1, 3, 4, 5]
    assert abs(float(lights[-1]["cdf"]) - 1.0) == 0.0


def test_scene_file_round_trip_from_python(parity_scene_file, tmp_path):
    a = scenes.HostScene.load(parity_scene_file)
    a.save(tmp_path / "again.rtgbscene")
    assert (tmp_path / "again.rtgbscene").read_bytes() == parity_scene_file.read_bytes()
    (tmp_path / "bad.rtgbscene").write_bytes(b"RTGBSCN1" + b"\0" * 8)
    with pytest.raises(Exception):
        scenes.HostScene.load(tmp_path / "bad.rtgbscene")


@pytest.mark.gpu
def test_scene_ir_v2_parity_scene_matches_oracle(parity_scene_file):
    cams = [pinhole(80, 60, 75.0), pinhole(64, 48, 60.0, k=(0.02, -0.01, 0.003), p=(0.001, -0.0015)),
            equi(72, 72, 180.0), equi(64, 48, 160.0, radial=(0.01, -0.003, 0.0008, -0.0002, 5e-5, -1e-5))]
    look_at(cams[0], (0.0, 2.5, 6.5), (0.0, 0.8, 0.0), (0.0, 1.0, 0.0))
    look_at(cams[1], (-4.5, 2.0, 3.0), (0.0, 0.8, -0.5), (0.0, 1.0, 0.0))
    look_at(cams[2], (0.0, 3.5, 0.5), (0.0, 0.0, 0.5), (0.0, 0.0, -1.0))
    look_at(cams[3], (4.0, 1.5, -4.0), (0.0, 0.8, 0.0), (0.0, 1.0, 0.0))
    rig = rig_of(*cams)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0)
    sc = scenes.HostScene.load(parity_scene_file)
    _, gpu, orc = render_both("", rig, prof, frames=2, scene=sc)
    for cam in range(4):
        gc, gr = gpu.path_records(cam, 1, 4)
        oc, orad = orc.path_records(cam, 1, 4)
        diverged, max_err, bad = compare_paths(gc, gr, oc, orad, rel=1e-4)
        assert diverged <= 2e-3, f"camera {cam}: {diverged:.2e} of paths diverged"
        assert bad == 0, f"camera {cam}: {bad} identical paths over 1e-4 relative (max {max_err:.2e})"
        assert float(np.mean(gr)) > 0.0


@pytest.mark.gpu
def test_render_realtime_renders_the_scene_file(parity_scene_file, tmp_path):
    if not _build.CLI.exists():
        _build.build_all()
    res = subprocess.run([str(_build.CLI), "--scene-file", str(parity_scene_file), "--camera-count", "2", "--frames", "2",
                          "--warmup-frames", "1", "--width", "96", "--height", "72", "--output-dir", str(tmp_path)],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    summary = json.loads((tmp_path / "benchmark_summary.json").read_text())
    assert summary["metadata"]["camera_count"] == 2 and summary["extensions"]["rays_traced"] > 0
    assert all(r["average_luminance"] > 0.0 for r in summary["per-camera"])
    for f in range(2):
        for c in range(2):
            assert (tmp_path / f"frame_{f:04d}_cam_{c}.png").stat().st_size > 0
