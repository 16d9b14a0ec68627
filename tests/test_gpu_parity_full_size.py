"""GPU-vs-oracle parity at the configurations' full sizes.

The other parity tests run shrunken frames; these run the measured
configurations at their own resolution, sample count, depth and scene size,
where effects that only appear at scale would show: queue capacities at
millions of paths, Morton precision over millions of primitives, the
traversal bound, equal-t ties in dense meshes. The GPU renders whole frames;
the oracle renders every frame in full where ReSTIR needs the previous frame's
reservoirs (the benchmark frame), else every k-th row (row_stride), and the
paths of those rows are compared with the gates of test_gpu_parity.py
(legacy materials) and test_openpbr_render.py (OpenPBR). The diverged-path
fraction of each configuration is written to the JSON file named by
RTGB_PARITY_REPORT when that variable is set.
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import compare_paths
from ray_tracing_gb300 import scenes

ROOT = Path(__file__).resolve().parent.parent
pytestmark = pytest.mark.gpu

REL = 1e-4


def _report(name: str, **fields):
    path = os.environ.get("RTGB_PARITY_REPORT")
    if not path:
        return
    p = Path(path)
    data = json.loads(p.read_text()) if p.exists() else {}
    data[name] = fields
    p.write_text(json.dumps(data, indent=1))


def _rows_mask(width: int, height: int, spp: int, stride: int) -> np.ndarray:
    """Path mask of the rows y % stride == 0 (paths are pixel-major, sample-minor)."""
    rows = (np.arange(height) % stride) == 0
    return np.repeat(np.repeat(rows, width), spp)


def _paths(gpu, orc, cam, width, height, spp, mb, stride):
    gc, gr = gpu.path_records(cam, spp, mb)
    oc, orad = orc.path_records(cam, spp, mb)
    m = _rows_mask(width, height, spp, stride)
    return gc[m], gr[m], oc[m], orad[m]


def _gate_legacy(gc, gr, oc, orad, max_diverged):
    diverged, max_err, bad = compare_paths(gc, gr, oc, orad, rel=REL)
    assert diverged <= max_diverged, f"{diverged:.2e} of paths diverged"
    assert bad == 0, f"{bad} identical paths over {REL} relative (max {max_err:.2e})"
    return diverged, max_err


def _gate_openpbr(gc, gr, oc, orad, max_diverged):
    diverged, max_err, bad = compare_paths(gc, gr, oc, orad, rel=REL)
    assert diverged <= max_diverged, f"{diverged:.2e} of paths diverged"
    same = np.all(gc == oc, axis=1)
    err = (np.abs(gr - orad) / np.maximum(np.abs(orad), 1e-6))[same].max(axis=1)
    assert np.quantile(err, 0.999) <= 5e-5, f"99.9th percentile {np.quantile(err, 0.999):.2e}"
    assert max_err <= 1e-3, f"max relative error {max_err:.2e} on identical paths"
    assert bad <= 1e-3 * same.sum(), f"{bad} identical paths over {REL} relative"
    return diverged, max_err


def _render(sc, rig, prof, frames, stride, oracle_bvh=True):
    from oracle.binding import OracleRenderer
    from ray_tracing_gb300.renderer import Renderer
    gpu = Renderer(debug_path_records=True)
    gpu.prepare_scene(sc.view)
    orc = OracleRenderer(sc.view, use_reference_bvh=oracle_bvh)
    orc.set_path_records(True)
    for _ in range(frames):
        gpu.render_frame(rig, prof, rig.active_count)
        orc.render_frame(rig, prof, rig.active_count, row_stride=stride)
    return gpu, orc


def test_benchmark_frame_random_spheres_4x640x480_restir32():
    """The benchmark frame itself: 1024 analytic rect lights, 4 x 640x480,
    1 spp, depth 4, 32-candidate ReSTIR with temporal and spatial reuse, three
    frames so the reuse reads real history; every path and reservoir."""
    sys.path.insert(0, str(ROOT))
    import bench
    sc, rig, prof = bench.make_inputs()
    prof.enable_denoise = 0
    gpu, orc = _render(sc, rig, prof, frames=3, stride=1)
    out = {}
    for cam in range(4):
        w, h = rig.cameras[cam].width, rig.cameras[cam].height
        d, e = _gate_legacy(*_paths(gpu, orc, cam, w, h, 1, 4, 1), max_diverged=2e-3)
        g, o = gpu.reservoirs(cam), orc.reservoirs(cam)
        agree = float(np.mean(g["light_index"] == o["light_index"]))
        valid = float(np.mean(g["valid"] == o["valid"]))
        assert agree > 0.99 and valid > 0.99, (agree, valid)
        out[f"camera{cam}"] = {"diverged": d, "max_rel_err_identical": e, "reservoir_light_agreement": agree}
    _report("C2_random_spheres_4x640x480_restir32_3frames", paths=4 * 640 * 480, **out)
    gpu.close()
    orc.close()
    sc.close()


def test_cornell_box_256x256_64spp_depth8():
    sc = scenes.HostScene("cornell_box")
    rig = scenes.default_rig("cornell_box", 1)
    prof = scenes.profile("quality", samples_per_pixel=64, max_bounces=8, enable_denoise=0, enable_restir_di=0)
    assert (rig.cameras[0].width, rig.cameras[0].height) == (256, 256)
    stride = 4
    gpu, orc = _render(sc, rig, prof, frames=1, stride=stride, oracle_bvh=False)
    d, e = _gate_legacy(*_paths(gpu, orc, 0, 256, 256, 64, 8, stride), max_diverged=2e-3)
    _report("C1_cornell_256x256_64spp_d8", row_stride=stride, paths_compared=64 * 256 * 64, diverged=d,
            max_rel_err_identical=e)
    gpu.close()
    orc.close()
    sc.close()


def test_c3_terrain_1m_triangles_mixed_rig():
    """C3: 999,712 triangles (displaced terrain + 200 icosphere instances),
    constant OpenPBR, 256 emissive triangles; 2 x pinhole32 640x480 and
    2 x equi62_lut1d 1280x1024 in one launch; 1 spp, depth 4."""
    sc = scenes.HostScene("triangle_terrain_pbr", detail=1000000)
    rig = scenes.default_rig("triangle_terrain_pbr", 4)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0, enable_restir_di=1)
    stride = 16
    gpu, orc = _render(sc, rig, prof, frames=1, stride=stride)
    assert gpu.acceleration_info().traversal_stack_overflows == 0
    out = {}
    for cam in range(4):
        w, h = rig.cameras[cam].width, rig.cameras[cam].height
        d, e = _gate_openpbr(*_paths(gpu, orc, cam, w, h, 1, 4, stride), max_diverged=2e-2)
        out[f"camera{cam}"] = {"size": f"{w}x{h}", "model": int(rig.cameras[cam].model), "diverged": d,
                               "max_rel_err_identical": e}
    _report("C3_terrain_1Mtri_2pinhole640_2equi1280", triangles=sc.view.triangle_count, row_stride=stride, **out)
    gpu.close()
    orc.close()
    sc.close()


def _c5(constant_walls: bool):
    sc = scenes.HostScene("textured_room")
    if constant_walls:
        v = sc.view
        for i in range(v.texture_count):
            if v.textures[i].type == 3:   # the walls' 3D noise -> a constant grey
                v.textures[i].type = 0
                v.textures[i].color[0] = v.textures[i].color[1] = v.textures[i].color[2] = 0.55
    rig = scenes.default_rig("textured_room", 4)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=6, enable_denoise=0, enable_restir_di=1,
                          restir_initial_candidates=32, restir_temporal_reuse=1, restir_spatial_neighbors=1)
    return sc, rig, prof


def test_c5_textured_room_4m_triangles_1080p():
    """C5 as measured: 3,996,544 triangles, checker-textured floor, 3D-noise
    walls, 4096 emissive OpenPBR triangles; 2 x pinhole32 + 2 x equi62_lut1d at
    1920x1080; 1 spp, depth 6.

    The walls' hash noise (fract(sin(dot(p, k)) * 43758.5453), programs.cu:184-209)
    is chaotic in the position: its slope is about 3.5e6 per unit length, so
    hit points that differ in the last bit, as the points after a BSDF sample
    do (the sampled direction goes through CUDA's and the host's sinf/cosf/powf,
    which differ in the last bit now and then), see unrelated colours from
    there on. Paths therefore stay identical only up to the first scatter off a
    wall (measured: 0.02 % of paths differ at depth 2, 4.2 % at depth 6, and
    with the noise replaced by a constant 0.07 % at depth 6, the next test).
    What is checked here: the divergence bound, the bounce-0 AOVs (the noise
    itself at identical points, through the shared single-precision sine)
    pixel for pixel, and the image means."""
    sc, rig, prof = _c5(constant_walls=False)
    stride = 32
    gpu, orc = _render(sc, rig, prof, frames=1, stride=stride)
    assert gpu.acceleration_info().traversal_stack_overflows == 0
    out = {}
    for cam in range(4):
        w, h = rig.cameras[cam].width, rig.cameras[cam].height
        assert (w, h) == (1920, 1080)
        gc, gr, oc, orad = _paths(gpu, orc, cam, w, h, 1, 6, stride)
        diverged, _, _ = compare_paths(gc, gr, oc, orad, rel=REL)
        assert diverged <= 0.06, f"{diverged:.2e} of paths diverged"
        rows = np.arange(h) % stride == 0
        for buf in ("albedo", "normal", "depth"):
            g = gpu.buffer(cam, buf)[rows]
            o = orc.buffer(cam, buf)[rows]
            close = np.isclose(g, o, rtol=1e-5, atol=1e-6)
            assert close.mean() > 0.999, f"cam {cam} {buf}: {1 - close.mean():.2e} mismatched"
        gm, om = float(gr.mean()), float(orad.mean())
        assert abs(gm - om) <= 0.03 * om, (gm, om)
        out[f"camera{cam}"] = {"model": int(rig.cameras[cam].model), "diverged": diverged, "mean_gpu": gm,
                               "mean_oracle": om}
    _report("C5_textured_room_4Mtri_4x1920x1080_d6", triangles=sc.view.triangle_count, row_stride=stride, **out)
    gpu.close()
    orc.close()
    sc.close()


def test_c5_room_with_constant_walls_paths_match():
    """The C5 configuration with the walls' noise replaced by a constant grey:
    path-by-path gates. Six bounces of OpenPBR in a closed room condition the
    radiance a little worse than the gallery scene's (the GGX term amplifies
    last-bit direction changes after each glossy bounce), so the bounds are the
    measured ones with margin: 0.07 % of paths diverged, 99.9th percentile of
    identical-path error 1.3e-4, 0.13 % of identical paths over 1e-4, worst
    1.3e-2."""
    sc, rig, prof = _c5(constant_walls=True)
    stride = 32
    gpu, orc = _render(sc, rig, prof, frames=1, stride=stride)
    out = {}
    for cam in range(4):
        w, h = rig.cameras[cam].width, rig.cameras[cam].height
        gc, gr, oc, orad = _paths(gpu, orc, cam, w, h, 1, 6, stride)
        diverged, max_err, bad = compare_paths(gc, gr, oc, orad, rel=REL)
        assert diverged <= 2e-3, f"{diverged:.2e} of paths diverged"
        same = np.all(gc == oc, axis=1)
        err = (np.abs(gr - orad) / np.maximum(np.abs(orad), 1e-6))[same].max(axis=1)
        q = float(np.quantile(err, 0.999))
        assert q <= 3e-4, f"99.9th percentile {q:.2e}"
        assert max_err <= 5e-2, f"max relative error {max_err:.2e} on identical paths"
        assert bad <= 3e-3 * same.sum(), f"{bad} identical paths over {REL} relative"
        out[f"camera{cam}"] = {"diverged": diverged, "q999": q, "max_rel_err_identical": max_err,
                               "over_1e-4": bad / max(int(same.sum()), 1)}
    _report("C5_room_constant_walls_4x1920x1080_d6", row_stride=stride, **out)
    gpu.close()
    orc.close()
    sc.close()
