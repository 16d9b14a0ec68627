"""Parity of the sm_103a wavefront path with the CPU oracle (through the C ABI).

Per path, the GPU and the oracle record the primitive hit at every bounce
(hit codes) and the final radiance. Paths whose hit codes agree must agree in
radiance within 1e-4 relative (1e-6 absolute floor); paths whose codes differ
are equal-t ties between the LBVH traversal order and the reference's
first-found order, or one-ulp differences of sinf/cosf/powf between CUDA and
the host libm — they must stay a tiny fraction.
"""
import numpy as np
import pytest

from _png import read_png
from helpers import compare_paths, equi, look_at, pinhole, render_both, rig_of, scaled_rig
from ray_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu

REL = 1e-4          # radiance tolerance along identical paths (1e-4 relative per pixel)
MAX_DIVERGED = 2e-3  # fraction of paths allowed to take a different (tied) branch


def _check_camera(gpu, orc, cam, spp, mb, max_diverged=MAX_DIVERGED):
    gc, gr = gpu.path_records(cam, spp, mb)
    oc, orad = orc.path_records(cam, spp, mb)
    diverged, max_err, bad = compare_paths(gc, gr, oc, orad, rel=REL)
    assert diverged <= max_diverged, f"camera {cam}: {diverged:.2e} of paths diverged"
    assert bad == 0, f"camera {cam}: {bad} identical paths over {REL} relative (max {max_err:.2e})"
    return diverged


def test_restir_acceptance_gpu_matches_reference_goldens():
    from pathlib import Path
    gold = Path(__file__).resolve().parent / "golden" / "restir_di"
    sc = scenes.HostScene("restir_acceptance")
    rig = scenes.default_rig("restir_acceptance", 1)
    from ray_tracing_gb300.renderer import Renderer
    out = {}
    for name, spp, restir, frames in (("reference", 256, False, 1), ("baseline", 16, False, 1),
                                      ("restir", 1, True, 2)):
        r = Renderer()
        r.prepare_scene(sc.view)
        for _ in range(frames):
            r.render_frame(rig, scenes.restir_acceptance_profile(spp, restir), 1)
        out[name] = r.download(0).beauty_rgba
        if name == "restir":
            d = r.restir_diagnostics(0)
            assert d.temporal_reuse_count > 0 and d.spatial_reuse_count > 0 and d.bias_corrected_count > 0
        r.close()
    for name, beauty in out.items():
        golden = read_png(gold / f"{name}.png").astype(int)
        diff = np.abs(scenes.display_u8(beauty[..., :3]).astype(int) - golden)
        assert diff.max() <= 2, f"{name}: max display error {diff.max()} (gate 2)"


def test_restir_acceptance_paths_and_reservoirs_match_oracle():
    rig = scenes.default_rig("restir_acceptance", 1)
    prof = scenes.restir_acceptance_profile(1, True)
    sc, gpu, orc = render_both("restir_acceptance", rig, prof, frames=3)
    _check_camera(gpu, orc, 0, 1, 1, max_diverged=0.0)
    g, o = gpu.reservoirs(0), orc.reservoirs(0)
    assert np.array_equal(g["valid"], o["valid"])
    assert np.array_equal(g["light_index"], o["light_index"])
    assert np.array_equal(g["candidate_count"], o["candidate_count"])
    assert np.array_equal(g["temporal_candidate_count"], o["temporal_candidate_count"])
    assert np.array_equal(g["spatial_candidate_count"], o["spatial_candidate_count"])
    assert np.allclose(g["estimator_weight"], o["estimator_weight"], rtol=1e-5, atol=0)


def test_cornell_box_paths_match_oracle():
    rig = scaled_rig(scenes.default_rig("cornell_box", 1), 0.5)   # 128x128, fx = fy = 64 / tan 20 deg
    prof = scenes.profile("quality", samples_per_pixel=4, max_bounces=8, rr_start_bounce=3, enable_denoise=0)
    sc, gpu, orc = render_both("cornell_box", rig, prof)
    _check_camera(gpu, orc, 0, 4, 8)
    gb = gpu.download(0).beauty_rgba
    ob = orc.buffer(0, "beauty")
    assert np.mean(np.abs(gb - ob)) < 1e-3 * max(1.0, float(np.mean(ob)))


def test_random_spheres_restir_four_cameras_match_oracle():
    rig = scaled_rig(scenes.default_rig("random_spheres", 4), 0.125)  # 4 x 80x60
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, restir_initial_candidates=32,
                          restir_spatial_neighbors=1, enable_denoise=0)
    sc, gpu, orc = render_both("random_spheres", rig, prof, frames=3, detail=256)
    for cam in range(4):
        _check_camera(gpu, orc, cam, 1, 4)
        g, o = gpu.reservoirs(cam), orc.reservoirs(cam)
        agree = float(np.mean(g["light_index"] == o["light_index"]))
        assert agree > 0.99


def test_bouncing_spheres_metal_glass_environment_match_oracle():
    rig = scaled_rig(scenes.default_rig("bouncing_spheres", 2), 0.2)
    prof = scenes.profile("balanced", samples_per_pixel=2, max_bounces=6, enable_restir_di=0, enable_denoise=0)
    sc, gpu, orc = render_both("bouncing_spheres", rig, prof, frames=2)
    for cam in range(2):
        _check_camera(gpu, orc, cam, 2, 6, max_diverged=5e-3)


def test_final_room_and_smoke_match_oracle():
    for name in ("final_room", "smoke"):
        rig = scaled_rig(scenes.default_rig(name, 2), 0.2)
        prof = scenes.profile("realtime", max_bounces=3, enable_denoise=0)
        sc, gpu, orc = render_both(name, rig, prof, frames=2)
        for cam in range(2):
            _check_camera(gpu, orc, cam, 1, 3)
            for buf in ("normal", "albedo", "depth", "flow", "flow_trustworthiness", "denoiser_normal"):
                g = gpu.buffer(cam, buf)
                o = orc.buffer(cam, buf)
                close = np.isclose(g, o, rtol=1e-5, atol=1e-6)
                assert close.mean() > 0.999, f"{name} cam {cam} {buf}: {1 - close.mean():.2e} mismatched"


def test_mixed_pinhole_equi_triangle_scene_matches_oracle():
    cams = [pinhole(64, 48, 90.0), pinhole(64, 48, 90.0, k=(0.02, -0.01, 0.003), p=(0.001, -0.0015)),
            equi(96, 80, 180.0), equi(96, 80, 180.0, radial=(0.01, -0.003, 0.0008, -0.0002, 5e-5, -1e-5),
                                       tangential=(0.0007, -0.0005))]
    for i, c in enumerate(cams):
        ang = np.radians(90.0 * i)
        look_at(c, (0.0, 4.0, 0.0), (np.sin(ang), 3.6, np.cos(ang)), (0.0, 1.0, 0.0))
    rig = rig_of(*cams)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0)
    sc, gpu, orc = render_both("triangle_terrain", rig, prof, frames=2, detail=20000, oracle_bvh=True)
    for cam in range(4):
        _check_camera(gpu, orc, cam, 1, 4)


def test_direction_debug_matches_oracle():
    import ctypes as C
    from oracle.binding import load as load_oracle
    from ray_tracing_gb300.renderer import Renderer
    cams = [pinhole(64, 48, 70.0, k=(0.02, -0.01, 0.003), p=(0.001, -0.0015)), equi(64, 48, 170.0)]
    look_at(cams[0], (1.0, -2.0, 3.5), (1.5, -2.0, 4.5), (0, 1, 0))
    look_at(cams[1], (-1.5, 0.75, 2.25), (-1.5, 0.5, 3.25), (0, 1, 0))
    rig = rig_of(*cams)
    r = Renderer()
    orc = load_oracle()
    for i in range(2):
        g = r.render_direction_debug(rig, i)
        o = np.empty_like(g)
        orc.orc_direction_debug(C.byref(rig.cameras[i]), o.ctypes.data)
        assert np.abs(g.astype(int) - o.astype(int)).max() <= 1   # reference contract: +-2 LSB


def _display_u8(v: np.ndarray) -> np.ndarray:
    """linear_to_display_u8 (src/realtime/display_transfer.h:9-15): sqrt of the
    clamped-positive value, clamp to [0, 0.999], scale by 255 in float32, round
    half away from zero (the values are non-negative, so floor(x + 0.5) in
    float64 is exact)."""
    c = np.clip(np.sqrt(np.maximum(v.astype(np.float32), np.float32(0))), np.float32(0), np.float32(0.999))
    return np.floor((c * np.float32(255)).astype(np.float64) + 0.5).astype(np.uint8)


def test_tonemap_matches_display_transfer():
    from ray_tracing_gb300.renderer import Renderer
    rig = scaled_rig(scenes.default_rig("random_spheres", 2), 0.15)
    prof = scenes.profile("balanced", samples_per_pixel=2, max_bounces=3, enable_denoise=0)
    sc = scenes.HostScene("random_spheres")
    r = Renderer()
    r.prepare_scene(sc.view)
    r.render_frame(rig, prof, 2)
    for cam in range(2):
        beauty = r.download(cam).beauty_rgba
        got = r.tonemap_rgba8(cam)
        assert np.array_equal(got[..., :3], _display_u8(beauty[..., :3]))
        assert np.all(got[..., 3] == 255)
        assert 0 < got[..., :3].mean() < 254


def test_lbvh_morton_order_matches_cpu_restatement():
    from oracle.lbvh import lbvh_reference
    from ray_tracing_gb300.renderer import Renderer
    for name, detail in (("random_spheres", 64), ("triangle_terrain", 30000), ("cornell_box", 0)):
        sc = scenes.HostScene(name, detail=detail)
        r = Renderer()
        r.prepare_scene(sc.view)
        keys, order, children = r.lbvh()
        ref_keys, ref_order, ref_children = lbvh_reference(sc.view)
        assert np.array_equal(keys, ref_keys), f"{name}: Morton codes differ"
        assert np.array_equal(order, ref_order), f"{name}: leaf order differs"
        assert np.array_equal(children, ref_children), f"{name}: hierarchy differs"
        assert r.acceleration_info().traversal_stack_overflows == 0
