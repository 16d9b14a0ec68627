"""The reference's path-tracing gates (tests/test_optix_path_trace.cpp:9-171),
checked on the oracle, which restates the same per-pixel path: front / back
facing emitters, sphere-light solid-angle sampling, visibility of occluded
light, and MIS energy preservation when BSDF sampling joins light sampling.
Scenes, camera (pinhole 200 px focal, 64 x 64, identity pose) and profiles
(realtime preset, given spp and bounces, RR after the last bounce) are the
test's; colours become constant textures. CPU only."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi, scenes

SIZE = 64
CENTER = SIZE // 2


def legacy(v):
    """legacy_renderer_to_world (frame_convention.h:33-35)."""
    return (v[0], -v[2], v[1])


class _Scene:
    """rtgb_scene arrays built in Python (kept alive with the view)."""

    def __init__(self):
        self.textures, self.materials, self.spheres, self.quads, self.tris = [], [], [], [], []

    def _material(self, mtype, color):
        t = abi.Texture(type=0, even_texture=-1, odd_texture=-1, u_address_mode=1, v_address_mode=1, filter_type=1,
                        scale=1.0)
        t.color[:] = color
        self.textures.append(t)
        m = abi.Material(albedo_texture=-1, emission_texture=-1, ior=1.0, fuzz=0.0, type=mtype, openpbr_index=-1)
        if mtype == 3:
            m.emission_texture = len(self.textures) - 1
        else:
            m.albedo_texture = len(self.textures) - 1
        self.materials.append(m)
        return len(self.materials) - 1

    def light(self, color):
        return self._material(3, color)

    def diffuse(self, color):
        return self._material(0, color)

    def triangle(self, m, p0, p1, p2):
        t = abi.Triangle(material_index=m)
        t.p0[:], t.p1[:], t.p2[:] = p0, p1, p2
        self.tris.append(t)

    def quad(self, m, o, u, v):
        q = abi.Quad(material_index=m)
        q.origin[:], q.edge_u[:], q.edge_v[:] = o, u, v
        self.quads.append(q)

    def sphere(self, m, c, r):
        s = abi.Sphere(radius=r, material_index=m)
        s.center[:] = c
        self.spheres.append(s)

    def view(self) -> abi.Scene:
        def arr(t, items):
            a = (t * max(1, len(items)))(*items)
            self._keep.append(a)
            return C.cast(a, C.POINTER(t)), len(items)
        self._keep = []
        v = abi.Scene()
        v.textures, v.texture_count = arr(abi.Texture, self.textures)
        v.materials, v.material_count = arr(abi.Material, self.materials)
        v.spheres, v.sphere_count = arr(abi.Sphere, self.spheres)
        v.quads, v.quad_count = arr(abi.Quad, self.quads)
        v.triangles, v.triangle_count = arr(abi.Triangle, self.tris)
        return v


def _rig():
    rig = abi.CameraRig()
    rig.active_count = 1
    c = rig.cameras[0]
    c.enabled, c.width, c.height, c.model = 1, SIZE, SIZE, 0
    c.pinhole = abi.Pinhole32(200.0, 200.0, 32.0, 32.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    # CameraRig::add_pinhole with the identity body pose, packed (camera_rig.cpp:73-97)
    identity = (C.c_double * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1)
    zero = (C.c_double * 3)(0, 0, 0)
    assert abi.load().rtgb_pack_camera_pose(identity, zero, c.rotation, c.translation) == 0
    return rig


def _render(scene: _Scene, spp=4, bounces=1) -> np.ndarray:
    from oracle.binding import OracleRenderer
    prof = scenes.profile("realtime", samples_per_pixel=spp, max_bounces=bounces, rr_start_bounce=bounces + 1,
                          enable_denoise=0)
    view = scene.view()
    orc = OracleRenderer(view, use_reference_bvh=True)
    orc.reset_sequence(0)
    orc.render_frame(_rig(), prof, 1)
    beauty = orc.buffer(0, "beauty")
    orc.close()
    return beauty[..., :3].astype(np.float64).mean(axis=2)  # per-pixel (r + g + b) / 3


def _triangle_light_scene(front: bool, occluder: bool = False) -> _Scene:
    s = _Scene()
    light = s.light((20.0, 20.0, 20.0))
    diffuse = s.diffuse((0.8, 0.8, 0.8))
    dark = s.diffuse((0.0, 0.0, 0.0))
    a, b, c = legacy((-0.8, 1.2, 1.0)), legacy((0.0, 2.4, 1.0)), legacy((0.8, 1.2, 1.0))
    s.triangle(light, a, b, c) if front else s.triangle(light, a, c, b)
    s.quad(diffuse, legacy((-3.0, -3.0, -4.0)), legacy((6.0, 0.0, 0.0)), legacy((0.0, 6.0, 0.0)))
    if occluder:
        s.sphere(dark, (0.0, 1.5, 0.9), 0.65)
    return s


@pytest.fixture(scope="module")
def frames():
    out = {}
    out["front_direct"] = _render(_triangle_light_scene(True))
    out["back_direct"] = _render(_triangle_light_scene(False))
    out["unoccluded"] = _render(_triangle_light_scene(True), spp=256)
    out["occluded"] = _render(_triangle_light_scene(True, occluder=True), spp=256)
    out["light_only"] = _render(_triangle_light_scene(True), spp=512, bounces=1)
    out["light_and_bsdf"] = _render(_triangle_light_scene(True), spp=512, bounces=2)
    s = _Scene()
    light, diffuse = s.light((20.0, 20.0, 20.0)), s.diffuse((0.8, 0.8, 0.8))
    s.sphere(light, (0.0, -1.0, 1.8), 0.6)
    s.quad(diffuse, legacy((-3.0, -3.0, -4.0)), legacy((6.0, 0.0, 0.0)), legacy((0.0, 6.0, 0.0)))
    out["sphere_direct"] = _render(s, spp=64)
    for front in (True, False):
        e = _Scene()
        light = e.light((20.0, 20.0, 20.0))
        a, b, c = legacy((-1.2, -1.0, -3.0)), legacy((1.2, -1.0, -3.0)), legacy((0.0, 1.2, -3.0))
        e.triangle(light, a, b, c) if front else e.triangle(light, a, c, b)
        out["front_emissive" if front else "back_emissive"] = _render(e)
    return out


def test_front_and_back_facing_direct_light(frames):
    assert frames["front_direct"].shape == (SIZE, SIZE)
    assert frames["front_direct"].mean() > 0.05
    assert frames["back_direct"].mean() < 0.25 * frames["front_direct"].mean()


def test_sphere_light_and_visibility(frames):
    assert frames["sphere_direct"][CENTER, CENTER] > 0.01
    assert frames["occluded"][CENTER, CENTER] < 0.5 * frames["unoccluded"][CENTER, CENTER]


def test_mis_preserves_direct_light_energy(frames):
    lo = frames["light_only"][CENTER, CENTER]
    assert abs(frames["light_and_bsdf"][CENTER, CENTER] - lo) < 0.05 * lo


def test_front_and_back_facing_emissive_hits(frames):
    front = frames["front_emissive"][CENTER, CENTER]
    assert front > 1.0
    assert frames["back_emissive"][CENTER, CENTER] < 0.1 * front
