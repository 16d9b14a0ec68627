"""Device flattening of instanced meshes (rtgb_prepare_scene_instanced,
mesh_flatten.cu) against a numpy restatement of the host lowering's
arithmetic (add_v2_mesh, realtime_scene_adapter.cpp:289-346): points by the
3 x 4 transform and normals by the transposed normal matrix in double
precision, in the host's order of operations, then rounded to float;
winding flips, subset and instance materials, prototypes without normals /
texcoords, an empty prototype and thousands of instances after the scene's
own triangles. The SceneIR v2 harness checks the same path against the C++
host lowering of a real scene (tests/test_scene_ir_v2.py)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi

TRI = np.dtype([("p0", "<f4", 3), ("p1", "<f4", 3), ("p2", "<f4", 3), ("n0", "<f4", 3), ("n1", "<f4", 3),
                ("n2", "<f4", 3), ("uv0", "<f4", 2), ("uv1", "<f4", 2), ("uv2", "<f4", 2),
                ("material_index", "<i4"), ("has_vertex_normals", "<i4"), ("has_texcoords", "<i4")])
assert TRI.itemsize == C.sizeof(abi.Triangle)


def _prototype(rng, points, tris, normals, texcoords):
    p = {"points": rng.uniform(-1, 1, (points, 3)), "corners": rng.integers(0, max(points, 1), (tris, 3)).astype(np.int32),
         "normals": rng.normal(size=(tris, 3, 3)) if normals else None,
         "texcoords": rng.uniform(0, 1, (tris, 3, 2)) if texcoords else None,
         "materials": np.where(rng.random(tris) < 0.3, rng.integers(0, 4, tris), abi.INSTANCE_MATERIAL).astype(np.int32)}
    return p


def _instance(rng, prototype):
    lin = rng.normal(size=(3, 3))
    if rng.random() < 0.5:
        lin[0] *= -1.0  # mirrored: negative determinant
    t = rng.uniform(-20, 20, 3)
    world = np.concatenate([lin, t[:, None]], axis=1)
    inv = np.linalg.inv(lin)
    flip = int(rng.random() < 0.5)
    return {"prototype": prototype, "material": int(rng.integers(0, 4)), "flip": flip, "world": world, "inv": inv}


def _expected(protos, insts) -> np.ndarray:
    out = []
    for inst in insts:
        p = protos[inst["prototype"]]
        n = len(p["materials"])
        if n == 0:
            continue
        e = np.zeros(n, dtype=TRI)
        slot = [0, 2, 1] if inst["flip"] else [0, 1, 2]
        w, a = inst["world"], inst["inv"].reshape(-1)
        for k, name in enumerate(("p0", "p1", "p2")):
            pts = p["points"][p["corners"][:, slot[k]]]
            x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
            for r in range(3):
                e[name][:, r] = ((w[r, 0] * x + w[r, 1] * y) + w[r, 2] * z + w[r, 3]).astype(np.float32)
        if p["normals"] is not None:
            for k, name in enumerate(("n0", "n1", "n2")):
                nn = p["normals"][:, slot[k]]
                t0 = a[0] * nn[:, 0] + a[3] * nn[:, 1] + a[6] * nn[:, 2]
                t1 = a[1] * nn[:, 0] + a[4] * nn[:, 1] + a[7] * nn[:, 2]
                t2 = a[2] * nn[:, 0] + a[5] * nn[:, 1] + a[8] * nn[:, 2]
                ln = np.sqrt(t0 * t0 + t1 * t1 + t2 * t2)
                e[name] = np.stack([t0 / ln, t1 / ln, t2 / ln], axis=1).astype(np.float32)
            e["has_vertex_normals"] = 1
        if p["texcoords"] is not None:
            for k, name in enumerate(("uv0", "uv1", "uv2")):
                e[name] = p["texcoords"][:, slot[k]].astype(np.float32)
            e["has_texcoords"] = 1
        e["material_index"] = np.where(p["materials"] == abi.INSTANCE_MATERIAL, inst["material"], p["materials"])
        out.append(e)
    return np.concatenate(out) if out else np.zeros(0, dtype=TRI)


class _MeshSet:
    def __init__(self, protos, insts):
        self._keep = []

        def ptr(a, t):
            if a is None:
                return None
            a = np.ascontiguousarray(a)
            self._keep.append(a)
            return a.ctypes.data_as(C.POINTER(t))

        self.protos = (abi.MeshPrototype * len(protos))()
        for i, p in enumerate(protos):
            v = self.protos[i]
            v.points = ptr(p["points"].astype(np.float64), C.c_double)
            v.point_count = len(p["points"])
            v.triangle_count = len(p["materials"])
            v.corner_points = ptr(p["corners"], C.c_int32)
            v.corner_normals = ptr(p["normals"], C.c_double)
            v.corner_texcoords = ptr(p["texcoords"], C.c_double)
            v.triangle_materials = ptr(p["materials"], C.c_int32)
        self.insts = (abi.MeshInstance * len(insts))()
        for i, s in enumerate(insts):
            v = self.insts[i]
            v.prototype, v.material, v.flip_winding = s["prototype"], s["material"], s["flip"]
            v.world[:] = list(s["world"].reshape(-1))
            v.normal_matrix[:] = list(s["inv"].reshape(-1))
        self.set = abi.MeshSet(self.protos, len(protos), self.insts, len(insts))


def _base_scene(rng, own_triangles):
    keep = []
    mats = (abi.Material * 4)()
    for i in range(4):
        mats[i].albedo_texture, mats[i].emission_texture, mats[i].type, mats[i].openpbr_index = 0, -1, 0, -1
    tex = (abi.Texture * 1)()
    tex[0].type, tex[0].even_texture, tex[0].odd_texture = 0, -1, -1
    tex[0].color[:] = (0.5, 0.5, 0.5)
    tris = (abi.Triangle * max(1, own_triangles))()
    for i in range(own_triangles):
        tris[i].p0[:] = rng.uniform(-5, 5, 3)
        tris[i].p1[:] = rng.uniform(-5, 5, 3)
        tris[i].p2[:] = rng.uniform(-5, 5, 3)
        tris[i].material_index = 1
    keep += [mats, tex, tris]
    v = abi.Scene()
    v.materials, v.material_count = C.cast(mats, C.POINTER(abi.Material)), 4
    v.textures, v.texture_count = C.cast(tex, C.POINTER(abi.Texture)), 1
    v.triangles, v.triangle_count = C.cast(tris, C.POINTER(abi.Triangle)), own_triangles
    v.background[:] = (0.2, 0.2, 0.2)
    return v, keep


def _case(seed=3, instances=3000):
    rng = np.random.default_rng(seed)
    protos = [_prototype(rng, 40, 60, True, True), _prototype(rng, 12, 20, False, True),
              _prototype(rng, 30, 45, True, False), _prototype(rng, 0, 0, False, False),
              _prototype(rng, 8, 11, False, False)]
    insts = [_instance(rng, int(rng.integers(0, len(protos)))) for _ in range(instances)]
    return rng, protos, insts


@pytest.mark.gpu
def test_device_flattening_matches_the_host_arithmetic():
    from ray_tracing_gb300.renderer import Renderer
    rng, protos, insts = _case()
    scene, keep = _base_scene(rng, 257)
    ms = _MeshSet(protos, insts)
    with Renderer() as r:
        r.prepare_scene_instanced(scene, ms.set)
        got = r.triangles()
        lights, _, _, tmap = r.light_table()
    want = _expected(protos, insts)
    own = np.frombuffer(bytes(C.string_at(scene.triangles, 257 * TRI.itemsize)), dtype=np.uint8).reshape(257, -1)
    assert got.shape[0] == 257 + len(want)
    assert np.array_equal(got[:257], own)  # the scene's own triangles come first, unchanged
    assert got[257:].tobytes() == want.tobytes()
    assert len(tmap) == got.shape[0]  # maps cover the flattened triangles
    assert len(lights) == 1 and lights[0]["type"] == 3  # the environment only


@pytest.mark.gpu
def test_reprepare_with_an_equal_mesh_set_is_a_reuse_and_a_change_refits():
    from ray_tracing_gb300.renderer import Renderer
    rng, protos, insts = _case(seed=4, instances=200)
    scene, keep = _base_scene(rng, 0)
    with Renderer() as r:
        ms1 = _MeshSet(protos, insts)  # the sets' arrays must outlive the calls
        r.prepare_scene_instanced(scene, ms1.set)
        first = r.triangles()
        ms2 = _MeshSet(protos, insts)
        r.prepare_scene_instanced(scene, ms2.set)
        info = abi.AccelerationInfo()
        abi.check(r.lib.rtgb_acceleration_info_get(r.h, C.byref(info)), r.h)
        assert abi.UPDATE_KINDS[info.update_kind] == "reuse"
        insts[7]["world"] = insts[7]["world"] * 1.5
        ms3 = _MeshSet(protos, insts)
        r.prepare_scene_instanced(scene, ms3.set)
        abi.check(r.lib.rtgb_acceleration_info_get(r.h, C.byref(info)), r.h)
        assert abi.UPDATE_KINDS[info.update_kind] == "refit"
        assert r.triangles().tobytes() != first.tobytes()
        assert r.triangles().tobytes() == _expected(protos, insts).tobytes()


@pytest.mark.gpu
def test_zero_length_normal_fails_with_the_reference_message():
    from ray_tracing_gb300.renderer import Renderer
    rng, protos, insts = _case(seed=5, instances=10)
    protos[0]["normals"][3, 1] = 0.0  # one corner normal of zero length
    insts = [dict(i, prototype=0) for i in insts]
    scene, keep = _base_scene(rng, 0)
    with Renderer() as r:
        ms = _MeshSet(protos, insts)
        with pytest.raises(abi.RtgbError, match="singular or zero-length mesh normal"):
            r.prepare_scene_instanced(scene, ms.set)


@pytest.mark.gpu
def test_out_of_range_corner_is_rejected_on_the_host():
    from ray_tracing_gb300.renderer import Renderer
    rng, protos, insts = _case(seed=6, instances=4)
    protos[1]["corners"][0, 2] = 12  # the prototype has 12 points
    scene, keep = _base_scene(rng, 0)
    with Renderer() as r:
        ms = _MeshSet(protos, insts)
        with pytest.raises(abi.RtgbError, match="mesh point index is out of range"):
            r.prepare_scene_instanced(scene, ms.set)


def test_mesh_structs_match_the_header_sizes():
    assert C.sizeof(abi.MeshInstance) == 184
    assert C.sizeof(abi.MeshPrototype) == 48
    assert abi.INSTANCE_MATERIAL == -(2 ** 31)
