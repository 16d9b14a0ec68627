"""Host-side scene builders and rig helpers (CPU, no GPU): the C5 textured
room's composition and the rig orbit used by its 60-frame measurement."""
from __future__ import annotations

import numpy as np

from ray_tracing_gb300 import scenes


def _emissive_triangles(sc) -> int:
    v = sc.view
    tris = np.ctypeslib.as_array(v.triangles, (v.triangle_count,))
    mats = np.ctypeslib.as_array(v.materials, (v.material_count,))
    opb = np.ctypeslib.as_array(v.openpbr_materials, (v.openpbr_material_count,))
    lit = [i for i, m in enumerate(mats) if m["openpbr_index"] >= 0 and opb[m["openpbr_index"]]["emission_luminance"] > 0]
    return int(np.isin(tris["material_index"], lit).sum())


def test_textured_room_composition():
    sc = scenes.HostScene("textured_room", detail=400000)
    c = sc.counts()
    assert 380000 <= c["triangles"] <= 420000
    assert c["materials"] == 604 and c["textures"] == 4 and c["spheres"] == c["quads"] == 0
    assert _emissive_triangles(sc) == 4096
    v = sc.view
    tris = np.ctypeslib.as_array(v.triangles, (v.triangle_count,))
    pts = np.concatenate([tris["p0"], tris["p1"], tris["p2"]])
    assert pts.min(0)[0] >= -15.0 and pts.max(0)[0] <= 15.0 and pts.max(0)[1] <= 8.0 + 1e-6
    tex = np.ctypeslib.as_array(v.textures, (v.texture_count,))
    opb = np.ctypeslib.as_array(v.openpbr_materials, (v.openpbr_material_count,))
    bound = {int(tex[t]["type"]) for t in opb["color_texture"][:, 0] if t >= 0}
    assert bound == {1, 3}  # base colours bound to the checker (floor) and the 3D noise (walls)
    full = scenes.HostScene("textured_room")
    assert 3900000 <= full.counts()["triangles"] <= 4100000


def test_textured_room_rig_is_mixed_1080p():
    rig = scenes.default_rig("textured_room", 4)
    assert rig.active_count == 4
    assert [(c.width, c.height, c.model) for c in rig.cameras[:4]] == [(1920, 1080, 0), (1920, 1080, 1)] * 2


def test_orbit_rig_rotates_poses_about_the_vertical_axis():
    rig = scenes.default_rig("textured_room", 4)
    same = scenes.orbit_rig(rig, 360.0)
    quarter = scenes.orbit_rig(rig, 90.0, center=(1.0, 0.0, 2.0))
    for i in range(4):
        r0 = np.array(rig.cameras[i].rotation[:]).reshape(3, 3)
        t0 = np.array(rig.cameras[i].translation[:])
        assert np.allclose(np.array(same.cameras[i].rotation[:]).reshape(3, 3), r0, atol=1e-12)
        assert np.allclose(np.array(same.cameras[i].translation[:]), t0, atol=1e-12)
        r1 = np.array(quarter.cameras[i].rotation[:]).reshape(3, 3)
        t1 = np.array(quarter.cameras[i].translation[:])
        assert np.allclose(r1.T @ r1, np.eye(3), atol=1e-12)
        d0, d1 = t0 - (1.0, 0.0, 2.0), t1 - (1.0, 0.0, 2.0)
        # a quarter turn about +y: (x, z) -> (z, -x), height unchanged
        assert np.allclose(d1, (d0[2], d0[1], -d0[0]), atol=1e-12)
        assert np.allclose(r1[:, 2], (r0[2, 2], r0[1, 2], -r0[0, 2]), atol=1e-12)
    # the source rig is untouched
    assert rig.cameras[0].translation[2] == -9.0
