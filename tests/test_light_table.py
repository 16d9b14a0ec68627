"""The emissive light table built on the device (light_table.cu) against the
oracle's sequential build_light_distribution (packed_scene_preparation.cpp:
265-302): every PackedLight record bit for bit (type, primitive index,
selection pdf, cdf), and the primitive -> light maps.

The device splits the work over chunks of 2048 primitives and one warp for the
normalisation; the synthetic scene below spans many chunks with lights in
every position class (first / last of a chunk, runs, none), zero-area and
non-emissive primitives, weights over twelve orders of magnitude, and with
and without the environment entry."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi, scenes

BUILTIN = [("cornell_box", 0, 0), ("random_spheres", 0, 0), ("final_room", 0, 0), ("smoke", 0, 0),
           ("openpbr_gallery", 1, 0), ("triangle_terrain_pbr", 2, 60000), ("textured_room", 0, 300000)]


class _Scene:
    """Primitive arrays for rtgb_scene, kept alive with the view."""

    def __init__(self, background=(0.0, 0.0, 0.0)):
        self.textures, self.materials, self.spheres, self.quads, self.tris = [], [], [], [], []
        self.texels = []  # RGB triplets of the image textures
        self.background = background

    def emissive_image(self, rgb_rows) -> int:
        """A diffuse light whose emission is an image texture (its average
        luminance weighs the light: sum / count per channel, as the reference
        divides)."""
        h, w = len(rgb_rows), len(rgb_rows[0])
        t = abi.Texture(type=2, even_texture=-1, odd_texture=-1, image_offset=len(self.texels), image_width=w,
                        image_height=h)
        for row in rgb_rows:
            self.texels.extend(tuple(px) for px in row)
        self.textures.append(t)
        self.materials.append(abi.Material(albedo_texture=-1, emission_texture=len(self.textures) - 1, type=3,
                                           openpbr_index=-1))
        return len(self.materials) - 1

    def emissive(self, rgb) -> int:
        t = abi.Texture(type=0, even_texture=-1, odd_texture=-1)
        t.color[:] = rgb
        self.textures.append(t)
        self.materials.append(abi.Material(albedo_texture=-1, emission_texture=len(self.textures) - 1, type=3,
                                           openpbr_index=-1))
        return len(self.materials) - 1

    def diffuse(self) -> int:
        t = abi.Texture(type=0, even_texture=-1, odd_texture=-1)
        t.color[:] = (0.5, 0.5, 0.5)
        self.textures.append(t)
        self.materials.append(abi.Material(albedo_texture=len(self.textures) - 1, emission_texture=-1, type=0,
                                           openpbr_index=-1))
        return len(self.materials) - 1

    def view(self) -> abi.Scene:
        self._keep = []

        def arr(t, items):
            a = (t * max(1, len(items)))(*items)
            self._keep.append(a)
            return C.cast(a, C.POINTER(t)), len(items)

        v = abi.Scene()
        v.textures, v.texture_count = arr(abi.Texture, self.textures)
        v.materials, v.material_count = arr(abi.Material, self.materials)
        v.spheres, v.sphere_count = arr(abi.Sphere, self.spheres)
        v.quads, v.quad_count = arr(abi.Quad, self.quads)
        v.triangles, v.triangle_count = arr(abi.Triangle, self.tris)
        flat = [c for px in self.texels for c in px]
        texels = (C.c_float * max(1, len(flat)))(*flat)
        self._keep.append(texels)
        v.image_texels, v.image_texel_count = C.cast(texels, C.POINTER(C.c_float)), len(self.texels)
        v.background[:] = self.background
        return v


def _synthetic(background) -> _Scene:
    rng = np.random.default_rng(7)
    s = _Scene(background)
    lights = [s.emissive((10.0 ** e, 0.7 * 10.0 ** e, 0.2)) for e in range(-6, 6)]
    # image emitters: 7 x 5 and 3 x 11 texels, so sum / count and sum * (1 / count) differ
    lights += [s.emissive_image(rng.uniform(0.0, 3.0, (5, 7, 3)).tolist()),
               s.emissive_image(rng.uniform(0.0, 9.0, (11, 3, 3)).tolist())]
    dull = s.diffuse()
    for i in range(3000):  # spheres: every third one emits
        sp = abi.Sphere(radius=float(rng.uniform(0.01, 2.0)), material_index=lights[i % 14] if i % 3 == 0 else dull)
        sp.center[:] = rng.uniform(-50, 50, 3)
        s.spheres.append(sp)
    for i in range(2500):  # quads: runs of emitters across chunk boundaries
        q = abi.Quad(material_index=lights[(i // 7) % 14] if (i // 97) % 2 == 0 else dull)
        q.origin[:] = rng.uniform(-50, 50, 3)
        q.edge_u[:] = rng.uniform(-1, 1, 3)
        q.edge_v[:] = rng.uniform(-1, 1, 3) if i % 50 else q.edge_u[:]  # some zero-area quads
        s.quads.append(q)
    for i in range(9000):  # triangles: random emitters, degenerate ones, out-of-range materials
        t = abi.Triangle(material_index=lights[int(rng.integers(14))] if rng.random() < 0.4 else dull)
        if i % 1000 == 999:
            t.material_index = 1000
        p0 = rng.uniform(-50, 50, 3)
        t.p0[:] = p0
        t.p1[:] = p0 + rng.uniform(-2, 2, 3)
        t.p2[:] = p0 + rng.uniform(-2, 2, 3) if i % 333 else p0
        s.tris.append(t)
    return s


def _device_table(view):
    from ray_tracing_gb300.renderer import Renderer
    with Renderer() as r:
        r.prepare_scene(view)
        return r.light_table()


def _oracle_table(view):
    from oracle.binding import OracleRenderer
    o = OracleRenderer(view)
    try:
        return o.light_table()
    finally:
        o.close()


def _check(view):
    lights, sl, ql, tl = _device_table(view)
    want = _oracle_table(view)
    assert lights.shape == want.shape
    assert lights.tobytes() == want.tobytes()  # pdf and cdf bit for bit
    for kind, got_map, count in ((0, sl, view.sphere_count), (1, ql, view.quad_count), (2, tl, view.triangle_count)):
        expect = np.full(count, -1, dtype=np.int32)
        sel = np.nonzero(want["type"] == kind)[0]
        expect[want["primitive_index"][sel]] = sel
        assert np.array_equal(got_map, expect)
    return lights


@pytest.mark.gpu
@pytest.mark.parametrize("name,seed,detail", BUILTIN)
def test_builtin_scene_light_tables_match_oracle(name, seed, detail):
    with scenes.HostScene(name, seed=seed, detail=detail) as sc:
        lights = _check(sc.view)
    assert len(lights) > 0
    assert lights["cdf"][-1] == 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("background", [(0.0, 0.0, 0.0), (0.3, 0.5, 0.9)])
def test_many_chunk_light_table_matches_oracle(background):
    s = _synthetic(background)
    lights = _check(s.view())
    assert len(lights) > 4000  # many 2048-primitive chunks hold lights
    env = np.nonzero(lights["type"] == 3)[0]
    assert list(env) == ([len(lights) - 1] if background[0] > 0 else [])


@pytest.mark.gpu
def test_scene_without_lights_has_an_empty_table():
    s = _Scene()
    m = s.diffuse()
    t = abi.Triangle(material_index=m)
    t.p1[:] = (1.0, 0.0, 0.0)
    t.p2[:] = (0.0, 1.0, 0.0)
    s.tris.append(t)
    lights = _check(s.view())
    assert len(lights) == 0


def _restated_table(s: _Scene) -> np.ndarray:
    """build_light_distribution (packed_scene_preparation.cpp:190-302) as
    single-precision Python: every operation a float32 operation in the
    reference's order."""
    f = np.float32

    def lum(c):
        return max(f(0.0), f(0.2126) * c[0] + f(0.7152) * c[1] + f(0.0722) * c[2])

    def average(ti):
        t = s.textures[ti]
        if t.type == 0:
            return [max(f(t.color[k]), f(0.0)) for k in range(3)]
        if t.type == 2:
            n = t.image_width * t.image_height
            acc = [f(0.0)] * 3
            for px in s.texels[t.image_offset:t.image_offset + n]:
                acc = [acc[k] + f(px[k]) for k in range(3)]
            return [max(acc[k] / f(n), f(0.0)) for k in range(3)]
        raise AssertionError("texture type not used here")

    def mat_lum(mi):
        if mi < 0 or mi >= len(s.materials) or s.materials[mi].type != 3:
            return f(0.0)
        return lum(average(s.materials[mi].emission_texture))

    four_pi = f(4.0) * f(np.pi)
    rows = []

    def append(kind, i, w):
        if np.isfinite(w) and w > f(1e-12):
            rows.append([kind, i, w])

    for i, sp in enumerate(s.spheres):
        r = f(sp.radius)
        append(0, i, four_pi * r * r * mat_lum(sp.material_index))
    for i, q in enumerate(s.quads):
        u, v = [f(x) for x in q.edge_u], [f(x) for x in q.edge_v]
        c = (u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0])
        append(1, i, np.sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) * mat_lum(q.material_index))
    for i, t in enumerate(s.tris):
        p0, p1, p2 = [f(x) for x in t.p0], [f(x) for x in t.p1], [f(x) for x in t.p2]
        a = [p1[k] - p0[k] for k in range(3)]
        b = [p2[k] - p0[k] for k in range(3)]
        c = (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])
        append(2, i, f(0.5) * np.sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) * mat_lum(t.material_index))
    append(3, -1, four_pi * lum([f(x) for x in s.background]))
    total = f(0.0)
    for row in rows:
        total = total + row[2]
    out = np.zeros(len(rows), dtype=abi.LIGHT_DTYPE)
    cdf = f(0.0)
    for k, (kind, i, w) in enumerate(rows):
        pdf = w / total
        cdf = cdf + pdf
        out[k] = (kind, i, pdf, cdf)
    if len(rows):
        out["cdf"][-1] = 1.0
    return out


@pytest.mark.parametrize("background", [(0.0, 0.0, 0.0), (0.3, 0.5, 0.9)])
def test_oracle_light_table_is_the_sequential_single_precision_build(background):
    # pins the oracle's restatement (which pins the device table above),
    # image-texture emitters included: their average divides by the texel count
    s = _synthetic(background)
    got = _oracle_table(s.view())
    want = _restated_table(s)
    assert got.tobytes() == want.tobytes()


def test_light_record_layout():
    assert abi.LIGHT_DTYPE.itemsize == 16
    assert hasattr(abi.load(), "rtgb_download_light_table")
