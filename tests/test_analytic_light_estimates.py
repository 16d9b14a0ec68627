"""Quantitative analytic-light estimates (the setup of the reference's
tests/test_analytic_light_quantitative.cpp:27-340), checked on the oracle
against an independent quadrature of the irradiance.

One 1 x 1 pixel camera looks at a Lambertian receiver (albedo 0.5) lit by a
single unit-radiance light of each type (sphere, disk, rect, cylinder,
distant cone of 15 degrees, dome), 16384 samples, one bounce. The expected
pixel is albedo / pi x E with E = the irradiance at the receiver point,
integrated here numerically in double precision (area lights over their
emitting side, the cone over its solid angle); the dome is the reference's
furnace case (E = pi). Tolerance: the reference's max(0.004, 5 % of scale).
CPU only."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

from ray_tracing_gb300 import abi, scenes

ALBEDO = 0.5
SAMPLES = 16384
RECEIVER = np.array([0.0, 0.0, -4.0])      # legacy renderer coordinates
RECEIVER_N = np.array([0.0, 0.0, 1.0])
CENTER = np.array([0.0, 1.5, -2.0])
TO_LIGHT = (CENTER - RECEIVER) / np.linalg.norm(CENTER - RECEIVER)
TYPES = {"sphere": 0, "disk": 1, "rect": 2, "cylinder": 3, "distant": 4, "dome": 5}


def to_world(v):
    """legacy_renderer_to_world (frame_convention.h:33-35)."""
    return np.array([v[0], -v[2], v[1]])


def light_basis(kind):
    """make_estimator_light: (basis_x, basis_y, basis_z) columns in legacy coordinates."""
    x, y, z = np.eye(3)
    if kind == "distant":
        return x, y, TO_LIGHT
    if kind == "cylinder":
        return y, z, x
    if kind in ("disk", "rect"):
        n = (RECEIVER - CENTER) / np.linalg.norm(RECEIVER - CENTER)
        return x, np.cross(x, n), -n
    return x, y, z


def build_scene(kind):
    tex = abi.Texture(type=0, even_texture=-1, odd_texture=-1, u_address_mode=1, v_address_mode=1, filter_type=1, scale=1.0)
    tex.color[:] = (ALBEDO, ALBEDO, ALBEDO)
    mat = abi.Material(albedo_texture=0, emission_texture=-1, ior=1.0, fuzz=0.0, type=0, openpbr_index=-1)
    quad = abi.Quad(material_index=0)
    quad.origin[:] = to_world((-2.0, -2.0, -4.0))
    quad.edge_u[:] = to_world((4.0, 0.0, 0.0))
    quad.edge_v[:] = to_world((0.0, 4.0, 0.0))
    l = abi.AnalyticLight(type=TYPES[kind], selection_pdf=1.0, cdf=1.0, radius=0.5, width=1.0, height=1.0, length=1.0,
                          cos_theta_max=1.0)
    l.position[:] = to_world(CENTER)
    l.radiance[:] = (1.0, 1.0, 1.0)
    bx, by, bz = light_basis(kind)
    l.basis_x[:], l.basis_y[:], l.basis_z[:] = to_world(bx), to_world(by), to_world(bz)
    if kind == "sphere":
        l.radius, l.world_area = 0.75, 4.0 * math.pi * 0.75 ** 2
    elif kind == "cylinder":
        l.radius, l.length, l.world_area = 0.75, 1.5, 2.0 * math.pi * 0.75 * 1.5
    elif kind == "disk":
        l.radius, l.world_area = 1.0, math.pi
    elif kind == "rect":
        l.width, l.height, l.world_area = 2.0, 2.0, 4.0
    elif kind == "distant":
        l.cos_theta_max = math.cos(math.radians(15.0))
    keep = [(abi.Texture * 1)(tex), (abi.Material * 1)(mat), (abi.Quad * 1)(quad), (abi.AnalyticLight * 1)(l)]
    v = abi.Scene()
    v.textures, v.texture_count = C.cast(keep[0], C.POINTER(abi.Texture)), 1
    v.materials, v.material_count = C.cast(keep[1], C.POINTER(abi.Material)), 1
    v.quads, v.quad_count = C.cast(keep[2], C.POINTER(abi.Quad)), 1
    v.analytic_lights, v.analytic_light_count = C.cast(keep[3], C.POINTER(abi.AnalyticLight)), 1
    return v, keep


def oracle_estimate(kind):
    from oracle.binding import OracleRenderer
    view, keep = build_scene(kind)
    rig = abi.CameraRig()
    rig.active_count = 1
    c = rig.cameras[0]
    c.enabled, c.width, c.height, c.model = 1, 1, 1, 0
    c.pinhole = abi.Pinhole32(1e6, 1e6, 0.5, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0)
    identity = (C.c_double * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1)
    zero = (C.c_double * 3)(0, 0, 0)
    assert abi.load().rtgb_pack_camera_pose(identity, zero, c.rotation, c.translation) == 0
    prof = scenes.profile("realtime", samples_per_pixel=SAMPLES, max_bounces=1, rr_start_bounce=2, enable_denoise=0)
    orc = OracleRenderer(view, use_reference_bvh=True)
    orc.reset_sequence(0)
    orc.render_frame(rig, prof, 1)
    out = orc.buffer(0, "beauty")[0, 0, :3].astype(np.float64)
    orc.close()
    del keep
    return out


def _area_irradiance(points, normals, dA):
    """E = sum L cos_r cos_l / d^2 dA over the emitting side (unit radiance)."""
    d = points - RECEIVER
    dist2 = np.einsum("ij,ij->i", d, d)
    w = d / np.sqrt(dist2)[:, None]
    cos_r = np.clip(w @ RECEIVER_N, 0.0, None)
    cos_l = np.clip(-np.einsum("ij,ij->i", normals, w), 0.0, None)
    return float(np.sum(cos_r * cos_l / dist2 * dA))


def expected_irradiance(kind, n=600):
    bx, by, bz = light_basis(kind)
    if kind == "dome":
        return math.pi
    if kind == "sphere":
        d = np.linalg.norm(CENTER - RECEIVER)
        return math.pi * (0.75 / d) ** 2 * float(TO_LIGHT @ RECEIVER_N)
    if kind == "distant":
        ct = math.cos(math.radians(15.0))
        i = np.arange(n * n) + 0.5
        cos_t = 1.0 - (1.0 - ct) * i / (n * n)         # uniform in solid angle
        phi = 2.399963229728653 * i
        s = np.sqrt(1.0 - cos_t ** 2)
        t1 = np.cross(bz, [1.0, 0.0, 0.0])
        t1 /= np.linalg.norm(t1)
        t2 = np.cross(bz, t1)
        dirs = cos_t[:, None] * bz + s[:, None] * (np.cos(phi)[:, None] * t1 + np.sin(phi)[:, None] * t2)
        return float(np.mean(np.clip(dirs @ RECEIVER_N, 0.0, None)) * 2.0 * math.pi * (1.0 - ct))
    u = (np.arange(n) + 0.5) / n
    if kind == "rect":
        a, b = np.meshgrid(u - 0.5, u - 0.5, indexing="ij")
        pts = CENTER + 2.0 * a.reshape(-1, 1) * bx + 2.0 * b.reshape(-1, 1) * by
        normal = -np.cross(bx, by)
        return _area_irradiance(pts, np.tile(normal, (len(pts), 1)), 4.0 / (n * n))
    if kind == "disk":
        r, ph = np.meshgrid(np.sqrt(u), 2.0 * math.pi * u, indexing="ij")   # equal-area rings
        pts = CENTER + (r * np.cos(ph)).reshape(-1, 1) * bx + (r * np.sin(ph)).reshape(-1, 1) * by
        normal = -np.cross(bx, by)
        return _area_irradiance(pts, np.tile(normal, (len(pts), 1)), math.pi / (n * n))
    # cylinder: lateral surface, outward normals, around axis bz
    ph, z = np.meshgrid(2.0 * math.pi * u, (u - 0.5) * 1.5, indexing="ij")
    radial = np.cos(ph).reshape(-1, 1) * bx + np.sin(ph).reshape(-1, 1) * by
    pts = CENTER + 0.75 * radial + z.reshape(-1, 1) * bz
    return _area_irradiance(pts, radial, 2.0 * math.pi * 0.75 * 1.5 / (n * n))


@pytest.mark.parametrize("kind", list(TYPES))
def test_unit_radiance_estimate_matches_quadrature(kind):
    got = oracle_estimate(kind)
    want = ALBEDO / math.pi * expected_irradiance(kind)
    assert np.all(np.isfinite(got)) and np.all(got >= 0.0)
    assert got.max() <= ALBEDO + 0.04                       # finite-energy bound
    tol = max(0.004, 0.05 * max(0.02, float(got.max()), want))
    assert np.abs(got - want).max() <= tol, (kind, got, want)
    # tighter than the reference's gate: 16384 samples leave ~0.1-0.25 % noise
    assert np.abs(got - want).max() <= 0.01 * want, (kind, got, want)
    if kind == "dome":
        assert np.abs(got - ALBEDO).max() <= 0.025            # unit-environment furnace
