"""Host scenes, rigs and profiles through the C ABI's authoring helpers.

Thin Python handles over ``rtgb_host_scene_*``, ``rtgb_default_rig`` and
``rtgb_profile_preset`` (C++23 host code in ``librtgb.so``), so tests, the
bench and the oracle all consume the exact arrays the library produces.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class HostScene:
    """A builtin or procedural scene owned by the C++ host library."""

    def __init__(self, name: str, seed: int = 0, detail: int = 0, *, path=None):
        """A builtin scene by name, or (``path=``) a scene file written by
        rtgb_host_scene_save, e.g. one lowered from SceneIR v2."""
        self.lib = abi.load()
        self.ptr = C.c_void_p()
        if path is not None:
            self.name = str(path)
            abi.check(self.lib.rtgb_host_scene_load(str(path).encode(), C.byref(self.ptr)),
                      what=f"rtgb_host_scene_load({path})")
        else:
            self.name = name
            abi.check(self.lib.rtgb_host_scene_create(name.encode(), seed, detail, C.byref(self.ptr)),
                      what=f"rtgb_host_scene_create({name})")
        self.view = abi.Scene()
        abi.check(self.lib.rtgb_host_scene_view(self.ptr, C.byref(self.view)), what="rtgb_host_scene_view")

    @classmethod
    def load(cls, path) -> "HostScene":
        return cls("", path=path)

    def save(self, path) -> None:
        abi.check(self.lib.rtgb_host_scene_save(self.ptr, str(path).encode()), what=f"rtgb_host_scene_save({path})")

    def close(self):
        if self.ptr:
            self.lib.rtgb_host_scene_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __enter__(self) -> "HostScene":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def counts(self) -> dict[str, int]:
        v = self.view
        return {"spheres": v.sphere_count, "quads": v.quad_count, "triangles": v.triangle_count,
                "media": v.medium_count, "analytic_lights": v.analytic_light_count,
                "materials": v.material_count, "textures": v.texture_count}


def default_rig(scene_name: str, camera_count: int, width: int = 0, height: int = 0) -> abi.CameraRig:
    rig = abi.CameraRig()
    abi.check(abi.load().rtgb_default_rig(scene_name.encode(), camera_count, width, height, C.byref(rig)),
              what=f"rtgb_default_rig({scene_name})")
    return rig


def orbit_rig(rig: abi.CameraRig, degrees: float, center=(0.0, 0.0, 0.0)) -> abi.CameraRig:
    """A copy of `rig` with every camera pose turned by `degrees` about the
    vertical (+y) axis through `center`: R' = Ry R, t' = Ry (t - c) + c (the
    pose rotation's columns are the camera axes in world space)."""
    out = abi.CameraRig()
    C.pointer(out)[0] = rig
    a = np.radians(degrees)
    ry = np.array([[np.cos(a), 0.0, np.sin(a)], [0.0, 1.0, 0.0], [-np.sin(a), 0.0, np.cos(a)]])
    c = np.asarray(center, np.float64)
    for i in range(rig.active_count):
        cam = out.cameras[i]
        r = np.array(cam.rotation[:], np.float64).reshape(3, 3)
        t = np.array(cam.translation[:], np.float64)
        cam.rotation[:] = (ry @ r).ravel().tolist()
        cam.translation[:] = (ry @ (t - c) + c).tolist()
    return out


def profile(name: str, **overrides) -> abi.RenderProfile:
    p = abi.RenderProfile()
    abi.check(abi.load().rtgb_profile_preset(name.encode(), C.byref(p)), what=f"rtgb_profile_preset({name})")
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def restir_acceptance_profile(spp: int, restir: bool, spatial_neighbors: int = 1) -> abi.RenderProfile:
    """make_profile of utils/render_restir_acceptance.cpp:101-118."""
    return profile("realtime", samples_per_pixel=spp, max_bounces=1, rr_start_bounce=2, enable_denoise=0,
                   enable_restir_di=int(restir), restir_initial_candidates=8, restir_temporal_reuse=int(restir),
                   restir_max_history_age=20, restir_max_temporal_candidates=64,
                   restir_spatial_neighbors=spatial_neighbors if restir else 0, restir_max_spatial_candidates=8,
                   restir_bias_correction=1, restir_min_analytic_lights=16)


def display_u8(linear: np.ndarray) -> np.ndarray:
    """display_channel of utils/render_restir_acceptance.cpp:149-153 (Reinhard, sqrt, lround)."""
    x = np.maximum(linear.astype(np.float32), np.float32(0.0))
    mapped = x / (np.float32(1.0) + x)
    enc = np.sqrt(mapped)
    v = np.float32(255.0) * np.minimum(enc, np.float32(1.0))
    # lround of the float product: half away from zero (values are non-negative)
    return np.floor(v.astype(np.float64) + 0.5).astype(np.uint8)
