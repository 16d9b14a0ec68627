"""Shared helpers for the parity tests (GPU path vs the CPU oracle)."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ray_tracing_gb300 import abi, scenes


def look_at(cam: abi.Camera, eye, target, up):
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    fwd = target - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    for r in range(3):
        cam.rotation[r * 3 + 0] = right[r]
        cam.rotation[r * 3 + 1] = down[r]
        cam.rotation[r * 3 + 2] = fwd[r]
        cam.translation[r] = eye[r]


def pinhole(w, h, hfov_deg, k=(0.0, 0.0, 0.0), p=(0.0, 0.0)) -> abi.Camera:
    c = abi.Camera()
    c.enabled, c.width, c.height, c.model = 1, w, h, 0
    f = 0.5 * w / math.tan(0.5 * math.radians(hfov_deg))
    c.pinhole = abi.Pinhole32(f, f, 0.5 * w, 0.5 * h, k[0], k[1], k[2], p[0], p[1])
    return c


def equi(w, h, fov_deg, radial=(0.0,) * 6, tangential=(0.0, 0.0)) -> abi.Camera:
    c = abi.Camera()
    c.enabled, c.width, c.height, c.model = 1, w, h, 1
    f = 0.5 * w / (0.5 * math.radians(fov_deg))
    rad = (C.c_double * 6)(*radial)
    tan = (C.c_double * 2)(*tangential)
    abi.check(abi.load().rtgb_make_equi62_lut1d(w, h, f, f, 0.5 * w, 0.5 * h, rad, tan, C.byref(c.equi)),
              what="rtgb_make_equi62_lut1d")
    return c


def rig_of(*cams) -> abi.CameraRig:
    rig = abi.CameraRig()
    rig.active_count = len(cams)
    for i, c in enumerate(cams):
        rig.cameras[i] = c
    return rig


def scaled_rig(rig: abi.CameraRig, scale: float) -> abi.CameraRig:
    """Same poses, resolution scaled (pinhole intrinsics scaled; equi LUT rebuilt)."""
    out = abi.CameraRig()
    out.active_count = rig.active_count
    for i in range(rig.active_count):
        src = rig.cameras[i]
        w, h = max(8, int(src.width * scale)), max(8, int(src.height * scale))
        if src.model == 0:
            c = abi.Camera()
            C.memmove(C.byref(c), C.byref(src), C.sizeof(abi.Camera))
            c.width, c.height = w, h
            s = w / src.width
            c.pinhole.fx, c.pinhole.fy = src.pinhole.fx * s, src.pinhole.fy * s
            c.pinhole.cx, c.pinhole.cy = 0.5 * w, 0.5 * h
        else:
            fov = math.degrees(src.width / src.equi.fx)
            c = equi(w, h, fov)
            for k in range(9):
                c.rotation[k] = src.rotation[k]
            for k in range(3):
                c.translation[k] = src.translation[k]
        out.cameras[i] = c
    return out


def compare_paths(gc, gr, oc, orad, rel=1e-4, floor=1e-6):
    """Hit-code identity per path and radiance agreement on identical paths.

    Returns (fraction of paths whose hit codes differ, max relative error over
    identical paths, number of identical paths over tolerance)."""
    same = np.all(gc == oc, axis=1)
    diverged = 1.0 - float(same.mean())
    g = gr[same].astype(np.float64)
    o = orad[same].astype(np.float64)
    err = np.abs(g - o) / np.maximum(np.abs(o), floor)
    bad = int(np.sum(np.any(np.abs(g - o) > rel * np.maximum(np.abs(o), floor), axis=1)))
    return diverged, float(err.max() if err.size else 0.0), bad


def render_both(scene_name, rig, profile, frames=1, seed=0, detail=0, oracle_bvh=False, active=None, records=True,
                scene=None):
    """Renders `frames` frames with the GPU path and the oracle; returns both.
    `scene` (a HostScene) replaces the builtin scene of `scene_name`."""
    from oracle.binding import OracleRenderer
    from ray_tracing_gb300.renderer import Renderer

    sc = scene if scene is not None else scenes.HostScene(scene_name, seed=seed, detail=detail)
    active = active or rig.active_count
    gpu = Renderer(debug_path_records=records)
    gpu.prepare_scene(sc.view)
    orc = OracleRenderer(sc.view, use_reference_bvh=oracle_bvh)
    orc.set_path_records(records)
    for _ in range(frames):
        gpu.render_frame(rig, profile, active)
        orc.render_frame(rig, profile, active)
    return sc, gpu, orc
