"""Python mirror of the reference's renderer surface over the C ABI.

``Renderer`` follows ``RendererPool`` / ``OptixRenderer``
(src/realtime/gpu/renderer_pool.h:30-53, optix_renderer.h:69-128):
``prepare_scene``, ``reset_sequence``, ``reset_accumulation``,
``render_frame`` (all active cameras, one launch sequence), per-camera
downloads, ``restir_diagnostics`` and ``render_direction_debug``. Errors come
back as :class:`abi.RtgbError` carrying the library's message — the
exceptions the reference throws.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


@dataclass
class CameraFrame:
    """RadianceFrame of src/realtime/gpu/frame_types.h:14-22 (host arrays)."""
    camera_index: int
    width: int
    height: int
    beauty_rgba: np.ndarray
    normal_rgba: np.ndarray
    albedo_rgba: np.ndarray
    depth: np.ndarray
    render_ms: float
    download_ms: float

    @property
    def average_luminance(self) -> float:
        b = self.beauty_rgba.astype(np.float64)
        return float(np.mean(0.2126 * b[..., 0] + 0.7152 * b[..., 1] + 0.0722 * b[..., 2]))


class Renderer:
    def __init__(self, device: int = 0, use_cuda_graph: bool = True, debug_path_records: bool = False,
                 stage_timing: bool = False, shade_order: int = 0, debug_traversal_limit: int = 0,
                 debug_rejection_limit: int = 0):
        self.lib = abi.load()
        missing = getattr(self.lib, "rtgb_missing_symbols", [])
        if missing:
            raise RuntimeError(f"librtgb.so lacks {missing}: rebuild with __graft_entry__.build()")
        self.h = C.c_void_p()
        info = abi.CreateInfo(device, int(use_cuda_graph), int(debug_path_records), int(stage_timing), int(shade_order),
                              int(debug_traversal_limit), int(debug_rejection_limit))
        st = self.lib.rtgb_create(C.byref(info), C.byref(self.h))
        if st != abi.OK:
            raise abi.RtgbError(st, "rtgb_create failed (no CUDA device?)")
        self.last_views: abi.FrameViews | None = None
        self._scene_ref = None

    def close(self):
        if self.h:
            self.lib.rtgb_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self) -> "Renderer":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def _check(self, st, what):
        abi.check(st, self.h, what)

    def prepare_scene(self, scene: abi.Scene) -> None:
        self._check(self.lib.rtgb_prepare_scene(self.h, C.byref(scene)), "prepare_scene")
        self._scene_ref = scene

    def prepare_scene_instanced(self, scene: abi.Scene, meshes: abi.MeshSet) -> None:
        """rtgb_prepare_scene_instanced: the scene plus `meshes`' instances
        flattened into triangles on the device."""
        self._check(self.lib.rtgb_prepare_scene_instanced(self.h, C.byref(scene), C.byref(meshes)),
                    "prepare_scene_instanced")
        self._scene_ref = scene

    def triangles(self) -> np.ndarray:
        """rtgb_download_triangles: the device triangle array, one row of raw
        rtgb_triangle bytes (abi.Triangle's layout) per triangle."""
        n = C.c_int32()
        self._check(self.lib.rtgb_download_triangles(self.h, None, 0, C.byref(n)), "download_triangles")
        out = (abi.Triangle * max(1, n.value))()
        self._check(self.lib.rtgb_download_triangles(self.h, out, n.value, C.byref(n)), "download_triangles")
        return np.frombuffer(out, dtype=np.uint8, count=n.value * C.sizeof(abi.Triangle)).reshape(n.value, -1)

    def reset_sequence(self, sample_stream: int) -> None:
        self._check(self.lib.rtgb_reset_sequence(self.h, sample_stream), "reset_sequence")

    def reset_accumulation(self) -> None:
        self._check(self.lib.rtgb_reset_accumulation(self.h), "reset_accumulation")

    def render_frame(self, rig: abi.CameraRig, profile: abi.RenderProfile, active: int) -> abi.FrameViews:
        views = abi.FrameViews()
        self._check(self.lib.rtgb_render_frame(self.h, C.byref(rig), C.byref(profile), active, C.byref(views)),
                    "render_frame")
        self.last_views = views
        return views

    def render_frame_async(self, rig: abi.CameraRig, profile: abi.RenderProfile, active: int) -> None:
        self._check(self.lib.rtgb_render_frame_async(self.h, C.byref(rig), C.byref(profile), active),
                    "render_frame_async")

    def frame_stats(self) -> abi.FrameViews:
        views = abi.FrameViews()
        self._check(self.lib.rtgb_frame_stats(self.h, C.byref(views)), "frame_stats")
        self.last_views = views
        return views

    def ray_totals(self) -> np.ndarray:
        out = (C.c_uint64 * 4)()
        self._check(self.lib.rtgb_ray_totals(self.h, out), "ray_totals")
        return np.array(list(out), dtype=np.uint64)

    def stage_times(self) -> np.ndarray:
        """Per-launch device ms of the last frame: raygen, (trace, shade, shadow) per bounce, finalize, resolve."""
        buf = (C.c_float * 256)()
        n = C.c_int32()
        self._check(self.lib.rtgb_stage_times(self.h, buf, 256, C.byref(n)), "stage_times")
        return np.array(buf[: n.value], dtype=np.float64)

    def set_debug_limits(self, traversal_limit: int = 0, rejection_limit: int = 0) -> None:
        """rtgb_set_debug_limits: loop bounds of later frames (0 = default)."""
        self._check(self.lib.rtgb_set_debug_limits(self.h, traversal_limit, rejection_limit), "set_debug_limits")

    def launch_grids(self) -> list[tuple[int, int]]:
        """rtgb_launch_grids: (grid, block) of every wavefront launch slot in use."""
        grids = (C.c_int32 * 64)()
        blocks = (C.c_int32 * 64)()
        n = C.c_int32()
        self._check(self.lib.rtgb_launch_grids(self.h, grids, blocks, 64, C.byref(n)), "launch_grids")
        return list(zip(list(grids)[: n.value], list(blocks)[: n.value]))

    def autotune_launches(self, rig: abi.CameraRig, profile: abi.RenderProfile, active: int,
                          frames: int = 4) -> dict:
        """rtgb_autotune_launches: picks the fastest grid scale per stage group
        for this rig and profile; returns the measured table and the choice."""
        t = abi.LaunchTuning()
        self._check(self.lib.rtgb_autotune_launches(self.h, C.byref(rig), C.byref(profile), active, frames,
                                                    C.byref(t)), "autotune_launches")
        cands = [{"grid_scale": float(t.scales[c]), "block": "half" if t.block_halved[c] else "kernel's"}
                 for c in range(abi.TUNE_CANDIDATES)]
        return {"candidates": cands,
                "group_ms": {abi.TUNE_GROUP_NAMES[g]: [round(t.group_ms[c][g], 4) for c in range(abi.TUNE_CANDIDATES)]
                             for g in range(abi.TUNE_GROUPS)},
                "frame_ms": [round(x, 4) for x in t.frame_ms],
                "chosen": {abi.TUNE_GROUP_NAMES[g]: cands[t.chosen[g]] for g in range(abi.TUNE_GROUPS)},
                "tuned_frame_ms": round(t.tuned_frame_ms, 4)}

    def stream_ptr(self) -> int:
        return int(self.lib.rtgb_stream(self.h) or 0)

    def _size(self, cam: int) -> tuple[int, int]:
        v = self.last_views
        if v is None or cam >= v.camera_count:
            raise abi.RtgbError(1, f"camera_index out of range: {cam}")
        return v.cameras[cam].width, v.cameras[cam].height

    def download(self, cam: int) -> CameraFrame:
        w, h = self._size(cam)
        beauty = np.empty((h, w, 4), np.float32)
        normal = np.empty((h, w, 4), np.float32)
        albedo = np.empty((h, w, 4), np.float32)
        depth = np.empty((h, w), np.float32)
        ms = C.c_float()
        self._check(self.lib.rtgb_download_frame(self.h, cam, beauty.ctypes.data, normal.ctypes.data,
                                                 albedo.ctypes.data, depth.ctypes.data, C.byref(ms)), "download")
        return CameraFrame(cam, w, h, beauty, normal, albedo, depth, self.last_views.cameras[cam].render_ms,
                           ms.value)

    @staticmethod
    def _host_ptr(buf):
        if buf is None:
            return None
        if isinstance(buf, int):
            return buf
        if isinstance(buf, np.ndarray):
            return buf.ctypes.data
        return int(buf.data_ptr())  # a torch CPU tensor (pinned for overlap)

    def download_async(self, cam: int, beauty=None, normal=None, albedo=None, depth=None) -> None:
        """rtgb_download_frame_async: enqueues the last frame's copies into the
        given host buffers (numpy arrays, torch CPU tensors or addresses) and
        returns; the buffers are filled once wait_downloads returns."""
        self._check(self.lib.rtgb_download_frame_async(self.h, cam, self._host_ptr(beauty), self._host_ptr(normal),
                                                       self._host_ptr(albedo), self._host_ptr(depth)),
                    "download_frame_async")

    def wait_downloads(self, keep_latest: bool = False) -> None:
        """rtgb_wait_downloads: all asynchronous downloads done, or all but the
        latest frame's."""
        self._check(self.lib.rtgb_wait_downloads(self.h, 1 if keep_latest else 0), "wait_downloads")

    def light_table(self) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
        """rtgb_download_light_table: the device-built PackedLight records
        (abi.LIGHT_DTYPE) and the sphere / quad / triangle -> light maps."""
        n = C.c_int32()
        self._check(self.lib.rtgb_download_light_table(self.h, None, 0, C.byref(n), None, None, None),
                    "download_light_table")
        sc = self._scene_ref
        tris = C.c_int32()  # the scene's triangles and any flattened instances
        self._check(self.lib.rtgb_download_triangles(self.h, None, 0, C.byref(tris)), "download_triangles")
        lights = np.zeros(n.value, dtype=abi.LIGHT_DTYPE)
        maps = [np.zeros(k, dtype=np.int32) for k in (sc.sphere_count, sc.quad_count, tris.value)]
        ptr = [m.ctypes.data if m.size else None for m in maps]
        self._check(self.lib.rtgb_download_light_table(self.h, lights.ctypes.data if n.value else None, n.value,
                                                       C.byref(n), *ptr), "download_light_table")
        return lights, maps[0], maps[1], maps[2]

    BUFFERS = {"beauty": (0, 4), "normal": (1, 4), "denoiser_normal": (2, 4), "albedo": (3, 4), "depth": (4, 1),
               "flow": (5, 2), "flow_trustworthiness": (6, 1), "denoised": (8, 4)}

    def set_denoiser(self, params) -> None:
        """Loads the U-Net parameters (flat float32, layer order; None clears them)."""
        if params is None:
            self._check(self.lib.rtgb_set_denoiser_params(self.h, None, 0), "set_denoiser_params")
            self._denoiser_params = None
            return
        arr = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.lib.rtgb_set_denoiser_params(self.h, arr.ctypes.data, arr.size), "set_denoiser_params")
        self._denoiser_params = arr

    def buffer(self, cam: int, name: str) -> np.ndarray:
        which, ch = self.BUFFERS[name]
        w, h = self._size(cam)
        out = np.empty((h, w, ch) if ch > 1 else (h, w), np.float32)
        self._check(self.lib.rtgb_download_buffer(self.h, cam, which, out.ctypes.data, out.nbytes), "download_buffer")
        return out

    def reservoirs(self, cam: int) -> np.ndarray:
        w, h = self._size(cam)
        out = np.zeros(w * h, dtype=abi.RESERVOIR_DTYPE)
        self._check(self.lib.rtgb_download_reservoirs(self.h, cam, out.ctypes.data, out.nbytes), "reservoirs")
        return out

    def restir_diagnostics(self, cam: int) -> abi.RestirDiagnostics:
        d = abi.RestirDiagnostics()
        self._check(self.lib.rtgb_restir_diagnostics(self.h, cam, C.byref(d)), "restir_diagnostics")
        return d

    def path_records(self, cam: int, spp: int, max_bounces: int):
        w, h = self._size(cam)
        paths = w * h * spp
        codes = np.empty((paths, max_bounces), np.int32)
        rad = np.empty((paths, 3), np.float32)
        self._check(self.lib.rtgb_download_path_records(self.h, cam, codes.ctypes.data, max_bounces,
                                                        rad.ctypes.data, paths), "path_records")
        return codes, rad

    def render_direction_debug(self, rig: abi.CameraRig, cam: int) -> np.ndarray:
        c = rig.cameras[cam]
        out = np.empty((c.height, c.width, 4), np.uint8)
        self._check(self.lib.rtgb_render_direction_debug(self.h, C.byref(rig), cam, out.ctypes.data),
                    "render_direction_debug")
        return out

    def tonemap_rgba8(self, cam: int) -> np.ndarray:
        w, h = self._size(cam)
        out = np.empty((h, w, 4), np.uint8)
        self._check(self.lib.rtgb_tonemap_rgba8(self.h, cam, out.ctypes.data), "tonemap")
        return out

    def acceleration_info(self) -> abi.AccelerationInfo:
        a = abi.AccelerationInfo()
        self._check(self.lib.rtgb_acceleration_info_get(self.h, C.byref(a)), "acceleration_info")
        return a

    def lbvh(self):
        n = self.acceleration_info().primitive_count
        keys = np.empty(n, np.uint32)
        order = np.empty(n, np.int32)
        children = np.empty((max(n - 1, 0), 2), np.int32)
        self._check(self.lib.rtgb_download_lbvh(self.h, keys.ctypes.data, order.ctypes.data, children.ctypes.data),
                    "download_lbvh")
        return keys, order, children

    def bvh4(self):
        """(children (nodes, 4) int32, boxes (nodes, 2, 3, 4) float32: lo/hi, axis, child)."""
        n = self.acceleration_info().wide_node_count
        children = np.empty((n, 4), np.int32)
        boxes = np.empty((n, 2, 3, 4), np.float32)
        self._check(self.lib.rtgb_download_bvh4(self.h, children.ctypes.data, boxes.ctypes.data), "download_bvh4")
        return children, boxes

    def lbvh_boxes(self) -> np.ndarray:
        """(nodes, 2, 2, 3): per internal node the left and right child's (lo, hi) box."""
        n = self.acceleration_info().primitive_count
        boxes = np.empty((max(n - 1, 0), 2, 2, 3), np.float32)
        self._check(self.lib.rtgb_download_lbvh_boxes(self.h, boxes.ctypes.data), "download_lbvh_boxes")
        return boxes
