"""ctypes binding of the CPU oracle (``oracle/_bin/liborc.so``) — TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
``cpu_baseline`` / ``--impl reference`` legs import this module; the product
(``ray_tracing_gb300``) never does.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ray_tracing_gb300 import abi
from ray_tracing_gb300 import build as _build

P = C.POINTER
_lib = None

_SIGS = {
    "orc_create": (C.c_void_p, [P(abi.Scene), C.c_int, C.c_int]),
    "orc_destroy": (None, [C.c_void_p]),
    "orc_reset_sequence": (None, [C.c_void_p, C.c_uint32]),
    "orc_reset_accumulation": (None, [C.c_void_p]),
    "orc_set_path_records": (None, [C.c_void_p, C.c_int]),
    "orc_sample_stream": (C.c_uint32, [C.c_void_p]),
    "orc_light_table": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "orc_render_frame": (C.c_int, [C.c_void_p, P(abi.CameraRig), P(abi.RenderProfile), C.c_int, C.c_int, C.c_int,
                                   C.c_int]),
    "orc_get_buffer": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_size_t]),
    "orc_get_path_records": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int64]),
    "orc_last_rays": (C.c_uint64, [C.c_void_p, C.c_int]),
    "orc_direction_debug": (C.c_int, [P(abi.Camera), C.c_void_p]),
    "orc_unproject": (None, [P(abi.Camera), C.c_double, C.c_double, P(C.c_float)]),
    "orc_noise_sinf": (C.c_float, [C.c_float]),
    "orc_project": (None, [P(abi.Camera), P(C.c_float), P(C.c_float)]),
    "orc_reservoir_update": (C.c_int, [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                       C.c_float]),
    "orc_reservoir_finalize": (None, [C.c_void_p]),
    "orc_reservoir_finalize_basic": (None, [C.c_void_p, C.c_float, C.c_float, C.c_int]),
    "orc_reservoir_merge": (None, [C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_float, C.c_int, P(C.c_int)]),
    "orc_surface_valid": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_int]),
    "orc_uniform_cone_pdf": (C.c_float, [C.c_float]),
    "orc_area_pdf": (C.c_float, [C.c_float, C.c_float, C.c_float]),
    "orc_power_heuristic": (C.c_float, [C.c_float, C.c_float]),
    "orc_sample_cdf": (C.c_int, [P(C.c_float), C.c_int, C.c_float]),
    "orc_rng_for": (C.c_uint32, [C.c_int, C.c_int, C.c_uint32]),
    "orc_rnd": (C.c_float, [P(C.c_uint32)]),
}


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.ORACLE_LIB
        if not path.exists():
            _build.build_oracle()
        lib = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


BUFFERS = {"beauty": (0, 4), "normal": (1, 4), "denoiser_normal": (2, 4), "albedo": (3, 4), "depth": (4, 1),
           "flow": (5, 2), "flow_trustworthiness": (6, 1)}


class OracleRenderer:
    """CPU restatement of the reference renderer (one state per camera slot)."""

    def __init__(self, scene: abi.Scene, use_reference_bvh: bool = True, threads: int = 0):
        self.lib = load()
        self._scene = scene
        self.h = self.lib.orc_create(C.byref(scene), int(use_reference_bvh), int(threads))
        if not self.h:
            raise RuntimeError("orc_create failed")
        self.sizes: dict[int, tuple[int, int]] = {}

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def reset_sequence(self, stream: int):
        self.lib.orc_reset_sequence(self.h, stream)

    def reset_accumulation(self):
        self.lib.orc_reset_accumulation(self.h)

    def set_path_records(self, on: bool):
        self.lib.orc_set_path_records(self.h, int(on))

    def render_frame(self, rig: abi.CameraRig, profile: abi.RenderProfile, active: int, rows=None, row_stride=1):
        """Renders every active camera; `rows` = (first, end) restricts to a band, `row_stride` samples it."""
        y0, y1 = rows if rows else (0, 0)
        if row_stride > 1 and not rows:
            y0, y1 = 0, 1 << 30
        st = self.lib.orc_render_frame(self.h, C.byref(rig), C.byref(profile), active, y0, y1, row_stride)
        if st != 0:
            raise RuntimeError(f"orc_render_frame status {st}")
        for i in range(active):
            self.sizes[i] = (rig.cameras[i].width, rig.cameras[i].height)

    def buffer(self, cam: int, name: str) -> np.ndarray:
        which, ch = BUFFERS[name]
        w, h = self.sizes[cam]
        out = np.zeros((h, w, ch) if ch > 1 else (h, w), dtype=np.float32)
        st = self.lib.orc_get_buffer(self.h, cam, which, out.ctypes.data, out.nbytes)
        if st != 0:
            raise RuntimeError("orc_get_buffer failed")
        return out

    def light_table(self) -> np.ndarray:
        """build_light_distribution's PackedLight records (abi.LIGHT_DTYPE)."""
        n = self.lib.orc_light_table(self.h, None, 0)
        out = np.zeros(n, dtype=abi.LIGHT_DTYPE)
        self.lib.orc_light_table(self.h, out.ctypes.data if n else None, n)
        return out

    def reservoirs(self, cam: int) -> np.ndarray:
        w, h = self.sizes[cam]
        out = np.zeros(w * h, dtype=abi.RESERVOIR_DTYPE)
        st = self.lib.orc_get_buffer(self.h, cam, 7, out.ctypes.data, out.nbytes)
        if st != 0:
            raise RuntimeError("orc_get_buffer(reservoirs) failed")
        return out

    def path_records(self, cam: int, spp: int, max_bounces: int):
        w, h = self.sizes[cam]
        paths = w * h * spp
        codes = np.zeros((paths, max_bounces), dtype=np.int32)
        rad = np.zeros((paths, 3), dtype=np.float32)
        st = self.lib.orc_get_path_records(self.h, cam, codes.ctypes.data, max_bounces, rad.ctypes.data, paths)
        if st != 0:
            raise RuntimeError("orc_get_path_records failed")
        return codes, rad

    def rays(self, cam: int) -> int:
        return int(self.lib.orc_last_rays(self.h, cam))
