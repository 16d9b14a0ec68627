"""ctypes mirror of ``include/rtgb.h`` (the C ABI of the sm_103a path tracer).

The structures below must match the header field for field; ``tests/``
checks every exported symbol and the structure sizes against the library.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

MAX_CAMERAS = 4
EQUI_LUT_SIZE = 1024

OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARGUMENT", 2: "RUNTIME_ERROR", 3: "NOT_PREPARED",
                4: "DEVICE_FAULT_FLAG", 5: "UNSUPPORTED"}

f3 = C.c_float * 3


class Texture(C.Structure):
    _fields_ = [("type", C.c_int32), ("even_texture", C.c_int32), ("odd_texture", C.c_int32),
                ("image_offset", C.c_int32), ("image_width", C.c_int32), ("image_height", C.c_int32),
                ("u_address_mode", C.c_int32), ("v_address_mode", C.c_int32), ("filter_type", C.c_int32),
                ("scale", C.c_float), ("color", f3)]


class Material(C.Structure):
    _fields_ = [("albedo_texture", C.c_int32), ("emission_texture", C.c_int32), ("ior", C.c_float),
                ("fuzz", C.c_float), ("type", C.c_int32), ("openpbr_index", C.c_int32)]


OPENPBR_PARAMS = [
    ("base_weight", 1), ("base_color", 3), ("base_diffuse_roughness", 1), ("base_metalness", 1),
    ("specular_weight", 1), ("specular_color", 3), ("specular_roughness", 1), ("specular_ior", 1),
    ("specular_roughness_anisotropy", 1), ("transmission_weight", 1), ("transmission_color", 3),
    ("transmission_depth", 1), ("transmission_dispersion_scale", 1), ("transmission_dispersion_abbe_number", 1),
    ("subsurface_weight", 1), ("subsurface_color", 3), ("subsurface_radius", 1), ("subsurface_radius_scale", 3),
    ("subsurface_scatter_anisotropy", 1), ("fuzz_weight", 1), ("fuzz_color", 3), ("fuzz_roughness", 1),
    ("coat_weight", 1), ("coat_color", 3), ("coat_roughness", 1), ("coat_roughness_anisotropy", 1),
    ("coat_ior", 1), ("coat_darkening", 1), ("thin_film_weight", 1), ("thin_film_thickness", 1),
    ("thin_film_ior", 1), ("emission_luminance", 1), ("emission_color", 3), ("geometry_opacity", 1),
]

# OpenPbrCoreMaterial defaults (src/common/openpbr_core.h:33-77)
OPENPBR_DEFAULTS = {
    "base_weight": 1.0, "base_color": (0.8, 0.8, 0.8), "base_diffuse_roughness": 0.0, "base_metalness": 0.0,
    "specular_weight": 1.0, "specular_color": (1.0, 1.0, 1.0), "specular_roughness": 0.3, "specular_ior": 1.5,
    "specular_roughness_anisotropy": 0.0, "transmission_weight": 0.0, "transmission_color": (1.0, 1.0, 1.0),
    "transmission_depth": 0.0, "transmission_dispersion_scale": 0.0, "transmission_dispersion_abbe_number": 20.0,
    "subsurface_weight": 0.0, "subsurface_color": (0.8, 0.8, 0.8), "subsurface_radius": 1.0,
    "subsurface_radius_scale": (1.0, 0.5, 0.25), "subsurface_scatter_anisotropy": 0.0, "fuzz_weight": 0.0,
    "fuzz_color": (1.0, 1.0, 1.0), "fuzz_roughness": 0.5, "coat_weight": 0.0, "coat_color": (1.0, 1.0, 1.0),
    "coat_roughness": 0.0, "coat_roughness_anisotropy": 0.0, "coat_ior": 1.6, "coat_darkening": 1.0,
    "thin_film_weight": 0.0, "thin_film_thickness": 0.5, "thin_film_ior": 1.4, "emission_luminance": 0.0,
    "emission_color": (1.0, 1.0, 1.0), "geometry_opacity": 1.0, "geometry_thin_walled": 0,
}


class OpenPbrMaterial(C.Structure):
    _fields_ = ([(n, C.c_float if k == 1 else f3) for n, k in OPENPBR_PARAMS]
                + [("geometry_thin_walled", C.c_int32), ("color_texture", C.c_int32 * 4),
                   ("color_space", C.c_int32 * 4), ("scalar_texture", C.c_int32 * 2)])

    @classmethod
    def make(cls, **kw) -> "OpenPbrMaterial":
        """Material with the reference defaults, overridden by `kw`; all textures unbound."""
        m = cls()
        vals = dict(OPENPBR_DEFAULTS)
        vals.update(kw)
        for name, value in vals.items():
            if name in ("color_texture", "color_space", "scalar_texture"):
                continue
            if isinstance(value, (tuple, list)):
                getattr(m, name)[:] = [float(v) for v in value]
            else:
                setattr(m, name, value)
        m.color_texture[:] = list(kw.get("color_texture", (-1, -1, -1, -1)))
        m.color_space[:] = list(kw.get("color_space", (1, 1, 1, 1)))
        m.scalar_texture[:] = list(kw.get("scalar_texture", (-1, -1)))
        return m


class DeviceInfo(C.Structure):
    _fields_ = [("name", C.c_char * 256), ("device", C.c_int32), ("major", C.c_int32), ("minor", C.c_int32),
                ("multiprocessors", C.c_int32), ("driver_version", C.c_int32), ("runtime_version", C.c_int32),
                ("total_bytes", C.c_uint64), ("used_bytes", C.c_uint64)]


class Sphere(C.Structure):
    _fields_ = [("center", f3), ("radius", C.c_float), ("material_index", C.c_int32)]


class Quad(C.Structure):
    _fields_ = [("origin", f3), ("edge_u", f3), ("edge_v", f3), ("material_index", C.c_int32)]


class Triangle(C.Structure):
    _fields_ = [("p0", f3), ("p1", f3), ("p2", f3), ("n0", f3), ("n1", f3), ("n2", f3),
                ("uv0", C.c_float * 2), ("uv1", C.c_float * 2), ("uv2", C.c_float * 2),
                ("material_index", C.c_int32), ("has_vertex_normals", C.c_int32), ("has_texcoords", C.c_int32)]


class Medium(C.Structure):
    _fields_ = [("local_center_or_min", f3), ("radius", C.c_float), ("local_max", f3), ("density", C.c_float),
                ("rotation_row0", f3), ("rotation_row1", f3), ("rotation_row2", f3), ("translation", f3),
                ("material_index", C.c_int32), ("boundary_type", C.c_int32)]


class AnalyticLight(C.Structure):
    _fields_ = [("type", C.c_int32), ("position", f3), ("basis_x", f3), ("basis_y", f3), ("basis_z", f3),
                ("radiance", f3), ("radius", C.c_float), ("width", C.c_float), ("height", C.c_float),
                ("length", C.c_float), ("world_area", C.c_float), ("cos_theta_max", C.c_float),
                ("selection_pdf", C.c_float), ("cdf", C.c_float), ("delta", C.c_int32),
                ("treat_as_point", C.c_int32), ("treat_as_line", C.c_int32)]


class Scene(C.Structure):
    _fields_ = [("textures", C.POINTER(Texture)), ("texture_count", C.c_int32),
                ("image_texels", C.POINTER(C.c_float)), ("image_texel_count", C.c_int32),
                ("materials", C.POINTER(Material)), ("material_count", C.c_int32),
                ("spheres", C.POINTER(Sphere)), ("sphere_count", C.c_int32),
                ("quads", C.POINTER(Quad)), ("quad_count", C.c_int32),
                ("triangles", C.POINTER(Triangle)), ("triangle_count", C.c_int32),
                ("media", C.POINTER(Medium)), ("medium_count", C.c_int32),
                ("analytic_lights", C.POINTER(AnalyticLight)), ("analytic_light_count", C.c_int32),
                ("background", f3),
                ("openpbr_materials", C.POINTER(OpenPbrMaterial)), ("openpbr_material_count", C.c_int32)]


INSTANCE_MATERIAL = -2147483648  # RTGB_INSTANCE_MATERIAL


class MeshPrototype(C.Structure):
    _fields_ = [("points", C.POINTER(C.c_double)), ("point_count", C.c_int32), ("triangle_count", C.c_int32),
                ("corner_points", C.POINTER(C.c_int32)), ("corner_normals", C.POINTER(C.c_double)),
                ("corner_texcoords", C.POINTER(C.c_double)), ("triangle_materials", C.POINTER(C.c_int32))]


class MeshInstance(C.Structure):
    _fields_ = [("prototype", C.c_int32), ("material", C.c_int32), ("flip_winding", C.c_int32),
                ("reserved", C.c_int32), ("world", C.c_double * 12), ("normal_matrix", C.c_double * 9)]


class MeshSet(C.Structure):
    _fields_ = [("prototypes", C.POINTER(MeshPrototype)), ("prototype_count", C.c_int32),
                ("instances", C.POINTER(MeshInstance)), ("instance_count", C.c_int32)]


class Pinhole32(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("fx", "fy", "cx", "cy", "k1", "k2", "k3", "p1", "p2")]


class Equi62Lut1d(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fx", C.c_double), ("fy", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("radial", C.c_double * 6),
                ("tangential", C.c_double * 2), ("lut", C.c_double * EQUI_LUT_SIZE), ("lut_step", C.c_double)]


class Camera(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("width", C.c_int32), ("height", C.c_int32), ("model", C.c_int32),
                ("rotation", C.c_double * 9), ("translation", C.c_double * 3),
                ("pinhole", Pinhole32), ("equi", Equi62Lut1d)]


class CameraRig(C.Structure):
    _fields_ = [("active_count", C.c_int32), ("cameras", Camera * MAX_CAMERAS)]


class RenderProfile(C.Structure):
    _fields_ = [("samples_per_pixel", C.c_int32), ("max_bounces", C.c_int32), ("enable_denoise", C.c_int32),
                ("rr_start_bounce", C.c_int32), ("accumulation_reset_rotation_deg", C.c_double),
                ("accumulation_reset_translation", C.c_double), ("enable_restir_di", C.c_int32),
                ("restir_initial_candidates", C.c_int32), ("restir_temporal_reuse", C.c_int32),
                ("restir_max_history_age", C.c_int32), ("restir_max_temporal_candidates", C.c_int32),
                ("restir_spatial_neighbors", C.c_int32), ("restir_max_spatial_candidates", C.c_int32),
                ("restir_bias_correction", C.c_int32), ("restir_min_analytic_lights", C.c_int32),
                ("restir_emissive", C.c_int32)]


class CreateInfo(C.Structure):
    _fields_ = [("device", C.c_int32), ("use_cuda_graph", C.c_int32), ("debug_path_records", C.c_int32),
                ("stage_timing", C.c_int32), ("shade_order", C.c_int32), ("debug_traversal_limit", C.c_int32),
                ("debug_rejection_limit", C.c_int32)]


class CameraFrameView(C.Structure):
    _fields_ = [("camera_index", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("beauty", C.c_void_p), ("normal", C.c_void_p), ("denoiser_normal", C.c_void_p),
                ("albedo", C.c_void_p), ("depth", C.c_void_p), ("flow", C.c_void_p),
                ("flow_trustworthiness", C.c_void_p), ("render_ms", C.c_float), ("denoise_ms", C.c_float),
                ("download_ms", C.c_float)]


class FrameViews(C.Structure):
    _fields_ = [("camera_count", C.c_int32), ("cameras", CameraFrameView * MAX_CAMERAS),
                ("frame_render_ms", C.c_float), ("sample_stream", C.c_uint32), ("rays_traced", C.c_uint64),
                ("primary_rays", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("restir_visibility_rays", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("active_paths", C.c_uint64 * 64), ("restir_pixels", C.c_uint64),
                ("shadow_per_bounce", C.c_uint64 * 64)]


TUNE_CANDIDATES = 8
TUNE_GROUPS = 5
TUNE_GROUP_NAMES = ("raygen", "trace", "shade", "shadow", "finalize+resolve")


class LaunchTuning(C.Structure):
    _fields_ = [("scales", C.c_float * TUNE_CANDIDATES), ("block_halved", C.c_int32 * TUNE_CANDIDATES),
                ("group_ms", (C.c_float * TUNE_GROUPS) * TUNE_CANDIDATES),
                ("frame_ms", C.c_float * TUNE_CANDIDATES), ("chosen", C.c_int32 * TUNE_GROUPS),
                ("tuned_frame_ms", C.c_float)]


class RestirDiagnostics(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("pixel_count", "active_reservoir_count", "temporal_reuse_count",
                                         "spatial_reuse_count", "bias_corrected_count", "max_candidate_count",
                                         "max_age")]


class AccelerationInfo(C.Structure):
    _fields_ = [("primitive_count", C.c_int32), ("node_count", C.c_int32),
                ("analytic_light_node_count", C.c_int32), ("analytic_bvh_light_count", C.c_int32),
                ("build_ms", C.c_float), ("traversal_stack_overflows", C.c_int32),
                ("update_kind", C.c_int32), ("generation", C.c_int32), ("wide_node_count", C.c_int32)]

# AccelerationUpdateKind (gpu_scene_acceleration.cpp:247-295)
UPDATE_KINDS = ("reuse", "update", "refit", "rebuild")


# 84-byte RestirReservoir (src/common/restir_di.h:36-48)
RESERVOIR_DTYPE = np.dtype([
    ("light_index", "<i4"), ("u0", "<f4"), ("u1", "<f4"),
    ("position", "<f4", 3), ("normal", "<f4", 3), ("material_type", "<i4"), ("primitive_type", "<i4"),
    ("primitive_index", "<i4"), ("weight_sum", "<f4"), ("selected_target", "<f4"), ("estimator_weight", "<f4"),
    ("candidate_count", "<i4"), ("temporal_candidate_count", "<i4"), ("spatial_candidate_count", "<i4"),
    ("bias_correction_source_count", "<i4"), ("age", "<i4"), ("valid", "<i4"),
])
assert RESERVOIR_DTYPE.itemsize == 84

# 16-byte PackedLight (src/common/light_sampling.h:15-27): type 0 sphere, 1 quad,
# 2 triangle, 3 environment
LIGHT_DTYPE = np.dtype([("type", "<i4"), ("primitive_index", "<i4"), ("selection_pdf", "<f4"), ("cdf", "<f4")])
assert LIGHT_DTYPE.itemsize == 16

Handle = C.c_void_p
P = C.POINTER

# name -> (restype, argtypes); every rtgb_* symbol declared in include/rtgb.h
SIGNATURES = {
    "rtgb_create": (C.c_int, [P(CreateInfo), P(Handle)]),
    "rtgb_destroy": (None, [Handle]),
    "rtgb_last_error": (C.c_char_p, [Handle]),
    "rtgb_prepare_scene": (C.c_int, [Handle, P(Scene)]),
    "rtgb_prepare_scene_instanced": (C.c_int, [Handle, P(Scene), P(MeshSet)]),
    "rtgb_download_triangles": (C.c_int, [Handle, C.c_void_p, C.c_int32, P(C.c_int32)]),
    "rtgb_reset_sequence": (C.c_int, [Handle, C.c_uint32]),
    "rtgb_reset_accumulation": (C.c_int, [Handle]),
    "rtgb_render_frame": (C.c_int, [Handle, P(CameraRig), P(RenderProfile), C.c_int32, P(FrameViews)]),
    "rtgb_render_frame_async": (C.c_int, [Handle, P(CameraRig), P(RenderProfile), C.c_int32]),
    "rtgb_frame_stats": (C.c_int, [Handle, P(FrameViews)]),
    "rtgb_ray_totals": (C.c_int, [Handle, P(C.c_uint64)]),
    "rtgb_stage_times": (C.c_int, [Handle, P(C.c_float), C.c_int32, P(C.c_int32)]),
    "rtgb_set_debug_limits": (C.c_int, [Handle, C.c_int32, C.c_int32]),
    "rtgb_launch_grids": (C.c_int, [Handle, P(C.c_int32), P(C.c_int32), C.c_int32, P(C.c_int32)]),
    "rtgb_download_frame": (C.c_int, [Handle, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      P(C.c_float)]),
    "rtgb_download_frame_async": (C.c_int, [Handle, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtgb_wait_downloads": (C.c_int, [Handle, C.c_int32]),
    "rtgb_download_light_table": (C.c_int, [Handle, C.c_void_p, C.c_int32, P(C.c_int32), C.c_void_p, C.c_void_p,
                                            C.c_void_p]),
    "rtgb_download_buffer": (C.c_int, [Handle, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t]),
    "rtgb_restir_diagnostics": (C.c_int, [Handle, C.c_int32, P(RestirDiagnostics)]),
    "rtgb_download_reservoirs": (C.c_int, [Handle, C.c_int32, C.c_void_p, C.c_size_t]),
    "rtgb_render_direction_debug": (C.c_int, [Handle, P(CameraRig), C.c_int32, C.c_void_p]),
    "rtgb_tonemap_rgba8": (C.c_int, [Handle, C.c_int32, C.c_void_p]),
    "rtgb_acceleration_info_get": (C.c_int, [Handle, P(AccelerationInfo)]),
    "rtgb_stream": (C.c_void_p, [Handle]),
    "rtgb_download_path_records": (C.c_int, [Handle, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                             C.c_int64]),
    "rtgb_download_lbvh": (C.c_int, [Handle, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtgb_download_lbvh_boxes": (C.c_int, [Handle, C.c_void_p]),
    "rtgb_download_bvh4": (C.c_int, [Handle, C.c_void_p, C.c_void_p]),
    "rtgb_trainer_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, P(C.c_void_p)]),
    "rtgb_trainer_destroy": (None, [C.c_void_p]),
    "rtgb_trainer_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, P(C.c_float)]),
    "rtgb_trainer_gradients": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rtgb_trainer_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rtgb_trainer_last_error": (C.c_char_p, [C.c_void_p]),
    "rtgb_conv3x3_wgrad_bf16": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                           C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_char_p, C.c_size_t]),
    "rtgb_host_scene_create": (C.c_int, [C.c_char_p, C.c_uint32, C.c_int64, P(C.c_void_p)]),
    "rtgb_host_scene_destroy": (None, [C.c_void_p]),
    "rtgb_host_scene_view": (C.c_int, [C.c_void_p, P(Scene)]),
    "rtgb_autotune_launches": (C.c_int, [Handle, P(CameraRig), P(RenderProfile), C.c_int32, C.c_int32,
                                         P(LaunchTuning)]),
    "rtgb_host_scene_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "rtgb_host_scene_load": (C.c_int, [C.c_char_p, P(C.c_void_p)]),
    "rtgb_host_scene_from_view": (C.c_int, [P(Scene), P(C.c_void_p)]),
    "rtgb_make_equi62_lut1d": (C.c_int, [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
                                         C.c_double, P(C.c_double), P(C.c_double), P(Equi62Lut1d)]),
    "rtgb_pack_camera_pose": (C.c_int, [P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double)]),
    "rtgb_default_rig": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, P(CameraRig)]),
    "rtgb_profile_preset": (C.c_int, [C.c_char_p, P(RenderProfile)]),
    "rtgb_denoiser_param_count": (C.c_int64, []),
    "rtgb_load_denoiser_file": (C.c_int, [Handle, C.c_char_p]),
    "rtgb_device_info_get": (C.c_int, [Handle, C.c_void_p]),
    "rtgb_set_denoiser_params": (C.c_int, [Handle, C.c_void_p, C.c_int64]),
    "rtgb_conv3x3_pack_weights": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "rtgb_conv3x3_bf16": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                    C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                    C.c_char_p, C.c_size_t]),
    "rtgb_build_lbvh_static": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]),
}

STATIC_LBVH_MAX_PRIMITIVES = 131072

_lib = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load ``librtgb.so`` (building it in-tree when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build()")
        _build.build_product()
    lib = C.CDLL(str(path))
    missing = []
    for name, (res, args) in SIGNATURES.items():
        try:
            fn = getattr(lib, name)
        except AttributeError:
            missing.append(name)
            continue
        fn.restype = res
        fn.argtypes = args
    lib.rtgb_missing_symbols = missing
    _lib = lib
    return lib


class RtgbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def check(status: int, handle=None, what: str = "") -> None:
    if status != OK:
        msg = what
        if handle is not None:
            raw = load().rtgb_last_error(handle)
            if raw:
                msg = f"{what}: {raw.decode()}"
        raise RtgbError(status, msg)
