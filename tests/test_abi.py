"""The C ABI library: loads without a GPU, exports every declared entry point,
and its structure layouts match the header as a C compiler sees them."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from ray_tracing_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "rtgb.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(rtgb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = abi.load()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(abi.SIGNATURES), "abi.SIGNATURES must mirror include/rtgb.h"


STRUCTS = {
    "rtgb_texture": abi.Texture, "rtgb_material": abi.Material, "rtgb_sphere": abi.Sphere,
    "rtgb_quad": abi.Quad, "rtgb_triangle": abi.Triangle, "rtgb_medium": abi.Medium,
    "rtgb_analytic_light": abi.AnalyticLight, "rtgb_scene": abi.Scene, "rtgb_pinhole32": abi.Pinhole32,
    "rtgb_equi62_lut1d": abi.Equi62Lut1d, "rtgb_camera": abi.Camera, "rtgb_camera_rig": abi.CameraRig,
    "rtgb_render_profile": abi.RenderProfile, "rtgb_create_info": abi.CreateInfo,
    "rtgb_camera_frame_view": abi.CameraFrameView, "rtgb_frame_views": abi.FrameViews,
    "rtgb_restir_stats": abi.RestirDiagnostics, "rtgb_acceleration_info": abi.AccelerationInfo,
    "rtgb_openpbr_material": abi.OpenPbrMaterial, "rtgb_device_info": abi.DeviceInfo,
    "rtgb_launch_tuning": abi.LaunchTuning, "rtgb_mesh_prototype": abi.MeshPrototype,
    "rtgb_mesh_instance": abi.MeshInstance, "rtgb_mesh_set": abi.MeshSet,
}


def test_struct_layouts_match_the_header(tmp_path):
    src = tmp_path / "sizes.c"
    lines = ['#include <stdio.h>', '#include "rtgb.h"', "int main(void) {"]
    for name in STRUCTS:
        lines.append(f'  printf("{name} %zu\\n", sizeof({name}));')
    lines.append("  return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    for line in out.splitlines():
        name, size = line.split()
        assert C.sizeof(STRUCTS[name]) == int(size), name


def test_create_without_gpu_reports_an_error_instead_of_crashing():
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert abi.load().rtgb_create(None, C.byref(h)) == 2
    assert not h.value


def test_null_arguments_are_invalid():
    lib = abi.load()
    assert lib.rtgb_prepare_scene(None, None) == 1
    assert lib.rtgb_render_frame(None, None, None, 1, None) == 1
    assert lib.rtgb_reset_sequence(None, 0) == 1
    assert lib.rtgb_download_frame(None, 0, None, None, None, None, None) == 1
    assert lib.rtgb_autotune_launches(None, None, None, 1, 4, None) == 1
    assert lib.rtgb_host_scene_save(None, b"x") == 1
    assert lib.rtgb_host_scene_from_view(None, None) == 1


def test_scene_files_refuse_bad_input(tmp_path):
    lib = abi.load()
    out = C.c_void_p()
    assert lib.rtgb_host_scene_load(str(tmp_path / "missing.rtgbscene").encode(), C.byref(out)) == 1 and not out.value
    (tmp_path / "wrong.rtgbscene").write_bytes(b"NOTASCENE" * 8)
    assert lib.rtgb_host_scene_load(str(tmp_path / "wrong.rtgbscene").encode(), C.byref(out)) == 1 and not out.value
    # a header whose record sizes disagree with this build's structs
    import struct
    bad = b"RTGBSCN1" + struct.pack("<I", 1) + struct.pack("<9I", *([7] * 9))
    (tmp_path / "layout.rtgbscene").write_bytes(bad)
    assert lib.rtgb_host_scene_load(str(tmp_path / "layout.rtgbscene").encode(), C.byref(out)) == 1 and not out.value
    # a file claiming more records than it holds
    from ray_tracing_gb300 import scenes
    sc = scenes.HostScene("cornell_box")
    sc.save(tmp_path / "ok.rtgbscene")
    data = bytearray((tmp_path / "ok.rtgbscene").read_bytes())
    data[8 + 4 + 36:8 + 4 + 36 + 8] = struct.pack("<Q", 1 << 40)  # texture count
    (tmp_path / "huge.rtgbscene").write_bytes(bytes(data))
    assert lib.rtgb_host_scene_load(str(tmp_path / "huge.rtgbscene").encode(), C.byref(out)) == 1 and not out.value
    again = scenes.HostScene.load(tmp_path / "ok.rtgbscene")
    assert again.counts() == sc.counts()
