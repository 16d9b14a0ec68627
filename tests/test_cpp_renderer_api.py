"""The C++ call surface of include/rtgb_renderer.hpp (OptixRenderer /
RendererPool of the reference over the C ABI): it compiles against the
header, links librtgb.so, and maps statuses to the reference's exceptions.
CPU: error mapping and pool bounds (without a GPU, creating a renderer must
throw std::runtime_error rather than crash). GPU: a pool renders a frame and
each camera's host frame carries the luminance the library's frame has."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

from ray_tracing_gb300 import build as _build

ROOT = Path(__file__).resolve().parent.parent

PROGRAM = r"""
#include <cstdio>
#include <stdexcept>
#include <string>
#include "rtgb_renderer.hpp"

static int fails = 0;
#define EXPECT(c, what) do { if (!(c)) { ++fails; std::fprintf(stderr, "FAILED %s\n", what); } } while (0)

int main(int argc, char** argv) {
    bool threw = false;
    try { rtgb::detail::check(RTGB_INVALID_ARGUMENT, nullptr, "x"); } catch (const std::invalid_argument&) { threw = true; }
    EXPECT(threw, "invalid argument maps to std::invalid_argument");
    threw = false;
    try { rtgb::detail::check(RTGB_DEVICE_FAULT_FLAG, nullptr, "x"); } catch (const std::runtime_error& e) {
        threw = std::string(e.what()) == "x";
    }
    EXPECT(threw, "other statuses map to std::runtime_error");
    threw = false;
    try { rtgb::detail::check_request(RTGB_INVALID_ARGUMENT, nullptr, "r"); } catch (const std::runtime_error& e) {
        threw = std::string(e.what()) == "r";
    }
    EXPECT(threw, "a rejected render request is std::runtime_error, as validate_render_pool_request throws");
    threw = false;
    try { rtgb::RendererPool pool(5); } catch (const std::runtime_error& e) {
        threw = std::string(e.what()) == "RendererPool requires renderer_count in [1, 4]";
    }
    EXPECT(threw, "pool size bound");
    const bool gpu = argc > 1 && std::string(argv[1]) == "gpu";
    if (!gpu) {
        threw = false;
        try { rtgb::OptixRenderer r; } catch (const std::runtime_error&) { threw = true; }
        EXPECT(threw, "no device: creating a renderer throws");
    } else {
        rtgb_host_scene* hs = nullptr;
        EXPECT(rtgb_host_scene_create("cornell_box", 0, 0, &hs) == RTGB_OK, "scene");
        rtgb_scene view{};
        rtgb_host_scene_view(hs, &view);
        rtgb_camera_rig rig{};
        rtgb_default_rig("cornell_box", 2, 64, 64, &rig);
        rtgb_render_profile prof{};
        rtgb_profile_preset("realtime", &prof);
        prof.enable_denoise = 0;
        rtgb::RendererPool pool(2);
        pool.prepare_scene(view);
        pool.reset_sequence(3);
        const auto frames = pool.render_frame(rig, prof, 2);
        EXPECT(frames.size() == 2 && frames[1].camera_index == 1, "one result per camera, sorted");
        EXPECT(frames[0].frame.width == 64 && frames[0].frame.beauty_rgba.size() == 64 * 64 * 4, "frame shape");
        EXPECT(frames[0].frame.average_luminance > 0.0 && frames[0].timing.render_ms > 0.0, "luminance and timing");
        threw = false;
        try { (void)pool.render_frame(rig, prof, 3); } catch (const std::runtime_error&) { threw = true; }
        EXPECT(threw, "more active cameras than the pool holds");
        rtgb_host_scene_destroy(hs);
    }
    std::printf("cpp_renderer_api failures=%d\n", fails);
    return fails == 0 ? 0 : 1;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if not _build.LIB.exists():
        _build.build_all()
    d = tmp_path_factory.mktemp("cppapi")
    src = d / "api.cpp"
    src.write_text(PROGRAM)
    exe = d / "api"
    subprocess.run(["g++", "-std=c++23", "-O1", "-Wall", "-Wextra", "-I", str(ROOT / "include"), str(src),
                    "-L", str(_build.LIB_DIR), "-lrtgb", f"-Wl,-rpath,{_build.LIB_DIR}", "-o", str(exe)], check=True)
    return exe


def test_error_mapping_and_pool_bounds(program):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the no-device path cannot be checked")
    res = subprocess.run([str(program)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr


@pytest.mark.gpu
def test_pool_renders_a_frame(program):
    res = subprocess.run([str(program), "gpu"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
