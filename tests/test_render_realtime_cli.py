"""The render_realtime CLI (utils/render_realtime.cpp's flags and artifacts).

CPU: argument validation, and the report writer, PNG writer and OpenEXR writer
through small harnesses compiled against the CLI's headers (schema-3 summary,
CSV columns, nearest-rank percentiles, FNV-1a64 manifest digests as
tests/test_realtime_benchmark_report.cpp of the reference checks them; EXR
files read back by an independent parser of the published file layout).
GPU: a short run writes every artifact, the EXR frames holding the same linear
radiance whose mean luminance the summary reports.
"""
from __future__ import annotations

import csv
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from _exr import read_exr
from _png import read_png
from ray_tracing_gb300 import build as _build

ROOT = Path(__file__).resolve().parent.parent
CLI_DIR = ROOT / "ray_tracing_gb300" / "csrc" / "cli"
CSV_HEAD = ("frame_index,sample_stream,camera_count,profile,width,height,samples_per_pixel,max_bounces,"
            "denoise_enabled,frame_ms,pipeline_ms,render_ms,denoise_ms,download_ms,render_work_ms,"
            "denoise_work_ms,download_work_ms,image_write_ms,host_overhead_ms,fps")


def fnv1a64(data: bytes) -> str:
    h = 14695981039346656037
    for b in data:
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}"


def nearest_rank(values, p):
    v = sorted(values)
    rank = int(np.ceil(p * len(v)))
    return v[0] if rank <= 1 else v[min(rank - 1, len(v) - 1)]


@pytest.fixture(scope="module")
def cli():
    path = _build.CLI
    if not path.exists():
        _build.build_all()
    return path


@pytest.mark.parametrize("args,message", [
    (["--camera-count", "5"], "--camera-count must be in [1, 4]"),
    (["--frames", "0"], "--frames must be >= 1"),
    (["--warmup-frames", "-1"], "--warmup-frames must be >= 0"),
    (["--seed", "4294967295", "--frames", "2", "--warmup-frames", "0"], "exceeds uint32 sample streams"),
    (["--profile", "fast"], "--profile must be one of"),
    (["--scene", "no_such_scene"], "--scene must reference a registered realtime scene"),
    (["--bogus"], "unknown argument"),
    (["--scene-file", "no_such_file.rtgbscene"], "--scene-file must name a readable scene file"),
])
def test_argument_validation(cli, tmp_path, args, message):
    res = subprocess.run([str(cli), "--output-dir", str(tmp_path), *args], capture_output=True, text=True, timeout=60)
    assert res.returncode != 0
    assert message in res.stderr


HARNESS = r"""
#include "benchmark_report.h"
#include "png_writer.h"
int main(int argc, char** argv) {
    namespace R = rtgb::report;
    R::Report r;
    r.scene = "smoke"; r.profile = "bal,anced"; r.camera_count = 2; r.width = 64; r.height = 48;
    r.frames_requested = 5; r.warmup_frames = 3; r.random_seed = 7; r.samples_per_pixel = 2; r.max_bounces = 4;
    r.denoise_enabled = true;
    const double fms[5] = {4.0, 1.0, 3.0, 5.0, 2.0};
    for (int i = 0; i < 5; ++i) {
        R::FrameSample f;
        f.frame_index = i; f.sample_stream = 10 + i; f.camera_count = 2; f.profile = r.profile; f.width = 64;
        f.height = 48; f.samples_per_pixel = 2; f.max_bounces = 4; f.denoise_enabled = true;
        f.frame_ms = fms[i]; f.pipeline_ms = fms[i] / 2; f.render_ms = 0.5; f.fps = 1000.0 / fms[i];
        f.rays_traced = 1000000;
        f.cameras.push_back({0, 0.5, 0.1, 0.2, 0.25});
        f.cameras.push_back({1, 0.5, 0.1, 0.2, 0.75});
        r.frames.push_back(f);
    }
    r.aggregate = R::aggregate_of(r.frames);
    std::filesystem::path d = argv[1];
    R::write_csv(r, d / "benchmark_frames.csv");
    R::write_json(r, d / "benchmark_summary.json");
    R::write_manifest(r, {d / "benchmark_frames.csv", d / "benchmark_summary.json"}, d / "benchmark_manifest.json");
    std::vector<uint8_t> rgb(7 * 5 * 3);
    for (size_t i = 0; i < rgb.size(); ++i) rgb[i] = static_cast<uint8_t>(i * 37 % 251);
    rtgb::png::write_rgb(d / "t.png", 7, 5, rgb.data());
    (void)argc;
    return 0;
}
"""


def test_report_and_png_writers(tmp_path):
    src = tmp_path / "harness.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "harness"
    subprocess.run(["g++", "-std=c++23", "-O1", "-I", str(CLI_DIR), str(src), "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path)], check=True)
    rows = list(csv.reader(open(tmp_path / "benchmark_frames.csv")))
    assert ",".join(rows[0]).startswith(CSV_HEAD)
    assert len(rows) == 6 and rows[1][3] == "bal,anced"
    summary = json.loads((tmp_path / "benchmark_summary.json").read_text())
    assert summary["schema_version"] == 3
    assert summary["metadata"]["measurement_sample_stream_start"] == 10
    assert summary["metadata"]["rng_algorithm"] == "hashed_pixel_sample_stream_v1"
    agg = summary["aggregate"]["frame_ms"]
    fms = [4.0, 1.0, 3.0, 5.0, 2.0]
    assert agg["avg"] == pytest.approx(3.0) and agg["max"] == 5.0
    for p, key in ((0.5, "p50"), (0.95, "p95"), (0.99, "p99")):
        assert agg[key] == nearest_rank(fms, p)
    assert len(summary["frames"]) == 5 and len(summary["per-camera"]) == 10
    assert summary["extensions"]["rays_traced"] == 5000000
    manifest = json.loads((tmp_path / "benchmark_manifest.json").read_text())
    assert manifest["report_schema_version"] == 3 and manifest["per_camera_record_count"] == 10
    for art in manifest["artifacts"]:
        data = (tmp_path / art["filename"]).read_bytes()
        assert art["size_bytes"] == len(data)
        assert art["digest"] == fnv1a64(data)
    img = read_png(tmp_path / "t.png")
    want = (np.arange(7 * 5 * 3) * 37 % 251).astype(np.uint8).reshape(5, 7, 3)
    assert np.array_equal(img, want)


EXR_HARNESS = r"""
#include <cmath>
#include "exr_writer.h"
int main(int argc, char** argv) {
    std::filesystem::path d = argv[1];
    const int w = 13, h = 6;
    std::vector<float> rgba(static_cast<size_t>(w) * h * 4);
    for (size_t i = 0; i < rgba.size(); ++i) rgba[i] = std::ldexp(static_cast<float>(i % 97) - 20.0f, static_cast<int>(i % 7) - 3);
    rtgb::exr::write_rgba(d / "rgb.exr", w, h, rgba.data());
    rtgb::exr::write_rgba(d / "rgba.exr", w, h, rgba.data(), true);
    bool threw = false;
    try {
        rtgb::exr::encode(w, h, {"R", "G"}, rgba.data());
    } catch (const std::runtime_error&) {
        threw = true;
    }
    (void)argc;
    return threw ? 0 : 3;
}
"""


def test_exr_writer(tmp_path):
    src = tmp_path / "exr.cpp"
    src.write_text(EXR_HARNESS)
    exe = tmp_path / "exr"
    subprocess.run(["g++", "-std=c++23", "-O1", "-I", str(CLI_DIR), str(src), "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path)], check=True)
    w, h = 13, 6
    i = np.arange(w * h * 4)
    want = np.ldexp((i % 97).astype(np.float32) - 20.0, (i % 7) - 3).astype(np.float32).reshape(h, w, 4)
    for name, chans in (("rgb", ["B", "G", "R"]), ("rgba", ["A", "B", "G", "R"])):
        attrs, img = read_exr(tmp_path / f"{name}.exr")
        assert attrs["channels"] == chans
        assert attrs["dataWindow"] == (0, 0, w - 1, h - 1) and attrs["displayWindow"] == (0, 0, w - 1, h - 1)
        assert attrs["lineOrder"] == 0 and attrs["pixelAspectRatio"] == 1.0 and attrs["screenWindowWidth"] == 1.0
        for k, c in enumerate("RGBA"):
            if c in chans:
                assert np.array_equal(img[c], want[..., k]), c
    size = (tmp_path / "rgb.exr").stat().st_size
    assert size > h * (8 + 8 + w * 3 * 4)


@pytest.mark.gpu
def test_cli_writes_all_artifacts(cli, tmp_path):
    res = subprocess.run([str(cli), "--scene", "smoke", "--camera-count", "2", "--frames", "2", "--warmup-frames", "1",
                          "--seed", "5", "--width", "96", "--height", "72", "--output-dir", str(tmp_path), "--write-exr"],
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    assert "summary profile=balanced" in res.stdout
    rows = list(csv.reader(open(tmp_path / "benchmark_frames.csv")))
    assert len(rows) == 3 and rows[1][1] == "6" and rows[2][1] == "7"
    summary = json.loads((tmp_path / "benchmark_summary.json").read_text())
    assert summary["metadata"]["camera_count"] == 2 and summary["environment"]["compute_capability"] == "10.3"
    assert summary["extensions"]["rays_traced"] > 0
    for f in range(2):
        for c in range(2):
            img = read_png(tmp_path / f"frame_{f:04d}_cam_{c}.png")
            assert img.shape == (72, 96, 3) and img.max() > 0
            _, hdr = read_exr(tmp_path / f"frame_{f:04d}_cam_{c}.exr")
            assert hdr["R"].shape == (72, 96) and all(np.isfinite(hdr[k]).all() for k in "RGB")
            lum = (0.2126 * hdr["R"].astype(np.float64) + 0.7152 * hdr["G"] + 0.0722 * hdr["B"]).mean()
            rec = [r for r in summary["per-camera"] if r["frame_index"] == f and r["camera_index"] == c]
            assert len(rec) == 1 and lum == pytest.approx(rec[0]["average_luminance"], rel=1e-5)
