"""Row-band sampling of the 1080p equal-relMSE comparison (CPU).

bench.py judges 4 x 1920x1080 frames on row bands rendered as cropped
cameras. A crop keeps the pose and intrinsics and shifts the principal point
by the band's first row, so each of its pixels unprojects to exactly the
direction of the full camera's pixel in that row: checked here on the CPU
oracle's camera models (pinhole32 with distortion and the 180-degree
equi62_lut1d fisheye of the C5 rig)."""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from helpers import equi, pinhole  # noqa: E402


def _dir(lib, cam, px, py):
    out = (C.c_float * 3)()
    lib.orc_unproject(C.byref(cam), px, py, out)
    return tuple(out)


def test_band_starts_are_in_range_and_ordered():
    for h in (1080, 480, 64):
        starts = bench.band_starts(h)
        assert len(starts) == bench.BAND_COUNT
        assert starts == sorted(starts)
        assert all(0 <= y0 <= h - bench.BAND_ROWS for y0 in starts)
    assert len(set(bench.band_starts(1080))) == bench.BAND_COUNT


def test_cropped_cameras_trace_the_full_cameras_rays():
    from oracle.binding import load
    lib = load()
    cams = [pinhole(1920, 1080, 90.0, k=(0.02, -0.01, 0.003), p=(0.001, -0.0015)), equi(1920, 1080, 180.0)]
    for cam in cams:
        for y0 in bench.band_starts(cam.height):
            crop = bench.crop_camera(cam, y0, bench.BAND_ROWS)
            assert crop.height == bench.BAND_ROWS and crop.width == cam.width
            for j in (0, bench.BAND_ROWS - 1):
                for x in (0, 7, cam.width // 2, cam.width - 1):
                    assert _dir(lib, crop, x + 0.5, j + 0.5) == _dir(lib, cam, x + 0.5, y0 + j + 0.5)


def test_band_rigs_cover_every_band_once():
    from ray_tracing_gb300 import abi
    rig = abi.CameraRig()
    rig.active_count = 4
    for i in range(4):
        rig.cameras[i] = pinhole(1920, 1080, 90.0) if i % 2 == 0 else equi(1920, 1080, 180.0)
    groups = bench.band_rigs(rig, 4)
    seen = [key for _, part in groups for key in part]
    assert len(seen) == len(set(seen)) == 4 * bench.BAND_COUNT
    assert all(rr.active_count <= 4 for rr, _ in groups)
    full = np.arange(1080 * 3 * 2, dtype=np.float64).reshape(1080, 2, 3)
    rows = bench.band_rows_of(full, 1080)
    assert rows.shape == (bench.BAND_COUNT * bench.BAND_ROWS, 2, 3)
    assert np.array_equal(rows[: bench.BAND_ROWS], full[bench.band_starts(1080)[0]:][: bench.BAND_ROWS])
