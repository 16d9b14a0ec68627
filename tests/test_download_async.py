"""Pipelined downloads: rtgb_download_frame_async and rtgb_wait_downloads.

The copies of frame i run on the handle's copy stream while frame i+1 renders;
frame i+2 reuses frame i's device buffers (beauty, AOVs and the denoiser's
output) and waits for those copies on the device. The same frame sequence is
rendered twice, once in the reference's order (rtgb_render_frame, then the
waiting rtgb_download_frame per camera) and once pipelined, and every frame's
host bytes must be identical, with and without the denoiser.
"""
from __future__ import annotations

import numpy as np
import pytest

from ray_tracing_gb300 import abi, denoiser, scenes

CAMS, W, H, FRAMES = 2, 160, 96, 6


def _setup(denoise: int):
    sc = scenes.HostScene("random_spheres", seed=3, detail=64)
    rig = scenes.default_rig("random_spheres", CAMS, W, H)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=3, enable_denoise=denoise,
                          enable_restir_di=1, restir_initial_candidates=8, restir_min_analytic_lights=8)
    params = None
    if denoise:
        torch = pytest.importorskip("torch")
        torch.manual_seed(5)
        params = denoiser.flatten(denoiser.build_model())
    return sc, rig, prof, params


def _renderer(sc, params):
    from ray_tracing_gb300.renderer import Renderer
    r = Renderer()
    r.prepare_scene(sc.view)
    if params is not None:
        r.set_denoiser(params)
    return r


def _pinned_set(torch):
    return [[torch.zeros(W * H * 4, dtype=torch.float32, pin_memory=True) for _ in range(3)]
            + [torch.zeros(W * H, dtype=torch.float32, pin_memory=True)] for _ in range(CAMS)]


def _snapshot(host_set):
    return [[t.numpy().copy() for t in cam] for cam in host_set]


def _blocking_frames(sc, rig, prof, params):
    with _renderer(sc, params) as r:
        out = []
        for _ in range(FRAMES):
            r.render_frame(rig, prof, CAMS)
            frame = []
            for c in range(CAMS):
                f = r.download(c)
                frame.append([f.beauty_rgba.reshape(-1), f.normal_rgba.reshape(-1), f.albedo_rgba.reshape(-1),
                              f.depth.reshape(-1)])
            out.append(frame)
        return out


def _assert_same(got, want):
    assert len(got) == len(want)
    for i, (g, w) in enumerate(zip(got, want)):
        for c in range(CAMS):
            for k, name in enumerate(("beauty", "normal", "albedo", "depth")):
                assert np.array_equal(g[c][k], w[c][k]), f"frame {i} camera {c} {name}"


@pytest.mark.gpu
@pytest.mark.parametrize("denoise", [0, 1])
def test_double_buffered_pipeline_matches_blocking(denoise):
    torch = pytest.importorskip("torch")
    sc, rig, prof, params = _setup(denoise)
    want = _blocking_frames(sc, rig, prof, params)
    # consecutive frames differ, so a stale or overwritten buffer would show
    assert not np.array_equal(want[0][0][0], want[1][0][0])
    host = [_pinned_set(torch), _pinned_set(torch)]
    got = []
    with _renderer(sc, params) as r:
        for i in range(FRAMES):
            r.render_frame_async(rig, prof, CAMS)
            for c in range(CAMS):
                r.download_async(c, *host[i & 1][c])
            r.wait_downloads(keep_latest=True)
            if i > 0:
                got.append(_snapshot(host[(i - 1) & 1]))
        r.wait_downloads()
        got.append(_snapshot(host[(FRAMES - 1) & 1]))
        v = r.frame_stats()
        assert v.camera_count == CAMS
    _assert_same(got, want)


@pytest.mark.gpu
def test_frames_in_flight_wait_for_their_copies():
    # no host wait until the end: frame i+2 overwrites frame i's device buffers
    # only after frame i's copies (the device-side wait), so every host set
    # holds its own frame
    torch = pytest.importorskip("torch")
    sc, rig, prof, params = _setup(1)
    want = _blocking_frames(sc, rig, prof, params)
    host = [_pinned_set(torch) for _ in range(FRAMES)]
    with _renderer(sc, params) as r:
        for i in range(FRAMES):
            r.render_frame_async(rig, prof, CAMS)
            for c in range(CAMS):
                r.download_async(c, *host[i][c])
        r.wait_downloads()
    _assert_same([_snapshot(h) for h in host], want)


@pytest.mark.gpu
def test_async_download_errors():
    torch = pytest.importorskip("torch")
    sc, rig, prof, params = _setup(0)
    buf = torch.zeros(W * H * 4, dtype=torch.float32, pin_memory=True)
    with _renderer(sc, params) as r:
        with pytest.raises(abi.RtgbError, match="no frame has been rendered"):
            r.download_async(0, buf)
        r.wait_downloads()  # nothing enqueued: returns at once
        r.render_frame(rig, prof, CAMS)
        with pytest.raises(abi.RtgbError, match="camera_index out of range"):
            r.download_async(CAMS, buf)
        r.download_async(1, beauty=buf)  # NULL for the other buffers
        r.wait_downloads()
        ref = r.download(1).beauty_rgba.reshape(-1)
        assert np.array_equal(buf.numpy(), ref)


def test_async_entry_points_are_declared():
    lib = abi.load()
    for name in ("rtgb_download_frame_async", "rtgb_wait_downloads"):
        assert hasattr(lib, name)
