"""bench.py's host-side arithmetic (CPU): the roofline record of the launch slot
with the largest share of the frame, read against the committed ncu traffic
file, and the denoiser's FLOP count."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def _frame(mb=4):
    # raygen, (trace, shade, shadow) per bounce, finalize, resolve
    times = [0.05] + [0.15, 0.30, 0.10] * mb + [0.02, 0.08]
    stats = {"paths": 1000, "pixels": 1000, "active": [1000, 600, 300, 100], "restir_pixels": 900,
             "shadow_rays_per_bounce": [1800, 1000, 500, 200]}
    return times, stats


def test_roofline_picks_the_largest_slot_and_reads_traffic():
    times, stats = _frame()
    roof = bench.roofline([times, times], [stats, stats], spatial=1)
    assert roof["kernel"] == "k_shade@0"
    want_bytes = 1000 * bench.BYTES_SHADE + 900 * (84 + 84 * 2 + 84)
    assert roof["algorithmic_bytes_per_launch"] == pytest.approx(want_bytes)
    assert roof["achieved"] == pytest.approx(want_bytes / 0.30e-3 / 1e9)
    assert roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"])
    traffic = json.loads((ROOT / "profiles" / "roofline_traffic.json").read_text())
    assert roof["traffic"] == pytest.approx(float(traffic["k_shade@0"]))
    assert roof["unit"] == "GB/s" and roof["bound"] == "hbm"


def test_denoiser_flops_match_the_network():
    from ray_tracing_gb300 import denoiser
    # full, half and quarter resolution layers of the U-Net at 4 x 640x480
    full = (10 * 32 + 32 * 32 + 80 * 32 + 32 * 32 + 32 * 3) * 640 * 480
    half = (32 * 48 + 48 * 48 + 112 * 48 + 48 * 48) * 320 * 240
    quarter = (48 * 64 + 64 * 64) * 160 * 120
    assert bench.denoiser_flops(640, 480, 4) == pytest.approx(2 * 9 * 4 * (full + half + quarter))
    assert len(denoiser.LAYERS) == 11


def test_training_flops_count_forward_and_both_gradients():
    from ray_tracing_gb300 import denoiser
    n, h, w = 2, 64, 32
    fwd = bench.denoiser_flops(w, h, n)
    first = 2.0 * n * h * w * denoiser.LAYERS[0][0] * denoiser.LAYERS[0][1] * 9
    assert bench.training_flops(n, h, w) == pytest.approx(3 * fwd - first)


def test_mixed_1080p_rig_for_the_relmse_target():
    import math
    rig = bench.mixed_rig_1080p()
    assert rig.active_count == 4
    assert [(c.width, c.height, c.model) for c in rig.cameras[:4]] == [(1920, 1080, 0), (1920, 1080, 1)] * 2
    f = 960.0 / (math.pi / 2.0)
    for i in (1, 3):
        e = rig.cameras[i].equi
        assert e.fx == pytest.approx(f) and e.cx == 960.0 and e.cy == 540.0
        assert all(e.lut[k] <= e.lut[k + 1] for k in range(len(e.lut) - 1))   # monotone theta(r) table


def test_trimmed_relmse_drops_only_the_largest_errors():
    rng = np.random.default_rng(3)
    ref = rng.uniform(0.5, 1.5, (64, 100, 3))
    x = ref * (1.0 + rng.normal(0.0, 0.05, ref.shape))
    base = bench.relmse(x, ref)
    assert bench.relmse_trimmed(x, ref, trim=0.0) == pytest.approx(base)
    # one firefly dominates the plain relMSE but not the trimmed one
    y = x.copy()
    y[10, 20, 1] = 5000.0
    assert bench.relmse(y, ref) > 100 * base
    e = ((x - ref) ** 2 / (ref ** 2 + bench.RELMSE_EPS)).ravel()
    keep = e.size - int(np.floor(e.size * bench.TRIM_FRACTION))
    rest = np.delete(e, np.ravel_multi_index((10, 20, 1), ref.shape))  # the firefly is the largest error
    assert bench.relmse_trimmed(y, ref) == pytest.approx(np.sort(rest)[:keep].mean())
    assert bench.relmse_trimmed(y, ref) < 1.1 * base


def test_first_spp_within_reads_the_smallest_probe():
    trail = [{"spp": 1, "t": 9.0}, {"spp": 16, "t": 0.5}, {"spp": 8, "t": 0.7}, {"spp": 4, "t": 0.2},
             {"spp": 2, "t": None}]
    assert bench.first_spp_within(trail, "t", 0.6) == 4
    assert bench.first_spp_within(trail, "t", 0.1) is None
    assert bench.first_spp_within([], "t", 1.0) is None


def test_banded_search_and_trimmed_cross_check_with_a_fake_renderer(monkeypatch):
    # the search logic of the C5 equal-relMSE record on CPU: plain renders are
    # the reference plus noise shrinking as 1/sqrt(spp), with a firefly at 16 spp
    import types
    import ray_tracing_gb300.renderer as rmod

    class FakeRenderer:
        def __init__(self, *a, **k):
            pass

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            return False

        def prepare_scene(self, view):
            pass

        def reset_sequence(self, s):
            pass

    rng0 = np.random.default_rng(11)
    truth = [rng0.uniform(0.2, 2.0, (16, 40, 3)) for _ in range(2)]

    def fake_bands(r, rig, cameras, spp, max_bounces, per_frame):
        rng = np.random.default_rng(spp * 7 + rig)
        bands = [t * (1.0 + rng.normal(0.0, 0.8 / np.sqrt(spp), t.shape)) for t in truth[:cameras]]
        if spp == 16:
            bands[0][3, 5, 0] = 1e4  # a firefly
        return bands, 1.0

    monkeypatch.setattr(rmod, "Renderer", FakeRenderer)
    monkeypatch.setattr(bench, "plain_bands", fake_bands)
    monkeypatch.setattr(bench, "plain_render", lambda r, rig, spp, **k: (None, float(spp)))
    rng = np.random.default_rng(5)
    denoised = {0: [t * (1.0 + rng.normal(0.0, 0.1, t.shape)) for t in truth],
                1: [t * (1.0 + rng.normal(0.0, 0.1, t.shape)) for t in truth]}
    out = bench.banded_equal_relmse(types.SimpleNamespace(view=None), {0: 0, 1: 1}, {"nee": (denoised, 2.0)},
                                    max_bounces=6, cameras=2, ref_spp=4096, max_spp=1024, time_spp_cap=128)
    spp = out["plain"]["spp"]
    assert spp is not None and out["plain"]["relmse"] <= out["denoised"]["relmse"]
    assert out["speedup_at_equal_relmse"] == pytest.approx(out["plain"]["ms"] / 2.0)
    cc = out["trimmed_cross_check"]
    assert "error" not in cc and cc["plain_spp"] is not None
    assert cc["speedup"] == pytest.approx(cc["plain_ms"] / 2.0)
    trail = out["plain_search"]
    assert all("relmse_trimmed" in p for p in trail)
    # the firefly inflates the 16-spp relMSE, not its trimmed value
    p16 = next(p for p in trail if p["spp"] == 16)
    p8 = next(p for p in trail if p["spp"] == 8)
    assert p16["relmse"] > p8["relmse"] and p16["relmse_trimmed"] < p8["relmse_trimmed"]


def test_headline_equal_relmse_with_a_fake_renderer(monkeypatch):
    # the benchmark frame's search and its trimmed cross-check on CPU
    import types
    import ray_tracing_gb300.renderer as rmod

    rng0 = np.random.default_rng(2)
    truth = rng0.uniform(0.2, 2.0, (4, 12, 16, 3))

    class FakeRenderer:
        def __init__(self, *a, **k):
            self.rng = np.random.default_rng(9)

        def prepare_scene(self, view):
            pass

        def reset_sequence(self, s):
            pass

        def set_denoiser(self, w):
            pass

        def render_frame(self, rig, prof, n):
            cam = types.SimpleNamespace(denoise_ms=0.5)
            return types.SimpleNamespace(frame_render_ms=2.5, cameras=[cam])

        def buffer(self, c, name):
            noise = 0.1 if name == "denoised" else 1.0
            img = truth[c] * (1.0 + self.rng.normal(0.0, noise, truth[c].shape))
            return np.concatenate([img, np.ones(img.shape[:2] + (1,))], axis=-1)

        def close(self):
            pass

    def fake_plain(r, rig, spp, **k):
        rng = np.random.default_rng(spp)
        img = truth * (1.0 + rng.normal(0.0, 1.0 / np.sqrt(spp), truth.shape))
        return img, float(spp)

    monkeypatch.setattr(rmod, "Renderer", FakeRenderer)
    monkeypatch.setattr(bench, "plain_render", fake_plain)
    monkeypatch.setattr(bench, "_weights", lambda: np.zeros(1))
    out = bench.equal_relmse(types.SimpleNamespace(view=None), None, None, frames=3)
    assert out["plain"]["spp"] is not None
    assert out["speedup_at_equal_relmse"] == pytest.approx(out["plain"]["ms"] / 2.5)
    cc = out["trimmed_cross_check"]
    assert "error" not in cc and cc["plain_spp"] is not None
    assert cc["speedup"] == pytest.approx(cc["plain_ms"] / 2.5)
    assert all("relmse_trimmed" in p for p in out["plain_search"])
