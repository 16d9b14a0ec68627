"""bench.py's host-side arithmetic (CPU): the roofline record of the launch slot
with the largest share of the frame, read against the committed ncu traffic
file, and the denoiser's FLOP count."""
import json
import sys
from pathlib import Path

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
