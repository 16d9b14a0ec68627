"""Launch-shape autotuner (rtgb_autotune_launches).

The wavefront kernels loop grid-stride over their queues, so the grid a stage
launches with must not change any result. GPU: after tuning, a renderer
traces exactly the paths (hit codes and radiance, bit for bit) an untuned one
does, and the tuning report is well formed.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import scaled_rig
from ray_tracing_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def test_tuned_grids_trace_the_same_paths():
    from ray_tracing_gb300.renderer import Renderer
    sc = scenes.HostScene("random_spheres", detail=64)
    rig = scaled_rig(scenes.default_rig("random_spheres", 2), 0.2)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0, enable_restir_di=1,
                          restir_initial_candidates=8, restir_temporal_reuse=1, restir_spatial_neighbors=1)
    plain = Renderer(debug_path_records=True)
    tuned = Renderer(debug_path_records=True)
    for r in (plain, tuned):
        r.prepare_scene(sc.view)
    report = tuned.autotune_launches(rig, prof, 2, frames=2)
    assert [c["grid_scale"] for c in report["candidates"]] == [0.5, 1.0, 2.0, 4.0] * 2
    assert [c["block"] for c in report["candidates"]] == ["kernel's"] * 4 + ["half"] * 4
    assert set(report["chosen"]) == set(abi.TUNE_GROUP_NAMES)
    assert all(v in report["candidates"] for v in report["chosen"].values())
    assert all(x > 0.0 for x in report["frame_ms"]) and report["tuned_frame_ms"] > 0.0
    for name, row in report["group_ms"].items():
        assert all(np.isfinite(row)) and min(row) >= 0.0, name
    for r in (plain, tuned):
        r.reset_sequence(11)
        for _ in range(3):
            r.render_frame(rig, prof, 2)
    for cam in range(2):
        pc, pr = plain.path_records(cam, 1, 4)
        tc, tr = tuned.path_records(cam, 1, 4)
        assert np.array_equal(pc, tc)
        assert np.array_equal(pr, tr)
    plain.close()
    tuned.close()


def test_a_failed_tuning_leaves_the_handle_as_it_was():
    """A render that fails inside the tuner (here a profile the request
    validation refuses) must not leave a candidate's grids or the tuner's
    stage events in force: the handle keeps the grids it had, stage timing is
    off again, and the next frame renders."""
    from ray_tracing_gb300.renderer import Renderer
    sc = scenes.HostScene("random_spheres", detail=64)
    rig = scaled_rig(scenes.default_rig("random_spheres", 2), 0.2)
    good = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0)
    bad = scenes.profile("balanced", samples_per_pixel=5000, max_bounces=4, enable_denoise=0)
    r = Renderer()
    r.prepare_scene(sc.view)
    before = r.launch_grids()
    assert len(before) >= 13 and min(g for g, _ in before) > 0 and {b for _, b in before} <= {128, 256}
    with pytest.raises(abi.RtgbError):
        r.autotune_launches(rig, bad, 2, frames=1)
    assert r.launch_grids() == before
    r.render_frame(rig, good, 2)
    with pytest.raises(abi.RtgbError):
        r.stage_times()
    tuned = r.autotune_launches(rig, good, 2, frames=1)
    persistent = {"grid_scale": 1.0, "block": "kernel's"}
    assert r.launch_grids() != before or all(v == persistent for v in tuned["chosen"].values())
    r.close()
