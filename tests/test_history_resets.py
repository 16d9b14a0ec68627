"""History resets of the temporal path (tests/test_optix_temporal_reference.cpp:
190-240 of the reference): after a resize, and after reset_accumulation
following a camera jump, the next frame must equal a cold start with the same
sample stream (the reference's bound: 1e-6). Checked on the oracle, whose
frame sequencing restates optix_renderer.cpp:230-277; the GPU path's own
multi-frame sequences are compared with it in test_gpu_parity.py. CPU only."""
from __future__ import annotations

import numpy as np

from ray_tracing_gb300 import scenes

HISTORY = 3


def _beauty(orc, cam=0):
    return orc.buffer(cam, "beauty").astype(np.float64)


def _fresh(sc, rig, prof, stream):
    from oracle.binding import OracleRenderer
    orc = OracleRenderer(sc.view, use_reference_bvh=True)
    orc.reset_sequence(stream)
    orc.render_frame(rig, prof, 1)
    out = _beauty(orc)
    orc.close()
    return out


def test_resize_and_camera_jump_restart_history():
    from oracle.binding import OracleRenderer
    sc = scenes.HostScene("cornell_box")
    prof = scenes.profile("realtime", samples_per_pixel=2, max_bounces=3, enable_denoise=0)
    rig_a = scenes.default_rig("cornell_box", 1, 32, 24)
    rig_small = scenes.default_rig("cornell_box", 1, 24, 18)
    rig_jump = scenes.orbit_rig(rig_a, 25.0, center=(278.0, 278.0, 278.0))

    orc = OracleRenderer(sc.view, use_reference_bvh=True)
    orc.reset_sequence(300)
    for _ in range(HISTORY):
        orc.render_frame(rig_a, prof, 1)
    orc.render_frame(rig_small, prof, 1)
    resized = _beauty(orc)
    orc.close()
    assert np.abs(resized - _fresh(sc, rig_small, prof, 300 + HISTORY)).max() <= 1e-6

    orc = OracleRenderer(sc.view, use_reference_bvh=True)
    orc.reset_sequence(500)
    for _ in range(HISTORY):
        orc.render_frame(rig_a, prof, 1)
    orc.reset_accumulation()
    orc.render_frame(rig_jump, prof, 1)
    jumped = _beauty(orc)
    orc.close()
    assert np.abs(jumped - _fresh(sc, rig_jump, prof, 500 + HISTORY)).max() <= 1e-6

    # a small move without a reset keeps the history: the frame differs from a cold start
    rig_nudge = scenes.orbit_rig(rig_a, 0.5, center=(278.0, 278.0, 278.0))
    orc = OracleRenderer(sc.view, use_reference_bvh=True)
    orc.reset_sequence(700)
    for _ in range(HISTORY):
        orc.render_frame(rig_a, prof, 1)
    orc.render_frame(rig_nudge, prof, 1)
    nudged = _beauty(orc)
    orc.close()
    assert np.abs(nudged - _fresh(sc, rig_nudge, prof, 700 + HISTORY)).max() > 1e-3
