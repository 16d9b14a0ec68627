"""ReSTIR DI over emissive geometry (rtgb_render_profile::restir_emissive), GPU.

An extension without a reference counterpart (the reference resamples analytic
lights only), so there is no oracle to match path by path. What is checked:
the option is off by default and leaves the reference path untouched (the
parity tests run with it off); with it on, the reservoirs are live (initial
candidates, temporal and spatial reuse, BASIC bias correction all happen), the
frames are finite, and the accumulated image agrees with plain next-event
estimation in the mean (the estimator targets the same integral)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import equi, look_at, pinhole, rig_of
from ray_tracing_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rig():
    cams = [pinhole(96, 72, 90.0), equi(96, 80, 180.0)]
    for i, c in enumerate(cams):
        ang = np.radians(90.0 * i + 30.0)
        look_at(c, (0.0, 4.0, 0.0), (np.sin(ang), 3.6, np.cos(ang)), (0.0, 1.0, 0.0))
    return rig_of(*cams)


def _profile(emissive: bool):
    return scenes.profile("balanced", samples_per_pixel=1, max_bounces=3, enable_denoise=0, enable_restir_di=1,
                          restir_initial_candidates=16, restir_temporal_reuse=1, restir_spatial_neighbors=1,
                          restir_bias_correction=1, restir_emissive=int(emissive))


def _accumulate(sc, rig, prof, frames):
    from ray_tracing_gb300.renderer import Renderer
    r = Renderer()
    r.prepare_scene(sc.view)
    r.reset_sequence(3)
    for _ in range(frames):
        r.render_frame(rig, prof, 2)
    img = [r.download(c).beauty_rgba[..., :3].astype(np.float64) for c in range(2)]
    diag = [r.restir_diagnostics(c) for c in range(2)]
    r.close()
    return img, diag


def test_emissive_restir_is_live_and_agrees_with_nee_in_the_mean():
    sc = scenes.HostScene("triangle_terrain_pbr", detail=20000)
    rig = _rig()
    on, diag = _accumulate(sc, rig, _profile(True), 24)
    off, _ = _accumulate(sc, rig, _profile(False), 24)
    for c in range(2):
        assert np.isfinite(on[c]).all() and (on[c] >= 0.0).all()
        d = diag[c]
        assert d.active_reservoir_count > 0.3 * d.pixel_count
        assert d.temporal_reuse_count > 0 and d.spatial_reuse_count > 0 and d.bias_corrected_count > 0
        m_on, m_off = float(on[c].mean()), float(off[c].mean())
        assert abs(m_on - m_off) <= 0.05 * m_off, (c, m_on, m_off)
    sc.close()
