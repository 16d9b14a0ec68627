"""Bounded device loops that give up report it, and the handle stays usable.

Every loop of the device code without a fixed trip count is bounded: BVH
traversal (node visits per ray) and the rejection sampler of
random_in_unit_sphere (draws). The defaults never bind on real inputs, so the
debug fields of rtgb_create_info shrink them until they do. A frame in which a
loop reached its bound must return RTGB_DEVICE_FAULT_FLAG with the count in
the error message; after the bounds are restored (rtgb_set_debug_limits) the
same handle renders a clean frame that traces exactly the paths of a handle
that never gave up. These are plain SIMT loops that stop and return; nothing
faults or waits on the GPU.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import scaled_rig
from ray_tracing_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

FAULT = 4  # RTGB_DEVICE_FAULT_FLAG


def _setup():
    sc = scenes.HostScene("random_spheres", detail=64)
    rig = scaled_rig(scenes.default_rig("random_spheres", 2), 0.1)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0, enable_restir_di=1,
                          restir_initial_candidates=8, restir_temporal_reuse=1, restir_spatial_neighbors=1)
    return sc, rig, prof


@pytest.mark.parametrize("limits", [{"debug_traversal_limit": 2}, {"debug_rejection_limit": 1}])
def test_a_loop_that_gives_up_flags_the_frame_and_the_next_frame_is_clean(limits):
    from ray_tracing_gb300.renderer import Renderer
    sc, rig, prof = _setup()
    clean = Renderer(debug_path_records=True)
    bounded = Renderer(debug_path_records=True, **limits)
    for r in (clean, bounded):
        r.prepare_scene(sc.view)
    with pytest.raises(abi.RtgbError) as info:
        bounded.render_frame(rig, prof, 2)
    assert info.value.status == FAULT
    assert "reached their bound" in str(info.value)
    bounded.set_debug_limits(0, 0)
    for r in (clean, bounded):
        r.reset_sequence(5)
        r.reset_accumulation()
        r.render_frame(rig, prof, 2)
    for cam in range(2):
        cc, cr = clean.path_records(cam, 1, 4)
        bc, br = bounded.path_records(cam, 1, 4)
        assert np.array_equal(cc, bc)
        assert np.array_equal(cr, br)
    clean.close()
    bounded.close()


def test_bounds_large_enough_for_the_scene_change_nothing():
    from ray_tracing_gb300.renderer import Renderer
    sc, rig, prof = _setup()
    plain = Renderer(debug_path_records=True)
    roomy = Renderer(debug_path_records=True, debug_traversal_limit=4096, debug_rejection_limit=4096)
    for r in (plain, roomy):
        r.prepare_scene(sc.view)
        for _ in range(2):
            r.render_frame(rig, prof, 2)
    for cam in range(2):
        assert np.array_equal(plain.path_records(cam, 1, 4)[0], roomy.path_records(cam, 1, 4)[0])
    plain.close()
    roomy.close()
