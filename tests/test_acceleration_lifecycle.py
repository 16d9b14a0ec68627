"""The acceleration lifecycle of rtgb_prepare_scene (GpuSceneAcceleration::update,
src/realtime/gpu/gpu_scene_acceleration.cpp:247-295, and its benchmark
utils/benchmark_gpu_scene_lifecycle.cpp): reuse when nothing changed, update
when only non-geometry data changed, refit when the primitive counts are
unchanged but geometry moved, rebuild otherwise; the generation counter
advances on every kind but reuse.

A refit keeps the leaf order and hierarchy of the last rebuild and rewrites
only the node boxes, so it is checked three ways: every node box equals the
union of the (new) primitive boxes below it, the paths traced through the
refitted hierarchy match the oracle on the moved scene, and they match a
renderer that rebuilt from scratch, bit for bit wherever the two hit the same
primitives. The 4-wide BVH the rays traverse (collapsed from the binary one)
is checked after builds and refits: every leaf once, every node reached once,
every child box the exact union of the primitive boxes below it.
"""
import numpy as np
import pytest

from helpers import compare_paths, scaled_rig
from ray_tracing_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

REUSE, UPDATE, REFIT, REBUILD = range(4)


def _kind(r):
    a = r.acceleration_info()
    return a.update_kind, a.generation


def _subtree_boxes(children, leaf_lo, leaf_hi):
    """Union box of every internal node (Karras encoding: child < 0 is sorted slot ~child)."""
    m = children.shape[0]
    lo = np.full((m, 3), np.inf, np.float32)
    hi = np.full((m, 3), -np.inf, np.float32)
    done = np.zeros(m, bool)
    stack = [0]
    while stack:
        node = stack[-1]
        pending = [int(c) for c in children[node] if c >= 0 and not done[c]]
        if pending:
            stack.extend(pending)
            continue
        stack.pop()
        for c in children[node]:
            clo, chi = (leaf_lo[~c], leaf_hi[~c]) if c < 0 else (lo[c], hi[c])
            lo[node] = np.minimum(lo[node], clo)
            hi[node] = np.maximum(hi[node], chi)
        done[node] = True
    return lo, hi


def _child_box(c, lo, hi, leaf_lo, leaf_hi):
    return (leaf_lo[~c], leaf_hi[~c]) if c < 0 else (lo[c], hi[c])


def _move_spheres(view, amplitude):
    for i in range(view.sphere_count):
        s = view.spheres[i]
        s.center[0] += amplitude * np.sin(1.7 * i)
        s.center[1] += amplitude * np.cos(0.9 * i)


def _render(r, rig, prof, frames=1):
    for _ in range(frames):
        r.render_frame(rig, prof, rig.active_count)


def test_reuse_update_rebuild_kinds_and_generation():
    from ray_tracing_gb300.renderer import Renderer
    sc = scenes.HostScene("cornell_box")
    r = Renderer()
    r.prepare_scene(sc.view)
    assert _kind(r) == (REBUILD, 1)
    r.prepare_scene(sc.view)
    assert _kind(r) == (REUSE, 1)
    # a texture colour: non-geometry data, the hierarchy stays
    sc.view.textures[0].color[0] *= 0.5
    r.prepare_scene(sc.view)
    assert _kind(r) == (UPDATE, 2)
    sc.view.background[2] += 0.25
    r.prepare_scene(sc.view)
    assert _kind(r) == (UPDATE, 3)
    r.prepare_scene(sc.view)
    assert _kind(r) == (REUSE, 3)
    # fewer quads: the topology changed
    sc.view.quad_count -= 1
    r.prepare_scene(sc.view)
    assert _kind(r) == (REBUILD, 4)
    sc.view.quad_count += 1
    r.prepare_scene(sc.view)
    assert _kind(r) == (REBUILD, 5)
    # an invalid scene is refused before any state changes
    bad = abi.Scene()
    with pytest.raises(Exception):
        r.prepare_scene(bad)
    r.prepare_scene(sc.view)
    assert _kind(r) == (REUSE, 5)


def test_update_renders_the_new_materials():
    from oracle.binding import OracleRenderer
    from ray_tracing_gb300.renderer import Renderer
    rig = scaled_rig(scenes.default_rig("cornell_box", 1), 0.25)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_restir_di=0, enable_denoise=0)
    sc = scenes.HostScene("cornell_box")
    r = Renderer(debug_path_records=True)
    r.prepare_scene(sc.view)
    _render(r, rig, prof)
    before = r.download(0).beauty_rgba.copy()
    for t in range(sc.view.texture_count):
        for k in range(3):
            sc.view.textures[t].color[k] *= 0.6
    r.prepare_scene(sc.view)
    assert _kind(r)[0] == UPDATE
    _render(r, rig, prof)
    orc = OracleRenderer(sc.view)
    orc.set_path_records(True)
    _render(orc, rig, prof)
    gc, gr = r.path_records(0, 1, 4)
    oc, orad = orc.path_records(0, 1, 4)
    # 64x64 paths: a dozen land on the box's corner edges, equal-t ties
    diverged, max_err, bad = compare_paths(gc, gr, oc, orad)
    assert diverged <= 5e-3 and bad == 0, (diverged, max_err, bad)
    # the updated renderer is the one a fresh prepare of the new scene gives
    fresh = Renderer(debug_path_records=True)
    fresh.prepare_scene(sc.view)
    _render(fresh, rig, prof)
    fc, fr = fresh.path_records(0, 1, 4)
    assert np.array_equal(gc, fc) and np.array_equal(gr, fr)
    assert not np.array_equal(before, r.download(0).beauty_rgba)


@pytest.mark.parametrize("amplitude", [0.05, 0.6])
def test_refit_boxes_paths_and_rebuilt_equivalence(amplitude):
    from oracle.binding import OracleRenderer
    from oracle.lbvh import primitive_boxes
    from ray_tracing_gb300.renderer import Renderer
    rig = scaled_rig(scenes.default_rig("random_spheres", 2), 0.125)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, restir_initial_candidates=8,
                          enable_denoise=0)
    sc = scenes.HostScene("random_spheres", detail=256)
    r = Renderer(debug_path_records=True)
    r.prepare_scene(sc.view)
    _render(r, rig, prof)
    keys0, order0, children0 = r.lbvh()

    _move_spheres(sc.view, amplitude)
    r.prepare_scene(sc.view)
    assert _kind(r) == (REFIT, 2)
    keys1, order1, children1 = r.lbvh()
    assert np.array_equal(order0, order1) and np.array_equal(children0, children1)

    # every child box is the exact union of the moved primitive boxes below it
    lo, hi = primitive_boxes(sc.view)
    leaf_lo, leaf_hi = lo[order1], hi[order1]
    nlo, nhi = _subtree_boxes(children1, leaf_lo, leaf_hi)
    boxes = r.lbvh_boxes()
    for node in range(children1.shape[0]):
        for k in range(2):
            blo, bhi = _child_box(int(children1[node, k]), nlo, nhi, leaf_lo, leaf_hi)
            assert np.array_equal(boxes[node, k, 0], blo) and np.array_equal(boxes[node, k, 1], bhi), node

    _render(r, rig, prof, frames=2)
    fresh = Renderer(debug_path_records=True)
    fresh.prepare_scene(sc.view)
    assert _kind(fresh) == (REBUILD, 1)
    _render(fresh, rig, prof, frames=2)
    orc = OracleRenderer(sc.view)
    orc.set_path_records(True)
    _render(orc, rig, prof, frames=2)
    for cam in range(2):
        gc, gr = r.path_records(cam, 1, 4)
        fc, fr = fresh.path_records(cam, 1, 4)
        same = np.all(gc == fc, axis=1)
        assert 1.0 - same.mean() <= 1e-3
        assert np.array_equal(gr[same], fr[same])
        oc, orad = orc.path_records(cam, 1, 4)
        diverged, max_err, bad = compare_paths(gc, gr, oc, orad)
        assert diverged <= 2e-3 and bad == 0, (cam, diverged, max_err, bad)
    assert r.acceleration_info().traversal_stack_overflows == 0


def _check_bvh4(r, view):
    """Every leaf slot once, every node reached once from the root, every child
    box the exact union of the primitive boxes below it."""
    from oracle.lbvh import primitive_boxes
    _, order, _ = r.lbvh()
    children, boxes = r.bvh4()
    lo, hi = primitive_boxes(view)
    leaf_lo, leaf_hi = lo[order], hi[order]
    n4 = children.shape[0]
    empty = np.iinfo(np.int32).min
    seen_leaves = np.zeros(len(order), np.int32)
    seen_nodes = np.zeros(n4, np.int32)
    seen_nodes[0] = 1
    for i in range(n4):
        for k in range(4):
            c = int(children[i, k])
            if c == empty:
                continue
            if c >= 0:
                assert c > i, "children follow their parent (breadth-first)"
                seen_nodes[c] += 1
            else:
                seen_leaves[~c] += 1
    assert np.all(seen_leaves == 1) and np.all(seen_nodes == 1)
    # subtree unions, children before parents (reverse breadth-first order)
    ulo = np.zeros((n4, 3), np.float32)
    uhi = np.zeros((n4, 3), np.float32)
    for i in range(n4 - 1, -1, -1):
        cl, ch = [], []
        for k in range(4):
            c = int(children[i, k])
            if c == empty:
                continue
            blo, bhi = (ulo[c], uhi[c]) if c >= 0 else (leaf_lo[~c], leaf_hi[~c])
            assert np.array_equal(boxes[i, 0, :, k], blo) and np.array_equal(boxes[i, 1, :, k], bhi), (i, k)
            cl.append(blo)
            ch.append(bhi)
        ulo[i] = np.min(cl, axis=0)
        uhi[i] = np.max(ch, axis=0)
    return n4


@pytest.mark.parametrize("name,detail", [("random_spheres", 256), ("triangle_terrain", 20000), ("cornell_box", 0)])
def test_wide_bvh_structure_after_build_and_refit(name, detail):
    from ray_tracing_gb300.renderer import Renderer
    sc = scenes.HostScene(name, detail=detail)
    r = Renderer()
    r.prepare_scene(sc.view)
    n = sc.view.sphere_count + sc.view.quad_count + sc.view.triangle_count
    n4 = _check_bvh4(r, sc.view)
    assert (n - 1) // 3 <= n4 <= n - 1
    if sc.view.sphere_count:
        _move_spheres(sc.view, 0.3)
        r.prepare_scene(sc.view)
        assert _kind(r)[0] == REFIT
        assert _check_bvh4(r, sc.view) == n4
