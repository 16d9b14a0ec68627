"""rtgb_build_lbvh_static (the allocation-free LBVH build) against the
regular path: the Morton codes, leaf order and hierarchy it writes for a
scene's primitive boxes must equal what rtgb_prepare_scene builds and
rtgb_download_lbvh returns, call after call, and every node's inline child
boxes must be the exact union of its subtree. Collected last so it also runs
after every other GPU test in the same process."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi, scenes

SCENES = (("triangle_terrain", 30000), ("cornell_box", 0), ("random_spheres", 64))


def _boxes(scene):
    from oracle.lbvh import primitive_boxes
    lo, hi = primitive_boxes(scene)
    n = lo.shape[0]
    lo4 = np.zeros((n, 4), np.float32)
    hi4 = np.zeros((n, 4), np.float32)
    lo4[:, :3] = lo
    hi4[:, :3] = hi
    return lo4, hi4


def _static_build(lib, lo4, hi4):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    n = lo4.shape[0]
    t_lo = torch.from_numpy(lo4).to(dev)
    t_hi = torch.from_numpy(hi4).to(dev)
    keys = torch.empty(n, dtype=torch.int32, device=dev)
    order = torch.empty(n, dtype=torch.int32, device=dev)
    children = torch.empty((n - 1, 2), dtype=torch.int32, device=dev)
    nodes = torch.empty((n - 1, 16), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    msg = C.create_string_buffer(256)
    st = lib.rtgb_build_lbvh_static(0, t_lo.data_ptr(), t_hi.data_ptr(), n, keys.data_ptr(), order.data_ptr(),
                                    children.data_ptr(), nodes.data_ptr(), C.c_void_p(stream.cuda_stream), msg, 256)
    assert st == 0, f"{abi.STATUS_NAMES.get(st)}: {msg.value.decode()}"
    torch.cuda.synchronize(dev)
    return (keys.cpu().numpy().view(np.uint32), order.cpu().numpy(), children.cpu().numpy(),
            nodes.cpu().numpy())


def _check_node_boxes(lo4, hi4, order, children, nodes):
    n = lo4.shape[0]
    sub_lo = np.zeros((n - 1, 3), np.float32)
    sub_hi = np.zeros((n - 1, 3), np.float32)
    done = np.zeros(n - 1, bool)

    def child_box(c):
        if c < 0:
            k = order[~c]
            return lo4[k, :3], hi4[k, :3]
        return sub_lo[c], sub_hi[c]

    stack = [0]
    while stack:
        i = stack[-1]
        pending = [int(c) for c in children[i] if c >= 0 and not done[c]]
        if pending:
            stack.extend(pending)
            continue
        stack.pop()
        if done[i]:
            continue
        (l0, h0), (l1, h1) = child_box(children[i][0]), child_box(children[i][1])
        sub_lo[i] = np.minimum(l0, l1)
        sub_hi[i] = np.maximum(h0, h1)
        done[i] = True
        row = nodes[i]
        assert np.array_equal(row[0:3], l0) and np.array_equal(row[4:7], h0), f"node {i}: left child box"
        assert np.array_equal(row[8:11], l1) and np.array_equal(row[12:15], h1), f"node {i}: right child box"
        bits = row.view(np.int32)
        assert bits[3] == children[i][0] and bits[7] == children[i][1], f"node {i}: child links"
    assert done.all(), "hierarchy does not reach every internal node from the root"


@pytest.mark.gpu
def test_static_lbvh_matches_the_prepare_scene_build():
    from ray_tracing_gb300.renderer import Renderer
    lib = abi.load()
    expected = {}
    for name, detail in SCENES:
        sc = scenes.HostScene(name, detail=detail)
        r = Renderer()
        r.prepare_scene(sc.view)
        expected[name] = (_boxes(sc.view), r.lbvh())
    # the first scene twice in a row, then the others, then the first again
    for name in [SCENES[0][0], SCENES[0][0], SCENES[1][0], SCENES[2][0], SCENES[0][0]]:
        (lo4, hi4), (keys, order, children) = expected[name]
        s_keys, s_order, s_children, s_nodes = _static_build(lib, lo4, hi4)
        assert np.array_equal(s_keys, keys), f"{name}: Morton codes differ"
        assert np.array_equal(s_order, order), f"{name}: leaf order differs"
        assert np.array_equal(s_children, children), f"{name}: hierarchy differs"
        _check_node_boxes(lo4, hi4, s_order, s_children, s_nodes)


def test_static_lbvh_rejects_sizes_beyond_its_scratch():
    """Size checks come before any CUDA call, so this runs without a GPU too."""
    lib = abi.load()
    msg = C.create_string_buffer(256)
    st = lib.rtgb_build_lbvh_static(0, None, None, abi.STATIC_LBVH_MAX_PRIMITIVES + 1, None, None, None, None,
                                    None, msg, 256)
    assert st == 1
    assert b"static scratch limit" in msg.value
    st = lib.rtgb_build_lbvh_static(0, None, None, 1, None, None, None, None, None, msg, 256)
    assert st == 1 and msg.value


def test_static_limit_matches_the_header():
    import re
    from pathlib import Path
    text = (Path(__file__).resolve().parent.parent / "include" / "rtgb.h").read_text()
    m = re.search(r"#define RTGB_STATIC_LBVH_MAX_PRIMITIVES (\d+)", text)
    assert m and int(m.group(1)) == abi.STATIC_LBVH_MAX_PRIMITIVES
