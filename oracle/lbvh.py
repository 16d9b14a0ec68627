"""CPU restatement of the device LBVH build — TEST INFRASTRUCTURE ONLY.

Follows ray_tracing_gb300/csrc/lbvh.cu and renderer.cu (k_prim_records)
operation for operation in float32/uint32 numpy arithmetic: padded primitive
boxes, centroid bounds, 30-bit Morton codes, a stable sort by code (ties by
primitive index) and the Karras (2012) hierarchy with the index tie-break.
The reference itself has no LBVH (its host BVH is a median split,
src/realtime/gpu/gpu_scene_acceleration.cpp:145-179), so this restatement is
what pins the device build bit for bit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ray_tracing_gb300 import abi

F = np.float32


def _arr(ptr, count, ctype):
    if count == 0:
        return np.zeros(0, dtype=np.dtype(ctype))
    buf = (ctype * count).from_address(C.addressof(ptr.contents))
    return np.frombuffer(buf, dtype=np.dtype(ctype)).copy()


def primitive_boxes(scene: abi.Scene):
    """Padded boxes of spheres, quads, triangles (k_prim_records)."""
    sph = _arr(scene.spheres, scene.sphere_count, abi.Sphere) if scene.sphere_count else None
    qd = _arr(scene.quads, scene.quad_count, abi.Quad) if scene.quad_count else None
    tr = _arr(scene.triangles, scene.triangle_count, abi.Triangle) if scene.triangle_count else None
    los, his = [], []
    scale = F(0.0)
    if sph is not None:
        c = sph["center"].astype(F)
        r = np.abs(sph["radius"].astype(F))[:, None]
        los.append(c - r)
        his.append(c + r)
        scale = max(scale, F(np.max(np.abs(c) + r)))
    if qd is not None:
        o, u, v = (qd[k].astype(F) for k in ("origin", "edge_u", "edge_v"))
        p1, p2 = o + u, o + v
        p3 = (o + u) + v
        los.append(np.minimum(np.minimum(o, p1), np.minimum(p2, p3)))
        his.append(np.maximum(np.maximum(o, p1), np.maximum(p2, p3)))
        scale = max(scale, F(np.max((np.abs(o) + np.abs(u)) + np.abs(v))))
    if tr is not None:
        p0, p1, p2 = (tr[k].astype(F) for k in ("p0", "p1", "p2"))
        los.append(np.minimum(np.minimum(p0, p1), p2))
        his.append(np.maximum(np.maximum(p0, p1), p2))
        scale = max(scale, F(np.max(np.maximum(np.maximum(np.abs(p0), np.abs(p1)), np.abs(p2)))))
    lo = np.concatenate(los).astype(F)
    hi = np.concatenate(his).astype(F)
    pad = F(F(1e-5) + F(F(1e-5) * scale))
    return (lo - pad).astype(F), (hi + pad).astype(F)


def _expand_bits10(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint32)
    v = (v * np.uint32(0x00010001)) & np.uint32(0xFF0000FF)
    v = (v * np.uint32(0x00000101)) & np.uint32(0x0F00F00F)
    v = (v * np.uint32(0x00000011)) & np.uint32(0xC30C30C3)
    v = (v * np.uint32(0x00000005)) & np.uint32(0x49249249)
    return v


def _quantize10(c, lo, hi):
    extent = F(hi - lo)
    scale = F(F(1024.0) / extent) if extent > 0 else F(0.0)
    q = ((c - lo) * scale).astype(F)
    q = np.clip(q, F(0.0), F(1023.0))
    return q.astype(np.uint32)


def morton_codes(lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
    cen = ((lo + hi) * F(0.5)).astype(F)
    blo, bhi = cen.min(axis=0), cen.max(axis=0)
    with np.errstate(over="ignore"):
        x = _expand_bits10(_quantize10(cen[:, 0], blo[0], bhi[0]))
        y = _expand_bits10(_quantize10(cen[:, 1], blo[1], bhi[1]))
        z = _expand_bits10(_quantize10(cen[:, 2], blo[2], bhi[2]))
        return ((x << np.uint32(2)) | (y << np.uint32(1)) | z).astype(np.uint32)


def _clz32(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64)
    out = np.full(x.shape, 32, dtype=np.int64)
    nz = x > 0
    _, e = np.frexp(x[nz].astype(np.float64))
    out[nz] = 32 - e
    return out


def karras(keys: np.ndarray) -> np.ndarray:
    """Children of the n-1 internal nodes (c >= 0 internal, c < 0 leaf ~c)."""
    n = keys.size
    keys = keys.astype(np.uint32)
    i = np.arange(n - 1, dtype=np.int64)

    def delta(a, b):
        out = np.full(a.shape, -1, dtype=np.int64)
        ok = (b >= 0) & (b < n)
        ka, kb = keys[a[ok]], keys[b[ok]]
        eq = ka == kb
        v = np.empty(ka.shape, dtype=np.int64)
        v[eq] = 32 + _clz32((a[ok][eq] ^ b[ok][eq]).astype(np.uint32))
        v[~eq] = _clz32(ka[~eq] ^ kb[~eq])
        out[ok] = v
        return out

    d = np.where(delta(i, i + 1) - delta(i, i - 1) >= 0, 1, -1)
    dmin = delta(i, i - d)
    lmax = np.full(i.shape, 2, dtype=np.int64)
    grow = delta(i, i + lmax * d) > dmin
    while grow.any():
        lmax[grow] *= 2
        grow = delta(i, i + lmax * d) > dmin
    l = np.zeros_like(i)
    t = lmax // 2
    while (t >= 1).any():
        act = t >= 1
        cand = delta(i, i + (l + t) * d) > dmin
        l = np.where(act & cand, l + t, l)
        t = t // 2
    j = i + l * d
    dnode = delta(i, j)
    s = np.zeros_like(i)
    t = l.copy()
    while True:
        t = (t + 1) // 2
        cand = delta(i, i + (s + t) * d) > dnode
        s = np.where(cand, s + t, s)
        if not (t > 1).any():
            break
        # nodes whose t already reached 1 must not iterate again
        done = t <= 1
        t = np.where(done, 0, t)
        if done.all():
            break
    gamma = i + s * d + np.minimum(d, 0)
    lo, hi = np.minimum(i, j), np.maximum(i, j)
    left = np.where(lo == gamma, ~gamma, gamma)
    right = np.where(hi == gamma + 1, ~(gamma + 1), gamma + 1)
    return np.stack([left, right], axis=1).astype(np.int32)


def lbvh_reference(scene: abi.Scene):
    lo, hi = primitive_boxes(scene)
    codes = morton_codes(lo, hi)
    order = np.argsort(codes, kind="stable").astype(np.int32)
    keys = codes[order]
    return keys, order, karras(keys)
