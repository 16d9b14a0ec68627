"""Known-answer tests of the oracle's shared math, with the expected values of
the reference's own unit tests (tests/test_restir_di.cpp:30-110,
tests/test_light_sampling.cpp:48-67, :146-153)."""
import ctypes as C

import numpy as np
import pytest

from oracle.binding import load
from ray_tracing_gb300 import abi

lib = load()


def res():
    return np.zeros(1, dtype=abi.RESERVOIR_DTYPE)


def upd(r, light, target, weight, u, mult=1, u0=0.25, u1=0.75):
    return lib.orc_reservoir_update(r.ctypes.data, light, u0, u1, target, weight, mult, u)


def surface_into(r, x=0.0, material=5, prim=7):
    r["position"] = (x, 0.0, 2.0)
    r["normal"] = (0.0, 0.0, 1.0)
    r["material_type"] = material
    r["primitive_type"] = 2
    r["primitive_index"] = prim


def test_weighted_replacement_and_finalize():
    r = res()
    upd(r, 3, 1.0, 1.0, 0.0)
    upd(r, 9, 3.0, 3.0, 0.99)
    upd(r, 11, 0.0, 0.0, 0.5)
    lib.orc_reservoir_finalize(r.ctypes.data)
    assert r["valid"][0] != 0 and r["light_index"][0] == 3 and r["candidate_count"][0] == 3
    assert r["weight_sum"][0] == pytest.approx(4.0, abs=1e-7)
    assert r["estimator_weight"][0] == pytest.approx(4.0 / 3.0, abs=1e-7)


def previous():
    p = res()
    p["light_index"], p["u0"], p["u1"] = 21, 0.1, 0.2
    surface_into(p)
    p["weight_sum"], p["selected_target"], p["estimator_weight"] = 16.0, 4.0, 0.5
    p["candidate_count"], p["age"], p["valid"] = 8, 3, 1
    return p


def test_temporal_merge():
    m = res()
    upd(m, 4, 1.0, 2.0, 0.0)
    out = (C.c_int * 2)()
    lib.orc_reservoir_merge(m.ctypes.data, previous().ctypes.data, 2.0, 4, 0.0, 1, out)
    surface_into(m)
    lib.orc_reservoir_finalize(m.ctypes.data)
    assert m["light_index"][0] == 21 and m["candidate_count"][0] == 5 and m["temporal_candidate_count"][0] == 4
    assert out[0] == 4 and out[1] != 0 and m["age"][0] == 4
    assert m["weight_sum"][0] == pytest.approx(6.0, abs=1e-7)
    assert m["estimator_weight"][0] == pytest.approx(0.6, abs=1e-7)


def test_spatial_merge():
    s = res()
    upd(s, 4, 1.0, 2.0, 0.0)
    out = (C.c_int * 2)()
    lib.orc_reservoir_merge(s.ctypes.data, previous().ctypes.data, 2.0, 3, 0.0, 0, out)
    lib.orc_reservoir_finalize(s.ctypes.data)
    assert s["candidate_count"][0] == 4 and s["spatial_candidate_count"][0] == 3
    assert s["temporal_candidate_count"][0] == 0 and out[0] == 3 and out[1] != 0
    assert s["weight_sum"][0] == pytest.approx(5.0, abs=1e-7)
    assert s["estimator_weight"][0] == pytest.approx(0.625, abs=1e-7)


def test_basic_bias_correction():
    c = res()
    c["light_index"], c["weight_sum"], c["selected_target"], c["candidate_count"], c["valid"] = 8, 10.0, 2.0, 5, 1
    lib.orc_reservoir_finalize_basic(c.ctypes.data, 3.0, 12.0, 2)
    assert c["valid"][0] != 0 and c["bias_correction_source_count"][0] == 2
    assert c["estimator_weight"][0] == pytest.approx(1.25, abs=1e-7)


def test_temporal_surface_validity():
    p = previous()
    cur = res()
    surface_into(cur)

    def valid(surface):
        return lib.orc_surface_valid(surface["position"].ctypes.data if False else surf_ptr(surface), p.ctypes.data,
                                     0.01, 0.95, 20)

    def surf_ptr(r):
        return r.ctypes.data + 12  # RestirSurface starts after the 12-byte candidate

    assert lib.orc_surface_valid(surf_ptr(cur), p.ctypes.data, 0.01, 0.95, 20) == 1
    moved = res(); surface_into(moved, x=0.02)
    assert lib.orc_surface_valid(surf_ptr(moved), p.ctypes.data, 0.01, 0.95, 20) == 0
    flipped = res(); surface_into(flipped); flipped["normal"] = (0.0, 0.0, -1.0)
    assert lib.orc_surface_valid(surf_ptr(flipped), p.ctypes.data, 0.01, 0.95, 20) == 0
    other_mat = res(); surface_into(other_mat, material=0)
    assert lib.orc_surface_valid(surf_ptr(other_mat), p.ctypes.data, 0.01, 0.95, 20) == 0
    other_prim = res(); surface_into(other_prim, prim=8)
    assert lib.orc_surface_valid(surf_ptr(other_prim), p.ctypes.data, 0.01, 0.95, 20) == 0
    p["age"] = 20
    assert lib.orc_surface_valid(surf_ptr(cur), p.ctypes.data, 0.01, 0.95, 20) == 0


def test_light_cdf_boundaries():
    cdf = (C.c_float * 3)(0.2, 0.5, 1.0)
    assert [lib.orc_sample_cdf(cdf, 3, u) for u in (0.0, 0.2, 0.5, 1.0)] == [0, 1, 2, 2]
    acdf = (C.c_float * 3)(0.25, 0.75, 1.0)
    assert [lib.orc_sample_cdf(acdf, 3, u) for u in (0.0, 0.25, 0.75, 1.0)] == [0, 1, 2, 2]
    assert lib.orc_sample_cdf(None, 0, 0.5) == -1


def test_pdf_normalisations_and_power_heuristic():
    assert lib.orc_area_pdf(2.0, 8.0, 0.5) == pytest.approx(8.0, abs=1e-6)
    assert lib.orc_power_heuristic(0.25, 0.25) == pytest.approx(0.5, abs=1e-6)
    assert lib.orc_power_heuristic(0.2, 0.7) + lib.orc_power_heuristic(0.7, 0.2) == pytest.approx(1.0, abs=1e-6)
    assert lib.orc_power_heuristic(0.0, 1.0) == 0.0
    # uniform cone pdf integrates to 1 over its solid angle
    assert lib.orc_uniform_cone_pdf(0.5) * 2 * np.pi * 0.5 == pytest.approx(1.0, abs=1e-6)


def test_rng_is_the_reference_hashed_pixel_sample_stream():
    # hash_u32(pixel*1973 ^ (sample+1)*9277 ^ (stream+1)*26699 ^ 0x9e3779b9), then LCG 1664525/1013904223
    def hash_u32(x):
        x &= 0xFFFFFFFF
        x ^= x >> 16; x = (x * 0x7feb352d) & 0xFFFFFFFF
        x ^= x >> 15; x = (x * 0x846ca68b) & 0xFFFFFFFF
        x ^= x >> 16
        return x
    for pixel, sample, stream in ((0, 0, 0), (12345, 3, 7), (307199, 63, 20260718)):
        seed = ((pixel * 1973) ^ ((sample + 1) * 9277) ^ (((stream + 1) & 0xFFFFFFFF) * 26699) ^ 0x9e3779b9) & 0xFFFFFFFF
        assert lib.orc_rng_for(pixel, sample, stream) == hash_u32(seed)
    s = C.c_uint32(1)
    v = lib.orc_rnd(C.byref(s))
    assert s.value == (1 * 1664525 + 1013904223) & 0xFFFFFFFF
    assert v == pytest.approx((s.value & 0xFFFFFF) / 16777216.0, abs=0)
