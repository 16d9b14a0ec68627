"""OpenPBR BSDF known-answer tests (CPU).

tests/golden/openpbr/kats.npz holds 1536 seeded records answered by the
reference's own src/common/openpbr_core.h (compiled here by
oracle/build_ref.py; generator: tests/golden/make_openpbr_kats.py). The
repository's restatement (ray_tracing_gb300/csrc/openpbr.h, host build inside
the oracle library) must give the same 32-bit words for every output:
evaluate, sample, lobe probabilities, emission, subsurface medium and segment,
Henyey-Greenstein sampling, shading frames, sRGB decoding and boundary sampling.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import binding

GOLDEN = Path(__file__).resolve().parent / "golden" / "openpbr" / "kats.npz"
KAT_IN, KAT_OUT = 80, 64
EVENTS = ["none", "diffuse_reflection", "glossy_reflection", "glossy_transmission", "thin_walled_transmission",
          "opacity_passthrough", "coat_reflection", "fuzz_reflection", "subsurface_entry", "subsurface_exit"]


@pytest.fixture(scope="module")
def kats():
    d = np.load(GOLDEN)
    lib = binding.load()
    fn = lib.orc_openpbr_kat
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    inputs = np.ascontiguousarray(d["inputs"])
    out = np.zeros((inputs.shape[0], KAT_OUT), dtype=np.float32)
    assert fn(inputs.ctypes.data, inputs.shape[0], out.ctypes.data) == (KAT_IN << 16) | KAT_OUT
    return inputs, d["outputs"], out


def test_fixture_shape(kats):
    inputs, ref, _ = kats
    assert inputs.shape == (1536, KAT_IN) and ref.shape == (1536, KAT_OUT)


@pytest.mark.parametrize("name,cols", [
    ("evaluate", slice(0, 4)), ("sample", slice(4, 18)), ("lobes", slice(18, 30)), ("emission", slice(30, 33)),
    ("medium", slice(33, 41)), ("segment", slice(41, 46)), ("henyey_greenstein", slice(46, 49)),
    ("frame", slice(49, 58)), ("srgb", slice(58, 59)), ("boundary_sample", slice(59, 64)),
])
def test_bit_exact_against_reference_header(kats, name, cols):
    _, ref, out = kats
    a = out[:, cols].view(np.uint32)
    b = ref[:, cols].view(np.uint32)
    bad = np.argwhere(a != b)
    assert bad.size == 0, f"{name}: {len(bad)} words differ, first at record {bad[0][0]}"


def test_every_scatter_event_is_covered(kats):
    _, ref, _ = kats
    events = np.bincount(ref[:, 15].view(np.int32), minlength=len(EVENTS))
    assert all(events[i] > 0 for i in range(len(EVENTS))), dict(zip(EVENTS, events.tolist()))
    assert ref[:, 40].view(np.int32).sum() > 0 and ref[:, 45].view(np.int32).sum() > 0
