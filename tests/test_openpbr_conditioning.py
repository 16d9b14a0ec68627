"""How far one-ulp libm differences carry along OpenPBR paths (CPU).

The sm_103a path evaluates powf/expf/logf/sinf/cosf/acosf with CUDA's math
library, the oracle with the host's; the two differ in the last bit for some
arguments. This test builds a second oracle whose OpenPBR transcendental calls
are nudged by one ulp (oracle/ulp_perturb.h) and renders the OpenPBR gallery
with both. Discrete decisions stay the same on all but a few paths, and along
identical paths the radiance agrees to ~1e-7 for almost every path but reaches
~1e-4 on a handful: the GGX distribution term changes by 4 tan(theta)/alpha^2
per radian of half-vector change, so a one-ulp direction difference after a
few glossy bounces (alpha^2 ~ 4e-3 for roughness 0.25) is amplified that far.
The GPU-vs-oracle tolerance in test_openpbr_render.py rests on this
measurement.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import compare_paths
from ray_tracing_gb300 import build as _build
from ray_tracing_gb300 import scenes

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def perturbed_oracle(tmp_path_factory):
    out = tmp_path_factory.mktemp("orc_ulp") / "liborc_ulp.so"
    subprocess.run(["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    "-include", str(ROOT / "oracle" / "ulp_perturb.h"), "-I", str(_build.INCLUDE), "-I",
                    str(_build.CSRC), str(ROOT / "oracle" / "radiance_oracle.cpp"),
                    str(ROOT / "oracle" / "openpbr_kat.cpp"), "-o", str(out), "-lpthread"], check=True)
    return out


def _render(lib_path, rig, profile, spp, mb):
    import oracle.binding as ob
    saved_lib, saved_path = ob._lib, _build.ORACLE_LIB
    try:
        ob._lib = None
        _build.ORACLE_LIB = Path(lib_path)
        ob.load()
        sc = scenes.HostScene("openpbr_gallery")
        o = ob.OracleRenderer(sc.view)
        o.set_path_records(True)
        o.render_frame(rig, profile, 1)
        return o.path_records(0, spp, mb)
    finally:
        ob._lib, _build.ORACLE_LIB = saved_lib, saved_path


def test_one_ulp_libm_differences_along_openpbr_paths(perturbed_oracle):
    from test_openpbr_render import _profile
    spp, mb = 2, 8
    rig = scenes.default_rig("openpbr_gallery", 1, 96, 72)
    prof = _profile(False, spp, mb)
    ac, ar = _render(_build.ORACLE_LIB, rig, prof, spp, mb)
    bc, br = _render(perturbed_oracle, rig, prof, spp, mb)
    diverged, max_err, _ = compare_paths(ac, ar, bc, br)
    same = np.all(ac == bc, axis=1)
    err = (np.abs(ar - br) / np.maximum(np.abs(br), 1e-6))[same].max(axis=1)
    assert diverged < 5e-3
    assert np.quantile(err, 0.999) < 5e-5
    assert err.max() > 1e-6, "the perturbation did not reach the OpenPBR code"
    assert err.max() < 1e-3
