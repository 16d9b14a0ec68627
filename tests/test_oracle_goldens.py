"""The oracle against the reference's own golden images.

tests/golden/restir_di/{reference,baseline,restir}.png were rendered by the
reference's GPU renderer (utils/render_restir_acceptance.cpp) and are pinned by
sha256 in its manifest. The oracle re-renders the same scene, camera and
profiles and must match with the reference's own gate (max display error <= 2);
it matches every pixel exactly.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from _png import read_png
from oracle.binding import OracleRenderer
from ray_tracing_gb300 import scenes

GOLD = Path(__file__).resolve().parent / "golden" / "restir_di"


def test_golden_files_match_reference_manifest():
    manifest = json.loads((GOLD / "manifest.json").read_text())
    for image in manifest["images"]:
        assert hashlib.sha256((GOLD / image["path"]).read_bytes()).hexdigest() == image["sha256"]


def _oracle_frames():
    sc = scenes.HostScene("restir_acceptance")
    rig = scenes.default_rig("restir_acceptance", 1)
    out = {}
    r = OracleRenderer(sc.view)
    r.render_frame(rig, scenes.restir_acceptance_profile(256, False), 1)
    out["reference"] = r.buffer(0, "beauty")
    r = OracleRenderer(sc.view)
    r.render_frame(rig, scenes.restir_acceptance_profile(16, False), 1)
    out["baseline"] = r.buffer(0, "beauty")
    r = OracleRenderer(sc.view)
    for _ in range(2):
        r.render_frame(rig, scenes.restir_acceptance_profile(1, True), 1)
    out["restir"] = r.buffer(0, "beauty")
    out["_restir_reservoirs"] = r.reservoirs(0)
    return out


@pytest.fixture(scope="module")
def frames():
    return _oracle_frames()


@pytest.mark.parametrize("name", ["reference", "baseline", "restir"])
def test_oracle_matches_reference_golden(frames, name):
    golden = read_png(GOLD / f"{name}.png").astype(int)
    mine = scenes.display_u8(frames[name][..., :3]).astype(int)
    diff = np.abs(mine - golden)
    assert diff.max() <= 2, f"max display error {diff.max()}"
    assert int((diff > 0).sum()) == 0, "oracle reproduces the golden image exactly"


def test_oracle_restir_counters_follow_acceptance_gates(frames):
    res = frames["_restir_reservoirs"]
    valid = res["valid"] != 0
    assert valid.sum() > 0
    assert int(np.sum(valid & (res["temporal_candidate_count"] > 0))) > 0
    assert int(np.sum(valid & (res["spatial_candidate_count"] > 0))) > 0
    assert int(np.sum(valid & (res["bias_correction_source_count"] > 0))) > 0
