"""Copies the reference's ReSTIR DI acceptance goldens into tests/golden/restir_di.

Source: tests/references/restir_di/{reference,baseline,restir}.png and
manifest.json of the reference project (rendered by its GPU renderer through
utils/render_restir_acceptance.cpp). Each image is verified against the sha256
recorded in the reference's manifest before it is copied.
"""
import hashlib
import json
import os
import shutil
import sys
from pathlib import Path

# the reference checkout: first argument, else RTGB_REFERENCE_ROOT (as oracle/build_ref.py)
SRC = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ["RTGB_REFERENCE_ROOT"]) / "tests/references/restir_di"
DST = Path(__file__).resolve().parent / "restir_di"

manifest = json.loads((SRC / "manifest.json").read_text())
DST.mkdir(exist_ok=True)
for image in manifest["images"]:
    data = (SRC / image["path"]).read_bytes()
    if hashlib.sha256(data).hexdigest() != image["sha256"]:
        raise SystemExit(f"sha256 mismatch for {image['path']}")
    (DST / image["path"]).write_bytes(data)
shutil.copyfile(SRC / "manifest.json", DST / "manifest.json")
print("copied", [i["path"] for i in manifest["images"]])
