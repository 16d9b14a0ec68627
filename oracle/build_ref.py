"""Builds the reference-side known-answer drivers into oracle/_ref/ — TEST INFRASTRUCTURE.

The reference's OpenPBR BSDF (src/common/openpbr_core.h) is a self-contained
header (it includes only <cmath>), so it is compiled straight from where it lies
under the read-only reference checkout together with oracle/openpbr_kat.cpp
(built with -DKAT_REFERENCE). Output: oracle/_ref/libopenpbr_ref.so exporting
ref_openpbr_kat. Nothing is written outside oracle/_ref/. When the reference
checkout is absent (as on a machine that only runs the committed fixtures) the
script does nothing and exits 0.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("RTGB_REFERENCE_ROOT", "/root/reference"))
OUT = HERE / "_ref"
FLAGS = ["-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def build() -> Path | None:
    header_dir = REFERENCE / "src" / "common"
    if not (header_dir / "openpbr_core.h").exists():
        return None
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libopenpbr_ref.so"
    src = HERE / "openpbr_kat.cpp"
    deps = [src, header_dir / "openpbr_core.h"]
    if not lib.exists() or any(d.stat().st_mtime > lib.stat().st_mtime for d in deps):
        subprocess.run(["g++", *FLAGS, "-DKAT_REFERENCE", "-I", str(header_dir), str(src), "-o", str(lib)],
                       check=True)
    return lib


if __name__ == "__main__":
    out = build()
    print(out if out else "reference sources absent: nothing to build")
    sys.exit(0)
