"""Generates tests/golden/openpbr/kats.npz from the reference's OpenPBR header.

Run in a checkout where the reference sources are mounted:

    python oracle/build_ref.py            # -> oracle/_ref/libopenpbr_ref.so
    python tests/golden/make_openpbr_kats.py

Inputs are seeded random records (oracle/openpbr_kat.cpp documents the layout)
spread over material families that exercise every lobe of
src/common/openpbr_core.h: Oren-Nayar diffuse, rough and smooth dielectric
reflection and transmission, F82 metal, thin-walled glass, Cauchy dispersion,
thin-film interference on dielectrics and metals, coat (darkening, tint,
anisotropy), fuzz, the subsurface random walk (entry, exit through the boundary
material, segments), thin-walled subsurface, partial opacity, and fully random
mixes. Outputs are the reference header's answers for the same records.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from ray_tracing_gb300 import abi  # noqa: E402

KAT_IN, KAT_OUT = 80, 64
SEED = 20260718
RECORDS = 1536
FAMILIES = ["plastic", "metal", "glass", "thin_glass", "dispersive_glass", "film_dielectric", "film_metal",
            "coat", "fuzz", "random_walk", "thin_subsurface", "cutout", "mix"]
OUT = Path(__file__).resolve().parent / "openpbr"


def param_offsets() -> dict[str, tuple[int, int]]:
    off, table = 0, {}
    for name, k in abi.OPENPBR_PARAMS:
        table[name] = (off, k)
        off += k
    assert off == 50
    return table


def unit(rng, n=1):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def material(rng, family: str) -> np.ndarray:
    tab = param_offsets()
    words = np.zeros(51, dtype=np.float32)
    for name, (o, k) in tab.items():
        words[o:o + k] = abi.OPENPBR_DEFAULTS[name]
    thin = 0

    def put(name, value):
        o, k = tab[name]
        words[o:o + k] = value

    def col():
        return rng.uniform(0.02, 1.0, 3)

    rough = lambda: 0.0 if rng.random() < 0.2 else rng.uniform(0.0, 1.0)  # noqa: E731
    put("base_color", col())
    put("specular_roughness", rough())
    put("base_diffuse_roughness", rng.uniform(0, 1))
    put("specular_roughness_anisotropy", rng.uniform(0, 1) if rng.random() < 0.3 else 0.0)
    put("specular_ior", rng.uniform(1.05, 2.4) if rng.random() < 0.9 else rng.uniform(0.6, 0.95))
    if family == "metal":
        put("base_metalness", 1.0)
        put("specular_color", col())
    elif family in ("glass", "thin_glass", "dispersive_glass"):
        put("transmission_weight", 1.0 if rng.random() < 0.7 else rng.uniform(0.2, 1.0))
        put("transmission_color", col())
        put("transmission_depth", rng.choice([0.0, rng.uniform(0.1, 2.0)]))
        if family == "thin_glass":
            thin = 1
        if family == "dispersive_glass":
            put("transmission_dispersion_scale", rng.uniform(0.1, 1.0))
            put("transmission_dispersion_abbe_number", rng.uniform(10, 60))
    elif family in ("film_dielectric", "film_metal"):
        put("thin_film_weight", rng.uniform(0.3, 1.0))
        put("thin_film_thickness", rng.uniform(0.05, 1.2))
        put("thin_film_ior", rng.uniform(1.1, 2.2))
        if family == "film_metal":
            put("base_metalness", rng.uniform(0.5, 1.0))
        elif rng.random() < 0.5:
            put("transmission_weight", rng.uniform(0.2, 1.0))
            if rng.random() < 0.5:
                thin = 1
    elif family == "coat":
        put("coat_weight", rng.uniform(0.2, 1.0))
        put("coat_color", col())
        put("coat_roughness", rough())
        put("coat_roughness_anisotropy", rng.uniform(0, 1) if rng.random() < 0.3 else 0.0)
        put("coat_ior", rng.uniform(1.2, 2.0))
        put("coat_darkening", rng.uniform(0, 1))
        put("base_metalness", rng.choice([0.0, 1.0, rng.uniform(0, 1)]))
    elif family == "fuzz":
        put("fuzz_weight", rng.uniform(0.2, 1.0))
        put("fuzz_color", col())
        put("fuzz_roughness", rng.uniform(0.0, 1.0))
    elif family in ("random_walk", "thin_subsurface"):
        put("subsurface_weight", rng.uniform(0.3, 1.0))
        put("subsurface_color", col())
        put("subsurface_radius", rng.uniform(0.05, 2.0))
        put("subsurface_radius_scale", rng.uniform(0.1, 1.0, 3))
        put("subsurface_scatter_anisotropy", rng.uniform(-0.9, 0.9))
        if family == "thin_subsurface":
            thin = 1
    elif family == "cutout":
        put("geometry_opacity", rng.uniform(0.1, 0.9))
        thin = int(rng.random() < 0.5)
    elif family == "mix":
        for name in ("base_weight", "base_metalness", "specular_weight", "transmission_weight", "subsurface_weight",
                     "fuzz_weight", "coat_weight", "thin_film_weight", "coat_darkening"):
            put(name, rng.uniform(0, 1) if rng.random() < 0.7 else 0.0)
        for name in ("specular_color", "transmission_color", "subsurface_color", "fuzz_color", "coat_color"):
            put(name, col())
        put("coat_roughness", rough())
        put("fuzz_roughness", rng.uniform(0, 1))
        put("subsurface_radius", rng.uniform(0.0, 2.0))
        put("subsurface_scatter_anisotropy", rng.uniform(-0.9, 0.9))
        put("transmission_dispersion_scale", rng.uniform(0, 1) if rng.random() < 0.3 else 0.0)
        put("thin_film_thickness", rng.uniform(0.0, 1.0))
        put("geometry_opacity", 1.0 if rng.random() < 0.7 else rng.uniform(0, 1))
        thin = int(rng.random() < 0.3)
    if family != "mix" and rng.random() < 0.15:
        put("emission_luminance", rng.uniform(0.5, 5.0))
        put("emission_color", col())
    words[50] = np.array([thin], dtype=np.int32).view(np.float32)[0]
    return words


def make_inputs() -> np.ndarray:
    rng = np.random.default_rng(SEED)
    rec = np.zeros((RECORDS, KAT_IN), dtype=np.float32)
    for i in range(RECORDS):
        fam = FAMILIES[i % len(FAMILIES)]
        rec[i, :51] = material(rng, fam)
        n = unit(rng)[0]
        rec[i, 51:54] = n
        rec[i, 54:57] = unit(rng)[0] if rng.random() < 0.7 else 0.0
        wo = unit(rng)[0]
        # mostly on the normal's side; a third from below (exits, interior transmission)
        if (np.dot(wo, n) < 0) != (rng.random() < 0.33):
            wo = -wo
        wi = unit(rng)[0]
        if rng.random() < 0.1:
            wi = (2 * np.dot(wo, n) * n - wo).astype(np.float32)  # mirror direction
        rec[i, 57:60] = wo
        rec[i, 60:63] = wi
        rec[i, 63:66] = rng.random(3)
        rec[i, 66:69] = rng.uniform(0.0, 2.0, 3) if rng.random() < 0.8 else 0.0
        rec[i, 69] = rng.uniform(0.0, 3.0)
        rec[i, 70] = rng.random()
        rec[i, 71] = rng.uniform(0.0, 1.0)
        rec[i, 72] = rng.uniform(0.0, 1.0)
    return rec


def run(lib_path: Path, symbol: str, inputs: np.ndarray) -> np.ndarray:
    lib = C.CDLL(str(lib_path))
    fn = getattr(lib, symbol)
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    out = np.zeros((inputs.shape[0], KAT_OUT), dtype=np.float32)
    widths = fn(inputs.ctypes.data, inputs.shape[0], out.ctypes.data)
    assert widths == (KAT_IN << 16) | KAT_OUT, hex(widths)
    return out


def main() -> None:
    ref_lib = ROOT / "oracle" / "_ref" / "libopenpbr_ref.so"
    # the reference checkout: first argument, else RTGB_REFERENCE_ROOT (as oracle/build_ref.py)
    root = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ["RTGB_REFERENCE_ROOT"])
    header = root / "src" / "common" / "openpbr_core.h"
    inputs = make_inputs()
    outputs = run(ref_lib, "ref_openpbr_kat", inputs)
    OUT.mkdir(exist_ok=True)
    np.savez_compressed(OUT / "kats.npz", inputs=inputs, outputs=outputs,
                        header_sha256=np.array(hashlib.sha256(header.read_bytes()).hexdigest()),
                        families=np.array(FAMILIES))
    print(f"{RECORDS} records -> {OUT / 'kats.npz'}")


if __name__ == "__main__":
    main()
