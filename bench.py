#!/usr/bin/env python3
"""Benchmark of the realtime radiance path on GB300.

Workload (one step = one frame of every camera):
  seeded random-sphere field (ground r=1000 + 22x22 r=0.2 spheres: 80% Lambertian,
  15% metal, 5% dielectric) with 1024 emissive rect lights as analytic lights;
  4 pinhole32 cameras 640x480, 1 spp, depth 4, ReSTIR DI with 32 initial
  candidates, temporal reuse and 1 spatial neighbour, BASIC bias correction,
  then the BF16 U-Net denoiser on the tensor cores (when its trained weights
  are present: ray_tracing_gb300/weights/denoiser_unet.bf16).

value   = rays traced (primary + extension + shadow + ReSTIR visibility) per
          second of device time, inputs resident (Mrays/s); each frame is timed
          with CUDA events on the renderer's stream, an L2 flush runs between
          frames outside the events.
e2e     = the same metric through the C ABI with host buffers, wall-clock timed
          over the steps: rtgb_render_frame_async, then rtgb_download_frame_async
          of every camera's beauty/normal/albedo/depth into double-buffered
          pinned host memory (the copies of frame i overlap the rendering of
          frame i+1) and rtgb_wait_downloads; every frame is on the host when
          the clock stops. e2e.blocking is the reference's order instead:
          rtgb_render_frame, then the waiting rtgb_download_frame per camera.
equal_relmse: the headline comparison. A 4096-spp plain render of the same
          frame is the reference r; relMSE = mean((x - r)^2 / (r^2 + 1e-2)).
          The denoised pipeline's relMSE and ms/frame are measured, then the
          plain path (no ReSTIR, no denoiser) is run at doubling sample counts
          until its relMSE is no larger; its ms/frame there over the denoised
          ms/frame is the speed-up at equal relMSE. The C5 record adds
          trimmed_cross_check: both sides' relMSE without the largest 0.1 % of
          per-value errors (fireflies), read off the same probes.
roofline: the launch with the largest share of the frame, per-unit algorithmic
          bytes (SoA stream bytes per ray / path segment / pixel) over its CUDA-event durations, against the measured
          HBM copy bandwidth.
training: native training steps of the U-Net (rtgb_trainer_step: tcgen05
          forward, input- and weight-gradient convolutions, Adam) on 16 crops
          of 256 x 256, ms per step and algorithmic TFLOP/s.
workloads: the protocol's C1 (Cornell box, with the CPU oracle on the same
          full frame) and C3 (1 M triangles, OpenPBR, mixed pinhole / fisheye
          rig) configurations, ms per frame and Mrays/s.
cpu_baseline / --impl reference: the CPU oracle (restatement of the reference's
          radiance kernel, with the reference's median-split BVH) on all host
          threads, over a band of rows of the same workload.

Launch: python bench.py [--gpus N --steps K --warmup W] [--impl reference]
(under torchrun for N > 1: one process per GPU, independent replicas).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "4-cam ms/frame at equal relMSE to 4096spp ref, denoised vs plain; Mrays/s"
UNIT = "Mrays/s"
SEED = 20260718          # the reference protocol's default sequence seed
WIDTH, HEIGHT, CAMERAS = 640, 480, 4
LIGHTS = 1024
L2_FLUSH_BYTES = 256 << 20

# Algorithmic bytes per unit: SoA stream bytes read + written per ray, path
# segment or pixel; BVH node and primitive traffic is excluded.
BYTES_RAYGEN = 32 + 48          # per path: ray + path state
BYTES_TRACE = 32 + 16           # per ray: read ray, write hit
BYTES_SHADE = 16 + 48 + 48 + 32 + 32 + 16   # per path segment
BYTES_RESTIR_PER_SPATIAL = 84   # per reuse neighbour, added to 84 + 84 (history) + 84 (write)
BYTES_SHADOW = 32 + 4           # per shadow ray
BYTES_RESOLVE = 68 + 36 + 68 + 12  # per pixel (accumulate + resolve)


CPU_ROW_STRIDE = 4       # the CPU oracle renders every 4th row of each camera (both arms)


def workload_config(spatial=1, world=1):
    return {
        "workload": "random_spheres_4x640x480_1spp_d4_restir32",
        "scene": f"ground + 22x22 spheres, {LIGHTS} analytic rect lights",
        "cameras": f"{CAMERAS}x pinhole32 {WIDTH}x{HEIGHT}",
        "spp": 1, "max_bounces": 4, "restir_candidates": 32, "temporal_reuse": 1, "spatial_neighbors": spatial,
        "denoise": "BF16 U-Net (tcgen05 implicit-GEMM 3x3 convolutions)" if _weights() is not None
                    else "off (trained weights absent)",
        "seed": SEED, "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer written between timed frames",
        "parallelism": f"replicas{world}" if world > 1 else "single",
    }


def _weights():
    from ray_tracing_gb300 import denoiser
    return denoiser.load_weights()


def make_inputs():
    from ray_tracing_gb300 import scenes
    sc = scenes.HostScene("random_spheres", seed=0, detail=LIGHTS)
    rig = scenes.default_rig("random_spheres", CAMERAS, WIDTH, HEIGHT)
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4,
                          enable_denoise=1 if _weights() is not None else 0, enable_restir_di=1,
                          restir_initial_candidates=32, restir_temporal_reuse=1, restir_spatial_neighbors=1)
    return sc, rig, prof


# ---- equal-relMSE comparison ------------------------------------------------------

RELMSE_EPS = 1e-2
REFERENCE_SPP = 4096
SPP_PER_FRAME = 16      # plain renders above this run as several frames, averaged


def relmse(x: np.ndarray, ref: np.ndarray) -> float:
    x = x.astype(np.float64)
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + RELMSE_EPS)))


TRIM_FRACTION = 1e-3  # largest per-value errors left out of the firefly-trimmed relMSE


def relmse_trimmed(x: np.ndarray, ref: np.ndarray, trim: float = TRIM_FRACTION) -> float:
    """relMSE without the `trim` fraction of largest per-value errors: a
    cross-check that rare bright paths (fireflies) do not decide an
    equal-relMSE comparison on a small band sample."""
    e = ((x.astype(np.float64) - ref) ** 2 / (ref ** 2 + RELMSE_EPS)).ravel()
    keep = e.size - int(np.floor(e.size * trim))
    if keep <= 0:
        return 0.0
    if keep < e.size:
        e = np.partition(e, keep - 1)[:keep]
    return float(np.mean(e))


def first_spp_within(trail: list, key: str, target: float):
    """The smallest probed spp of `trail` whose `key` is no larger than
    `target` (None if none is)."""
    hits = sorted((p["spp"] for p in trail if p.get(key) is not None and p[key] <= target))
    return hits[0] if hits else None


def plain_render(r, rig, spp: int, cameras: int = CAMERAS, max_bounces: int = 4, per_frame: int = SPP_PER_FRAME,
                 images: bool = True):
    """Averaged beauty of `spp` plain samples per pixel (no ReSTIR, no denoiser),
    as frames of at most `per_frame` spp with the accumulation reset each
    frame; returns (per-camera images or None, device ms)."""
    from ray_tracing_gb300 import scenes
    chunks = [per_frame] * (spp // per_frame) + ([spp % per_frame] if spp % per_frame else [])
    acc, ms = None, 0.0
    for per in chunks:
        prof = scenes.profile("balanced", samples_per_pixel=per, max_bounces=max_bounces, enable_denoise=0,
                              enable_restir_di=0)
        r.reset_accumulation()
        v = r.render_frame(rig, prof, cameras)
        ms += v.frame_render_ms
        if images:
            cur = np.stack([r.buffer(c, "beauty")[..., :3].astype(np.float64) for c in range(cameras)]) * per
            acc = cur if acc is None else acc + cur
    return (acc / spp if images else None), ms


# ---- equal relMSE on row bands (1080p rigs) -------------------------------------------
#
# A 4096-spp reference of four 1920x1080 cameras costs minutes, so the large
# rigs are judged on row bands: each camera's band rows are rendered as
# cropped cameras (same pose and intrinsics, principal point shifted by the
# band's first row, height = the band), which trace exactly the full camera's
# rays for those rows. Per-pixel seeds differ from the full frame's, which
# changes the noise realisation, not its distribution.

BAND_COUNT = 8          # bands per camera, evenly spaced over the image
BAND_ROWS = 8           # rows per band


def band_starts(height: int, bands: int = BAND_COUNT, rows: int = BAND_ROWS) -> list[int]:
    return [max(0, min(height - rows, int((k + 0.5) * height / bands) - rows // 2)) for k in range(bands)]


def crop_camera(cam, y0: int, rows: int):
    import ctypes as C
    from ray_tracing_gb300 import abi
    c = abi.Camera()
    C.memmove(C.byref(c), C.byref(cam), C.sizeof(abi.Camera))
    c.height = rows
    if c.model == 0:
        c.pinhole.cy = cam.pinhole.cy - y0
    else:
        c.equi.cy = cam.equi.cy - y0
        c.equi.height = rows
    return c


def band_rigs(rig, cameras: int):
    """Rigs of up to four cropped cameras covering every camera's bands, with
    the (camera, first row) of each slot."""
    from ray_tracing_gb300 import abi
    crops = [(c, y0) for c in range(cameras) for y0 in band_starts(rig.cameras[c].height)]
    out = []
    for i in range(0, len(crops), 4):
        part = crops[i:i + 4]
        rr = abi.CameraRig()
        rr.active_count = len(part)
        for j, (c, y0) in enumerate(part):
            rr.cameras[j] = crop_camera(rig.cameras[c], y0, BAND_ROWS)
        out.append((rr, part))
    return out


def band_rows_of(full: np.ndarray, height: int) -> np.ndarray:
    """The band rows of one full-frame camera image, in band order."""
    return np.concatenate([full[y0:y0 + BAND_ROWS] for y0 in band_starts(height)], axis=0)


def plain_bands(r, rig, cameras: int, spp: int, max_bounces: int, per_frame: int):
    """Plain `spp`-sample render of every camera's bands; returns (per camera
    band image (rows, width, 3), device ms)."""
    parts, ms = {}, 0.0
    for rr, part in band_rigs(rig, cameras):
        img, t = plain_render(r, rr, spp, cameras=rr.active_count, max_bounces=max_bounces, per_frame=per_frame)
        ms += t
        for j, key in enumerate(part):
            parts[key] = img[j]
    bands = [np.concatenate([parts[(c, y0)] for y0 in band_starts(rig.cameras[c].height)], axis=0)
             for c in range(cameras)]
    return bands, ms


def banded_equal_relmse(sc, frame_rigs: dict, variants: dict, max_bounces: int, cameras: int = 4,
                        ref_spp: int = REFERENCE_SPP, max_spp: int = 1024, time_spp_cap: int = 128):
    """Equal-relMSE comparison on row bands. `frame_rigs`: frame -> rig;
    `variants`: name -> (frame -> per-camera band rows of a denoised pipeline's
    output at that frame, that pipeline's device ms per frame). Per variant the
    plain path (no ReSTIR, no denoiser) is searched by doubling then bisecting
    spp until the mean relMSE over the frames is no larger than the variant's
    mean; its ms/frame is the full rig's device time at that spp (measured up
    to `time_spp_cap` spp, larger counts scaled linearly from there). The
    first variant's result is the record's top level; the others sit under
    their names."""
    from ray_tracing_gb300.renderer import Renderer
    t0 = time.perf_counter()
    results = {}
    with Renderer() as r:
        r.prepare_scene(sc.view)
        r.reset_sequence(SEED + 1)
        refs = {f: plain_bands(r, rig, cameras, ref_spp, max_bounces, per_frame=64)[0] for f, rig in frame_rigs.items()}
        ref_secs = time.perf_counter() - t0

        def err(imgs, f):
            return float(np.mean([relmse(imgs[c], refs[f][c]) for c in range(cameras)]))

        def err_trimmed(imgs, f):
            return float(np.mean([relmse_trimmed(imgs[c], refs[f][c]) for c in range(cameras)]))

        probes = {}

        def probe(spp):
            if spp not in probes:
                per, trimmed = {}, []
                for f in frame_rigs:
                    imgs = plain_bands(r, frame_rigs[f], cameras, spp, max_bounces, per_frame=16)[0]
                    per[f] = err(imgs, f)
                    trimmed.append(err_trimmed(imgs, f))
                probes[spp] = {"spp": spp, "relmse": float(np.mean(list(per.values()))),
                               "relmse_trimmed": float(np.mean(trimmed)),
                               "per_frame": {str(f): v for f, v in per.items()}}
            return probes[spp]

        def plain_ms(spp):
            first = next(iter(frame_rigs))
            timed = min(spp, time_spp_cap)
            if timed not in timed_ms:
                timed_ms[timed] = plain_render(r, frame_rigs[first], timed, cameras=cameras,
                                               max_bounces=max_bounces, per_frame=4, images=False)[1]
            return timed_ms[timed] * spp / timed, timed

        timed_ms = {}
        for name, (denoised, den_ms) in variants.items():
            d_err = {f: err(denoised[f], f) for f in frame_rigs}
            target = float(np.mean(list(d_err.values())))
            trail, found, spp = [], None, 1
            while spp <= max_spp:
                trail.append(probe(spp))
                if trail[-1]["relmse"] <= target:
                    found = trail[-1]
                    break
                spp *= 2
            if found is not None and len(trail) >= 2:
                lo, hi = trail[-2]["spp"], trail[-1]["spp"]
                while hi - lo > max(1, lo // 8):
                    mid = (lo + hi) // 2
                    trail.append(probe(mid))
                    if trail[-1]["relmse"] <= target:
                        hi, found = mid, trail[-1]
                    else:
                        lo = mid
            plain = None
            if found is not None:
                ms, timed = plain_ms(found["spp"])
                plain = dict(found, ms=ms, timed_spp=timed)
            results[name] = {
                "denoised": {"relmse": target, "per_frame": {str(f): v for f, v in d_err.items()},
                             "ms_per_frame": den_ms},
                "plain": plain if plain is not None else {"spp": None, "note": f"not reached within {max_spp} spp"},
                "plain_search": trail,
                "speedup_at_equal_relmse": (plain["ms"] / den_ms) if plain is not None else None,
            }
            # cross-check on the same renders: both sides' relMSE without the
            # largest TRIM_FRACTION of per-value errors, the plain side read off
            # the probes the search above already took (no new search)
            try:
                d_trim = float(np.mean([err_trimmed(denoised[f], f) for f in frame_rigs]))
                t_spp = first_spp_within(list(probes.values()), "relmse_trimmed", d_trim)
                t_ms = plain_ms(t_spp)[0] if t_spp is not None else None
                results[name]["trimmed_cross_check"] = {
                    "trim_fraction": TRIM_FRACTION, "denoised_relmse_trimmed": d_trim,
                    "plain_spp": t_spp, "plain_ms": t_ms,
                    "speedup": (t_ms / den_ms) if t_ms is not None else None,
                    "note": "smallest probed spp within the trimmed target" if t_spp is not None
                            else "no probed spp within the trimmed target"}
            except Exception as e:  # the cross-check never costs the record
                results[name]["trimmed_cross_check"] = {"error": f"{type(e).__name__}: {e}"}
    names = list(results)
    out = {"eps": RELMSE_EPS, "reference_spp": ref_spp, "frames": [int(f) for f in frame_rigs],
           "sample": f"{BAND_COUNT} bands of {BAND_ROWS} rows per camera (evenly spaced), rendered as cropped "
                     f"cameras; {BAND_COUNT * BAND_ROWS} of each camera's rows",
           "reference_seconds": ref_secs}
    out.update(results[names[0]])
    for name in names[1:]:
        out[name] = results[name]
    return out


def mixed_rig_1080p(scene_name: str = "random_spheres"):
    """The benchmark scene's four cameras at 1920x1080 with cameras 1 and 3 as
    180-degree equi62_lut1d fisheyes (r = f theta, f = (w / 2) / (pi / 2), no
    distortion) at the same poses: the mixed-model 1080p rig of the
    equal-relMSE target."""
    import ctypes as C
    from ray_tracing_gb300 import abi, scenes
    rig = scenes.default_rig(scene_name, CAMERAS, 1920, 1080)
    lib = abi.load()
    for i in (1, 3):
        c = rig.cameras[i]
        f = (c.width / 2.0) / (np.pi / 2.0)
        radial = (C.c_double * 6)(*([0.0] * 6))
        tangential = (C.c_double * 2)(0.0, 0.0)
        abi.check(lib.rtgb_make_equi62_lut1d(c.width, c.height, f, f, c.width / 2.0, c.height / 2.0, radial, tangential,
                                             C.byref(c.equi)), what="rtgb_make_equi62_lut1d")
        c.model = 1
    return rig


def equal_relmse(sc, rig, prof, frames: int = 8):
    from ray_tracing_gb300.renderer import Renderer
    weights = _weights()
    r = Renderer()
    r.prepare_scene(sc.view)
    r.reset_sequence(SEED + 1)
    ref, ref_ms = plain_render(r, rig, REFERENCE_SPP)
    out = {"eps": RELMSE_EPS, "reference_spp": REFERENCE_SPP, "reference_ms": ref_ms}
    if weights is None:
        out["unavailable"] = "trained denoiser weights absent"
        return out
    # denoised pipeline: 1 spp + ReSTIR + U-Net, after warm-up frames for the reservoir history
    r.set_denoiser(weights)
    r.reset_sequence(SEED)
    for _ in range(5):
        r.render_frame(rig, prof, CAMERAS)
    d_err, d_ms, d_dn, n_err, d_trim = [], [], [], [], []
    for _ in range(frames):
        v = r.render_frame(rig, prof, CAMERAS)
        d_ms.append(v.frame_render_ms)
        d_dn.append(v.cameras[0].denoise_ms)
        den = np.stack([r.buffer(c, "denoised")[..., :3] for c in range(CAMERAS)])
        noisy = np.stack([r.buffer(c, "beauty")[..., :3] for c in range(CAMERAS)])
        d_err.append(relmse(den, ref))
        d_trim.append(relmse_trimmed(den, ref))
        n_err.append(relmse(noisy, ref))
    target = float(np.mean(d_err))
    den_ms = float(np.median(d_ms))
    r.set_denoiser(None)
    spp, found = 1, None
    trail = []
    while spp <= 2048:
        img, ms = plain_render(r, rig, spp)
        e = relmse(img, ref)
        trail.append({"spp": spp, "relmse": e, "relmse_trimmed": relmse_trimmed(img, ref), "ms": ms})
        if e <= target:
            found = trail[-1]
            break
        spp *= 2
    if found is not None and len(trail) >= 2:
        lo, hi = trail[-2]["spp"], trail[-1]["spp"]
        while hi - lo > max(1, lo // 8):
            mid = (lo + hi) // 2
            img, ms = plain_render(r, rig, mid)
            e = relmse(img, ref)
            trail.append({"spp": mid, "relmse": e, "relmse_trimmed": relmse_trimmed(img, ref), "ms": ms})
            if e <= target:
                hi, found = mid, trail[-1]
            else:
                lo = mid
    out.update({
        "denoised": {"relmse": target, "ms_per_frame": den_ms, "denoise_ms": float(np.median(d_dn)),
                     "noisy_input_relmse": float(np.mean(n_err)), "frames": frames},
        "plain": found if found is not None else {"spp": None, "note": "not reached within 2048 spp"},
        "plain_search": trail,
        "speedup_at_equal_relmse": (found["ms"] / den_ms) if found is not None else None,
    })
    # the firefly-trimmed cross-check on the same renders (as the C5 record's)
    try:
        t_target = float(np.mean(d_trim))
        t_spp = first_spp_within(trail, "relmse_trimmed", t_target)
        t_ms = next((p["ms"] for p in trail if p["spp"] == t_spp), None)
        out["trimmed_cross_check"] = {"trim_fraction": TRIM_FRACTION, "denoised_relmse_trimmed": t_target,
                                      "plain_spp": t_spp, "plain_ms": t_ms,
                                      "speedup": (t_ms / den_ms) if t_ms is not None else None}
    except Exception as e:  # the cross-check never costs the record
        out["trimmed_cross_check"] = {"error": f"{type(e).__name__}: {e}"}
    r.close()
    return out


# ---- clocks -------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, _, flags in rows:
            for n, f in zip(names, flags):
                if f.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


# ---- CPU oracle (baseline / reference arm) ----------------------------------------

def oracle_frames(sc, rig, prof, stride, frames, threads=0, cameras=CAMERAS):
    """Renders `frames` frames of every `stride`-th row on the CPU oracle;
    returns (rays traced in the last frame, seconds of the last frame)."""
    from oracle.binding import OracleRenderer
    orc = OracleRenderer(sc.view, use_reference_bvh=True, threads=threads)
    orc.reset_sequence(SEED)
    rays = secs = 0.0
    for _ in range(frames):
        t0 = time.perf_counter()
        orc.render_frame(rig, prof, cameras, row_stride=stride)
        secs = time.perf_counter() - t0
        rays = sum(orc.rays(c) for c in range(cameras))
    orc.close()
    return rays, secs


def gpu_frames(sc, rig, prof, cameras, warmup, frames):
    """Prepares the scene and renders warm-up then timed frames on the GPU;
    returns (prepare ms, ms per frame, Mrays/s) from the frames' CUDA events."""
    from ray_tracing_gb300.renderer import Renderer
    r = Renderer()
    t0 = time.perf_counter()
    r.prepare_scene(sc.view)
    prep_ms = 1000.0 * (time.perf_counter() - t0)
    r.reset_sequence(SEED)
    for _ in range(warmup):
        r.render_frame(rig, prof, cameras)
    ms = rays = 0.0
    for _ in range(frames):
        v = r.render_frame(rig, prof, cameras)
        ms += v.frame_render_ms
        rays += v.rays_traced
    r.close()
    return prep_ms, ms / frames, rays / (ms * 1e-3) / 1e6


def workload_records(names=("c1", "c3", "c5", "smoke", "c4"), steps=None, warmup=None):
    """The other configurations of the reference protocol, measured beside the
    headline one: C1 (Cornell box 256 x 256, 64 spp, depth 8; the CPU oracle
    on all host threads renders the same full frame), C3 (1 M triangles with
    200 icosphere instances, constant OpenPBR materials, 256 emissive
    triangles; 2 x pinhole32 640x480 + 2 x equi62_lut1d 1280x1024 fisheye in one
    launch; 1 spp, depth 4, ReSTIR DI on; no analytic lights, so emissive NEE
    carries the direct light), C5 (c5_record) with its equal-relMSE
    comparison, the reference's published smoke protocol and the C4 denoiser
    inference size. Each record is measured on its own: one that fails is
    reported as {"error": ...} and the others stand."""
    out = {}
    frames = {} if steps is None else {"steps": steps, "warmup": warmup if warmup is not None else 3}
    jobs = {
        "c1": ("C1_cornell_256x256_64spp_d8", c1_record),
        "c3": ("C3_terrain_1Mtri_openpbr_2pinhole640_2equi1280", lambda: c3_record(**frames)),
        "c5": ("C5_room_4Mtri_textured_openpbr_4x1920x1080_orbit60_d6",
               lambda: c5_record(frames=frames["steps"], warmup=frames["warmup"]) if frames else c5_record()),
        "smoke": ("published_protocol_smoke_realtime_4x640x480", smoke_record),
        "c4": ("C4_denoiser_inference_4x1280x720", c4_inference_record),
        "training": ("C4_training_16x256x256",
                     lambda: training_record(**({"steps": frames["steps"], "warmup": frames["warmup"]} if frames else {}))),
    }
    for key in names:
        name, fn = jobs[key]
        try:
            out[name] = fn()
        except Exception as e:  # one record's failure must not cost the others
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out


def c1_record():
    from ray_tracing_gb300 import scenes
    with scenes.HostScene("cornell_box") as sc:
        rig = scenes.default_rig("cornell_box", 1)
        prof = scenes.profile("quality", samples_per_pixel=64, max_bounces=8, enable_denoise=0, enable_restir_di=0)
        prep, ms, mrays = gpu_frames(sc, rig, prof, 1, 2, 5)
        cores = os.cpu_count() or 1
        rays, secs = oracle_frames(sc, rig, prof, 1, 1, threads=cores, cameras=1)
    return {"ms_per_frame": ms, "mrays_per_s": mrays, "prepare_ms": prep,
            "cpu_oracle": {"ms_per_frame": 1000.0 * secs, "mrays_per_s": rays / secs / 1e6, "cores": cores,
                           "sample": "the full frame, reference BVH"},
            "gpu_over_cpu": (1000.0 * secs) / ms if ms > 0 else None}


def c3_record(steps=10, warmup=3):
    from ray_tracing_gb300 import scenes
    with scenes.HostScene("triangle_terrain_pbr", detail=1000000) as sc:
        rig = scenes.default_rig("triangle_terrain_pbr", 4)
        prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0, enable_restir_di=1)
        prep, ms, mrays = gpu_frames(sc, rig, prof, 4, warmup, steps)
        return {"ms_per_frame": ms, "mrays_per_s": mrays, "prepare_ms": prep, "triangles": sc.view.triangle_count}


def smoke_record(frames=30, warmup=5):
    """The reference's published realtime protocol: the `smoke` scene (one
    sphere, one emissive quad), realtime profile (1 spp, 2 bounces, denoised),
    4 cameras at 640x480, timed per frame with CUDA events. Its published
    numbers are RTX 3090 ones (frame 31.07 ms average including host work,
    render critical path 1.54 ms, OptiX temporal denoise 7.29 ms); the render
    and denoise times here are the comparable parts."""
    from ray_tracing_gb300 import scenes
    from ray_tracing_gb300.renderer import Renderer
    weights = _weights()
    prof = scenes.profile("realtime", enable_denoise=1 if weights is not None else 0)
    with scenes.HostScene("smoke") as sc, Renderer() as r:
        rig = scenes.default_rig("smoke", 4, 640, 480)
        r.prepare_scene(sc.view)
        if weights is not None:
            r.set_denoiser(weights)
        r.reset_sequence(SEED)
        for _ in range(warmup):
            r.render_frame(rig, prof, 4)
        ms, dn = [], []
        for _ in range(frames):
            v = r.render_frame(rig, prof, 4)
            ms.append(v.frame_render_ms)
            dn.append(v.cameras[0].denoise_ms)
    return {"ms_per_frame": float(np.mean(ms)), "ms_p99": float(np.percentile(ms, 99)),
            "denoise_ms_per_frame": float(np.mean(dn)), "render_ms_per_frame": float(np.mean(ms) - np.mean(dn)),
            "spp": prof.samples_per_pixel, "max_bounces": prof.max_bounces, "denoised": weights is not None,
            "reference_rtx3090": {"frame_ms_avg": 31.0712, "render_critical_path_ms": 1.5418,
                                  "denoise_critical_path_ms": 7.2927, "source": ".planning/v2.0-BASELINE.json:210-222"}}


def c4_inference_record(frames=20, warmup=3):
    """The U-Net at the C4 inference size, 4 x 1280x720 in one batch: the
    denoiser stage's CUDA-event time inside frames of a cheap scene (one
    bounce of the smoke scene; the denoiser's cost does not depend on the
    content) and its algorithmic TFLOP/s against the measured dense BF16 rate."""
    from ray_tracing_gb300 import scenes
    from ray_tracing_gb300.renderer import Renderer
    weights = _weights()
    if weights is None:
        return {"unavailable": "trained denoiser weights absent"}
    prof = scenes.profile("realtime", max_bounces=1, enable_denoise=1)
    with scenes.HostScene("smoke") as sc, Renderer() as r:
        rig = scenes.default_rig("smoke", 4, 1280, 720)
        r.prepare_scene(sc.view)
        r.set_denoiser(weights)
        for _ in range(warmup):
            r.render_frame(rig, prof, 4)
        dn = []
        for _ in range(frames):
            dn.append(r.render_frame(rig, prof, 4).cameras[0].denoise_ms)
    rec = denoiser_record(dn, 1280, 720, 4)
    rec["frames"] = frames
    return rec


C5_EVAL_FRAMES = (0, 30, 59)
C5_SIZE = (0, 0)            # camera size override (0: the rig's 1920x1080), for profiling a smaller case
C5_RELMSE = True            # the equal-relMSE comparison of c5_record (bench.py --no-relmse turns it off)


def c5_orbit(sc, rig, prof, weights, frames, warmup, degrees_per_frame, eval_frames):
    """Renders the C5 orbit; returns per-frame ms, denoise ms, stage times, rays,
    the prepare time and, at `eval_frames`, the denoised output's band rows."""
    from ray_tracing_gb300 import scenes
    from ray_tracing_gb300.renderer import Renderer
    with Renderer(stage_timing=True) as r:
        t0 = time.perf_counter()
        r.prepare_scene(sc.view)
        prep_ms = 1000.0 * (time.perf_counter() - t0)
        if weights is not None:
            r.set_denoiser(weights)
        r.reset_sequence(SEED)
        for _ in range(warmup):
            r.render_frame(rig, prof, 4)
        r.reset_accumulation()
        ms, dn, stages, rays = [], [], [], 0
        bands, frame_rigs = {}, {}
        for f in range(frames):
            frig = scenes.orbit_rig(rig, degrees_per_frame * f)
            v = r.render_frame(frig, prof, 4)
            ms.append(v.frame_render_ms)
            dn.append(v.cameras[0].denoise_ms)
            stages.append(r.stage_times())
            rays += v.rays_traced
            if f in eval_frames:
                frame_rigs[f] = frig
                bands[f] = [band_rows_of(r.buffer(c, "denoised")[..., :3], frig.cameras[c].height)
                            for c in range(4)]
    return ms, dn, stages, rays, prep_ms, bands, frame_rigs


def c5_record(frames=60, warmup=3, degrees_per_frame=2.0, relmse_eval=True):
    """C5: the 4 M-triangle textured room (checker / 3D-noise OpenPBR, 600
    icosphere props, 4096 emissive triangles), 2 x pinhole32 + 2 x
    equi62_lut1d at 1920x1080 in one launch, the rig orbiting the room by
    `degrees_per_frame` each of `frames` frames; 1 spp, depth 6, ReSTIR DI
    (32 candidates, temporal + 1 spatial) and the U-Net denoiser when its
    weights are present. Frame times are the frames' CUDA events. The room has
    no analytic lights, so the reference's ReSTIR (analytic lights only) does
    nothing and the emissive NEE carries the direct light; `restir_emissive`
    is the same orbit with ReSTIR resampling the 4096 emissive triangles
    (rtgb_render_profile::restir_emissive). With the weights, `equal_relmse`
    compares the denoised output of frames 0, 30 and 59 of both orbits with
    4096-spp plain renders of the same frames (row bands, banded_equal_relmse)."""
    from ray_tracing_gb300 import scenes
    weights = _weights()
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=6, enable_denoise=1 if weights is not None else 0,
                          enable_restir_di=1, restir_initial_candidates=32, restir_temporal_reuse=1,
                          restir_spatial_neighbors=1)
    relmse_eval = relmse_eval and C5_RELMSE and weights is not None
    eval_frames = C5_EVAL_FRAMES if relmse_eval else ()
    with scenes.HostScene("textured_room") as sc:
        rig = scenes.default_rig("textured_room", 4, *C5_SIZE)
        ms, dn, stages, rays, prep_ms, bands, frame_rigs = c5_orbit(sc, rig, prof, weights, frames, warmup,
                                                                   degrees_per_frame, eval_frames)
        # per-stage mean ms: raygen, (trace, shade, shadow) per bounce, finalize + resolve
        st = np.mean(np.stack(stages), axis=0)
        mb = (len(st) - 3) // 3
        stage_ms = {"raygen": float(st[0]), "finalize+resolve": float(st[-2] + st[-1])}
        for b in range(mb):
            for k, name in enumerate(("trace", "shade", "shadow")):
                stage_ms[f"{name}@{b}"] = float(st[1 + 3 * b + k])
        rec = {"ms_per_frame": float(np.mean(ms)), "ms_p50": float(np.median(ms)), "ms_max": float(np.max(ms)),
               "denoise_ms_per_frame": float(np.mean(dn)), "mrays_per_s": rays / (sum(ms) * 1e-3) / 1e6,
               "prepare_ms": prep_ms, "triangles": sc.view.triangle_count, "frames": frames,
               "orbit_degrees_per_frame": degrees_per_frame, "denoised": weights is not None,
               "stage_ms": stage_ms}
        variants = {"nee": (bands, float(np.mean(ms)))}
        try:
            prof.restir_emissive = 1
            ems, edn, est, erays, _, ebands, _ = c5_orbit(sc, rig, prof, weights, frames, warmup, degrees_per_frame,
                                                          eval_frames)
            sh0 = float(np.mean(np.stack(est), axis=0)[2])
            rec["restir_emissive"] = {"ms_per_frame": float(np.mean(ems)), "ms_p50": float(np.median(ems)),
                                      "denoise_ms_per_frame": float(np.mean(edn)),
                                      "mrays_per_s": erays / (sum(ems) * 1e-3) / 1e6,
                                      "shade@0_ms (with the ReSTIR passes)": sh0}
            if ebands:
                variants["restir_emissive"] = (ebands, float(np.mean(ems)))
        except Exception as e:  # the reference-rule orbit above stands on its own
            rec["restir_emissive"] = {"error": f"{type(e).__name__}: {e}"}
        if bands:
            try:
                rec["equal_relmse"] = banded_equal_relmse(sc, frame_rigs, variants, max_bounces=6)
            except Exception as e:  # the frame timings above stand on their own
                rec["equal_relmse"] = {"error": f"{type(e).__name__}: {e}"}
    return rec


def cpu_baseline(sc, rig, prof):
    cores = os.cpu_count() or 1
    stride = CPU_ROW_STRIDE
    rays, secs = oracle_frames(sc, rig, prof, stride, frames=2, threads=cores)
    return {"value": rays / secs / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"CPU oracle (reference BVH, {cores} threads): every {stride}th row of each of the "
                      f"{CAMERAS} cameras, 2nd of 2 frames timed ({secs:.2f} s, {int(rays)} rays)"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    sc, rig, prof = make_inputs()
    cores = os.cpu_count() or 1
    stride = CPU_ROW_STRIDE
    from oracle.binding import OracleRenderer
    orc = OracleRenderer(sc.view, use_reference_bvh=True, threads=cores)
    orc.reset_sequence(SEED)
    for _ in range(args.warmup):
        orc.render_frame(rig, prof, CAMERAS, row_stride=stride)
    rays = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.render_frame(rig, prof, CAMERAS, row_stride=stride)
        rays += sum(orc.rays(c) for c in range(CAMERAS))
    secs = time.perf_counter() - t0
    value = rays / secs / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(world=world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"every {stride}th row of each camera per step; the reference's renderer "
                                   "needs CUDA/OptiX/Eigen and does not build here, so its radiance kernel runs as "
                                   "the C++ oracle restatement"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---- GPU arm --------------------------------------------------------------------------

def denoiser_flops(width: int, height: int, cameras: int) -> float:
    """Algorithmic FLOPs of one U-Net pass: 2 * pixels * C_in * C_out * 9 per
    convolution at its resolution, with the network's real channel counts."""
    from ray_tracing_gb300 import denoiser
    full = float(width * height * cameras)
    res = [full, full, full / 4, full / 4, full / 16, full / 16, full / 4, full / 4, full, full, full]
    return sum(2.0 * px * ci * co * 9 for px, (ci, co) in zip(res, denoiser.LAYERS))


def denoiser_record(denoise_ms, width=WIDTH, height=HEIGHT, cameras=CAMERAS):
    """Tensor-core roofline of the denoiser stage (all its launches) on
    `cameras` frames of width x height, against the measured dense BF16
    throughput."""
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("bf16_tflops")
    note = "of measured (burst)" if peak else "of fallback"
    peak = peak or 1900.0
    ms = float(np.mean(denoise_ms)) if denoise_ms else 0.0
    flops = denoiser_flops(width, height, cameras)
    achieved = flops / (ms * 1e-3) / 1e12 if ms > 0 else 0.0
    return {"ms_per_frame": ms, "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": note, "flops_per_frame": flops,
            "frame": f"{cameras} x {width}x{height}"}


TRAIN_BATCH, TRAIN_CROP = 16, 256     # the learned-denoiser training shape (16 crops of 256 x 256)


def training_flops(n: int, h: int, w: int) -> float:
    """Algorithmic FLOPs of one native training step: each convolution's forward,
    weight gradient and (all but the first layer) input gradient, real channel
    counts."""
    from ray_tracing_gb300 import denoiser
    full = float(n * h * w)
    res = [full, full, full / 4, full / 4, full / 16, full / 16, full / 4, full / 4, full, full, full]
    return sum(2.0 * px * ci * co * 9 * (2 if li == 0 else 3)
               for li, (px, (ci, co)) in enumerate(zip(res, denoiser.LAYERS)))


def training_record(steps: int = 10, warmup: int = 3):
    """Native training steps of the U-Net (rtgb_trainer_step: forward, loss,
    backward, Adam) on a resident synthetic batch; wall time per step (each
    step ends with the loss read back) and algorithmic TFLOP/s against the
    measured dense BF16 burst rate."""
    import ctypes as C
    import torch
    from ray_tracing_gb300 import abi, denoiser
    torch.manual_seed(0)
    flat = denoiser.flatten(denoiser.build_model()).astype(np.float32)
    n, hw = TRAIN_BATCH, TRAIN_CROP
    gen = torch.Generator(device="cuda").manual_seed(1)
    x = torch.rand((n, 10, hw, hw), device="cuda", generator=gen)
    xb = denoiser.blocked_input(x)
    target = torch.rand((n, hw, hw, 3), device="cuda", generator=gen).contiguous()
    lib = abi.load()
    tr = C.c_void_p()
    if lib.rtgb_trainer_create(n, hw, hw, flat.ctypes.data, flat.size, C.byref(tr)) != 0:
        return {"unavailable": "rtgb_trainer_create failed"}
    try:
        loss = C.c_float()
        for i in range(warmup + steps):
            if i == warmup:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
            if lib.rtgb_trainer_step(tr, C.c_void_p(xb.data_ptr()), C.c_void_p(target.data_ptr()), 1e-4,
                                     C.byref(loss)) != 0:
                return {"unavailable": lib.rtgb_trainer_last_error(tr).decode()}
        ms = 1000.0 * (time.perf_counter() - t0) / steps
    finally:
        lib.rtgb_trainer_destroy(tr)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("bf16_tflops") or 1900.0
    flops = training_flops(n, hw, hw)
    achieved = flops / (ms * 1e-3) / 1e12
    return {"batch": f"{n} x {hw}x{hw} crops, 10 input channels", "optimizer": "Adam", "ms_per_step": ms,
            "steps": steps, "flops_per_step": flops, "achieved_tflops": achieved, "peak_tflops": peak,
            "frac": achieved / peak, "peak_source": "of measured (burst)" if peaks.get("bf16_tflops") else "of fallback",
            "final_loss": float(loss.value)}


def roofline_traversal(stage_ms, frames_stats):
    """The traversal launches measured against L2 bandwidth: k_trace and k_shadow
    at bounce 0. Their SoA stream bytes are small next to the acceleration
    structure they walk, so `profiles/trace_l2.json` (one ncu capture of each
    bounce-0 launch of the benchmark frame) gives the L1, L2 and DRAM bytes
    per ray, BVH nodes and leaf records included; achieved = L2 bytes per ray x
    this run's rays / this run's CUDA-event time of the launch, peak = the L2
    byte rate at 100 % of lts__t_bytes in that capture."""
    path = ROOT / "profiles" / "trace_l2.json"
    if not path.exists():
        return None
    prof = json.loads(path.read_text())
    out = {}
    for name, idx, rays_of in (("k_trace@0", 1, lambda st: st["active"][0]),
                               ("k_shadow@0", 3, lambda st: st["shadow_rays_per_bounce"][0])):
        rec = prof.get(name)
        if not rec:
            continue
        rays = float(np.mean([rays_of(st) for st in frames_stats]))
        ms = float(np.mean([t[idx] for t in stage_ms]))
        per_ray = {k: rec[k] / rec["rays"] for k in ("l1_bytes", "l2_bytes", "dram_bytes")}
        peak = rec["l2_bytes"] / (rec["duration_ns"] * 1e-9) / (rec["l2_pct_of_peak"] / 100.0) / 1e9
        achieved = per_ray["l2_bytes"] * rays / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        out[name] = {"bound": "latency (traversal)", "unit": "GB/s", "achieved": achieved, "peak": peak,
                     "frac": achieved / peak, "peak_source": "L2 byte rate at 100 % of lts__t_bytes (ncu capture)",
                     "l1_bytes_per_ray": per_ray["l1_bytes"], "l2_bytes_per_ray": per_ray["l2_bytes"],
                     "dram_bytes_per_ray": per_ray["dram_bytes"], "avg_launch_ms": ms, "rays_per_launch": rays}
    return out


def roofline(stage_ms, frames_stats, spatial):
    """Roofline record of the launch slot (kernel at a bounce) with the largest
    average time per frame; per-unit algorithmic bytes over its
    CUDA-event durations, against the measured HBM copy bandwidth."""
    peaks = {}
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        peaks = json.loads(p.read_text())
    peak = peaks.get("hbm_gbs")
    peak_note = "of measured" if peak else "of fallback"
    peak = peak or 6800.0
    slots = {}

    def add(name, ms, nbytes):
        v = slots.setdefault(name, [0.0, 0.0, 0])
        v[0] += ms
        v[1] += nbytes
        v[2] += 1

    for times, st in zip(stage_ms, frames_stats):
        mb = (len(times) - 3) // 3
        add("k_raygen", times[0], st["paths"] * BYTES_RAYGEN)
        for b in range(mb):
            act = st["active"][b]
            restir = st["restir_pixels"] * (84 + 84 * (1 + spatial) + 84) if b == 0 else 0
            add(f"k_trace@{b}", times[1 + 3 * b], act * BYTES_TRACE)
            add(f"k_shade@{b}", times[2 + 3 * b], act * BYTES_SHADE + restir)
            add(f"k_shadow@{b}", times[3 + 3 * b], st["shadow_rays_per_bounce"][b] * BYTES_SHADOW)
        add("k_finalize+k_resolve", times[-2] + times[-1], st["pixels"] * BYTES_RESOLVE)
    name = max(slots, key=lambda k: slots[k][0])
    ms, nbytes, launches = slots[name]
    achieved = nbytes / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    traffic = None
    tpath = ROOT / "profiles" / "roofline_traffic.json"
    if tpath.exists():
        # DRAM bytes (read + write) per launch of each slot, from one ncu capture
        rec = json.loads(tpath.read_text()).get(name)
        traffic = float(rec) if isinstance(rec, (int, float)) else None
    frame_ms = sum(v[0] for v in slots.values())
    by_kernel = {}
    for k, v in slots.items():
        by_kernel[k.split("@")[0]] = by_kernel.get(k.split("@")[0], 0.0) + v[0] / max(len(stage_ms), 1)
    return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": peak_note,
            "avg_launch_ms": ms / max(launches, 1), "algorithmic_bytes_per_launch": nbytes / max(launches, 1),
            "share_of_frame": ms / frame_ms if frame_ms > 0 else None,
            "stage_ms_per_frame": by_kernel}


def profile_frames(n: int) -> None:
    """The benchmark frame rendered `n` times without the denoiser: scene
    preparation, then per frame raygen, (trace, material bucketing, shade,
    shadow) per bounce with the three ReSTIR passes at bounce 0, finalize and
    resolve; frame n-1 has full reservoir history."""
    from ray_tracing_gb300.renderer import Renderer
    sc, rig, prof = make_inputs()
    prof.enable_denoise = 0
    with Renderer() as r:
        r.prepare_scene(sc.view)
        r.reset_sequence(SEED)
        for _ in range(n):
            v = r.render_frame(rig, prof, CAMERAS)
        print(json.dumps({"frames": n, "restir_pixels": int(v.restir_pixels),
                          "active": [int(v.active_paths[b]) for b in range(prof.max_bounces)],
                          "shadow": [int(v.shadow_per_bounce[b]) for b in range(prof.max_bounces)]}))
    sc.close()


def e2e_measure(r, rig, prof, steps: int) -> dict:
    """Rays per wall-clock second through the C ABI with host buffers (the
    module docstring's e2e): pipelined downloads, and the blocking order."""
    import torch
    pixels = WIDTH * HEIGHT
    d2h = CAMERAS * pixels * (16 * 3 + 4)

    def host_set():
        return [[torch.empty(pixels * 4, dtype=torch.float32, pin_memory=True) for _ in range(3)]
                + [torch.empty(pixels, dtype=torch.float32, pin_memory=True)] for _ in range(CAMERAS)]

    host = [host_set(), host_set()]
    r.wait_downloads()
    torch.cuda.synchronize()
    rays0 = r.ray_totals()
    t0 = time.perf_counter()
    for i in range(steps):
        r.render_frame_async(rig, prof, CAMERAS)
        for c in range(CAMERAS):
            r.download_async(c, *host[i & 1][c])
        r.wait_downloads(keep_latest=True)  # frame i-1 is on the host
    r.wait_downloads()
    secs = time.perf_counter() - t0
    views = r.frame_stats()  # the device status of the last frame
    rays = float(np.sum(r.ray_totals() - rays0))
    out = {"value": rays / secs / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(views.h2d_bytes),
           "d2h_bytes_per_step": d2h, "steps": steps, "ms_per_step": 1000.0 * secs / steps,
           "downloads": "pipelined (rtgb_download_frame_async, double-buffered pinned host memory)"}
    # the reference's order: the frame, then each camera's waiting download
    torch.cuda.synchronize()
    rays0 = r.ray_totals()
    t0 = time.perf_counter()
    for _ in range(steps):
        r.render_frame(rig, prof, CAMERAS)
        for c in range(CAMERAS):
            b, n, a, d = host[0][c]
            st = r.lib.rtgb_download_frame(r.h, c, b.data_ptr(), n.data_ptr(), a.data_ptr(), d.data_ptr(), None)
            if st != 0:
                raise RuntimeError("rtgb_download_frame failed")
    secs = time.perf_counter() - t0
    rays = float(np.sum(r.ray_totals() - rays0))
    out["blocking"] = {"value": rays / secs / 1e6, "ms_per_step": 1000.0 * secs / steps}
    return out


def replica_reduce(value: float, op: str, device="cpu") -> float:
    """`value` combined over the replicas of the process group ("max": the
    slowest rank's time, "sum": whole-job totals); unchanged without a group.
    `device` is where the collective's tensor lives (cuda:N under NCCL, cpu
    under gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from ray_tracing_gb300.renderer import Renderer

    torch.cuda.set_device(local_rank)
    sc, rig, prof = make_inputs()
    r = Renderer(device=local_rank, stage_timing=True)
    r.prepare_scene(sc.view)
    weights = _weights() if prof.enable_denoise else None
    if weights is not None:
        r.set_denoiser(weights)
    # launch shapes picked by the library's autotuner for this scene and rig
    # (tuning frames are discarded; results do not depend on the grids)
    tuning = None
    if not args.no_autotune:
        try:
            tuning = r.autotune_launches(rig, prof, CAMERAS, frames=4)
        except Exception as e:  # a failed tuning leaves the handle's grids as they were
            tuning = {"error": f"{type(e).__name__}: {e}"}
    r.reset_sequence(SEED)
    stream = torch.cuda.ExternalStream(r.stream_ptr())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local_rank}")
    for _ in range(args.warmup):
        r.render_frame(rig, prof, CAMERAS)
    # raygen, (trace, reset, material bucketing x 3, shade, shadow) per bounce,
    # the three ReSTIR passes, finalize, resolve; the denoiser: pack, 11
    # convolutions (pooling and upsampling fused into them at these even
    # sizes), unpack per batch of equal-size cameras (one batch here)
    launches_per_frame = 1 + 7 * prof.max_bounces + 3 + 2 + (13 if weights is not None else 0)

    sampler = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local_rank)).split(",")[0])
                           if os.environ.get("CUDA_VISIBLE_DEVICES", "").isdigit() else local_rank)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    rays0 = r.ray_totals()
    frame_ms, stage_ms, frame_stats, denoise_ms = [], [], [], []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        ev0.record(stream)
        r.render_frame_async(rig, prof, CAMERAS)
        ev1.record(stream)
        v = r.frame_stats()
        denoise_ms.append(v.cameras[0].denoise_ms)
        frame_ms.append(ev0.elapsed_time(ev1))
        stage_ms.append(r.stage_times())
        frame_stats.append({"paths": WIDTH * HEIGHT * CAMERAS, "pixels": WIDTH * HEIGHT * CAMERAS,
                            "active": [int(v.active_paths[b]) for b in range(prof.max_bounces)],
                            "restir_pixels": int(v.restir_pixels),
                            "shadow_rays_per_bounce": [int(v.shadow_per_bounce[b]) for b in range(prof.max_bounces)]})
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    rays = float(np.sum(r.ray_totals() - rays0))
    total_ms = float(sum(frame_ms))
    total_ms = replica_reduce(total_ms, "max", f"cuda:{local_rank}")
    rays = replica_reduce(rays, "sum", f"cuda:{local_rank}")
    value = rays / (total_ms * 1e-3) / 1e6

    e2e = e2e_measure(r, rig, prof, max(3, args.steps))
    e2e["value"] = replica_reduce(e2e["value"], "sum", f"cuda:{local_rank}")
    e2e["blocking"]["value"] = replica_reduce(e2e["blocking"]["value"], "sum", f"cuda:{local_rank}")

    if rank != 0:
        return 0
    roof = roofline(stage_ms, frame_stats, spatial=1)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(world=world),
        "rays_per_frame": rays / args.steps / world,
        "roofline": roof,
        "roofline_traversal": roofline_traversal(stage_ms, frame_stats),
        "e2e": e2e,
        "clocks": clocks,
        "gpu_launches": launches_per_frame * args.steps,
        "denoiser": denoiser_record(denoise_ms) if weights is not None else None,
        "launch_tuning": tuning,
    }
    if world == 1 and not args.no_training:
        line["training"] = training_record()
    if world == 1 and not args.no_workloads:
        line["workloads"] = workload_records()
    if world == 1 and not args.no_relmse:
        line["equal_relmse"] = equal_relmse(sc, mixed_rig_1080p() if args.relmse_rig == "mixed1080" else rig, prof)
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, rig, prof)
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-relmse", action="store_true", help="skip the equal-relMSE comparison")
    ap.add_argument("--no-training", action="store_true", help="skip the native denoiser-training measurement")
    ap.add_argument("--no-workloads", action="store_true", help="skip the C1 / C3 / C5 workload records")
    ap.add_argument("--relmse-rig", choices=["bench", "mixed1080"], default="bench",
                    help="rig of the equal-relMSE comparison: the bench's 4 x 640x480 pinholes, or 2 pinhole + 2 "
                         "fisheye cameras at 1920x1080")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the persistent launch shapes instead of rtgb_autotune_launches' choice")
    ap.add_argument("--c5-size", default=None, help="WxH of the C5 cameras (default 1920x1080; for profiling)")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="render the benchmark frame this many times (no denoiser, no autotuning, untimed) and exit: "
                         "a fixed launch sequence for ncu captures")
    ap.add_argument("--workload", choices=["c1", "c3", "c5", "smoke", "c4", "training"], default=None,
                    help="measure only this protocol workload (steps / warmup frames) and print its record")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    global C5_SIZE, C5_RELMSE
    if args.c5_size:
        w, h = (int(v) for v in args.c5_size.lower().split("x"))
        C5_SIZE = (w, h)
    C5_RELMSE = not args.no_relmse
    if args.profile_frames > 0:
        if rank == 0:
            profile_frames(args.profile_frames)
        return 0
    if args.workload is not None:
        if rank == 0:
            print(json.dumps({"workloads": workload_records((args.workload,), args.steps, args.warmup)}), flush=True)
        return 0
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if args.impl == "reference":
            dist.init_process_group("gloo")
        else:
            import torch
            torch.cuda.set_device(local_rank)
            dist.init_process_group("nccl")
    from ray_tracing_gb300 import build
    if rank == 0:
        build.build_all()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
    else:
        rc = run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
