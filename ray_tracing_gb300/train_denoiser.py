"""Trains the U-Net denoiser on frames this path tracer renders.

For every training scene the renderer produces
  * noisy inputs: 1-spp frames with ReSTIR DI (temporal + spatial reuse), the
    configuration the denoiser runs on, several frames into a sequence so the
    reservoirs carry history; and
  * targets: plain path tracing (no ReSTIR) averaged to `--target-spp` samples
    per pixel, frames rendered independently (accumulation reset each frame).
The network (ray_tracing_gb300/denoiser.py) is trained on random crops with an
L1 loss on log1p(radiance) and saved as BF16 parameters in the layer order of
rtgb_set_denoiser_params.

    python -m ray_tracing_gb300.train_denoiser --out ray_tracing_gb300/weights/denoiser_unet.bf16

By default the optimisation runs on PyTorch (autograd and Adam as tooling);
with --native every training step runs on the library's own kernels
(rtgb_trainer_*: tcgen05 forward, input- and weight-gradient convolutions,
Adam), PyTorch only holding the rendered data and evaluating the validation
relMSE. Inference in the renderer always runs on the library's kernels.
"""
from __future__ import annotations

import argparse
import time
from pathlib import Path

import numpy as np

from . import denoiser, scenes
from .renderer import Renderer

TRAIN_SCENES = [
    ("random_spheres", 1, 1024), ("random_spheres", 2, 512), ("random_spheres", 3, 2048), ("random_spheres", 4, 256),
    ("random_spheres", 5, 1024), ("triangle_terrain", 1, 200000), ("triangle_terrain", 2, 100000),
    ("openpbr_gallery", 0, 24), ("openpbr_gallery", 1, 48), ("final_room", 0, 0), ("bouncing_spheres", 0, 0),
    ("cornell_box", 0, 0), ("smoke", 0, 0),
]
VALID_SCENE = ("random_spheres", 7, 1024)

# The learned-denoiser recipe of the benchmark protocol (seeded scenes of the
# 1 M-triangle terrain generator with constant OpenPBR materials and 256
# emissive triangles, 256 x 256 crops, 4096-spp targets, batch 16, Adam 1e-3,
# log-space L1), scaled down to `--c4-scenes` scenes, plus seeds of the
# textured-room generator (seeds other than the benchmark's 0) and the scenes
# above so the other workloads' material and lighting stay covered.
C4_SEED0 = 100


ORBIT_DEG = 2.0            # degrees per frame of the orbiting room sequences
ORBIT_FRAMES = (5, 30, 59)  # their captured frames (each with its own target)


def c4_scenes(count: int, rooms: int, orbit_rooms: int):
    """(name, seed, detail, orbit degrees per frame) of the c4 recipe."""
    return ([("triangle_terrain_pbr", C4_SEED0 + i, 0, 0.0) for i in range(count)]
            + [("textured_room", 1 + i, 0, 0.0) for i in range(rooms)]
            + [("textured_room", 1 + rooms + i, 0, ORBIT_DEG) for i in range(orbit_rooms)]
            + [(n, s, d, 0.0) for n, s, d in TRAIN_SCENES])


def noisy_profile():
    return scenes.profile("balanced", samples_per_pixel=1, max_bounces=4, enable_denoise=0, enable_restir_di=1,
                          restir_initial_candidates=32, restir_temporal_reuse=1, restir_spatial_neighbors=1)


def plain_profile(spp: int):
    return scenes.profile("balanced", samples_per_pixel=spp, max_bounces=4, enable_denoise=0, enable_restir_di=0)


def render_pair(name, seed, detail, width, height, cams, noisy_frames, target_spp, spp_per_frame, orbit_deg=0.0):
    """Per camera: (inputs (F, H, W, 10 source channels), target (H, W, 3)) of one scene. With `orbit_deg`
    the rig turns about the vertical axis by that many degrees per frame (the temporal accumulation then
    reprojects), and every captured frame gets its own target at its pose: (inputs (1, ...), target) pairs."""
    sc = scenes.HostScene(name, seed=seed, detail=detail)
    rig = scenes.default_rig(name, cams, width, height)
    r = Renderer()
    r.prepare_scene(sc.view)
    r.reset_sequence(1000 + seed)
    prof = noisy_profile()
    frames = [[] for _ in range(cams)]
    poses = []
    for f in range(noisy_frames[-1] + 1):
        frig = scenes.orbit_rig(rig, orbit_deg * f) if orbit_deg else rig
        r.render_frame(frig, prof, cams)
        if f in noisy_frames:
            poses.append(frig)
            for c in range(cams):
                frames[c].append(np.concatenate([r.buffer(c, "beauty")[..., :3], r.buffer(c, "albedo")[..., :3],
                                                 r.buffer(c, "denoiser_normal")[..., :3],
                                                 r.buffer(c, "depth")[..., None]], axis=-1))
    pprof = plain_profile(spp_per_frame)
    n = max(1, target_spp // spp_per_frame)

    def target(trig):
        acc = [None] * cams
        for _ in range(n):
            r.reset_accumulation()
            r.render_frame(trig, pprof, cams)
            for c in range(cams):
                cur = r.buffer(c, "beauty")[..., :3].astype(np.float64)
                acc[c] = cur if acc[c] is None else acc[c] + cur
        return [(a / n).astype(np.float32) for a in acc]

    if orbit_deg:
        out = []
        for k, trig in enumerate(poses):
            ys = target(trig)
            out += [(frames[c][k][None].astype(np.float32), ys[c]) for c in range(cams)]
    else:
        ys = target(rig)
        out = [(np.stack(frames[c]).astype(np.float32), ys[c]) for c in range(cams)]
    r.close()
    sc.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", type=Path, default=denoiser.WEIGHTS)
    ap.add_argument("--width", type=int, default=640)
    ap.add_argument("--height", type=int, default=480)
    ap.add_argument("--target-spp", type=int, default=1024)
    ap.add_argument("--spp-per-frame", type=int, default=16)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--native", action="store_true", help="train with the library's kernels (rtgb_trainer_*)")
    ap.add_argument("--recipe", choices=["default", "c4"], default="default",
                    help="c4: the protocol's recipe (terrain-generator scenes, 256 x 256 crops, 4096-spp targets, "
                         "batch 16, Adam 1e-3), scaled down to --c4-scenes scenes")
    ap.add_argument("--c4-scenes", type=int, default=48)
    ap.add_argument("--c4-rooms", type=int, default=6, help="textured-room seeds 1..N added to the c4 recipe")
    ap.add_argument("--c4-orbit-rooms", type=int, default=6,
                    help="further textured-room seeds rendered as orbiting sequences (the rig turning 2 degrees per "
                         "frame, frames 5, 30 and 59 captured with a target each)")
    ap.add_argument("--noisy-frames", default=None,
                    help="comma-separated frame indices of each scene's sequence used as noisy inputs (default 2,3,5; "
                         "c4: 2,5,12,24, so inputs with temporal accumulation are covered)")
    args = ap.parse_args(argv)
    scene_list = [(n, s, d, 0.0) for n, s, d in TRAIN_SCENES]
    noisy_frames = (2, 3, 5)
    if args.recipe == "c4":
        scene_list = c4_scenes(args.c4_scenes, args.c4_rooms, args.c4_orbit_rooms)
        noisy_frames = (2, 5, 12, 24)
        for name, default in (("width", 640), ("height", 480), ("target_spp", 1024), ("crop", 128), ("lr", 2e-3)):
            if getattr(args, name) == default:
                setattr(args, name, {"width": 320, "height": 256, "target_spp": 4096, "crop": 256, "lr": 1e-3}[name])
    if args.noisy_frames:
        noisy_frames = tuple(int(v) for v in args.noisy_frames.split(","))

    import torch
    dev = torch.device("cuda", 0)
    t0 = time.time()
    inputs, targets = [], []
    for name, seed, detail, orbit in scene_list:
        for x, y in render_pair(name, seed, detail, args.width, args.height, 4, ORBIT_FRAMES if orbit else noisy_frames,
                                args.target_spp, args.spp_per_frame, orbit):
            inputs.append(torch.from_numpy(x).to(dev))
            targets.append(torch.from_numpy(y).to(dev))
        print(f"rendered {name}/{seed}: {time.time() - t0:.1f} s", flush=True)
    valid = render_pair(*VALID_SCENE, args.width, args.height, 4, (3,), args.target_spp, args.spp_per_frame)
    vx = torch.from_numpy(np.stack([v[0][0] for v in valid])).to(dev)
    vy = torch.from_numpy(np.stack([v[1] for v in valid])).to(dev)

    def prep(src):  # (B, H, W, 10) AOVs -> network input (B, 10, H, W)
        return denoiser.make_input(src[..., 0:3], src[..., 3:6], src[..., 6:9], src[..., 9], xp=torch)

    torch.manual_seed(args.seed)
    gen = torch.Generator(device="cpu").manual_seed(args.seed)
    model = denoiser.build_model().to(dev)
    opt = torch.optim.Adam(model.parameters(), lr=args.lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, args.steps)
    cs = args.crop
    native = None
    if args.native:
        import ctypes as C
        import math
        from . import abi
        lib = abi.load()
        flat0 = denoiser.flatten(model)
        native = C.c_void_p()
        if lib.rtgb_trainer_create(args.batch, cs, cs, flat0.ctypes.data, flat0.size, C.byref(native)) != 0:
            raise RuntimeError("rtgb_trainer_create failed")
    for step in range(args.steps):
        xs, ys = [], []
        for _ in range(args.batch):
            si = int(torch.randint(len(inputs), (1,), generator=gen))
            fi = int(torch.randint(inputs[si].shape[0], (1,), generator=gen))
            H, W = inputs[si].shape[1:3]
            yy = int(torch.randint(0, H - cs + 1, (1,), generator=gen)) & ~3
            xx = int(torch.randint(0, W - cs + 1, (1,), generator=gen)) & ~3
            xs.append(inputs[si][fi, yy:yy + cs, xx:xx + cs])
            ys.append(targets[si][yy:yy + cs, xx:xx + cs])
        x = prep(torch.stack(xs))
        if native is not None:
            # cosine schedule as CosineAnnealingLR, the step on the library's kernels
            lr = 0.5 * args.lr * (1.0 + math.cos(math.pi * step / args.steps))
            xb = denoiser.blocked_input(x)
            yt = torch.log1p(torch.stack(ys).clamp_min(0)).contiguous()
            lv = C.c_float()
            if lib.rtgb_trainer_step(native, C.c_void_p(xb.data_ptr()), C.c_void_p(yt.data_ptr()), lr, C.byref(lv)) != 0:
                raise RuntimeError(lib.rtgb_trainer_last_error(native).decode())
            loss = torch.tensor(lv.value)
            if step % 500 == 0 or step == args.steps - 1:
                cur = np.empty(denoiser.param_count(), np.float32)
                lib.rtgb_trainer_params(native, cur.ctypes.data)
                denoiser.unflatten(model, cur)
        else:
            y = torch.log1p(torch.stack(ys).clamp_min(0)).permute(0, 3, 1, 2)
            loss = torch.nn.functional.l1_loss(model(x), y)
            opt.zero_grad(set_to_none=True)
            loss.backward()
            opt.step()
            sched.step()
        if step % 500 == 0 or step == args.steps - 1:
            with torch.no_grad():
                pred = torch.expm1(model(prep(vx)).clamp_min(0)).permute(0, 2, 3, 1)
                rel = ((pred - vy) ** 2 / (vy ** 2 + 1e-2)).mean().item()
                noisy = ((vx[..., 0:3] - vy) ** 2 / (vy ** 2 + 1e-2)).mean().item()
            print(f"step {step}: loss {loss.item():.4f}  valid relMSE {rel:.5f} (noisy {noisy:.5f})", flush=True)
    if native is not None:
        lib.rtgb_trainer_destroy(native)
    flat = denoiser.flatten(model)
    denoiser.save_weights(flat, args.out, {
        "trainer": "native (rtgb_trainer_*)" if args.native else "pytorch",
        "recipe": args.recipe, "noisy_frames": list(noisy_frames), "train_scenes": [f"{n}/{s}/{d}" + (f"/orbit{o}" if o else "") for n, s, d, o in scene_list],
        "valid_scene": "/".join(map(str, VALID_SCENE)), "width": args.width, "height": args.height,
        "target_spp": args.target_spp, "steps": args.steps, "batch": args.batch, "crop": args.crop, "lr": args.lr,
        "valid_relmse": rel, "valid_noisy_relmse": noisy})
    print(f"saved {args.out} ({time.time() - t0:.1f} s)")


if __name__ == "__main__":
    main()
