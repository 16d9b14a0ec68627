"""The U-Net denoiser end to end through the C ABI against its PyTorch mirror.

The GPU path stores every activation in BF16; the reference here runs the
same network in fp32 with BF16-rounded inputs, weights and activations, so the
remaining differences are fp32 summation order and the occasional BF16
rounding flip that follows from it. Bound: median relative error 2e-3, 99.9th
percentile 5e-2 (an activation that flips one BF16 step moves the output by up
to ~1 % and such flips can stack over eleven layers).
"""
from __future__ import annotations

import numpy as np
import pytest

from ray_tracing_gb300 import abi, denoiser, scenes


def test_parameter_count_matches_the_library():
    assert abi.load().rtgb_denoiser_param_count() == denoiser.param_count()


def test_flatten_roundtrip():
    torch = pytest.importorskip("torch")
    torch.manual_seed(0)
    m = denoiser.build_model()
    flat = denoiser.flatten(m)
    m2 = denoiser.build_model()
    denoiser.unflatten(m2, flat)
    assert np.array_equal(denoiser.flatten(m2), flat)
    bits = denoiser.to_bf16_bits(flat)
    back = denoiser.from_bf16_bits(bits)
    assert np.all(np.abs(back - flat) <= np.abs(flat) * 2.0 ** -8 + 1e-30)


@pytest.mark.gpu
def test_unet_matches_pytorch_mirror():
    torch = pytest.importorskip("torch")
    from ray_tracing_gb300.renderer import Renderer
    torch.manual_seed(1)
    model = denoiser.build_model()
    flat = denoiser.flatten(model)
    flat_bf16 = denoiser.from_bf16_bits(denoiser.to_bf16_bits(flat))
    denoiser.unflatten(model, flat_bf16)
    sc = scenes.HostScene("random_spheres", seed=3, detail=64)
    rig = scenes.default_rig("random_spheres", 3, 100, 70)   # ragged tiles and odd pooled sizes
    rig.cameras[2].width, rig.cameras[2].height = 72, 48      # a second batch shape
    rig.cameras[2].pinhole.cx, rig.cameras[2].pinhole.cy = 36.0, 24.0
    prof = scenes.profile("balanced", samples_per_pixel=1, max_bounces=3, enable_denoise=1, enable_restir_di=1,
                          restir_initial_candidates=8, restir_min_analytic_lights=8)
    r = Renderer()
    r.prepare_scene(sc.view)
    r.set_denoiser(flat)
    for _ in range(2):
        views = r.render_frame(rig, prof, 3)
    assert views.cameras[0].denoise_ms > 0.0
    model = model.cuda().eval()
    for cam in range(3):
        raw = r.buffer(cam, "beauty")
        alb = r.buffer(cam, "albedo")
        dn = r.buffer(cam, "denoiser_normal")
        dep = r.buffer(cam, "depth")
        x = denoiser.make_input(raw[None], alb[None], dn[None], dep[None])
        with torch.no_grad():
            y = model(torch.from_numpy(np.ascontiguousarray(x)).cuda(), bf16_activations=True)
        want = np.expm1(np.maximum(y[0].permute(1, 2, 0).cpu().numpy(), 0.0))
        got = r.buffer(cam, "denoised")[..., :3]
        assert np.array_equal(r.download(cam).beauty_rgba, r.buffer(cam, "denoised"))
        rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-2)
        assert np.median(rel) <= 2e-3, f"camera {cam}: median {np.median(rel):.2e}"
        assert np.quantile(rel, 0.999) <= 5e-2, f"camera {cam}: 99.9% {np.quantile(rel, 0.999):.2e}"
    # without parameters the plain beauty comes back
    r.set_denoiser(None)
    r.render_frame(rig, prof, 3)
    assert np.array_equal(r.download(0).beauty_rgba, r.buffer(0, "beauty"))
