"""Native training of the denoiser U-Net (rtgb_trainer_*): one step's parameter
gradients against PyTorch autograd of the same network, and a short Adam run
on a fixed batch.

The native step keeps activations and inter-layer gradients in BF16 (as the
inference path stores activations); the PyTorch mirror rounds every layer's
output to BF16, and autograd then rounds the gradient at each rounding point
too, so the two differ by fp32 summation order and by BF16 flips that
propagate backwards. Bound: the flat gradient vectors agree to cosine 0.999,
and every layer's weight gradient to 5 % relative L2 error.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi, denoiser

pytestmark = pytest.mark.gpu


def _blocked(a: np.ndarray) -> np.ndarray:
    """(n, c, h, w) -> channel-blocked (n, c/8, h, w, 8)."""
    n, c, h, w = a.shape
    return np.ascontiguousarray(a.reshape(n, c // 8, 8, h, w).transpose(0, 1, 3, 4, 2))


def _batch(rng, n, h, w):
    x = np.zeros((n, 16, h, w), np.float32)
    x[:, 0:3] = rng.uniform(0.0, 2.5, (n, 3, h, w))       # log1p radiance
    x[:, 3:6] = rng.uniform(0.0, 1.0, (n, 3, h, w))       # albedo
    x[:, 6:9] = rng.uniform(-1.0, 1.0, (n, 3, h, w))      # camera-space normal
    x[:, 9] = rng.uniform(0.5, 3.0, (n, h, w))            # log1p depth
    x = denoiser.from_bf16_bits(denoiser.to_bf16_bits(x.ravel())).reshape(x.shape)
    # a smooth target in log space
    t = 0.5 * (x[:, 0:3] + np.roll(x[:, 0:3], 1, axis=3)) + 0.1 * x[:, 3:6]
    return x, np.ascontiguousarray(t.transpose(0, 2, 3, 1)).astype(np.float32)


def _trainer(torch, flat, n, h, w):
    lib = abi.load()
    tr = C.c_void_p()
    st = lib.rtgb_trainer_create(n, h, w, flat.ctypes.data, flat.size, C.byref(tr))
    assert st == 0, "rtgb_trainer_create failed"
    return lib, tr


def test_one_step_gradients_match_autograd():
    torch = pytest.importorskip("torch")
    torch.manual_seed(3)
    model = denoiser.build_model()
    flat = denoiser.from_bf16_bits(denoiser.to_bf16_bits(denoiser.flatten(model))).astype(np.float32)
    denoiser.unflatten(model, flat)
    n, h, w = 2, 48, 40
    rng = np.random.default_rng(5)
    x, t = _batch(rng, n, h, w)
    dev = torch.device("cuda", 0)
    xb = torch.from_numpy(_blocked(x)).to(dev).to(torch.bfloat16).contiguous()
    tt = torch.from_numpy(t).to(dev).contiguous()
    lib, tr = _trainer(torch, flat, n, h, w)
    try:
        loss = C.c_float()
        st = lib.rtgb_trainer_step(tr, C.c_void_p(xb.data_ptr()), C.c_void_p(tt.data_ptr()), 0.0, C.byref(loss))
        assert st == 0, lib.rtgb_trainer_last_error(tr)
        got = np.empty_like(flat)
        assert lib.rtgb_trainer_gradients(tr, got.ctypes.data) == 0
    finally:
        lib.rtgb_trainer_destroy(tr)
    model = model.to(dev)
    out = model(torch.from_numpy(x[:, :10]).to(dev), bf16_activations=True)
    ref_loss = torch.nn.functional.l1_loss(out, tt.permute(0, 3, 1, 2))
    ref_loss.backward()
    parts = []
    for conv in model.convs:
        parts += [conv.weight.grad.detach().float().cpu().numpy().ravel(), conv.bias.grad.detach().float().cpu().numpy().ravel()]
    ref = np.concatenate(parts)
    assert abs(float(loss.value) - float(ref_loss.item())) <= 1e-3 * float(ref_loss.item())
    cos = float(np.dot(got, ref) / (np.linalg.norm(got) * np.linalg.norm(ref)))
    assert cos > 0.999, cos
    off = 0
    for li, (ci, co) in enumerate(denoiser.LAYERS):
        nw = co * ci * 9
        g, r = got[off:off + nw], ref[off:off + nw]
        rel = float(np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-12))
        assert rel < 0.05, f"layer {li}: weight gradient relative error {rel:.3e}"
        off += nw + co


def test_adam_steps_reduce_the_loss():
    torch = pytest.importorskip("torch")
    torch.manual_seed(4)
    flat = denoiser.flatten(denoiser.build_model()).astype(np.float32)
    n, h, w = 4, 32, 32
    x, t = _batch(np.random.default_rng(6), n, h, w)
    dev = torch.device("cuda", 0)
    xb = torch.from_numpy(_blocked(x)).to(dev).to(torch.bfloat16).contiguous()
    tt = torch.from_numpy(t).to(dev).contiguous()
    lib, tr = _trainer(torch, flat, n, h, w)
    try:
        losses = []
        for _ in range(40):
            loss = C.c_float()
            assert lib.rtgb_trainer_step(tr, C.c_void_p(xb.data_ptr()), C.c_void_p(tt.data_ptr()), 2e-3,
                                         C.byref(loss)) == 0, lib.rtgb_trainer_last_error(tr)
            losses.append(float(loss.value))
        params = np.empty_like(flat)
        assert lib.rtgb_trainer_params(tr, params.ctypes.data) == 0
    finally:
        lib.rtgb_trainer_destroy(tr)
    assert np.all(np.isfinite(losses)) and np.all(np.isfinite(params))
    assert losses[-1] < 0.5 * losses[0], losses
