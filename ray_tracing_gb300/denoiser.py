"""The learned denoiser's network in PyTorch: the training model and the
floating-point reference of the tensor-core inference path
(csrc/denoiser.cu, which runs the same network in BF16 on the GPU).

Network: a three-level U-Net of 3x3 convolutions (ReLU after every layer but
the last), 2x2 average pooling, nearest 2x upsampling and skip connections by
channel concatenation (skip first, upsampled second):

    full  in(10) -> 32 -> 32 ........................... cat(32 + 48) -> 32 -> 32 -> 3
    1/2           pool -> 48 -> 48 ....... cat(48 + 64) -> 48 -> 48 -> up
    1/4                   pool -> 64 -> 64 -> up

Input per pixel: log1p(radiance) (3), albedo (3), camera-space normal (3),
log1p(depth) (1). Output: log1p(radiance), mapped back with expm1.
``flatten`` / ``unflatten`` give the parameter order of
``rtgb_set_denoiser_params``: per layer the weight (out x in x 3 x 3) then the
bias.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

LAYERS = [  # (in, out) of the 11 convolutions, in order
    (10, 32), (32, 32), (32, 48), (48, 48), (48, 64), (64, 64), (112, 48), (48, 48), (80, 32), (32, 32), (32, 3),
]
# the trained parameters: param_count() little-endian BF16 values, layer order
# (also read by rtgb_load_denoiser_file); training metadata beside it as JSON
WEIGHTS = Path(__file__).resolve().parent / "weights" / "denoiser_unet.bf16"


def param_count() -> int:
    return sum(o * i * 9 + o for i, o in LAYERS)


def make_input(beauty: np.ndarray | "torch.Tensor", albedo, dnormal, depth, xp=np):
    """Network input (N, 10, H, W) from the frame AOVs (N, H, W, 4 / 1), as k_dn_pack builds it."""
    if xp is np:
        lb = np.log1p(np.maximum(beauty[..., :3], 0.0))
        ld = np.log1p(np.maximum(depth, 0.0))[..., None]
        return np.concatenate([lb, albedo[..., :3], dnormal[..., :3], ld], axis=-1).transpose(0, 3, 1, 2)
    lb = xp.log1p(beauty[..., :3].clamp_min(0.0))
    ld = xp.log1p(depth.clamp_min(0.0))[..., None]
    return xp.cat([lb, albedo[..., :3], dnormal[..., :3], ld], dim=-1).permute(0, 3, 1, 2)


def blocked_input(x):
    """Network input (N, 10, H, W) torch tensor -> the native path's layout:
    16 channels (6 zero), channel-blocked (N, 2, H, W, 8), BF16, contiguous."""
    import torch
    n, c, h, w = x.shape
    x16 = torch.zeros((n, 16, h, w), dtype=torch.float32, device=x.device)
    x16[:, :c] = x
    return x16.reshape(n, 2, 8, h, w).permute(0, 1, 3, 4, 2).to(torch.bfloat16).contiguous()


def build_model():
    import torch
    import torch.nn.functional as F

    class UNet(torch.nn.Module):
        def __init__(self):
            super().__init__()
            self.convs = torch.nn.ModuleList([torch.nn.Conv2d(i, o, 3, padding=1) for i, o in LAYERS])

        def forward(self, x, bf16_activations: bool = False):
            """log1p radiance (N, 3, H, W). With bf16_activations every layer's
            output is rounded to BF16 as the GPU path stores it."""
            q = (lambda t: t.to(torch.bfloat16).float()) if bf16_activations else (lambda t: t)
            c = self.convs
            x = q(x)
            e1 = q(F.relu(c[1](q(F.relu(c[0](x))))))
            p1 = q(F.avg_pool2d(e1, 2, ceil_mode=True))
            e2 = q(F.relu(c[3](q(F.relu(c[2](p1))))))
            p2 = q(F.avg_pool2d(e2, 2, ceil_mode=True))
            e3 = q(F.relu(c[5](q(F.relu(c[4](p2))))))
            u2 = _up(e3, e2.shape[-2:])
            d2 = q(F.relu(c[7](q(F.relu(c[6](torch.cat([e2, u2], 1)))))))
            u1 = _up(d2, e1.shape[-2:])
            d1 = q(F.relu(c[9](q(F.relu(c[8](torch.cat([e1, u1], 1)))))))
            return q(c[10](d1))

    return UNet()


def _up(t, hw):
    t = t.repeat_interleave(2, dim=2).repeat_interleave(2, dim=3)
    return t[..., : hw[0], : hw[1]]


def flatten(model) -> np.ndarray:
    parts = []
    for conv in model.convs:
        parts.append(conv.weight.detach().float().cpu().numpy().ravel())
        parts.append(conv.bias.detach().float().cpu().numpy().ravel())
    flat = np.concatenate(parts).astype(np.float32)
    assert flat.size == param_count()
    return flat


def unflatten(model, flat: np.ndarray) -> None:
    import torch
    assert flat.size == param_count()
    off = 0
    with torch.no_grad():
        for conv in model.convs:
            for t in (conv.weight, conv.bias):
                n = t.numel()
                t.copy_(torch.from_numpy(np.asarray(flat[off:off + n], np.float32).reshape(t.shape)))
                off += n


def to_bf16_bits(flat: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(flat, np.float32).view(np.uint32)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bf16_bits(bits: np.ndarray) -> np.ndarray:
    return (bits.astype(np.uint32) << 16).view(np.float32)


def load_weights(path: Path = WEIGHTS) -> np.ndarray | None:
    """The trained parameters shipped with the package (BF16), as float32."""
    if not path.exists():
        return None
    bits = np.fromfile(path, dtype="<u2")
    if bits.size != param_count():
        raise ValueError(f"{path}: {bits.size} values, expected {param_count()}")
    return from_bf16_bits(bits)


def save_weights(flat: np.ndarray, path: Path = WEIGHTS, meta: dict | None = None) -> None:
    import json
    path.parent.mkdir(parents=True, exist_ok=True)
    to_bf16_bits(flat).astype("<u2").tofile(path)
    if meta is not None:
        path.with_suffix(".json").write_text(json.dumps(meta, indent=1) + "\n")
