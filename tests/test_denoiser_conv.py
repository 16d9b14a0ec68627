"""The denoiser's 3x3 convolution primitive (tcgen05 implicit GEMM) against a
plain PyTorch fp32 conv2d of the same BF16-rounded inputs and weights.

Tolerance: the kernel accumulates in fp32 (another summation order than
PyTorch's) and rounds its output to BF16 (8 significant bits), so outputs must
agree within 1 % relative with a 1e-2 absolute floor scaled by the output's
magnitude.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi


def _pack(w: np.ndarray, cin: int) -> np.ndarray:
    cout, cin_used = w.shape[:2]
    out = np.zeros(9 * cin * cout, dtype=np.uint16)
    lib = abi.load()
    w = np.ascontiguousarray(w, dtype=np.float32)
    assert lib.rtgb_conv3x3_pack_weights(w.ctypes.data, cout, cin_used, cin, out.ctypes.data) == 0
    return out


def _bf16_round(a: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.view(np.float32)


def test_weight_packing_layout():
    rng = np.random.default_rng(1)
    cout, cin_used, cin = 16, 10, 16
    w = rng.standard_normal((cout, cin_used, 3, 3)).astype(np.float32)
    packed = _pack(w, cin).reshape(9, cin // 8, cout, 8)
    wr = _bf16_round(w)
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        for b in range(cin // 8):
            for j in range(8):
                ci = b * 8 + j
                want = wr[:, ci, dy, dx] if ci < cin_used else np.zeros(cout, np.float32)
                got = (packed[tap, b, :, j].astype(np.uint32) << 16).view(np.float32)
                assert np.array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("n,h,w,cin,cout,relu,ych,yoff", [
    (1, 16, 8, 16, 16, 0, 16, 0),      # one tile, one K step per tap
    (2, 37, 29, 16, 32, 1, 32, 0),     # ragged tiles at both borders
    (1, 45, 67, 48, 48, 1, 80, 32),    # write into a concatenation buffer at an offset
    (2, 33, 40, 112, 48, 1, 48, 0),    # the widest decoder layer
    (1, 24, 24, 128, 64, 0, 64, 0),    # largest shapes the kernel takes
])
def test_conv3x3_matches_torch(n, h, w, cin, cout, relu, ych, yoff):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(n * 1000 + h * 10 + cin)
    x = _bf16_round(rng.standard_normal((n, h, w, cin)).astype(np.float32))
    wt = rng.standard_normal((cout, cin, 3, 3)).astype(np.float32) * (1.0 / np.sqrt(9 * cin))
    bias = rng.standard_normal(cout).astype(np.float32) * 0.1
    packed = _pack(wt, cin)
    # channel-blocked [n][c/8][h][w][8] as the kernel reads it
    xb = np.ascontiguousarray(x.reshape(n, h, w, cin // 8, 8).transpose(0, 3, 1, 2, 4))
    xt = torch.from_numpy(xb).to(dev).to(torch.bfloat16).contiguous()
    pw = torch.from_numpy(packed.view(np.int16)).to(dev)
    bt = torch.from_numpy(bias).to(dev)
    y = torch.full((n, ych // 8, h, w, 8), 7.0, dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    msg = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev)
    st = abi.load().rtgb_conv3x3_bf16(xt.data_ptr(), n, h, w, cin, pw.data_ptr(), bt.data_ptr(), cout, relu,
                                       y.data_ptr(), ych, yoff, err.data_ptr(), C.c_void_p(stream.cuda_stream),
                                       msg, 256)
    assert st == 0, msg.value.decode()
    torch.cuda.synchronize(dev)
    assert int(err.item()) == 0, "a bounded wait in the kernel ran out"
    ref = torch.nn.functional.conv2d(torch.from_numpy(x).permute(0, 3, 1, 2).to(dev),
                                     torch.from_numpy(_bf16_round(wt)).to(dev), torch.from_numpy(bias).to(dev),
                                     padding=1)
    if relu:
        ref = torch.relu(ref)
    ref = ref.permute(0, 2, 3, 1).cpu().numpy()
    got = y.float().cpu().numpy().transpose(0, 2, 3, 1, 4).reshape(n, h, w, ych)
    out = got[..., yoff:yoff + cout]
    scale = max(1.0, float(np.abs(ref).max()))
    bad = np.abs(out - ref) > 1e-2 * np.maximum(np.abs(ref), 1e-2 * scale)
    assert not bad.any(), f"{bad.sum()} of {bad.size} outputs differ, max {np.abs(out - ref).max():.3e}"
    # channels outside [yoff, yoff + cout) are untouched
    other = np.delete(got, np.s_[yoff:yoff + cout], axis=-1)
    assert np.all(other == 7.0)
