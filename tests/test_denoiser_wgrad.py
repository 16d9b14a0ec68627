"""The denoiser convolution's weight and bias gradients (tcgen05, MN-major
operands) against PyTorch's fp32 conv2d weight gradient of the same
BF16-rounded inputs.

Tolerance: both sides accumulate the BF16 products in fp32, in different
orders, over up to ~2,500 pixels per weight; gradients must agree within
1e-3 relative with an absolute floor of 1e-4 of the largest gradient.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from ray_tracing_gb300 import abi


def _bf16_round(a: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(a, np.float32).view(np.uint32)
    return ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).view(np.float32)


def _blocked(a: np.ndarray) -> np.ndarray:
    n, h, w, c = a.shape
    return np.ascontiguousarray(a.reshape(n, h, w, c // 8, 8).transpose(0, 3, 1, 2, 4))


@pytest.mark.gpu
@pytest.mark.parametrize("n,h,w,cin,cout", [
    (1, 16, 8, 16, 16),      # one tile
    (2, 37, 29, 32, 32),     # ragged tiles at both borders
    (1, 45, 67, 48, 48),
    (2, 33, 40, 112, 48),    # the widest decoder layer
    (1, 24, 24, 128, 64),    # largest shapes; taps in two TMEM groups
])
def test_wgrad_matches_torch(n, h, w, cin, cout):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(n * 1000 + h * 10 + cin)
    x = _bf16_round(rng.standard_normal((n, h, w, cin)).astype(np.float32))
    dy = _bf16_round(rng.standard_normal((n, h, w, cout)).astype(np.float32))
    xt = torch.from_numpy(_blocked(x)).to(dev).to(torch.bfloat16).contiguous()
    dyt = torch.from_numpy(_blocked(dy)).to(dev).to(torch.bfloat16).contiguous()
    dw = torch.full((cout, cin, 3, 3), 7.0, dtype=torch.float32, device=dev)
    db = torch.full((cout,), 7.0, dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    msg = C.create_string_buffer(256)
    stream = torch.cuda.current_stream(dev)
    st = abi.load().rtgb_conv3x3_wgrad_bf16(xt.data_ptr(), n, h, w, cin, dyt.data_ptr(), cout, dw.data_ptr(),
                                             db.data_ptr(), err.data_ptr(), C.c_void_p(stream.cuda_stream), msg, 256)
    assert st == 0, msg.value.decode()
    torch.cuda.synchronize(dev)
    assert int(err.item()) == 0, "a bounded wait in the kernel ran out"
    xr = torch.from_numpy(x).permute(0, 3, 1, 2).to(dev)
    dyr = torch.from_numpy(dy).permute(0, 3, 1, 2).to(dev)
    ref_w = torch.nn.grad.conv2d_weight(xr, (cout, cin, 3, 3), dyr, padding=1).cpu().numpy()
    ref_b = dyr.sum(dim=(0, 2, 3)).cpu().numpy()
    got_w = dw.cpu().numpy()
    got_b = db.cpu().numpy()
    scale = float(np.abs(ref_w).max())
    bad = np.abs(got_w - ref_w) > 1e-3 * np.abs(ref_w) + 1e-4 * scale
    assert not bad.any(), f"{bad.sum()} of {bad.size} weight gradients differ, max {np.abs(got_w - ref_w).max():.3e}"
    assert np.allclose(got_b, ref_b, rtol=1e-3, atol=1e-4 * float(np.abs(ref_b).max()))


def test_wgrad_rejects_bad_shapes():
    msg = C.create_string_buffer(256)
    lib = abi.load()
    st = lib.rtgb_conv3x3_wgrad_bf16(C.c_void_p(16), 1, 8, 8, 24, C.c_void_p(16), 16, C.c_void_p(16), None, None,
                                     None, msg, 256)
    assert st == abi.STATUS_CODES["INVALID_ARGUMENT"] if hasattr(abi, "STATUS_CODES") else st == 1
    assert b"multiple of 16" in msg.value
