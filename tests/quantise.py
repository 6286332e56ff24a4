"""The mixed-precision form's frame storage restated on the host.

The engine stores each frame as 16-bit values of value / scale, with one
FP32 scale per frame and velocity component (the component's largest
magnitude): scale = max |fl32(v)|, inv = fl32(1 / scale), q = RN16(fl32(v) *
inv) in BF16 or FP16, round to nearest even throughout (k_maxabs /
k_quantize in flowvc-1_gb300/csrc/fvc_mixed_kernels.cu).  dequantised()
returns q * scale in FP64: frames carrying exactly the storage error and
nothing else, so that the FP64 form run on them separates the error of
16-bit storage from the error of the FP32 arithmetic."""
from __future__ import annotations

import numpy as np


def _bf16_round(x32):
    u = np.ascontiguousarray(x32, np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16  # round to nearest even (finite inputs)
    return (r << 16).astype(np.uint32).view(np.float32)


def dequantised(uvw, fmt):
    """uvw: N x 3 float64 frame; fmt "bf16" or "fp16".  Returns the N x 3
    float64 frame the 16-bit storage represents."""
    v32 = np.asarray(uvw, np.float64).astype(np.float32)
    out = np.empty(v32.shape, np.float64)
    for c in range(3):
        mx = np.float32(np.abs(v32[:, c]).max()) if len(v32) else np.float32(0)
        scale = mx if (mx > 0 and mx < np.float32(3.0e38)) else np.float32(1.0)
        inv = np.float32(1.0) / scale
        x = v32[:, c] * inv                       # one FP32 rounding
        q = _bf16_round(x) if fmt == "bf16" else x.astype(np.float16).astype(np.float32)
        out[:, c] = q.astype(np.float64) * np.float64(scale)
    return out
