"""BF16 storage as the library stores it (k_pack in kernels_sweep.cu), restated in numpy so
that the FP64 oracle can be fed the same rounded field: test infrastructure."""
import numpy as np


def bf16_bits(a):
    """Round-to-nearest-even BF16 patterns (upper 16 bits of float32) of finite inputs."""
    u = np.ascontiguousarray(a, np.float32).reshape(-1).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32)


def round_bf16(a):
    """Gradient components as stored: nearest even BF16, as float32."""
    return (bf16_bits(a) << 16).view(np.float32)


def curl_bf16(c, thr=None):
    """The stored curl: nearest even BF16, a nonzero curl never zero, and with a threshold
    every decision kept against the threshold's BF16 truncation.  Returns (curl as float32,
    the threshold the kernels compare against)."""
    c = np.ascontiguousarray(c, np.float32).reshape(-1)
    v = bf16_bits(c)
    v = np.where((c != 0) & ((v & 0x7FFF) == 0), v | 1, v)
    v = np.where(c == 0, c.view(np.uint32) >> 16, v)
    t_out = 0.0 if thr is None else thr
    if thr is not None and thr > 0:
        t = np.uint32(np.float32(thr).view(np.uint32) >> 16)
        pos = c > 0
        v = np.where(pos & (c < np.float32(thr)) & (v >= t), t - 1, v)
        v = np.where(pos & (c == np.float32(thr)), t, v)
        v = np.where(pos & (c > np.float32(thr)) & (v <= t), t + 1, v)
        t_out = float(np.uint32(t << 16).view(np.float32))
    return (v.astype(np.uint32) << 16).view(np.float32), t_out
