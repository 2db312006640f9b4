"""Helpers for GPU tests: numpy <-> torch device buffers in the library's formats."""
import numpy as np


def to_dev_f16(z):
    """complex numpy -> torch float16 [..., 2] interleaved on cuda:0."""
    import torch
    a = np.empty(z.shape + (2,), dtype=np.float16)
    a[..., 0] = z.real
    a[..., 1] = z.imag
    return torch.from_numpy(a).cuda()


def from_dev_f16(t):
    a = t.detach().cpu().numpy().astype(np.float64)
    return a[..., 0] + 1j * a[..., 1]


def to_dev_f32(z):
    import torch
    a = np.empty(z.shape + (2,), dtype=np.float32)
    a[..., 0] = z.real
    a[..., 1] = z.imag
    return torch.from_numpy(a).cuda()


def from_dev_f32(t):
    a = t.detach().cpu().numpy().astype(np.float64)
    return a[..., 0] + 1j * a[..., 1]


def f16_round(z):
    """The input exactly as the FP16 kernel sees it."""
    return (z.real.astype(np.float16).astype(np.float64)
            + 1j * z.imag.astype(np.float16).astype(np.float64))


def f32_round(z):
    """z with real and imaginary parts rounded to FP32 (complex128 result)."""
    return z.real.astype(np.float32).astype(np.float64) + 1j * z.imag.astype(np.float32).astype(np.float64)
