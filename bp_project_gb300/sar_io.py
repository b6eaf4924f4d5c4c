"""Range compression on the GPU (fast_bp/sar_io.py:116-139 ``range_compress`` surface).

The step just before back-projection: each raw LFM echo is correlated with the
Hamming-weighted chirp reference by FFT, with the exact lag kept so that output
sample k is the echo centred on raw sample k, and optionally Fourier-interpolated
by ``oversample``.  The FFTs are cuFFT calls through torch; the
steps around them are libsarbp kernels (``sarbp_rc_prepare`` / ``_filter`` /
``_crop``), so the data stays on the device from raw samples to BP input.
"""
from __future__ import annotations

import numpy as np
import torch
from scipy import fft as sp_fft
from scipy.signal import windows

from . import _native as nat
from . import core

C = 299792458.0
FC = 1.4e9
FS = 400e6

_RESPONSES: dict = {}


def matched_filter(tp=1e-6, bandwidth=200e6, chirp_sign=-1, fs=FS):
    """Time-reversed conjugate of the centred, Hamming-weighted LFM reference (complex64)."""
    n = round(tp * fs)
    t = (np.arange(n) - n // 2) / fs
    ref = np.exp(1j * np.pi * chirp_sign * bandwidth / tp * t ** 2).astype(np.complex64)
    ref *= windows.hamming(n, sym=False).astype(np.float32)
    return np.conj(ref[::-1])


def _response(h: np.ndarray, nfft: int, device) -> torch.Tensor:
    key = (h.tobytes(), nfft, str(device))
    if key not in _RESPONSES:
        _RESPONSES[key] = torch.fft.fft(torch.from_numpy(np.ascontiguousarray(h)).to(device), n=nfft).contiguous()
    return _RESPONSES[key]


def range_compress(raw, tp=1e-6, bandwidth=200e6, chirp_sign=-1, oversample=1, fs=FS):
    """Linear correlation of every pulse with the LFM reference, exact lag kept.

    raw: complex64 [pulses, samples] (array or CUDA tensor).  Returns complex64
    [pulses, samples * oversample]; a CUDA tensor if raw was one, else an array.
    Sample k of the output corresponds to the echo centred on raw sample k / oversample."""
    keep = isinstance(raw, torch.Tensor) and raw.is_cuda
    x = core.to_device(raw, torch.complex64)
    if x.dim() != 2:
        raise ValueError("raw data must be [pulses, samples]")
    oversample = int(oversample)
    if oversample < 1:
        raise ValueError("oversample must be a positive integer")
    pulses, samples = x.shape
    h = matched_filter(tp, bandwidth, chirp_sign, fs)
    n = len(h)
    nfft = sp_fft.next_fast_len(samples + n - 1)
    lib = nat.load()
    stream = core.stream_handle()
    padded = torch.empty((pulses, nfft), dtype=torch.complex64, device=x.device)
    nat.check(lib.sarbp_rc_prepare(core._ptr(x), pulses, samples, nfft, core._ptr(padded), stream), "rc_prepare")
    spectrum = torch.fft.fft(padded, dim=1)
    length = nfft * oversample
    product = spectrum if oversample == 1 else torch.empty((pulses, length), dtype=torch.complex64, device=x.device)
    nat.check(lib.sarbp_rc_filter(core._ptr(spectrum), core._ptr(_response(h, nfft, x.device)), pulses, nfft, length,
                                  core._ptr(product), stream), "rc_filter")
    corr = torch.fft.ifft(product, dim=1)
    offset = n - 1 - n // 2
    out = torch.empty((pulses, samples * oversample), dtype=torch.complex64, device=x.device)
    nat.check(lib.sarbp_rc_crop(core._ptr(corr), pulses, length, offset * oversample, samples * oversample,
                                float(oversample), core._ptr(out), stream), "rc_crop")
    return out if keep else out.cpu().numpy()
