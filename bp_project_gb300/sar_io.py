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


# ---- raw capture frames (fast_bp/sar_io.py:18-82) ---------------------------------------
MAGIC = bytes([0, 52, 0, 52, 243, 250, 243, 250])
HEADER_BYTES = 160
TRAILER_BYTES = 32
# (name, numpy type, shape, byte offset in the frame): the capture's on-disk header layout.
_HEADER = [("magic", "u1", (8,), 0), ("number", "<u4", (), 36), ("bandwidth", "<u4", (), 40), ("tp", "<i2", (), 48),
           ("delay", "<i2", (), 50), ("prt", "<u4", (), 52), ("window", "<i2", (), 60), ("heading", "<i2", (), 71),
           ("pitch", "<i2", (), 73), ("roll", "<i2", (), 75), ("lat", "<i8", (), 101), ("lon", "<i8", (), 109),
           ("alt", "<i4", (), 117), ("ve", "<i4", (), 121), ("vn", "<i4", (), 125), ("vu", "<i4", (), 129),
           ("lat_gnss", "<i8", (), 133), ("lon_gnss", "<i8", (), 141), ("gps_ms", "<u4", (), 149), ("sv", "u1", (), 155)]
_SCALE = {"lat": 1e-9, "lon": 1e-9, "lat_gnss": 1e-9, "lon_gnss": 1e-9, "alt": 1e-3, "ve": 0.01, "vn": 0.01,
          "vu": 0.01, "heading": 0.01, "pitch": 0.01, "roll": 0.01}


class Capture:
    """A raw capture file: headers parsed on the host, I/Q decoded on the GPU (``read``).

    Frames are located from the first start marker in the first 10 MB; a frame is
    valid when its marker is intact.  Attributes follow the reference reader:
    ``nr``, ``frame_size``, ``offset``, ``n``, ``valid_indices``, ``nav`` (scaled
    navigation fields of the valid frames), ``tp``, ``delay``, ``prf``,
    ``bandwidth``, ``time`` and ``summary``."""

    def __init__(self, path):
        from pathlib import Path
        self.path = Path(path)
        with self.path.open("rb") as f:
            head = f.read(10_000_000)
        self.offset = head.find(MAGIC)
        if self.offset < 0:
            raise ValueError("Frame marker not found in first 10 MB")
        window = int(np.frombuffer(head, "<i2", 1, self.offset + 60)[0])
        self.nr = round(window * 1e-8 * FS)
        self.frame_size = HEADER_BYTES + 4 * self.nr + TRAILER_BYTES
        size = self.path.stat().st_size
        count = (size - self.offset) // self.frame_size
        names, formats, offsets = [], [], []
        for name, dt, shape, off in _HEADER:
            names.append(name)
            formats.append((dt, shape) if shape else dt)
            offsets.append(off)
        names.append("iq")
        formats.append(("<i2", (self.nr, 2)))
        offsets.append(HEADER_BYTES)
        dtype = np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": self.frame_size})
        self.frames = np.memmap(self.path, dtype=dtype, mode="r", offset=self.offset, shape=(count,))
        self._bytes = np.memmap(self.path, dtype=np.uint8, mode="r", offset=self.offset,
                                shape=(count, self.frame_size))
        good = np.all(self.frames["magic"] == np.frombuffer(MAGIC, np.uint8), axis=1)
        self.valid_indices = np.flatnonzero(good)
        if not len(self.valid_indices):
            raise ValueError("No valid frames")
        self.n = len(self.valid_indices)
        self.nav = {k: np.asarray(self.frames[k][good], dtype=np.float64) * _SCALE.get(k, 1)
                    for k in ["number", "gps_ms", "sv", *_SCALE]}
        for k in ("tp", "delay", "prt", "bandwidth", "window"):
            if len(np.unique(np.asarray(self.frames[k][good]))) != 1:
                raise ValueError(f"Changing {k} requires per-pulse handling")
        first = self.frames[self.valid_indices[0]]
        self.tp = float(first["tp"]) * 1e-8
        self.delay = float(first["delay"]) * 1e-8 - 0.2e-6
        self.prf = 1 / (float(first["prt"]) * 1e-8)
        self.bandwidth = float(first["bandwidth"])
        self.time = (self.nav["number"] - self.nav["number"][0]) / self.prf
        if np.any(np.diff(self.time) <= 0):
            raise ValueError("Non-monotonic pulse numbering")
        self.summary = dict(file=str(self.path.resolve()), bytes=size, first_frame_offset=self.offset,
                            frame_bytes=self.frame_size, complete_frame_slots=count, valid_frames=self.n,
                            invalid_slots=int((~good).sum()), first_pulse=int(self.nav["number"][0]),
                            last_pulse=int(self.nav["number"][-1]),
                            missing_pulses=int(np.sum(np.diff(self.nav["number"]) - 1)), range_samples=self.nr,
                            sample_rate_hz=FS, carrier_hz=FC, bandwidth_hz=self.bandwidth, pulse_width_s=self.tp,
                            sampling_delay_s=self.delay, prf_hz=self.prf, duration_s=float(self.time[-1]),
                            discarded_partial_bytes=int((size - self.offset) % self.frame_size))

    def read(self, indices, device=None):
        """complex64 [len(indices), nr] of the valid pulses ``indices``: the frames' bytes go to the
        device once and ``sarbp_decode_iq`` converts them.  A CUDA tensor when ``device`` is given,
        else a host array."""
        rows = self.valid_indices[np.asarray(indices)]
        raw = np.ascontiguousarray(self._bytes[rows])
        dev = torch.device(device) if device is not None else torch.device("cuda")
        frames = torch.from_numpy(raw).pin_memory().to(dev, non_blocking=True)
        out = torch.empty((len(rows), self.nr), dtype=torch.complex64, device=dev)
        nat.check(nat.load().sarbp_decode_iq(core._ptr(frames), len(rows), self.frame_size, HEADER_BYTES, self.nr,
                                             core._ptr(out), core.stream_handle()), "decode_iq")
        return out if device is not None else out.cpu().numpy()
