"""Writes a small raw capture in the reference's on-disk frame format (fast_bp/sar_io.py:18-82):
an arbitrary prefix, then frames of a 160-byte header (8-byte start marker, pulse number,
bandwidth, pulse width, sampling delay, PRT, window, attitude, navigation), int16 I/Q pairs and
a 32-byte trailer.  Deterministic (seeded); two frames carry a corrupted marker and must be
skipped by the reader.  Used by make_golden.py (reference outputs) and by the tests."""
from __future__ import annotations

from pathlib import Path

import numpy as np

MAGIC = bytes([0, 52, 0, 52, 243, 250, 243, 250])
FS = 400e6


def write_capture(path: Path, frames: int = 24, window: int = 60, seed: int = 314) -> Path:
    rng = np.random.default_rng(seed)
    nr = round(window * 1e-8 * FS)
    size = 192 + 4 * nr
    buf = bytearray(rng.integers(0, 256, 37, dtype=np.uint8).tobytes())  # prefix before the first marker
    for i in range(frames):
        f = bytearray(size)
        f[0:8] = MAGIC if i not in (5, 17) else bytes(8)
        hdr = {36: ("<u4", 1000 + i + (i > 9)), 40: ("<u4", 200_000_000), 48: ("<i2", 100), 50: ("<i2", 200),
               52: ("<u4", 100_000), 60: ("<i2", window), 71: ("<i2", 1234 + i), 73: ("<i2", -20 + i),
               75: ("<i2", 7 - i), 101: ("<i8", 49_250_000_000 + 1000 * i), 109: ("<i8", -123_100_000_000 - 700 * i),
               117: ("<i4", 120_000 + 5 * i), 121: ("<i4", 3000 + i), 125: ("<i4", -1500 + 2 * i), 129: ("<i4", 10 - i),
               133: ("<i8", 49_250_000_100 + 1000 * i), 141: ("<i8", -123_100_000_100 - 700 * i),
               149: ("<u4", 5000 + 10 * (i // 3)), 155: ("u1", 11)}
        for off, (dt, val) in hdr.items():
            b = np.array([val], dtype=dt).tobytes()
            f[off:off + len(b)] = b
        iq = rng.integers(-2048, 2048, (nr, 2), dtype=np.int16)
        f[160:160 + 4 * nr] = iq.astype("<i2").tobytes()
        f[160 + 4 * nr:] = rng.integers(0, 256, 32, dtype=np.uint8).tobytes()
        buf += f
    buf += bytes(50)  # a partial frame at the end
    path = Path(path)
    path.write_bytes(bytes(buf))
    return path
