"""numpy-facing wrappers of the CPU oracle with the reference's function names.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Signatures follow
``fast_bp/ffbp.py``: ``bp_polar`` (:58), ``backproject_points`` (:43),
``regrid`` (:79), ``form_ffbp`` (:114), ``evaluate_image`` (:189),
``target_contributions`` (:202), ``cubic_weights`` (:17), ``sample1`` (:24),
``sample2`` (:32).  Each returns complex64 like the reference; the ``*_c128``
variants return the FP64 accumulators before the complex64 rounding (the
"FP64 oracle" image).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import build as _build
from .plan import LIGHT_SPEED, plan_ffbp

_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int64
_D = ctypes.c_double


def _load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(str(path))
        sig = {
            "oracle_set_threads": ([ctypes.c_int], ctypes.c_int),
            "oracle_bp_polar": ([_P, _I, _I, _P, _P, _D, _D, _I, _D, _D, _I, _D, _D, _D, _P, _P,
                                 ctypes.c_int, _P, _P], None),
            "oracle_backproject_points": ([_P, _I, _I, _P, _P, _I, _D, _D, _D, _P, _P, _P, _P], None),
            "oracle_regrid": ([_P, _I, _I, _P, _D, _D, _D, _D, _P, _D, _D, _I, _D, _D, _I, _D,
                               ctypes.c_int, _P, _P], None),
            "oracle_evaluate_image": ([_P, _I, _I, _P, _D, _D, _D, _D, _P, _I, _D, _P, _P], None),
            "oracle_target_contributions": ([_P, _I, _I, _P, _P, _I, _D, _D, _D, _P], None),
            "oracle_ffbp_execute": ([_P, _I, _I, _P, _P, _P, _I, _D, _D, _D, _P, _P, _P, _P], None),
        }
        for name, (args, res) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def set_threads(n: int = 0) -> int:
    """Set the OpenMP thread count (0 keeps the current one); returns the count in use."""
    return int(_load().oracle_set_threads(int(n)))


def _c64(a):
    a = np.ascontiguousarray(a)
    if a.dtype != np.complex64:
        raise TypeError("complex64 array expected")
    return a


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _outs(shape, c128):
    out = np.empty(shape, np.complex64)
    full = np.empty(shape, np.complex128) if c128 else None
    return out, full


def cubic_weights(t):
    """ffbp.py:17-21."""
    return (-t * (t - 1) * (t - 2) / 6, (t + 1) * (t - 1) * (t - 2) / 2,
            -(t + 1) * t * (t - 2) / 2, (t + 1) * t * (t - 1) / 6)


def sample1(row, q):
    """ffbp.py:24-29 (scalar, pure Python)."""
    i = int(math.floor(q))
    t = q - i
    if i < 1 or i + 2 >= len(row):
        return 0j
    w = cubic_weights(t)
    return w[0] * complex(row[i - 1]) + w[1] * complex(row[i]) + w[2] * complex(row[i + 1]) + w[3] * complex(row[i + 2])


def sample2(img, r, u):
    """ffbp.py:32-40 (scalar, pure Python)."""
    ir = int(math.floor(r))
    iu = int(math.floor(u))
    if ir < 1 or iu < 1 or ir + 2 >= img.shape[0] or iu + 2 >= img.shape[1]:
        return 0j
    wr = cubic_weights(r - ir)
    wu = cubic_weights(u - iu)
    z = 0j
    for a in range(4):
        for b in range(4):
            z += complex(img[ir + a - 1, iu + b - 1]) * wr[a] * wu[b]
    return z


def bp_polar(data, pos, origin, r0, dr, nr, u0, du, nu, r_start, data_dr, k, weight, phase, side,
             c128=False):
    """ffbp.py:58-76.  Returns complex64 [nr, nu] (and the complex128 image if ``c128``)."""
    data = _c64(data)
    p = data.shape[0]
    pos = _f64(pos, (p, 3))
    weight = _f64(weight, (p,))
    phase = _f64(phase, (p,))
    origin = _f64(origin, (3,))
    out, full = _outs((int(nr), int(nu)), c128)
    _load().oracle_bp_polar(_ptr(data), p, data.shape[1], _ptr(pos), _ptr(origin), r0, dr, int(nr),
                            u0, du, int(nu), r_start, data_dr, k, _ptr(weight), _ptr(phase), int(side),
                            _ptr(out), _ptr(full) if c128 else None)
    return (out, full) if c128 else out


def backproject_points(data, pos, xyz, r_start, dr, k, weight, phase, c128=False):
    """ffbp.py:43-55.  Returns complex64 [M] (and complex128 if ``c128``)."""
    data = _c64(data)
    p = data.shape[0]
    pos = _f64(pos, (p, 3))
    xyz = _f64(xyz)
    if xyz.ndim != 2 or xyz.shape[1] != 3:
        raise ValueError("xyz must be [M, 3]")
    weight = _f64(weight, (p,))
    phase = _f64(phase, (p,))
    out, full = _outs((xyz.shape[0],), c128)
    _load().oracle_backproject_points(_ptr(data), p, data.shape[1], _ptr(pos), _ptr(xyz), xyz.shape[0],
                                      r_start, dr, k, _ptr(weight), _ptr(phase), _ptr(out),
                                      _ptr(full) if c128 else None)
    return (out, full) if c128 else out


def regrid(img, src_origin, sr0, sdr, su0, sdu, dst_origin, r0, dr, nr, u0, du, nu, k, side, c128=False):
    """ffbp.py:79-95."""
    img = _c64(img)
    so = _f64(src_origin, (3,))
    do = _f64(dst_origin, (3,))
    out, full = _outs((int(nr), int(nu)), c128)
    _load().oracle_regrid(_ptr(img), img.shape[0], img.shape[1], _ptr(so), sr0, sdr, su0, sdu, _ptr(do),
                          r0, dr, int(nr), u0, du, int(nu), k, int(side), _ptr(out),
                          _ptr(full) if c128 else None)
    return (out, full) if c128 else out


def evaluate_image(img, origin, r0, dr, u0, du, xyz, k, c128=False):
    """ffbp.py:189-198."""
    img = _c64(img)
    origin = _f64(origin, (3,))
    xyz = _f64(xyz)
    out, full = _outs((xyz.shape[0],), c128)
    _load().oracle_evaluate_image(_ptr(img), img.shape[0], img.shape[1], _ptr(origin), r0, dr, u0, du,
                                  _ptr(xyz), xyz.shape[0], k, _ptr(out), _ptr(full) if c128 else None)
    return (out, full) if c128 else out


def target_contributions(data, pos, xyz, r_start, dr, k):
    """ffbp.py:201-211.  Returns complex64 [M, P]."""
    data = _c64(data)
    p = data.shape[0]
    pos = _f64(pos, (p, 3))
    xyz = _f64(xyz)
    out = np.empty((xyz.shape[0], p), np.complex64)
    _load().oracle_target_contributions(_ptr(data), p, data.shape[1], _ptr(pos), _ptr(xyz), xyz.shape[0],
                                        r_start, dr, k, _ptr(out))
    return out


@dataclass
class PolarImage:
    """ffbp.py:98-111."""
    image: np.ndarray
    origin: np.ndarray
    r0: float
    dr: float
    u0: float
    du: float
    side: int

    @property
    def r(self):
        return self.r0 + self.dr * np.arange(self.image.shape[0])

    @property
    def u(self):
        return self.u0 + self.du * np.arange(self.image.shape[1])


def form_ffbp(data, pos, r_start, data_dr, fc, extent, side=1, leaf_size=128, range_spacing=0.25,
              angular_oversample=2.5, weight=None, phase=None, plan=None):
    """ffbp.py:114-180 on the CPU oracle.  Returns (PolarImage, counts)."""
    data = _c64(data)
    p = data.shape[0]
    pos = _f64(pos, (p, 3))
    weight = np.ones(p) if weight is None else weight
    phase = np.zeros(p) if phase is None else phase
    weight = _f64(weight, (p,))
    phase = _f64(phase, (p,))
    k = 4 * np.pi * fc / LIGHT_SPEED
    if plan is None:
        plan = plan_ffbp(pos, fc, extent, side, leaf_size, range_spacing, angular_oversample)
    geom, idx = plan.tables()
    root = plan.root
    full = np.empty((root.nr, root.nu), np.complex64)
    counts = np.zeros(4, np.int64)
    _load().oracle_ffbp_execute(_ptr(data), p, data.shape[1], _ptr(pos), _ptr(geom), _ptr(idx), 0,
                                r_start, data_dr, k, _ptr(weight), _ptr(phase), _ptr(full), _ptr(counts))
    (ra, rb), (ua, ub) = plan.crop_r, plan.crop_u
    image = full[ra:rb, ua:ub].copy()
    result = PolarImage(image, root.origin.copy(), root.r0 + ra * root.dr, root.dr,
                        root.u0 + ua * root.du, root.du, int(side))
    names = ("leaves", "merges", "leaf_pixel_pulse_products", "merged_pixels")
    out_counts = {n: int(v) for n, v in zip(names, counts)}
    out_counts["shape"] = list(image.shape)
    return result, out_counts
