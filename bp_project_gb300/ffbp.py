"""Drop-in for the reference's image-formation functions (fast_bp/ffbp.py).

Same names, argument order and complex64 results as the reference's Numba
kernels, computed on the GPU by libsarbp.  numpy arrays are uploaded for the
call and results downloaded; torch CUDA tensors are used in place (and the
result stays on the device).  ``mode`` selects the precision policy; the
default ``"split"`` is the fast split-precision path (relative error vs FP64
~1e-6), ``"fp64"`` reproduces the reference's FP64 arithmetic.

Coordinates: x cross-track, y along-track, z height above a flat scene.
Polar radius is slant range to each node's phase centre, u = sin(horizontal
angle); stored node images are demodulated by exp(-j k radius) (ffbp.py:1-8).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import core
from .gpu_backend import LIGHT_SPEED, build_ffbp_plan

DEFAULT_MODE = "split"


def cubic_weights(t):
    """Four-point Lagrange weights at floor(x)-1 .. floor(x)+2 (ffbp.py:17-21)."""
    return (-t * (t - 1) * (t - 2) / 6, (t + 1) * (t - 1) * (t - 2) / 2,
            -(t + 1) * t * (t - 2) / 2, (t + 1) * t * (t - 1) / 6)


def sample1(row, q):
    """Range interpolation of one row at fractional bin q (ffbp.py:24-29), host scalar helper."""
    i = int(math.floor(q))
    t = q - i
    if i < 1 or i + 2 >= len(row):
        return 0j
    w = cubic_weights(t)
    return sum(w[a] * complex(row[i + a - 1]) for a in range(4))


def sample2(img, r, u):
    """4x4 Lagrange on a polar image (ffbp.py:32-40), host scalar helper."""
    ir = int(math.floor(r))
    iu = int(math.floor(u))
    if ir < 1 or iu < 1 or ir + 2 >= img.shape[0] or iu + 2 >= img.shape[1]:
        return 0j
    wr = cubic_weights(r - ir)
    wu = cubic_weights(u - iu)
    return sum(complex(img[ir + a - 1, iu + b - 1]) * wr[a] * wu[b] for a in range(4) for b in range(4))


def _on_device(*arrays):
    return any(isinstance(a, torch.Tensor) and a.is_cuda for a in arrays)


def _inputs(data, pos, weight, phase):
    dev = data.device if isinstance(data, torch.Tensor) and data.is_cuda else torch.device("cuda")
    d = core.to_device(data, torch.complex64, dev)
    p = d.shape[0]
    if weight is None:
        weight = np.ones(p)
    if phase is None:
        phase = np.zeros(p)
    return (d, core.to_device(pos, torch.float64, dev), core.to_device(weight, torch.float64, dev),
            core.to_device(phase, torch.float64, dev))


def _result(t, keep):
    if keep:
        return t
    return t.cpu().numpy()


def morton_order(xyz: np.ndarray) -> np.ndarray:
    """Permutation that groups ground points into compact 2-D blocks (Z-order on x, y)."""
    xy = xyz[:, :2]
    lo = xy.min(axis=0)
    span = max(float((xy.max(axis=0) - lo).max()), 1e-9)
    q = np.clip(((xy - lo) / span * 65535.0).astype(np.int64), 0, 65535)

    def spread(v):
        v = (v | (v << 8)) & 0x00FF00FF
        v = (v | (v << 4)) & 0x0F0F0F0F
        v = (v | (v << 2)) & 0x33333333
        v = (v | (v << 1)) & 0x55555555
        return v

    return np.argsort(spread(q[:, 0]) | (spread(q[:, 1]) << 1), kind="stable")


LATTICE_TOL_M = 1e-9  # points within 1 nm of an affine lattice are imaged on it (phase change < 1e-6 rad)


def lattice_of(points):
    """(origin, step_row, step_col, rows, cols) if ``points`` [n, 3] (float64) list an affine lattice
    origin + i step_row + j step_col in row-major order to within LATTICE_TOL_M, else None."""
    n = len(points)
    if n < 2:
        return None
    o, sc = points[0], points[1] - points[0]
    j = np.arange(n, dtype=np.float64)[:, None]
    off = np.abs(points - (o + j * sc)).max(axis=1) > LATTICE_TOL_M
    cols = int(np.argmax(off)) if off.any() else n
    if n % cols:
        return None
    rows = n // cols
    sr = points[cols] - o if rows > 1 else np.zeros(3)
    i, jj = np.divmod(np.arange(n), cols)
    if np.abs(points - (o + i[:, None] * sr + jj[:, None] * sc)).max() > LATTICE_TOL_M:
        return None
    return tuple(o), tuple(sr), tuple(sc), rows, cols


def backproject_points(data, pos, xyz, r_start, dr, k, weight, phase, mode=DEFAULT_MODE):
    """Direct BP at arbitrary xyz: sum_n w[n] sample1 exp(j(k r + phase[n])) (ffbp.py:43-55).

    In split mode a host point list that is an affine lattice in row-major order (the ground
    meshgrids of run.py) is imaged by the lattice kernel, whose row/column terms make it the
    fastest path; any other point list goes through the points kernel in Morton order."""
    keep = _on_device(data, xyz)
    d, p, w, ph = _inputs(data, pos, weight, phase)
    order = None
    if isinstance(xyz, torch.Tensor):
        pts = xyz.to(device=d.device, dtype=torch.float64).contiguous()
    else:
        host = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        grid = lattice_of(host) if mode == "split" and len(host) > 1024 else None
        if grid is not None:
            origin, sr, sc, rows, cols = grid
            img = core.backproject_lattice(d, p, w, ph, origin, sr, sc, rows, cols, r_start, dr, k, mode=mode)
            return _result(img.reshape(-1), keep)
        if mode == "split" and len(host) > 1024:
            order = morton_order(host)
            host = np.ascontiguousarray(host[order])
        pts = torch.from_numpy(host).to(d.device)
    out = core.backproject_points(d, p, w, ph, pts, r_start, dr, k, mode=mode)
    if order is not None:
        inv = torch.empty_like(torch.from_numpy(order))
        inv[torch.from_numpy(order)] = torch.arange(len(order))
        out = out[inv.to(out.device)]
    return _result(out, keep)


def bp_polar(data, pos, origin, r0, dr, nr, u0, du, nu, r_start, data_dr, k, weight, phase, side, mode=DEFAULT_MODE):
    """BP onto the polar grid (r, u) about ``origin``, demodulated by exp(-jkr) (ffbp.py:58-76)."""
    keep = _on_device(data)
    d, p, w, ph = _inputs(data, pos, weight, phase)
    grid = core.Grid(tuple(float(v) for v in np.asarray(origin, np.float64)), r0, dr, int(nr), u0, du, int(nu),
                     int(side))
    return _result(core.direct_polar(d, p, w, ph, grid, r_start, data_dr, k, mode=mode), keep)


def regrid(img, src_origin, sr0, sdr, su0, sdu, dst_origin, r0, dr, nr, u0, du, nu, k, side, mode="mixed"):
    """Child polar image -> parent polar grid, times exp(jk(rr - r)) (ffbp.py:79-95)."""
    keep = _on_device(img)
    image = core.to_device(img, torch.complex64)
    src = core.Grid(tuple(np.asarray(src_origin, np.float64)), sr0, sdr, image.shape[0], su0, sdu, image.shape[1],
                    int(side))
    dst = core.Grid(tuple(np.asarray(dst_origin, np.float64)), r0, dr, int(nr), u0, du, int(nu), int(side))
    return _result(core.regrid(image, src, dst, k, mode=mode), keep)


@dataclass
class PolarImage:
    """Polar result plus axes (ffbp.py:98-111)."""
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


_programs = {}


def form_ffbp(data, pos, r_start, data_dr, fc, extent, side=1, leaf_size=128, range_spacing=0.25,
              angular_oversample=2.5, weight=None, phase=None, verbose=True, mode=DEFAULT_MODE):
    """Polar FFBP of a fixed world sector (ffbp.py:114-180).  Returns (PolarImage, counts)."""
    start = time.perf_counter()
    k = 4 * np.pi * fc / LIGHT_SPEED
    keep = _on_device(data)
    pos_host = pos.detach().cpu().numpy() if isinstance(pos, torch.Tensor) else np.ascontiguousarray(pos, np.float64)
    plan = build_ffbp_plan(pos_host, fc, extent, side=side, leaf_size=leaf_size, range_spacing=range_spacing,
                           angular_oversample=angular_oversample)
    d, p, w, ph = _inputs(data, pos, weight, phase)
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode=mode, device=d.device)
    try:
        image = prog.execute(d, p, w, ph, r_start, data_dr, k)
        torch.cuda.current_stream().synchronize()
    finally:
        prog.close()
    counts = {key: plan.counts[key] for key in ("leaves", "merges", "leaf_pixel_pulse_products", "merged_pixels")}
    counts["elapsed_s"] = time.perf_counter() - start
    counts["shape"] = list(plan.shape)
    if verbose:
        print(f"FFBP: {counts['leaves']} leaves, {counts['merges']} merges, {counts['elapsed_s']:.3f} s", flush=True)
    result = PolarImage(_result(image, keep), plan.origin.copy(), plan.r0, plan.dr, plan.u0, plan.du, int(side))
    return result, counts


def polar_points(origin, r, u, side=1):
    """Ground xyz of a polar grid (ffbp.py:183-186)."""
    rr, uu = np.meshgrid(r, u, indexing="ij")
    gr = np.sqrt(rr**2 - origin[2] ** 2)
    return np.column_stack([(origin[0] + side * gr * np.sqrt(1 - uu**2)).ravel(), (origin[1] + gr * uu).ravel(),
                            np.zeros(rr.size)])


def evaluate_image(img, origin, r0, dr, u0, du, xyz, k):
    """Polar image -> ground points via sample2 times exp(jkr) (ffbp.py:189-198)."""
    keep = _on_device(img)
    image = core.to_device(img, torch.complex64)
    grid = core.Grid(tuple(np.asarray(origin, np.float64)), r0, dr, image.shape[0], u0, du, image.shape[1], 1)
    pts = core.to_device(xyz, torch.float64, image.device)
    return _result(core.evaluate_image(image, grid, pts, k), keep)


def target_contributions(data, pos, xyz, r_start, dr, k):
    """Per target, per pulse sample1 * exp(jkr): complex64 [targets, pulses] (ffbp.py:201-211)."""
    keep = _on_device(data)
    d = core.to_device(data, torch.complex64)
    p = core.to_device(pos, torch.float64, d.device)
    pts = core.to_device(xyz, torch.float64, d.device)
    return _result(core.target_contributions(d, p, pts, r_start, dr, k), keep)
