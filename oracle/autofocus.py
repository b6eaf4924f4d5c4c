"""CPU oracle of the reference's phase-gradient autofocus (fast_bp/autofocus.py).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): it checks the GPU
autofocus in ``tests/`` and is the CPU side of the autofocus timing.

A numpy/scipy restatement of ``pick_targets`` (autofocus.py:19-34),
``estimate_update`` (:37-79) and the iteration loop of ``main`` (:82-111),
with target contributions and FFBP from the C++ oracle (``reference.py``).
Pinned by ``tests/golden/autofocus.npz`` (outputs of the reference itself).
"""
from __future__ import annotations

import time

import numpy as np
from scipy import signal

from . import reference as ora


def pick_targets(image, r, u, origin, side, nr_tiles=12, nu_tiles=12):
    """Brightest cell per tile; cells below -35 dB of the brightest are dropped (autofocus.py:19-34)."""
    mag = np.abs(image)
    points, powers = [], []
    for rows in np.array_split(np.arange(len(r)), nr_tiles):
        for cols in np.array_split(np.arange(len(u)), nu_tiles):
            tile = mag[rows[0]:rows[-1] + 1, cols[0]:cols[-1] + 1]
            i, j = np.unravel_index(int(np.argmax(tile)), tile.shape)
            rr, uu = r[rows[i]], u[cols[j]]
            g = np.sqrt(rr * rr - origin[2] ** 2)
            points.append([origin[0] + side * g * np.sqrt(1 - uu * uu), origin[1] + g * uu, 0.0])
            powers.append(float(tile[i, j]) ** 2)
    points, powers = np.array(points), np.array(powers)
    keep = powers > powers.max() * 10 ** (-3.5)
    return points[keep], powers[keep]


def estimate_update(data, pos, points, r_start, dr, k, prf, cutoff, contributions=None):
    """Robust weighted LS fit of LOS phase-gradient residuals (autofocus.py:37-79)."""
    xi = ora.target_contributions(data, pos, points, r_start, dr, k) if contributions is None else contributions
    smooth = signal.sosfiltfilt(signal.butter(4, cutoff, fs=prf, output="sos"), xi, axis=1)
    cross = smooth[:, 1:] * np.conj(smooth[:, :-1])
    phi = np.angle(cross)
    amp = np.abs(cross)
    mean_amp = amp.mean(axis=1)
    strength = np.minimum(np.sqrt(mean_amp / np.median(mean_amp)), 3.0)
    coherence = np.abs(cross.sum(axis=1)) / amp.sum(axis=1)
    w = amp / (mean_amp[:, None] + 1e-12) * strength[:, None] * np.clip(coherence[:, None], 0, 1) ** 2
    w = np.minimum(w, 4.0)
    los = points[:, None, :] - pos[None, 1:, :]
    rng = np.linalg.norm(los, axis=2)
    ex_, ey_ = los[:, :, 0] / rng, los[:, :, 1] / rng
    target = phi / k
    for _ in range(3):
        sxx, sxy, syy = (w * ex_ * ex_).sum(0), (w * ex_ * ey_).sum(0), (w * ey_ * ey_).sum(0)
        bx, by = (w * ex_ * target).sum(0), (w * ey_ * target).sum(0)
        lam = 0.002 * (sxx + syy)
        det = np.maximum((sxx + lam) * (syy + lam) - sxy * sxy, 1e-12)
        dx = (bx * (syy + lam) - by * sxy) / det
        dy = (by * (sxx + lam) - bx * sxy) / det
        res = target - ex_ * dx - ey_ * dy
        sigma = 1.4826 * np.median(np.abs(res), axis=0) + 1e-6
        w = w * np.minimum(1.0, 2.5 * sigma[None, :] / (np.abs(res) + 1e-12))
    delta = np.zeros((len(pos), 3))
    delta[1:, 0] = np.cumsum(dx)
    delta[1:, 1] = np.cumsum(dy)
    delta[:, :2] = signal.detrend(delta[:, :2], axis=0, type="linear")
    delta[:, :2] = signal.savgol_filter(delta[:, :2], min(501, len(pos) // 2 * 2 - 1), 3, axis=0)
    peak = float(np.linalg.norm(delta[:, :2], axis=1).max())
    if peak > 1.0:
        delta /= peak
    return delta, dict(targets=len(points), cutoff_hz=cutoff, median_gradient_coherence=float(np.median(coherence)))


def phase_gradient_autofocus(data, pos, r_start, data_dr, fc, extent, prf, cutoffs=(12, 8, 5, 3, 2, 1), side=1,
                             leaf_size=64, range_spacing=0.5, angular_oversample=2.0, weight=None):
    """The iteration loop of autofocus.main (autofocus.py:88-110) on the CPU oracle."""
    k = 4 * np.pi * fc / ora.LIGHT_SPEED
    pos = np.array(pos, np.float64)
    best, best_pos, records = -np.inf, pos.copy(), []
    t0 = time.perf_counter()
    for it, cutoff in enumerate(cutoffs):
        img, _ = ora.form_ffbp(data, pos, r_start, data_dr, fc, extent, side=side, leaf_size=leaf_size,
                               range_spacing=range_spacing, angular_oversample=angular_oversample, weight=weight)
        power = np.abs(img.image) ** 2
        contrast = float(np.mean(power ** 2) / np.mean(power) ** 2)
        if contrast > best:
            best, best_pos = contrast, pos.copy()
        pts, _ = pick_targets(img.image, img.r, img.u, img.origin, img.side)
        delta, stats = estimate_update(data, pos, pts, r_start, data_dr, k, prf, cutoff)
        stats.update(iteration=it, input_contrast=contrast, elapsed_s=time.perf_counter() - t0)
        records.append(stats)
        pos = pos + delta
    return best_pos, records
