"""Autofocus on the GPU.

Two estimators of per-pulse navigation errors, both device-resident:

* ``estimate_update`` / ``pick_targets`` / ``phase_gradient_autofocus``: the
  reference's phase-gradient trajectory refinement (fast_bp/autofocus.py:19-111).
  Target contributions come from the ``sarbp_target_contributions`` kernel,
  the Butterworth smoothing of each target's pulse history from the
  ``sarbp_sosfiltfilt`` kernel, and the robust weighted least squares, the
  detrend and the Savitzky-Golay smoothing run as FP64 torch operations on
  the device.  scipy designs the filters (coefficients only).
* ``entropy_autofocus``: minimises the image entropy of a split-precision
  lattice image over per-pulse phase and position corrections, with the
  gradient from the adjoint kernel (``bp_project_gb300.autograd``) and L-BFGS.
  It has no counterpart in the reference.
"""
from __future__ import annotations

import ctypes
import functools
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch
from scipy import signal

from . import _native as nat
from . import core
from . import ffbp as ffbp_mod
from .autograd import backproject_lattice

LIGHT_SPEED = 299792458.0


# ---- Butterworth smoothing along pulses ------------------------------------------------

@dataclass(frozen=True)
class SmoothingFilter:
    """Second-order sections, their steady-state initial conditions and the odd-extension length."""
    sos: np.ndarray
    zi: np.ndarray
    padlen: int


@functools.lru_cache(maxsize=64)
def butter_lowpass(cutoff, fs, order=4) -> SmoothingFilter:
    """butter(order, cutoff, fs=fs, output='sos') with sosfiltfilt's default padding (autofocus.py:38).
    Cached per (cutoff, fs, order): the autofocus loop asks for the same few filters every pass."""
    sos = np.ascontiguousarray(signal.butter(order, cutoff, fs=fs, output="sos"), np.float64)
    zi = np.ascontiguousarray(signal.sosfilt_zi(sos), np.float64)
    ntaps = 2 * len(sos) + 1
    ntaps -= min(int((sos[:, 2] == 0).sum()), int((sos[:, 5] == 0).sum()))
    return SmoothingFilter(sos, zi, 3 * ntaps)


def sosfiltfilt(x: torch.Tensor, filt: SmoothingFilter) -> torch.Tensor:
    """Zero-phase filtering of each row of complex64 ``x`` [rows, n] -> complex128 [rows, n]."""
    core._require(x, "x", torch.complex64)
    if x.dim() != 2:
        raise ValueError("x must be [rows, n]")
    rows, n = x.shape
    dev = x.device
    sos = torch.from_numpy(filt.sos).to(dev)
    zi = torch.from_numpy(filt.zi).to(dev)
    y = torch.empty((rows, n), dtype=torch.complex128, device=dev)
    lib = nat.load()
    nbytes = int(lib.sarbp_sosfiltfilt_workspace(rows, n, filt.padlen))
    ws = torch.empty((max(nbytes, 1),), dtype=torch.uint8, device=dev)
    nat.check(lib.sarbp_sosfiltfilt(core._ptr(x), rows, n, core._ptr(sos), core._ptr(zi), len(filt.sos),
                                    filt.sos.ctypes.data_as(ctypes.c_void_p), filt.padlen, core._ptr(y),
                                    core._ptr(ws), nbytes, core.stream_handle()), "sosfiltfilt")
    return y


# ---- FP64 helpers on the device --------------------------------------------------------

def _median(x: torch.Tensor, dim=None) -> torch.Tensor:
    """numpy.median semantics: the middle value, or for even counts the mean of the two middle
    values formed as (a + b) / 2, the way numpy averages them.  One sort along ``dim``."""
    if dim is None:
        x, dim = x.reshape(-1), 0
    s = torch.sort(x, dim=dim).values
    n = s.shape[dim]
    upper = s.narrow(dim, n // 2, 1)
    if n % 2:
        return upper.squeeze(dim)
    return ((s.narrow(dim, n // 2 - 1, 1) + upper) / 2).squeeze(dim)


def detrend_linear(x: torch.Tensor) -> torch.Tensor:
    """Remove the least-squares line along dim 0 of [n, c] (scipy.signal.detrend type='linear')."""
    n = x.shape[0]
    t = torch.arange(n, dtype=x.dtype, device=x.device)
    t = t - t.mean()
    xc = x - x.mean(dim=0, keepdim=True)
    slope = (t[:, None] * xc).sum(dim=0, keepdim=True) / (t * t).sum()
    return xc - t[:, None] * slope


def _projection(window: int, polyorder: int) -> np.ndarray:
    """Least-squares polynomial smoothing matrix H (window x window): H @ y = fitted values."""
    s = (np.arange(window, dtype=np.float64) - (window - 1) / 2) / ((window - 1) / 2)
    v = np.vander(s, polyorder + 1, increasing=True)
    q, _ = np.linalg.qr(v)
    return q @ q.T


_SAVGOL_CACHE: dict = {}


def savgol_smooth(x: torch.Tensor, window: int, polyorder: int) -> torch.Tensor:
    """Savitzky-Golay smoothing along dim 0 of [n, c] with polynomial fits at the edges
    (scipy.signal.savgol_filter, deriv 0, mode 'interp')."""
    n = x.shape[0]
    if window % 2 != 1 or window > n or polyorder >= window:
        raise ValueError("window must be odd, <= the signal length and > polyorder")
    key = (window, polyorder, x.device)
    if key not in _SAVGOL_CACHE:
        h = _projection(window, polyorder)
        half = window // 2
        _SAVGOL_CACHE[key] = tuple(torch.from_numpy(np.ascontiguousarray(m)).to(x.device)
                                   for m in (h[half], h[:half], h[window - half:]))
    centre, left, right = _SAVGOL_CACHE[key]
    half = window // 2
    out = torch.empty_like(x)
    out[half:n - half] = torch.einsum("icw,w->ic", x.unfold(0, window, 1), centre)
    out[:half] = left @ x[:window]
    out[n - half:] = right @ x[n - window:]
    return out


# ---- phase-gradient autofocus (fast_bp/autofocus.py) -----------------------------------

def pick_targets(result, nr_tiles=12, nu_tiles=12):
    """Brightest cell of each of nr_tiles x nu_tiles image tiles (autofocus.py:19-34), one block per
    tile on the GPU (``sarbp_tile_argmax``).

    ``result`` is a ``PolarImage`` whose image is a CUDA tensor.  Returns
    (points float64 [T, 3], powers float64 [T]) on the image's device, cells
    35 dB or more below the brightest one dropped."""
    image = result.image
    if not isinstance(image, torch.Tensor):
        raise TypeError("pick_targets expects the image on the device (form_ffbp with device inputs)")
    nr, nu = image.shape
    if nr < nr_tiles or nu < nu_tiles:
        raise ValueError("the image has fewer rows or columns than tiles")
    dev = image.device
    a = image.abs().contiguous()  # float32 [nr, nu], numpy's complex64 magnitude
    ntiles = nr_tiles * nu_tiles
    tmax = torch.empty(ntiles, dtype=torch.float32, device=dev)
    first = torch.empty(ntiles, dtype=torch.int64, device=dev)
    nat.check(nat.load().sarbp_tile_argmax(core._ptr(a), nr, nu, nr_tiles, nu_tiles, core._ptr(tmax), core._ptr(first),
                                           core.stream_handle()), "tile_argmax")
    ir, iu = first // nu, first % nu
    r = result.r0 + result.dr * ir.double()
    u = result.u0 + result.du * iu.double()
    o = torch.as_tensor(np.asarray(result.origin, np.float64), device=dev)
    g = torch.sqrt(r * r - o[2] ** 2)
    pts = torch.stack([o[0] + result.side * g * torch.sqrt(1 - u * u), o[1] + g * u, torch.zeros_like(r)], dim=1)
    powers = tmax.double() ** 2
    good = powers > powers.max() * 10 ** (-35 / 10)
    return pts[good], powers[good]


def estimate_update(data, pos, points, r_start, dr, k, prf, cutoff):
    """Trajectory update from smoothed per-target phase gradients (autofocus.py:37-79).

    data complex64 [P, B], pos float64 [P, 3], points float64 [T, 3] (CUDA
    tensors or arrays).  Returns (delta float64 [P, 3] on the device, stats)."""
    d = core.to_device(data, torch.complex64)
    dev = d.device
    p = core.to_device(pos, torch.float64, dev)
    pts = core.to_device(points, torch.float64, dev)
    n = p.shape[0]
    xi = core.target_contributions(d, p, pts, r_start, dr, k)
    smooth = sosfiltfilt(xi, butter_lowpass(cutoff, prf))
    cross = smooth[:, 1:] * smooth[:, :-1].conj()
    gradient = torch.angle(cross)
    amp = cross.abs()
    target_power = amp.mean(dim=1)
    strength = torch.sqrt(target_power / _median(target_power)).clamp(max=3.0)
    coherence = cross.sum(dim=1).abs() / amp.sum(dim=1)
    w = (amp / (target_power[:, None] + 1e-12)) * strength[:, None]
    w = w * coherence.clamp(0, 1)[:, None] ** 2
    w = w.clamp(max=4.0)
    vec = pts[:, None, :] - p[None, 1:, :]
    dist = torch.linalg.norm(vec, dim=2)
    ux, uy = vec[:, :, 0] / dist, vec[:, :, 1] / dist
    rhs = gradient / k
    for _ in range(3):
        a = (w * ux * ux).sum(0)
        b = (w * ux * uy).sum(0)
        dd = (w * uy * uy).sum(0)
        ex = (w * ux * rhs).sum(0)
        ey = (w * uy * rhs).sum(0)
        reg = 0.002 * (a + dd)
        det = (a + reg) * (dd + reg) - b * b
        dx = (ex * (dd + reg) - ey * b) / det.clamp(min=1e-12)
        dy = (ey * (a + reg) - ex * b) / det.clamp(min=1e-12)
        residual = rhs - ux * dx - uy * dy
        scale = 1.4826 * _median(residual.abs(), dim=0) + 1e-6
        w = w * torch.clamp(2.5 * scale[None, :] / (residual.abs() + 1e-12), max=1.0)
    zero = torch.zeros(1, dtype=torch.float64, device=dev)
    delta = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    xy = torch.stack([torch.cat([zero, torch.cumsum(dx, 0)]), torch.cat([zero, torch.cumsum(dy, 0)])], dim=1)
    xy = detrend_linear(xy)
    xy = savgol_smooth(xy, min(501, n // 2 * 2 - 1), 3)
    delta[:, :2] = xy
    maxnorm = float(torch.linalg.norm(delta[:, :2], dim=1).max())
    if maxnorm > 1.0:
        delta = delta / maxnorm
    rms = torch.sqrt((delta ** 2).mean(dim=0)).tolist()
    stats = dict(targets=int(pts.shape[0]), cutoff_hz=cutoff, median_gradient_coherence=float(_median(coherence)),
                 delta_rms_m=rms, delta_max_m=delta.abs().max(dim=0).values.tolist())
    return delta, stats


def intensity_contrast(image: torch.Tensor) -> float:
    """mean(power^2) / mean(power)^2 of a complex image (autofocus.py:94)."""
    power = image.abs().double() ** 2
    return float((power ** 2).mean() / power.mean() ** 2)


def phase_gradient_autofocus(data, pos, r_start, data_dr, fc, extent, prf, cutoffs=(12, 8, 5, 3, 2, 1),
                             side=1, leaf_size=64, range_spacing=0.5, angular_oversample=2.0, weight=None,
                             nr_tiles=12, nu_tiles=12, mode=core.DEFAULT_MODE, callback=None):
    """The reference's autofocus loop (autofocus.py:82-111) on the GPU: per cutoff, FFBP,
    contrast, target picking and a trajectory update; keeps the position of highest contrast.

    Returns (best position float64 [P, 3] on the device, per-iteration records)."""
    d = core.to_device(data, torch.complex64)
    p = core.to_device(pos, torch.float64, d.device).clone()
    k = 4 * np.pi * fc / LIGHT_SPEED
    best, best_pos, records = -np.inf, p.clone(), []
    t0 = time.perf_counter()
    for iteration, cutoff in enumerate(cutoffs):
        result, _ = ffbp_mod.form_ffbp(d, p, r_start, data_dr, fc, extent, side=side, leaf_size=leaf_size,
                                       range_spacing=range_spacing, angular_oversample=angular_oversample,
                                       weight=weight, verbose=False, mode=mode)
        contrast = intensity_contrast(result.image)
        if contrast > best:
            best, best_pos = contrast, p.clone()
        points, _ = pick_targets(result, nr_tiles, nu_tiles)
        delta, stats = estimate_update(d, p, points, r_start, data_dr, k, prf, cutoff)
        stats.update(iteration=iteration, input_contrast=contrast, elapsed_s=time.perf_counter() - t0)
        records.append(stats)
        if callback is not None:
            callback(iteration, p, result, stats)
        p = p + delta
    return best_pos, records


# ---- gradient entropy autofocus --------------------------------------------------------

def image_entropy(image: torch.Tensor) -> torch.Tensor:
    """Shannon entropy (nats) of the normalised intensity of a complex image
    (sar_quality/metrics.py:6-22 focus_metrics['entropy_nats']); differentiable."""
    power = torch.view_as_real(image).double().pow(2).sum(-1).reshape(-1)
    prob = power / power.sum()
    return -(prob * torch.log(prob.clamp(min=1e-300))).sum()


@dataclass
class EntropyResult:
    phase: torch.Tensor          # float64 [P] corrected per-pulse phase
    position: torch.Tensor       # float64 [P, 3] corrected positions
    entropy: float
    history: list = field(default_factory=list)   # (elapsed s, entropy) per evaluation
    evaluations: int = 0


def entropy_autofocus(data, pos, weight, phase, origin, step_row, step_col, rows, cols, range_start, data_dr, k,
                      steps=40, estimate_position=True, target_entropy=None, history_size=20, time_limit=None):
    """Minimise the entropy of the lattice image over per-pulse phase and (optionally)
    position corrections with L-BFGS; gradients come from the adjoint BP kernel.

    Position corrections are scaled by 1/|k| so that a unit step in either
    parameter moves the pulse's phase by about one radian.  Stops after
    ``steps`` L-BFGS iterations, once the entropy is at or below
    ``target_entropy``, or after ``time_limit`` seconds."""
    d = core.to_device(data, torch.complex64)
    dev = d.device
    p0 = core.to_device(pos, torch.float64, dev)
    w = core.to_device(weight, torch.float64, dev)
    ph0 = core.to_device(phase, torch.float64, dev)
    n = p0.shape[0]
    theta = torch.zeros(n, dtype=torch.float64, device=dev, requires_grad=True)
    params = [theta]
    if estimate_position:
        xi = torch.zeros((n, 3), dtype=torch.float64, device=dev, requires_grad=True)
        params.append(xi)
    scale = 1.0 / abs(float(k))
    geo = (origin, step_row, step_col, rows, cols, range_start, data_dr, k)
    opt = torch.optim.LBFGS(params, lr=1.0, max_iter=steps, history_size=history_size,
                            tolerance_grad=1e-12, tolerance_change=1e-14, line_search_fn="strong_wolfe")
    history = []
    t0 = time.perf_counter()
    best = [math.inf, None]

    class _Done(Exception):
        pass

    def closure():
        opt.zero_grad()
        pos_c = p0 + scale * params[1] if estimate_position else p0
        img = backproject_lattice(d, pos_c, w, ph0 + theta, *geo)
        loss = image_entropy(img)
        loss.backward()
        value = float(loss.detach())
        history.append((time.perf_counter() - t0, value))
        if value < best[0]:
            best[0] = value
            best[1] = [t.detach().clone() for t in params]
        if target_entropy is not None and value <= target_entropy:
            raise _Done
        if time_limit is not None and history[-1][0] > time_limit:
            raise _Done
        return loss

    try:
        opt.step(closure)
    except _Done:
        pass
    final = best[1] if best[1] is not None else [t.detach() for t in params]
    position = p0 + scale * final[1] if estimate_position else p0.clone()
    return EntropyResult(ph0 + final[0], position, best[0], history, len(history))
