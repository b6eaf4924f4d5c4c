"""Image-quality metrics with the reference's conventions (sar_quality/metrics.py:1-74).

``focus_metrics``   entropy and contrast of a complex image (:6-22);
``fidelity``        relative complex error, SER, coherence and phase statistics of
                    an estimate against a reference image (:25-39);
``impulse_metrics`` 1-D impulse response: half-power width (IRW), first-null
                    main lobe, peak and integrated sidelobe ratios (:42-74).

These run on host arrays of modest size (images are downloaded once, cuts are
1-D); numpy 2 has no ``trapz``, so the integrals use ``numpy.trapezoid``.
"""
from __future__ import annotations

import numpy as np
from scipy.signal import find_peaks


def _host(z):
    if hasattr(z, "detach"):
        z = z.detach().cpu().numpy()
    return np.asarray(z)


def focus_metrics(z) -> dict:
    z = _host(z)
    finite = np.isfinite(z)
    nonzero = np.abs(z) > 0
    out = dict(samples=int(z.size), finite_fraction=float(finite.mean()), nonzero_fraction=float(nonzero.mean()))
    if not finite.all() or not nonzero.any():
        return dict(out, valid=False, reason="Non-finite or zero-energy image")
    amp = np.abs(z).astype(np.float64).ravel()
    amp /= amp.max()
    power = amp * amp
    prob = power / power.sum()
    pos = prob[prob > 0]
    entropy = float(-(pos * np.log(pos)).sum())
    top = max(1, z.size // 100)
    return dict(out, valid=True, entropy_nats=entropy, normalized_entropy=entropy / np.log(z.size),
                intensity_contrast=float(power.std() / power.mean()),
                amplitude_contrast=float(amp.std() / amp.mean()),
                brightest_1pct_energy_fraction=float(np.sort(prob)[-top:].sum()))


def fidelity(reference, estimate) -> dict:
    ref = _host(reference).astype(np.complex128).ravel()
    est = _host(estimate).astype(np.complex128).ravel()
    norm = np.linalg.norm(ref)
    err = np.linalg.norm(est - ref) / norm
    strong = np.abs(ref) >= np.abs(ref).max() * 10 ** (-30 / 20)
    dphi = np.angle(est[strong] * ref[strong].conj())
    bias = np.angle(np.mean(np.exp(1j * dphi)))
    spread = np.angle(np.exp(1j * (dphi - bias)))
    return dict(relative_complex_error=float(err), ser_db=float(-20 * np.log10(max(err, 1e-300))),
                complex_coherence=float(abs(np.vdot(ref, est)) / (norm * np.linalg.norm(est))),
                phase_bias_deg=float(np.rad2deg(bias)), phase_std_deg_above_minus30db=float(np.rad2deg(spread.std())),
                phase_mask_samples=int(strong.sum()))


def impulse_metrics(x, z) -> dict:
    """1-D impulse response metrics of the cut z(x).

    IRW: width between the linear half-power crossings either side of the peak.
    Main lobe: between the nearest local power minima outside those crossings.
    PSLR = 10 log10(max sidelobe power / peak power); ISLR = 10 log10(sidelobe
    energy / main-lobe energy), energies by trapezoidal integration over x."""
    x = np.asarray(x, np.float64)
    p = np.abs(_host(z)) ** 2
    if not np.isfinite(p).all() or p.max() <= 0:
        return dict(valid=False, reason="Invalid power")
    peak = int(np.argmax(p))
    p = p / p[peak]
    below_left = np.flatnonzero(p[:peak] <= 0.5)
    below_right = np.flatnonzero(p[peak + 1:] <= 0.5) + peak + 1
    if not len(below_left) or not len(below_right):
        return dict(valid=False, reason="Half-power crossing absent")
    il, ir = int(below_left[-1]), int(below_right[0])
    xl = np.interp(0.5, p[il:il + 2], x[il:il + 2])
    xr = np.interp(0.5, p[ir - 1:ir + 1][::-1], x[ir - 1:ir + 1][::-1])
    minima = find_peaks(-p)[0]
    left_min, right_min = minima[minima < il], minima[minima > ir]
    if not len(left_min) or not len(right_min):
        return dict(valid=True, irw_m=float(xr - xl), peak_offset_m=float(x[peak]), sidelobes_valid=False,
                    reason="First minima absent")
    ml, mr = int(left_min[-1]), int(right_min[0])
    main = np.trapezoid(p[ml:mr + 1], x[ml:mr + 1])
    side = np.trapezoid(p[:ml + 1], x[:ml + 1]) + np.trapezoid(p[mr:], x[mr:])
    return dict(valid=True, sidelobes_valid=True, irw_m=float(xr - xl), peak_offset_m=float(x[peak]),
                pslr_db=float(10 * np.log10(max(p[:ml].max(), p[mr + 1:].max()))),
                islr_db=float(10 * np.log10(side / main)),
                mainlobe_bounds_m=[float(x[ml]), float(x[mr])],
                mainlobe_minima_db=[float(10 * np.log10(p[ml] + 1e-300)), float(10 * np.log10(p[mr] + 1e-300))],
                integration_bounds_m=[float(x[0]), float(x[-1])], step_m=float(x[1] - x[0]))
