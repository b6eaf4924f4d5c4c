"""Deterministic inputs of the autofocus golden cases (shared by make_golden.py and the tests).

``recovery``  the reference's own autofocus known-answer scene
              (fast_bp/validate_autofocus.py:8-18): 4096 pulses on a straight
              18 m high track, 4 point targets, a detrended sinusoidal
              cross-/along-track error; corrected RMSE must fall below 0.35x
              the initial one (validate_autofocus.py:20).
``cluttered`` 1024 pulses, 12 seeded targets of unequal strength, an error in
              all three axes and complex noise: exercises the robust weights.
``picks``     a seeded polar image with bright points for pick_targets.

The data is rebuilt from these recipes at test time (only the outputs of the
reference are stored), so the fixtures stay small.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
from scipy import signal

C = 299792458.0
FC = 1.4e9
FS = 400e6


def _echoes(track, targets, amplitudes, r0, nbins, k, width):
    dr = C / (2 * FS)
    rr = r0 + dr * np.arange(nbins)
    data = np.zeros((len(track), nbins), np.complex64)
    for xyz, a in zip(targets, amplitudes):
        d = np.linalg.norm(track - xyz, axis=1)
        data += (a * np.exp(-1j * k * d)[:, None] * np.sinc((rr[None, :] - d[:, None]) / width)).astype(np.complex64)
    return data


def recovery():
    n = 4096
    t = np.linspace(0, 4, n)
    truth = np.column_stack([np.zeros(n), np.linspace(-70, 70, n), np.full(n, 18.0)])
    targets = np.array([[710.0, -290.0, 0.0], [720.0, 320.0, 0.0], [810.0, -100.0, 0.0], [870.0, 280.0, 0.0]])
    k = -4 * np.pi * FC / C
    err = np.column_stack([0.06 * np.sin(2 * np.pi * t), 0.12 * np.cos(np.pi * t), np.zeros(n)])
    err[:, :2] = signal.detrend(err[:, :2], axis=0)
    r0 = 650.0
    data = _echoes(truth, targets, np.ones(len(targets)), r0, 900, k, C / 400e6)
    return SimpleNamespace(data=data, pos=truth + err, err=err, points=targets, r_start=r0, dr=C / (2 * FS), k=k,
                           prf=1024.0, cutoff=15.0)


def cluttered():
    n = 1024
    rng = np.random.default_rng(4242)
    t = np.linspace(0, 1, n)
    truth = np.column_stack([0.02 * t, np.linspace(-40, 40, n), np.full(n, 25.0)])
    targets = np.column_stack([rng.uniform(600, 900, 12), rng.uniform(-200, 200, 12), np.zeros(12)])
    amplitudes = rng.uniform(0.2, 3.0, 12) * np.exp(2j * np.pi * rng.uniform(size=12))
    k = 4 * np.pi * FC / C
    err = np.column_stack([0.03 * np.sin(5 * t) + 0.01 * t * t, 0.05 * np.cos(3 * t), 0.02 * np.sin(7 * t)])
    r0 = 560.0
    data = _echoes(truth, targets, amplitudes, r0, 1400, k, C / 300e6)
    noise = 0.05 * (rng.standard_normal(data.shape) + 1j * rng.standard_normal(data.shape))
    data = (data + noise).astype(np.complex64)
    return SimpleNamespace(data=data, pos=truth + err, err=err, points=targets, r_start=r0, dr=C / (2 * FS), k=k,
                           prf=800.0, cutoff=8.0)


def picks():
    """A polar image 250 x 190 with 40 bright cells over weak noise, and its axes."""
    rng = np.random.default_rng(99)
    img = (0.01 * (rng.standard_normal((250, 190)) + 1j * rng.standard_normal((250, 190)))).astype(np.complex64)
    rows = rng.integers(0, 250, 40)
    cols = rng.integers(0, 190, 40)
    img[rows, cols] += (rng.uniform(0.5, 5.0, 40) * np.exp(1j * rng.uniform(0, 6.28, 40))).astype(np.complex64)
    # an all-dark corner: its cells fall below the 35 dB power floor
    img[200:, 150:] *= 1e-3
    return SimpleNamespace(image=img, origin=np.array([1.5, -3.0, 40.0]), r0=600.0, dr=0.5, u0=-0.3, du=0.003,
                           side=-1)
