"""Differentiable split-precision lattice back-projection.

``backproject_lattice`` forms the image with the split-precision lattice kernel
(``sarbp_backproject_lattice``) and, on backward, runs the adjoint kernel
(``sarbp_backproject_lattice_adjoint``): per pulse it recomputes every pixel's
contribution w_n v_pn exp(i (k d_pn + phase_n)) and returns the gradients of a
real loss with respect to the antenna positions, the per-pulse phases and the
per-pulse weights.  The range-compressed data is not differentiable here.

The reference has no differentiable imaging operator: its autofocus
(fast_bp/autofocus.py:37-79) estimates per-pulse phase errors from target
contributions.  This operator lets an image-quality loss (entropy, sharpness)
be minimised by gradient descent over position and phase errors.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as nat
from . import core


def adjoint(data, pos, weight, phase, lattice: nat.Lattice, range_start, data_dr, k, grad_image,
            want=(True, True, True)):
    """Per-pulse gradients (pos [P,3], phase [P], weight [P], float64) of a real loss whose
    gradient with respect to the lattice image is ``grad_image`` (complex64, dl/dRe + i dl/dIm)."""
    p, s = core.check_pulses(data, pos, weight, phase)
    rows, cols = int(lattice.rows), int(lattice.cols)
    core._require(grad_image, "grad_image", torch.complex64, (rows, cols))
    dev = data.device
    g_pos = torch.empty((p, 3), dtype=torch.float64, device=dev) if want[0] else None
    g_phase = torch.empty((p,), dtype=torch.float64, device=dev) if want[1] else None
    g_weight = torch.empty((p,), dtype=torch.float64, device=dev) if want[2] else None
    lib = nat.load()
    nbytes = int(lib.sarbp_backproject_lattice_adjoint_workspace(ctypes.byref(lattice), p))
    ws = torch.empty((max(nbytes, 1),), dtype=torch.uint8, device=dev)
    nat.check(lib.sarbp_backproject_lattice_adjoint(
        core._ptr(data), p, s, core._ptr(pos), core._ptr(weight), core._ptr(phase), ctypes.byref(lattice),
        float(range_start), float(data_dr), float(k), core._ptr(grad_image), core._ptr(g_pos), core._ptr(g_phase),
        core._ptr(g_weight), core._ptr(ws), nbytes, core.stream_handle()), "backproject_lattice_adjoint")
    return g_pos, g_phase, g_weight


class _LatticeBP(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, phase, weight, data, lattice, range_start, data_dr, k):
        pos_c, phase_c, weight_c = pos.detach().contiguous(), phase.detach().contiguous(), weight.detach().contiguous()
        img = core.backproject_lattice(data, pos_c, weight_c, phase_c, lattice.origin, lattice.step_row,
                                       lattice.step_col, lattice.rows, lattice.cols, range_start, data_dr, k,
                                       mode="split", pulse_split=0)  # 0: the split that fills the GPU
        ctx.save_for_backward(pos_c, phase_c, weight_c, data)
        ctx.geometry = (lattice, range_start, data_dr, k)
        return img

    @staticmethod
    def backward(ctx, grad_image):
        pos, phase, weight, data = ctx.saved_tensors
        lattice, range_start, data_dr, k = ctx.geometry
        want = ctx.needs_input_grad[:3]
        if not any(want):
            return (None,) * 8
        g_pos, g_phase, g_weight = adjoint(data, pos, weight, phase, lattice, range_start, data_dr, k,
                                           grad_image.contiguous(), want=want)
        return g_pos, g_phase, g_weight, None, None, None, None, None


def backproject_lattice(data, pos, weight, phase, origin, step_row, step_col, rows, cols, range_start, data_dr, k):
    """Split-precision direct BP on origin + i*step_row + j*step_col -> complex64 [rows, cols],
    differentiable with respect to ``pos``, ``phase`` and ``weight`` (float64 CUDA tensors)."""
    lattice = nat.lattice(origin, step_row, step_col, rows, cols)
    return _LatticeBP.apply(pos, phase, weight, data, lattice, float(range_start), float(data_dr), float(k))
