"""Tensor-level API over libsarbp (device tensors in, device tensors out).

Every function enqueues CUDA kernels of libsarbp on the current torch stream
and returns without synchronising.  Inputs are torch CUDA tensors:

* ``data``   complex64 [pulses, samples], C-contiguous (range-compressed pulses)
* ``pos``    float64 [pulses, 3] antenna positions (x cross-track, y along-track, z)
* ``weight`` float64 [pulses], ``phase`` float64 [pulses]

Modes: ``"fp64"``, ``"fp32"``, ``"mixed"`` follow the reference's precision
policies (fast_bp/gpu/kernels.cu:1-6); ``"split"`` is the fast split-precision
path.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as nat

DEFAULT_MODE = "split"


def stream_handle(stream: torch.cuda.Stream | None = None) -> ctypes.c_void_p:
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _require(t, name, dtype, shape=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch CUDA tensor")
    if not t.is_cuda:
        raise TypeError(f"{name} must live on a CUDA device")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise TypeError(f"{name} must be C-contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}, got {tuple(t.shape)}")
    return t


def check_pulses(data, pos, weight, phase):
    _require(data, "data", torch.complex64)
    if data.dim() != 2:
        raise TypeError("range-compressed data must be C-contiguous complex64 [pulse, range]")
    p = data.shape[0]
    _require(pos, "position", torch.float64, (p, 3))
    _require(weight, "weight", torch.float64, (p,))
    _require(phase, "phase", torch.float64, (p,))
    return p, data.shape[1]


@dataclass
class Grid:
    """Polar grid (fast_bp/gpu_backend.py:60-78 NodePlan geometry)."""
    origin: tuple
    r0: float
    dr: float
    nr: int
    u0: float
    du: float
    nu: int
    side: int = 1

    def native(self) -> nat.PolarGrid:
        return nat.polar_grid(self.origin, self.r0, self.dr, self.nr, self.u0, self.du, self.nu, self.side)


def _workspace(nbytes: int, device) -> torch.Tensor | None:
    if nbytes <= 0:
        return None
    return torch.empty(int(nbytes), dtype=torch.uint8, device=device)


def direct_polar(data, pos, weight, phase, grid: Grid, range_start, data_dr, k, mode=DEFAULT_MODE,
                 chunk_pulses=64, pulse_split=1, out=None):
    """Direct BP of every pulse onto a polar grid -> complex64 [nr, nu] (ffbp.bp_polar semantics)."""
    p, s = check_pulses(data, pos, weight, phase)
    g = grid.native()
    if out is None:
        out = torch.empty((grid.nr, grid.nu), dtype=torch.complex64, device=data.device)
    _require(out, "out", torch.complex64, (grid.nr, grid.nu))
    m = nat.mode_id(mode)
    lib = nat.load()
    ws = _workspace(lib.sarbp_direct_polar_workspace(m, ctypes.byref(g), p, int(pulse_split)), data.device)
    nat.check(lib.sarbp_direct_polar(_ptr(data), p, s, _ptr(pos), _ptr(weight), _ptr(phase), ctypes.byref(g),
                                     float(range_start), float(data_dr), float(k), m, int(chunk_pulses),
                                     int(pulse_split), _ptr(out), _ptr(ws), 0 if ws is None else ws.numel(),
                                     stream_handle()), "direct_polar")
    return out


def backproject_points(data, pos, weight, phase, xyz, range_start, data_dr, k, mode=DEFAULT_MODE, pulse_split=1,
                       out=None):
    """Direct BP at points xyz float64 [M, 3] -> complex64 [M] (ffbp.backproject_points semantics)."""
    p, s = check_pulses(data, pos, weight, phase)
    _require(xyz, "xyz", torch.float64)
    if xyz.dim() != 2 or xyz.shape[1] != 3:
        raise ValueError("xyz must be [M, 3]")
    n = xyz.shape[0]
    if out is None:
        out = torch.empty((n,), dtype=torch.complex64, device=data.device)
    _require(out, "out", torch.complex64, (n,))
    m = nat.mode_id(mode)
    lib = nat.load()
    ws = _workspace(lib.sarbp_backproject_points_workspace(m, n, int(pulse_split)), data.device)
    nat.check(lib.sarbp_backproject_points(_ptr(data), p, s, _ptr(pos), _ptr(weight), _ptr(phase), _ptr(xyz), n,
                                           float(range_start), float(data_dr), float(k), m, int(pulse_split),
                                           _ptr(out), _ptr(ws), 0 if ws is None else ws.numel(), stream_handle()),
              "backproject_points")
    return out


def lattice_pulse_split(origin, step_row, step_col, rows, cols, mode=DEFAULT_MODE):
    """The pulse split backproject_lattice(pulse_split=0) uses for this lattice on the current GPU."""
    lat = nat.lattice(origin, step_row, step_col, rows, cols)
    nbytes = nat.load().sarbp_backproject_lattice_workspace(nat.mode_id(mode), ctypes.byref(lat), 0)
    return max(1, int(nbytes) // (int(rows) * int(cols) * 8))


def backproject_lattice(data, pos, weight, phase, origin, step_row, step_col, rows, cols, range_start, data_dr, k,
                        mode=DEFAULT_MODE, pulse_split=0, out=None):
    """Direct BP on the lattice origin + i*step_row + j*step_col -> complex64 [rows, cols].

    pulse_split > 1 splits each tile's pulses over that many CTAs (partial images summed in
    fixed order); 0 (the default) lets the library pick the split that fills the GPU for this
    lattice, which also shortens each FP32 partial sum."""
    p, s = check_pulses(data, pos, weight, phase)
    lat = nat.lattice(origin, step_row, step_col, rows, cols)
    if out is None:
        out = torch.empty((int(rows), int(cols)), dtype=torch.complex64, device=data.device)
    _require(out, "out", torch.complex64, (int(rows), int(cols)))
    m = nat.mode_id(mode)
    lib = nat.load()
    ws = _workspace(lib.sarbp_backproject_lattice_workspace(m, ctypes.byref(lat), int(pulse_split)), data.device)
    nat.check(lib.sarbp_backproject_lattice(_ptr(data), p, s, _ptr(pos), _ptr(weight), _ptr(phase),
                                            ctypes.byref(lat), float(range_start), float(data_dr), float(k), m,
                                            int(pulse_split), _ptr(out), _ptr(ws), 0 if ws is None else ws.numel(),
                                            stream_handle()), "backproject_lattice")
    return out


def regrid(image, src: Grid, dst: Grid, k, mode="mixed", out=None):
    """Child polar image -> parent grid (ffbp.regrid / regrid_* kernels) -> complex64 [dst.nr, dst.nu]."""
    _require(image, "image", torch.complex64, (src.nr, src.nu))
    if out is None:
        out = torch.empty((dst.nr, dst.nu), dtype=torch.complex64, device=image.device)
    _require(out, "out", torch.complex64, (dst.nr, dst.nu))
    gs, gd = src.native(), dst.native()
    nat.call("sarbp_regrid", _ptr(image), ctypes.byref(gs), ctypes.byref(gd), float(k), nat.mode_id(mode), _ptr(out),
             stream_handle())
    return out


def merge_regrid(left, left_grid: Grid, right, right_grid: Grid, dst: Grid, k, mode="mixed", out=None):
    """Both child regrids rounded to complex64 then added (merge_regrid_* kernels)."""
    _require(left, "left", torch.complex64, (left_grid.nr, left_grid.nu))
    _require(right, "right", torch.complex64, (right_grid.nr, right_grid.nu))
    if out is None:
        out = torch.empty((dst.nr, dst.nu), dtype=torch.complex64, device=left.device)
    _require(out, "out", torch.complex64, (dst.nr, dst.nu))
    gl, gr, gd = left_grid.native(), right_grid.native(), dst.native()
    nat.call("sarbp_merge_regrid", _ptr(left), ctypes.byref(gl), _ptr(right), ctypes.byref(gr), ctypes.byref(gd),
             float(k), nat.mode_id(mode), _ptr(out), stream_handle())
    return out


def evaluate_image(image, grid: Grid, xyz, k, out=None):
    """Polar image -> ground points (ffbp.evaluate_image) -> complex64 [M]."""
    _require(image, "image", torch.complex64, (grid.nr, grid.nu))
    _require(xyz, "xyz", torch.float64)
    n = xyz.shape[0]
    if out is None:
        out = torch.empty((n,), dtype=torch.complex64, device=image.device)
    g = grid.native()
    nat.call("sarbp_evaluate_image", _ptr(image), ctypes.byref(g), _ptr(xyz), n, float(k), _ptr(out),
             stream_handle())
    return out


def evaluate_lattice(image, grid: Grid, origin, step_row, step_col, rows, cols, k, out=None):
    """Polar image -> ground lattice origin + i*step_row + j*step_col (z ignored), split precision."""
    _require(image, "image", torch.complex64, (grid.nr, grid.nu))
    lat = nat.lattice(origin, step_row, step_col, rows, cols)
    if out is None:
        out = torch.empty((int(rows), int(cols)), dtype=torch.complex64, device=image.device)
    _require(out, "out", torch.complex64, (int(rows), int(cols)))
    nat.check(nat.load().sarbp_evaluate_lattice(_ptr(image), ctypes.byref(grid.native()), ctypes.byref(lat),
                                                float(k), _ptr(out), stream_handle()), "evaluate_lattice")
    return out


def target_contributions(data, pos, xyz, range_start, data_dr, k, out=None):
    """Per target, per pulse sample1 * exp(jkr) (ffbp.target_contributions) -> complex64 [M, P]."""
    _require(data, "data", torch.complex64)
    p, s = data.shape
    _require(pos, "position", torch.float64, (p, 3))
    _require(xyz, "xyz", torch.float64)
    n = xyz.shape[0]
    if out is None:
        out = torch.empty((n, p), dtype=torch.complex64, device=data.device)
    nat.call("sarbp_target_contributions", _ptr(data), p, s, _ptr(pos), _ptr(xyz), n, float(range_start),
             float(data_dr), float(k), _ptr(out), stream_handle())
    return out


def fill_range_phase_lut(samples, range_start, data_dr, k, device="cuda"):
    lut = torch.empty((int(samples),), dtype=torch.complex64, device=device)
    nat.call("sarbp_fill_range_phase_lut", int(samples), float(range_start), float(data_dr), float(k), _ptr(lut),
             stream_handle())
    return lut


def direct_polar_lut(data, pos, weight, phase, grid: Grid, range_start, data_dr, k, lut, out=None):
    """Mixed-geometry direct BP with the range-bin phase LUT (gpu/precision_probe.cu:118-164)."""
    p, s = check_pulses(data, pos, weight, phase)
    if out is None:
        out = torch.empty((grid.nr, grid.nu), dtype=torch.complex64, device=data.device)
    g = grid.native()
    nat.call("sarbp_direct_polar_lut", _ptr(data), p, s, _ptr(pos), _ptr(weight), _ptr(phase), ctypes.byref(g),
             float(range_start), float(data_dr), float(k), _ptr(lut), _ptr(out), stream_handle())
    return out


def direct_polar_phase32(data, pos, weight, phase, grid: Grid, range_start, data_dr, k, wrapped=False, out=None):
    """Mixed-geometry direct BP with the phase cast to FP32 for sincosf (gpu/precision_probe.cu:19-79);
    ``wrapped`` reduces the FP64 phase with remainder(phase, 2 pi) first."""
    p, s = check_pulses(data, pos, weight, phase)
    if out is None:
        out = torch.empty((grid.nr, grid.nu), dtype=torch.complex64, device=data.device)
    g = grid.native()
    nat.call("sarbp_direct_polar_phase32", _ptr(data), p, s, _ptr(pos), _ptr(weight), _ptr(phase), ctypes.byref(g),
             float(range_start), float(data_dr), float(k), int(bool(wrapped)), _ptr(out), stream_handle())
    return out


def fp32_peak_tflops(packed: bool = False, iters: int = 16384) -> float:
    """Measured FP32 issue rate of the current GPU in TFLOP/s (FMA = 2): eight independent FMA
    chains per thread at full occupancy, scalar or packed f32x2 (sarbp_fp32_peak)."""
    out = ctypes.c_double()
    nat.call("sarbp_fp32_peak", int(bool(packed)), int(iters), ctypes.byref(out))
    return float(out.value)


def add_inplace(left, right):
    nat.call("sarbp_add_inplace", _ptr(left), _ptr(right), left.numel(), stream_handle())
    return left


def crop(image, r_begin, u_begin, nr, nu, out=None):
    if out is None:
        out = torch.empty((nr, nu), dtype=torch.complex64, device=image.device)
    nat.call("sarbp_crop", _ptr(image), image.shape[1], int(r_begin), int(u_begin), int(nr), int(nu), _ptr(out),
             stream_handle())
    return out


def cast_c128_to_c64(t, out=None):
    if out is None:
        out = torch.empty(t.shape, dtype=torch.complex64, device=t.device)
    nat.call("sarbp_cast_c128_to_c64", _ptr(t), _ptr(out), t.numel(), stream_handle())
    return out


def node_array(nodes):
    """Pre-order NodePlan-like objects -> ctypes sarbp_ffbp_node array (children as indices)."""
    arr = (nat.FFBPNode * len(nodes))()
    index = {id(n): i for i, n in enumerate(nodes)}
    for i, n in enumerate(nodes):
        e = arr[i]
        e.origin[:] = [float(v) for v in n.origin]
        e.r0, e.dr, e.u0, e.du = float(n.r0), float(n.dr), float(n.u0), float(n.du)
        e.nr, e.nu, e.side = int(n.nr), int(n.nu), int(n.side)
        e.a, e.b = int(n.a), int(n.b)
        left = getattr(n, "left", None)
        right = getattr(n, "right", None)
        e.left = -1 if left is None else (left if isinstance(left, int) else index[id(left)])
        e.right = -1 if right is None else (right if isinstance(right, int) else index[id(right)])
    return arr


class FFBPProgram:
    """Level-batched FFBP over a node tree (one launch for the leaves, one per height; in split mode
    ``merge_queue=True`` runs the merges as one dependency-counting queue launch instead).

    ``nodes`` is a pre-order sequence of objects with the NodePlan fields
    (origin, r0, dr, nr, u0, du, nu, side, a, b, left/right children).  The
    root's crop window is fused into the last merge, which writes the output
    directly.  The workspace (node images + device tables) is allocated once.
    In split mode the merge tiles stage their children's footprints in shared memory by TMA
    (``staging=False``: they gather from the child images; the image is the same).
    """

    def __init__(self, nodes, crop_r, crop_u, mode=DEFAULT_MODE, device="cuda", merge_queue=False, staging=True):
        self.mode = mode
        arr = node_array(nodes)
        self.crop = (int(crop_r[0]), int(crop_u[0]), int(crop_r[1] - crop_r[0]), int(crop_u[1] - crop_u[0]))
        handle = ctypes.c_void_p()
        lib = nat.load()
        nat.check(lib.sarbp_ffbp_plan_create(arr, len(nodes), *self.crop, nat.mode_id(mode), ctypes.byref(handle)),
                  "ffbp_plan_create")
        self._handle = handle
        if merge_queue:
            # all merge levels as one dependency-counting launch instead of one launch per tree height
            nat.check(lib.sarbp_ffbp_set_merge_queue(handle, 1), "ffbp_set_merge_queue")
        if not staging:
            nat.check(lib.sarbp_ffbp_set_staging(handle, 0), "ffbp_set_staging")
        self.workspace_bytes = int(lib.sarbp_ffbp_workspace_bytes(handle))
        self.launch_count = int(lib.sarbp_ffbp_launch_count(handle))
        self.workspace = torch.empty(max(self.workspace_bytes, 256), dtype=torch.uint8, device=device)
        nat.check(lib.sarbp_ffbp_bind(handle, _ptr(self.workspace), self.workspace.numel(), stream_handle()),
                  "ffbp_bind")
        self.shape = (self.crop[2], self.crop[3])
        staged = ctypes.c_int(0)
        nat.check(lib.sarbp_ffbp_staging(handle, ctypes.byref(staged)), "ffbp_staging")
        self.staged = bool(staged.value)

    def execute(self, data, pos, weight, phase, range_start, data_dr, k, out=None):
        p, s = check_pulses(data, pos, weight, phase)
        if out is None:
            out = torch.empty(self.shape, dtype=torch.complex64, device=data.device)
        _require(out, "out", torch.complex64, self.shape)
        nat.check(nat.load().sarbp_ffbp_execute(self._handle, _ptr(data), p, s, _ptr(pos), _ptr(weight), _ptr(phase),
                                                float(range_start), float(data_dr), float(k), _ptr(out),
                                                stream_handle()), "ffbp_execute")
        return out

    def set_node_image(self, node: int, image):
        """Supply the image (complex64 [nr, nu]) of external node ``node`` (a leaf whose pulse range is
        [-1, -1)); the copy is enqueued on the current stream, so ``image`` must stay alive until the
        stream has run it (the next execute on the same stream is ordered after it)."""
        _require(image, "image", torch.complex64)
        nat.check(nat.load().sarbp_ffbp_set_node_image(self._handle, int(node), _ptr(image), stream_handle()),
                  "ffbp_set_node_image")

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            nat.load().sarbp_ffbp_plan_destroy(self._handle)
            self._handle = None
        self.workspace = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def to_device(array, dtype, device="cuda") -> torch.Tensor:
    """numpy -> contiguous CUDA tensor (tensors already on a CUDA device pass through)."""
    if isinstance(array, torch.Tensor):
        t = array.to(device=device, dtype=dtype)
        return t.contiguous()
    a = np.ascontiguousarray(array)
    return torch.from_numpy(a).to(device=device, dtype=dtype).contiguous()
