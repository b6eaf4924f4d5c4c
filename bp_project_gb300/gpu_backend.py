"""Drop-in for the reference's CUDA baseline surface (fast_bp/gpu_backend.py).

Same names, arguments, return values and exception types as the reference:
``MODES``, ``NodePlan``, ``FFBPPlan``, ``DeviceInputs``, ``build_ffbp_plan``,
``CudaBaseline`` (``upload`` / ``run_direct`` / ``run_ffbp`` / ``download``)
and ``cuda_environment``.  Device arrays are torch CUDA tensors instead of
CuPy arrays; the kernels are libsarbp's sm_103a kernels (no NVRTC, no CuPy).

Besides the reference's three precision policies, every entry point accepts
``mode="split"``, the split-precision fast path.
"""
from __future__ import annotations

import platform
import time
from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np
import torch

from . import _native as nat
from . import core

MODES = ("fp64", "fp32", "mixed")
SPLIT = "split"
ALL_MODES = MODES + (SPLIT,)
LIGHT_SPEED = 299792458.0


@dataclass
class NodePlan:
    index: int
    a: int
    b: int
    origin: np.ndarray
    r0: float
    dr: float
    nr: int
    u0: float
    du: float
    nu: int
    side: int
    left: Optional["NodePlan"] = None
    right: Optional["NodePlan"] = None

    @property
    def is_leaf(self):
        return self.left is None

    def grid(self) -> core.Grid:
        return core.Grid(tuple(self.origin), self.r0, self.dr, self.nr, self.u0, self.du, self.nu, self.side)


@dataclass
class FFBPPlan:
    root: NodePlan
    origins: np.ndarray
    crop_r: tuple
    crop_u: tuple
    origin: np.ndarray
    r0: float
    dr: float
    nr: int
    u0: float
    du: float
    nu: int
    side: int
    counts: dict
    extent: tuple
    leaf_size: int
    angular_oversample: float

    @property
    def shape(self):
        return self.nr, self.nu

    def nodes(self):
        """Nodes in pre-order (index order)."""
        out = []

        def walk(n):
            out.append(n)
            if n.left is not None:
                walk(n.left)
                walk(n.right)

        walk(self.root)
        return out

    def grid(self) -> core.Grid:
        """The cropped output grid."""
        return core.Grid(tuple(self.origin), self.r0, self.dr, self.nr, self.u0, self.du, self.nu, self.side)


@dataclass
class DeviceInputs:
    data: torch.Tensor
    pos64: torch.Tensor
    pos32: torch.Tensor
    weight64: torch.Tensor
    weight32: torch.Tensor
    phase64: torch.Tensor
    phase32: torch.Tensor
    origins64: torch.Tensor
    origins32: torch.Tensor
    h2d_event_ms: float
    h2d_wall_ms: float
    bytes_uploaded: int


def build_ffbp_plan(position, fc, extent, side=1, leaf_size=128, range_spacing=0.25, angular_oversample=2.5):
    """Exact FP64 node tree and crop (fast_bp/gpu_backend.py:121-224, ffbp.py:133-177).

    The sector boundary is sampled with 129 points per edge; every node covers
    the sector about its own phase centre with 8-cell guards; leaves hold at
    most ``leaf_size`` pulses and nodes split at ``(a+b)//2``.  The numpy
    operations are the reference's, in its order, so the integer grid sizes
    and the crop match the reference bit for bit.
    """
    position = np.ascontiguousarray(position, dtype=np.float64)
    wavelength = LIGHT_SPEED / abs(float(fc))
    centre = position.mean(axis=0)
    rmin, rmax, umin, umax = (float(x) for x in extent)
    us = np.linspace(umin, umax, 129)
    rs = np.linspace(rmin, rmax, 129)
    rb = np.r_[np.full_like(us, rmin), np.full_like(us, rmax), rs, rs]
    ub = np.r_[us, us, np.full_like(rs, umin), np.full_like(rs, umax)]
    ground = np.sqrt(rb**2 - centre[2] ** 2)
    bx = centre[0] + side * ground * np.sqrt(1.0 - ub**2)
    by = centre[1] + ground * ub
    counts = {"leaves": 0, "merges": 0, "leaf_pixel_pulse_products": 0, "merged_pixels": 0}
    nodes = []

    def make(a, b):
        origin = position[a:b].mean(axis=0)
        dx = bx - origin[0]
        dy = by - origin[1]
        gr = np.sqrt(dx * dx + dy * dy)
        rr = np.sqrt(gr * gr + origin[2] ** 2)
        uu = dy / gr
        aperture = np.linalg.norm(np.ptp(position[a:b, :2], axis=0))
        du = min(0.025, wavelength / (2.0 * max(aperture, 0.1) * angular_oversample))
        u0 = max(-0.995, float(uu.min()) - 8.0 * du)
        u1 = min(0.995, float(uu.max()) + 8.0 * du)
        r0 = float(rr.min()) - 8.0 * range_spacing
        nr = int(np.ceil((rr.max() - r0) / range_spacing)) + 9
        nu = int(np.ceil((u1 - u0) / du)) + 1
        node = NodePlan(len(nodes), a, b, np.ascontiguousarray(origin, dtype=np.float64), r0, float(range_spacing),
                        nr, u0, float(du), nu, int(side))
        nodes.append(node)
        if b - a <= leaf_size:
            counts["leaves"] += 1
            counts["leaf_pixel_pulse_products"] += nr * nu * (b - a)
        else:
            mid = (a + b) // 2
            node.left = make(a, mid)
            node.right = make(mid, b)
            counts["merges"] += 1
            counts["merged_pixels"] += 2 * nr * nu
        return node

    root = make(0, len(position))
    root_r = root.r0 + root.dr * np.arange(root.nr)
    root_u = root.u0 + root.du * np.arange(root.nu)
    ri = np.flatnonzero((root_r >= rmin) & (root_r <= rmax))
    ui = np.flatnonzero((root_u >= umin) & (root_u <= umax))
    if len(ri) == 0 or len(ui) == 0:
        raise ValueError("Requested extent does not intersect the planned root grid")
    origins = np.ascontiguousarray(np.stack([n.origin for n in nodes]), dtype=np.float64)
    counts = dict(counts)
    counts.update(nodes=len(nodes), shape=[int(len(ri)), int(len(ui))],
                  direct_pixel_pulse_products=int(len(ri) * len(ui) * len(position)))
    return FFBPPlan(root=root, origins=origins, crop_r=(int(ri[0]), int(ri[-1]) + 1),
                    crop_u=(int(ui[0]), int(ui[-1]) + 1), origin=root.origin.copy(),
                    r0=float(root.r0 + ri[0] * root.dr), dr=float(root.dr), nr=int(len(ri)),
                    u0=float(root.u0 + ui[0] * root.du), du=float(root.du), nu=int(len(ui)), side=int(side),
                    counts=counts, extent=tuple(float(x) for x in extent), leaf_size=int(leaf_size),
                    angular_oversample=float(angular_oversample))


def _check_mode(mode):
    if mode not in ALL_MODES:
        raise ValueError(f"mode must be one of {MODES}")


class CudaBaseline:
    """Execute BP / FFBP with libsarbp (fast_bp/gpu_backend.py:227-561 surface)."""

    kernel_names = (
        "plain_polar_kernel<fp64|fp32|mixed>", "split_polar_kernel", "split_lattice_kernel", "split_points_kernel",
        "split_leaf_kernel", "split_merge_kernel", "plain_ffbp_leaf_kernel", "plain_ffbp_merge_kernel",
        "plain_regrid_kernel", "plain_merge_kernel", "evaluate_kernel", "target_contrib_kernel", "add_kernel",
        "cast_kernel", "crop_kernel", "sum_parts_kernel",
    )

    def __init__(self, block_size=128, device=None):
        if block_size <= 0:
            raise ValueError("block_size must be positive")
        if not torch.cuda.is_available():
            raise RuntimeError("CudaBaseline needs a CUDA device")
        self.block_size = int(block_size)  # kept for metadata; libsarbp chooses its own CTA shapes
        self.device = torch.device("cuda" if device is None else device)
        start = time.perf_counter()
        nat.load()
        torch.cuda.synchronize(self.device)
        self.compile_seconds = time.perf_counter() - start
        self.source_path = Path(nat.__file__).resolve().parent / "csrc"
        self.peak_pool_used_bytes = int(torch.cuda.memory_allocated(self.device))
        self._programs = {}

    def _track_memory(self):
        self.peak_pool_used_bytes = max(self.peak_pool_used_bytes, int(torch.cuda.max_memory_allocated(self.device)))

    def upload(self, data, position, weight, phase, plan):
        data = np.ascontiguousarray(data) if not data.flags.c_contiguous else data
        if data.dtype != np.complex64 or data.ndim != 2:
            raise TypeError("range-compressed data must be C-contiguous complex64 [pulse, range]")
        position64 = np.ascontiguousarray(position, dtype=np.float64)
        weight64 = np.ascontiguousarray(weight, dtype=np.float64)
        phase64 = np.ascontiguousarray(phase, dtype=np.float64)
        if position64.shape != (data.shape[0], 3):
            raise ValueError("position shape does not match the pulse count")
        if weight64.shape != (data.shape[0],) or phase64.shape != (data.shape[0],):
            raise ValueError("weight and phase must have one value per pulse")
        if not (np.isfinite(position64).all() and np.isfinite(weight64).all() and np.isfinite(phase64).all()):
            raise ValueError("position, weight and phase must be finite")
        host_start = time.perf_counter()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
        dev = self.device
        device = DeviceInputs(
            data=torch.from_numpy(data).to(dev),
            pos64=torch.from_numpy(position64).to(dev),
            pos32=torch.from_numpy(position64.astype(np.float32)).to(dev),
            weight64=torch.from_numpy(weight64).to(dev),
            weight32=torch.from_numpy(weight64.astype(np.float32)).to(dev),
            phase64=torch.from_numpy(phase64).to(dev),
            phase32=torch.from_numpy(phase64.astype(np.float32)).to(dev),
            origins64=torch.from_numpy(np.ascontiguousarray(plan.origins)).to(dev),
            origins32=torch.from_numpy(np.ascontiguousarray(plan.origins, dtype=np.float32)).to(dev),
            h2d_event_ms=0.0, h2d_wall_ms=0.0, bytes_uploaded=0)
        end.record()
        end.synchronize()
        device.h2d_event_ms = float(start.elapsed_time(end))
        device.h2d_wall_ms = 1000.0 * (time.perf_counter() - host_start)
        arrays = (device.data, device.pos64, device.pos32, device.weight64, device.weight32, device.phase64,
                  device.phase32, device.origins64, device.origins32)
        device.bytes_uploaded = int(sum(a.numel() * a.element_size() for a in arrays))
        self._track_memory()
        return device

    def _program(self, plan, mode):
        key = (id(plan), mode)
        prog = self._programs.get(key)
        if prog is None or prog[0] is not plan:
            prog = (plan, core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode=mode, device=self.device))
            self._programs[key] = prog
        return prog[1]

    def run_ffbp(self, plan, device, mode, range_start, data_dr, k):
        _check_mode(mode)
        wall_start = time.perf_counter()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        prog = self._program(plan, mode)
        start.record()
        out = prog.execute(device.data, device.pos64, device.weight64, device.phase64, range_start, data_dr, k)
        end.record()
        end.synchronize()
        self._track_memory()
        return out, float(start.elapsed_time(end)), 1000.0 * (time.perf_counter() - wall_start)

    def run_direct(self, plan, device, mode, range_start, data_dr, k, chunk_pulses=64):
        _check_mode(mode)
        if chunk_pulses <= 0:
            raise ValueError("chunk_pulses must be positive")
        wall_start = time.perf_counter()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
        out = core.direct_polar(device.data, device.pos64, device.weight64, device.phase64, plan.grid(), range_start,
                                data_dr, k, mode=mode, chunk_pulses=chunk_pulses)
        end.record()
        end.synchronize()
        self._track_memory()
        return out, float(start.elapsed_time(end)), 1000.0 * (time.perf_counter() - wall_start)

    @staticmethod
    def download(array):
        start = time.perf_counter()
        result = array.detach().cpu().numpy()
        return result, 1000.0 * (time.perf_counter() - start)


def cuda_environment():
    props = torch.cuda.get_device_properties(0)
    free, total = torch.cuda.mem_get_info(0)
    lib = nat.load()
    return {
        "gpu": props.name,
        "compute_capability": f"{props.major}.{props.minor}",
        "multiprocessors": int(props.multi_processor_count),
        "gpu_memory_bytes": int(total),
        "gpu_free_bytes_at_query": int(free),
        "cuda_runtime_version": torch.version.cuda,
        "torch_version": torch.__version__,
        "numpy_version": np.__version__,
        "python_version": platform.python_version(),
        "platform": platform.platform(),
        "kernel_backend": lib.sarbp_version().decode(),
        "fast_math": False,
    }
