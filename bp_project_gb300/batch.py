"""Many scenes in one schedule: persistent work-queue kernels over uneven scenes.

``SceneBatch`` binds a list of scenes (direct BP onto a flat lattice, or FFBP
of a planned tree) to ``sarbp_batch_*``: all scenes' direct tiles run in one
persistent launch that drains a largest-first work queue, all FFBP leaf tiles in
a second one, and the FFBP merges as one persistent launch per tree height
across all scenes.
``execute`` only enqueues work on the current stream (no allocation, no
synchronisation), so the whole batch can be captured in one CUDA graph
(``capture_graph`` / ``replay``), like ``ResidentProgram``.  With
``concurrent=True`` the FFBP chain runs on a stream of the batch's own, forked
from and joined back to the current stream, beside the direct queue: the
latency-bound merges and the issue-bound direct tiles then share the SMs.

The reference images one scene at a time; its ``BatchedResidentProgram``
(fast_bp/batched_resident_backend.py:23-157) batches the levels of one tree.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import torch

from . import _native as nat
from . import core


@dataclass
class DirectScene:
    """Split-precision direct BP of one scene onto origin + i*step_row + j*step_col (z steps 0)."""
    data: torch.Tensor        # complex64 [P, B]
    pos: torch.Tensor         # float64 [P, 3]
    weight: torch.Tensor      # float64 [P]
    phase: torch.Tensor       # float64 [P]
    range_start: float
    data_dr: float
    k: float
    origin: tuple
    step_row: tuple
    step_col: tuple
    rows: int
    cols: int
    tile_lc: int = 0          # log2 of tile columns (2..5); 0 = 5 (32 x 32 tiles)
    chunk_pulses: int = 0     # 0 = default
    out: torch.Tensor | None = None


@dataclass
class FFBPScene:
    """Split-precision FFBP of one scene over a plan from ``gpu_backend.build_ffbp_plan``."""
    data: torch.Tensor
    pos: torch.Tensor
    weight: torch.Tensor
    phase: torch.Tensor
    range_start: float
    data_dr: float
    k: float
    plan: object
    chunk_pulses: int = 0
    out: torch.Tensor | None = None
    _nodes: object = field(default=None, repr=False)


class SceneBatch:
    """A fixed set of scenes formed by one schedule (inputs and outputs bound at construction)."""

    def __init__(self, scenes, blocks_per_sm=0, device=None, concurrent=False):
        if not scenes:
            raise ValueError("a batch needs at least one scene")
        self.scenes = list(scenes)
        arr = (nat.BatchScene * len(self.scenes))()
        for i, sc in enumerate(self.scenes):
            p, s = core.check_pulses(sc.data, sc.pos, sc.weight, sc.phase)
            e = arr[i]
            e.data, e.pulses, e.samples = sc.data.data_ptr(), p, s
            e.pos, e.weight, e.phase = sc.pos.data_ptr(), sc.weight.data_ptr(), sc.phase.data_ptr()
            e.range_start, e.data_dr, e.k = float(sc.range_start), float(sc.data_dr), float(sc.k)
            e.chunk_pulses = int(sc.chunk_pulses)
            if isinstance(sc, DirectScene):
                shape = (int(sc.rows), int(sc.cols))
                e.kind = nat.BATCH_DIRECT
                e.lattice = nat.lattice(sc.origin, sc.step_row, sc.step_col, sc.rows, sc.cols)
                e.tile_lc = int(sc.tile_lc)
            elif isinstance(sc, FFBPScene):
                plan = sc.plan
                shape = tuple(plan.shape)
                e.kind = nat.BATCH_FFBP
                sc._nodes = core.node_array(plan.nodes())
                e.nodes = ctypes.cast(sc._nodes, ctypes.POINTER(nat.FFBPNode))
                e.n_nodes = len(sc._nodes)
                e.crop_r0, e.crop_u0 = int(plan.crop_r[0]), int(plan.crop_u[0])
                e.crop_nr, e.crop_nu = shape
            else:
                raise TypeError("scenes must be DirectScene or FFBPScene")
            if sc.out is None:
                sc.out = torch.empty(shape, dtype=torch.complex64, device=sc.data.device)
            core._require(sc.out, "out", torch.complex64, shape)
            e.out = sc.out.data_ptr()
        self._arr = arr
        lib = nat.load()
        handle = ctypes.c_void_p()
        nat.check(lib.sarbp_batch_create(arr, len(self.scenes), int(blocks_per_sm), ctypes.byref(handle)),
                  "batch_create")
        self._handle = handle
        dev = device or self.scenes[0].data.device
        self.workspace_bytes = int(lib.sarbp_batch_workspace_bytes(handle))
        self.workspace = torch.empty(max(self.workspace_bytes, 256), dtype=torch.uint8, device=dev)
        nat.check(lib.sarbp_batch_bind(handle, core._ptr(self.workspace), self.workspace.numel(),
                                       core.stream_handle()), "batch_bind")
        nat.check(lib.sarbp_batch_set_concurrent(handle, int(bool(concurrent))), "batch_set_concurrent")
        self.concurrent = bool(concurrent)
        self.launch_count = int(lib.sarbp_batch_launch_count(handle))
        vals = [ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()]
        nat.check(lib.sarbp_batch_info(handle, *[ctypes.byref(v) for v in vals]), "batch_info")
        self.info = dict(bp_items=vals[0].value, merge_items=vals[1].value, max_height=vals[2].value,
                         bp_blocks=vals[3].value, pixel_pulses=vals[4].value)
        self._graph = None

    @property
    def outputs(self):
        return [sc.out for sc in self.scenes]

    def execute(self):
        if self._handle is None:
            raise RuntimeError("batch is closed")
        nat.check(nat.load().sarbp_batch_execute(self._handle, core.stream_handle()), "batch_execute")

    def scene_latencies_ms(self):
        """Per-scene completion times (ms from the batch's start) of one traced execution: each
        work item raises its scene's slot to the GPU's nanosecond timer when it finishes."""
        if self._handle is None:
            raise RuntimeError("batch is closed")
        lib = nat.load()
        trace = torch.zeros(len(self.scenes) + 1, dtype=torch.int64, device=self.workspace.device)
        nat.check(lib.sarbp_batch_set_trace(self._handle, core._ptr(trace)), "batch_set_trace")
        try:
            self.execute()
            torch.cuda.synchronize(self.workspace.device)
        finally:
            nat.check(lib.sarbp_batch_set_trace(self._handle, None), "batch_set_trace")
        t = trace.cpu().numpy()
        return (t[:-1] - t[-1]) / 1e6

    def capture_graph(self):
        """Capture one execute into a CUDA graph (warm once first, so the capture sees no first-use work)."""
        self.execute()
        torch.cuda.current_stream().synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self.execute()
        self._graph = graph
        return graph

    def replay(self):
        if self._graph is None:
            raise RuntimeError("capture_graph must run before replay")
        self._graph.replay()

    def close(self):
        if getattr(self, "_handle", None) is not None and self._handle.value:
            nat.load().sarbp_batch_destroy(self._handle)
        self._handle = None
        self._graph = None
        self.workspace = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
