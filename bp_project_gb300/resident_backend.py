"""Preallocated, asynchronous BP programs (fast_bp/resident_backend.py surface).

All input arrays stay owned by the caller.  Construction allocates the output
and the FFBP workspace (node images and device tables) once.  ``execute`` and
``replay`` only enqueue kernels on the current torch stream: they do not
allocate, synchronise, record events or copy to the host.  Outputs are
overwritten by the next execution, and a program is not safe for concurrent
execution because its workspace is shared between invocations
(fast_bp/resident_backend.py:1-7, :24-32).

The reference's ``variant="original"`` (per-node regrid + add) and
``variant="fused"`` (both child regrids in one kernel) round each child image
to complex64 before the FP32 add; both map to libsarbp's level-batched
program, which keeps those rounding points.
"""
from __future__ import annotations

from collections import Counter

import torch

from . import core
from .gpu_backend import ALL_MODES, MODES


class ResidentProgram:
    """A reusable direct-BP or FFBP schedule with fixed inputs and grid."""

    def __init__(self, backend, plan, device, mode, range_start, data_dr, k, algorithm="ffbp", variant="original",
                 chunk_pulses=64):
        if mode not in ALL_MODES:
            raise ValueError(f"mode must be one of {MODES}")
        if algorithm not in ("direct", "ffbp"):
            raise ValueError("algorithm must be direct or ffbp")
        if variant not in ("original", "fused"):
            raise ValueError("variant must be original or fused")
        if algorithm == "direct" and variant != "original":
            raise ValueError("fused variant is only defined for FFBP")
        if chunk_pulses <= 0:
            raise ValueError("chunk_pulses must be positive")
        if plan.nr * plan.nu <= 0:
            raise ValueError("empty image grids are unsupported")
        self.backend = backend
        self.plan = plan
        self.device = device
        self.mode = mode
        self.algorithm = algorithm
        self.variant = variant
        self.range_start = float(range_start)
        self.data_dr = float(data_dr)
        self.k = float(k)
        self.chunk_pulses = int(chunk_pulses)
        self._graph = None
        self._graph_stream = None
        self._closed = False
        dev = device.data.device
        self.output = torch.empty(plan.shape, dtype=torch.complex64, device=dev)
        self._ffbp = None
        if algorithm == "ffbp":
            self._ffbp = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode=mode, device=dev)
            self.launch_count = self._ffbp.launch_count
            names = ["ffbp_leaves"] + [f"ffbp_merge_height_{h}" for h in range(1, self.launch_count)]
            workspace = self._ffbp.workspace_bytes
        else:
            self.launch_count = 1
            names = [f"direct_{mode}"]
            workspace = 0
        self.operations = [{"name": n, "count": int(plan.nr * plan.nu)} for n in names]
        counts = Counter(op["name"] for op in self.operations)
        out_bytes = self.output.numel() * self.output.element_size()
        self.metadata = {
            "algorithm": algorithm,
            "variant": variant,
            "mode": mode,
            "shape": [int(x) for x in plan.shape],
            "block_size": int(getattr(backend, "block_size", 256)),
            "chunk_pulses": self.chunk_pulses if algorithm == "direct" else None,
            "kernel_launch_count": self.launch_count,
            "kernel_counts": dict(counts),
            "memset_count": 0,
            "device_operation_count": self.launch_count,
            "workspace_bytes": int(workspace + out_bytes),
            "workspace_buffer_count": 2 if algorithm == "ffbp" else 1,
            "origin_table_bytes": 0,
            "total_owned_device_bytes": int(workspace + out_bytes),
            "workspace_policy": "one arena for all node images and device tables, allocated at construction",
            "input_data_shared": True,
            "output_dtype": "complex64",
            "zeroing_in_execute": False,
            "graph_supported": None,
            "graph_error": None,
            "arithmetic": "libsarbp sm_103a kernels; split = split precision, others = reference policies",
            "fusion": "level-batched; child regrids rounded to complex64 then FP32 add" if algorithm == "ffbp" else None,
            "merge_staging": ("TMA tensor copies of each child's footprint into shared memory"
                              if self._ffbp is not None and self._ffbp.staged else None),
        }

    def execute(self):
        """Enqueue one complete image computation on the current CUDA stream."""
        if self._closed:
            raise RuntimeError("program is closed")
        d = self.device
        if self._ffbp is not None:
            self._ffbp.execute(d.data, d.pos64, d.weight64, d.phase64, self.range_start, self.data_dr, self.k,
                               out=self.output)
        else:
            core.direct_polar(d.data, d.pos64, d.weight64, d.phase64, self.plan.grid(), self.range_start,
                              self.data_dr, self.k, mode=self.mode, chunk_pulses=self.chunk_pulses, out=self.output)
        return self.output

    def capture_graph(self, warmup=True):
        """Capture ``execute`` into a CUDA graph (may synchronise; record failures in metadata)."""
        if self._closed:
            raise RuntimeError("program is closed")
        if self._graph is not None:
            return True
        try:
            torch.cuda.current_stream().synchronize()
            stream = torch.cuda.Stream()
            with torch.cuda.stream(stream):
                if warmup:
                    self.execute()
                    stream.synchronize()
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph, stream=stream):
                    self.execute()
            stream.synchronize()
            self._graph = graph
            self._graph_stream = stream
            self.metadata["graph_supported"] = True
            self.metadata["graph_error"] = None
            return True
        except Exception as exc:  # recorded, as the reference does (resident_backend.py:282-292)
            self._graph = None
            self.metadata["graph_supported"] = False
            self.metadata["graph_error"] = f"{type(exc).__name__}: {exc}"
            return False

    def replay(self):
        """Enqueue the captured graph on the current stream, without a fence."""
        if self._closed:
            raise RuntimeError("program is closed")
        if self._graph is None:
            raise RuntimeError("capture_graph() must succeed before replay()")
        self._graph.replay()
        return self.output

    def close(self):
        """Drop owned device memory after the caller has synchronised its work."""
        self._graph = None
        self._graph_stream = None
        if self._ffbp is not None:
            self._ffbp.close()
        self._ffbp = None
        self.operations = []
        self.output = None
        self.device = None
        self._closed = True
