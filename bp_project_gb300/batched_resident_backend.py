"""Level-batched preallocated FFBP (fast_bp/batched_resident_backend.py surface).

libsarbp's FFBP program is level-batched already: one launch covers every
leaf and one launch covers each tree height, with the root crop fused into
the last merge.  Node images live in one arena addressed through a device
node table (fast_bp/batched_resident_backend.py:72-150 uses per-node
allocations and a pointer table instead).
"""
from __future__ import annotations

from .resident_backend import ResidentProgram


class BatchedResidentProgram(ResidentProgram):
    """ResidentProgram-compatible, fused FFBP batched across each tree level."""

    def __init__(self, backend, plan, device, mode, range_start, data_dr, k, chunk_pulses=64):
        super().__init__(backend, plan, device, mode, range_start, data_dr, k, algorithm="ffbp", variant="fused",
                         chunk_pulses=chunk_pulses)
        self.variant = "batched_fused"
        heights = self.launch_count - 1
        self.metadata.update({
            "variant": self.variant,
            "batch_stages": [{"height": h, "kernel": "ffbp_leaves" if h == 0 else "ffbp_merges"}
                             for h in range(heights + 1)],
            "extra_table_bytes": 0,
            "extra_table_count": 0,
            "batch_mapping": "one CTA per node pixel tile; nodes grouped by subtree height",
            "fusion": "leaf BP per tile; each merge tile regrids both children (footprints staged in shared memory "
                      "by TMA in split mode), each rounded to complex64, then an FP32 add",
        })
