"""FP64 FFBP planner restated for the oracle (test infrastructure only).

Follows the reference's planner step for step: ``fast_bp/gpu_backend.py:121-224``
(``build_ffbp_plan``) and the identical inline planning of
``fast_bp/ffbp.py:124-177`` (``form_ffbp``).  The numpy operations are kept in
the reference's order (mean, ptp, norm, linspace, ceil) because the plan
integers (grid sizes and crop) must match the reference bit for bit.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

LIGHT_SPEED = 299792458.0


@dataclass
class OracleNode:
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
    left: int = -1
    right: int = -1


@dataclass
class OraclePlan:
    nodes: list
    crop_r: tuple
    crop_u: tuple
    counts: dict = field(default_factory=dict)

    @property
    def root(self):
        return self.nodes[0]

    def tables(self):
        """Flatten to the (geom float64 [N,8], idx int64 [N,6]) arrays oracle.cpp walks."""
        geom = np.zeros((len(self.nodes), 8), dtype=np.float64)
        idx = np.zeros((len(self.nodes), 6), dtype=np.int64)
        for i, n in enumerate(self.nodes):
            geom[i] = (*n.origin, n.r0, n.dr, n.u0, n.du, n.side)
            idx[i] = (n.a, n.b, n.nr, n.nu, n.left, n.right)
        return geom, idx


def plan_ffbp(position, fc, extent, side=1, leaf_size=128, range_spacing=0.25, angular_oversample=2.5):
    """Node tree in pre-order (parent before children), crop of the root grid, counts.

    Boundary sampling of the sector: ffbp.py:133-138.  Per-node geometry:
    ffbp.py:142-152.  Binary split at (a+b)//2 with leaves of at most
    ``leaf_size`` pulses: ffbp.py:153-169.  Crop: ffbp.py:174-177.
    """
    position = np.ascontiguousarray(position, dtype=np.float64)
    wavelength = LIGHT_SPEED / abs(float(fc))
    centre = position.mean(axis=0)
    rmin, rmax, umin, umax = (float(v) for v in extent)
    us = np.linspace(umin, umax, 129)
    rs = np.linspace(rmin, rmax, 129)
    rb = np.r_[np.full_like(us, rmin), np.full_like(us, rmax), rs, rs]
    ub = np.r_[us, us, np.full_like(rs, umin), np.full_like(rs, umax)]
    ground = np.sqrt(rb**2 - centre[2] ** 2)
    bx = centre[0] + side * ground * np.sqrt(1.0 - ub**2)
    by = centre[1] + ground * ub
    nodes = []
    counts = {"leaves": 0, "merges": 0, "leaf_pixel_pulse_products": 0, "merged_pixels": 0}

    def visit(a, b):
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
        me = len(nodes)
        nodes.append(OracleNode(a, b, np.ascontiguousarray(origin), r0, float(range_spacing), nr,
                                u0, float(du), nu, int(side)))
        if b - a <= leaf_size:
            counts["leaves"] += 1
            counts["leaf_pixel_pulse_products"] += nr * nu * (b - a)
        else:
            mid = (a + b) // 2
            nodes[me].left = visit(a, mid)
            nodes[me].right = visit(mid, b)
            counts["merges"] += 1
            counts["merged_pixels"] += 2 * nr * nu
        return me

    visit(0, len(position))
    root = nodes[0]
    r = root.r0 + root.dr * np.arange(root.nr)
    u = root.u0 + root.du * np.arange(root.nu)
    ri = np.flatnonzero((r >= rmin) & (r <= rmax))
    ui = np.flatnonzero((u >= umin) & (u <= umax))
    if len(ri) == 0 or len(ui) == 0:
        raise ValueError("Requested extent does not intersect the planned root grid")
    return OraclePlan(nodes, (int(ri[0]), int(ri[-1]) + 1), (int(ui[0]), int(ui[-1]) + 1), counts)
