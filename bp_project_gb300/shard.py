"""BP over several GPUs, one process per GPU: direct BP by pixel bands or pulse ranges, FFBP by subtrees.

Direct back-projection shards two ways without changing a single bit of the
image that one GPU forms:

* **Row bands** (``by="rows"``).  Every rank reads all pulses (the inputs are
  broadcast, or each rank loads them itself) and images a band of lattice rows.
  Bands start on multiples of the lattice tile height (32 rows: lattice tiles
  are 32 x 32 pixels), so every tile of a band is a tile of the whole lattice
  and runs exactly the arithmetic it runs on one GPU, provided the band's
  origin ``origin + b * step_row`` is exact in FP64 (true for the power-of-two
  pixel spacings of the benchmark scenes; otherwise the band's pixel positions
  may differ from the whole lattice's by one FP64 rounding, and the images by
  FP32 rounding).  The bands are then gathered; there is no other exchange.
* **Pulse ranges** (``by="pulses"``).  Rank r images pulses
  ``[P r / W, P (r + 1) / W)`` of the whole lattice (it needs only those pulses'
  data) into a partial image.  The partial images are summed on one rank in
  rank order, ``((part_0 + part_1) + part_2) + ...`` in FP32, which is the
  order the library's pulse-split sum uses on one GPU
  (``sum_parts_kernel``); the result equals the one-GPU image with
  ``pulse_split = W`` bit for bit.  This generalises the reference's running
  accumulator over pulse chunks (fast_bp/gpu/kernels.cu:240-271,
  fast_bp/gpu_backend.py:535-541) from chunks in one launch to ranks.

Collectives go through ``torch.distributed`` (NCCL between GPUs; the host
logic is tested with gloo ranks on the CPU).  Complex tensors travel as their
real views.  Nothing here uses cluster multicast or reads another GPU's memory
directly: remote bands and partial images arrive as local copies.
"""
from __future__ import annotations

import torch

from . import core

LATTICE_TILE_ROWS = 32  # rows of a split-precision lattice tile (1024 pixels, 32 columns)


def row_bands(rows: int, parts: int, align: int = LATTICE_TILE_ROWS) -> list[tuple[int, int]]:
    """``parts`` contiguous [begin, end) row bands covering ``[0, rows)`` exactly, every begin a
    multiple of ``align``; bands differ by at most one ``align`` block (trailing bands may be empty
    when there are fewer blocks than parts)."""
    if rows < 0 or parts < 1 or align < 1:
        raise ValueError("rows must be >= 0, parts and align >= 1")
    blocks = -(-rows // align)
    out = []
    for part in range(parts):
        b = min(rows, (blocks * part // parts) * align)
        e = min(rows, (blocks * (part + 1) // parts) * align)
        out.append((b, e))
    return out


def pulse_ranges(pulses: int, parts: int) -> list[tuple[int, int]]:
    """The library's pulse split: part s holds pulses ``[P s / S, P (s + 1) / S)`` (integer division)."""
    if pulses < 0 or parts < 1:
        raise ValueError("pulses must be >= 0 and parts >= 1")
    return [(pulses * s // parts, pulses * (s + 1) // parts) for s in range(parts)]


def band_origin(origin, step_row, row_begin: int):
    """Origin of the sub-lattice that starts at row ``row_begin`` (FP64, as the library forms pixels)."""
    return tuple(float(o) + row_begin * float(s) for o, s in zip(origin, step_row))


def _dist():
    import torch.distributed as dist
    return dist


def gather_rows(band: torch.Tensor, bands, rank: int, world: int, group=None) -> torch.Tensor:
    """All-gather row bands into the whole image on every rank.  ``band`` is this rank's
    complex64 [e - b, cols] band of ``bands``; bands are padded to the longest for the collective."""
    dist = _dist()
    cols = band.shape[1]
    rows = bands[-1][1] if bands else 0
    longest = max(e - b for b, e in bands)
    if band.shape[0] != bands[rank][1] - bands[rank][0]:
        raise ValueError(f"rank {rank} band has {band.shape[0]} rows, expected {bands[rank][1] - bands[rank][0]}")
    send = torch.zeros((longest, cols, 2), dtype=torch.float32, device=band.device)
    send[: band.shape[0]] = torch.view_as_real(band)
    recv = [torch.empty_like(send) for _ in range(world)]
    dist.all_gather(recv, send, group=group)
    out = torch.empty((rows, cols), dtype=torch.complex64, device=band.device)
    for r, (b, e) in enumerate(bands):
        if e > b:
            out[b:e] = torch.view_as_complex(recv[r][: e - b].contiguous())
    return out


def reduce_in_rank_order(partial: torch.Tensor, rank: int, world: int, dst: int = 0, group=None, add=None):
    """Sum every rank's partial image on rank ``dst`` as ((p_0 + p_1) + p_2) + ... (FP32, elementwise),
    the order of the library's pulse-split sum.  Returns the sum on ``dst`` and None elsewhere.

    ``add(acc, x)`` adds in place; for CUDA tensors it defaults to the library's sarbp_add_inplace.
    Partials are gathered, not reduced by the collective, because a collective's summation order is
    not specified."""
    dist = _dist()
    if add is None:
        if not partial.is_cuda:
            raise ValueError("partial images on the host need an explicit add")
        add = core.add_inplace
    flat = torch.view_as_real(partial.contiguous())
    if rank == dst:
        recv = [torch.empty_like(flat) for _ in range(world)]
        dist.gather(flat, gather_list=recv, dst=dst, group=group)
        acc = torch.view_as_complex(recv[0]).clone()
        for r in range(1, world):
            add(acc, torch.view_as_complex(recv[r]))
        return acc
    dist.gather(flat, gather_list=None, dst=dst, group=group)
    return None


def lattice_band(data, pos, weight, phase, origin, step_row, step_col, rows, cols, range_start, data_dr, k, *,
                 rank: int, world: int, pulse_split: int = 1):
    """This rank's row band of the lattice image (all pulses): complex64 [e - b, cols] for
    ``row_bands(rows, world)[rank] = (b, e)``."""
    b, e = row_bands(int(rows), world)[rank]
    band = torch.zeros((e - b, int(cols)), dtype=torch.complex64, device=data.device)
    if e > b:
        core.backproject_lattice(data, pos, weight, phase, band_origin(origin, step_row, b), step_row, step_col,
                                 e - b, cols, range_start, data_dr, k, mode="split", pulse_split=pulse_split,
                                 out=band)
    return band


def lattice_pulse_part(data, pos, weight, phase, origin, step_row, step_col, rows, cols, range_start, data_dr, k, *,
                       rank: int, world: int):
    """This rank's partial lattice image over its pulses ``pulse_ranges(P, world)[rank]``."""
    b, e = pulse_ranges(int(data.shape[0]), world)[rank]
    if e <= b:
        raise ValueError(f"rank {rank} has no pulses ({data.shape[0]} pulses over {world} ranks)")
    return core.backproject_lattice(data[b:e], pos[b:e], weight[b:e], phase[b:e], origin, step_row, step_col, rows,
                                    cols, range_start, data_dr, k, mode="split", pulse_split=1)


def direct_lattice(data, pos, weight, phase, origin, step_row, step_col, rows, cols, range_start, data_dr, k, *,
                   rank: int, world: int, by: str = "rows", pulse_split: int = 1, group=None, dst: int = 0):
    """Split-precision direct BP of one lattice over ``world`` ranks (see the module docstring).

    ``by="rows"``: ``data``/``pos``/``weight``/``phase`` hold all pulses; returns the whole image on
    every rank (``pulse_split`` applies within each band).  ``by="pulses"``: they hold all pulses
    too, and this rank images its own range of them; returns the image on ``dst`` (None elsewhere),
    equal to the one-GPU image with ``pulse_split = world``."""
    geo = (origin, step_row, step_col, rows, cols, range_start, data_dr, k)
    if by == "rows":
        band = lattice_band(data, pos, weight, phase, *geo, rank=rank, world=world, pulse_split=pulse_split)
        return gather_rows(band, row_bands(int(rows), world), rank, world, group)
    if by == "pulses":
        if pulse_split != 1:
            raise ValueError("pulse sharding splits the pulses across ranks; pulse_split must be 1")
        part = lattice_pulse_part(data, pos, weight, phase, *geo, rank=rank, world=world)
        return reduce_in_rank_order(part, rank, world, dst=dst, group=group)
    raise ValueError(f"by must be 'rows' or 'pulses' (got {by!r})")


def polar_pulse_part(data, pos, weight, phase, grid, range_start, data_dr, k, *, rank: int, world: int):
    """This rank's partial polar image over its pulses ``pulse_ranges(P, world)[rank]``."""
    b, e = pulse_ranges(int(data.shape[0]), world)[rank]
    if e <= b:
        raise ValueError(f"rank {rank} has no pulses ({data.shape[0]} pulses over {world} ranks)")
    return core.direct_polar(data[b:e], pos[b:e], weight[b:e], phase[b:e], grid, range_start, data_dr, k,
                             mode="split", pulse_split=1)


def direct_polar_pulses(data, pos, weight, phase, grid, range_start, data_dr, k, *, rank: int, world: int,
                        group=None, dst: int = 0):
    """Split-precision direct BP onto a polar grid (the CudaBaseline.run_direct surface) with the
    pulses sharded over ranks; returns on ``dst`` the one-GPU image of ``pulse_split = world``."""
    part = polar_pulse_part(data, pos, weight, phase, grid, range_start, data_dr, k, rank=rank, world=world)
    return reduce_in_rank_order(part, rank, world, dst=dst, group=group)


# ---- FFBP: subtrees per rank, the top levels on one rank -------------------------------------
#
# FFBP's tree is independent below depth d: with 2^d >= world subtrees rooted at depth d, every
# rank forms its subtrees as ordinary plans (their roots' full images), sends the roots to one rank,
# and that rank forms the top of the tree as a plan whose leaves are the subtree roots, marked
# external (pulse range [-1, -1)) and supplied with sarbp_ffbp_set_node_image.  The top merges run
# the same kernels on the same tiles as the one-GPU plan, so the image is the same bit for bit.
# Each rank only needs the pulses of its subtrees.


class TreeNode:
    """The NodePlan fields a plan needs (children as objects), for re-rooted and re-leafed trees."""

    __slots__ = ("origin", "r0", "dr", "nr", "u0", "du", "nu", "side", "a", "b", "left", "right")

    def __init__(self, n, a=None, b=None, left=None, right=None):
        self.origin = tuple(float(v) for v in n.origin)
        self.r0, self.dr, self.u0, self.du = float(n.r0), float(n.dr), float(n.u0), float(n.du)
        self.nr, self.nu, self.side = int(n.nr), int(n.nu), int(n.side)
        self.a = int(n.a) if a is None else a
        self.b = int(n.b) if b is None else b
        self.left, self.right = left, right


def _children(n):
    left, right = getattr(n, "left", None), getattr(n, "right", None)
    return [] if left is None else [left, right]


def ffbp_cut(root, parts: int):
    """Cut the tree under ``root`` (a NodePlan-like object, children as objects) for ``parts`` ranks.

    Returns (subtrees, top, external): ``subtrees`` lists the pre-order node lists of the 2^d subtrees
    rooted at depth d = ceil(log2 parts) (a leaf shallower than d is its own subtree), in pre-order;
    ``top`` is the pre-order node list of the tree above them with each subtree root as an external
    leaf; ``external[s]`` is subtree s's root index in ``top``."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    depth = max(0, (parts - 1).bit_length())
    subtrees, top, external = [], [], []

    def preorder(n, out):
        out.append(n)
        for c in _children(n):
            preorder(c, out)

    def copy_tree(n):
        kids = _children(n)
        return TreeNode(n, left=copy_tree(kids[0]) if kids else None, right=copy_tree(kids[1]) if kids else None)

    def walk(n, d):
        if d == depth or not _children(n):
            nodes = []
            preorder(copy_tree(n), nodes)
            subtrees.append(nodes)
            ext = TreeNode(n, a=-1, b=-1)
            external.append(ext)
            return ext
        t = TreeNode(n)
        kids = _children(n)
        t.left, t.right = walk(kids[0], d + 1), walk(kids[1], d + 1)
        return t

    top_root = walk(root, 0)
    preorder(top_root, top)
    index = {id(n): i for i, n in enumerate(top)}
    return subtrees, top, [index[id(e)] for e in external]


def subtree_ranges(n_subtrees: int, parts: int) -> list[tuple[int, int]]:
    """Contiguous blocks of subtrees per rank: rank r forms subtrees [n r / W, n (r + 1) / W)."""
    return [(n_subtrees * r // parts, n_subtrees * (r + 1) // parts) for r in range(parts)]


def send_images(images, owner_of, rank: int, world: int, dst: int = 0, group=None):
    """Move every subtree-root image to rank ``dst`` with point-to-point copies.  ``images`` maps
    subtree index -> complex64 tensor: on its owner the formed image, on ``dst`` a preallocated
    receive buffer of the right shape.  Returns the complete {subtree: image} on ``dst``, {} elsewhere."""
    dist = _dist()
    out = {}
    for s_, owner in enumerate(owner_of):
        if owner == dst:
            if rank == dst:
                out[s_] = images[s_]
            continue
        if rank == owner:
            dist.send(torch.view_as_real(images[s_].contiguous()), dst=dst, group=group)
        elif rank == dst:
            dist.recv(torch.view_as_real(images[s_]), src=owner, group=group)
            out[s_] = images[s_]
    return out


def ffbp_subtree_images(data, pos, weight, phase, subtrees, subtree_ids, range_start, data_dr, k):
    """Form the root images (complex64, full grid) of the given subtrees, each as its own plan."""
    out = {}
    for s_ in subtree_ids:
        nodes_s = subtrees[s_]
        root = nodes_s[0]
        prog = core.FFBPProgram(nodes_s, (0, root.nr), (0, root.nu), mode="split", device=data.device)
        out[s_] = prog.execute(data, pos, weight, phase, range_start, data_dr, k).clone()
        prog.close()  # host-only; the workspace returns to torch's stream-ordered cache
    return out


def ffbp_top(data, pos, weight, phase, top, external, images, crop_r, crop_u, range_start, data_dr, k):
    """Form the top of the tree from the subtree roots' images: the cropped root image."""
    prog = core.FFBPProgram(top, crop_r, crop_u, mode="split", device=data.device)
    for s_, idx in enumerate(external):
        prog.set_node_image(idx, images[s_])
    out = prog.execute(data, pos, weight, phase, range_start, data_dr, k).clone()
    prog.close()
    return out


def ffbp(data, pos, weight, phase, plan, range_start, data_dr, k, *, rank: int, world: int, group=None, dst: int = 0):
    """Split-precision FFBP of ``plan`` (gpu_backend.build_ffbp_plan) over ``world`` ranks: subtrees per
    rank, the top levels on rank ``dst``.  Returns the cropped root image on ``dst`` (None elsewhere),
    equal to core.FFBPProgram's on one GPU."""
    subtrees, top, external = ffbp_cut(plan.nodes()[0], world)
    owner_of = [r for r, (b, e) in enumerate(subtree_ranges(len(subtrees), world)) for _ in range(e - b)]
    mine = [s_ for s_, r in enumerate(owner_of) if r == rank]
    images = ffbp_subtree_images(data, pos, weight, phase, subtrees, mine, range_start, data_dr, k)
    if world > 1:
        if rank == dst:
            for s_, r in enumerate(owner_of):
                if r != dst:
                    root = subtrees[s_][0]
                    images[s_] = torch.empty((root.nr, root.nu), dtype=torch.complex64, device=data.device)
        images = send_images(images, owner_of, rank, world, dst=dst, group=group)
    if rank != dst:
        return None
    return ffbp_top(data, pos, weight, phase, top, external, images, plan.crop_r, plan.crop_u, range_start, data_dr,
                    k)
