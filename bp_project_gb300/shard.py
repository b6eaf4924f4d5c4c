"""Direct BP over several GPUs, one process per GPU: pixel bands or pulse ranges.

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
