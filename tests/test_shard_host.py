"""Host logic of the multi-GPU partitions (bp_project_gb300.shard), without a GPU: the direct-BP
band and pulse partitions, the FFBP subtree cut and its plans with external nodes, and the
collectives (band gather, rank-order reduction, subtree-root transfer) run as gloo ranks on the
CPU, with synthetic bands, partial images and subtree roots standing in for the GPU's."""
import ctypes
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from bp_project_gb300 import shard  # noqa: E402


@pytest.mark.parametrize("rows", [0, 1, 31, 32, 33, 100, 2048, 2049])
@pytest.mark.parametrize("parts", [1, 2, 3, 5, 8])
def test_row_bands_cover_exactly_on_tile_boundaries(rows, parts):
    bands = shard.row_bands(rows, parts)
    assert len(bands) == parts
    assert bands[0][0] == 0 and bands[-1][1] == rows
    for (b0, e0), (b1, e1) in zip(bands, bands[1:]):
        assert e0 == b1
    for b, e in bands:
        assert b <= e and b % shard.LATTICE_TILE_ROWS == 0
    sizes = [-(-(e - b) // 32) for b, e in bands]
    assert max(sizes) - min(sizes) <= 1


def _kernel_split_range(p0, p1, parts, part):
    """split_range of split.cu: b = p0 + len * part / parts (64-bit integer division)."""
    n = p1 - p0
    return p0 + n * part // parts, p0 + n * (part + 1) // parts


@pytest.mark.parametrize("pulses", [1, 7, 31, 1024, 4097])
@pytest.mark.parametrize("parts", [1, 2, 3, 4, 8])
def test_pulse_ranges_are_the_kernels_split(pulses, parts):
    ranges = shard.pulse_ranges(pulses, parts)
    assert ranges == [_kernel_split_range(0, pulses, parts, s) for s in range(parts)]
    assert ranges[0][0] == 0 and ranges[-1][1] == pulses
    assert all(e0 == b1 for (_, e0), (b1, _) in zip(ranges, ranges[1:]))


def test_band_origin_is_exact_for_power_of_two_steps():
    origin, step = (2134.298046, -511.75, 0.0), (0.5, 0.0, 0.0)
    for b in range(0, 2048, 32):
        o = shard.band_origin(origin, step, b)
        for i in (0, 1, 17, 31):
            assert o[0] + i * step[0] == origin[0] + (b + i) * step[0]


def test_argument_errors():
    with pytest.raises(ValueError):
        shard.row_bands(10, 0)
    with pytest.raises(ValueError):
        shard.pulse_ranges(-1, 2)


def _synthetic(rows, cols, seed):
    g = np.random.default_rng(seed)
    return torch.from_numpy((g.standard_normal((rows, cols)) + 1j * g.standard_normal((rows, cols)))
                            .astype(np.complex64))


def _rank(rank, world, port, rows, cols, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from bp_project_gb300 import shard as sh
        full = _synthetic(rows, cols, 1)
        bands = sh.row_bands(rows, world)
        b, e = bands[rank]
        gathered = sh.gather_rows(full[b:e].clone(), bands, rank, world)
        parts = [_synthetic(rows, cols, 10 + r) for r in range(world)]
        summed = sh.reduce_in_rank_order(parts[rank], rank, world, dst=0, add=lambda a, x: a.add_(x))
        with pytest.raises(ValueError):
            sh.reduce_in_rank_order(parts[rank], rank, world)  # host tensors need an explicit add
        out[rank] = (gathered.numpy(), None if summed is None else summed.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,rows", [(2, 100), (3, 70)])
def test_gather_and_rank_order_reduction_over_gloo(world, rows):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cols = 24
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(world, port, rows, cols, out), nprocs=world, join=True, start_method="spawn")
    results = dict(out)
    manager.shutdown()
    full = _synthetic(rows, cols, 1).numpy()
    parts = [_synthetic(rows, cols, 10 + r).numpy() for r in range(world)]
    want = parts[0].copy()
    for p in parts[1:]:
        want = (want + p).astype(np.complex64)  # ((p0 + p1) + p2): FP32 elementwise, rank order
    for rank in range(world):
        gathered, summed = results[rank]
        assert np.array_equal(gathered, full)  # every band, on every rank
        if rank == 0:
            assert np.array_equal(summed, want)
        else:
            assert summed is None


def _c1_plan(golden):
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    g = golden("plans")
    fc, rmin, rmax, umin, umax, side, leaf, rs, osr = g["c1_args"]
    return build_ffbp_plan(g["c1_position"], fc, (rmin, rmax, umin, umax), side=int(side), leaf_size=int(leaf),
                           range_spacing=rs, angular_oversample=osr)


def _leaves(nodes):
    return [(n.a, n.b) for n in nodes if getattr(n, "left", None) is None]


@pytest.mark.parametrize("parts", [1, 2, 3, 4, 8])
def test_ffbp_cut_covers_the_tree(golden, parts):
    plan = _c1_plan(golden)
    nodes = plan.nodes()
    subtrees, top, external = shard.ffbp_cut(nodes[0], parts)
    depth = max(0, (parts - 1).bit_length())
    assert len(subtrees) == 2 ** depth >= parts
    # the subtrees' leaves are the plan's leaves, in order, and each subtree's pulses are contiguous
    assert sum((_leaves(s_) for s_ in subtrees), []) == _leaves(nodes)
    for s_ in subtrees:
        lv = _leaves(s_)
        assert all(b0 == a1 for (_, b0), (a1, _) in zip(lv, lv[1:]))
    # the top tree: the plan's nodes above depth d, then the external subtree roots as leaves
    assert len(top) == (2 ** depth - 1) + len(subtrees)
    for s_, idx in enumerate(external):
        e, r = top[idx], subtrees[s_][0]
        assert (e.a, e.b, e.left) == (-1, -1, None)
        assert (e.nr, e.nu, e.r0, e.u0) == (r.nr, r.nu, r.r0, r.u0)
    ranges = shard.subtree_ranges(len(subtrees), parts)
    assert ranges[0][0] == 0 and ranges[-1][1] == len(subtrees)
    assert all(e0 == b1 for (_, e0), (b1, _) in zip(ranges, ranges[1:]))


def test_plans_with_external_nodes_on_host(golden):
    from bp_project_gb300 import _native as nat
    from bp_project_gb300 import build, core
    build.build()
    h = nat.load()
    plan = _c1_plan(golden)
    subtrees, top, external = shard.ffbp_cut(plan.nodes()[0], 4)
    arr = core.node_array(top)
    handle = ctypes.c_void_p()
    crop = (plan.crop_r[0], plan.crop_u[0], plan.crop_r[1] - plan.crop_r[0], plan.crop_u[1] - plan.crop_u[0])
    assert h.sarbp_ffbp_plan_create(arr, len(arr), *crop, nat.mode_id("split"), ctypes.byref(handle)) == 0
    assert h.sarbp_ffbp_launch_count(handle) == 3 + 1 + 2  # prologues, (empty) leaf stage, two merge levels
    fake = ctypes.c_void_p(0x10000)
    assert h.sarbp_ffbp_set_node_image(handle, external[0], fake, None) == nat.SARBP_ERR_PLAN  # not bound
    h.sarbp_ffbp_plan_destroy(handle)
    # the root cannot be external
    arr[0].left = arr[0].right = -1
    arr[0].a = arr[0].b = -1
    assert h.sarbp_ffbp_plan_create(arr, 1, 0, 0, 1, 1, nat.mode_id("split"), ctypes.byref(handle)) == \
        nat.SARBP_ERR_PLAN


def _send_rank(rank, world, port, shapes, owner_of, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from bp_project_gb300 import shard as sh
        images = {}
        for s_, (shape, owner) in enumerate(zip(shapes, owner_of)):
            if owner == rank:
                images[s_] = _synthetic(*shape, 100 + s_)
            elif rank == 0:
                images[s_] = torch.empty(shape, dtype=torch.complex64)
        got = sh.send_images(images, owner_of, rank, world, dst=0)
        out[rank] = {k: v.numpy() for k, v in got.items()}
    finally:
        dist.destroy_process_group()


def test_subtree_images_reach_the_top_rank_over_gloo():
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    world = 3
    shapes = [(5, 7), (6, 7), (5, 8), (6, 8)]
    owner_of = [r for r, (b, e) in enumerate(shard.subtree_ranges(4, world)) for _ in range(e - b)]
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_send_rank, args=(world, port, shapes, owner_of, out), nprocs=world, join=True,
                       start_method="spawn")
    results = dict(out)
    manager.shutdown()
    assert set(results[0]) == {0, 1, 2, 3}
    for s_, shape in enumerate(shapes):
        assert np.array_equal(results[0][s_], _synthetic(*shape, 100 + s_).numpy())
    assert results[1] == {} and results[2] == {}
