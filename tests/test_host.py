"""Host-side checks that need no GPU: the C ABI loads and validates, the planner is bit-exact."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    from bp_project_gb300 import build
    build.build()
    from bp_project_gb300 import _native
    return _native


def _declared_symbols():
    text = (ROOT / "include" / "sarbp.h").read_text()
    return sorted(set(re.findall(r"\b(sarbp_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    handle = lib.load()
    declared = _declared_symbols()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(handle, name), name
        assert name in lib.SIGNATURES, f"{name} has no ctypes signature"
    assert handle.sarbp_abi_version() == 1
    assert b"sm_103a" in handle.sarbp_version()


def test_status_mapping(lib):
    with pytest.raises(ValueError):
        lib.check(lib.SARBP_ERR_VALUE, "x")
    with pytest.raises(TypeError):
        lib.check(lib.SARBP_ERR_TYPE, "x")
    with pytest.raises(RuntimeError):
        lib.check(lib.SARBP_ERR_CUDA, "x")
    lib.check(lib.SARBP_OK)


def test_capi_rejects_bad_arguments_before_touching_the_gpu(lib):
    h = lib.load()
    g = lib.polar_grid((0, 0, 10), 100.0, 0.5, 16, -0.1, 0.01, 16, 1)
    fake = ctypes.c_void_p(0x10000)  # never dereferenced: validation fails first
    args = [fake, 8, 64, fake, fake, fake, ctypes.byref(g), 90.0, 0.5, -50.0]
    assert h.sarbp_direct_polar(None, 8, 64, fake, fake, fake, ctypes.byref(g), 90.0, 0.5, -50.0, 3, 64, 1, fake,
                                None, 0, None) == lib.SARBP_ERR_TYPE
    assert h.sarbp_direct_polar(*args, 7, 64, 1, fake, None, 0, None) == lib.SARBP_ERR_VALUE       # mode
    assert h.sarbp_direct_polar(*args, 3, 0, 1, fake, None, 0, None) == lib.SARBP_ERR_VALUE        # chunk
    assert h.sarbp_direct_polar(*args, 3, 64, 9, fake, None, 0, None) == lib.SARBP_ERR_VALUE       # split > pulses
    assert h.sarbp_direct_polar(*args, 3, 64, 4, fake, None, 0, None) == lib.SARBP_ERR_WORKSPACE   # no scratch
    assert b"workspace" in h.sarbp_last_error()
    empty = lib.polar_grid((0, 0, 10), 100.0, 0.5, 0, -0.1, 0.01, 16, 1)
    assert h.sarbp_direct_polar(fake, 8, 64, fake, fake, fake, ctypes.byref(empty), 90.0, 0.5, -50.0, 3, 64, 1, fake,
                                None, 0, None) == lib.SARBP_ERR_VALUE
    assert b"empty image grids are unsupported" in h.sarbp_last_error()
    bad_side = lib.polar_grid((0, 0, 10), 100.0, 0.5, 4, -0.1, 0.01, 4, 0)
    assert h.sarbp_regrid(fake, ctypes.byref(bad_side), ctypes.byref(g), 1.0, 0, fake, None) == lib.SARBP_ERR_VALUE
    nan_grid = lib.polar_grid((0, 0, 10), float("nan"), 0.5, 4, -0.1, 0.01, 4, 1)
    assert h.sarbp_evaluate_image(fake, ctypes.byref(nan_grid), fake, 4, 1.0, fake, None) == lib.SARBP_ERR_VALUE
    assert h.sarbp_backproject_points(fake, 8, 64, fake, fake, fake, fake, 0, 90.0, 0.5, 1.0, 3, 1, fake, None, 0,
                                      None) == lib.SARBP_ERR_VALUE
    assert h.sarbp_ffbp_execute(None, fake, 8, 64, fake, fake, fake, 90.0, 0.5, 1.0, fake, None) == lib.SARBP_ERR_TYPE
    assert h.sarbp_direct_polar_workspace(3, ctypes.byref(g), 8, 4) == 4 * 16 * 16 * 8
    lat = lib.lattice((0, 0, 0), (0.5, 0, 0), (0, 0.5, 0), 64, 64)
    adj = [fake, 8, 64, fake, fake, fake, ctypes.byref(lat), 90.0, 0.5, -50.0, fake]
    # 2 x 2 tiles of 32 x 32 pixels, 8 pulses, 5 partial sums each
    assert h.sarbp_backproject_lattice_adjoint_workspace(ctypes.byref(lat), 8) == 4 * 8 * 5 * 4
    assert h.sarbp_backproject_lattice_adjoint(*adj, None, None, None, fake, 1 << 20, None) == lib.SARBP_ERR_VALUE
    assert h.sarbp_backproject_lattice_adjoint(*adj, fake, None, None, fake, 16, None) == lib.SARBP_ERR_WORKSPACE


def _node_array(lib, plan):
    nodes = plan.nodes()
    arr = (lib.FFBPNode * len(nodes))()
    for i, n in enumerate(nodes):
        e = arr[i]
        e.origin[:] = list(n.origin)
        e.r0, e.dr, e.u0, e.du = n.r0, n.dr, n.u0, n.du
        e.nr, e.nu, e.side, e.a, e.b = n.nr, n.nu, n.side, n.a, n.b
        e.left = -1 if n.left is None else n.left.index
        e.right = -1 if n.right is None else n.right.index
    return arr


@pytest.mark.parametrize("mode", ["fp64", "split"])
def test_ffbp_plan_object_on_host(golden, lib, mode):
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    g = golden("plans")
    fc, rmin, rmax, umin, umax, side, leaf, rs, osr = g["c1_args"]
    plan = build_ffbp_plan(g["c1_position"], fc, (rmin, rmax, umin, umax), side=int(side), leaf_size=int(leaf),
                           range_spacing=rs, angular_oversample=osr)
    arr = _node_array(lib, plan)
    h = lib.load()
    handle = ctypes.c_void_p()
    crop = (plan.crop_r[0], plan.crop_u[0], plan.nr, plan.nu)
    assert h.sarbp_ffbp_plan_create(arr, len(arr), *crop, lib.mode_id(mode), ctypes.byref(handle)) == 0
    # one launch for all leaves + one per tree height (8 merge levels for 256 leaves); the split path
    # adds three prologue launches (geometry tables, leaf pulses, child records), and with the merge
    # queue runs all merges as one launch
    assert h.sarbp_ffbp_launch_count(handle) == (12 if mode == "split" else 9)
    if mode == "split":
        assert h.sarbp_ffbp_set_merge_queue(handle, 1) == 0
        assert h.sarbp_ffbp_launch_count(handle) == 5
        assert h.sarbp_ffbp_set_merge_queue(handle, 0) == 0
        assert h.sarbp_ffbp_launch_count(handle) == 12
        assert h.sarbp_ffbp_set_wait_limit(handle, 0.0, -1) == lib.SARBP_ERR_VALUE
        assert h.sarbp_ffbp_set_wait_limit(handle, 1.0, len(arr) - 1) == lib.SARBP_ERR_VALUE  # a leaf
        assert h.sarbp_ffbp_set_wait_limit(handle, 1.0, 0) == 0
        # merge-tile staging: on by default, switchable before bind; nothing staged until bound
        assert h.sarbp_ffbp_set_staging(handle, 2) == lib.SARBP_ERR_VALUE
        assert h.sarbp_ffbp_set_staging(handle, 0) == 0
        assert h.sarbp_ffbp_set_staging(handle, 1) == 0
        staged = ctypes.c_int(-1)
        assert h.sarbp_ffbp_staging(handle, ctypes.byref(staged)) == 0 and staged.value == 0
        assert h.sarbp_ffbp_staging(handle, None) == lib.SARBP_ERR_TYPE
    else:
        assert h.sarbp_ffbp_set_merge_queue(handle, 1) == lib.SARBP_ERR_VALUE
    ws = h.sarbp_ffbp_workspace_bytes(handle)
    # node images (split mode: rows padded to an even length) + tables, tile records, node list
    images = sum(n.nr * n.nu * 8 for n in plan.nodes()[1:])
    assert images <= ws <= images * 1.06 + (1 << 26)
    # binding without a workspace is refused on the host
    assert h.sarbp_ffbp_bind(handle, None, 0, None) == lib.SARBP_ERR_WORKSPACE
    h.sarbp_ffbp_plan_destroy(handle)
    bad = _node_array(lib, plan)
    bad[0].left = 0  # a child must follow its parent
    assert h.sarbp_ffbp_plan_create(bad, len(bad), *crop, 3, ctypes.byref(handle)) == lib.SARBP_ERR_PLAN


@pytest.mark.parametrize("name", ["c0", "c1", "c3", "validate", "left"])
def test_product_planner_matches_reference_bit_for_bit(golden, name):
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    g = golden("plans")
    fc, rmin, rmax, umin, umax, side, leaf, rs, osr = g[f"{name}_args"]
    plan = build_ffbp_plan(g[f"{name}_position"], fc, (rmin, rmax, umin, umax), side=int(side), leaf_size=int(leaf),
                           range_spacing=rs, angular_oversample=osr)
    nodes = plan.nodes()
    geom = np.array([[*n.origin, n.r0, n.dr, n.u0, n.du, n.side] for n in nodes])
    idx = np.array([[n.a, n.b, n.nr, n.nu, -1 if n.left is None else n.left.index,
                     -1 if n.right is None else n.right.index] for n in nodes])
    np.testing.assert_array_equal(idx, g[f"{name}_idx"])
    np.testing.assert_array_equal(geom, g[f"{name}_geom"])  # same numpy operations -> identical bits
    np.testing.assert_array_equal([*plan.crop_r, *plan.crop_u], g[f"{name}_crop"])
    c = plan.counts
    np.testing.assert_array_equal([c["leaves"], c["merges"], c["leaf_pixel_pulse_products"], c["merged_pixels"],
                                   c["nodes"]], g[f"{name}_counts"])
    np.testing.assert_array_equal([plan.r0, plan.dr, plan.u0, plan.du, plan.nr, plan.nu], g[f"{name}_root"])


def test_planner_rejects_disjoint_extent():
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    pos = np.column_stack([np.zeros(32), np.linspace(-5, 5, 32), np.full(32, 100.0)])
    with pytest.raises(ValueError, match="does not intersect"):
        build_ffbp_plan(pos, 1e9, (1000.0, 1000.0 + 1e-9, 0.2, 0.2 + 1e-12), leaf_size=8)


def test_scene_generation_is_seeded():
    from bp_project_gb300 import scenes
    cfg = scenes.scaled(scenes.CONFIGS["c0"], pulses=64, samples=512, image_side=32)
    a = scenes.synthesize(cfg)
    b = scenes.synthesize(cfg)
    assert a.data.dtype == np.complex64 and a.data.shape == (64, 512)
    np.testing.assert_array_equal(a.data, b.data)
    assert np.abs(a.data).max() > 0.5  # the targets are in the range window
    assert a.lattice.points().shape == (32 * 32, 3)
    rmin, rmax, umin, umax = a.extent
    assert rmin < cfg.near_slant + 1 and rmax > rmin and umin < 0 < umax


def test_batch_create_validates_scenes_on_host(lib):
    h = lib.load()
    fake = 0x10000  # never dereferenced: validation fails first
    sc = (lib.BatchScene * 1)()
    e = sc[0]
    e.data = e.pos = e.weight = e.phase = e.out = fake
    e.pulses, e.samples = 8, 64
    e.range_start, e.data_dr, e.k = 90.0, 0.5, 1.0
    e.kind = lib.BATCH_DIRECT
    e.lattice = lib.lattice((0, 0, 0), (0.5, 0, 0.1), (0, 0.5, 0), 64, 64)  # tilted: not batchable
    handle = ctypes.c_void_p()
    assert h.sarbp_batch_create(sc, 1, 0, ctypes.byref(handle)) == lib.SARBP_ERR_VALUE
    assert b"flat" in h.sarbp_last_error()
    e.lattice = lib.lattice((0, 0, 0), (0.5, 0, 0), (0, 0.5, 0), 64, 64)
    e.tile_lc = 7
    assert h.sarbp_batch_create(sc, 1, 0, ctypes.byref(handle)) == lib.SARBP_ERR_VALUE
    e.tile_lc = 0
    e.kind = 5
    assert h.sarbp_batch_create(sc, 1, 0, ctypes.byref(handle)) == lib.SARBP_ERR_VALUE
    e.kind = lib.BATCH_FFBP  # FFBP scene without nodes
    assert h.sarbp_batch_create(sc, 1, 0, ctypes.byref(handle)) == lib.SARBP_ERR_VALUE
    e.data = 0
    assert h.sarbp_batch_create(sc, 1, 0, ctypes.byref(handle)) == lib.SARBP_ERR_TYPE
    assert h.sarbp_batch_create(sc, 0, 0, ctypes.byref(handle)) == lib.SARBP_ERR_VALUE
    assert h.sarbp_batch_execute(None, None) == lib.SARBP_ERR_TYPE


def test_batch_scene_list_matches_the_uneven_workload():
    from collections import Counter

    from bp_project_gb300 import scenes
    cfgs = scenes.batch_configs()
    assert len(cfgs) == 64 and Counter(k for _, k in cfgs) == {"direct": 32, "ffbp": 32}
    assert {c.pulses for c, _ in cfgs} <= set(range(512, 8193, 512))
    assert {c.image_side for c, _ in cfgs} <= {256, 512, 1024, 2048}
    assert all(3.5e3 <= c.near_slant <= 8e3 and 4 <= c.n_targets <= 16 for c, _ in cfgs)
    assert scenes.batch_configs()[5][0] == cfgs[5][0]  # seeded


def test_range_compress_entry_points_validate_on_host(lib):
    h = lib.load()
    fake = ctypes.c_void_p(0x10000)
    assert h.sarbp_rc_prepare(None, 4, 100, 128, fake, None) == lib.SARBP_ERR_TYPE
    assert h.sarbp_rc_prepare(fake, 4, 100, 50, fake, None) == lib.SARBP_ERR_VALUE
    assert h.sarbp_rc_filter(fake, fake, 4, 128, 100, fake, None) == lib.SARBP_ERR_VALUE
    assert h.sarbp_rc_crop(fake, 4, 100, 60, 50, 1.0, fake, None) == lib.SARBP_ERR_VALUE


def test_decode_iq_validates_on_host(lib):
    h = lib.load()
    fake = ctypes.c_void_p(0x10000)
    assert h.sarbp_decode_iq(None, 4, 1152, 160, 240, fake, None) == lib.SARBP_ERR_TYPE
    assert h.sarbp_decode_iq(fake, 4, 1152, 160, 300, fake, None) == lib.SARBP_ERR_VALUE  # I/Q past the frame
    assert h.sarbp_decode_iq(fake, 4, 1150, 160, 240, fake, None) == lib.SARBP_ERR_TYPE   # misaligned frames


def test_lattice_detection_for_point_lists():
    """ffbp.lattice_of recognises row-major affine lattices (to 1 nm) and rejects anything else."""
    from bp_project_gb300.ffbp import lattice_of
    xs = 2645.8 + np.arange(40) * 0.5
    ys = -12.3 + np.arange(70) * 0.5
    xx, yy = np.meshgrid(xs, ys, indexing="ij")
    pts = np.column_stack([xx.ravel(), yy.ravel(), np.zeros(xx.size)])
    origin, sr, sc, rows, cols = lattice_of(pts)
    assert (rows, cols) == (40, 70) and np.allclose(sr, (0.5, 0, 0)) and np.allclose(sc, (0, 0.5, 0))
    assert np.allclose(origin, pts[0])
    tilted = pts + np.column_stack([np.zeros(len(pts)), np.zeros(len(pts)), 0.01 * np.repeat(np.arange(40), 70)])
    assert lattice_of(tilted)[3:] == (40, 70)
    shuffled = pts[np.random.default_rng(0).permutation(len(pts))]
    assert lattice_of(shuffled) is None
    nudged = pts.copy()
    nudged[500, 0] += 1e-6
    assert lattice_of(nudged) is None
    assert lattice_of(pts[:1000]) is None  # not whole rows


def test_static_entry_point_checks_like_the_workspace_entry_point(lib):
    """The allocation-free entry point rejects misaligned pointers, non-finite grids and
    oversized splits with the workspace entry point's statuses, before any GPU call."""
    h = lib.load()
    fake = ctypes.c_void_p(0x10000)  # never dereferenced: validation fails first
    odd = ctypes.c_void_p(0x10004)   # 4-byte aligned only
    g = lib.polar_grid((0, 0, 10), 100.0, 0.5, 16, -0.1, 0.01, 16, 1)

    def both(data, grid, split=1, chunk=64):
        a = h.sarbp_direct_polar(data, 8, 64, fake, fake, fake, ctypes.byref(grid), 90.0, 0.5, -50.0, 3, chunk,
                                 split, fake, fake, 1 << 30, None)
        b = h.sarbp_direct_polar_static(data, 8, 64, fake, fake, fake, ctypes.byref(grid), 90.0, 0.5, -50.0, chunk,
                                        split, fake, None)
        return a, b

    assert both(odd, g) == (lib.SARBP_ERR_TYPE, lib.SARBP_ERR_TYPE)
    assert b"aligned" in h.sarbp_last_error()
    for field in ("r0", "dr", "u0", "du"):
        bad = lib.polar_grid((0, 0, 10), 100.0, 0.5, 16, -0.1, 0.01, 16, 1)
        setattr(bad, field, float("nan"))
        assert both(fake, bad) == (lib.SARBP_ERR_VALUE, lib.SARBP_ERR_VALUE), field
        assert b"finite" in h.sarbp_last_error()
    bad = lib.polar_grid((float("inf"), 0, 10), 100.0, 0.5, 16, -0.1, 0.01, 16, 1)
    assert both(fake, bad) == (lib.SARBP_ERR_VALUE, lib.SARBP_ERR_VALUE)
    assert both(fake, g, chunk=0) == (lib.SARBP_ERR_VALUE, lib.SARBP_ERR_VALUE)
    assert both(fake, g, split=9) == (lib.SARBP_ERR_VALUE, lib.SARBP_ERR_VALUE)
    # A split whose product with nr * nu would wrap 64 bits is refused, not wrapped past the check.
    huge = lib.polar_grid((0, 0, 10), 100.0, 0.5, 1 << 30, -0.1, 0.01, 1 << 30, 1)
    st = h.sarbp_direct_polar_static(fake, 1 << 20, 64, fake, fake, fake, ctypes.byref(huge), 90.0, 0.5, -50.0, 64,
                                     1 << 4, fake, None)
    assert st == lib.SARBP_ERR_VALUE
    assert b"exceeds the static scratch" in h.sarbp_last_error()
