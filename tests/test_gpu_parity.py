"""GPU parity: libsarbp (through its C ABI) against the reference's outputs and the FP64 oracle.

Tolerances (relative complex L2 error, ||est - ref|| / ||ref||):
* reference policies, as the reference asserts them (gpu_baseline.py:206-213):
  fp64 <= 1e-5, mixed <= 1e-3, fp32 finite (engineering target ~1e-2);
* split precision: <= 1e-5 vs FP64 for direct BP, <= 1e-4 vs the reference FFBP.
"""
import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DIRECT_TOL = {"fp64": 1e-5, "mixed": 1e-3, "fp32": 5e-2, "split": 1e-5}
FFBP_TOL = {"fp64": 1e-5, "mixed": 1e-3, "fp32": 5e-2, "split": 1e-4}


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build
    build.build()
    from bp_project_gb300 import _native
    _native.load()
    return _native


@pytest.fixture(scope="module")
def backend(lib):
    from bp_project_gb300.gpu_backend import CudaBaseline
    return CudaBaseline()


def _dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


def _op_case(golden, case):
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    g = golden("operator_validation")
    p = f"case{case}_"
    range_start, data_dr, fc, k, side, *extent = g[p + "scalars"]
    plan = build_ffbp_plan(g[p + "position"], fc, extent, side=int(side), leaf_size=8, range_spacing=0.5,
                           angular_oversample=3.0)
    return g, p, plan, range_start, data_dr, fc, k, int(side), extent


@pytest.mark.parametrize("case", [0, 1])
@pytest.mark.parametrize("mode", ["fp64", "fp32", "mixed", "split"])
def test_operator_validation(golden, backend, case, mode):
    """gpu_baseline.gpu_operator_validation: odd pulse count, both k signs and sides, phase ramp, chunk 7."""
    g, p, plan, range_start, data_dr, fc, k, side, extent = _op_case(golden, case)
    device = backend.upload(g[p + "data"], g[p + "position"], g[p + "weight"], g[p + "phase"], plan)
    direct, _, _ = backend.run_direct(plan, device, mode, range_start, data_dr, k, chunk_pulses=7)
    ff, _, _ = backend.run_ffbp(plan, device, mode, range_start, data_dr, k)
    direct, _ = backend.download(direct)
    ff, _ = backend.download(ff)
    assert np.isfinite(direct).all() and np.isfinite(ff).all()
    assert direct.shape == g[p + "direct"].shape and ff.shape == g[p + "ffbp"].shape
    e_direct = rel_err(g[p + "direct"], direct)
    e_ffbp = rel_err(g[p + "ffbp"], ff)
    print(f"case {case} {mode}: direct {e_direct:.3e}, ffbp {e_ffbp:.3e}")
    assert e_direct <= DIRECT_TOL[mode]
    assert e_ffbp <= FFBP_TOL[mode]


@pytest.mark.parametrize("case", [0, 1])
def test_split_direct_vs_fp64_oracle(golden, lib, case):
    from bp_project_gb300 import core
    from oracle import reference as ora
    g, p, plan, range_start, data_dr, fc, k, side, extent = _op_case(golden, case)
    _, full = ora.bp_polar(g[p + "data"], g[p + "position"], plan.origin, plan.r0, plan.dr, plan.nr, plan.u0,
                           plan.du, plan.nu, range_start, data_dr, k, g[p + "weight"], g[p + "phase"], side, c128=True)
    args = (_dev(g[p + "data"], torch.complex64), _dev(g[p + "position"], torch.float64),
            _dev(g[p + "weight"], torch.float64), _dev(g[p + "phase"], torch.float64))
    for split in (1, 3):
        img = core.direct_polar(*args, plan.grid(), range_start, data_dr, k, mode="split", pulse_split=split)
        err = rel_err(full, img.cpu().numpy())
        print(f"case {case} pulse_split {split}: split vs FP64 {err:.3e}")
        assert err <= 1e-5


def test_points_and_helpers(golden, lib):
    from bp_project_gb300 import ffbp
    g = golden("points")
    r_start, ddr, fc, k, *extent = g["scalars"]
    for mode, tol in (("split", 1e-5), ("fp64", 1e-6), ("mixed", 1e-5)):
        out = ffbp.backproject_points(g["data"], g["position"], g["points"], r_start, ddr, k, g["weight"], g["phase"],
                                      mode=mode)
        err = rel_err(g["direct"], out)
        print(f"backproject_points {mode}: {err:.3e}")
        assert err <= tol
    ax = g["ffbp_axes"]
    ev = ffbp.evaluate_image(g["ffbp"], ax[:3], ax[3], ax[4], ax[5], ax[6], g["eval_points"], k)
    assert rel_err(g["evaluate"], ev) <= 1e-5
    tc = ffbp.target_contributions(g["data"], g["position"], g["targets"], r_start, ddr, k)
    assert rel_err(g["contrib"], tc) <= 1e-5
    # The evaluation points are a lattice (x fastest): the split-precision lattice path matches too.
    from bp_project_gb300 import core
    pts = g["eval_points"]
    xs, ys = np.unique(pts[:, 0]), np.unique(pts[:, 1])
    assert len(xs) * len(ys) == len(pts)
    image = torch.from_numpy(g["ffbp"]).cuda()
    grid = core.Grid(tuple(ax[:3]), ax[3], ax[4], image.shape[0], ax[5], ax[6], image.shape[1], 1)
    lat = core.evaluate_lattice(image, grid, (xs[0], ys[0], 0.0), (0.0, ys[1] - ys[0], 0.0), (xs[1] - xs[0], 0.0, 0.0),
                                len(ys), len(xs), k)
    err = rel_err(g["evaluate"], lat.cpu().numpy().ravel())
    print(f"evaluate_lattice vs reference: {err:.3e}")
    assert err <= 1e-5
    img, counts = ffbp.form_ffbp(g["data"], g["position"], r_start, ddr, fc, extent, leaf_size=32, range_spacing=0.5,
                                 angular_oversample=2.0, weight=g["weight"], verbose=False)
    assert img.image.shape == g["ffbp"].shape
    assert rel_err(g["ffbp"], img.image) <= 1e-4


@pytest.mark.parametrize("mode,tol", [("fp64", 1e-6), ("mixed", 1e-5), ("fp32", 5e-2), ("split", 1e-5)])
def test_regrid(golden, lib, mode, tol):
    from bp_project_gb300 import ffbp
    g = golden("kernels")
    sr0, sdr, su0, sdu, r0, dr, nr, u0, du, nu, k = g["grid"]
    for side in (1, -1):
        out = ffbp.regrid(g["image"], g["src_origin"], sr0, sdr, su0, sdu, g["dst_origin"], r0, dr, int(nr), u0, du,
                          int(nu), k, side, mode=mode)
        assert rel_err(g[f"regrid_side{side}"], out) <= tol


def _scene(name, **kw):
    from bp_project_gb300 import scenes
    cfg = scenes.CONFIGS[name] if not kw else scenes.scaled(scenes.CONFIGS[name], **kw)
    return scenes.synthesize(cfg, device="cuda")


def _lattice_split(scene, mode="split", pulse_split=1):
    from bp_project_gb300 import core
    lat = scene.lattice
    args = (_dev(scene.data, torch.complex64), _dev(scene.position, torch.float64), _dev(scene.weight, torch.float64),
            _dev(scene.phase, torch.float64))
    return core.backproject_lattice(*args, lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols,
                                    scene.range_start, scene.data_dr, scene.k, mode=mode, pulse_split=pulse_split)


def test_c0_full_image_vs_fp64_oracle(lib):
    """Config 0 at full size (1024 pulses x 2048 bins, 512^2 ground grid): split and FP64 kernels vs the oracle."""
    from oracle import reference as ora
    sc = _scene("c0")
    _, full = ora.backproject_points(sc.data, sc.position, sc.lattice.points(), sc.range_start, sc.data_dr, sc.k,
                                     sc.weight, sc.phase, c128=True)
    full = full.reshape(sc.lattice.rows, sc.lattice.cols)
    split = _lattice_split(sc).cpu().numpy()
    err = rel_err(full, split)
    print(f"c0 split vs FP64: {err:.3e}")
    assert err <= 1e-5
    # Point-target peaks: same pixel as the FP64 image around every target.
    amp_ref, amp = np.abs(full), np.abs(split)
    lat = sc.lattice
    for t in sc.targets:
        i = int(round((t[0] - lat.origin[0]) / lat.step_row[0]))
        j = int(round((t[1] - lat.origin[1]) / lat.step_col[1]))
        win = (slice(max(i - 6, 0), i + 7), slice(max(j - 6, 0), j + 7))
        assert np.unravel_index(amp_ref[win].argmax(), amp_ref[win].shape) == \
            np.unravel_index(amp[win].argmax(), amp[win].shape)
    mixed = _lattice_split(sc, mode="mixed").cpu().numpy()
    assert rel_err(full, mixed) <= 1e-5


@pytest.mark.parametrize("shape,step,tilt,shift", [((37, 45), 0.5, 0.0, 0.0),      # ragged tile edges
                                                   ((64, 100), 1.3, 0.0, "edge"),  # runs past the range window
                                                   ((33, 31), 0.7, 0.12, 0.0)])    # tilted (3-D) lattice
def test_ragged_and_edge_lattices_vs_fp64_oracle(lib, shape, step, tilt, shift):
    """Lattices that are not tile multiples, that extend beyond the data's range window (pixels
    with no sample1 support must be exactly the oracle's), and that are not flat."""
    from bp_project_gb300 import core
    from oracle import reference as ora
    sc = _scene("c0", pulses=384, image_side=64)
    lat = sc.lattice
    rows, cols = shape
    if shift == "edge":  # centre the lattice's rows on the far end of the range window
        far = sc.range_start + (sc.data.shape[1] - 3) * sc.data_dr
        edge = np.sqrt(far ** 2 - sc.config.altitude ** 2)
        shift = edge - lat.origin[0] - 0.5 * rows * step
    origin = (lat.origin[0] + shift, lat.origin[1], 0.0)
    srow, scol = (step, 0.0, tilt), (0.0, step, 0.0)
    i = np.arange(rows)[:, None, None]
    j = np.arange(cols)[None, :, None]
    pts = (np.array(origin) + i * np.array(srow) + j * np.array(scol)).reshape(-1, 3)
    _, ref = ora.backproject_points(sc.data, sc.position, pts, sc.range_start, sc.data_dr, sc.k, sc.weight, sc.phase,
                                    c128=True)
    args = [_dev(a, dt) for a, dt in ((sc.data, torch.complex64), (sc.position, torch.float64),
                                      (sc.weight, torch.float64), (sc.phase, torch.float64))]
    for mode, tol in (("split", 1e-5), ("fp64", 1e-6)):
        out = core.backproject_lattice(*args, origin, srow, scol, rows, cols, sc.range_start, sc.data_dr, sc.k,
                                       mode=mode).cpu().numpy().ravel()
        zero = np.abs(ref) == 0
        if shift:
            assert zero.any() and (~zero).any()  # part of the lattice lies outside the range window
        assert np.all(out[zero] == 0)
        err = rel_err(ref, out)
        print(f"{shape} step {step} tilt {tilt} shift {shift} {mode}: {err:.2e}")
        assert err <= tol


@pytest.mark.parametrize("step", [6.0, 1.0, 0.9])
def test_lattice_tiles_outside_the_envelope_match_fp64(lib, step):
    """Coarse lattices whose 32 x 32 tiles are too wide for the fast path's precision envelope
    (K rho^2 > 8 R at 6 m and 1 m spacing, windows of ~330 and ~55 bins): every pulse takes the
    lattice tiles' two-float fallback, which must meet the split tolerance against the FP64
    oracle.  At 0.9 m the tiles fit the envelope again (fast path, wide windows)."""
    from bp_project_gb300 import core
    from oracle import reference as ora
    sc = _scene("c0", pulses=384, image_side=64)
    lat = sc.lattice
    rows = cols = 40
    centre = lat.origin + 0.5 * lat.rows * lat.step_row + 0.5 * lat.cols * lat.step_col
    origin = tuple(centre - 0.5 * step * np.array([rows, cols, 0.0]))
    srow, scol = (step, 0.0, 0.0), (0.0, step, 0.0)
    i = np.arange(rows)[:, None, None]
    j = np.arange(cols)[None, :, None]
    pts = (np.array(origin) + i * np.array(srow) + j * np.array(scol)).reshape(-1, 3)
    _, ref = ora.backproject_points(sc.data, sc.position, pts, sc.range_start, sc.data_dr, sc.k, sc.weight, sc.phase,
                                    c128=True)
    args = [_dev(a, dt) for a, dt in ((sc.data, torch.complex64), (sc.position, torch.float64),
                                      (sc.weight, torch.float64), (sc.phase, torch.float64))]
    out = core.backproject_lattice(*args, origin, srow, scol, rows, cols, sc.range_start, sc.data_dr, sc.k,
                                   mode="split").cpu().numpy().ravel()
    err = rel_err(ref, out)
    print(f"lattice step {step} m (two-float fallback tiles): {err:.2e}")
    assert err <= 1e-5


def test_points_outside_the_envelope_match_fp64(lib):
    """Points scattered over the whole scene: every 1024-point tile is too wide for the split
    path's precision envelope, so every pulse takes the two-float fallback; it must still meet
    the split tolerance against the FP64 oracle (and the tiles that fit still use the fast path)."""
    from bp_project_gb300 import core
    from oracle import reference as ora
    sc = _scene("c0", pulses=384, image_side=256)
    rng = np.random.default_rng(12)
    lat = sc.lattice
    span = lat.rows * lat.step_row[0]
    pts = np.column_stack([lat.origin[0] + rng.uniform(0, span, 3000), lat.origin[1] + rng.uniform(0, span, 3000),
                           rng.uniform(-2, 2, 3000)])
    _, ref = ora.backproject_points(sc.data, sc.position, pts, sc.range_start, sc.data_dr, sc.k, sc.weight, sc.phase,
                                    c128=True)
    args = [_dev(a, dt) for a, dt in ((sc.data, torch.complex64), (sc.position, torch.float64),
                                      (sc.weight, torch.float64), (sc.phase, torch.float64))]
    out = core.backproject_points(*args, _dev(pts, torch.float64), sc.range_start, sc.data_dr, sc.k,
                                  mode="split").cpu().numpy()
    err = rel_err(ref, out)
    print(f"scattered points (two-float fallback): {err:.2e}")
    assert err <= 1e-5


def test_backproject_points_on_a_meshgrid_uses_the_lattice_kernel(lib):
    """ffbp.backproject_points with run.py's kind of ground meshgrid (host float64, row-major) is imaged by
    the lattice kernel: identical to core.backproject_lattice, within 1e-5 of the FP64 oracle; a shuffled
    copy of the same points (no lattice) goes through the points kernel and agrees to 1e-5."""
    from bp_project_gb300 import core, ffbp
    from oracle import reference as ora
    sc = _scene("c0", pulses=384, image_side=64)
    lat = sc.lattice
    rows, cols = 48, 40
    i = np.arange(rows)[:, None, None]
    j = np.arange(cols)[None, :, None]
    pts = (lat.origin + i * lat.step_row + j * lat.step_col).reshape(-1, 3)
    img = ffbp.backproject_points(sc.data, sc.position, pts, sc.range_start, sc.data_dr, sc.k, sc.weight, sc.phase,
                                  mode="split")
    args = [_dev(a, dt) for a, dt in ((sc.data, torch.complex64), (sc.position, torch.float64),
                                      (sc.weight, torch.float64), (sc.phase, torch.float64))]
    direct = core.backproject_lattice(*args, tuple(lat.origin), tuple(lat.step_row), tuple(lat.step_col), rows, cols,
                                      sc.range_start, sc.data_dr, sc.k, mode="split").cpu().numpy().ravel()
    assert np.array_equal(img.view(np.uint32), direct.view(np.uint32))
    _, ref = ora.backproject_points(sc.data, sc.position, pts, sc.range_start, sc.data_dr, sc.k, sc.weight, sc.phase,
                                    c128=True)
    assert rel_err(ref, img) <= 1e-5
    perm = np.random.default_rng(5).permutation(len(pts))
    shuffled = ffbp.backproject_points(sc.data, sc.position, pts[perm], sc.range_start, sc.data_dr, sc.k, sc.weight,
                                       sc.phase, mode="split")
    assert rel_err(ref[perm], shuffled) <= 1e-5


def test_evaluate_lattice_matches_points_path(lib):
    """Split-precision evaluate onto the 512^2 ground lattice vs the FP64-geometry points kernel."""
    from bp_project_gb300 import core
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    sc = _scene("c0")
    cfg = sc.config
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    args = [_dev(a, dt) for a, dt in ((sc.data, torch.complex64), (sc.position, torch.float64),
                                      (sc.weight, torch.float64), (sc.phase, torch.float64))]
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split", device="cuda")
    polar = prog.execute(*args, sc.range_start, sc.data_dr, sc.k)
    lat = sc.lattice
    fast = core.evaluate_lattice(polar, plan.grid(), lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols, sc.k)
    ref = core.evaluate_image(polar, plan.grid(), _dev(lat.points(), torch.float64), sc.k)
    err = rel_err(ref.cpu().numpy(), fast.cpu().numpy().ravel())
    print(f"evaluate_lattice vs points kernel: {err:.3e}")
    assert err <= 1e-5
    prog.close()


@pytest.mark.slow
def test_c1_direct_sampled_pixels(lib):
    """Config 1 at full size (4096 x 8192, 2048^2): split image vs FP64 oracle on 4096 random pixels."""
    from oracle import reference as ora
    sc = _scene("c1")
    img = _lattice_split(sc).cpu().numpy().ravel()
    rng = np.random.default_rng(1)
    idx = rng.choice(img.size, 4096, replace=False)
    ref = ora.backproject_points(sc.data, sc.position, sc.lattice.take(idx), sc.range_start, sc.data_dr, sc.k,
                                 sc.weight, sc.phase, c128=True)[1]
    err = rel_err(ref, img[idx])
    print(f"c1 sampled split vs FP64: {err:.3e}")
    assert err <= 1e-5


@pytest.mark.slow
def test_c2_direct_sampled_pixels(lib):
    """Config 2 at full size (30 km, 10 GHz, 8192 x 16384, 4096^2 at 0.25 m): split lattice image vs the FP64
    oracle on 2048 random pixels -- the long-range, fine-grid regime of the separable lattice loop."""
    from oracle import reference as ora
    sc = _scene("c2")
    img = _lattice_split(sc).cpu().numpy().ravel()
    rng = np.random.default_rng(2)
    idx = rng.choice(img.size, 2048, replace=False)
    ref = ora.backproject_points(sc.data, sc.position, sc.lattice.take(idx), sc.range_start, sc.data_dr, sc.k,
                                 sc.weight, sc.phase, c128=True)[1]
    err = rel_err(ref, img[idx])
    print(f"c2 sampled split vs FP64: {err:.3e}")
    assert err <= 1e-5


@pytest.mark.slow
def test_c1_ffbp_vs_reference_ffbp(lib):
    """Config 1 at full size: split FFBP (16-pulse leaves, 8 merge levels, root 3084 x 25031) within 1e-4 of the
    reference FFBP (oracle restatement of ffbp.form_ffbp on the same plan)."""
    from bp_project_gb300 import core
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    from oracle import reference as ora
    sc = _scene("c1")
    cfg = sc.config
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split")
    img = prog.execute(_dev(sc.data, torch.complex64), _dev(sc.position, torch.float64),
                       _dev(sc.weight, torch.float64), _dev(sc.phase, torch.float64), sc.range_start, sc.data_dr,
                       sc.k).cpu().numpy()
    prog.close()
    ref, counts = ora.form_ffbp(sc.data, sc.position, sc.range_start, sc.data_dr, cfg.fc, sc.extent, side=1,
                                leaf_size=cfg.leaf_size, range_spacing=cfg.range_spacing,
                                angular_oversample=cfg.angular_oversample, weight=sc.weight, phase=sc.phase)
    assert counts["leaves"] == 256 and counts["merges"] == 255
    err = rel_err(ref.image, img)
    print(f"c1 split FFBP vs reference FFBP: {err:.3e}")
    assert err <= 1e-4


def test_c2_geometry_ffbp_vs_reference_ffbp(lib):
    """The 30 km precision-stress geometry (10 GHz, 300 MHz, 150 m/s, 1.5 kHz) at 2048 pulses onto a 512^2
    image at 0.25 m: split FFBP (16-pulse leaves, merge tiles up to 1.5x the squarest radius) within 1e-4
    of the reference FFBP (oracle restatement of ffbp.form_ffbp on the same plan)."""
    from bp_project_gb300 import core
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    from oracle import reference as ora
    sc = _scene("c2", pulses=2048, samples=4096, image_side=512)
    cfg = sc.config
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split")
    img = prog.execute(_dev(sc.data, torch.complex64), _dev(sc.position, torch.float64),
                       _dev(sc.weight, torch.float64), _dev(sc.phase, torch.float64), sc.range_start, sc.data_dr,
                       sc.k).cpu().numpy()
    prog.close()
    ref, counts = ora.form_ffbp(sc.data, sc.position, sc.range_start, sc.data_dr, cfg.fc, sc.extent, side=1,
                                leaf_size=cfg.leaf_size, range_spacing=cfg.range_spacing,
                                angular_oversample=cfg.angular_oversample, weight=sc.weight, phase=sc.phase)
    assert counts["leaves"] == 128
    err = rel_err(ref.image, img)
    print(f"c2-geometry split FFBP vs reference FFBP: {err:.3e}")
    assert err <= 1e-4
    peak_ref = np.unravel_index(np.abs(ref.image).argmax(), ref.image.shape)
    assert np.unravel_index(np.abs(img).argmax(), img.shape) == peak_ref


def test_linearity_and_pulse_split(lib):
    """BP is linear in the data; splitting the aperture over CTAs changes only FP32 rounding."""
    from bp_project_gb300 import scenes
    sc = _scene("c0", pulses=512, samples=2048, image_side=256)
    rng = np.random.default_rng(3)
    other = (rng.standard_normal(sc.data.shape) + 1j * rng.standard_normal(sc.data.shape)).astype(np.complex64)
    a, b = 0.7 - 0.2j, -1.3 + 0.4j
    mix = scenes.Scene(**{**sc.__dict__, "data": (a * sc.data + b * other).astype(np.complex64)})
    x = _lattice_split(sc).cpu().numpy()
    y = _lattice_split(scenes.Scene(**{**sc.__dict__, "data": other})).cpu().numpy()
    z = _lattice_split(mix).cpu().numpy()
    assert rel_err(a * x.astype(np.complex128) + b * y, z) <= 1e-5
    z4 = _lattice_split(sc, pulse_split=4).cpu().numpy()
    assert rel_err(x, z4) <= 1e-6
    z0 = _lattice_split(sc, pulse_split=0).cpu().numpy()  # the split that fills the GPU (64 tiles here: > 1)
    assert rel_err(x, z0) <= 1e-6


@pytest.mark.parametrize("pulses,rows,cols", [(3, 7, 5), (64, 1, 1), (40, 33, 65)])
def test_auto_pulse_split_small_cases(lib, pulses, rows, cols):
    """pulse_split=0 picks at most `pulses` splits and matches the unsplit image to FP32 rounding."""
    from bp_project_gb300 import core
    sc = _scene("c0", pulses=pulses, image_side=64)
    lat = sc.lattice
    args = [_dev(a, dt) for a, dt in ((sc.data, torch.complex64), (sc.position, torch.float64),
                                      (sc.weight, torch.float64), (sc.phase, torch.float64))]
    geo = (lat.origin, lat.step_row, lat.step_col, rows, cols, sc.range_start, sc.data_dr, sc.k)
    one = core.backproject_lattice(*args, *geo, mode="split", pulse_split=1).cpu().numpy()
    auto = core.backproject_lattice(*args, *geo, mode="split", pulse_split=0).cpu().numpy()
    assert np.abs(one).max() > 0
    assert rel_err(one, auto) <= 1e-6


def test_resident_graph_replay_bitexact(golden, backend):
    from bp_project_gb300.batched_resident_backend import BatchedResidentProgram
    from bp_project_gb300.resident_backend import ResidentProgram
    g, p, plan, range_start, data_dr, fc, k, side, extent = _op_case(golden, 0)
    device = backend.upload(g[p + "data"], g[p + "position"], g[p + "weight"], g[p + "phase"], plan)
    for prog in (ResidentProgram(backend, plan, device, "split", range_start, data_dr, k, algorithm="direct"),
                 ResidentProgram(backend, plan, device, "split", range_start, data_dr, k, algorithm="ffbp",
                                 variant="fused"),
                 BatchedResidentProgram(backend, plan, device, "mixed", range_start, data_dr, k)):
        eager = prog.execute().clone()
        assert prog.capture_graph(), prog.metadata["graph_error"]
        prog.output.zero_()
        out = prog.replay()
        torch.cuda.synchronize()
        assert torch.equal(eager, out)
        prog.close()


def test_direct_polar_lut_probe(golden, lib):
    from bp_project_gb300 import core
    g, p, plan, range_start, data_dr, fc, k, side, extent = _op_case(golden, 0)
    args = (_dev(g[p + "data"], torch.complex64), _dev(g[p + "position"], torch.float64),
            _dev(g[p + "weight"], torch.float64), _dev(g[p + "phase"], torch.float64))
    lut = core.fill_range_phase_lut(g[p + "data"].shape[1], range_start, data_dr, k)
    out = core.direct_polar_lut(*args, plan.grid(), range_start, data_dr, k, lut)
    assert rel_err(g[p + "direct"], out.cpu().numpy()) <= 1e-4


@pytest.mark.parametrize("case", [0, 1])
def test_direct_polar_phase32_probes(golden, lib, case):
    """The FP32-sincos phase probes (gpu/precision_probe.cu:19-79) on the operator-validation recipe,
    against the reference's own FP64 direct BP: both within 1e-6 (a numpy restatement of the probe
    arithmetic gives 1.9e-7 unwrapped, 8e-8 wrapped, on these cases), the same peak pixel, and the
    FP64 remainder(phase, 2 pi) no worse than the plain cast."""
    from bp_project_gb300 import core
    g, p, plan, range_start, data_dr, fc, k, side, extent = _op_case(golden, case)
    args = (_dev(g[p + "data"], torch.complex64), _dev(g[p + "position"], torch.float64),
            _dev(g[p + "weight"], torch.float64), _dev(g[p + "phase"], torch.float64))
    ref = g[p + "direct"]
    errs = {}
    for wrapped in (False, True):
        out = core.direct_polar_phase32(*args, plan.grid(), range_start, data_dr, k, wrapped=wrapped).cpu().numpy()
        assert np.isfinite(out).all()
        errs[wrapped] = rel_err(ref, out)
        assert errs[wrapped] <= 1e-6, (wrapped, errs[wrapped])
        assert (np.unravel_index(np.abs(out).argmax(), out.shape)
                == np.unravel_index(np.abs(ref).argmax(), ref.shape))
    assert errs[True] <= 1.2 * errs[False] + 1e-8, errs
