"""Generate golden vectors by running the reference implementation itself.

Run in a container where the reference checkout is mounted (it is read-only
and never needed at test time):

    python tests/golden/make_golden.py /path/to/bp_project

The reference's CPU path is ``fast_bp/ffbp.py`` (Numba) and its FP64 planner
is ``fast_bp/gpu_backend.py:build_ffbp_plan``.  Numba and CuPy are not
installed here, so a no-op ``numba`` module (``njit`` returns the function,
``prange`` is ``range``) and an empty ``cupy`` module are placed in
``sys.modules`` first; the reference code then runs unchanged as pure
Python.  The outputs are stored as small compressed ``.npz`` fixtures next
to this script; tests compare the CPU oracle and the GPU path against them.

Cases
-----
operator_validation.npz
    The reference's GPU operator-validation recipe
    (``fast_bp/gpu_baseline.py:121-187``, seed 20260916): 31 pulses x 512
    random complex samples, leaf 8, both signs of k and both look sides,
    Hann weights and a phase ramp.  Stores inputs, the reference FFBP image
    (``form_ffbp``) and the reference direct image (``bp_polar`` on the plan
    grid), plus the flattened plan.
points.npz
    A reduced ``fast_bp/validate.py`` scene (analytic sinc point targets on
    a non-uniform 3-D track): ``backproject_points`` on point clusters,
    ``form_ffbp`` + ``evaluate_image``, and ``target_contributions``.
kernels.npz
    ``regrid`` of a random polar image, ``sample1`` / ``sample2`` /
    ``cubic_weights`` at random coordinates (including out-of-support ones).
plans.npz
    ``build_ffbp_plan`` on the benchmark trajectories (1024 pulses / leaf 64
    and 4096 pulses / leaf 16) and on the validate.py track, flattened.
autofocus.npz
    ``autofocus.estimate_update`` (fast_bp/autofocus.py:37-79) on the
    scenes of ``autofocus_scene.py`` (the reference's own recovery scene and
    a cluttered one), and ``autofocus.pick_targets`` (:19-34) on a seeded
    polar image.  matplotlib is absent here, so an empty module stands in
    for it (autofocus.py only plots in ``main``).

range_compress.npz
    ``sar_io.range_compress`` (fast_bp/sar_io.py:116-139) on seeded raw
    echoes (oversample 1 and 2), and the lag of the LFM point test of
    ``validate.py:54-59`` (oversample 4).
capture.npz
    ``sar_io.Capture`` (fast_bp/sar_io.py:18-82) on the synthetic raw capture
    written by ``capture_file.py``: frame count, valid frames, timing fields,
    navigation and ``read`` of a few pulses.
metrics.npz
    ``sar_quality/metrics.py`` (focus_metrics, fidelity, impulse_metrics) on
    seeded images and impulse cuts.  numpy 2 removed ``trapz``; the
    generator aliases it to ``numpy.trapezoid`` (same trapezoidal rule)
    before importing the module.

``python tests/golden/make_golden.py /path/to/bp_project autofocus`` rebuilds
only the named fixtures.
"""
from __future__ import annotations

import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def import_reference(root: Path):
    nb = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if args and callable(args[0]) and not kwargs:
            return args[0]
        return lambda fn: fn

    nb.njit = njit
    nb.prange = range
    nb.set_num_threads = lambda n: None
    sys.modules["numba"] = nb
    cp = types.ModuleType("cupy")
    cp.ndarray = object
    sys.modules["cupy"] = cp
    os.environ.setdefault("FAST_BP_CUDA_ROOT", "/usr/local/cuda" if Path("/usr/local/cuda").exists() else str(root))
    sys.path.insert(0, str(root / "fast_bp"))
    import ffbp  # noqa: E402
    import gpu_backend  # noqa: E402
    return ffbp, gpu_backend


def flatten_plan(plan):
    """Pre-order node arrays of a reference FFBPPlan."""
    nodes = []

    def walk(n):
        nodes.append(n)
        if n.left is not None:
            walk(n.left)
            walk(n.right)

    walk(plan.root)
    nodes.sort(key=lambda n: n.index)
    geom = np.array([[*n.origin, n.r0, n.dr, n.u0, n.du, n.side] for n in nodes], np.float64)
    idx = np.array([[n.a, n.b, n.nr, n.nu, -1 if n.left is None else n.left.index,
                     -1 if n.right is None else n.right.index] for n in nodes], np.int64)
    crop = np.array([*plan.crop_r, *plan.crop_u], np.int64)
    counts = np.array([plan.counts[k] for k in ("leaves", "merges", "leaf_pixel_pulse_products",
                                                 "merged_pixels", "nodes")], np.int64)
    root = np.array([plan.r0, plan.dr, plan.u0, plan.du, plan.nr, plan.nu], np.float64)
    return geom, idx, crop, counts, root


def operator_validation(ffbp, gb):
    from scipy.signal.windows import hann
    C, FC = 299792458.0, 1.4e9
    rng = np.random.default_rng(20260916)
    out = {}
    for case, (sign, side) in enumerate(((-1, 1), (1, -1))):
        pulses, samples = 31, 512
        slow = np.arange(pulses, dtype=np.float64)
        position = np.column_stack([0.05 * np.sin(0.37 * slow),
                                    np.linspace(-15.0, 15.0, pulses) + 0.03 * np.sin(slow),
                                    18.0 + 0.1 * np.cos(0.23 * slow)])
        data = (rng.standard_normal((pulses, samples)) + 1j * rng.standard_normal((pulses, samples))).astype(np.complex64)
        weight = hann(pulses)
        phase = np.linspace(-0.2, 0.3, pulses)
        range_start, data_dr = 900.0, 0.5
        extent = (1080.0, 1120.0, -0.05, 0.05)
        fc = sign * FC
        k = 4.0 * np.pi * fc / C
        plan = gb.build_ffbp_plan(position, fc, extent, side=side, leaf_size=8, range_spacing=0.5,
                                  angular_oversample=3.0)
        img, counts = ffbp.form_ffbp(data, position, range_start, data_dr, fc, extent, side=side, leaf_size=8,
                                     range_spacing=0.5, angular_oversample=3.0, weight=weight, phase=phase,
                                     verbose=False)
        direct = ffbp.bp_polar(data, position, plan.origin, plan.r0, plan.dr, plan.nr, plan.u0, plan.du,
                               plan.nu, range_start, data_dr, k, weight, phase, side)
        geom, idx, crop, cnt, root = flatten_plan(plan)
        p = f"case{case}_"
        out.update({p + "data": data, p + "position": position, p + "weight": weight, p + "phase": phase,
                    p + "scalars": np.array([range_start, data_dr, fc, k, side, *extent]),
                    p + "ffbp": img.image, p + "ffbp_axes": np.array([*img.origin, img.r0, img.dr, img.u0, img.du]),
                    p + "direct": direct, p + "geom": geom, p + "idx": idx, p + "crop": crop,
                    p + "counts": cnt, p + "root": root})
        print(f"operator case {case}: plan {plan.shape}, ffbp peak "
              f"{np.unravel_index(np.abs(img.image).argmax(), img.image.shape)}, direct peak "
              f"{np.unravel_index(np.abs(direct).argmax(), direct.shape)}", flush=True)
    return out


def validate_track(n):
    t = np.linspace(-1, 1, n)
    return np.column_stack([0.08 * np.sin(5 * t), 50 * t + 0.4 * t * t, 18 + 0.15 * np.sin(2 * t)])


def points_case(ffbp):
    from scipy.signal.windows import hann
    C, FC, FS = 299792458.0, 1.4e9, 400e6
    k = 4 * np.pi * FC / C
    n = 64
    pos = validate_track(n)
    targets = np.array([[710.31, -145.27, 0.0], [987.21, 31.72, 0.0]])
    strength = np.array([1, complex(0.7, 0.3)])
    r_start, ddr = 500.0, C / (2 * FS)
    rr = r_start + ddr * np.arange(1500)
    data = np.zeros((n, len(rr)), np.complex64)
    for xyz, a in zip(targets, strength):
        distance = np.linalg.norm(pos - xyz, axis=1)
        data += (a * np.exp(-1j * k * distance)[:, None]
                 * np.sinc((rr[None, :] - distance[:, None]) / (C / (2 * 200e6)))).astype(np.complex64)
    w = hann(n)
    phase = np.zeros(n)
    clusters = []
    for xyz in targets:
        x = xyz[0] + np.arange(-3, 3.01, 0.6)
        y = xyz[1] + np.arange(-8, 8.01, 0.8)
        xx, yy = np.meshgrid(x, y)
        clusters.append(np.column_stack([xx.ravel(), yy.ravel(), np.zeros(xx.size)]))
    points = np.vstack(clusters)
    direct = ffbp.backproject_points(data, pos, points, r_start, ddr, k, w, phase)
    extent = (718.0, 732.0, -0.215, -0.185)
    img, counts = ffbp.form_ffbp(data, pos, r_start, ddr, FC, extent, leaf_size=32, range_spacing=0.5,
                                 angular_oversample=2.0, weight=w, verbose=False)
    cl = clusters[0]
    fast = ffbp.evaluate_image(img.image, img.origin, img.r0, img.dr, img.u0, img.du, cl, k)
    contrib = ffbp.target_contributions(data, pos, targets, r_start, ddr, k)
    print(f"points: {len(points)} points, ffbp {img.image.shape}, counts {counts}", flush=True)
    return {"data": data, "position": pos, "weight": w, "phase": phase, "points": points,
            "scalars": np.array([r_start, ddr, FC, k, *extent]), "direct": direct, "ffbp": img.image,
            "ffbp_axes": np.array([*img.origin, img.r0, img.dr, img.u0, img.du]),
            "eval_points": cl, "evaluate": fast, "targets": targets, "contrib": contrib,
            "counts": np.array([counts[k] for k in ("leaves", "merges", "leaf_pixel_pulse_products",
                                                     "merged_pixels")], np.int64)}


def kernels_case(ffbp):
    rng = np.random.default_rng(77)
    img = (rng.standard_normal((40, 36)) + 1j * rng.standard_normal((40, 36))).astype(np.complex64)
    so = np.array([0.3, -4.0, 18.5])
    do = np.array([0.1, 2.0, 18.2])
    sr0, sdr, su0, sdu = 1000.0, 0.5, -0.05, 0.003
    r0, dr, nr, u0, du, nu = 1002.0, 0.5, 30, -0.04, 0.0021, 33
    k = -58.7
    out = {}
    for side in (1, -1):
        out[f"regrid_side{side}"] = ffbp.regrid(img, so, sr0, sdr, su0, sdu, do, r0, dr, nr, u0, du, nu, k, side)
    row = (rng.standard_normal(64) + 1j * rng.standard_normal(64)).astype(np.complex64)
    q = np.concatenate([rng.uniform(-2, 66, 200), np.arange(-2, 66, 1.0), [0.999999, 1.0, 60.9999, 61.0, 61.0001]])
    s1 = np.array([ffbp.sample1(row, float(v)) for v in q], np.complex128)
    qr = rng.uniform(-2, 42, 300)
    qu = rng.uniform(-2, 38, 300)
    s2 = np.array([ffbp.sample2(img, float(a), float(b)) for a, b in zip(qr, qu)], np.complex128)
    t = rng.uniform(-0.5, 1.5, 50)
    cw = np.array([ffbp.cubic_weights(float(v)) for v in t], np.float64)
    out.update({"image": img, "src_origin": so, "dst_origin": do,
                "grid": np.array([sr0, sdr, su0, sdu, r0, dr, nr, u0, du, nu, k]),
                "row": row, "q": q, "sample1": s1, "qr": qr, "qu": qu, "sample2": s2, "t": t, "cubic": cw})
    return out


def plans_case(gb):
    sys.path.insert(0, str(REPO))
    from bp_project_gb300 import scenes
    out = {}
    for name in ("c0", "c1", "c3"):
        cfg = scenes.CONFIGS[name]
        pos = scenes.trajectory(cfg)
        extent = scenes.polar_extent(cfg, pos)
        plan = gb.build_ffbp_plan(pos, cfg.fc, extent, side=1, leaf_size=cfg.leaf_size,
                                  range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
        geom, idx, crop, cnt, root = flatten_plan(plan)
        out.update({f"{name}_position": pos, f"{name}_args": np.array([cfg.fc, *extent, 1, cfg.leaf_size,
                                                                       cfg.range_spacing, cfg.angular_oversample]),
                    f"{name}_geom": geom, f"{name}_idx": idx, f"{name}_crop": crop, f"{name}_counts": cnt,
                    f"{name}_root": root})
        print(f"plan {name}: {plan.shape}, counts {plan.counts}", flush=True)
    pos = validate_track(512)
    plan = gb.build_ffbp_plan(pos, 1.4e9, (650, 1300, -0.5, 0.18), side=1, leaf_size=64, range_spacing=0.25,
                              angular_oversample=3.0)
    geom, idx, crop, cnt, root = flatten_plan(plan)
    out.update({"validate_position": pos, "validate_args": np.array([1.4e9, 650, 1300, -0.5, 0.18, 1, 64, 0.25, 3.0]),
                "validate_geom": geom, "validate_idx": idx, "validate_crop": crop, "validate_counts": cnt,
                "validate_root": root})
    # A left-looking, negative-carrier plan on the same track.
    plan = gb.build_ffbp_plan(pos * np.array([-1, 1, 1]), -1.4e9, (650, 1300, -0.5, 0.18), side=-1, leaf_size=32,
                              range_spacing=0.5, angular_oversample=2.0)
    geom, idx, crop, cnt, root = flatten_plan(plan)
    out.update({"left_position": pos * np.array([-1, 1, 1]),
                "left_args": np.array([-1.4e9, 650, 1300, -0.5, 0.18, -1, 32, 0.5, 2.0]),
                "left_geom": geom, "left_idx": idx, "left_crop": crop, "left_counts": cnt, "left_root": root})
    return out


def import_autofocus():
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    import autofocus  # noqa: E402
    return autofocus


def autofocus_case():
    sys.path.insert(0, str(HERE))
    import autofocus_scene as scene
    af = import_autofocus()
    out = {}
    for name in ("recovery", "cluttered"):
        s = getattr(scene, name)()
        delta, stats = af.estimate_update(s.data, s.pos, s.points, s.r_start, s.dr, s.k, s.prf, s.cutoff)
        before = float(np.sqrt(np.mean(s.err[:, :2] ** 2)))
        after = float(np.sqrt(np.mean((s.err + delta)[:, :2] ** 2)))
        out.update({f"{name}_delta": delta, f"{name}_coherence": stats["median_gradient_coherence"],
                    f"{name}_rmse": np.array([before, after]), f"{name}_data_probe": s.data[::97, ::31]})
        print(f"autofocus {name}: rmse {before:.4f} -> {after:.4f}, coherence "
              f"{stats['median_gradient_coherence']:.4f}", flush=True)
    p = scene.picks()
    result = types.SimpleNamespace(image=p.image, origin=p.origin, side=p.side,
                                   r=p.r0 + p.dr * np.arange(p.image.shape[0]),
                                   u=p.u0 + p.du * np.arange(p.image.shape[1]))
    for tiles in ((12, 12), (7, 5)):
        pts, powers = af.pick_targets(result, *tiles)
        out[f"picks_{tiles[0]}x{tiles[1]}_points"] = pts
        out[f"picks_{tiles[0]}x{tiles[1]}_powers"] = powers
        print(f"pick_targets {tiles}: {len(pts)} targets", flush=True)
    return out


def range_compress_inputs():
    """Seeded raw echoes for the range-compression golden case (rebuilt by the tests)."""
    rng = np.random.default_rng(1160)
    raw = (rng.standard_normal((6, 700)) + 1j * rng.standard_normal((6, 700))).astype(np.complex64)
    fs = 400e6
    t = (np.arange(700) - 311.7) / fs  # one chirp centred at a fractional sample, plus noise
    raw[2] += (3 * np.exp(-1j * np.pi * 200e6 / 1e-6 * t ** 2) * (np.abs(t) < 0.5e-6)).astype(np.complex64)
    return raw


def lfm_point_raw():
    """validate.py:55-56: one LFM echo centred at sample 1512.4 of 4000."""
    fs = 400e6
    tr = (np.arange(4000) - 1512.4) / fs
    return (np.exp(-1j * np.pi * 200e6 / 1e-6 * tr ** 2) * (np.abs(tr) < 0.5e-6)).astype(np.complex64)[None, :]


def range_compress_case(root):
    sys.path.insert(0, str(root / "fast_bp"))
    import sar_io  # noqa: E402
    raw = range_compress_inputs()
    out = {"os1": sar_io.range_compress(raw), "os2": sar_io.range_compress(raw, oversample=2),
           "os1_up": sar_io.range_compress(raw, chirp_sign=1, tp=0.8e-6, bandwidth=150e6)}
    lfm = sar_io.range_compress(lfm_point_raw(), oversample=4)
    out["lfm_peak"] = np.array(np.argmax(np.abs(lfm[0])) / 4)
    out["lfm_near_peak"] = lfm[0, 6000:6100]
    print(f"range_compress: lfm peak {float(out['lfm_peak']):.3f} (echo at 1512.4)", flush=True)
    return out


def capture_case(root):
    import tempfile
    sys.path.insert(0, str(root / "fast_bp"))
    sys.path.insert(0, str(HERE))
    import sar_io  # noqa: E402
    from capture_file import write_capture
    with tempfile.TemporaryDirectory() as tmp:
        cap = sar_io.Capture(write_capture(Path(tmp) / "capture.dat"))
        idx = np.array([0, 3, 4, 10, cap.n - 1])
        out = {"n": np.array(cap.n), "nr": np.array(cap.nr), "offset": np.array(cap.offset),
               "frame_size": np.array(cap.frame_size), "valid_indices": cap.valid_indices,
               "scalars": np.array([cap.tp, cap.delay, cap.prf, cap.bandwidth]), "time": cap.time,
               "read_idx": idx, "read": cap.read(idx)}
        for k, v in cap.nav.items():
            out["nav_" + k] = v
        out["summary"] = np.array([cap.summary[k] for k in ("complete_frame_slots", "valid_frames", "invalid_slots",
                                                             "first_pulse", "last_pulse", "missing_pulses",
                                                             "discarded_partial_bytes")])
    print(f"capture: {cap.n} valid frames of {cap.nr} samples", flush=True)
    return out


def metrics_cases():
    """Seeded inputs of the metrics golden case (rebuilt by the tests)."""
    rng = np.random.default_rng(515)
    img = (0.02 * (rng.standard_normal((96, 80)) + 1j * rng.standard_normal((96, 80)))).astype(np.complex64)
    img[40, 33] += 3.0
    img[10:14, 60:63] += 0.7j
    est = (img + 0.01 * (rng.standard_normal(img.shape) + 1j * rng.standard_normal(img.shape))
           * np.exp(0.05j)).astype(np.complex64)
    cuts = []
    for shift, width, window in ((0.0, 1.0, False), (0.37, 1.3, True), (-0.21, 0.8, False)):
        x = np.linspace(-12, 12, 481)
        z = np.sinc((x - shift) / width).astype(np.complex128)
        if window:
            z = z * (0.54 + 0.46 * np.cos(np.pi * np.clip((x - shift) / 12, -1, 1)))
        z = z + 1e-4 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
        cuts.append((x, z))
    return img, est, cuts


def metrics_case(root):
    np.trapz = np.trapezoid  # removed in numpy 2; the reference calls it
    sys.path.insert(0, str(root / "sar_quality"))
    import metrics as ref  # noqa: E402
    img, est, cuts = metrics_cases()
    out = {}
    fm = ref.focus_metrics(img)
    out["focus"] = np.array([fm["entropy_nats"], fm["normalized_entropy"], fm["intensity_contrast"],
                             fm["amplitude_contrast"], fm["brightest_1pct_energy_fraction"]])
    fd = ref.fidelity(img, est)
    out["fidelity"] = np.array([fd["relative_complex_error"], fd["ser_db"], fd["complex_coherence"],
                                fd["phase_bias_deg"], fd["phase_std_deg_above_minus30db"], fd["phase_mask_samples"]])
    for i, (x, z) in enumerate(cuts):
        m = ref.impulse_metrics(x, z)
        out[f"impulse{i}"] = np.array([m["irw_m"], m["peak_offset_m"], m["pslr_db"], m["islr_db"],
                                       *m["mainlobe_bounds_m"], *m["mainlobe_minima_db"]])
        print(f"impulse {i}: irw {m['irw_m']:.4f} pslr {m['pslr_db']:.2f} islr {m['islr_db']:.2f}", flush=True)
    return out


CASES = {
    "operator_validation": lambda ffbp, gb: operator_validation(ffbp, gb),
    "points": lambda ffbp, gb: points_case(ffbp),
    "kernels": lambda ffbp, gb: kernels_case(ffbp),
    "plans": lambda ffbp, gb: plans_case(gb),
    "autofocus": lambda ffbp, gb: autofocus_case(),
    "metrics": lambda ffbp, gb: metrics_case(ROOT_ARG[0]),
    "range_compress": lambda ffbp, gb: range_compress_case(ROOT_ARG[0]),
    "capture": lambda ffbp, gb: capture_case(ROOT_ARG[0]),
}
ROOT_ARG = [Path("/root/reference")]


def main():
    root = Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference")
    names = sys.argv[2:] or list(CASES)
    ROOT_ARG[0] = root
    ffbp, gb = import_reference(root)
    for name in names:
        np.savez_compressed(HERE / f"{name}.npz", **CASES[name](ffbp, gb))


if __name__ == "__main__":
    main()
