"""Nsight / ncu profiling target (counterpart of fast_bp/resident_profile_target.py).

Runs one named workload a few times on cuda:0 so that a profiler can capture
its kernels:

    python -m bp_project_gb300.profile_target --workload direct --config c1 --reps 2
    python -m bp_project_gb300.profile_target --workload ffbp   --config c1 --reps 2

Workloads: ``direct`` (split-precision direct BP on the scene's ground
lattice), ``polar`` (split-precision direct BP onto a 1024 x 4096 window of the
scene's FFBP root polar grid, the ``CudaBaseline.run_direct`` surface),
``ffbp`` (level-batched FFBP + split evaluation onto the lattice; ``--no-staging``: merge tiles
gather from the child images instead of staging their footprints by TMA),
``plain`` (the FP64-phase mixed kernel on a 64-row band of the lattice),
``adjoint`` (forward + adjoint of lattice BP, the entropy autofocus step),
``range`` (range compression of the scene's data treated as raw echoes),
``batch`` (a small uneven scene batch through the persistent kernels),
``all`` (every product kernel once on a small scene: direct BP in all modes on
lattice, polar grid and points, FFBP, evaluation, target contributions, the
LUT probe, adjoint, range compression, I/Q decode, phase-history filter).
Prints one JSON line with event timings (not for benchmarking under a
profiler: bench.py is the benchmark).

As in the reference's profiling target (fast_bp/resident_profile_target.py:83-99),
``--warmups`` runs untimed repetitions first, and the measured repetitions run
between cudaProfilerStart and cudaProfilerStop inside an NVTX range named
``sarbp_profile``, so that a profiler can capture only them
(``ncu --profile-from-start off`` or an NVTX filter).
"""
from __future__ import annotations

import argparse
import json

import torch

from . import build, core, scenes
from .gpu_backend import build_ffbp_plan


def _all_kernels(scene, data, pos, wt, ph, dev):
    """One call of every product kernel on the scene (small scenes keep this to tens of ms)."""
    import numpy as np

    from .autofocus import butter_lowpass, image_entropy, pick_targets, sosfiltfilt
    from .ffbp import PolarImage
    from .autograd import backproject_lattice
    from .sar_io import range_compress
    cfg, lat = scene.config, scene.lattice
    plan = build_ffbp_plan(scene.position, cfg.fc, scene.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    progs = {m: core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode=m, device=dev)
             for m in ("split", "mixed")}
    grid = plan.grid()
    from .ffbp import morton_order
    sample = lat.take(np.arange(0, lat.rows * lat.cols, 7))
    pts = torch.from_numpy(np.ascontiguousarray(sample[morton_order(sample)])).to(dev)  # as ffbp.backproject_points
    targets = torch.from_numpy(scene.targets).to(dev)
    lut = core.fill_range_phase_lut(data.shape[1], scene.range_start, scene.data_dr, scene.k, device=dev)
    frames = torch.zeros((64, 160 + 4 * data.shape[1] + 32), dtype=torch.uint8, device=dev)
    from . import _native as nat
    decoded = torch.empty((64, data.shape[1]), dtype=torch.complex64, device=dev)

    def run():
        for mode in ("split", "fp32", "mixed", "fp64"):
            rows = lat.rows if mode in ("split", "fp32") else 32
            core.backproject_lattice(data, pos, wt, ph, lat.origin, lat.step_row, lat.step_col, rows, lat.cols,
                                     scene.range_start, scene.data_dr, scene.k, mode=mode)
        small = core.Grid(grid.origin, grid.r0, grid.dr, min(grid.nr, 256), grid.u0, grid.du, min(grid.nu, 256),
                          grid.side)
        for mode in ("split", "mixed"):
            core.direct_polar(data, pos, wt, ph, small, scene.range_start, scene.data_dr, scene.k, mode=mode)
            core.backproject_points(data, pos, wt, ph, pts, scene.range_start, scene.data_dr, scene.k, mode=mode)
        core.direct_polar_lut(data, pos, wt, ph, small, scene.range_start, scene.data_dr, scene.k, lut)
        for m, prog in progs.items():
            polar = prog.execute(data, pos, wt, ph, scene.range_start, scene.data_dr, scene.k)
        core.evaluate_lattice(polar, grid, lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols, scene.k)
        pick_targets(PolarImage(polar, plan.origin.copy(), plan.r0, plan.dr, plan.u0, plan.du, 1))
        core.evaluate_image(polar, grid, pts, scene.k)
        contrib = core.target_contributions(data, pos, targets, scene.range_start, scene.data_dr, scene.k)
        sosfiltfilt(contrib, butter_lowpass(12.0, cfg.prf))
        p = pos.clone().requires_grad_()
        image_entropy(backproject_lattice(data, p, wt, ph, lat.origin, lat.step_row, lat.step_col, lat.rows,
                                          lat.cols, scene.range_start, scene.data_dr, scene.k)).backward()
        range_compress(data, tp=1e-6, bandwidth=cfg.bandwidth, fs=cfg.fs, oversample=2)
        nat.check(nat.load().sarbp_decode_iq(core._ptr(frames), 64, frames.shape[1], 160, data.shape[1],
                                             core._ptr(decoded), core.stream_handle()), "decode_iq")
    return run


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", choices=("direct", "polar", "ffbp", "plain", "adjoint", "range", "batch", "all"),
                    default="direct")
    ap.add_argument("--config", default="c1")
    ap.add_argument("--pulses", type=int, default=None, help="scale the scene to this many pulses")
    ap.add_argument("--side", type=int, default=None, help="scale the ground image to side x side pixels")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--mode", default="split")
    ap.add_argument("--warmups", type=int, default=0, help="untimed repetitions before the profiled range")
    ap.add_argument("--no-staging", action="store_true",
                    help="ffbp: merge tiles gather from the child images instead of staging their footprints by TMA")
    args = ap.parse_args(argv)
    build.build()
    torch.cuda.set_device(0)
    cfg = scenes.CONFIGS[args.config]
    if args.pulses or args.side:
        cfg = scenes.scaled(cfg, pulses=args.pulses, image_side=args.side)
    scene = scenes.synthesize(cfg, device="cuda")
    dev = torch.device("cuda", 0)
    data = torch.from_numpy(scene.data).to(dev)
    pos = torch.from_numpy(scene.position).to(dev)
    wt = torch.from_numpy(scene.weight).to(dev)
    ph = torch.from_numpy(scene.phase).to(dev)
    lat = scene.lattice
    torch.cuda.synchronize()
    times = []
    image_shape = [lat.rows, lat.cols]
    if args.workload in ("direct", "plain"):
        rows = lat.rows if args.workload == "direct" else 64
        out = torch.empty((rows, lat.cols), dtype=torch.complex64, device=dev)
        mode = args.mode if args.workload == "direct" else "mixed"

        def run():
            core.backproject_lattice(data, pos, wt, ph, lat.origin, lat.step_row, lat.step_col, rows, lat.cols,
                                     scene.range_start, scene.data_dr, scene.k, mode=mode, out=out)
        units = rows * lat.cols * cfg.pulses
    elif args.workload == "polar":
        plan = build_ffbp_plan(scene.position, cfg.fc, scene.extent, side=1, leaf_size=cfg.leaf_size,
                               range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
        g = plan.grid()
        nr, nu = min(1024, g.nr), min(4096, g.nu)
        r_off, u_off = (g.nr - nr) // 2, (g.nu - nu) // 2
        sub = core.Grid(g.origin, g.r0 + r_off * g.dr, g.dr, nr, g.u0 + u_off * g.du, g.du, nu, g.side)
        out = torch.empty((nr, nu), dtype=torch.complex64, device=dev)

        def run():
            core.direct_polar(data, pos, wt, ph, sub, scene.range_start, scene.data_dr, scene.k, mode=args.mode,
                              out=out)
        units = nr * nu * cfg.pulses
        image_shape = [nr, nu]
    elif args.workload == "all":
        run = _all_kernels(scene, data, pos, wt, ph, dev)
        units = lat.rows * lat.cols * cfg.pulses
    elif args.workload == "adjoint":
        from .autofocus import image_entropy
        from .autograd import backproject_lattice
        geo = (tuple(lat.origin), tuple(lat.step_row), tuple(lat.step_col), lat.rows, lat.cols, scene.range_start,
               scene.data_dr, scene.k)

        def run():
            p = pos.clone().requires_grad_()
            f = ph.clone().requires_grad_()
            image_entropy(backproject_lattice(data, p, wt, f, *geo)).backward()
        units = lat.rows * lat.cols * cfg.pulses
    elif args.workload == "range":
        from .sar_io import range_compress

        def run():
            range_compress(data, tp=1e-6, bandwidth=cfg.bandwidth, oversample=1, fs=cfg.fs)
        units = data.numel()
    elif args.workload == "batch":
        from .batch import DirectScene, FFBPScene, SceneBatch
        items = []
        for c, kind in scenes.batch_configs(count=8, seed=11, pulse_choices=(1024, 2048), side_choices=(512, 1024)):
            sc = scenes.synthesize(c, device="cuda")
            common = dict(data=torch.from_numpy(sc.data).to(dev), pos=torch.from_numpy(sc.position).to(dev),
                          weight=torch.from_numpy(sc.weight).to(dev), phase=torch.from_numpy(sc.phase).to(dev),
                          range_start=sc.range_start, data_dr=sc.data_dr, k=sc.k)
            if kind == "direct":
                L = sc.lattice
                items.append(DirectScene(**common, origin=tuple(L.origin), step_row=tuple(L.step_row),
                                         step_col=tuple(L.step_col), rows=L.rows, cols=L.cols))
            else:
                pl = build_ffbp_plan(sc.position, c.fc, sc.extent, side=1, leaf_size=c.leaf_size,
                                     range_spacing=c.range_spacing, angular_oversample=c.angular_oversample)
                items.append(FFBPScene(**common, plan=pl))
        batch = SceneBatch(items)

        def run():
            batch.execute()
        units = batch.info["pixel_pulses"]
    else:
        plan = build_ffbp_plan(scene.position, cfg.fc, scene.extent, side=1, leaf_size=cfg.leaf_size,
                               range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
        prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode=args.mode, device=dev,
                                staging=not args.no_staging)
        ground = torch.empty((lat.rows, lat.cols), dtype=torch.complex64, device=dev)
        grid = plan.grid()

        def run():
            polar = prog.execute(data, pos, wt, ph, scene.range_start, scene.data_dr, scene.k)
            core.evaluate_lattice(polar, grid, lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols, scene.k,
                                  out=ground)
        units = lat.rows * lat.cols * cfg.pulses
    for _ in range(args.warmups):
        run()
    torch.cuda.synchronize()
    torch.cuda.profiler.start()  # cudaProfilerStart: the capture range of --profile-from-start off
    nvtx = True
    try:
        torch.cuda.nvtx.range_push("sarbp_profile")
    except (AttributeError, RuntimeError):  # torch built without NVTX: the profiler API range remains
        nvtx = False
    try:
        for _ in range(args.reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            run()
            b.record()
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
    finally:
        if nvtx:
            torch.cuda.nvtx.range_pop()
        torch.cuda.profiler.stop()
    print(json.dumps({"workload": args.workload, "config": cfg.name, "pulses": cfg.pulses,
                      "image": image_shape, "mode": args.mode, "ms": times,
                      "gpix_pulse_per_s": [units / (t / 1e3) / 1e9 for t in times]}), flush=True)


if __name__ == "__main__":
    main()
