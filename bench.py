"""Benchmark: direct BP throughput (Gpixel*pulses/s) on the 4096-pulse / 2048^2 scene, plus FFBP img/s.

Workload (one "step"): split-precision direct back-projection of 4096 pulses x
8192 range bins (complex64, 268 MB, larger than L2) onto a 2048 x 2048 ground
lattice at 0.5 m, fc 9.6 GHz, 150 MHz, 4 km near slant range; seeded
synthetic scene (25 point targets over clutter scatterers).  Also reported:
FFBP on the same scene (leaves of 16 pulses, 8 merge levels) in images/s,
errors against the FP64 oracle, the plain FP64-phase kernel on the same
pixels, the CPU oracle on a bounded pixel sample, and the roofline of the
dominant kernel.  The same line carries, each with the clocks sampled while it
ran:

* ``c2_direct``: split direct BP on the 30 km precision-stress scene (8192
  pulses x 16384 bins -> 4096^2 lattice at 0.25 m) and its sampled error vs FP64;
* ``autofocus``: on the 2048-pulse / 1024^2 scene with navigation errors, the
  reference's phase-gradient autofocus on the CPU oracle (its seconds and the
  entropy it reaches), the GPU port of that loop, and the gradient entropy
  autofocus's wall time to the same entropy, for a rough and a smooth error model;
* ``batch``: 64 uneven scenes as one CUDA graph against the same scenes formed
  one at a time (ms per graph, speed-up, per-scene latency spread).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --workload autofocus     # autofocus wall time on the 2048-pulse scene
    python bench.py --workload batch         # 64 uneven scenes, persistent kernels, one CUDA graph

For N > 1 run under torch.distributed.run: every rank images its own copy of
the scene (weak scaling, no data-path collective); the timed region is
bracketed by barriers and the maximum over ranks is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "BP Gpixel·pulses/s and FFBP img/s at stated err vs FP64; autofocus iters/s"
UNIT = "Gpixel·pulses/s"
WORKLOAD = "c1 direct BP: 4096 pulses x 8192 bins -> 2048x2048 ground lattice @0.5 m, 9.6 GHz, split precision"
FP32_FLOPS_PER_PX_PULSE = 54.0      # algorithmic FP32 work per pixel-pulse (FMA = 2)
MUFU_PER_PX_PULSE = 3.0
CPU_SAMPLE_PIXELS = 1 << 20         # bounded CPU-baseline sample (all 4096 pulses): ~10 s on 16 cores
REF_SAMPLE_PIXELS = 131072          # pixels per step of the reference arm (~1 s on 16 cores)
# DRAM bytes (read + write) of one split_lattice_kernel launch on this workload, from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum): only the ~920 range bins per pulse that the scene spans
# are read, so traffic is far below the algorithmic 302 MB.
NCU_TRAFFIC_BYTES = 32.980992e6 + 83.194880e6  # 4 pulse splits: the partial images are written
L2_FLUSH_BYTES = 256 << 20          # written between timed steps: twice GB300's 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--config", default="c1")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ffbp", action="store_true")
    ap.add_argument("--no-autofocus", action="store_true")
    ap.add_argument("--no-c2", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--workload", choices=("direct", "autofocus", "batch"), default="direct")
    ap.add_argument("--scenes", type=int, default=64)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


class Clocks:
    """Sample nvidia-smi clocks and throttle reasons while the timed region runs."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return False
        time.sleep(0.15)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)
        return False

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        return json.loads(path.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def cpu_baseline(scene, pixels, seed=11):
    """FP64 oracle (C++/OpenMP restatement of the reference's Numba BP) on a bounded pixel sample."""
    from oracle import reference as ora
    threads = ora.set_threads(0)
    rng = np.random.default_rng(seed)
    idx = rng.choice(scene.lattice.rows * scene.lattice.cols, pixels, replace=False)
    pts = scene.lattice.take(idx)
    t0 = time.perf_counter()
    out = ora.backproject_points(scene.data, scene.position, pts, scene.range_start, scene.data_dr, scene.k,
                                 scene.weight, scene.phase, c128=True)[1]
    dt = time.perf_counter() - t0
    return {"value": pixels * scene.config.pulses / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "seconds": dt,
            "sample": f"{pixels} random pixels of the 2048^2 lattice x all {scene.config.pulses} pulses "
                      f"(FP64 C++/OpenMP restatement of ffbp.backproject_points)"}, idx, out


def replica_rate(total_ms, units, steps, world, dist=None, device=None):
    """Whole-job rate of ``world`` independent replicas: the slowest rank's timed total (max over
    ranks, so every rank returns the same) and all ranks' units.  Returns (total_ms, Gunits/s)."""
    if world > 1:
        import torch
        t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, world * units * steps / (total_ms / 1e3) / 1e9


def run_reference(args, rank):
    """Reference arm: the reference's CPU BP (restated, FP64, all host threads) on a bounded sample per step."""
    if rank != 0:
        return
    from bp_project_gb300 import scenes
    from oracle import build as oracle_build
    from oracle import reference as ora
    oracle_build.build()
    scene = scenes.synthesize(scenes.CONFIGS[args.config])
    threads = ora.set_threads(0)
    rng = np.random.default_rng(5)
    npix = scene.lattice.rows * scene.lattice.cols
    times = []
    for step in range(args.warmup + args.steps):
        pts = scene.lattice.take(rng.choice(npix, REF_SAMPLE_PIXELS, replace=False))
        t0 = time.perf_counter()
        ora.backproject_points(scene.data, scene.position, pts, scene.range_start, scene.data_dr, scene.k,
                               scene.weight, scene.phase)
        if step >= args.warmup:
            times.append(time.perf_counter() - t0)
    per_step = statistics.mean(times)
    value = REF_SAMPLE_PIXELS * scene.config.pulses / per_step / 1e9
    sample = (f"{REF_SAMPLE_PIXELS} random pixels of the 2048^2 lattice x all {scene.config.pulses} pulses per step "
              f"(FP64 C++/OpenMP restatement of ffbp.backproject_points; the reference's Numba path cannot run here)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD.replace("split precision", "FP64 CPU"), "pulses": scene.config.pulses,
                       "samples": scene.config.samples, "image": [scene.lattice.rows, scene.lattice.cols],
                       "sample_pixels_per_step": REF_SAMPLE_PIXELS},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def autofocus_scene(device, walk_sigma=1e-3):
    """The 2048-pulse / 1024^2 scene with navigation errors: the data are formed on the true
    track and carry a per-pulse phase error; imaging starts from the perturbed track, phase 0."""
    from scipy.signal.windows import hann

    from bp_project_gb300 import scenes
    cfg = scenes.CONFIGS["c3"]
    sc = scenes.synthesize(cfg, device=device)
    err, phase_err = scenes.inject_trajectory_error(sc, walk_sigma=walk_sigma)
    data = (sc.data * np.exp(-1j * phase_err)[:, None].astype(np.complex64)).astype(np.complex64)
    return sc, data, sc.position + err, hann(cfg.pulses), np.zeros(cfg.pulses)


def autofocus_case(dev, walk_sigma):
    """Reference PGA (CPU oracle) vs its GPU port vs the gradient entropy autofocus on one error model."""
    import torch

    from bp_project_gb300.autofocus import entropy_autofocus, image_entropy, phase_gradient_autofocus
    from bp_project_gb300.autograd import backproject_lattice
    from oracle import autofocus as oaf
    from oracle import reference as ora
    sc, data, nav, weight, phase = autofocus_scene(str(dev), walk_sigma)
    cfg, lat = sc.config, sc.lattice
    geo = (tuple(lat.origin), tuple(lat.step_row), tuple(lat.step_col), lat.rows, lat.cols, sc.range_start,
           sc.data_dr, sc.k)
    d = torch.from_numpy(data).to(dev)
    w = torch.from_numpy(weight).to(dev)
    ph = torch.from_numpy(phase).to(dev)
    nav_t = torch.from_numpy(nav).to(dev)

    def entropy(pos):
        with torch.no_grad():
            return float(image_entropy(backproject_lattice(d, torch.as_tensor(pos).to(dev), w, ph, *geo)))

    pga_args = dict(side=1, leaf_size=64, range_spacing=0.5, angular_oversample=2.0, weight=weight)
    threads = ora.set_threads(0)
    t0 = time.perf_counter()
    ref_pos, ref_records = oaf.phase_gradient_autofocus(data, nav, sc.range_start, sc.data_dr, cfg.fc, sc.extent,
                                                        cfg.prf, **pga_args)
    ref_s = time.perf_counter() - t0
    e_ref = entropy(ref_pos)

    phase_gradient_autofocus(d, nav_t, sc.range_start, sc.data_dr, cfg.fc, sc.extent, cfg.prf, cutoffs=(12,),
                             **pga_args)  # warm-up
    entropy_autofocus(d, nav_t, w, ph, *geo, steps=2)  # warm-up
    torch.cuda.synchronize()
    with Clocks(dev.index or 0) as clocks:
        t0 = time.perf_counter()
        gpu_pos, gpu_records = phase_gradient_autofocus(d, nav_t, sc.range_start, sc.data_dr, cfg.fc, sc.extent,
                                                        cfg.prf, **pga_args)
        torch.cuda.synchronize()
        gpu_pga_s = time.perf_counter() - t0
        to_target = entropy_autofocus(d, nav_t, w, ph, *geo, steps=500, target_entropy=e_ref, time_limit=120)
        t_target = to_target.history[-1][0]
        full = entropy_autofocus(d, nav_t, w, ph, *geo, steps=100)
    e_gpu_pga = entropy(gpu_pos)
    return {
        "errors": f"2 cm LOS sinusoid (3 periods), {walk_sigma * 1e3:g} mm/pulse random walk (detrended), "
                  f"3*pi quadratic phase in the data",
        "reference_pga_cpu": {"seconds": ref_s, "iterations": len(ref_records), "threads": threads,
                              "entropy": e_ref, "kind": "port",
                              "what": "oracle FFBP (C++/OpenMP) + numpy/scipy estimate_update, autofocus.py loop"},
        "gpu_pga": {"seconds": gpu_pga_s, "iterations": len(gpu_records),
                    "iters_per_s": len(gpu_records) / gpu_pga_s, "entropy": e_gpu_pga},
        "entropy_autofocus": {"seconds_to_reference_entropy": t_target, "reached": to_target.entropy <= e_ref,
                              "evaluations": to_target.evaluations, "final_entropy_100_steps": full.entropy,
                              "final_evaluations": full.evaluations, "final_seconds": full.history[-1][0]},
        "entropies": {"initial": entropy(nav), "true_track": entropy(sc.position), "reference_pga": e_ref,
                      "gpu_pga": e_gpu_pga, "entropy_autofocus": full.entropy},
        "speedup_vs_reference_pga": ref_s / t_target,
        "speedup_vs_gpu_pga": gpu_pga_s / t_target,
        "clocks": clocks.summary(),
    }


def autofocus_wall(dev):
    """Wall time of the gradient entropy autofocus to the entropy that the reference's phase-gradient
    autofocus reaches (CPU oracle, all host threads), beside the GPU port of that loop, for the full
    error model (with the 1 mm/pulse random walk) and a smooth one (without it)."""
    rough = autofocus_case(dev, 1e-3)
    smooth = autofocus_case(dev, 0.0)
    return {
        "pga_iters_per_s": rough["gpu_pga"]["iters_per_s"],
        "entropy_evals_per_s": rough["entropy_autofocus"]["final_evaluations"]
        / rough["entropy_autofocus"]["final_seconds"],
        "seconds_to_reference_entropy": {"rough": rough["entropy_autofocus"]["seconds_to_reference_entropy"],
                                         "smooth": smooth["entropy_autofocus"]["seconds_to_reference_entropy"]},
        "workload": "2048 pulses x 4096 bins, 1024^2 lattice @0.5 m, 16 targets + 1024 clutter; PGA: FFBP (leaf "
                    "64) + 12x12 target picks + estimate_update per iteration; entropy: forward + adjoint BP per "
                    "L-BFGS evaluation",
        "rough": rough, "smooth": smooth,
    }


def c2_direct(dev, steps, warmup, sample_pixels=16384, seed=13):
    """Split direct BP on the 30 km precision-stress scene (8192 pulses x 16384 bins -> 4096^2 lattice at
    0.25 m): throughput with a flushed L2 before every step, and the error against the FP64 oracle on a
    random pixel sample."""
    import torch

    from bp_project_gb300 import core, scenes
    from oracle import reference as ora
    cfg = scenes.CONFIGS["c2"]
    t0 = time.perf_counter()
    sc = scenes.synthesize(cfg, device=str(dev))
    synth_s = time.perf_counter() - t0
    lat = sc.lattice
    data = torch.from_numpy(sc.data).to(dev)
    pos, wt, ph = (torch.from_numpy(a).to(dev) for a in (sc.position, sc.weight, sc.phase))
    out = torch.empty((lat.rows, lat.cols), dtype=torch.complex64, device=dev)

    def step():
        core.backproject_lattice(data, pos, wt, ph, lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols,
                                 sc.range_start, sc.data_dr, sc.k, mode="split", out=out)

    for _ in range(max(warmup, 3)):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    with Clocks(dev.index or 0) as clocks:
        for i in range(steps):
            flush.zero_()
            ev0[i].record(stream)
            step()
            ev1[i].record(stream)
        torch.cuda.synchronize()
    ms = statistics.mean(ev0[i].elapsed_time(ev1[i]) for i in range(steps))
    npix = lat.rows * lat.cols
    rng = np.random.default_rng(seed)
    idx = rng.choice(npix, sample_pixels, replace=False)
    ref = ora.backproject_points(sc.data, sc.position, lat.take(idx), sc.range_start, sc.data_dr, sc.k, sc.weight,
                                 sc.phase, c128=True)[1]
    est = out.reshape(-1)[torch.from_numpy(idx).to(dev)].cpu().numpy().astype(np.complex128)
    return {"gpix_pulse_s": npix * cfg.pulses / (ms / 1e3) / 1e9, "ms": ms, "steps": steps,
            "err_vs_fp64": float(np.linalg.norm(est - ref) / np.linalg.norm(ref)),
            "err_sample": f"{sample_pixels} random pixels x all {cfg.pulses} pulses, complex L2 vs the FP64 oracle",
            "pulse_split": core.lattice_pulse_split(lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols,
                                                    "split"),
            "workload": "c2 direct BP: 8192 pulses x 16384 bins -> 4096x4096 ground lattice @0.25 m, 10 GHz, "
                        "300 MHz, 30 km near slant, split precision; L2 flushed before every step",
            "synthesis_s": synth_s, "clocks": clocks.summary()}


def run_autofocus(args, rank):
    """Autofocus on the 2048-pulse scene: wall time of the gradient entropy autofocus to reach the entropy
    that the reference's phase-gradient autofocus (6 iterations, CPU oracle, all host threads) reaches,
    for the full error model and for a smooth one (no random walk) that the phase-gradient method can follow."""
    if rank != 0:
        return
    import torch

    from bp_project_gb300 import build
    from oracle import build as oracle_build
    build.build()
    oracle_build.build()
    dev = torch.device("cuda", 0)
    rough = autofocus_case(dev, 1e-3)
    smooth = autofocus_case(dev, 0.0)
    line = {
        "metric": "autofocus wall time to the reference autofocus's entropy", "value":
        rough["entropy_autofocus"]["seconds_to_reference_entropy"], "unit": "s", "higher_is_better": False,
        "n_gpus": 1, "data": "synthetic", "dtype": "f32 (split precision BP)",
        "config": {"workload": "c3 autofocus: 2048 pulses x 4096 bins, 1024^2 lattice @0.5 m, 16 targets + 1024 "
                               "clutter; entropy of the split direct BP image with Hann weights",
                   "errors": rough["errors"]},
        **rough,
        "smooth_errors": smooth,
    }
    print(json.dumps(line), flush=True)


def batch_measure(dev, scenes_count, steps, warmup, pulse_choices=None, side_choices=(256, 512, 1024, 2048),
                  tune=True):
    """Independent scenes of uneven size (half direct BP, half FFBP) as one CUDA graph of
    persistent work-queue launches, tile shapes from the autotuner (``tune``); against the same
    scenes formed one at a time through the single-scene entry points.  Returns the measurement
    dict.  The defaults are the 64-scene workload: pulses U{512..8192}, sides U{256..2048}."""
    import torch

    from bp_project_gb300 import autotune, core, scenes
    from bp_project_gb300.batch import DirectScene, FFBPScene, SceneBatch
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    t0 = time.perf_counter()
    cfgs = scenes.batch_configs(count=scenes_count, pulse_choices=pulse_choices, side_choices=side_choices)
    items = []
    for cfg, kind in cfgs:
        sc = scenes.synthesize(cfg, device=str(dev))
        common = dict(data=torch.from_numpy(sc.data).to(dev), pos=torch.from_numpy(sc.position).to(dev),
                      weight=torch.from_numpy(sc.weight).to(dev), phase=torch.from_numpy(sc.phase).to(dev),
                      range_start=sc.range_start, data_dr=sc.data_dr, k=sc.k)
        if kind == "direct":
            lat = sc.lattice
            items.append(DirectScene(**common, origin=tuple(lat.origin), step_row=tuple(lat.step_row),
                                     step_col=tuple(lat.step_col), rows=lat.rows, cols=lat.cols))
        else:
            plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                                   range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
            items.append(FFBPScene(**common, plan=plan))
    synth_s = time.perf_counter() - t0

    # Autotune the tile x chunk shape per image side on a 1024-pulse slice of one scene of that side.
    t0 = time.perf_counter()
    choices = {}
    for sc in items:
        side = max(getattr(sc, "rows", 0), getattr(sc, "cols", 0))
        if tune and isinstance(sc, DirectScene) and side not in choices:
            n = min(1024, sc.data.shape[0])
            rep = DirectScene(**{**sc.__dict__, "data": sc.data[:n].contiguous(), "pos": sc.pos[:n].contiguous(),
                                 "weight": sc.weight[:n].contiguous(), "phase": sc.phase[:n].contiguous(),
                                 "out": None})
            choices[side], _ = autotune.tune_direct(rep, cache=None, reps=2)
    tune_s = time.perf_counter() - t0
    default_ref = {}
    for i, sc in enumerate(items):  # single-scene results before the tuned shapes are applied
        if isinstance(sc, DirectScene) and i < 8:
            default_ref[i] = core.backproject_lattice(sc.data, sc.pos, sc.weight, sc.phase, sc.origin, sc.step_row,
                                                      sc.step_col, sc.rows, sc.cols, sc.range_start, sc.data_dr,
                                                      sc.k, mode="split", pulse_split=1)
    if tune:
        autotune.apply(items, choices)
        (blocks, concurrent), block_timings = autotune.tune_blocks(items)
    else:
        (blocks, concurrent), block_timings = (0, False), {}

    batch = SceneBatch(items, blocks_per_sm=blocks, concurrent=concurrent)
    graph = batch.capture_graph()
    for _ in range(max(warmup, 3) - 1):
        batch.replay()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clocks:
        e0.record(stream)
        for _ in range(steps):
            batch.replay()
        e1.record(stream)
        torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1) / steps

    # The same scenes one at a time (single-scene entry points, default shapes), one pass.
    progs = [core.FFBPProgram(sc.plan.nodes(), sc.plan.crop_r, sc.plan.crop_u, mode="split", device=dev)
             if isinstance(sc, FFBPScene) else None for sc in items]

    def sequential():
        for sc, prog in zip(items, progs):
            if prog is None:
                core.backproject_lattice(sc.data, sc.pos, sc.weight, sc.phase, sc.origin, sc.step_row, sc.step_col,
                                         sc.rows, sc.cols, sc.range_start, sc.data_dr, sc.k, mode="split")
            else:
                prog.execute(sc.data, sc.pos, sc.weight, sc.phase, sc.range_start, sc.data_dr, sc.k)

    sequential()
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev.index or 0) as seq_clocks:
        s0.record(stream)
        sequential()
        s1.record(stream)
        torch.cuda.synchronize()
    seq_ms = s0.elapsed_time(s1)
    errs = [float((items[i].out - r).abs().norm() / r.abs().norm()) for i, r in default_ref.items()]
    for p in progs:
        if p is not None:
            p.close()
    px = batch.info["pixel_pulses"]
    direct_px = sum(sc.rows * sc.cols * sc.data.shape[0] for sc in items if isinstance(sc, DirectScene))
    lat_ms = batch.scene_latencies_ms()  # one traced execution, outside the timed replays
    kinds = ["direct" if isinstance(sc, DirectScene) else "ffbp" for sc in items]

    def spread(v):
        v = np.sort(np.asarray(v, dtype=np.float64))
        if not len(v):
            return None
        return {"min": float(v[0]), "median": float(np.median(v)), "p90": float(np.quantile(v, 0.9)),
                "max": float(v[-1])}
    line = {
        "metric": "batched scenes: Gpixel·pulses/s (direct-equivalent) and scenes/s", "value": px / (batch_ms / 1e3) / 1e9,
        "unit": "Gpixel·pulses/s", "higher_is_better": True, "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": batch_ms, "data": "synthetic", "dtype": "f32 (split precision)",
        "config": {"workload": f"{len(items)} scenes: pulses U{{{','.join(str(int(p)) for p in pulse_choices) if pulse_choices is not None else '512..8192 step 512'}}}, "
                               f"side U{{{','.join(str(v) for v in side_choices)}}} "
                               "@0.5 m, half direct BP / half FFBP (leaf 16), near slant U(3.5, 8) km, 4-16 "
                               "targets + 256 clutter, 9.6 GHz / 150 MHz",
                   "scenes": len(items), "direct_pixel_pulses": direct_px, "all_pixel_pulses": px,
                   "l2": "inputs far larger than L2 (%.1f GB of range data)" % (
                       sum(sc.data.numel() * 8 for sc in items) / 1e9)},
        "scenes_per_s": len(items) / (batch_ms / 1e3),
        "graph": "one CUDA graph per batch: %d launches (memset, 3 FFBP prologues, persistent direct and leaf launches, %d persistent "
                 "merge levels)%s" % (batch.launch_count, batch.info["max_height"],
                                      "; the FFBP chain on a forked branch beside the direct queue" if concurrent
                                      else ""),
        "batch_info": batch.info, "autotune": {str(k): list(v) for k, v in choices.items()},
        "autotune_blocks_per_sm": {"chosen": blocks, "concurrent": concurrent, "ms": block_timings},
        "autotune_s": tune_s, "synthesis_s": synth_s,
        "sequential_ms": seq_ms, "speedup_vs_sequential": seq_ms / batch_ms,
        "sequential_clocks": seq_clocks.summary(),
        "scene_latency_ms": {"all": spread(lat_ms),
                             "direct": spread([t for t, k in zip(lat_ms, kinds) if k == "direct"]),
                             "ffbp": spread([t for t, k in zip(lat_ms, kinds) if k == "ffbp"]),
                             "how": "completion of each scene's last work item from the batch's start (GPU "
                                    "nanosecond timer), one traced execution"},
        "tuned_vs_default_shape_err_max": max(errs) if errs else None,
        "workspace_gb": batch.workspace_bytes / 1e9,
        "clocks": clocks.summary(),
        # graph replays bypass the C ABI's launch counter: count the graph's kernel nodes
        "gpu_launches": steps * (batch.launch_count - 1),
    }
    batch.close()
    return line


def run_batch(args, rank):
    """The batch workload alone, as its own JSON line."""
    if rank != 0:
        return
    import torch

    from bp_project_gb300 import build
    build.build()
    print(json.dumps(batch_measure(torch.device("cuda", 0), args.scenes, args.steps, args.warmup)), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload == "batch":
        run_batch(args, rank)
        return
    if args.workload == "autofocus":
        run_autofocus(args, rank)
        return
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import torch
    import torch.distributed as dist

    from bp_project_gb300 import _native, build, core, scenes
    from bp_project_gb300.gpu_backend import build_ffbp_plan

    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    cfg = scenes.CONFIGS[args.config]
    scene = scenes.synthesize(cfg, device=str(dev))
    lat = scene.lattice
    npix = lat.rows * lat.cols
    units = npix * cfg.pulses

    data = torch.from_numpy(scene.data).to(dev)
    pos = torch.from_numpy(scene.position).to(dev)
    wt = torch.from_numpy(scene.weight).to(dev)
    ph = torch.from_numpy(scene.phase).to(dev)
    out = torch.empty((lat.rows, lat.cols), dtype=torch.complex64, device=dev)

    def step():
        core.backproject_lattice(data, pos, wt, ph, lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols,
                                 scene.range_start, scene.data_dr, scene.k, mode="split", out=out)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    stream = torch.cuda.current_stream()
    # The range windows a launch touches (~32 MB) and the image (33.5 MB) would fit the 129 MB L2, so
    # every timed step starts from a flushed L2: a 256 MB write between steps, outside its events.
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = _native.launch_count()
    with Clocks(local) as clocks:
        for i in range(args.steps):
            flush.zero_()
            ev0[i].record(stream)
            step()
            ev1[i].record(stream)
        barrier()
    launches = _native.launch_count() - launches0
    per_launch_ms = [ev0[i].elapsed_time(ev1[i]) for i in range(args.steps)]
    total_ms, value = replica_rate(sum(per_launch_ms), units, args.steps, world, dist, dev)
    ms_per_step = total_ms / args.steps
    image = out.cpu().numpy()

    # End to end through the public API: every step copies its inputs from pinned host memory to the
    # device, forms the image (core.backproject_lattice, the C ABI) and reads the image back to the host.
    # Two buffer sets and one stream per copy direction: step i+1's upload and step i-1's read-back
    # overlap step i's BP.
    host_data = torch.from_numpy(scene.data).pin_memory()
    host_pos = torch.from_numpy(scene.position).pin_memory()
    host_w = torch.from_numpy(scene.weight).pin_memory()
    host_ph = torch.from_numpy(scene.phase).pin_memory()
    host_outs = [torch.empty((lat.rows, lat.cols), dtype=torch.complex64).pin_memory() for _ in range(2)]
    bufs = [[torch.empty_like(t, device=dev) for t in (host_data, host_pos, host_w, host_ph)] for _ in range(2)]
    outs = [torch.empty((lat.rows, lat.cols), dtype=torch.complex64, device=dev) for _ in range(2)]
    up_stream, down_stream = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
    loaded = [torch.cuda.Event() for _ in range(2)]
    formed = [torch.cuda.Event() for _ in range(2)]
    freed = [torch.cuda.Event() for _ in range(2)]
    for ev_ in freed:
        ev_.record(stream)

    def e2e_step(i):
        b = i % 2
        with torch.cuda.stream(up_stream):
            up_stream.wait_event(freed[b])  # step i-2 has finished with buffer set b
            for d, h in zip(bufs[b], (host_data, host_pos, host_w, host_ph)):
                d.copy_(h, non_blocking=True)
            loaded[b].record(up_stream)
        stream.wait_event(loaded[b])
        core.backproject_lattice(*bufs[b], lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols,
                                 scene.range_start, scene.data_dr, scene.k, mode="split", out=outs[b])
        formed[b].record(stream)
        with torch.cuda.stream(down_stream):
            down_stream.wait_event(formed[b])
            host_outs[b].copy_(outs[b], non_blocking=True)
            freed[b].record(down_stream)

    for i in range(2):
        e2e_step(i)
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    up_stream.wait_event(e0)
    down_stream.wait_event(e0)
    for i in range(args.steps):
        e2e_step(i)
    stream.wait_stream(up_stream)
    stream.wait_stream(down_stream)  # the last image is back on the host
    e1.record(stream)
    barrier()
    e2e_total, e2e_value = replica_rate(e0.elapsed_time(e1), units, args.steps, world, dist, dev)
    e2e_ms = e2e_total / args.steps
    host_out = host_outs[0]
    h2d = sum(t.numel() * t.element_size() for t in (host_data, host_pos, host_w, host_ph))
    d2h = host_out.numel() * host_out.element_size()

    extra = {}
    if rank == 0:
        # Plain FP64-phase kernel (the reference's mixed policy) on the same lattice, one timed pass.
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        mixed_out = torch.empty_like(out)
        rows_m = 256  # a 256-row band keeps the slow FP64 kernel to ~a second
        origin_m = lat.origin
        s0.record(stream)
        core.backproject_lattice(data, pos, wt, ph, origin_m, lat.step_row, lat.step_col, rows_m, lat.cols,
                                 scene.range_start, scene.data_dr, scene.k, mode="mixed", out=mixed_out[:rows_m])
        s1.record(stream)
        torch.cuda.synchronize()
        mixed_rate = rows_m * lat.cols * cfg.pulses / (s0.elapsed_time(s1) / 1e3) / 1e9
        extra["plain_fp64_phase_gpix_pulse_s"] = mixed_rate
        extra["split_over_plain_fp64_phase"] = value / world / mixed_rate
        band = image[:rows_m].astype(np.complex128)
        extra["split_vs_plain_fp64_phase_err"] = float(np.linalg.norm(band - mixed_out[:rows_m].cpu().numpy())
                                                       / np.linalg.norm(band))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import build as oracle_build
        oracle_build.build()
        cpu, idx, ref = cpu_baseline(scene, CPU_SAMPLE_PIXELS)
        est = image.ravel()[idx].astype(np.complex128)
        extra["err_vs_fp64"] = float(np.linalg.norm(est - ref) / np.linalg.norm(ref))
        extra["err_vs_fp64_sample"] = f"{CPU_SAMPLE_PIXELS} random pixels, complex L2"

    if rank == 0 and not args.no_ffbp:
        ext = scene.extent
        plan = build_ffbp_plan(scene.position, cfg.fc, ext, side=1, leaf_size=cfg.leaf_size,
                               range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
        prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split", device=dev)
        grid = plan.grid()
        ground = torch.empty((lat.rows, lat.cols), dtype=torch.complex64, device=dev)

        def ffbp_step():
            polar = prog.execute(data, pos, wt, ph, scene.range_start, scene.data_dr, scene.k)
            core.evaluate_lattice(polar, grid, lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols, scene.k,
                                  out=ground)
            return polar

        for _ in range(2):
            ffbp_step()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nrep = max(3, args.steps // 2)
        f0.record(stream)
        for _ in range(nrep):
            ffbp_step()
        f1.record(stream)
        torch.cuda.synchronize()
        ffbp_ms = f0.elapsed_time(f1) / nrep
        g = ground.cpu().numpy().reshape(lat.rows, lat.cols).astype(np.complex128)
        # Direct BP onto the FFBP root's polar grid: the surface of the reference's CudaBaseline.run_direct
        # (split precision, one pulse pass per tile), and the FFBP image against it on that grid.
        polar_direct = torch.empty((grid.nr, grid.nu), dtype=torch.complex64, device=dev)

        def polar_step():
            return core.direct_polar(data, pos, wt, ph, grid, scene.range_start, scene.data_dr, scene.k, mode="split",
                                     out=polar_direct)

        polar_step()
        torch.cuda.synchronize()
        f0.record(stream)
        for _ in range(2):
            polar_step()
        f1.record(stream)
        torch.cuda.synchronize()
        polar_ms = f0.elapsed_time(f1) / 2
        polar_ffbp = ffbp_step()
        torch.cuda.synchronize()
        diff = (polar_ffbp.to(torch.complex128) - polar_direct.to(torch.complex128)).abs().pow(2).sum()
        norm = polar_direct.to(torch.complex128).abs().pow(2).sum()
        extra["polar_direct"] = {
            "gpix_pulse_s": grid.nr * grid.nu * cfg.pulses / (polar_ms / 1e3) / 1e9, "ms": polar_ms,
            "grid": [grid.nr, grid.nu], "pulses": cfg.pulses,
            "ffbp_vs_direct_err_polar": float(torch.sqrt(diff / norm)),
            "what": "core.direct_polar (sarbp_direct_polar, the CudaBaseline.run_direct path) onto the FFBP root's "
                    "cropped polar grid, split precision, one pulse pass per tile"}
        del polar_direct, polar_ffbp
        extra.update({
            "ffbp_img_per_s": 1e3 / ffbp_ms, "ffbp_ms": ffbp_ms,
            "ffbp_config": f"leaf {cfg.leaf_size}, {plan.counts['leaves']} leaves, {plan.counts['merges']} merges, "
                           f"root polar {plan.nr}x{plan.nu}, range spacing {cfg.range_spacing} m, angular oversample "
                           f"{cfg.angular_oversample}; polar FFBP + split evaluate onto the 2048^2 lattice",
            "ffbp_launches": prog.launch_count + 1,
            "ffbp_vs_direct_err": float(np.linalg.norm(g - image) / np.linalg.norm(image)),
        })
        prog.close()

    if rank == 0 and not args.no_c2:
        from oracle import build as oracle_build
        oracle_build.build()
        extra["c2_direct"] = c2_direct(dev, steps=min(args.steps, 5), warmup=args.warmup)

    if rank == 0 and not args.no_autofocus:
        from oracle import build as oracle_build
        oracle_build.build()
        extra["autofocus"] = autofocus_wall(dev)

    if rank == 0 and not args.no_batch:
        b = batch_measure(dev, args.scenes, steps=min(args.steps, 5), warmup=args.warmup)
        keep = ("value", "unit", "ms_per_step", "steps", "scenes_per_s", "sequential_ms", "speedup_vs_sequential",
                "scene_latency_ms", "graph", "gpu_launches", "clocks", "sequential_clocks",
                "tuned_vs_default_shape_err_max", "autotune", "autotune_blocks_per_sm", "autotune_s", "synthesis_s")
        extra["batch"] = {"workload": b["config"]["workload"], **{k_: b[k_] for k_ in keep}}
        # Many small scenes, where one-at-a-time forming leaves the GPU idle between short launches.
        b = batch_measure(dev, 256, steps=min(args.steps, 5), warmup=args.warmup, pulse_choices=(512, 1024),
                          side_choices=(256, 512), tune=False)
        extra["batch_small"] = {"workload": b["config"]["workload"],
                                **{k_: b[k_] for k_ in keep if k_ not in ("autotune", "autotune_blocks_per_sm")}}

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    peaks, peak_kind = measured_peaks()
    clk = clocks.summary()
    kernel_ms = statistics.mean(per_launch_ms)
    alg_bytes = 8.0 * cfg.pulses * cfg.samples + 48.0 * cfg.pulses + 8.0 * npix  # data + pos/w/phase + image
    achieved_gbs = alg_bytes / (kernel_ms / 1e3) / 1e9
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    fp32_derived = sm_count * 128 * 2 * sm_mhz * 1e6 / 1e12
    # Measured FP32 issue rate (sarbp_fp32_peak: independent FMA chains at full occupancy), the
    # better of scalar FFMA and packed FFMA2, taken right after the timed region.
    fp32_measured = {"ffma": core.fp32_peak_tflops(packed=False), "ffma2": core.fp32_peak_tflops(packed=True)}
    fp32_peak = max(fp32_measured.values())
    fp32_achieved = units * FP32_FLOPS_PER_PX_PULSE / (kernel_ms / 1e3) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (split precision: FP64 per tile-pulse)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "pulses": cfg.pulses, "samples": cfg.samples,
                   "image": [lat.rows, lat.cols], "pixel_spacing_m": cfg.pixel_spacing,
                   "l2": "L2 flushed between timed steps (256 MB write outside the step's events); 268 MB range data",
                   "pulse_split": core.lattice_pulse_split(lat.origin, lat.step_row, lat.step_col, lat.rows, lat.cols,
                                                           "split"),
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
                "path": "every step: pinned host data/pos/weight/phase -> device, core.backproject_lattice (C ABI), "
                        "image -> pinned host; uploads and read-backs on their own streams overlap the "
                        "neighbouring steps' BP"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved_gbs / peaks["hbm_gbs"], "traffic": NCU_TRAFFIC_BYTES,
                     "kernel": "split_lattice_kernel", "note": f"peak of {peak_kind}; algorithmic bytes "
                     f"{alg_bytes / 1e6:.1f} MB per launch; the kernel is FP32/MUFU-issue bound (roofline_fp32)"},
        "roofline_fp32": {"bound": "fp32_issue", "achieved": fp32_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                          "frac": fp32_achieved / fp32_peak, "peak_kind": "measured",
                          "peak_measured": fp32_measured, "peak_derived": fp32_derived,
                          "note": f"{FP32_FLOPS_PER_PX_PULSE:.0f} algorithmic FP32 flops + {MUFU_PER_PX_PULSE:.0f} "
                                  f"MUFU per pixel-pulse; peak measured on this GPU in this run (sarbp_fp32_peak, "
                                  f"independent FMA chains at full occupancy); derived {sm_count} SMs x 128 lanes x "
                                  f"2 x median SM clock {sm_mhz:.0f} MHz = {fp32_derived:.1f}"},
        "kernel_ms": kernel_ms,
        "clocks": clk,
        "gpu_launches": int(launches),
        "cpu_baseline": cpu,
        **extra,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
