"""Point-target precision report: each precision mode against FP64 on fine cuts through every target.

For every point target of a scene this forms, with direct BP at arbitrary
points (``backproject_points``), a fine ``side x side`` patch around the
target and a range cut (x) and an azimuth cut (y) through the FP64 peak,
in each requested mode and in FP64.  It reports per mode:

* whether the patch's peak index equals the FP64 one for every target;
* the largest IRW change (dB, 10 log10 of the width ratio) and the largest
  PSLR and ISLR changes (dB) over all targets and both cuts
  (``metrics.impulse_metrics``, the reference's 1-D convention);
* the relative complex L2 error of the patches and cuts against FP64.

``python -m bp_project_gb300.precision_report --config c2`` prints the table
(the 30 km, 8192-pulse scene is the precision stress case: FP32 ranges there
carry about 2 mm of rounding, about 0.8 rad of phase at 10 GHz).
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np
import torch

from . import core, metrics, scenes


def _cuts(target, half_width, n):
    t = np.linspace(-half_width, half_width, n)
    xs = np.column_stack([target[0] + t, np.full(n, target[1]), np.zeros(n)])
    ys = np.column_stack([np.full(n, target[0]), target[1] + t, np.zeros(n)])
    return t, xs, ys


def _patch(target, half_width, side):
    t = np.linspace(-half_width, half_width, side)
    xx, yy = np.meshgrid(target[0] + t, target[1] + t, indexing="ij")
    return np.column_stack([xx.ravel(), yy.ravel(), np.zeros(xx.size)])


def point_target_report(config="c2", modes=("split", "fp32", "mixed"), side=48, cut_points=257, max_targets=None,
                        device="cuda", scene=None):
    cfg = scenes.CONFIGS[config] if isinstance(config, str) else config
    sc = scene if scene is not None else scenes.synthesize(cfg, device=device)
    dev = torch.device(device)
    data = torch.as_tensor(sc.data).to(dev)
    pos = torch.as_tensor(sc.position).to(dev)
    w = torch.as_tensor(sc.weight).to(dev)
    ph = torch.as_tensor(sc.phase).to(dev)
    res = sc.config.resolution
    targets = sc.targets if max_targets is None else sc.targets[:max_targets]
    patch_half = 1.5 * res
    cut_half = 6.0 * res

    points, layout = [], []
    for tgt in targets:
        t, xs, ys = _cuts(tgt, cut_half, cut_points)
        pt = _patch(tgt, patch_half, side)
        layout.append((len(points), pt.shape[0], xs.shape[0]))
        points.append(np.vstack([pt, xs, ys]))
    offsets = np.cumsum([0] + [p.shape[0] for p in points])
    xyz = torch.as_tensor(np.vstack(points)).to(dev)

    def form(mode):
        out = core.backproject_points(data, pos, w, ph, xyz, sc.range_start, sc.data_dr, sc.k, mode=mode)
        return out.cpu().numpy()

    ref = form("fp64")
    report = {"config": sc.config.name, "targets": len(targets), "pulses": sc.config.pulses,
              "points": int(xyz.shape[0]), "patch": [side, side], "cut_points": cut_points,
              "patch_half_width_m": patch_half, "cut_half_width_m": cut_half, "modes": {}}
    t = np.linspace(-cut_half, cut_half, cut_points)
    ref_metrics = []
    for i in range(len(targets)):
        o = offsets[i]
        npatch = side * side
        xcut = ref[o + npatch:o + npatch + cut_points]
        ycut = ref[o + npatch + cut_points:o + npatch + 2 * cut_points]
        ref_metrics.append((metrics.impulse_metrics(t, xcut), metrics.impulse_metrics(t, ycut)))
    for mode in modes:
        est = form(mode)
        same_peak, d_irw, d_pslr, d_islr = 0, 0.0, 0.0, 0.0
        for i in range(len(targets)):
            o = offsets[i]
            npatch = side * side
            if int(np.abs(est[o:o + npatch]).argmax()) == int(np.abs(ref[o:o + npatch]).argmax()):
                same_peak += 1
            for c in range(2):
                seg = est[o + npatch + c * cut_points:o + npatch + (c + 1) * cut_points]
                m, r = metrics.impulse_metrics(t, seg), ref_metrics[i][c]
                if not (m.get("sidelobes_valid") and r.get("sidelobes_valid")):
                    d_irw = d_pslr = d_islr = math.inf
                    continue
                d_irw = max(d_irw, abs(10 * math.log10(m["irw_m"] / r["irw_m"])))
                d_pslr = max(d_pslr, abs(m["pslr_db"] - r["pslr_db"]))
                d_islr = max(d_islr, abs(m["islr_db"] - r["islr_db"]))
        err = float(np.linalg.norm(est.astype(np.complex128) - ref) / np.linalg.norm(ref))
        report["modes"][mode] = {"peak_index_equal": f"{same_peak}/{len(targets)}", "peaks_all_equal":
                                 same_peak == len(targets), "max_delta_irw_db": d_irw, "max_delta_pslr_db": d_pslr,
                                 "max_delta_islr_db": d_islr, "relative_l2_error": err}
    irw = [m["irw_m"] for pair in ref_metrics for m in pair if m.get("valid")]
    pslr = [m["pslr_db"] for pair in ref_metrics for m in pair if m.get("sidelobes_valid")]
    report["fp64_irw_m_range"] = [float(min(irw)), float(max(irw))] if irw else None
    report["fp64_pslr_db_range"] = [float(min(pslr)), float(max(pslr))] if pslr else None
    return report


def markdown(report) -> str:
    lines = [f"Scene {report['config']}: {report['targets']} targets, {report['pulses']} pulses, "
             f"{report['points']} points (patch {report['patch'][0]}x{report['patch'][1]} over "
             f"+-{report['patch_half_width_m']:.3f} m, cuts of {report['cut_points']} points over "
             f"+-{report['cut_half_width_m']:.3f} m); FP64 IRW {report['fp64_irw_m_range']} m, "
             f"PSLR {report['fp64_pslr_db_range']} dB.", "",
             "| mode | peak index = FP64 | max dIRW (dB) | max dPSLR (dB) | max dISLR (dB) | rel. L2 error |",
             "|---|---|---|---|---|---|"]
    for mode, r in report["modes"].items():
        lines.append(f"| {mode} | {r['peak_index_equal']} | {r['max_delta_irw_db']:.2e} | "
                     f"{r['max_delta_pslr_db']:.2e} | {r['max_delta_islr_db']:.2e} | {r['relative_l2_error']:.2e} |")
    return "\n".join(lines)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--modes", default="split,fp32,mixed")
    ap.add_argument("--json", default=None)
    args = ap.parse_args(argv)
    rep = point_target_report(args.config, tuple(args.modes.split(",")))
    print(markdown(rep))
    if args.json:
        with open(args.json, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()
