"""Autotuner for the pixel-tile x pulse-chunk shape of split-precision direct BP.

The tunables are the tile shape (``tile_lc``: 1 << lc columns by 1024 >> lc rows;
the reference's equivalent knob is the 256-thread block over a flat pixel range)
and the pulses staged per chunk (``chunk_pulses``, the reference's
``--chunk-pulses``, gpu_baseline.py:413), plus the CTAs per SM of the persistent
batch launch and whether the batch's FFBP chain runs on its own stream beside the
direct queue.  For a scene class (image side, pixel spacing, range geometry)
``tune_direct`` times every candidate on a representative scene through
``SceneBatch`` (CUDA events, after a warm-up) and keeps the fastest; results are
cached per device and class in a JSON file.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import torch

from .batch import DirectScene, SceneBatch

TILE_LCS = (3, 4, 5)
CHUNKS = (16, 32, 64)
BLOCKS_PER_SM = (2, 3, 4)
DEFAULT_CACHE = Path(os.environ.get("SARBP_AUTOTUNE_CACHE", Path(__file__).resolve().parent / ".autotune.json"))


def _key(scene: DirectScene, device) -> str:
    name = torch.cuda.get_device_name(device).replace(" ", "_")
    spacing = max(abs(v) for v in scene.step_row)
    return f"{name}|direct|side{max(scene.rows, scene.cols)}|dx{spacing:.3g}|dr{scene.data_dr:.4g}"


def _time(scenes, blocks_per_sm, reps, concurrent=False):
    batch = SceneBatch(scenes, blocks_per_sm=blocks_per_sm, concurrent=concurrent)
    try:
        batch.execute()
        torch.cuda.synchronize()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(reps):
            batch.execute()
        stop.record()
        torch.cuda.synchronize()
        return start.elapsed_time(stop) / reps
    finally:
        batch.close()


def tune_direct(scene: DirectScene, cache: Path | None = DEFAULT_CACHE, reps=3, retune=False,
                tile_lcs=TILE_LCS, chunks=CHUNKS, blocks=BLOCKS_PER_SM):
    """Best (tile_lc, chunk_pulses, blocks_per_sm) for scenes like ``scene``; returns (choice, timings)."""
    key = _key(scene, scene.data.device)
    table = {}
    if cache is not None and Path(cache).exists():
        table = json.loads(Path(cache).read_text())
        if key in table and not retune:
            return tuple(table[key]["best"]), table[key]["timings"]
    timings = {}
    for lc in tile_lcs:
        for ch in chunks:
            for bps in blocks:
                cand = DirectScene(**{**scene.__dict__, "tile_lc": lc, "chunk_pulses": ch, "out": None})
                timings[f"{lc},{ch},{bps}"] = _time([cand], bps, reps)
    best = min(timings, key=timings.get)
    choice = tuple(int(v) for v in best.split(","))
    if cache is not None:
        table[key] = {"best": list(choice), "timings": timings}
        Path(cache).write_text(json.dumps(table, indent=1, sort_keys=True))
    return choice, timings


def apply(scenes, choices):
    """Set tile_lc / chunk_pulses of direct scenes from {side: (lc, chunk, blocks)}."""
    for sc in scenes:
        if isinstance(sc, DirectScene):
            lc, ch, _ = choices[max(sc.rows, sc.cols)]
            sc.tile_lc, sc.chunk_pulses = lc, ch


def tune_blocks(scenes, blocks=BLOCKS_PER_SM, reps=1, concurrent=(False, True)):
    """CTAs per SM of the persistent direct launch, and whether the FFBP chain runs on its own stream
    beside it, for the whole batch (timed on the batch itself).  Returns ((blocks_per_sm, concurrent),
    {"blocks,concurrent": ms})."""
    timings = {}
    for conc in concurrent:
        for bps in blocks:
            fresh = [type(sc)(**{**sc.__dict__, "out": None}) for sc in scenes]
            timings[f"{bps},{int(conc)}"] = _time(fresh, bps, reps, conc)
    best = min(timings, key=timings.get)
    bps, conc = best.split(",")
    return (int(bps), bool(int(conc))), timings
