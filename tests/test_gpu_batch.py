"""Scene batches: persistent work-queue kernels over uneven scenes.

Each scene of a batch must equal, bit for bit, the single-scene split-precision
entry point with the same tile shape (the per-tile arithmetic is the same code;
only the scheduling differs), including after graph capture and replay.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build
    build.build()
    from bp_project_gb300 import _native
    _native.load()
    return _native


def make_scenes(configs):
    from bp_project_gb300 import scenes
    from bp_project_gb300.batch import DirectScene, FFBPScene
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    out = []
    for cfg, kind in configs:
        sc = scenes.synthesize(cfg, device="cuda")
        dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a)).to("cuda", dt)
        common = dict(data=dev(sc.data, torch.complex64), pos=dev(sc.position, torch.float64),
                      weight=dev(sc.weight, torch.float64), phase=dev(sc.phase, torch.float64),
                      range_start=sc.range_start, data_dr=sc.data_dr, k=sc.k)
        if kind == "direct":
            lat = sc.lattice
            out.append(DirectScene(**common, origin=tuple(lat.origin), step_row=tuple(lat.step_row),
                                   step_col=tuple(lat.step_col), rows=lat.rows, cols=lat.cols))
        else:
            plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                                   range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
            out.append(FFBPScene(**common, plan=plan))
    return out


def single(sc):
    from bp_project_gb300 import core
    from bp_project_gb300.batch import DirectScene
    if isinstance(sc, DirectScene):
        return core.backproject_lattice(sc.data, sc.pos, sc.weight, sc.phase, sc.origin, sc.step_row, sc.step_col,
                                        sc.rows, sc.cols, sc.range_start, sc.data_dr, sc.k, mode="split",
                                        pulse_split=1)  # a batch scene sums its pulses in one pass
    prog = core.FFBPProgram(sc.plan.nodes(), sc.plan.crop_r, sc.plan.crop_u, mode="split", device=sc.data.device)
    try:
        return prog.execute(sc.data, sc.pos, sc.weight, sc.phase, sc.range_start, sc.data_dr, sc.k).clone()
    finally:
        prog.close()


@pytest.fixture(scope="module")
def small_batch(lib):
    from bp_project_gb300 import scenes
    cfgs = scenes.batch_configs(count=8, seed=7, pulse_choices=(512, 1024, 1536), side_choices=(256, 512))
    return make_scenes(cfgs)


def test_batch_equals_single_scene_paths(small_batch):
    from bp_project_gb300.batch import SceneBatch
    batch = SceneBatch(small_batch)
    batch.execute()
    torch.cuda.synchronize()
    kinds = []
    for sc in small_batch:
        ref = single(sc)
        torch.cuda.synchronize()
        assert torch.equal(sc.out, ref), type(sc).__name__
        assert float(sc.out.abs().max()) > 0
        kinds.append(type(sc).__name__)
    assert "DirectScene" in kinds and "FFBPScene" in kinds
    print(batch.info, "launches", batch.launch_count)
    # The persistent direct launch keeps the single-scene lattice kernel's four CTAs per SM.
    n_direct = sum(-(-sc.rows // 32) * -(-sc.cols // 32) for sc in small_batch if type(sc).__name__ == "DirectScene")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert batch.info["bp_blocks"] == min(n_direct, 4 * sms), (batch.info, n_direct, sms)
    assert batch.launch_count == 1 + 4 + 1 + batch.info["max_height"]  # memset, prologues + leaves, direct, merges
    # graph capture + replay reproduce the eager result
    first = [o.clone() for o in batch.outputs]
    for o in batch.outputs:
        o.zero_()
    batch.capture_graph()
    for o in batch.outputs:
        o.zero_()
    batch.replay()
    torch.cuda.synchronize()
    for a, b in zip(first, batch.outputs):
        assert torch.equal(a, b)
    batch.close()


def test_batch_scene_latency_trace(small_batch):
    """A traced execution reports every scene's completion after the batch's start, within the batch's own
    duration, and leaves the images unchanged; FFBP scenes finish with their root merge."""
    from bp_project_gb300.batch import SceneBatch
    batch = SceneBatch(small_batch)
    batch.execute()
    torch.cuda.synchronize()
    first = [o.clone() for o in batch.outputs]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    lat = batch.scene_latencies_ms()
    e1.record()
    torch.cuda.synchronize()
    total = e0.elapsed_time(e1)
    print("scene latencies (ms):", np.round(lat, 3), "batch", round(total, 3))
    assert len(lat) == len(small_batch)
    assert np.all(lat > 0) and np.all(lat <= total * 1.05 + 0.05)
    for a, b in zip(first, batch.outputs):
        assert torch.equal(a, b)
    batch.close()


def test_batch_tile_shapes_and_chunks(small_batch):
    """Other tile shapes / chunks stay within split precision of the default; chunks alone change nothing."""
    from bp_project_gb300.batch import DirectScene, SceneBatch
    direct = [sc for sc in small_batch if isinstance(sc, DirectScene)][:2]
    ref = [single(sc) for sc in direct]
    for lc, ch in ((3, 8), (4, 16), (5, 8), (5, 64)):
        cands = [DirectScene(**{**sc.__dict__, "tile_lc": lc, "chunk_pulses": ch, "out": None}) for sc in direct]
        batch = SceneBatch(cands, blocks_per_sm=2)
        batch.execute()
        torch.cuda.synchronize()
        for sc, r in zip(cands, ref):
            if lc == 5:
                assert torch.equal(sc.out, r)
            else:
                err = float((sc.out - r).abs().norm() / r.abs().norm())
                assert err < 5e-6, (lc, ch, err)
        batch.close()


def test_autotune_picks_a_measured_candidate(small_batch, tmp_path):
    from bp_project_gb300.autotune import tune_direct
    from bp_project_gb300.batch import DirectScene
    sc = next(s for s in small_batch if isinstance(s, DirectScene))
    choice, timings = tune_direct(sc, cache=tmp_path / "tune.json", reps=1, tile_lcs=(4, 5), chunks=(16, 32),
                                  blocks=(2, 3))
    assert f"{choice[0]},{choice[1]},{choice[2]}" in timings and len(timings) == 8
    assert min(timings.values()) == timings[f"{choice[0]},{choice[1]},{choice[2]}"]
    again, _ = tune_direct(sc, cache=tmp_path / "tune.json")
    assert again == choice  # served from the cache


def test_concurrent_batch_equals_single_stream_batch(small_batch):
    """The FFBP chain on the batch's own stream beside the direct queue gives the same images, eagerly
    and from a captured graph (both branches recorded in one graph)."""
    from bp_project_gb300.batch import SceneBatch
    refs = [single(sc) for sc in small_batch]
    torch.cuda.synchronize()
    for bps in (2, 4):
        fresh = [type(sc)(**{**sc.__dict__, "out": None}) for sc in small_batch]
        batch = SceneBatch(fresh, blocks_per_sm=bps, concurrent=True)
        batch.execute()
        torch.cuda.synchronize()
        for sc, r in zip(fresh, refs):
            assert torch.equal(sc.out, r), (bps, type(sc).__name__)
        batch.capture_graph()
        for o in batch.outputs:
            o.zero_()
        for _ in range(2):
            batch.replay()
        torch.cuda.synchronize()
        for sc, r in zip(fresh, refs):
            assert torch.equal(sc.out, r), (bps, "graph", type(sc).__name__)
        lat = batch.scene_latencies_ms()
        assert len(lat) == len(fresh) and np.all(lat > 0)
        batch.close()
