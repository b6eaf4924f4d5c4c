"""FFBP merge tiles that stage each child's footprint in shared memory by TMA (the default in split
mode) form the same image, bit for bit, as merge tiles that gather the stencils from the child
images in global memory; no staging wait runs out."""
import ctypes

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


def _images(config, **scale):
    from bp_project_gb300 import core, scenes
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    base = scenes.batch_configs(64)[int(config[5:])][0] if config.startswith("batch") else scenes.CONFIGS[config]
    cfg = scenes.scaled(base, **scale) if scale else base
    sc = scenes.synthesize(cfg, device="cuda")
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sc.data, sc.position, sc.weight, sc.phase)]
    out = {}
    for staging in (True, False):
        prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split", staging=staging)
        assert prog.staged == staging
        for _ in range(2):  # a second execute reuses the tensor maps and the node images
            out[staging] = prog.execute(*dev, sc.range_start, sc.data_dr, sc.k).clone()
        prog.close()
    torch.cuda.synchronize()
    return out


def _timeouts(lib):
    n = ctypes.c_int(-1)
    lib.check(lib.load().sarbp_wait_timeouts(ctypes.byref(n)))
    return n.value


# c1 and c2 geometries (32 x 32 and 16 x 64 merge tiles, boxes under 9.5 KB per child), the c0 scene, and
# a 7.7 km scene of the batch workload whose lowest merge levels run on 8 x 128 tiles with boxes of about
# 12.9 KB per child (six CTAs per SM)
@pytest.mark.parametrize("config,scale", [("c1", dict(pulses=1024, samples=4096, image_side=512)),
                                          ("c2", dict(pulses=2048, samples=4096, image_side=512)),
                                          ("c0", {}),
                                          ("batch6", dict(pulses=1024))])
def test_staged_merge_equals_gathered_merge(lib, config, scale):
    before = _timeouts(lib)
    out = _images(config, **scale)
    assert torch.equal(out[True], out[False])
    assert float(out[True].abs().max()) > 0
    assert _timeouts(lib) == before


@pytest.mark.slow
def test_staged_merge_equals_gathered_merge_c1(lib):
    """The 4096-pulse / 2048^2 plan (8 merge levels, footprints of 16 x 71 and 24-30 x 39 elements)."""
    before = _timeouts(lib)
    out = _images("c1")
    assert torch.equal(out[True], out[False])
    assert _timeouts(lib) == before


def test_a_staged_wait_that_runs_out_falls_back_to_the_child_images(lib):
    """The root's merge tiles declare 16 bytes more than their TMA copies deliver (the withheld node
    of sarbp_ffbp_set_wait_limit), so every root warp's wait runs out after 5 ms: those warps gather
    from the child images instead, the image is the same bit for bit, the waits are counted, and the
    GPU stays usable."""
    import time
    from bp_project_gb300 import core, scenes
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    cfg = scenes.scaled(scenes.CONFIGS["c1"], pulses=1024, samples=4096, image_side=512)
    sc = scenes.synthesize(cfg, device="cuda")
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sc.data, sc.position, sc.weight, sc.phase)]
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split", staging=False)
    want = prog.execute(*dev, sc.range_start, sc.data_dr, sc.k)
    torch.cuda.synchronize()
    prog.close()

    h = lib.load()
    arr = core.node_array(plan.nodes())
    handle = ctypes.c_void_p()
    crop = (plan.crop_r[0], plan.crop_u[0], plan.crop_r[1] - plan.crop_r[0], plan.crop_u[1] - plan.crop_u[0])
    lib.check(h.sarbp_ffbp_plan_create(arr, len(arr), *crop, lib.mode_id("split"), ctypes.byref(handle)))
    try:
        lib.check(h.sarbp_ffbp_set_wait_limit(handle, 0.005, 0))
        ws = torch.empty(h.sarbp_ffbp_workspace_bytes(handle), dtype=torch.uint8, device="cuda")
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        lib.check(h.sarbp_ffbp_bind(handle, ctypes.c_void_p(ws.data_ptr()), ws.numel(), stream))
        staged = ctypes.c_int(0)
        lib.check(h.sarbp_ffbp_staging(handle, ctypes.byref(staged)))
        assert staged.value == 1
        before = _timeouts(lib)
        got = torch.zeros_like(want)
        p, s = dev[0].shape
        ptr = lambda t: ctypes.c_void_p(t.data_ptr())
        t0 = time.perf_counter()
        lib.check(h.sarbp_ffbp_execute(handle, ptr(dev[0]), p, s, ptr(dev[1]), ptr(dev[2]), ptr(dev[3]),
                                       sc.range_start, sc.data_dr, sc.k, ptr(got), stream))
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
        counted = _timeouts(lib) - before
    finally:
        h.sarbp_ffbp_plan_destroy(handle)
    assert counted > 0
    assert elapsed < 10.0
    assert torch.equal(got, want)
    # the GPU keeps working: a plain staged plan forms the same image with no wait running out
    out = _images("c1", pulses=1024, samples=4096, image_side=512)
    assert torch.equal(out[True], out[False])


def test_far_range_ffbp_vs_reference_ffbp(lib):
    """A 7.7 km scene of the uneven batch workload (1024 pulses onto 256² at 0.5 m), whose lowest merge
    levels stage 12.9 KB footprints: split FFBP within 1e-4 of the reference FFBP (oracle restatement of
    ffbp.form_ffbp on the same plan), with the same peak pixel."""
    from bp_project_gb300 import core, scenes
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    from conftest import rel_err
    from oracle import reference as ora
    cfg = scenes.scaled(scenes.batch_configs(64)[6][0], pulses=1024)
    sc = scenes.synthesize(cfg, device="cuda")
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sc.data, sc.position, sc.weight, sc.phase)]
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split")
    assert prog.staged
    img = prog.execute(*dev, sc.range_start, sc.data_dr, sc.k).cpu().numpy()
    prog.close()
    ref, _ = ora.form_ffbp(sc.data, sc.position, sc.range_start, sc.data_dr, cfg.fc, sc.extent, side=1,
                           leaf_size=cfg.leaf_size, range_spacing=cfg.range_spacing,
                           angular_oversample=cfg.angular_oversample, weight=sc.weight, phase=sc.phase)
    err = rel_err(ref.image, img)
    print(f"far-range split FFBP vs reference FFBP: {err:.3e}")
    assert err <= 1e-4
    assert np.unravel_index(np.abs(img).argmax(), img.shape) == np.unravel_index(np.abs(ref.image).argmax(),
                                                                                   ref.image.shape)
