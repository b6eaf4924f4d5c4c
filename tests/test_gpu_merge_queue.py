"""FFBP merges as one dependency-counting queue launch: the same image as one launch per tree height,
and a wait that runs out (a node whose children are never counted complete) ends the launch with an
error status the host reads, without hanging the GPU."""
import ctypes
import time

import numpy as np
import pytest

from conftest import rel_err

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


def _scene():
    from bp_project_gb300 import scenes
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    cfg = scenes.scaled(scenes.CONFIGS["c1"], pulses=1024, samples=4096, image_side=512)
    sc = scenes.synthesize(cfg, device="cuda")
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sc.data, sc.position, sc.weight, sc.phase)]
    return sc, plan, dev


def test_queue_equals_one_launch_per_height(lib):
    from bp_project_gb300 import core
    sc, plan, dev = _scene()
    out = {}
    for queue in (False, True):
        prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split", merge_queue=queue)
        if queue:
            assert prog.launch_count == 5  # three prologues, the leaves, the merge queue
        for _ in range(2):  # the second execute starts from the counters' reset, not the first's end state
            out[queue] = prog.execute(*dev, sc.range_start, sc.data_dr, sc.k).clone()
        prog.close()
    torch.cuda.synchronize()
    assert torch.equal(out[True], out[False])
    assert float(out[True].abs().max()) > 0


def _raw_plan(lib, plan, limit_s, withheld):
    from bp_project_gb300 import core
    h = lib.load()
    arr = core.node_array(plan.nodes())
    handle = ctypes.c_void_p()
    crop = (plan.crop_r[0], plan.crop_u[0], plan.crop_r[1] - plan.crop_r[0], plan.crop_u[1] - plan.crop_u[0])
    lib.check(h.sarbp_ffbp_plan_create(arr, len(arr), *crop, lib.mode_id("split"), ctypes.byref(handle)))
    lib.check(h.sarbp_ffbp_set_merge_queue(handle, 1))
    lib.check(h.sarbp_ffbp_set_wait_limit(handle, limit_s, withheld))
    ws = torch.empty(h.sarbp_ffbp_workspace_bytes(handle), dtype=torch.uint8, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib.check(h.sarbp_ffbp_bind(handle, ctypes.c_void_p(ws.data_ptr()), ws.numel(), stream))
    return h, handle, ws, crop, stream


def _execute(lib, h, handle, dev, sc, crop, stream):
    out = torch.zeros((crop[2], crop[3]), dtype=torch.complex64, device="cuda")
    p, s = dev[0].shape
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    lib.check(h.sarbp_ffbp_execute(handle, ptr(dev[0]), p, s, ptr(dev[1]), ptr(dev[2]), ptr(dev[3]), sc.range_start,
                                   sc.data_dr, sc.k, ptr(out), stream))
    torch.cuda.synchronize()
    status = ctypes.c_int(-1)
    lib.check(h.sarbp_ffbp_status(handle, ctypes.byref(status)))
    return out, status.value


def test_a_wait_that_runs_out_reports_an_error(lib):
    """The root is withheld (its children are never counted complete): every root tile's wait runs
    out after 0.2 s, the launch ends, and the status says so.  A plan without the withheld node then
    forms the image normally on the same GPU."""
    from bp_project_gb300 import core
    sc, plan, dev = _scene()
    h, handle, ws, crop, stream = _raw_plan(lib, plan, 0.2, 0)
    t0 = time.perf_counter()
    _, status = _execute(lib, h, handle, dev, sc, crop, stream)
    elapsed = time.perf_counter() - t0
    h.sarbp_ffbp_plan_destroy(handle)
    assert status == 1
    assert elapsed < 10.0
    h, handle, ws, crop, stream = _raw_plan(lib, plan, 5.0, -1)
    good, status = _execute(lib, h, handle, dev, sc, crop, stream)
    h.sarbp_ffbp_plan_destroy(handle)
    assert status == 0
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split", merge_queue=False)
    want = prog.execute(*dev, sc.range_start, sc.data_dr, sc.k)
    torch.cuda.synchronize()
    prog.close()
    assert torch.equal(good, want)
