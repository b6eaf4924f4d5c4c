"""The allocation-free direct BP entry point (sarbp_direct_polar_static).

Callers that cannot allocate device memory where they image (hosts that own
all device memory through their own pool, real-time loops where cudaMalloc
would synchronise, cgo/JNI hosts that only see the buffers they were handed)
use this entry point: the pulse-split scratch lives in a fixed 16 MiB device
array inside the library instead of a caller workspace.  The test calls it
through the C ABI twice in a row, on different inputs, and compares each
result with the workspace-taking sarbp_direct_polar.  The file sorts last so a
run that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SPLIT = 3
PULSE_SPLIT = 3
TOL = 1e-6  # same kernels and summation order as the workspace path: results agree to FP32 rounding


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build
    build.build()
    from bp_project_gb300 import _native
    _native.load()
    return _native


def _case(golden, case):
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    g = golden("operator_validation")
    p = f"case{case}_"
    range_start, data_dr, fc, k, side, *extent = g[p + "scalars"]
    plan = build_ffbp_plan(g[p + "position"], fc, extent, side=int(side), leaf_size=8, range_spacing=0.5,
                           angular_oversample=3.0)
    dev = [torch.from_numpy(np.ascontiguousarray(g[p + name])).cuda()
           for name in ("data", "position", "weight", "phase")]
    return dev, plan, float(range_start), float(data_dr), float(k)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_static_scratch_matches_workspace_entry_point(golden, lib):
    h = lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for case in (0, 1):  # two calls in a row through the shared scratch
        (data, pos, w, ph), plan, range_start, data_dr, k = _case(golden, case)
        grid = lib.polar_grid(plan.origin, plan.r0, plan.dr, plan.nr, plan.u0, plan.du, plan.nu, plan.side)
        p, s = data.shape
        want = torch.empty((plan.nr, plan.nu), dtype=torch.complex64, device="cuda")
        ws_bytes = h.sarbp_direct_polar_workspace(SPLIT, ctypes.byref(grid), p, PULSE_SPLIT)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
        lib.check(h.sarbp_direct_polar(_ptr(data), p, s, _ptr(pos), _ptr(w), _ptr(ph), ctypes.byref(grid),
                                       range_start, data_dr, k, SPLIT, 64, PULSE_SPLIT, _ptr(want), _ptr(ws), ws_bytes,
                                       stream))
        got = torch.full((plan.nr, plan.nu), float("nan"), dtype=torch.complex64, device="cuda")
        lib.check(h.sarbp_direct_polar_static(_ptr(data), p, s, _ptr(pos), _ptr(w), _ptr(ph), ctypes.byref(grid),
                                              range_start, data_dr, k, 64, PULSE_SPLIT, _ptr(got), stream))
        torch.cuda.synchronize()
        a, b = want.cpu().numpy(), got.cpu().numpy()
        assert np.isfinite(b).all()
        assert rel_err(a, b) <= TOL


def test_static_scratch_rejects_oversized_requests(lib):
    h = lib.load()
    cap = h.sarbp_static_scratch_elements()
    assert cap == 1 << 21
    grid = lib.polar_grid((0.0, 0.0, 100.0), 1000.0, 0.25, 1024, -0.1, 1e-4, 1024, 1)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    st = h.sarbp_direct_polar_static(_ptr(dummy), 4, 1, _ptr(dummy), _ptr(dummy), _ptr(dummy), ctypes.byref(grid),
                                     0.0, 1.0, 1.0, 64, 4, _ptr(dummy), None)
    assert st == lib.SARBP_ERR_VALUE
    assert b"exceeds the static scratch" in h.sarbp_last_error()
