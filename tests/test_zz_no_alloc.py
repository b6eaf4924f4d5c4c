"""The allocation-free direct BP entry point (sarbp_direct_polar_static).

Callers that cannot allocate device memory where they image (hosts that own
all device memory through their own pool, real-time loops where cudaMalloc
would synchronise, cgo/JNI hosts that only see the buffers they were handed)
use this entry point: the pulse-split scratch lives in a fixed 16 MiB device
array inside the library instead of a caller workspace.  The test calls it
through the C ABI twice in a row, on different inputs (the larger first), and
requires each image to be bit-identical to the workspace-taking
sarbp_direct_polar's.  The file sorts last so a
run that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SPLIT = 3
# The static and workspace entry points run the same split kernel and the same fixed-order sum of
# partial images with the same tile, window and chunk choice, so their images must be bit-identical.


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


def _workspace_image(h, lib, dev, grid, plan, range_start, data_dr, k, pulse_split, stream):
    data, pos, w, ph = dev
    p, s = data.shape
    want = torch.empty((plan.nr, plan.nu), dtype=torch.complex64, device="cuda")
    ws_bytes = h.sarbp_direct_polar_workspace(SPLIT, ctypes.byref(grid), p, pulse_split)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device="cuda")
    lib.check(h.sarbp_direct_polar(_ptr(data), p, s, _ptr(pos), _ptr(w), _ptr(ph), ctypes.byref(grid), range_start,
                                   data_dr, k, SPLIT, 64, pulse_split, _ptr(want), _ptr(ws), ws_bytes, stream))
    return want


def _static_image(h, lib, dev, grid, plan, range_start, data_dr, k, pulse_split, stream):
    data, pos, w, ph = dev
    p, s = data.shape
    got = torch.full((plan.nr, plan.nu), float("nan"), dtype=torch.complex64, device="cuda")
    lib.check(h.sarbp_direct_polar_static(_ptr(data), p, s, _ptr(pos), _ptr(w), _ptr(ph), ctypes.byref(grid),
                                          range_start, data_dr, k, 64, pulse_split, _ptr(got), stream))
    return got


@pytest.mark.parametrize("pulse_split", [3, 1])
def test_static_scratch_matches_workspace_entry_point(golden, lib, pulse_split):
    """Two calls in a row (two scenes, the larger first) through the shared scratch: each image is
    bit-identical to the workspace entry point's.  pulse_split 1 writes straight into out."""
    h = lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    cases = [_case(golden, c) for c in (0, 1)]
    cases.sort(key=lambda c: -(c[1].nr * c[1].nu))  # a larger call, then a smaller one
    for dev, plan, range_start, data_dr, k in cases:
        grid = lib.polar_grid(plan.origin, plan.r0, plan.dr, plan.nr, plan.u0, plan.du, plan.nu, plan.side)
        want = _workspace_image(h, lib, dev, grid, plan, range_start, data_dr, k, pulse_split, stream)
        got = _static_image(h, lib, dev, grid, plan, range_start, data_dr, k, pulse_split, stream)
        torch.cuda.synchronize()
        assert torch.isfinite(torch.view_as_real(got)).all()
        assert torch.equal(want, got)


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
