"""Measurement entry points: the FP32 issue-rate microbenchmark behind the FP32 roofline, and the
count of kernel waits that ran out (none in the default build, which has no waiting kernels)."""
import ctypes

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


def test_fp32_peak_is_a_plausible_rate(lib):
    from bp_project_gb300 import core
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    nominal = sms * 128 * 2 * 2.1e9 / 1e12  # lanes x FMA x a clock a little above the maximum
    for packed in (False, True):
        t = core.fp32_peak_tflops(packed=packed, iters=4096)
        assert 0.25 * nominal < t < 1.05 * nominal, (packed, t, nominal)
    h = lib.load()
    out = ctypes.c_double()
    assert h.sarbp_fp32_peak(2, 16, ctypes.byref(out)) == lib.SARBP_ERR_VALUE
    assert h.sarbp_fp32_peak(0, 0, ctypes.byref(out)) == lib.SARBP_ERR_VALUE


def test_no_kernel_wait_ran_out(lib):
    from bp_project_gb300 import core, scenes
    sc = scenes.synthesize(scenes.scaled(scenes.CONFIGS["c0"], pulses=64, image_side=64), device="cuda")
    L = sc.lattice
    dev = [torch.from_numpy(a).cuda() for a in (sc.data, sc.position, sc.weight, sc.phase)]
    core.backproject_lattice(*dev, L.origin, L.step_row, L.step_col, L.rows, L.cols, sc.range_start, sc.data_dr, sc.k,
                             mode="split")
    count = ctypes.c_int(-1)
    lib.check(lib.load().sarbp_wait_timeouts(ctypes.byref(count)))
    assert count.value == 0
