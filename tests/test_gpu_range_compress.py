"""Range compression on the GPU against the reference's sar_io.range_compress outputs
(tests/golden/range_compress.npz).  Tolerance: relative complex L2 error <= 1e-5 (single-
precision FFTs of two libraries); the LFM point echo of validate.py:54-59 must be found within
0.25 samples of 1512.4 with 4x oversampling, as the reference asserts."""
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_err

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden import lfm_point_raw, range_compress_inputs  # noqa: E402

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


def test_range_compress_matches_reference(golden, lib):
    from bp_project_gb300.sar_io import range_compress
    g = golden("range_compress")
    raw = range_compress_inputs()
    for key, kw in (("os1", {}), ("os2", {"oversample": 2}),
                    ("os1_up", {"chirp_sign": 1, "tp": 0.8e-6, "bandwidth": 150e6})):
        out = range_compress(raw, **kw)
        assert out.shape == g[key].shape and out.dtype == np.complex64
        err = rel_err(g[key], out)
        print(f"range_compress {key}: {err:.2e}")
        assert err <= 1e-5
    # device in, device out
    dev = range_compress(torch.from_numpy(raw).cuda())
    assert dev.is_cuda and rel_err(g["os1"], dev.cpu().numpy()) <= 1e-5


def test_lfm_point_lag(golden, lib):
    from bp_project_gb300.sar_io import range_compress
    g = golden("range_compress")
    out = range_compress(lfm_point_raw(), oversample=4)
    found = np.argmax(np.abs(out[0])) / 4
    assert abs(found - 1512.4) <= 0.25
    assert found == float(g["lfm_peak"])
    assert rel_err(g["lfm_near_peak"], out[0, 6000:6100]) <= 1e-5


def test_range_compress_rejects_bad_windows(lib):
    import ctypes
    h = lib.load()
    fake = ctypes.c_void_p(0x10000)
    assert h.sarbp_rc_prepare(fake, 4, 100, 50, fake, None) == lib.SARBP_ERR_VALUE
    assert h.sarbp_rc_crop(fake, 4, 100, 60, 50, 1.0, fake, None) == lib.SARBP_ERR_VALUE
    assert h.sarbp_rc_filter(fake, fake, 4, 128, 256, fake, None) == lib.SARBP_ERR_VALUE  # in place + oversampling
