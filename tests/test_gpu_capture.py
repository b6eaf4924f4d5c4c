"""Raw capture reader against the reference's sar_io.Capture on a synthetic capture file in its
frame format (tests/golden/capture_file.py writes it; tests/golden/capture.npz holds the
reference's parse and read)."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from capture_file import write_capture  # noqa: E402

torch = pytest.importorskip("torch")


def _capture(tmp_path):
    from bp_project_gb300.sar_io import Capture
    return Capture(write_capture(tmp_path / "capture.dat"))


def test_capture_headers_match_reference(golden, tmp_path):
    """Host-side parse: frame layout, valid frames, timing and navigation."""
    g = golden("capture")
    cap = _capture(tmp_path)
    assert cap.n == int(g["n"]) and cap.nr == int(g["nr"]) and cap.offset == int(g["offset"])
    assert cap.frame_size == int(g["frame_size"])
    np.testing.assert_array_equal(cap.valid_indices, g["valid_indices"])
    np.testing.assert_array_equal([cap.tp, cap.delay, cap.prf, cap.bandwidth], g["scalars"])
    np.testing.assert_array_equal(cap.time, g["time"])
    for k, v in cap.nav.items():
        np.testing.assert_array_equal(v, g["nav_" + k])
    s = cap.summary
    np.testing.assert_array_equal([s[k] for k in ("complete_frame_slots", "valid_frames", "invalid_slots",
                                                  "first_pulse", "last_pulse", "missing_pulses",
                                                  "discarded_partial_bytes")], g["summary"])


@pytest.mark.gpu
def test_capture_read_decodes_on_the_gpu(golden, tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build
    build.build()
    g = golden("capture")
    cap = _capture(tmp_path)
    host = cap.read(g["read_idx"])
    assert host.dtype == np.complex64
    np.testing.assert_array_equal(host, g["read"])  # int16 -> float32 is exact
    dev = cap.read(g["read_idx"], device="cuda")
    assert dev.is_cuda
    np.testing.assert_array_equal(dev.cpu().numpy(), g["read"])
