"""Autofocus pieces that need no GPU: the CPU oracle against the reference's own outputs
(tests/golden/autofocus.npz), and the product's FP64 torch smoothing helpers against scipy."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import autofocus_scene as scene  # noqa: E402

torch = pytest.importorskip("torch")


def _close(est, ref, rel):
    est, ref = np.asarray(est), np.asarray(ref)
    return float(np.abs(est - ref).max()) <= rel * float(np.abs(ref).max())


@pytest.mark.parametrize("name", ["recovery", "cluttered"])
def test_oracle_estimate_update_matches_reference(golden, name):
    from oracle import autofocus as oaf
    g = golden("autofocus")
    s = getattr(scene, name)()
    np.testing.assert_allclose(s.data[::97, ::31], g[f"{name}_data_probe"], rtol=0, atol=2e-6)
    delta, stats = oaf.estimate_update(s.data, s.pos, s.points, s.r_start, s.dr, s.k, s.prf, s.cutoff)
    assert _close(delta, g[f"{name}_delta"], 1e-6)
    assert abs(stats["median_gradient_coherence"] - float(g[f"{name}_coherence"])) < 1e-9
    before, after = g[f"{name}_rmse"]
    if name == "recovery":  # validate_autofocus.py:20
        assert after < 0.35 * before
        err = s.err + delta
        assert np.sqrt(np.mean(err[:, :2] ** 2)) < 0.35 * before


@pytest.mark.parametrize("tiles", [(12, 12), (7, 5)])
def test_oracle_pick_targets_matches_reference(golden, tiles):
    from oracle import autofocus as oaf
    g = golden("autofocus")
    p = scene.picks()
    r = p.r0 + p.dr * np.arange(p.image.shape[0])
    u = p.u0 + p.du * np.arange(p.image.shape[1])
    pts, powers = oaf.pick_targets(p.image, r, u, p.origin, p.side, *tiles)
    key = f"picks_{tiles[0]}x{tiles[1]}"
    np.testing.assert_array_equal(pts, g[key + "_points"])
    np.testing.assert_array_equal(powers, g[key + "_powers"])
    assert len(pts) < tiles[0] * tiles[1] or tiles == (7, 5)  # the dark corner is dropped


def test_savgol_and_detrend_match_scipy():
    from scipy import signal
    from bp_project_gb300.autofocus import detrend_linear, savgol_smooth
    rng = np.random.default_rng(3)
    x = np.cumsum(rng.standard_normal((1500, 2)), axis=0)
    for window in (5, 101, 501):
        ref = signal.savgol_filter(x, window, 3, axis=0)
        est = savgol_smooth(torch.from_numpy(x), window, 3).numpy()
        assert _close(est, ref, 1e-10), window  # summation order only
    ref = signal.detrend(x, axis=0, type="linear")
    est = detrend_linear(torch.from_numpy(x)).numpy()
    assert _close(est, ref, 1e-12)


def test_butter_lowpass_padding_matches_scipy():
    from scipy import signal
    from bp_project_gb300.autofocus import butter_lowpass
    f = butter_lowpass(12.0, 1000.0)
    assert f.padlen == 15 and f.sos.shape == (2, 6)
    x = np.random.default_rng(1).standard_normal(64)
    # sosfiltfilt with the explicit padlen equals its default
    np.testing.assert_array_equal(signal.sosfiltfilt(f.sos, x), signal.sosfiltfilt(f.sos, x, padlen=f.padlen))


@pytest.mark.parametrize("shape,dim", [((60,), None), ((61,), None), ((60, 2047), 0), ((59, 100), 0), ((7, 8), 1)])
def test_median_matches_numpy_exactly(shape, dim):
    from bp_project_gb300.autofocus import _median
    x = np.random.default_rng(sum(shape)).standard_normal(shape)
    est = _median(torch.from_numpy(x), dim).numpy()
    np.testing.assert_array_equal(est, np.median(x, axis=dim))


def test_rounded_sosfiltfilt_restatement_equals_scipy():
    """The separately rounded forward-backward recursion that the GPU filter test compares against
    bit for bit equals scipy.signal.sosfiltfilt on this host."""
    from scipy import signal

    from bp_project_gb300.autofocus import butter_lowpass
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_gpu_autofocus import _sosfiltfilt_rounded
    rng = np.random.default_rng(3)
    x = (rng.standard_normal((5, 400)) + 1j * rng.standard_normal((5, 400))).astype(np.complex64)
    for cutoff in (12.0, 1.0):
        f = butter_lowpass(cutoff, 1000.0)
        np.testing.assert_array_equal(_sosfiltfilt_rounded(f.sos, f.zi, f.padlen, x),
                                      signal.sosfiltfilt(f.sos, x, axis=1))
