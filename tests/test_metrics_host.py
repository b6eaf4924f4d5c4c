"""Quality metrics against the reference's sar_quality/metrics.py outputs (tests/golden/metrics.npz)."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden import metrics_cases  # noqa: E402


def test_metrics_match_reference(golden):
    from bp_project_gb300 import metrics
    g = golden("metrics")
    img, est, cuts = metrics_cases()
    fm = metrics.focus_metrics(img)
    np.testing.assert_allclose([fm["entropy_nats"], fm["normalized_entropy"], fm["intensity_contrast"],
                                fm["amplitude_contrast"], fm["brightest_1pct_energy_fraction"]], g["focus"],
                               rtol=1e-12)
    fd = metrics.fidelity(img, est)
    np.testing.assert_allclose([fd["relative_complex_error"], fd["ser_db"], fd["complex_coherence"],
                                fd["phase_bias_deg"], fd["phase_std_deg_above_minus30db"],
                                fd["phase_mask_samples"]], g["fidelity"], rtol=1e-12)
    for i, (x, z) in enumerate(cuts):
        m = metrics.impulse_metrics(x, z)
        np.testing.assert_allclose([m["irw_m"], m["peak_offset_m"], m["pslr_db"], m["islr_db"],
                                    *m["mainlobe_bounds_m"], *m["mainlobe_minima_db"]], g[f"impulse{i}"], rtol=1e-12)


def test_metrics_invalid_inputs():
    from bp_project_gb300 import metrics
    assert metrics.focus_metrics(np.zeros((4, 4), np.complex64))["valid"] is False
    assert metrics.impulse_metrics(np.arange(5.0), np.zeros(5))["valid"] is False
    x = np.linspace(-1, 1, 9)
    assert metrics.impulse_metrics(x, np.ones(9))["valid"] is False  # no half-power crossing
