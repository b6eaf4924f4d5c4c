"""Point-target precision on the 30 km, 8192-pulse scene: split precision against FP64.

Bar: the peak pixel index of every target's fine patch equals the FP64 one, and
IRW (as 10 log10 of the width ratio), PSLR and ISLR on range and azimuth cuts
through every target stay within 0.05 dB of FP64.  The FP64 GPU path itself is
checked against the CPU oracle on one target's points.
"""
import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu, pytest.mark.slow]

DB_TOL = 0.05


@pytest.fixture(scope="module")
def c2_scene():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build, scenes
    build.build()
    return scenes.synthesize(scenes.CONFIGS["c2"], device="cuda")


def test_split_point_targets_match_fp64(c2_scene):
    from bp_project_gb300.precision_report import markdown, point_target_report
    rep = point_target_report(scene=c2_scene, modes=("split", "fp32"))
    print(markdown(rep))
    s = rep["modes"]["split"]
    assert s["peaks_all_equal"]
    assert s["max_delta_irw_db"] <= DB_TOL
    assert s["max_delta_pslr_db"] <= DB_TOL
    assert s["max_delta_islr_db"] <= DB_TOL
    assert s["relative_l2_error"] <= 1e-5


def test_fp64_points_match_oracle_at_30km(c2_scene):
    from bp_project_gb300 import core
    from bp_project_gb300.precision_report import _cuts, _patch
    from oracle import reference as ora
    sc = c2_scene
    tgt = sc.targets[0]
    _, xs, ys = _cuts(tgt, 3.0, 129)
    pts = np.vstack([_patch(tgt, 0.75, 24), xs, ys])
    ref = ora.backproject_points(sc.data, sc.position, pts, sc.range_start, sc.data_dr, sc.k, sc.weight, sc.phase,
                                 c128=True)[1]
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda()
    for mode, tol in (("fp64", 1e-6), ("split", 1e-5)):
        out = core.backproject_points(dev(sc.data), dev(sc.position), dev(sc.weight), dev(sc.phase), dev(pts),
                                      sc.range_start, sc.data_dr, sc.k, mode=mode).cpu().numpy()
        e = rel_err(ref, out)
        print(f"{mode} vs oracle at 30 km: {e:.2e}")
        assert e <= tol
