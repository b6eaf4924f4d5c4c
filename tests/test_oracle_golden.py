"""Pin the CPU oracle against outputs of the reference implementation itself.

The fixtures in tests/golden were produced by tests/golden/make_golden.py,
which runs the reference's fast_bp/ffbp.py and build_ffbp_plan unchanged.
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import reference as ora
from oracle.plan import plan_ffbp

FP64_TOL = 1e-12  # oracle and reference are both FP64; differences are last-ulp libm/rounding effects


def _plan_matches(gold, prefix, plan):
    geom, idx = plan.tables()
    assert idx.shape == gold[prefix + "idx"].shape
    np.testing.assert_array_equal(idx, gold[prefix + "idx"])
    np.testing.assert_allclose(geom, gold[prefix + "geom"], rtol=0, atol=1e-12 * np.abs(gold[prefix + "geom"]).max())
    np.testing.assert_array_equal(np.array([*plan.crop_r, *plan.crop_u]), gold[prefix + "crop"])
    c = plan.counts
    np.testing.assert_array_equal([c["leaves"], c["merges"], c["leaf_pixel_pulse_products"], c["merged_pixels"],
                                   len(plan.nodes)], gold[prefix + "counts"])


@pytest.mark.parametrize("name", ["c0", "c1", "c3", "validate", "left"])
def test_plan_matches_reference_planner(golden, name):
    g = golden("plans")
    fc, rmin, rmax, umin, umax, side, leaf, rs, osr = g[f"{name}_args"]
    plan = plan_ffbp(g[f"{name}_position"], fc, (rmin, rmax, umin, umax), side=int(side), leaf_size=int(leaf),
                     range_spacing=rs, angular_oversample=osr)
    _plan_matches(g, f"{name}_", plan)


@pytest.mark.parametrize("case", [0, 1])
def test_operator_validation_recipe(golden, case):
    g = golden("operator_validation")
    p = f"case{case}_"
    range_start, data_dr, fc, k, side, *extent = g[p + "scalars"]
    side = int(side)
    plan = plan_ffbp(g[p + "position"], fc, extent, side=side, leaf_size=8, range_spacing=0.5,
                     angular_oversample=3.0)
    _plan_matches(g, p, plan)
    root_r0, root_dr, root_u0, root_du, nr, nu = g[p + "root"]
    direct = ora.bp_polar(g[p + "data"], g[p + "position"], plan.root.origin, root_r0, root_dr, int(nr), root_u0,
                          root_du, int(nu), range_start, data_dr, k, g[p + "weight"], g[p + "phase"], side)
    assert rel_err(g[p + "direct"], direct) < 1e-7
    img, counts = ora.form_ffbp(g[p + "data"], g[p + "position"], range_start, data_dr, fc, extent, side=side,
                                leaf_size=8, range_spacing=0.5, angular_oversample=3.0, weight=g[p + "weight"],
                                phase=g[p + "phase"])
    assert img.image.shape == g[p + "ffbp"].shape
    assert rel_err(g[p + "ffbp"], img.image) < 1e-7
    np.testing.assert_allclose([*img.origin, img.r0, img.dr, img.u0, img.du], g[p + "ffbp_axes"], rtol=FP64_TOL)


def test_recorded_reference_peaks(golden):
    """Peak pixels recorded by the reference (results/gpu_baseline/operator_validation.json, case k<0, side +1)."""
    g = golden("operator_validation")
    ff = np.abs(g["case0_ffbp"])
    di = np.abs(g["case0_direct"])
    assert np.unravel_index(ff.argmax(), ff.shape) == (7, 73)
    assert np.unravel_index(di.argmax(), di.shape) == (33, 29)


def test_points_case(golden):
    g = golden("points")
    r_start, ddr, fc, k, *extent = g["scalars"]
    direct = ora.backproject_points(g["data"], g["position"], g["points"], r_start, ddr, k, g["weight"], g["phase"])
    assert rel_err(g["direct"], direct) < 1e-7
    img, counts = ora.form_ffbp(g["data"], g["position"], r_start, ddr, fc, extent, leaf_size=32, range_spacing=0.5,
                                angular_oversample=2.0, weight=g["weight"])
    assert rel_err(g["ffbp"], img.image) < 1e-7
    np.testing.assert_array_equal([counts[n] for n in ("leaves", "merges", "leaf_pixel_pulse_products",
                                                        "merged_pixels")], g["counts"])
    ev = ora.evaluate_image(img.image, img.origin, img.r0, img.dr, img.u0, img.du, g["eval_points"], k)
    assert rel_err(g["evaluate"], ev) < 1e-6
    tc = ora.target_contributions(g["data"], g["position"], g["targets"], r_start, ddr, k)
    assert rel_err(g["contrib"], tc) < 1e-7


def test_kernels_case(golden):
    g = golden("kernels")
    sr0, sdr, su0, sdu, r0, dr, nr, u0, du, nu, k = g["grid"]
    for side in (1, -1):
        out = ora.regrid(g["image"], g["src_origin"], sr0, sdr, su0, sdu, g["dst_origin"], r0, dr, int(nr), u0, du,
                         int(nu), k, side)
        assert rel_err(g[f"regrid_side{side}"], out) < 1e-7
    # The fixtures come from the reference run as pure Python, where numpy 2 evaluates
    # python-float * complex64-scalar in complex64; under Numba (and in the oracle) the
    # products are complex128.  The two agree to complex64 rounding (~6e-8 relative per term).
    s1 = np.array([ora.sample1(g["row"], float(q)) for q in g["q"]])
    np.testing.assert_allclose(s1, g["sample1"], rtol=1e-6, atol=1e-6)
    assert np.array_equal(s1 == 0, g["sample1"] == 0)
    s2 = np.array([ora.sample2(g["image"], float(a), float(b)) for a, b in zip(g["qr"], g["qu"])])
    np.testing.assert_allclose(s2, g["sample2"], rtol=1e-6, atol=1e-6)
    assert np.array_equal(s2 == 0, g["sample2"] == 0)
    cw = np.array([ora.cubic_weights(float(t)) for t in g["t"]])
    np.testing.assert_array_equal(cw, g["cubic"])
    # Support rule (ffbp.py:27): zero unless 1 <= floor(q) <= len-3.
    assert ora.sample1(g["row"], 0.999) == 0 and ora.sample1(g["row"], 62.0) == 0
    assert ora.sample1(g["row"], 1.0) != 0 and ora.sample1(g["row"], 61.999) != 0


def test_oracle_threads():
    assert ora.set_threads(0) >= 1
