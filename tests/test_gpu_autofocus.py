"""GPU autofocus against the reference's own outputs (tests/golden/autofocus.npz).

Tolerances: sosfiltfilt kernel vs scipy <= 1e-12 relative (FP64 recursion,
complex64 odd extension); estimate_update deltas within 1e-4 of the largest
reference correction (the target contributions are computed in FP32 on the
GPU, complex64 in the reference); pick_targets points identical and powers
within 1e-6 (|z| of complex64 on the GPU vs numpy).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import autofocus_scene as scene  # noqa: E402

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


def _rel_max(est, ref):
    est, ref = np.asarray(est), np.asarray(ref)
    return float(np.abs(est - ref).max() / np.abs(ref).max())


def _sosfiltfilt_rounded(sos, zi, padlen, x):
    """Forward-backward biquad cascade with every product and sum rounded on its own (numpy ufuncs
    never contract), over an odd extension formed in float32 per component: the arithmetic the
    kernel performs, for an exact comparison."""
    def ext(c):
        c = c.astype(np.float32)
        left = np.float32(2) * c[:, :1] - c[:, padlen:0:-1]
        right = np.float32(2) * c[:, -1:] - c[:, -2:-padlen - 2:-1]
        return np.concatenate([left, c, right], axis=1).astype(np.float64)

    def run(v):
        out = np.empty_like(v)
        z = [[zi[s, 0] * v[:, 0], zi[s, 1] * v[:, 0]] for s in range(len(sos))]
        for i in range(v.shape[1]):
            cur = v[:, i]
            for s, (b0, b1, b2, _, a1, a2) in enumerate(sos):
                y = b0 * cur + z[s][0]
                z[s][0] = (b1 * cur - a1 * y) + z[s][1]
                z[s][1] = b2 * cur - a2 * y
                cur = y
            out[:, i] = cur
        return out

    ch = np.concatenate([ext(x.real), ext(x.imag)])
    y = run(run(ch)[:, ::-1])[:, ::-1][:, padlen:padlen + x.shape[1]]
    return y[:x.shape[0]] + 1j * y[x.shape[0]:]


@pytest.mark.parametrize("shape,cutoff,fs", [((7, 300), 12.0, 1000.0), ((144, 2048), 1.0, 1000.0), ((1, 16), 50, 400)])
def test_sosfiltfilt_matches_scipy(lib, shape, cutoff, fs):
    from scipy import signal
    from bp_project_gb300.autofocus import butter_lowpass, sosfiltfilt
    rng = np.random.default_rng(sum(shape))
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    f = butter_lowpass(cutoff, fs)
    ref = signal.sosfiltfilt(f.sos, x, axis=1)
    est = sosfiltfilt(torch.from_numpy(x).cuda(), f).cpu().numpy()
    assert est.dtype == np.complex128
    err = _rel_max(est, ref)
    print(f"sosfiltfilt {shape}: {err:.2e}")
    assert err <= 1e-12
    # bit for bit the separately rounded recursion (the pipelined cascade changes no rounding)
    np.testing.assert_array_equal(est, _sosfiltfilt_rounded(f.sos, f.zi, f.padlen, x))


def test_sosfiltfilt_rejects_short_rows(lib):
    from bp_project_gb300.autofocus import butter_lowpass, sosfiltfilt
    with pytest.raises(ValueError, match="padlen"):
        sosfiltfilt(torch.zeros((2, 15), dtype=torch.complex64, device="cuda"), butter_lowpass(12.0, 1000.0))


@pytest.mark.parametrize("name", ["recovery", "cluttered"])
def test_estimate_update_matches_reference(golden, lib, name):
    from bp_project_gb300.autofocus import estimate_update
    g = golden("autofocus")
    s = getattr(scene, name)()
    delta, stats = estimate_update(torch.from_numpy(s.data).cuda(), torch.from_numpy(s.pos).cuda(),
                                   torch.from_numpy(s.points).cuda(), s.r_start, s.dr, s.k, s.prf, s.cutoff)
    delta = delta.cpu().numpy()
    err = _rel_max(delta, g[f"{name}_delta"])
    print(f"estimate_update {name}: {err:.2e}, coherence {stats['median_gradient_coherence']:.6f}")
    assert err <= 1e-4
    assert abs(stats["median_gradient_coherence"] - float(g[f"{name}_coherence"])) < 1e-5
    if name == "recovery":  # validate_autofocus.py:20
        before = np.sqrt(np.mean(s.err[:, :2] ** 2))
        assert np.sqrt(np.mean((s.err + delta)[:, :2] ** 2)) < 0.35 * before


@pytest.mark.parametrize("tiles", [(12, 12), (7, 5)])
def test_pick_targets_matches_reference(golden, lib, tiles):
    from bp_project_gb300.autofocus import pick_targets
    from bp_project_gb300.ffbp import PolarImage
    g = golden("autofocus")
    p = scene.picks()
    result = PolarImage(torch.from_numpy(p.image).cuda(), p.origin, p.r0, p.dr, p.u0, p.du, p.side)
    pts, powers = pick_targets(result, *tiles)
    key = f"picks_{tiles[0]}x{tiles[1]}"
    np.testing.assert_allclose(pts.cpu().numpy(), g[key + "_points"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(powers.cpu().numpy(), g[key + "_powers"], rtol=1e-6)


def test_entropy_autofocus_refocuses_injected_errors(lib):
    """Config-3 geometry at 512 pulses x 128^2: the gradient autofocus brings the entropy of the
    image formed on the perturbed track below the entropy of the image on the true track plus 1%."""
    from bp_project_gb300 import scenes
    from bp_project_gb300.autofocus import entropy_autofocus, image_entropy
    from bp_project_gb300.autograd import backproject_lattice
    cfg = scenes.scaled(scenes.CONFIGS["c3"], pulses=512, image_side=128)
    sc = scenes.synthesize(cfg, device="cuda")
    err, phase_err = scenes.inject_trajectory_error(sc)
    lat = sc.lattice
    geo = (tuple(lat.origin), tuple(lat.step_row), tuple(lat.step_col), lat.rows, lat.cols,
           sc.range_start, sc.data_dr, sc.k)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda()
    data, w = dev(sc.data), dev(sc.weight)
    truth = float(image_entropy(backproject_lattice(data, dev(sc.position), w, dev(sc.phase), *geo)))
    pos, phase = dev(sc.position + err), dev(sc.phase + phase_err)
    start = float(image_entropy(backproject_lattice(data, pos, w, phase, *geo)))
    res = entropy_autofocus(data, pos, w, phase, *geo, steps=60)
    print(f"entropy: truth {truth:.4f}, perturbed {start:.4f}, autofocus {res.entropy:.4f} "
          f"after {res.evaluations} evaluations, {res.history[-1][0]:.2f} s")
    assert start > truth + 0.5
    assert res.entropy < truth * 1.01


@pytest.mark.parametrize("shape,tiles", [((37, 53), (7, 5)), ((64, 64), (12, 12)), ((300, 211), (12, 12))])
def test_tile_argmax_matches_numpy(lib, shape, tiles):
    """sarbp_tile_argmax: numpy.array_split tiles, per-tile np.argmax (first index of the maximum), also on
    an image whose tiles are constant (every cell ties)."""
    from bp_project_gb300 import _native as nat, core
    nr, nu = shape
    rows = np.array_split(np.arange(nr), tiles[0])
    cols = np.array_split(np.arange(nu), tiles[1])
    rng = np.random.default_rng(nr * nu)
    for img in (rng.random(shape, dtype=np.float32), np.ones(shape, np.float32),
                np.round(rng.random(shape, dtype=np.float32) * 4) / 4):
        a = torch.from_numpy(img).cuda()
        n = tiles[0] * tiles[1]
        tmax = torch.empty(n, dtype=torch.float32, device="cuda")
        first = torch.empty(n, dtype=torch.int64, device="cuda")
        nat.check(nat.load().sarbp_tile_argmax(core._ptr(a), nr, nu, tiles[0], tiles[1], core._ptr(tmax),
                                               core._ptr(first), core.stream_handle()), "tile_argmax")
        want_max, want_idx = [], []
        for r in rows:
            for c in cols:
                sub = img[r[0]:r[-1] + 1, c[0]:c[-1] + 1]
                i, j = np.unravel_index(np.argmax(sub), sub.shape)
                want_max.append(sub[i, j])
                want_idx.append((r[0] + i) * nu + c[0] + j)
        assert np.array_equal(tmax.cpu().numpy(), np.array(want_max, np.float32))
        assert np.array_equal(first.cpu().numpy(), np.array(want_idx))
