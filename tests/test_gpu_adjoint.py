"""Adjoint of split-precision lattice BP against FP64 torch autograd and finite differences.

The FP64 reference is a plain torch restatement of the reference's direct BP on
points (fast_bp/ffbp.py:43-55 with sample1, ffbp.py:17-29), differentiated by
torch autograd.  Tolerances (relative L2 over all pulses):
* adjoint vs FP64 autograd: position, phase and weight gradients <= 1e-4;
* adjoint vs central differences of the split forward (h = 1e-4 m, 1e-4 rad): <= 2e-3.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ADJ_TOL = 1e-4
FD_TOL = 2e-3


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build
    build.build()
    from bp_project_gb300 import _native
    _native.load()
    return _native


def _lagrange(t):
    return (-t * (t - 1) * (t - 2) / 6, (t + 1) * (t - 1) * (t - 2) / 2,
            -(t + 1) * t * (t - 2) / 2, (t + 1) * t * (t - 1) / 6)


def torch_lattice_bp(data, pos, weight, phase, origin, step_row, step_col, rows, cols, range_start, data_dr, k,
                     chunk=32):
    """FP64 differentiable direct BP on a lattice (complex128 [rows, cols])."""
    dev = pos.device
    f64 = torch.float64
    i = torch.arange(rows, dtype=f64, device=dev)[:, None, None]
    j = torch.arange(cols, dtype=f64, device=dev)[None, :, None]
    pts = (torch.tensor(origin, dtype=f64, device=dev) + i * torch.tensor(step_row, dtype=f64, device=dev)
           + j * torch.tensor(step_col, dtype=f64, device=dev)).reshape(-1, 3)
    x = data.to(torch.complex128)
    samples = x.shape[1]
    img = torch.zeros(pts.shape[0], dtype=torch.complex128, device=dev)
    for c0 in range(0, pos.shape[0], chunk):
        c1 = min(c0 + chunk, pos.shape[0])
        d = torch.linalg.norm(pts[None] - pos[c0:c1, None, :], dim=-1)
        q = (d - range_start) / data_dr
        fl = torch.floor(q).detach()
        t = q - fl
        valid = (fl >= 1) & (fl <= samples - 3)
        idx = fl.clamp(1, samples - 3).long()
        rowsel = x[c0:c1]
        v = torch.zeros_like(d, dtype=torch.complex128)
        for a, wa in enumerate(_lagrange(t)):
            v = v + wa * torch.gather(rowsel, 1, idx + (a - 1))
        v = torch.where(valid, v, torch.zeros_like(v))
        ang = k * d + phase[c0:c1, None]
        img = img + (weight[c0:c1, None] * v * torch.polar(torch.ones_like(ang), ang)).sum(0)
    return img.reshape(rows, cols)


def _scene(tilt, coarse=1.0):
    from bp_project_gb300 import scenes
    cfg = scenes.scaled(scenes.CONFIGS["c3"], pulses=256, image_side=128)
    sc = scenes.synthesize(cfg, device="cuda")
    lat = sc.lattice
    step_row = np.array(lat.step_row, float) * coarse
    step_col = np.array(lat.step_col, float) * coarse
    origin = np.array(lat.origin, float) + 0.5 * (1.0 - coarse) * lat.rows * (step_row / coarse + step_col / coarse)
    if tilt:
        step_row = step_row + np.array([0.0, 0.0, 0.05])
    rng = np.random.default_rng(7)
    phase = sc.phase + rng.normal(0.0, 0.3, sc.phase.shape)
    weight = sc.weight * (1.0 + 0.1 * rng.standard_normal(sc.weight.shape))
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a)).to("cuda", dt)
    return dict(data=dev(sc.data, torch.complex64), pos=dev(sc.position, torch.float64),
                weight=dev(weight, torch.float64), phase=dev(phase, torch.float64),
                origin=tuple(origin), step_row=tuple(step_row), step_col=tuple(step_col),
                rows=lat.rows, cols=lat.cols, range_start=sc.range_start, data_dr=sc.data_dr, k=sc.k)


def _loss(img, target):
    """Intensity plus a correlation term: exercises both G = 2I and a fixed complex G."""
    img = img.to(torch.complex128)
    return (img.abs() ** 2).sum() * 1e-6 + (target.conj() * img).real.sum()


def _rel(a, b):
    a = a.detach().double().cpu().numpy().ravel()
    b = b.detach().double().cpu().numpy().ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("tilt,coarse", [(False, 1.0), (True, 1.0), (False, 6.0)])
def test_adjoint_matches_fp64_autograd(lib, tilt, coarse):
    """coarse = 6: 3 m steps, so every 32 x 32 tile is outside the fast path's precision envelope and the
    forward and adjoint run their two-float fallbacks."""
    from bp_project_gb300.autograd import backproject_lattice
    s = _scene(tilt, coarse)
    geo = (s["origin"], s["step_row"], s["step_col"], s["rows"], s["cols"], s["range_start"], s["data_dr"], s["k"])
    g = torch.Generator(device="cuda").manual_seed(3)
    target = torch.randn((s["rows"], s["cols"]), dtype=torch.complex128, device="cuda", generator=g)

    ins = [s["pos"].clone().requires_grad_(), s["phase"].clone().requires_grad_(),
           s["weight"].clone().requires_grad_()]
    img = backproject_lattice(s["data"], ins[0], ins[2], ins[1], *geo)
    _loss(img, target).backward()

    ref_ins = [s["pos"].clone().requires_grad_(), s["phase"].clone().requires_grad_(),
               s["weight"].clone().requires_grad_()]
    ref_img = torch_lattice_bp(s["data"], ref_ins[0], ref_ins[2], ref_ins[1], *geo)
    _loss(ref_img, target).backward()

    e_img = _rel(torch.view_as_real(img.detach().to(torch.complex128)), torch.view_as_real(ref_img.detach()))
    errs = [_rel(a.grad, b.grad) for a, b in zip(ins, ref_ins)]
    print(f"tilt={tilt} coarse={coarse}: image {e_img:.2e}, grad pos {errs[0]:.2e}, phase {errs[1]:.2e}, "
          f"weight {errs[2]:.2e}")
    assert e_img <= 1e-5
    assert max(errs) <= ADJ_TOL


def test_adjoint_matches_finite_differences(lib):
    from bp_project_gb300.autograd import backproject_lattice
    s = _scene(False)
    geo = (s["origin"], s["step_row"], s["step_col"], s["rows"], s["cols"], s["range_start"], s["data_dr"], s["k"])
    g = torch.Generator(device="cuda").manual_seed(5)
    target = torch.randn((s["rows"], s["cols"]), dtype=torch.complex128, device="cuda", generator=g)

    def loss(pos, phase):
        with torch.no_grad():
            return float(_loss(backproject_lattice(s["data"], pos, s["weight"], phase, *geo), target))

    pos = s["pos"].clone().requires_grad_()
    phase = s["phase"].clone().requires_grad_()
    _loss(backproject_lattice(s["data"], pos, s["weight"], phase, *geo), target).backward()
    fd, an = [], []
    for n in (0, 77, 128, 255):
        for c in range(3):
            h = 1e-4
            p1, p2 = s["pos"].clone(), s["pos"].clone()
            p1[n, c] += h
            p2[n, c] -= h
            fd.append((loss(p1, s["phase"]) - loss(p2, s["phase"])) / (2 * h))
            an.append(float(pos.grad[n, c]))
        h = 1e-4
        f1, f2 = s["phase"].clone(), s["phase"].clone()
        f1[n] += h
        f2[n] -= h
        fd.append((loss(s["pos"], f1) - loss(s["pos"], f2)) / (2 * h))
        an.append(float(phase.grad[n]))
    fd, an = np.array(fd), np.array(an)
    err = float(np.linalg.norm(fd - an) / np.linalg.norm(fd))
    print(f"finite differences: rel err {err:.2e}")
    assert err <= FD_TOL


def test_adjoint_is_deterministic(lib):
    from bp_project_gb300 import _native as nat
    from bp_project_gb300.autograd import adjoint
    s = _scene(False)
    lat = nat.lattice(s["origin"], s["step_row"], s["step_col"], s["rows"], s["cols"])
    grad = torch.randn((s["rows"], s["cols"]), dtype=torch.complex64, device="cuda")
    a = adjoint(s["data"], s["pos"], s["weight"], s["phase"], lat, s["range_start"], s["data_dr"], s["k"], grad)
    b = adjoint(s["data"], s["pos"], s["weight"], s["phase"], lat, s["range_start"], s["data_dr"], s["k"], grad)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    only_phase = adjoint(s["data"], s["pos"], s["weight"], s["phase"], lat, s["range_start"], s["data_dr"], s["k"],
                         grad, want=(False, True, False))
    assert only_phase[0] is None and torch.equal(only_phase[1], a[1])
