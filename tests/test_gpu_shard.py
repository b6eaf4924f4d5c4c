"""Multi-GPU partitions of direct BP (bp_project_gb300.shard), emulated on one GPU: every rank's
share runs as its own launch (no launch waits on another), then the bands are assembled and the
partial images summed in rank order with the library's add kernel, exactly as the ranks' collectives
would.  Row bands must give the one-GPU image bit for bit; pulse ranges the one-GPU image of
pulse_split = world bit for bit.  The collectives themselves are tested with gloo ranks on the CPU
(tests/test_shard_host.py)."""
import numpy as np
import pytest

from conftest import rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build, scenes
    build.build()
    cfg = scenes.scaled(scenes.CONFIGS["c1"], pulses=512, samples=4096, image_side=400)
    sc = scenes.synthesize(cfg, device="cuda")
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sc.data, sc.position, sc.weight, sc.phase)]
    lat = sc.lattice
    geo = (tuple(lat.origin), tuple(lat.step_row), tuple(lat.step_col), lat.rows, lat.cols, sc.range_start,
           sc.data_dr, sc.k)
    return sc, dev, geo


@pytest.mark.parametrize("world", [2, 3, 8])
def test_row_bands_reproduce_the_one_gpu_image(scene, world):
    from bp_project_gb300 import core, shard
    sc, dev, geo = scene
    full = core.backproject_lattice(*dev, *geo, mode="split", pulse_split=1)
    rows = geo[3]
    image = torch.empty_like(full)
    for rank, (b, e) in enumerate(shard.row_bands(rows, world)):
        band = shard.lattice_band(*dev, *geo, rank=rank, world=world, pulse_split=1)
        assert band.shape == (e - b, geo[4])
        image[b:e] = band
    torch.cuda.synchronize()
    assert torch.equal(image, full)


@pytest.mark.parametrize("world", [2, 4, 7])
def test_pulse_ranges_reproduce_the_one_gpu_pulse_split(scene, world):
    from bp_project_gb300 import core, shard
    sc, dev, geo = scene
    want = core.backproject_lattice(*dev, *geo, mode="split", pulse_split=world)
    parts = [shard.lattice_pulse_part(*dev, *geo, rank=r, world=world) for r in range(world)]
    acc = parts[0].clone()
    for p in parts[1:]:
        core.add_inplace(acc, p)
    torch.cuda.synchronize()
    assert torch.equal(acc, want)
    one = core.backproject_lattice(*dev, *geo, mode="split", pulse_split=1)
    assert rel_err(one.cpu().numpy(), acc.cpu().numpy()) <= 1e-6


def test_polar_pulse_ranges_reproduce_the_one_gpu_pulse_split(golden):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bp_project_gb300 import build, core, shard
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    build.build()
    g = golden("operator_validation")
    range_start, data_dr, fc, k, side, *extent = g["case1_scalars"]
    plan = build_ffbp_plan(g["case1_position"], fc, extent, side=int(side), leaf_size=8, range_spacing=0.5,
                           angular_oversample=3.0)
    dev = [torch.from_numpy(np.ascontiguousarray(g["case1_" + n])).cuda()
           for n in ("data", "position", "weight", "phase")]
    world = 3
    want = core.direct_polar(*dev, plan.grid(), range_start, data_dr, k, mode="split", pulse_split=world)
    parts = [shard.polar_pulse_part(*dev, plan.grid(), range_start, data_dr, k, rank=r, world=world)
             for r in range(world)]
    acc = parts[0].clone()
    for p in parts[1:]:
        core.add_inplace(acc, p)
    torch.cuda.synchronize()
    assert torch.equal(acc, want)
    assert rel_err(g["case1_direct"], acc.cpu().numpy()) <= 1e-5


@pytest.mark.parametrize("world", [2, 3, 4])
def test_ffbp_subtrees_reproduce_the_one_gpu_image(scene, world):
    """FFBP over ranks: each rank's subtrees as their own plans, then the top of the tree from the
    subtree roots' images (external nodes); the image equals the one-GPU plan's bit for bit."""
    from bp_project_gb300 import core, shard
    from bp_project_gb300.gpu_backend import build_ffbp_plan
    sc, dev, geo = scene
    cfg = sc.config
    plan = build_ffbp_plan(sc.position, cfg.fc, sc.extent, side=1, leaf_size=cfg.leaf_size,
                           range_spacing=cfg.range_spacing, angular_oversample=cfg.angular_oversample)
    prog = core.FFBPProgram(plan.nodes(), plan.crop_r, plan.crop_u, mode="split")
    want = prog.execute(*dev, sc.range_start, sc.data_dr, sc.k).clone()
    prog.close()
    subtrees, top, external = shard.ffbp_cut(plan.nodes()[0], world)
    images = {}
    for r, (b, e) in enumerate(shard.subtree_ranges(len(subtrees), world)):  # rank by rank
        images.update(shard.ffbp_subtree_images(*dev, subtrees, range(b, e), sc.range_start, sc.data_dr, sc.k))
    got = shard.ffbp_top(*dev, top, external, images, plan.crop_r, plan.crop_u, sc.range_start, sc.data_dr, sc.k)
    torch.cuda.synchronize()
    assert torch.equal(got, want)
