"""The further constraint operators of the reference (sphere collision,
inter-particle collision, glue) against the oracle's FP32 restatement: bit-exact
positions, glue lists and ids that follow the neighbour search's reorder."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ctx(st, maxn=160, L=5, grid=((-8, -8, -8), (120, 120, 120))):
    from apbf_gb300.api import Context

    n = st["position"].shape[0]
    ctx = Context(particle_capacity=n, max_neighbors=maxn, max_log2res=L)
    ctx.set_scene(grid[0], grid[1], L, (0.0, 0.0, 0.0))
    ctx.upload(st)
    return ctx


def _searched(orc, ctx, grid=((-8, -8, -8), (120, 120, 120)), L=5):
    """Device neighbour search, then an oracle state with the device's rows."""
    from apbf_gb300.api import neighborhood_green

    neighborhood_green().set_data(ctx).set_range_scale(1.0).set_position_range(grid[0], grid[1], L).apply()
    st, _ = ctx.download()
    fs = orc.FluidState(st)
    n = st["position"].shape[0]
    nb = ctx.neighbors_view()
    cnt = nb["count"][:n].cpu().numpy()
    idx = nb["index"][:, :n].cpu().numpy().view(np.uint32)
    orc.set_rows(fs, [idx[:c, i].copy() for i, c in enumerate(cnt)])  # the device's row order
    return fs


@pytest.mark.parametrize("hollow", [True, False])
def test_sphere_collision_bit_exact(orc, hollow):
    from apbf_gb300.api import sphere_collision

    rng = np.random.default_rng(1 if hollow else 2)
    st = scenes.make_state(rng.uniform(0, 100, size=(8000, 3)))
    st["radius"][:] = rng.uniform(0.5, 2.0, size=8000).astype(np.float32)
    ctx = _ctx(st)
    c, R = (50.0, 48.0, 52.0), 35.0
    sphere_collision().set_data(ctx).set_sphere(c, R, hollow).apply()
    g, _ = ctx.download()
    fs = orc.FluidState(st)
    orc.sphere_collision(fs, c, R, hollow)
    assert np.array_equal(g["position"], fs.state()["position"])
    moved = np.any(g["position"][:, :3] != st["position"][:, :3], axis=1).mean()
    assert 0.1 < moved < 0.9
    ctx.close()


@pytest.mark.parametrize("adaptive_radii", [False, True])
def test_inter_particle_collision_bit_exact(orc, adaptive_radii):
    from apbf_gb300.api import inter_particle_collision

    rng = np.random.default_rng(3)
    pos = scenes.lattice([10, 10, 10], [14, 14, 14], 1.6, 0.3, rng)  # overlapping unit spheres
    st = scenes.make_state(pos)
    if adaptive_radii:
        st["radius"][:] = rng.choice(np.float32([1.0, 1.26]), size=pos.shape[0])
        st["kernel_width"][:] = st["radius"] * 4.0
    ctx = _ctx(st)
    fs = _searched(orc, ctx)
    inter_particle_collision().set_data(ctx).apply()
    g, _ = ctx.download()
    orc.inter_particle_collision(fs)
    o = fs.state()
    assert np.array_equal(g["position"], o["position"])
    assert np.abs(g["position"][:, :3].astype(np.int64) - fs.state()["position"][:, :3]).max() == 0
    ctx.close()


def test_glue_bit_exact_and_follows_reorder(orc):
    from apbf_gb300.api import glue, neighborhood_green

    rng = np.random.default_rng(4)
    pos = scenes.lattice([10, 10, 10], [12, 12, 12], 2.2, 0.3, rng)
    st = scenes.make_state(pos)
    ctx = _ctx(st)
    fs = _searched(orc, ctx)
    gl = glue().set_data(ctx, capacity=200_000).set_stability(0.5)
    gl.applyNewGlue()
    g0, g1, gd = gl.view()
    o0, o1, od = orc.glue_generate(fs, 200_000)
    assert g0.size > 1000
    assert np.array_equal(g0, o0) and np.array_equal(g1, o1) and np.array_equal(gd, od)
    # stretch the glue (move every particle a little), then enforce it
    import torch

    v = ctx.fluid_view()
    n = st["position"].shape[0]

    sd, _ = ctx.download()
    moved = sd["position"].copy()
    moved[:, :3] += rng.integers(-40000, 40000, size=(n, 3)).astype(np.int32)
    v["position"][:n].copy_(torch.from_numpy(moved).cuda())
    gl.apply()
    g, _ = ctx.download()
    fo = orc.FluidState({**sd, "position": moved})
    orc.glue_apply(fo, o0, o1, od, 0.5)
    assert np.array_equal(g["position"], fo.state()["position"])
    # a neighbour search reorders the particles: the glue names the same particles
    before = {tuple(sorted((tuple(g["position"][a, :3]), tuple(g["position"][b, :3])))) for a, b in zip(g0, g1)}
    neighborhood_green().set_data(ctx).set_range_scale(1.0).set_position_range((-8, -8, -8), (120, 120, 120),
                                                                                5).apply()
    h, _ = ctx.download()
    a0, a1, _ = gl.view()
    after = {tuple(sorted((tuple(h["position"][a, :3]), tuple(h["position"][b, :3])))) for a, b in zip(a0, a1)}
    assert before == after
    ctx.close()


def test_save_particle_info_files(tmp_path):
    """save_particle_info: the reference's files, one value per particle in list order
    (data.csv sorted by the distance to the centre), values as the state has them."""
    from apbf_gb300.api import neighborhood_green

    rng = np.random.default_rng(9)
    pos = scenes.lattice([10, 10, 10], [10, 10, 10], 2.0, 0.2, rng)
    st = scenes.make_state(pos)
    ctx = _ctx(st)
    neighborhood_green().set_data(ctx).set_range_scale(1.0).set_position_range((-8, -8, -8), (120, 120, 120),
                                                                                5).apply()
    g, _ = ctx.download()
    n = g["position"].shape[0]
    cnt = ctx.neighbors_view()["count"][:n].cpu().numpy()
    ctx.save_particle_info(tmp_path, center=(0.0, 10.0, -60.0))
    names = ["centerDist", "radius", "neighborCount", "kernelWidth", "targetRadius", "boundaryDistance"]
    vals = {k: np.array([float(x) for x in (tmp_path / f"{k}.txt").read_text().split(";") if x]) for k in names}
    p = g["position"][:, :3].astype(np.float32) / np.float32(262144.0)
    cd = np.sqrt(np.sum((p - np.float32([0, 10, -60])) ** 2, axis=1))
    assert all(v.size == n for v in vals.values())
    assert np.allclose(vals["centerDist"], cd, rtol=1e-5)  # 6 significant digits
    assert np.array_equal(vals["neighborCount"], cnt)
    assert np.allclose(vals["radius"], g["radius"]) and np.allclose(vals["kernelWidth"], g["kernel_width"], rtol=1e-5)
    lines = (tmp_path / "data.csv").read_text().strip().splitlines()
    assert lines[0].startswith("center distance,boundary distance,kernel width,neighbor count")
    d = np.array([[float(x) for x in ln.split(",")] for ln in lines[1:]])
    assert d.shape == (n, 10) and np.all(np.diff(d[:, 0]) >= 0)
    ctx.close()
