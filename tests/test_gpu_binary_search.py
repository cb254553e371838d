"""GPU parity of neighborhood_binary_search::apply against the oracle: the 96-bit
position codes, the sort permutation, the reordered state and every neighbour row
(entries in the same order) bit-exact; the rows equal the Green search's as sets;
whole substeps with the binary search in lockstep with the oracle's."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ctx(cap, maxn=256, L=5):
    from apbf_gb300.api import Context

    return Context(particle_capacity=cap, max_neighbors=maxn, max_log2res=L)


def _random_state(n, seed, lo, hi, kw_lo, kw_hi, dups=0):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(lo, hi, size=(n, 3))
    if dups:
        pos[-dups:] = pos[:dups]  # equal positions: equal codes
    st = scenes.make_state(pos)
    st["kernel_width"] = rng.uniform(kw_lo, kw_hi, size=n).astype(np.float32)
    return st


def _device_rows(ctx):
    """Rows in the device's order."""
    n, _ = ctx.lengths()
    nb = ctx.neighbors_view()
    cnt = nb["count"][:n].cpu().numpy()
    idx = nb["index"][:, :n].cpu().numpy().view(np.uint32)
    return [idx[: cnt[i], i].astype(np.int64) for i in range(n)]


@pytest.mark.parametrize("seed,lo,hi,kw_lo,kw_hi,dups,scale", [
    (0, 0.0, 30.0, 2.0, 4.0, 0, 1.0),
    (1, -15.0, 15.0, 1.0, 7.5, 200, 1.0),   # across the sign boundary, equal codes
    (2, -20.0, 20.0, 3.0, 3.0, 0, 1.5),
])
def test_binary_search_parity(orc, seed, lo, hi, kw_lo, kw_hi, dups, scale):
    from apbf_gb300.api import neighborhood_binary_search

    st = _random_state(12000, seed, lo, hi, kw_lo, kw_hi, dups)
    n = st["position"].shape[0]
    transfers = {"source": np.arange(0, 400, 2, dtype=np.uint32), "target": np.arange(1, 401, 2, dtype=np.uint32),
                 "time_left": np.linspace(0.1, 1.0, 200).astype(np.float32)}
    ctx = _ctx(n, maxn=1024)  # radii up to 7.5 at 0.44 particles per unit volume: up to ~830 neighbours
    ctx.upload(st, transfers)
    neighborhood_binary_search().set_data(ctx).set_range_scale(scale).apply()
    info = ctx.check_status()
    g, gt = ctx.download()
    g_perm, _ = ctx.debug_sort()
    g_rows = _device_rows(ctx)
    g_codes = ctx.position_codes().cpu().numpy().view(np.uint32)
    fs = orc.FluidState(st, transfers=transfers)
    perm, codes, tot = orc.neighborhood_binary_search(fs, scale, 1 << 24)
    o = fs.state()
    assert np.array_equal(g_perm, perm)
    assert np.array_equal(g_codes, codes)
    for k in o:
        assert np.array_equal(g[k], o[k]), k
    ot = fs.transfers()
    for k in ot:
        assert np.array_equal(gt[k], ot[k]), k
    assert info.pairs == tot
    for i, (a, b) in enumerate(zip(g_rows, fs.rows())):
        assert np.array_equal(a, b), i
    ctx.close()


def test_binary_search_largest_level(orc):
    """Search radii of more than 2^30 units: cell level 31, two cells per axis (the
    offsets -1 and +1 name the same cell, scanned once)."""
    from apbf_gb300.api import neighborhood_binary_search

    st = _random_state(1500, 5, -3000.0, 3000.0, 4200.0, 9000.0)
    n = st["position"].shape[0]
    ctx = _ctx(n, maxn=1536)
    ctx.upload(st)
    neighborhood_binary_search().set_data(ctx).apply()
    info = ctx.check_status()
    g_rows = _device_rows(ctx)
    fs = orc.FluidState(st)
    _, _, tot = orc.neighborhood_binary_search(fs, 1.0, 1 << 24)
    assert info.pairs == tot
    for i, (a, b) in enumerate(zip(g_rows, fs.rows())):
        assert np.array_equal(a, b), i
    assert max(len(r) for r in g_rows) == n - 1 and all(len(set(r.tolist())) == len(r) for r in g_rows)
    ctx.close()


def test_rows_equal_green_as_sets():
    """The same neighbours as the Green search (the two sorts order the particles
    differently: particles are matched by position)."""
    from apbf_gb300.api import neighborhood_binary_search, neighborhood_green

    st = _random_state(20000, 7, 0.0, 40.0, 2.0, 6.0)
    n = st["position"].shape[0]
    out = []
    for method in ("green", "bs"):
        ctx = _ctx(n, maxn=512, L=5)
        ctx.upload(st)
        if method == "green":
            neighborhood_green().set_data(ctx).set_position_range((0, 0, 0), (40, 40, 40), 5).apply()
        else:
            neighborhood_binary_search().set_data(ctx).apply()
        ctx.check_status()
        g, _ = ctx.download()
        keys = [tuple(p) for p in g["position"][:, :3].tolist()]
        rows = _device_rows(ctx)
        out.append({keys[i]: {keys[j] for j in rows[i]} for i in range(n)})
        ctx.close()
    assert out[0] == out[1]


def test_substeps_with_binary_search_lockstep(orc):
    """apbf_substep with the binary search: each substep from the device's state on
    both sides; the neighbour search and reorder are exact, the Jacobi passes agree
    within the FP32 / FP64 tolerance of the Green substep tests."""
    from dataclasses import replace

    from apbf_gb300.api import Context

    spec = scenes.dam_break(n_side=12, seed=0, iterations=4)
    rng = np.random.default_rng(0)
    pos = scenes.lattice([20, 20, 20], [12] * 3, 1.8, 0.2, rng)
    spec = replace(spec, state=scenes.make_state(pos), box_min=np.zeros((0, 4), np.float32),
                   box_max=np.zeros((0, 4), np.float32))
    ctx = Context(particle_capacity=spec.n, max_neighbors=128, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1, solver_iterations=spec.iterations)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.set_neighborhood_search("binary_search")
    ctx.upload(spec.state)
    last_dt = 1.0
    for step in range(4):
        before, _ = ctx.download()
        ctx.substep(spec.dt)
        ctx.check_status()
        g, _ = ctx.download()
        fs = orc.FluidState(before)
        sc = orc.make_scene(orc.settings_from(ctx.settings), spec.grid_min, spec.grid_max, spec.log2res,
                            spec.acceleration, search_method=3)
        sc.last_dt = last_dt
        orc.substep(fs, sc, (spec.box_min, spec.box_max), np.float32(spec.dt), 1 << 22)
        last_dt = spec.dt
        o = fs.state()
        x = g["position"][:, :3].astype(np.int64)
        xo = o["position"][:, :3].astype(np.int64)
        assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), (step, np.abs(x - xo).max())
        assert np.array_equal(g["radius"], o["radius"])
    ctx.close()


def test_graph_substeps_same_with_either_search():
    """Whole-substep graphs pick up a change of the search (graphs captured with the
    other search are not replayed); adaptive substeps run with the binary search."""
    from apbf_gb300.api import Context

    spec = scenes.water_drop(total=20_000, seed=3, basic_pbf=False)
    res = []
    for mode in (0, 2):
        ctx = Context(particle_capacity=spec.n * 2, max_neighbors=256, max_log2res=max(spec.log2res, 3))
        ctx.set_settings(basic_pbf=0, solver_iterations=6, density_error_target=1e-3)
        ctx.load_scene(spec)
        ctx.set_solve_graph(mode)
        for step in range(6):
            ctx.set_neighborhood_search("binary_search" if step % 3 else "green")
            ctx.substep(spec.dt)
        ctx.check_status()
        res.append(ctx.download()[0])
        ctx.close()
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k
