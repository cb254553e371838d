"""GPU parity of neighborhood_green::apply against the oracle: Morton keys, the sort
permutation, the reordered particle state and the transfer remap bit-exact;
neighbour rows equal as sets; overflow reported with the size needed."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu

GRID = ((0.0, 0.0, 0.0), (32.0, 32.0, 32.0))


def _ctx(cap, maxn=128, L=7):
    from apbf_gb300.api import Context

    return Context(particle_capacity=cap, max_neighbors=maxn, max_log2res=L)


def _random_scene(n, seed, kw_lo=4.0, kw_hi=4.0, spread=30.0):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-0.1 * spread, spread, size=(n, 3))
    st = scenes.make_state(pos)
    st["kernel_width"] = rng.uniform(kw_lo, kw_hi, size=n).astype(np.float32)
    return st


def _run_both(orc, st, scale, L, cap=None, transfers=None, grid=GRID, maxn=512):
    from apbf_gb300.api import neighborhood_green

    n = st["position"].shape[0]
    ctx = _ctx(cap or max(n, 1), maxn=maxn, L=max(L, 3))
    ctx.upload(st, transfers)
    neighborhood_green().set_data(ctx).set_range_scale(scale).set_position_range(grid[0], grid[1], L).apply()
    info = ctx.check_status()
    g_state, g_tr = ctx.download()
    g_perm, g_keys = ctx.debug_sort()
    g_rows = ctx.download_rows()
    fs = orc.FluidState(st, transfers=transfers)
    perm, keys, tot = orc.neighborhood_green(fs, scale, grid[0], grid[1], L, 1 << 24)
    return ctx, info, (g_state, g_tr, g_perm, g_keys, g_rows), (fs.state(), fs.transfers(), perm, keys, fs.rows(), tot)


@pytest.mark.parametrize("seed,kw_hi,scale,L", [(0, 4.0, 1.0, 3), (1, 7.5, 1.0, 4), (2, 4.0, 1.5, 5), (3, 3.0, 1.0, 6)])
def test_green_parity_random(orc, seed, kw_hi, scale, L):
    st = _random_scene(6000, seed, 2.0, kw_hi)
    ctx, info, g, o = _run_both(orc, st, scale, L)
    assert np.array_equal(g[2], o[2]), "sort permutation"
    assert np.array_equal(g[3], o[3]), "sorted keys"
    for k in o[0]:
        assert np.array_equal(g[0][k], o[0][k]), k
    assert info.pairs == o[5]
    for i, (a, b) in enumerate(zip(g[4], o[4])):
        assert np.array_equal(a, b), i
    ctx.close()


def test_green_parity_dam_break(orc):
    spec = scenes.dam_break(n_side=16)
    ctx, info, g, o = _run_both(orc, spec.state, 1.0, spec.log2res, grid=(spec.grid_min, spec.grid_max))
    assert np.array_equal(g[2], o[2])
    for k in o[0]:
        assert np.array_equal(g[0][k], o[0][k]), k
    assert info.pairs == o[5] and info.pairs > 20 * 4096
    assert all(np.array_equal(a, b) for a, b in zip(g[4], o[4]))
    # the reference's pair list: every (i, j) of every row, as uvec2
    pairs = ctx.export_pairs(info.pairs + 10)
    assert pairs.shape[0] == info.pairs
    exp = np.concatenate([np.stack([np.full(len(r), i), r], 1) for i, r in enumerate(o[4]) if len(r)])
    assert np.array_equal(np.unique(pairs.astype(np.int64), axis=0), np.unique(exp, axis=0))
    ctx.close()


def test_transfers_remapped(orc):
    st = _random_scene(3000, 9)
    rng = np.random.default_rng(9)
    ids = rng.permutation(3000)[:200].astype(np.uint32)
    tr = {"source": ids[:100], "target": ids[100:], "time_left": rng.uniform(-1, 2, 100).astype(np.float32)}
    ctx, info, g, o = _run_both(orc, st, 1.0, 4, transfers=tr)
    for k in ("source", "target", "time_left"):
        assert np.array_equal(g[1][k], o[1][k]), k
    ctx.close()


def test_particles_outside_grid_are_clamped(orc):
    st = _random_scene(2000, 5, spread=60.0)  # grid covers [0, 32]^3 only
    ctx, info, g, o = _run_both(orc, st, 1.0, 4)
    assert np.array_equal(g[2], o[2])
    assert all(np.array_equal(a, b) for a, b in zip(g[4], o[4]))
    ctx.close()


@pytest.mark.parametrize("n", [0, 1, 2])
def test_tiny_inputs(orc, n):
    st = _random_scene(n, 11)
    ctx, info, g, o = _run_both(orc, st, 1.0, 3, cap=64)
    assert info.pairs == o[5]
    assert np.array_equal(g[2], o[2])
    ctx.close()


def test_neighbor_overflow_reports_required(orc):
    from apbf_gb300 import _native
    from apbf_gb300.api import neighborhood_green

    spec = scenes.dam_break(n_side=10)
    ctx = _ctx(1000, maxn=8, L=max(5, spec.log2res))
    ctx.upload(spec.state)
    neighborhood_green().set_data(ctx).set_position_range(spec.grid_min, spec.grid_max, spec.log2res).apply()
    info = ctx.status()
    assert ctx.last_status_code == 2  # APBF_ERR_CAPACITY
    assert info.flags & _native.FLAG_NEIGHBOR_OVERFLOW
    fs = orc.FluidState(spec.state)
    orc.neighborhood_green(fs, 1.0, spec.grid_min, spec.grid_max, spec.log2res, 1 << 22)
    assert info.required_neighbors == max(len(r) for r in fs.rows())
    ctx.close()
