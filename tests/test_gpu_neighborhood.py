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


def _pairs_sorted(count: np.ndarray, index: np.ndarray, mask: int = 0xFFFFFFFF) -> np.ndarray:
    """(i << 32 | entry) keys of column-major rows, sorted."""
    n = count.shape[0]
    m = int(count.max()) if n else 0
    idx = index[:m, :n].astype(np.int64) & mask
    live = np.arange(m)[:, None] < count[None, :].astype(np.int64)
    ii = np.broadcast_to(np.arange(n, dtype=np.int64)[None, :], (m, n))[live]
    return np.sort((ii << 32) | idx[live])


@pytest.mark.parametrize("seed,scale,L", [(4, 1.0, 4), (5, 1.5, 5), (6, 1.0, 3)])
def test_correction_rows(seed, scale, L):
    """With differing search radii the position update of particle i sums over i's own
    row and then over i's correction row: entries flagged (bit 31) are the j of i's row
    whose radius does not reach i (their terms are subtracted again), the others the k
    whose rows hold i although i's radius does not reach k (added).  So own row minus
    flagged plus added is exactly the transpose of the rows, the set the reference's
    atomic scatter (incompressibility_3.comp:62-66) adds to i."""
    from apbf_gb300.api import neighborhood_green

    st = _random_scene(6000, seed, 2.0, 4.5)
    n = st["position"].shape[0]
    ctx = _ctx(n, maxn=512, L=max(L, 3))
    ctx.upload(st)
    neighborhood_green().set_data(ctx).set_range_scale(scale).set_position_range(GRID[0], GRID[1], L).apply()
    ctx.check_status()
    g, _ = ctx.download()
    fw = ctx.neighbors_view()
    rv = ctx.reverse_neighbors_view()
    assert rv["kind"] == 1
    fc = fw["count"][:n].cpu().numpy().astype(np.int64)
    fi = fw["index"][:, :n].cpu().numpy().view(np.uint32).astype(np.int64)
    cc = rv["count"][:n].cpu().numpy().astype(np.int64)
    ci = rv["index"][:, :n].cpu().numpy().view(np.uint32).astype(np.int64)
    fwd = _pairs_sorted(fc, fi)  # (i << 32 | j): j in i's row
    flagged = _pairs_sorted(cc, ci) if n else fwd[:0]
    sub_ = flagged[(flagged & 0x80000000) != 0] & ~np.int64(0x80000000)
    add = flagged[(flagged & 0x80000000) == 0]
    # the flagged entries are exactly the one-sided pairs of the rows
    R = np.floor(g["kernel_width"].astype(np.float64) * np.float64(np.float32(scale)) * 262144.0).astype(np.int64)
    pos = g["position"][:, :3].astype(np.int64)
    i_, j_ = fwd >> 32, fwd & 0xFFFFFFFF
    one_sided = np.sum((pos[j_] - pos[i_]) ** 2, axis=1) > R[j_] * R[j_]
    assert np.array_equal(np.sort(sub_), np.sort(fwd[one_sided]))
    assert one_sided.any(), "the scene should have one-sided pairs"
    # own row - subtracted + added == transpose of the rows, as multisets
    transpose = np.sort(((fwd & 0xFFFFFFFF) << 32) | (fwd >> 32))
    delta = np.sort(np.concatenate([np.setdiff1d(fwd, sub_, assume_unique=True), add]))
    assert np.array_equal(delta, transpose)
    ctx.close()
