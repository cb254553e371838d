"""GPU parity of the adaptive stages against the oracle, in lockstep on identical
inputs (the oracle is given the device's neighbour rows):

  kernel width from boundary distance, kernel-width spreading + row pruning,
  split/merge decisions and claims (find_split_and_merge_1..3,
  remove_impossible_splits, duplicate_these, initialize_split_particles):
      bit-exact (integer and plain FP32 arithmetic, claims in index order)
  particle transfer (volumes and masses through cbrt / division):
      inverse mass and radius within 1e-5 relative; everything else bit-exact
"""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu

GRID = ((-4.0, -4.0, -4.0), (60.0, 60.0, 60.0))


def _ctx(cap, maxn=1024, tcap=10000):
    from apbf_gb300.api import Context

    return Context(particle_capacity=cap, max_neighbors=maxn, transfer_capacity=tcap, max_log2res=5)


def _adaptive_state(n_side=10, seed=0):
    """Small particles compressed deep inside (merge candidates) next to a layer of
    large particles at the surface (split candidates)."""
    rng = np.random.default_rng(seed)
    small = scenes.lattice([2, 2, 2], [n_side] * 3, 0.9, 0.05, rng)
    big = scenes.lattice([2, 2 + 0.9 * n_side + 2.0, 2], [n_side // 2, 2, n_side // 2], 4.0, 0.1, rng)
    st = scenes.make_state(np.concatenate([small, big]))
    nb = big.shape[0]
    st["radius"][-nb:] = 2.0
    st["inverse_mass"][-nb:] = np.float32(1.0 / 64.0)
    bd = rng.uniform(40.0, 80.0, size=st["radius"].shape)
    bd[-nb:] = 1.0
    st["boundary_distance"] = (bd * 262144).astype(np.uint32)
    st["kernel_width"][-nb:] = 8.0
    st["boundariness"][:] = (rng.uniform(0, 1, st["radius"].size) > 0.7).astype(np.float32)
    return st


def _search(ctx, st, scale=1.0):
    from apbf_gb300.api import neighborhood_green

    ctx.upload(st)
    neighborhood_green().set_data(ctx).set_range_scale(scale).set_position_range(GRID[0], GRID[1], 4).apply()
    ctx.check_status()
    before, tr = ctx.download()
    return before, tr, ctx.download_rows()


def _assert_states_equal(g, o, skip=()):
    assert g["position"].shape == o["position"].shape
    for k in o:
        if k in skip:
            continue
        assert np.array_equal(g[k], o[k]), k


def test_kernel_width_from_boundary_distance_bit_exact(orc):
    from apbf_gb300.api import kernel_width_from_boundary_distance

    rng = np.random.default_rng(1)
    st = scenes.make_state(rng.uniform(0, 30, size=(5000, 3)))
    st["boundary_distance"] = (rng.uniform(0, 90, 5000) * 262144).astype(np.uint32)
    st["kernel_width"] = rng.uniform(3.0, 12.0, 5000).astype(np.float32)
    st["radius"] = rng.uniform(1.0, 2.0, 5000).astype(np.float32)
    ctx = _ctx(5000)
    ctx.upload(st)
    kernel_width_from_boundary_distance().set_data(ctx).apply()
    g, _ = ctx.download()
    fs = orc.FluidState(st)
    orc.kernel_width_from_boundary_distance(fs, orc.settings_from(ctx.settings))
    assert np.array_equal(g["kernel_width"], fs.state()["kernel_width"])
    ctx.close()


def test_spread_kernel_width_bit_exact(orc):
    from apbf_gb300.api import spread_kernel_width

    st = _adaptive_state(n_side=9, seed=2)
    st["target_radius"] = np.random.default_rng(2).uniform(1.0, 2.5, st["radius"].size).astype(np.float32)
    ctx = _ctx(st["radius"].size)
    ctx.set_settings(base_kernel_width_on_boundary_distance=0)
    before, _, rows = _search(ctx, st, scale=1.5)
    spread_kernel_width().set_data(ctx).apply()
    info = ctx.check_status()
    g, _ = ctx.download()
    g_rows = ctx.download_rows()
    fs = orc.FluidState(before)
    orc.set_rows(fs, rows)
    orc.spread_kernel_width(fs, orc.settings_from(ctx.settings))
    o_rows = fs.rows()
    assert np.array_equal(g["kernel_width"], fs.state()["kernel_width"])
    assert all(np.array_equal(np.sort(a), np.sort(b)) for a, b in zip(g_rows, o_rows))
    assert info.pairs == sum(len(r) for r in o_rows) < sum(len(r) for r in rows)
    ctx.close()


def _update_both(orc, st, tcap=10000, cap_extra=2000, **settings):
    from apbf_gb300.api import update_transfers

    cap = st["radius"].size + cap_extra
    ctx = _ctx(cap, tcap=tcap)
    ctx.set_settings(**settings)
    before, tr0, rows = _search(ctx, st)
    update_transfers().set_data(ctx).apply()
    info = ctx.status()
    g, gtr = ctx.download()
    fs = orc.FluidState(before, cap=cap, tcap=max(tcap, 1))
    orc.set_rows(fs, rows)
    orc.update_transfers(fs, orc.settings_from(ctx.settings), tcap)
    return ctx, info, g, gtr, fs


def test_update_transfers_bit_exact(orc):
    st = _adaptive_state()
    ctx, info, g, gtr, fs = _update_both(orc, st)
    o, otr = fs.state(), fs.transfers()
    assert np.sum(otr["time_left"] > 0) > 10 and np.sum(otr["time_left"] <= 0) > 5  # merges and splits happened
    _assert_states_equal(g, o)
    for k in ("source", "target", "time_left"):
        assert np.array_equal(gtr[k], otr[k]), k
    assert info.flags == 0
    ctx.close()


def test_update_transfers_capacity_limit(orc):
    st = _adaptive_state(seed=3)
    ctx, info, g, gtr, fs = _update_both(orc, st, tcap=12)
    o, otr = fs.state(), fs.transfers()
    assert otr["source"].size == 12
    _assert_states_equal(g, o)
    for k in ("source", "target", "time_left"):
        assert np.array_equal(gtr[k], otr[k]), k
    assert info.flags & 0x2  # APBF_FLAG_TRANSFER_OVERFLOW
    ctx.close()


def test_update_transfers_merge_only_and_split_only(orc):
    for kw in (dict(split=0), dict(merge=0)):
        st = _adaptive_state(seed=4)
        ctx, info, g, gtr, fs = _update_both(orc, st, **kw)
        _assert_states_equal(g, fs.state())
        otr = fs.transfers()
        for k in ("source", "target", "time_left"):
            assert np.array_equal(gtr[k], otr[k]), (kw, k)
        ctx.close()


def test_particle_transfer_after_update(orc):
    from apbf_gb300.api import particle_transfer

    st = _adaptive_state(seed=5)
    ctx, info, g, gtr, fs = _update_both(orc, st, merge_duration=0.01)
    m0 = ctx.reduce_fp64()[0]
    dt = np.float32(1.0 / 240.0)
    for step in range(4):
        particle_transfer().set_data(ctx).apply(float(dt))
        ctx.check_status()
        orc.particle_transfer(fs, dt)
        g, gtr = ctx.download()
        o, otr = fs.state(), fs.transfers()
        assert g["position"].shape == o["position"].shape, step
        _assert_states_equal(g, o, skip=("inverse_mass", "radius"))
        for k in ("inverse_mass", "radius"):
            assert np.allclose(g[k], o[k], rtol=1e-5, atol=0), (step, k)
        for k in ("source", "target", "time_left"):
            assert np.array_equal(gtr[k], otr[k]), (step, k)
        assert ctx.reduce_fp64()[0] == pytest.approx(m0, rel=1e-6)  # mass is conserved
    assert g["position"].shape[0] < st["radius"].size + 40  # finished merges deleted particles
    ctx.close()


def test_adaptive_water_drop_rollout():
    from apbf_gb300.api import Context

    spec = scenes.water_drop(total=20_000, iterations=4)
    ctx = Context(particle_capacity=int(spec.n * 1.5), max_neighbors=512, max_log2res=spec.log2res)
    ctx.set_settings(basic_pbf=0, solver_iterations=spec.iterations)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    m0 = ctx.reduce_fp64()[0]
    for _ in range(20):
        ctx.substep(spec.dt)
    ctx.check_status()
    g, tr = ctx.download()
    assert np.all(np.isfinite(g["velocity"])) and np.all(np.isfinite(g["inverse_mass"]))
    assert ctx.reduce_fp64()[0] == pytest.approx(m0, rel=1e-5)
    assert tr["source"].size > 0 or g["position"].shape[0] != spec.n  # adaptivity did something
    ctx.close()
