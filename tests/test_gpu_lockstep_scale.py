"""Whole substeps at the benched scenes' scale in stage lockstep with the FP64
oracle: a 32 768-particle dam break, a waterfall after its emitter has brought it
past 100 000 particles (the 1 M waterfall with lengths scaled by 1/2), and an
adaptive water drop whose kernel widths are spread across neighbours
(base_kernel_width_on_boundary_distance off, the spread_kernel_width path of
pool.cpp:87-89).  Each stage of a substep runs on the device; the oracle starts
that stage from the device's input state and runs it in FP64; then:
  velocity handling, kernel width, box collision: bit for bit;
  neighbour search: Morton keys, sort permutation, reordered state bit for bit and
    every neighbour set equal;
  spread kernel width: widths bit for bit, pruned neighbour sets equal;
  each Jacobi pass: density and squared-gradient sums within 1e-5 relative + 4
    fixed-point units, positions within 1e-5 of their magnitude + 64 units;
  update_transfers: particle state and transfer list bit for bit;
  particle transfer: lists bit for bit, masses and radii within 1e-5 relative."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _boxes(ctx, spec):
    """The scene's boxes for the oracle, the rotation rows as the device holds them."""
    ob = spec.meta.get("oriented_boxes")
    bmin, bmax = spec.box_min, spec.box_max
    if ob is not None:
        bmin = np.concatenate([bmin, ob[0]])
        bmax = np.concatenate([bmax, ob[1]])
    rot = ctx.box_rotations(bmin.shape[0]).reshape(bmin.shape[0], 12)
    return bmin, bmax, rot


def _rows(ctx):
    return [r.astype(np.uint32) for r in ctx.download_rows()]


def _check_pass(dbg, out, before, after, o_after):
    d = dbg["density"].astype(np.int64) - out["density"].astype(np.int64)
    assert np.all(np.abs(d) <= 1e-5 * out["density"] + 4), np.abs(d).max()
    q = dbg["sq_grad_sum"].astype(np.int64) - out["sq_grad_sum"].astype(np.int64)
    assert np.all(np.abs(q) <= 1e-5 * out["sq_grad_sum"] + 4 + 2e-4 * out["sq_grad_sum"].max()), np.abs(q).max()
    x = after["position"][:, :3].astype(np.int64)
    xo = o_after["position"][:, :3].astype(np.int64)
    assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), np.abs(x - xo).max()


def _lockstep_substep(orc, ctx, spec, last_dt):
    """One substep of pool::update (source/pool.cpp:67-106), stage by stage, each
    checked against the oracle from the device's input state."""
    from apbf_gb300.api import (box_collision, incompressibility, kernel_width_from_boundary_distance,
                                neighborhood_green, particle_transfer, spread_kernel_width, update_transfers,
                                velocity_handling)

    s = ctx.settings
    os_ = orc.settings_from(s)
    adaptive = not s.basic_pbf
    bmin, bmax, rot = _boxes(ctx, spec)
    dt = np.float32(spec.dt)
    cap = ctx.capacity

    def oracle_from_device(rows=None):
        st, tr = ctx.download()
        fs = orc.FluidState(st, transfers=tr, cap=cap)
        if rows is not None:
            orc.set_rows(fs, rows)
        return fs

    # velocity handling (velocity_handling.cpp:15-31)
    fs = oracle_from_device()
    velocity_handling().set_data(ctx).set_acceleration(spec.acceleration).apply(spec.dt)
    orc.velocity_handling(fs, dt, np.float32(last_dt), spec.acceleration)
    g, _ = ctx.download()
    for k in ("position", "velocity", "pos_backup"):
        assert np.array_equal(g[k], fs.state()[k]), k
    if adaptive and (s.merge or s.split):
        fs = oracle_from_device()
        particle_transfer().set_data(ctx).apply(spec.dt)
        orc.particle_transfer(fs, dt)
        g, gtr = ctx.download()
        o, otr = fs.state(), fs.transfers()
        assert g["position"].shape == o["position"].shape
        for k in ("position", "transferring"):
            assert np.array_equal(g[k], o[k]), k
        for k in ("inverse_mass", "radius"):
            assert np.allclose(g[k], o[k], rtol=1e-5, atol=0), k
        for k in ("source", "target"):
            assert np.array_equal(gtr[k], otr[k]), k
    if adaptive and s.base_kernel_width_on_boundary_distance:
        fs = oracle_from_device()
        kernel_width_from_boundary_distance().set_data(ctx).apply()
        orc.kernel_width_from_boundary_distance(fs, os_)
        assert np.array_equal(ctx.download()[0]["kernel_width"], fs.state()["kernel_width"])
    # neighbourhood (neighborhood_green.cpp:27-77) with the range scale of pool.cpp:83
    scale = 1.0 if (s.basic_pbf or s.base_kernel_width_on_boundary_distance) else 1.5
    fs = oracle_from_device()
    neighborhood_green().set_data(ctx).set_range_scale(scale).set_position_range(
        spec.grid_min, spec.grid_max, spec.log2res).apply()
    ctx.check_status()
    perm_d, keys_d = ctx.debug_sort()
    perm_o, keys_o, _ = orc.neighborhood_green(fs, scale, spec.grid_min, spec.grid_max, spec.log2res,
                                               int(cap * 160))
    assert np.array_equal(keys_d, keys_o) and np.array_equal(perm_d, perm_o)
    g, _ = ctx.download()
    o = fs.state()
    for k in o:
        if k != "position":
            assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["position"][:, :3], o["position"][:, :3])
    rows = _rows(ctx)
    assert all(np.array_equal(a, b) for a, b in zip(rows, fs.rows()))
    if adaptive and not s.base_kernel_width_on_boundary_distance:
        fs = oracle_from_device(rows)
        spread_kernel_width().set_data(ctx).apply()
        ctx.check_status()
        orc.spread_kernel_width(fs, os_)
        assert np.array_equal(ctx.download()[0]["kernel_width"], fs.state()["kernel_width"])
        rows = _rows(ctx)
        assert all(np.array_equal(a, np.sort(b)) for a, b in zip(rows, fs.rows()))
    # solverIterations x (box collision, one incompressibility iteration), pool.cpp:91-95
    ctx.set_debug(True)
    for _ in range(s.solver_iterations):
        fs = oracle_from_device(rows)
        box_collision().set_data(ctx).apply()
        orc.box_collision(fs, bmin, bmax, rot)
        assert np.array_equal(ctx.download()[0]["position"][:, :3], fs.state()["position"][:, :3])
        before, _ = ctx.download()
        fs = oracle_from_device(rows)
        incompressibility().set_data(ctx).apply()
        ctx.check_status()
        dbg = ctx.debug_incompressibility()
        out = orc.incompressibility(fs, os_)
        _check_pass(dbg, out, before, ctx.download()[0], fs.state())
    ctx.set_debug(False)
    if adaptive:
        fs = oracle_from_device(rows)
        update_transfers().set_data(ctx).apply()
        ctx.check_status()
        orc.update_transfers(fs, os_, ctx.transfer_capacity)
        g, gtr = ctx.download()
        o, otr = fs.state(), fs.transfers()
        for k in o:
            assert np.array_equal(g[k], o[k]), k
        for k in otr:
            assert np.array_equal(gtr[k], otr[k]), k


def _scene(name):
    from apbf_gb300.api import Context

    if name == "dam_break_32k":
        spec, maxn, pre = scenes.dam_break(n_side=32, seed=3), 160, 20
    elif name == "waterfall_100k":
        spec = scenes.waterfall(initial=48_000, seed=5, scale=0.5, per_substep=800)
        maxn, pre = 256, 80
    else:  # the water drop with kernel widths spread across neighbours
        spec = scenes.water_drop(total=30_000, seed=6, basic_pbf=False)
        spec.meta["settings"] = {"base_kernel_width_on_boundary_distance": 0}
        maxn, pre = 256, 30
    cap = max(int(spec.n * 1.3) + 1024, int(spec.meta.get("capacity", 0)))
    ctx = Context(particle_capacity=cap, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=spec.iterations,
                     **spec.meta.get("settings", {}))
    ctx.load_scene(spec)
    for _ in range(pre):
        ctx.substep(spec.dt)
    ctx.check_status()
    return spec, ctx


@pytest.mark.parametrize("name", ["dam_break_32k", "waterfall_100k", "water_drop_spread"])
def test_substep_stage_lockstep_at_scale(orc, name):
    spec, ctx = _scene(name)
    n = ctx.lengths()[0]
    if name == "waterfall_100k":
        assert n >= 100_000, n
    if name == "water_drop_spread":
        assert not ctx.settings.base_kernel_width_on_boundary_distance
    for _ in range(2):
        _lockstep_substep(orc, ctx, spec, last_dt=spec.dt)
    ctx.close()
