"""GPU parity of one Jacobi incompressibility iteration (incompressibility_0..3)
and of the FP32 glue stages, in lockstep with the oracle on identical inputs.

Tolerances (FP32 device vs FP64 oracle):
  density / squared-gradient sums (2^18 fixed point): |d| <= 1e-5 * value + 4 units
  weighted gradient sums: |d| <= 1e-5 * |sum| + 2e-4 * scale of the row + 4 units
  lambda: |d| <= 1e-4 * |lambda| + (d lambda / d rho) * 8 fixed-point density units
          + |lambda| * (relative change of its denominator when every per-pair term of
          the squared-gradient and weighted-gradient sums moves by one fixed-point unit):
          1 - rho/rho0 cancels near rest, and every per-pair term is truncated to an
          integer, where FP32 and FP64 may fall on different sides
  positions: |d| <= 1e-5 * |x| + 64 fixed units (64 / 2^18 = 2.4e-4 radii)
Box collision and velocity handling are plain FP32 and must match bit for bit.
"""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ctx(cap, maxn=320, L=6):
    from apbf_gb300.api import Context

    return Context(particle_capacity=cap, max_neighbors=maxn, max_log2res=L)


def _compressed_block(n_side=14, spacing=1.85, seed=0, kw_jitter=0.0):
    rng = np.random.default_rng(seed)
    st = scenes.make_state(scenes.lattice([2, 2, 2], [n_side] * 3, spacing, 0.25, rng))
    if kw_jitter:
        st["kernel_width"] = (4.0 + rng.uniform(0, kw_jitter, st["radius"].size)).astype(np.float32)
        st["radius"] = (1.0 + rng.uniform(0, 0.3, st["radius"].size)).astype(np.float32)
        st["inverse_mass"] = (1.0 / (2.0 * st["radius"].astype(np.float64)) ** 3).astype(np.float32)
    st["boundariness"][:] = rng.uniform(0, 1, st["radius"].size).astype(np.float32)
    return st


GRID = ((-4.0, -4.0, -4.0), (60.0, 60.0, 60.0))


def _settings(orc, ctx, **kw):
    ctx.set_settings(basic_pbf=1, **kw)
    return orc.settings_from(ctx.settings)


def _lockstep(orc, st, **kw):
    from apbf_gb300.api import incompressibility, neighborhood_green

    n = st["position"].shape[0]
    ctx = _ctx(n)
    os_ = _settings(orc, ctx, **kw)
    ctx.upload(st)
    ctx.set_debug(True)
    neighborhood_green().set_data(ctx).set_position_range(GRID[0], GRID[1], 4).apply()
    ctx.check_status()
    rows = ctx.download_rows()
    before, _ = ctx.download()
    incompressibility().set_data(ctx).apply()
    ctx.check_status()
    dbg = ctx.debug_incompressibility()
    after, _ = ctx.download()
    fs = orc.FluidState(before)
    orc.set_rows(fs, rows)
    out = orc.incompressibility(fs, os_)
    ctx.close()
    return before, after, dbg, fs.state(), out, rows


def _lambda_tolerance(before, out, rows, rmin=1.0):
    """Tolerance of lambda from the oracle's sums (incompressibility_2.comp:81-98 in
    FP64): 1e-4 relative, 8 fixed-point units of density, and one unit per pair in
    the squared-gradient and weighted-gradient sums."""
    r = before["radius"].astype(np.float64)
    im = before["inverse_mass"].astype(np.float64)
    ird = (2.0 * r) ** 3 * im
    wgs = out["grad_sum"].astype(np.float64) / 262144.0
    sqs = out["sq_grad_sum"].astype(np.float64) / 262144.0 + np.sum(wgs * wgs, axis=1) * im
    denom = ird * ird * (sqs + 0.01) * ((2.0 * rmin) ** 3 / ird * im)
    dlam_drho = ird / denom
    cnt = np.array([len(x) for x in rows], np.float64) + 4.0
    unit = cnt / 262144.0
    d_sqs = unit + 2.0 * np.sqrt(np.sum(wgs * wgs, axis=1)) * unit * im * np.sqrt(3.0)
    lam = np.abs(out["lambda"]).astype(np.float64)
    return 1e-4 * lam + dlam_drho * 8.0 / 262144.0 + lam * d_sqs / (sqs + 0.01)


def _check(before, after, dbg, o_after, out, rows):
    d = dbg["density"].astype(np.int64) - out["density"].astype(np.int64)
    assert np.all(np.abs(d) <= 1e-5 * out["density"] + 4), np.abs(d).max()
    q = dbg["sq_grad_sum"].astype(np.int64) - out["sq_grad_sum"].astype(np.int64)
    assert np.all(np.abs(q) <= 1e-5 * out["sq_grad_sum"] + 4 + 2e-4 * out["sq_grad_sum"].max())
    g = dbg["grad_sum"].astype(np.int64) - out["grad_sum"].astype(np.int64)
    gscale = np.abs(out["grad_sum"]).max()
    assert np.all(np.abs(g) <= 1e-5 * np.abs(out["grad_sum"]) + 2e-4 * gscale + 4), np.abs(g).max()
    lam_ok = np.abs(dbg["lambda"] - out["lambda"]) <= _lambda_tolerance(before, out, rows)
    assert np.all(lam_ok), (np.flatnonzero(~lam_ok)[:5], dbg["lambda"][~lam_ok][:5], out["lambda"][~lam_ok][:5])
    x = after["position"][:, :3].astype(np.int64)
    xo = o_after["position"][:, :3].astype(np.int64)
    tol = 1e-5 * np.abs(xo) + 64
    assert np.all(np.abs(x - xo) <= tol), np.abs(x - xo).max()
    moved = np.abs(xo - before["position"][:, :3]).max()
    assert moved > 1000  # the iteration did something
    # boundariness: equal except where FP32 and FP64 fall on different sides of a threshold
    assert np.mean(after["boundariness"] == o_after["boundariness"]) > 0.99


def test_incompressibility_gauss_default(orc):
    _check(*_lockstep(orc, _compressed_block()))


@pytest.mark.parametrize("hk,gk", [(0, 0), (2, 2), (3, 3), (4, 4), (1, 2)])
def test_incompressibility_other_kernels(orc, hk, gk):
    _check(*_lockstep(orc, _compressed_block(n_side=10), height_kernel_id=hk, gradient_kernel_id=gk))


@pytest.mark.parametrize("method", [0, 1, 2])
def test_incompressibility_boundariness_methods(orc, method):
    _check(*_lockstep(orc, _compressed_block(n_side=10, seed=method), boundariness_calculation_method=method))


def test_incompressibility_variable_kernel_width(orc):
    # search radii differ: the position update gathers over the transposed rows
    before, after, dbg, o_after, out, rows = _lockstep(orc, _compressed_block(n_side=11, kw_jitter=3.0))
    _check(before, after, dbg, o_after, out, rows)
    n = len(rows)
    sym = all(i in set(rows[j].tolist()) for i in range(n) for j in rows[i].tolist()[:2])
    assert not sym


def test_box_collision_bit_exact(orc):
    from apbf_gb300.api import box_collision

    rng = np.random.default_rng(5)
    pos = rng.uniform(-6, 40, size=(5000, 3))
    st = scenes.make_state(pos)
    bmin, bmax = scenes.wall_boxes([0, 0, 0], [32, 32, 32])
    ctx = _ctx(5000)
    ctx.upload(st)
    box_collision().set_data(ctx, bmin, bmax).apply()
    g, _ = ctx.download()
    fs = orc.FluidState(st)
    orc.box_collision(fs, bmin, bmax)
    assert np.array_equal(g["position"], fs.state()["position"])
    ctx.close()


def test_velocity_handling_bit_exact(orc):
    from apbf_gb300.api import velocity_handling

    rng = np.random.default_rng(6)
    st = scenes.make_state(rng.uniform(0, 50, size=(4000, 3)))
    st["pos_backup"][:, :3] -= rng.integers(-30000, 30000, size=(4000, 3)).astype(np.int32)
    ctx = _ctx(4000)
    ctx.upload(st)
    vh = velocity_handling().set_data(ctx).set_acceleration((0.0, -392.4, 0.0))
    vh.apply(1.0 / 120.0)   # first call infers with the initial last dt of 1 (velocity_handling.h:17)
    vh.apply(1.0 / 120.0)
    g, _ = ctx.download()
    fs = orc.FluidState(st)
    orc.velocity_handling(fs, np.float32(1 / 120), np.float32(1.0), (0.0, -392.4, 0.0))
    orc.velocity_handling(fs, np.float32(1 / 120), np.float32(1 / 120), (0.0, -392.4, 0.0))
    o = fs.state()
    for k in ("position", "velocity", "pos_backup"):
        assert np.array_equal(g[k], o[k]), k
    ctx.close()


def test_nonfinite_lambda_flagged(orc):
    from apbf_gb300 import _native
    from apbf_gb300.api import incompressibility, neighborhood_green

    st = _compressed_block(n_side=6)
    st["inverse_mass"][3] = np.nan
    ctx = _ctx(st["radius"].size)
    ctx.set_settings(basic_pbf=1)
    ctx.upload(st)
    neighborhood_green().set_data(ctx).set_position_range(GRID[0], GRID[1], 4).apply()
    incompressibility().set_data(ctx).apply()
    info = ctx.status()
    assert info.flags & _native.FLAG_NONFINITE
    assert ctx.last_status_code == 3
    ctx.close()
