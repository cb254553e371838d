"""Whole plain-PBF substeps (pool::update with basicPbf) on the GPU against the
oracle: the first substep in lockstep, then rollouts compared statistically
(FP32 and FP64 trajectories separate slowly through float -> int truncations),
determinism (two runs are bit-identical) and the FP64 reductions."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _setup(spec, maxn=128):
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=spec.n, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=spec.iterations)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    return ctx


def _oracle(orc, spec, ctx):
    fs = orc.FluidState(spec.state)
    sc = orc.make_scene(orc.settings_from(ctx.settings), spec.grid_min, spec.grid_max, spec.log2res,
                        spec.acceleration)
    return fs, sc


def _free_block(n_side=12, seed=0):
    """A compressed block in free fall, no walls: every difference between the FP32
    device path and the FP64 oracle is then a per-pair truncation difference."""
    from dataclasses import replace

    spec = scenes.dam_break(n_side=n_side, seed=seed, iterations=4)
    rng = np.random.default_rng(seed)
    pos = scenes.lattice([20, 20, 20], [n_side] * 3, 1.8, 0.2, rng)
    return replace(spec, state=scenes.make_state(pos), box_min=np.zeros((0, 4), np.float32),
                   box_max=np.zeros((0, 4), np.float32))


def _match(g_pos, o_pos):
    """Pairs every device particle with the nearest oracle particle.  After the
    first substep the two trajectories differ by FP32 truncations, so particles near
    a cell boundary can fall in different Morton cells and the two sort permutations
    differ: particles are compared by position, not by index."""
    from scipy.spatial import cKDTree

    d, k = cKDTree(o_pos).query(g_pos)
    return d, k


def test_free_block_substeps_lockstep(orc):
    # each substep starts from the same state on both sides (the oracle is re-synced
    # to the device state): positions within 1e-5 of their magnitude + 64 units
    spec = _free_block()
    ctx = _setup(spec)
    last_dt = 1.0
    for step in range(4):
        before, _ = ctx.download()
        ctx.substep(spec.dt)
        ctx.check_status()
        g, _ = ctx.download()
        fs, sc = _oracle(orc, spec, ctx)
        fs = orc.FluidState(before)
        sc.last_dt = last_dt
        orc.substep(fs, sc, (spec.box_min, spec.box_max), np.float32(spec.dt), 1 << 22)
        last_dt = spec.dt
        o = fs.state()
        x = g["position"][:, :3].astype(np.int64)
        xo = o["position"][:, :3].astype(np.int64)
        assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), (step, np.abs(x - xo).max())
        moved = np.abs(xo - before["position"][:, :3]).max() / 262144.0
        assert moved > 0.01
    ctx.close()


def test_dam_break_substeps_match_oracle(orc):
    pytest.importorskip("scipy")
    spec = scenes.dam_break(n_side=12, iterations=4)
    ctx = _setup(spec)
    fs, sc = _oracle(orc, spec, ctx)
    for step in range(12):
        ctx.substep(spec.dt)
        orc.substep(fs, sc, (spec.box_min, spec.box_max), np.float32(spec.dt), 1 << 22)
        ctx.check_status()
        g, _ = ctx.download()
        o = fs.state()
        d, k = _match(g["position"][:, :3] / 262144.0, o["position"][:, :3] / 262144.0)
        # one-to-one, and the ensemble stays together (wall jitter of up to 0.05 radii,
        # box_collision.comp:46-47, decorrelates the two trajectories near walls)
        assert np.unique(k).size > 0.99 * spec.n, step
        assert np.mean(d) < 0.01 * (step + 1), (step, np.mean(d))
        assert np.percentile(d, 99) < 0.06 * (step + 1), (step, np.percentile(d, 99))
    e_gpu = ctx.reduce_fp64()
    assert e_gpu[0] == pytest.approx(orc.reduce(fs)[0], rel=1e-9)  # mass
    ctx.close()


def test_substep_deterministic():
    spec = scenes.dam_break(n_side=16)
    results = []
    for _ in range(2):
        ctx = _setup(spec)
        for _ in range(5):
            ctx.substep(spec.dt)
        ctx.check_status()
        results.append(ctx.download()[0])
        ctx.close()
    for k in results[0]:
        assert np.array_equal(results[0][k], results[1][k]), k


def test_dam_break_config0_runs_and_stays_incompressible():
    spec = scenes.dam_break(n_side=32, iterations=4)
    ctx = _setup(spec)
    for _ in range(40):
        ctx.substep(spec.dt)
    info = ctx.check_status()
    red = ctx.reduce_fp64()
    g, _ = ctx.download()
    assert np.all(np.isfinite(g["velocity"]))
    assert red[0] == pytest.approx(spec.n * 8.0, rel=1e-9)
    assert 0.0 <= red[2] < 0.05  # mean compression error of the last iteration
    assert info.pairs > 20 * spec.n
    ctx.close()


def test_iterations_stop_at_error_target(orc):
    """density_error_target: the device stops the Jacobi iterations at the first
    density pass whose mean compression error is at most the target, like the
    oracle's or_substep.  The target is put between two consecutive errors of the
    oracle's own sequence so that FP32 and FP64 agree on where to stop."""
    spec = _free_block(n_side=12)
    ctx = _setup(spec)
    s = orc.settings_from(ctx.settings)
    # the oracle's error sequence for this substep
    fs = orc.FluidState(spec.state)
    orc.velocity_handling(fs, np.float32(spec.dt), np.float32(1.0), spec.acceleration)
    orc.neighborhood_green(fs, 1.0, spec.grid_min, spec.grid_max, spec.log2res, 1 << 22)
    errs = []
    for _ in range(6):
        errs.append(orc.density_error(fs, s)[0])
        orc.incompressibility(fs, s)
    assert errs[2] > 1.05 * errs[3] > 0, errs
    target = float(np.sqrt(errs[2] * errs[3]))

    ctx.set_settings(solver_iterations=10, density_error_target=target)
    ctx.check_status()  # clear the pass counter
    ctx.substep(spec.dt)
    info = ctx.check_status()
    assert info.density_passes == 4  # three corrections, then the pass that meets the target
    g, _ = ctx.download()
    s2 = orc.settings_from(ctx.settings)
    fs2 = orc.FluidState(spec.state)
    sc = orc.make_scene(s2, spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    orc.substep(fs2, sc, (spec.box_min, spec.box_max), np.float32(spec.dt), 1 << 22)
    o = fs2.state()
    x = g["position"][:, :3].astype(np.int64)
    xo = o["position"][:, :3].astype(np.int64)
    assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), np.abs(x - xo).max()
    red = ctx.reduce_fp64()
    assert red[2] <= target < errs[2]
    ctx.close()
