"""The waterfall scene's new stages against the oracle: the emitter (bit-exact
positions, velocities and attributes of the appended particles), oriented-box
collision (bit-exact), and a scaled waterfall that runs with split/merge."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_emitter_substeps_bit_exact(orc):
    """Substeps with no Jacobi pass (emission, velocity handling, neighbour search
    and reorder only) from an empty list: every appended particle equals the
    oracle's, in the same sorted order."""
    from apbf_gb300.api import Context

    spec = scenes.waterfall(initial=0, scale=0.25, per_substep=300)
    e = spec.meta["emitter"]
    cap = 4000
    ctx = Context(particle_capacity=cap, max_neighbors=128, max_log2res=spec.log2res)
    ctx.set_settings(basic_pbf=1, solver_iterations=0)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_emitter(**e)
    ctx.set_lengths(0, 0)
    fs = orc.FluidState({k: v[:0] for k, v in spec.state.items()}, cap=cap)
    sc = orc.make_scene(orc.settings_from(ctx.settings), spec.grid_min, spec.grid_max, spec.log2res,
                        spec.acceleration)
    est = np.zeros(2, np.float64)
    last_dt = 1.0
    no_boxes = (np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32))
    for step in range(6):
        ctx.substep(spec.dt)
        k, _ = orc.emit(fs, ctx.emitter, est, np.float32(spec.dt), np.float32(last_dt))
        sc.last_dt = last_dt
        orc.substep(fs, sc, no_boxes, np.float32(spec.dt), 1 << 20)
        last_dt = spec.dt
        ctx.check_status()
        g, _ = ctx.download()
        o = fs.state()
        assert g["position"].shape[0] == o["position"].shape[0] == fs.n, step
        for key in g:
            assert np.array_equal(g[key], o[key]), (step, key)
    assert fs.n > 0
    # the stream rate: per_substep on average
    assert abs(fs.n - 6 * 300) <= e["nx"] * e["nz"]
    ctx.close()


def test_emitter_respects_capacity_and_limit(orc):
    from apbf_gb300._native import FLAG_PARTICLE_OVERFLOW, ApbfError
    from apbf_gb300.api import Context

    spec = scenes.waterfall(initial=0, scale=0.25, per_substep=300)
    e = dict(spec.meta["emitter"])
    ctx = Context(particle_capacity=700, max_neighbors=128, max_log2res=spec.log2res)
    ctx.set_settings(basic_pbf=1, solver_iterations=0)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    e["max_particles"] = 500
    ctx.set_emitter(**e)
    ctx.set_lengths(0, 0)
    for _ in range(4):
        ctx.substep(spec.dt)
    assert ctx.lengths()[0] == 500
    ctx.check_status()
    e["max_particles"] = 0
    ctx.set_emitter(**e)  # restarts the stream, unlimited: the capacity stops it
    for _ in range(3):
        ctx.substep(spec.dt)
    assert ctx.lengths()[0] == 700
    info = ctx.status()
    assert info.flags & FLAG_PARTICLE_OVERFLOW
    ctx.close()


def test_oriented_box_collision_bit_exact(orc):
    """Particles around and inside a rotated box (and an axis-aligned one): the
    box-collision stage equals the oracle's push-out in the box frame."""
    from apbf_gb300.api import Context, box_collision

    rng = np.random.default_rng(3)
    n = 6000
    pos = rng.uniform([0, 0, 0], [120, 120, 120], size=(n, 3))
    st = scenes.make_state(pos)
    ctx = Context(particle_capacity=n, max_neighbors=64, max_log2res=5)
    ctx.set_scene((-4, -4, -4), (130, 130, 130), 5, (0.0, 0.0, 0.0))
    bmin = np.array([[10, 10, 10, 0]], np.float32)
    bmax = np.array([[40, 30, 50, 0]], np.float32)
    ctx.set_boxes(bmin, bmax)
    th = 0.7
    q = np.array([[0.2, 0.3, 0.5, 0.0], [0.0, 0.0, np.sin(th / 2), np.cos(th / 2)]], np.float32)
    q[0, 3] = np.sqrt(1.0 - np.sum(q[0, :3] ** 2))
    ctx.set_oriented_boxes(np.array([[70, 60, 60, 0], [60, 90, 30, 0]], np.float32),
                           np.array([[25, 8, 15, 0], [30, 5, 20, 0]], np.float32), q)
    ctx.upload(st)
    box_collision().set_data(ctx).apply()
    g, _ = ctx.download()
    rot = ctx.box_rotations(3)
    assert rot[0, 0, 3] == 0 and rot[1, 0, 3] == 1 and rot[2, 0, 3] == 1
    allmin = np.concatenate([bmin, np.array([[70, 60, 60, 0], [60, 90, 30, 0]], np.float32)])
    allmax = np.concatenate([bmax, np.array([[25, 8, 15, 0], [30, 5, 20, 0]], np.float32)])
    fs = orc.FluidState(st)
    orc.box_collision(fs, allmin, allmax, rot)
    o = fs.state()
    assert np.array_equal(g["position"], o["position"])
    moved = np.any(g["position"][:, :3] != st["position"][:, :3], axis=1)
    assert moved.sum() > 150  # the boxes (4 % of the volume) did push particles
    ctx.close()


def test_scaled_waterfall_runs_adaptive():
    """A scaled waterfall with split/merge: the stream lands on the slope and runs
    into the tank; the particle count follows the emission, no particle ends inside
    the slope, every substep converges, mass is conserved by split/merge."""
    from apbf_gb300.api import Context

    spec = scenes.waterfall(initial=20_000, scale=0.3, per_substep=300)
    ctx = Context(particle_capacity=150_000, max_neighbors=256, max_log2res=spec.log2res)
    ctx.set_settings(basic_pbf=0, solver_iterations=40, density_error_target=2e-3)
    ctx.load_scene(spec)
    ctx.check_status()
    m0 = ctx.reduce_fp64()[0]
    steps = 90
    for _ in range(steps):
        ctx.substep(spec.dt)
    info = ctx.check_status()
    red = ctx.reduce_fp64()
    st, _ = ctx.download()
    # mass: the initial fluid plus what the emitter appended (8 per unit-radius particle);
    # split/merge moves mass between particles and conserves it
    e = spec.meta["emitter"]
    layer_dt = 2.0 * e["radius"] / e["speed"]
    emitted = int(np.ceil(steps * np.float32(spec.dt) / layer_dt - 1e-9)) * e["nx"] * e["nz"]
    assert red[0] == pytest.approx(m0 + 8.0 * emitted, rel=1e-4)
    c, h, q = spec.meta["oriented_boxes"]
    rot = ctx.box_rotations(len(spec.box_min) + 1)[-1]
    p = st["position"][:, :3].astype(np.float64) / 262144.0
    local = (p - c[0, :3]) @ rot[:, :3].T.astype(np.float64)
    inside = np.all(np.abs(local) < h[0, :3] - 1.0, axis=1)
    assert inside.sum() == 0
    # the stream reached the slope and ran down it (particles below the slope's top end)
    assert np.sum(p[:, 1] < c[0, 1]) > spec.n
    assert info.converged_substeps >= steps // 2
    ctx.close()
