"""The solve loop graph (Jacobi passes 1.. of a substep as one graph launch with a
device-side while loop) against the per-pass launches: bit-identical states,
pass counts and convergence counts, fewer host launches."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _run(spec, graph: bool, substeps: int, iterations: int, target: float, warm=None, maxn=128):
    import torch

    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=spec.n, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=iterations,
                     density_error_target=target)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    ctx.set_solve_graph(graph)
    if warm is not None:
        ctx.mlp_load(torch.from_numpy(warm).cuda())
        ctx.set_warm_start(True)
    ctx.check_status()
    l0 = ctx.launch_count()
    for _ in range(substeps):
        ctx.substep(spec.dt)
    info = ctx.check_status()
    launches = ctx.launch_count() - l0
    st, _ = ctx.download()
    ctx.close()
    return st, info.density_passes, info.converged_substeps, launches


def _same(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("iterations,target", [(30, 1e-3), (5, 0.0), (4, 0.0), (7, 2e-3)])
def test_graph_matches_launches_dam_break(iterations, target):
    spec = scenes.dam_break(n_side=16)
    a = _run(spec, True, 12, iterations, target)
    b = _run(spec, False, 12, iterations, target)
    _same(a[0], b[0])
    assert a[1] == b[1] and a[2] == b[2], (a[1:], b[1:])
    if target > 0:
        assert a[3] < b[3], (a[3], b[3])


@pytest.mark.parametrize("mode", [1, 2])
def test_graph_runs_every_pass_without_target_after_converged_substeps(mode):
    """Substeps with an error target converge (and set the device flag); a substep
    without a target then runs all solver_iterations passes in the graph modes too."""
    from apbf_gb300.api import Context

    spec = scenes.dam_break(n_side=16)
    ctx = Context(particle_capacity=spec.n, max_neighbors=128, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1, solver_iterations=40, density_error_target=5e-2)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    ctx.set_solve_graph(mode)
    for _ in range(4):
        ctx.substep(spec.dt)
    info = ctx.check_status()
    assert info.converged_substeps == 4
    ctx.set_settings(solver_iterations=9, density_error_target=0.0)
    for _ in range(2):
        ctx.substep(spec.dt)
    info = ctx.check_status()
    assert info.density_passes == 18, info.density_passes
    ctx.close()


def _warm_params(seed=0):
    from oracle import mlp_oracle as M

    rng = np.random.default_rng(seed)
    p = np.zeros(M.P_N, np.float32)
    p[M.P_IS:M.P_IS + 6] = 0.1
    p[M.P_W1:M.P_B1] = rng.normal(size=M.H * M.F) * 0.3
    p[M.P_W2:M.P_B2] = rng.normal(size=M.H * M.H) * 0.1
    p[M.P_W3:M.P_B3] = rng.normal(size=M.H) * 0.05
    p[M.P_YS] = 0.2
    p[M.P_YM] = -0.3
    return p


def test_graph_matches_launches_with_warm_start():
    from oracle import mlp_oracle as M

    rng = np.random.default_rng(0)
    p = np.zeros(M.P_N, np.float32)
    p[M.P_IS:M.P_IS + 6] = 0.1
    p[M.P_W1:M.P_B1] = rng.normal(size=M.H * M.F) * 0.3
    p[M.P_W2:M.P_B2] = rng.normal(size=M.H * M.H) * 0.1
    p[M.P_W3:M.P_B3] = rng.normal(size=M.H) * 0.05
    p[M.P_YS] = 0.2
    p[M.P_YM] = -0.3
    spec = scenes.water_drop(total=20_000, seed=3, basic_pbf=True)
    a = _run(spec, True, 30, 40, 1e-3, warm=p, maxn=160)
    b = _run(spec, False, 30, 40, 1e-3, warm=p, maxn=160)
    _same(a[0], b[0])
    assert a[1] == b[1] and a[2] == b[2], (a[1:], b[1:])
    assert a[3] < b[3]


def _run_mode(spec, mode, substeps, iterations, target, maxn=128, warm=None):
    import torch

    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=int(spec.n * 1.3) + 64, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=iterations,
                     density_error_target=target)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    ctx.set_solve_graph(mode)
    if warm is not None:
        ctx.mlp_load(torch.from_numpy(warm).cuda())
        ctx.set_warm_start(True)
    ctx.check_status()
    for _ in range(substeps):
        ctx.substep(spec.dt)
    info = ctx.check_status()
    st, tr = ctx.download()
    ctx.close()
    return st, tr, info.density_passes, info.converged_substeps


@pytest.mark.parametrize("scene", ["dam_break", "water_drop_adaptive"])
def test_whole_substep_graph_matches_launches(scene):
    if scene == "dam_break":
        spec, maxn, it, tg = scenes.dam_break(n_side=16), 128, 30, 1e-3
    else:
        spec, maxn, it, tg = scenes.water_drop(total=20_000, seed=1, basic_pbf=False), 256, 8, 0.0
    a = _run_mode(spec, 2, 10, it, tg, maxn)
    b = _run_mode(spec, 0, 10, it, tg, maxn)
    _same(a[0], b[0])
    _same(a[1], b[1])
    assert a[2:] == b[2:]


def test_whole_substep_graph_with_warm_start():
    from oracle import mlp_oracle as M

    rng = np.random.default_rng(1)
    p = np.zeros(M.P_N, np.float32)
    p[M.P_IS:M.P_IS + 6] = 0.1
    p[M.P_W1:M.P_B1] = rng.normal(size=M.H * M.F) * 0.3
    p[M.P_W2:M.P_B2] = rng.normal(size=M.H * M.H) * 0.1
    p[M.P_W3:M.P_B3] = rng.normal(size=M.H) * 0.05
    p[M.P_YS] = 0.2
    p[M.P_YM] = -0.3
    spec = scenes.water_drop(total=20_000, seed=3, basic_pbf=True)
    a = _run_mode(spec, 2, 25, 40, 1e-3, 160, warm=p)
    b = _run_mode(spec, 1, 25, 40, 1e-3, 160, warm=p)
    _same(a[0], b[0])
    assert a[2:] == b[2:]


@pytest.mark.parametrize("persistent", [True, False])
def test_batch_matches_separate_contexts(persistent):
    """Scenes of different sizes and kinds (plain and adaptive, different pass limits
    and targets, one with the learned warm start and projected passes) advanced by
    one graph launch per substep -- their solves as one batched persistent launch or
    as loops in the scenes' branches -- end bit-identical to the same scenes advanced
    one context at a time."""
    import torch

    from apbf_gb300 import _native as N
    from apbf_gb300.api import Batch, Context

    specs = [(scenes.dam_break(n_side=12), 128, 30, 1e-3), (scenes.dam_break(n_side=16, seed=2), 128, 30, 1e-3),
             (scenes.water_drop(total=20_000, seed=4, basic_pbf=True), 160, 40, 1e-3),
             (scenes.water_drop(total=15_000, seed=5, basic_pbf=False), 256, 8, 0.0),
             (scenes.water_drop(total=12_000, seed=6, basic_pbf=True), 160, 12, 2e-3)]
    warm = _warm_params()

    def make(spec, maxn, it, tg, k):
        ctx = Context(particle_capacity=int(spec.n * 1.3) + 64, max_neighbors=maxn,
                      max_log2res=max(spec.log2res, 3))
        ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=it, density_error_target=tg)
        ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
        ctx.set_boxes(spec.box_min, spec.box_max)
        ctx.upload(spec.state)
        if k == 4:  # the learned warm start and projected passes
            ctx.mlp_load(torch.from_numpy(warm).cuda())
            ctx.set_warm_start(N.WARM_LEARNED | N.WARM_PROJECTED)
        return ctx

    dt = specs[0][0].dt
    batched = [make(*s, k) for k, s in enumerate(specs)]
    batch = Batch(batched)
    batch.set_persistent_solve(persistent)
    for _ in range(8):
        batch.substep(dt)
    single = [make(*s, k) for k, s in enumerate(specs)]
    for c in single:
        for _ in range(8):
            c.substep(dt)
    for a, b in zip(batched, single):
        ia, ib = a.check_status(), b.check_status()
        assert (ia.density_passes, ia.converged_substeps) == (ib.density_passes, ib.converged_substeps)
        sa, ta = a.download()
        sb, tb = b.download()
        _same(sa, sb)
        _same(ta, tb)
    batch.close()
    for c in batched + single:
        c.close()
