"""The persistent solve (Jacobi passes 1.. of a substep in one cooperative launch
with grid barriers) against per-kernel launches: bit-identical states, pass counts
and convergence counts, with and without an error target, with equal and with
adaptive kernel widths, with the warm start's projected passes, inside a
whole-substep graph, and with fewer launches."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _warm_params(seed):
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


def _run(spec, persistent, graph_mode, substeps, iterations, target, maxn=128, warm=None, projected=False):
    import torch

    from apbf_gb300 import _native as N
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=int(spec.n * 1.3) + 64, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=iterations,
                     density_error_target=target)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    ctx.set_solve_graph(graph_mode)
    ctx.set_persistent_solve(persistent)
    if warm is not None:
        ctx.mlp_load(torch.from_numpy(warm).cuda())
        ctx.set_warm_start(N.WARM_LEARNED | (N.WARM_PROJECTED if projected else 0))
    elif projected:
        ctx.set_warm_start(N.WARM_PROJECTED)
    ctx.check_status()
    l0 = ctx.launch_count()
    for _ in range(substeps):
        ctx.substep(spec.dt)
    info = ctx.check_status()
    launches = ctx.launch_count() - l0
    st, tr = ctx.download()
    ctx.close()
    return st, tr, info.density_passes, info.converged_substeps, launches


def _same(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("iterations,target", [(30, 1e-3), (5, 0.0), (4, 0.0), (7, 2e-3), (2, 0.0)])
def test_persistent_matches_launches_dam_break(iterations, target):
    spec = scenes.dam_break(n_side=16)
    a = _run(spec, True, 0, 12, iterations, target)
    b = _run(spec, False, 0, 12, iterations, target)
    _same(a[0], b[0])
    assert a[2:4] == b[2:4], (a[2:4], b[2:4])
    assert a[4] < b[4], (a[4], b[4])  # one launch instead of two per pass


def test_persistent_matches_launches_adaptive_widths():
    """Split/merge and kernel-width spreading: unequal widths (solve records and
    positions gathered, transposed rows when radii differ)."""
    spec = scenes.water_drop(total=20_000, seed=1, basic_pbf=False)
    a = _run(spec, True, 0, 10, 8, 0.0, maxn=256)
    b = _run(spec, False, 0, 10, 8, 0.0, maxn=256)
    _same(a[0], b[0])
    _same(a[1], b[1])
    assert a[2:4] == b[2:4]


@pytest.mark.parametrize("warm", [False, True])
def test_persistent_matches_launches_projected(warm):
    spec = scenes.water_drop(total=20_000, seed=3, basic_pbf=True)
    p = _warm_params(2) if warm else None
    a = _run(spec, True, 0, 25, 40, 1e-3, maxn=160, warm=p, projected=True)
    b = _run(spec, False, 0, 25, 40, 1e-3, maxn=160, warm=p, projected=True)
    _same(a[0], b[0])
    assert a[2:4] == b[2:4]


def test_persistent_inside_substep_graph():
    """Captured into the whole-substep graph (a cooperative kernel node)."""
    spec = scenes.dam_break(n_side=16, seed=4)
    a = _run(spec, True, 2, 12, 30, 1e-3)
    b = _run(spec, False, 0, 12, 30, 1e-3)
    _same(a[0], b[0])
    assert a[2:4] == b[2:4]
