"""Substeps of an empty state and of one and two particles under every solve form
(per-kernel launches, the solve-loop graph, the whole-substep graph, the persistent
solve, an error target, the learned warm start): no error flags, lengths kept, and
with a fixed pass count the positions of the oracle's substep from the same state.
An empty state has no density error, so a solve with a target stops at once."""
from dataclasses import replace

import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu

FORMS = {
    "per_kernel": dict(graph=0),
    "loop_graph": dict(graph=1),
    "substep_graph": dict(graph=2),
    "persistent": dict(graph=2, persistent=True),
    "target": dict(graph=2, target=1e-3),
    "learned": dict(graph=2, target=1e-3, learned=True),
}


def _tiny(n):
    spec = scenes.dam_break(n_side=8, iterations=4)
    # reference units: 2.5 apart, inside one kernel width (4) of each other
    pos = np.array([[20.0, 20.0, 20.0], [22.5, 20.0, 20.0]], np.float64)[:n]
    return replace(spec, state=scenes.make_state(pos))


def _ctx(spec, form):
    from apbf_gb300 import _native as N
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=64, max_neighbors=32, max_log2res=max(spec.log2res, 3))
    target = form.get("target", 0.0)
    ctx.set_settings(basic_pbf=1, solver_iterations=20 if target else spec.iterations,
                     density_error_target=target)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    ctx.set_solve_graph(form["graph"])
    if form.get("persistent"):
        ctx.set_persistent_solve(True)
    if form.get("learned"):
        from apbf_gb300.warmstart import WarmStartNet

        net = WarmStartNet(seed=0)
        net.omega_max, net.min_neighbors = 2.0, 0.0
        ctx.mlp_load(net.params)
        ctx.set_warm_start(N.WARM_LEARNED | N.WARM_PROJECTED)
    return ctx


@pytest.mark.parametrize("form", sorted(FORMS))
@pytest.mark.parametrize("n", [0, 1, 2])
def test_tiny_states(orc, n, form):
    f = FORMS[form]
    spec = _tiny(n)
    ctx = _ctx(spec, f)
    exact = "target" not in f  # a fixed pass count: the oracle's substep applies
    last_dt = 1.0
    for step in range(3):
        before, _ = ctx.download()
        ctx.substep(spec.dt)
        info = ctx.check_status()  # raises on any error flag
        assert ctx.lengths() == (n, 0)
        g, _ = ctx.download()
        assert all(v.shape[0] == n for v in g.values())
        assert np.all(np.isfinite(g["velocity"]))
        if n == 0:
            assert info.pairs == 0
            continue
        assert info.pairs == (2 if n == 2 else 0), info.pairs
        if not exact:
            continue
        fs = orc.FluidState(before)
        sc = orc.make_scene(orc.settings_from(ctx.settings), spec.grid_min, spec.grid_max, spec.log2res,
                            spec.acceleration)
        sc.last_dt = last_dt
        orc.substep(fs, sc, (spec.box_min, spec.box_max), np.float32(spec.dt), 1 << 22)
        last_dt = spec.dt
        o = fs.state()
        x = g["position"][:, :3].astype(np.int64)
        xo = o["position"][:, :3].astype(np.int64)
        assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), (step, np.abs(x - xo).max())
    if n == 0 and "target" in f:
        assert info.density_passes <= 1  # converged at the first measured pass
    ctx.close()
