"""Launch-shape tuning: every threads-per-particle choice of the Jacobi gather
passes gives bit-identical substeps (the gathered sums are wrapping integer sums),
and the autotuner leaves the particle state as it found it."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ctx(spec, iterations, target=0.0, maxn=128):
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=spec.n, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=iterations, density_error_target=target)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    return ctx


@pytest.mark.parametrize("name", ["dam_break", "water_drop_adaptive"])
def test_gather_lanes_bit_identical(name):
    if name == "dam_break":
        spec, maxn = scenes.dam_break(n_side=16), 128
    else:
        spec, maxn = scenes.water_drop(total=20_000, seed=2, basic_pbf=False), 256
    results = []
    for lanes, block, per_sm in ((1, 256, 8), (2, 256, 8), (4, 128, 2), (8, 256, 4), (1, 128, 4), (2, 128, 8)):
        ctx = _ctx(spec, 5, maxn=maxn)
        ctx.set_tuning(gather_lanes=lanes, pass_block=block, pass_blocks_per_sm=per_sm)
        assert ctx.tuning() == {"gather_lanes": lanes, "pass_block": block, "pass_blocks_per_sm": per_sm}
        for _ in range(8):
            ctx.substep(spec.dt)
        ctx.check_status()
        results.append(ctx.download()[0])
        ctx.close()
    for r in results[1:]:
        for k in r:
            assert np.array_equal(r[k], results[0][k]), k


def test_autotune_keeps_state():
    spec = scenes.dam_break(n_side=20)
    ctx = _ctx(spec, 6, target=1e-3)
    for _ in range(5):
        ctx.substep(spec.dt)
    ctx.check_status()
    before, _ = ctx.download()
    res = ctx.autotune()
    assert res["gather_lanes"] in (1, 2, 4, 8) and res["pass_block"] in (128, 256)
    assert len(res["pass_ms"]) == 24 and all(v > 0 for v in res["pass_ms"].values())
    assert ctx.tuning() == {k: res[k] for k in ("gather_lanes", "pass_block", "pass_blocks_per_sm")}
    after, _ = ctx.download()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    info = ctx.check_status()
    assert info.density_passes == 0  # the tuning passes are not counted
    # and the simulation continues like an untuned twin
    ref = _ctx(spec, 6, target=1e-3)
    for _ in range(5):
        ref.substep(spec.dt)
    for _ in range(3):
        ctx.substep(spec.dt)
        ref.substep(spec.dt)
    a, _ = ctx.download()
    b, _ = ref.download()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    ctx.close()
    ref.close()


def test_set_tuning_rejects_bad_shapes():
    from apbf_gb300._native import ApbfError

    spec = scenes.dam_break(n_side=8)
    ctx = _ctx(spec, 2)
    for bad in (dict(gather_lanes=3), dict(pass_block=192), dict(pass_blocks_per_sm=0), dict(pass_blocks_per_sm=9)):
        with pytest.raises(ApbfError):
            ctx.set_tuning(**bad)
    ctx.close()
