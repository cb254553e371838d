"""The reference's operator API as a binding would use it: the stage objects
(set_data / apply) run in pool::update order (SubstepStages.update) give the state
that apbf_substep gives, bit for bit, over several substeps of a plain and of an
adaptive scene, and of a small waterfall's pre-filled stream over its oriented slope
box (the stage objects have no emitter stage, so the emitter is off).  apbf_substep
fuses the box passes into the kernels before them and runs the passes from graphs;
the stages launch every pass on its own."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ctx(spec, maxn):
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=int(spec.n * 1.3) + 512, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=spec.iterations)
    ctx.load_scene(spec)
    return ctx


@pytest.mark.parametrize("name", ["dam_break", "water_drop_adaptive", "waterfall"])
def test_stage_objects_equal_substep(name):
    from apbf_gb300.api import SubstepStages

    if name == "dam_break":
        spec, maxn, steps = scenes.dam_break(n_side=14, seed=2), 128, 8
    elif name == "waterfall":
        spec, maxn, steps = scenes.waterfall(initial=12_000, seed=3, scale=0.35, per_substep=300), 256, 60
        spec.meta["emitter"] = None
    else:
        spec, maxn, steps = scenes.water_drop(total=20_000, seed=4, basic_pbf=False), 256, 40
    fused, staged = _ctx(spec, maxn), _ctx(spec, maxn)
    stages = SubstepStages(staged)
    for _ in range(steps):
        fused.substep(spec.dt)
        stages.update(spec.dt)
    a_info, b_info = fused.check_status(), staged.check_status()
    assert a_info.pairs == b_info.pairs
    a, at = fused.download()
    b, bt = staged.download()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    for k in at:
        assert np.array_equal(at[k], bt[k]), k
    if name == "water_drop_adaptive":  # the adaptive stages acted
        assert np.unique(a["target_radius"]).size > 1 or at["source"].size > 0 or np.unique(a["radius"]).size > 1
    fused.close()
    staged.close()
