"""Stages on the caller's own device memory (apbf_bind_lists), the reference's
ownership model: its stage objects keep pointers to lists the scene owns
(neighborhood_green.h:11, incompressibility.h:11, update_transfers.h:11,
particle_transfer.h:11).  A context bound to torch-allocated lists gives, stage by
stage and through apbf_substep, the states a context on its own lists gives, bit for
bit; the results sit in the caller's tensors (the current set as the views name it)
and the caller's length words follow every call."""
import numpy as np
import pytest
import torch

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ctx(spec, maxn):
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=int(spec.n * 1.3) + 512, max_neighbors=maxn, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=spec.iterations)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    return ctx


def _fill_caller(lists, state):
    """The scene's state written straight into the caller's set 0 and length words."""
    from apbf_gb300.api import FLUID_FIELDS

    n = state["position"].shape[0]
    for name, (dt, comps) in FLUID_FIELDS.items():
        a = np.ascontiguousarray(state[name]).view(np.int32 if dt == torch.int32 else np.float32)
        lists.fluid[0][name][:n].copy_(torch.from_numpy(a.reshape((n, comps) if comps > 1 else (n,))))
    lists.len_particles.fill_(n)
    lists.len_transfers.fill_(0)


@pytest.mark.parametrize("name,mode", [("dam_break", "stages"), ("water_drop_adaptive", "stages"),
                                       ("water_drop_adaptive", "substep")])
def test_bound_lists_equal_own_lists(name, mode):
    from apbf_gb300.api import CallerLists, SubstepStages

    if name == "dam_break":
        spec, maxn, steps = scenes.dam_break(n_side=14, seed=2), 128, 6
    else:
        spec, maxn, steps = scenes.water_drop(total=20_000, seed=4, basic_pbf=False), 256, 30
    own, bound = _ctx(spec, maxn), _ctx(spec, maxn)
    own.upload(spec.state)
    lists = CallerLists.for_context(bound)
    _fill_caller(lists, spec.state)
    bound.bind_lists(lists)
    run_own = SubstepStages(own).update if mode == "stages" else own.substep
    run_bound = SubstepStages(bound).update if mode == "stages" else bound.substep
    mine = {t["position"].data_ptr() for t in lists.fluid}
    for _ in range(steps):
        run_own(spec.dt)
        run_bound(spec.dt)
        torch.cuda.synchronize()
        assert bound.fluid_view()["position"].data_ptr() in mine  # the current set is the caller's
        assert int(lists.len_particles.item()) == bound.lengths()[0] == own.lengths()[0]
        assert int(lists.len_transfers.item()) == own.lengths()[1]
    own.check_status()
    bound.check_status()
    a, at = own.download()
    b, bt = bound.download()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    for k in at:
        assert np.array_equal(at[k], bt[k]), k
    # the caller's rows are the search's rows
    n = own.lengths()[0]
    assert np.array_equal(lists.count[:n].cpu().numpy(), own.neighbors_view()["count"][:n].cpu().numpy())
    bound.unbind_lists()
    own.close()
    bound.close()


def test_bind_rejects_bad_lists():
    from apbf_gb300._native import ApbfError
    from apbf_gb300.api import CallerLists

    spec = scenes.dam_break(n_side=8)
    ctx = _ctx(spec, 64)
    good = CallerLists.for_context(ctx)
    small = CallerLists(ctx.capacity - 1, ctx.transfer_capacity, good.row_stride, 64)
    with pytest.raises(ApbfError):
        ctx.bind_lists(small)
    wrong_stride = CallerLists(ctx.capacity, ctx.transfer_capacity, good.row_stride + 32, 64)
    with pytest.raises(ApbfError):
        ctx.bind_lists(wrong_stride)
    ctx.bind_lists(good)
    with pytest.raises(ApbfError):  # twice
        ctx.bind_lists(good)
    ctx.unbind_lists()
    ctx.close()
