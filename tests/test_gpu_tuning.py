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
        assert ctx.tuning() == {"gather_lanes": lanes, "pass_block": block, "pass_blocks_per_sm": per_sm,
                                "filter_in_density": 0, "sort_digit_bits": 0, "search_log2res": 0}
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
    assert ctx.tuning() == {k: v for k, v in res.items() if k != "pass_ms"}
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


@pytest.mark.parametrize("lanes", [1, 4])
def test_deferred_filter_identical(lanes):
    """The Gauss boundariness filter run in the position pass (symmetric rows) gives
    the same substeps as running it in the density pass; a converged pass still
    filters."""
    spec = scenes.water_drop(total=30_000, seed=8, basic_pbf=True)
    out = []
    for inline in (1, 0):
        ctx = _ctx(spec, 30, target=2e-3, maxn=192)
        ctx.set_tuning(gather_lanes=lanes, filter_in_density=inline)
        for _ in range(25):
            ctx.substep(spec.dt)
        info = ctx.check_status()
        out.append((ctx.download()[0], info.density_passes, info.converged_substeps))
        ctx.close()
    (a, pa, ca), (b, pb, cb) = out
    assert (pa, ca) == (pb, cb)
    assert np.any(a["boundariness"] == 0) and np.any(a["boundariness"] > 0)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_search_tuning_restores_the_state_and_keeps_results():
    """apbf_autotune_search times sort digit widths and search grids, leaves the state
    it ran on unchanged, and its choice gives the same neighbour sets."""
    from apbf_gb300.api import Context

    spec = scenes.water_drop(total=30_000, seed=5, basic_pbf=True)

    def make():
        c = Context(particle_capacity=spec.n + 512, max_neighbors=160, max_log2res=spec.log2res + 1)
        c.set_settings(basic_pbf=1, solver_iterations=12, density_error_target=1e-3)
        c.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
        c.set_boxes(spec.box_min, spec.box_max)
        c.upload(spec.state)
        for _ in range(3):
            c.substep(spec.dt)
        return c

    ctx, ref = make(), make()
    before, _ = ctx.download()
    choice = ctx.autotune_search()
    assert choice["sort_digit_bits"] in (6, 7, 8)
    assert all(v > 0 for v in choice["sort_ms"].values())
    after, _ = ctx.download()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    # the next substep's search (on the same positions in both) finds the same pairs
    ctx.substep(spec.dt)
    ref.substep(spec.dt)
    assert ctx.check_status().pairs == ref.check_status().pairs, choice
    ctx.close()
    ref.close()


def test_tuners_on_spread_kernel_width_scene():
    """Kernel widths spread across neighbours (the rows the substep leaves are
    transposed rows) and the search tuner (whose searches leave correction rows while
    the status it restores names the transposed kind): the pass tuner and the next
    substeps run on those rows without error and the state stays finite."""
    spec = scenes.water_drop(total=20_000, seed=9, basic_pbf=False)
    ctx = _ctx(spec, spec.iterations, maxn=256)
    ctx.set_settings(base_kernel_width_on_boundary_distance=0)
    for _ in range(15):
        ctx.substep(spec.dt)
    ctx.check_status()
    ctx.autotune_search()
    ctx.autotune()
    for _ in range(5):
        ctx.substep(spec.dt)
    ctx.check_status()
    g, _ = ctx.download()
    assert np.all(np.isfinite(g["velocity"]))
    ctx.close()
