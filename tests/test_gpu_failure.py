"""The failure path of the bounded device-side waits, exercised without a fault or a
hang: apbf_set_wait_limit(inject) makes each wait treat the flag it waits for as
never set, so the sort's and the scan's decoupled look-backs and the persistent
solve's grid barrier run out after a few spins.  The kernels return, the status
reports APBF_ERR_SPIN_LIMIT with the wait that gave up, and once the limit is back
to its default the same context sorts, scans and solves correctly again."""
import numpy as np
import pytest
import torch

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu

SPIN_LIMIT = 4  # APBF_ERR_SPIN_LIMIT


def _ctx(cap, maxn=8, L=3):
    from apbf_gb300.api import Context

    return Context(particle_capacity=cap, max_neighbors=maxn, max_log2res=L)


def _expect_give_up(ctx, where):
    torch.cuda.synchronize()
    info = ctx.status()
    assert ctx.last_status_code == SPIN_LIMIT, ctx.last_status_code
    assert info.spin_where == where, info.spin_where


def test_sort_lookback_gives_up_and_recovers():
    from apbf_gb300.api import algorithms

    n = 1 << 18  # 64 tiles of 4096 keys: every tile but the first waits on a predecessor
    ctx = _ctx(n)
    rng = np.random.default_rng(11)
    k = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    keys = torch.from_numpy(k.view(np.int32)).cuda()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    ok, ov = torch.empty_like(keys), torch.empty_like(vals)
    ctx.set_wait_limit(64, inject=True)
    algorithms.sort(ctx, keys, vals, cnt, n, ok, ov)
    _expect_give_up(ctx, 1)
    ctx.set_wait_limit(0)
    algorithms.sort(ctx, keys, vals, cnt, n, ok, ov)
    torch.cuda.synchronize()
    ctx.check_status()
    order = np.argsort(k, kind="stable").astype(np.uint32)
    assert np.array_equal(ov.cpu().numpy().view(np.uint32), order)
    ctx.close()


def test_scan_lookback_gives_up_and_recovers():
    from apbf_gb300.api import algorithms

    n = 1 << 18
    ctx = _ctx(n)
    v = np.random.default_rng(12).integers(0, 100, size=n).astype(np.uint32)
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    ctx.set_wait_limit(64, inject=True)
    d = torch.from_numpy(v.view(np.int32)).cuda()
    algorithms.prefix_sum(ctx, d, cnt, n)
    _expect_give_up(ctx, 2)
    ctx.set_wait_limit(0)
    d = torch.from_numpy(v.view(np.int32)).cuda()
    algorithms.prefix_sum(ctx, d, cnt, n)
    torch.cuda.synchronize()
    ctx.check_status()
    assert np.array_equal(d.cpu().numpy().view(np.uint32), np.cumsum(v, dtype=np.uint64).astype(np.uint32))
    ctx.close()


def test_persistent_solve_barrier_gives_up_and_recovers():
    spec = scenes.dam_break(n_side=16)

    def make():
        ctx = _ctx(int(spec.n * 1.3) + 64, maxn=128, L=max(spec.log2res, 3))
        ctx.set_settings(basic_pbf=1, solver_iterations=6, density_error_target=0.0)
        ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
        ctx.set_boxes(spec.box_min, spec.box_max)
        ctx.upload(spec.state)
        ctx.set_solve_graph(0)
        ctx.set_persistent_solve(True)
        return ctx

    ctx = make()
    ctx.set_wait_limit(64, inject=True)
    ctx.substep(spec.dt)
    _expect_give_up(ctx, 3)
    # restored: the same context runs substeps again, identical to a context whose first
    # substep did not give up (both restart from the scene's state after one substep)
    ctx.set_wait_limit(0)
    ctx.upload(spec.state)
    ref = make()
    ref.substep(spec.dt)
    ref.check_status()
    ref.upload(spec.state)
    for _ in range(3):
        ctx.substep(spec.dt)
        ref.substep(spec.dt)
    ctx.check_status()
    ref.check_status()
    a, _ = ctx.download()
    b, _ = ref.download()
    for key in a:
        assert np.array_equal(a[key], b[key]), key
    ctx.close()
    ref.close()
