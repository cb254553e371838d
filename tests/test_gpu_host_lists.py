"""apbf_fluid_write / apbf_fluid_read (gpu_list::write / read of the particle lists
from and into host memory): round trips, lengths, fields left alone, and a
host-driven run (state written, one substep, state read back, every step) that ends
bit-identical to the same substeps on the device-resident state."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ctx(spec, cap):
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=cap, max_neighbors=160, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=20, density_error_target=1e-3)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    return ctx


def _host(cap):
    import torch

    from apbf_gb300.api import FLUID_FIELDS

    h = {k: torch.zeros((cap, c) if c > 1 else (cap,), dtype=dt).pin_memory() for k, (dt, c) in FLUID_FIELDS.items()}
    h["lambda_prev"] = torch.zeros(cap, dtype=torch.float32).pin_memory()
    return h


def test_write_read_round_trip():
    import torch

    spec = scenes.dam_break(n_side=12)
    n, cap = spec.n, spec.n + 500
    ctx = _ctx(spec, cap)
    ctx.upload(spec.state)
    a = _host(cap)
    cnt = torch.zeros(1, dtype=torch.int32).pin_memory()
    ctx.fluid_read(a, n, cnt)
    torch.cuda.synchronize()
    assert int(cnt[0]) == n
    st, _ = ctx.download()
    for k in st:
        got = a[k][:n].numpy()
        exp = st[k].view(got.dtype)
        if k in ("position", "pos_backup"):
            got, exp = got[:, :3], exp[:, :3]
        assert np.array_equal(got, exp), k
    # a shorter state written back: new length, the given fields replaced, absent ones kept
    b = {k: v.clone().pin_memory() for k, v in a.items() if k not in ("radius",)}
    b["velocity"][:, 1] += 1.0
    ctx.fluid_write(b, n - 100)
    torch.cuda.synchronize()
    assert ctx.lengths()[0] == n - 100
    c = _host(cap)
    ctx.fluid_read(c, cap, cnt)
    torch.cuda.synchronize()
    assert int(cnt[0]) == n - 100
    assert torch.equal(c["velocity"][: n - 100], b["velocity"][: n - 100])
    assert torch.equal(c["radius"][: n - 100], a["radius"][: n - 100])
    ctx.close()


def test_host_driven_substeps_match_resident():
    import torch

    spec = scenes.water_drop(total=20_000, seed=2, basic_pbf=True)
    cap = spec.n + 1000
    res = _ctx(spec, cap)
    res.upload(spec.state)
    hd = _ctx(spec, cap)
    hd.upload(spec.state)
    h = _host(cap)
    cnt = torch.zeros(1, dtype=torch.int32).pin_memory()
    n = spec.n
    hd.fluid_read(h, n, cnt)
    torch.cuda.synchronize()
    for _ in range(6):
        res.substep(spec.dt)
        hd.fluid_write(h, n)
        hd.substep(spec.dt)
        n, _ = hd.lengths()
        hd.fluid_read(h, n, cnt)
        torch.cuda.synchronize()
    a, _ = res.download()
    b, _ = hd.download()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert res.check_status().density_passes == hd.check_status().density_passes
    res.close()
    hd.close()


def test_pageable_and_unaligned_host_arrays():
    """Page-locked host arrays go through the one-launch copy kernel (16-byte units,
    or 4-byte units when an array starts off a 16-byte boundary), pageable ones
    through cudaMemcpyAsync; one call may mix them, in both directions."""
    import torch

    from apbf_gb300.api import FLUID_FIELDS

    spec = scenes.dam_break(n_side=12, seed=4)
    n, cap = spec.n, spec.n + 300
    ctx = _ctx(spec, cap)
    ctx.upload(spec.state)
    ref = _host(cap)
    cnt = torch.zeros(1, dtype=torch.int32).pin_memory()
    ctx.fluid_read(ref, n, cnt)
    torch.cuda.synchronize()

    def unaligned(dt, comp):
        flat = torch.zeros(cap * comp + 1, dtype=dt).pin_memory()
        v = flat[1:]  # starts 4 bytes past the allocation
        return v.view(cap, comp) if comp > 1 else v

    fields = dict(FLUID_FIELDS, lambda_prev=(torch.float32, 1))
    mixed = {}
    for k, (name, (dtype, c)) in enumerate(fields.items()):
        if k % 3 == 0:
            mixed[name] = np.zeros((cap, c) if c > 1 else (cap,), dtype=np.int32 if dtype == torch.int32 else np.float32)
        elif k % 3 == 1:
            mixed[name] = unaligned(dtype, c)
        else:
            mixed[name] = torch.zeros((cap, c) if c > 1 else (cap,), dtype=dtype).pin_memory()
    assert any(t.data_ptr() % 16 for t in mixed.values() if isinstance(t, torch.Tensor))
    ctx.fluid_read(mixed, n, cnt)
    torch.cuda.synchronize()
    for name in fields:
        got = mixed[name][:n]
        got = got.numpy() if isinstance(got, torch.Tensor) else got
        assert np.array_equal(got.view(np.uint32), ref[name][:n].numpy().view(np.uint32)), name
    # written back from the mixed arrays (changed), read into aligned pinned arrays
    mixed["velocity"][:n, 0] += 2.5
    ctx.fluid_write(mixed, n)
    out = _host(cap)
    ctx.fluid_read(out, n, cnt)
    torch.cuda.synchronize()
    for name in fields:
        exp = mixed[name][:n]
        exp = exp.numpy() if isinstance(exp, torch.Tensor) else exp
        assert np.array_equal(out[name][:n].numpy().view(np.uint32), exp.view(np.uint32)), name
    assert int(cnt[0]) == n
    ctx.close()
