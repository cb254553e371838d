"""Oracle self-consistency: kernel gradients against finite differences of the
heights (kernels.glsl), Jacobi invariants, box collision containment, velocity
handling in exact FP32 and the adaptive stages' conservation laws."""
import ctypes as C

import numpy as np
import pytest

from apbf_gb300 import scenes


def _h(orc, kid, r, kw):
    a = (C.c_double * 3)(*r)
    return orc.lib().or_kernel_height(kid, a, kw)


def _g(orc, kid, r, kw):
    a = (C.c_double * 3)(*r)
    o = (C.c_double * 3)()
    orc.lib().or_kernel_gradient(kid, a, kw, o)
    return np.array(list(o))


@pytest.mark.parametrize("kid", [0, 1, 3, 4])  # poly6 height pairs with the spiky gradient: not a derivative pair
def test_gradient_is_height_derivative(orc, kid):
    kw = 4.0
    rng = np.random.default_rng(kid)
    for _ in range(20):
        r = rng.uniform(-2.5, 2.5, size=3)
        if np.linalg.norm(r) < 0.2 or abs(np.linalg.norm(r) - kw / 2) < 1e-3:
            continue
        g = _g(orc, kid, r, kw)
        eps = 1e-6
        fd = np.array([(_h(orc, kid, r + eps * e, kw) - _h(orc, kid, r - eps * e, kw)) / (2 * eps) for e in np.eye(3)])
        assert np.allclose(g, fd, rtol=1e-5, atol=1e-9), (kid, r, g, fd)


def test_gauss_density_of_lattice_near_one(orc):
    # rest lattice (spacing 2r) with the default Gauss kernel: rho * rho0^-1 close to 1 in the bulk
    st = scenes.make_state(scenes.lattice([1, 1, 1], [12, 12, 12], 2.0, 0.0, np.random.default_rng(0)))
    fs = orc.FluidState(st)
    orc.neighborhood_green(fs, 1.0, (-4.0, -4.0, -4.0), (28.0, 28.0, 28.0), 3, 1 << 20)
    s = orc.settings_from({**_defaults(), "basic_pbf": 1})
    out = orc.incompressibility(fs, s)
    dens = out["density"] / 262144.0
    centre = np.all(np.abs(st["position"][:, :3] / 262144.0 - 12.0) < 3.0, axis=1)
    s2 = fs.state()
    centre = np.all(np.abs(s2["position"][:, :3] / 262144.0 - 12.0) < 3.0, axis=1)
    ratio = dens[centre] * (2.0 ** 3) * (1.0 / 8.0)
    assert np.all(np.abs(ratio - 1.0) < 0.1), ratio


def _defaults():
    return dict(height_kernel_id=1, gradient_kernel_id=1, merge=1, split=1, base_kernel_width_on_target_radius=1,
                base_kernel_width_on_boundary_distance=1, update_target_radius=1, update_boundariness=1,
                boundariness_calculation_method=2, basic_pbf=0, solver_iterations=3, boundariness_adaption_speed=0.5,
                kernel_width_adaption_speed=0.01, boundariness_self_grad_length_factor=2.0,
                boundariness_underpressure_factor=4.0, merge_duration=2.0, split_duration=0.0,
                smallest_target_radius=1.0, target_radius_offset=10.0, target_radius_scale_factor=0.3)


def test_compressed_block_expands(orc):
    # a lattice compressed to spacing 1.8r has lambda < 0 inside and spreads out
    st = scenes.make_state(scenes.lattice([1, 1, 1], [10, 10, 10], 1.8, 0.0, np.random.default_rng(0)))
    fs = orc.FluidState(st)
    orc.neighborhood_green(fs, 1.0, (-4.0, -4.0, -4.0), (28.0, 28.0, 28.0), 3, 1 << 20)
    before = fs.state()["position"][:, :3].astype(np.float64)
    out = orc.incompressibility(fs, orc.settings_from({**_defaults(), "basic_pbf": 1}))
    after = fs.state()["position"][:, :3].astype(np.float64)
    assert np.sum(out["lambda"] < 0) > 0.5 * fs.n
    spread = lambda p: np.mean(np.linalg.norm(p - p.mean(axis=0), axis=1))
    assert spread(after) > spread(before)


def test_box_collision_contains(orc):
    rng = np.random.default_rng(3)
    pos = rng.uniform(-6, 40, size=(500, 3))
    st = scenes.make_state(pos)
    bmin, bmax = scenes.wall_boxes([0, 0, 0], [32, 32, 32])
    fs = orc.FluidState(st)
    orc.box_collision(fs, bmin, bmax)
    p = fs.state()["position"][:, :3] / 262144.0
    inside = np.all((p > -0.2) & (p < 34.3), axis=1)
    start_inside = np.all((pos > 1.2) & (pos < 30.8), axis=1)
    assert np.all(inside[start_inside])
    # particles that started inside (clear of the walls) do not move
    s_in = fs.state()["position"][start_inside]
    assert np.array_equal(s_in, st["position"][start_inside])


def test_velocity_handling_fp32(orc):
    st = scenes.make_state(np.array([[10.0, 10.0, 10.0], [20.0, 5.0, 3.0]]))
    st["pos_backup"][0, :3] -= np.array([1000, -2000, 5], np.int32)
    fs = orc.FluidState(st)
    orc.velocity_handling(fs, np.float32(1 / 120), np.float32(1 / 120), (0.0, -392.4, 0.0))
    s = fs.state()
    dt = np.float32(1.0 / 120.0)
    v0 = np.float32(1000) / (dt * np.float32(262144.0))
    assert s["velocity"][0, 0] == v0
    a = np.float32(-392.4) * dt
    assert s["velocity"][1, 1] == np.float32(0.0) + a
    assert np.array_equal(s["pos_backup"], st["position"])


def _adaptive_state(orc, n_side=10, seed=0):
    """A compressed block of small particles deep inside (merge candidates: nearest
    neighbour closer than one radius, large boundary distance) next to a layer of
    large particles at the surface (split candidates: radius above 1.26 x target)."""
    rng = np.random.default_rng(seed)
    small = scenes.lattice([1, 1, 1], [n_side, n_side, n_side], 0.9, 0.05, rng)
    big = scenes.lattice([1, 1 + 0.9 * n_side + 2.0, 1], [n_side // 2, 2, n_side // 2], 4.0, 0.1, rng)
    st = scenes.make_state(np.concatenate([small, big]))
    nb = big.shape[0]
    st["radius"][-nb:] = 2.0
    st["inverse_mass"][-nb:] = np.float32(1.0 / 64.0)
    bd = np.full(st["radius"].shape, 60.0)
    bd[-nb:] = 1.0
    st["boundary_distance"] = (bd * 262144).astype(np.uint32)
    st["kernel_width"][-nb:] = 8.0
    return st


def test_update_transfers_and_transfer_conserve_mass(orc):
    st = _adaptive_state(orc)
    fs = orc.FluidState(st, cap=int(st["radius"].size * 2))
    s = orc.settings_from(_defaults())
    orc.neighborhood_green(fs, 1.0, (-4.0, -4.0, -4.0), (28.0, 28.0, 28.0), 3, 1 << 20)
    m0, v0, _ = orc.reduce(fs)
    orc.update_transfers(fs, s, 10000)
    tr = fs.transfers()
    assert np.sum(tr["time_left"] > 0) > 0   # merges
    assert np.sum(tr["time_left"] <= 0) > 0  # splits
    # claims are exclusive: every particle appears in at most one transfer
    ids = np.concatenate([tr["source"], tr["target"]])
    assert np.unique(ids).size == ids.size
    tf = fs.state()["transferring"]
    assert set(np.flatnonzero(tf).tolist()) == set(ids.tolist())
    m1, v1, _ = orc.reduce(fs)
    assert m1 == pytest.approx(m0, rel=1e-12)  # duplicates carry no mass until the transfer runs
    for _ in range(3):
        orc.particle_transfer(fs, np.float32(1 / 240))
        m2, v2, _ = orc.reduce(fs)
        assert m2 == pytest.approx(m0, rel=1e-6)
        assert v2 == pytest.approx(v0, rel=1e-5)


def test_update_transfers_deterministic(orc):
    st = _adaptive_state(orc, seed=4)
    res = []
    for _ in range(2):
        fs = orc.FluidState(st, cap=int(st["radius"].size * 2))
        orc.neighborhood_green(fs, 1.0, (-4.0, -4.0, -4.0), (28.0, 28.0, 28.0), 3, 1 << 20)
        orc.update_transfers(fs, orc.settings_from(_defaults()), 10000)
        res.append((fs.state(), fs.transfers()))
    for k in res[0][0]:
        assert np.array_equal(res[0][0][k], res[1][0][k])
    for k in res[0][1]:
        assert np.array_equal(res[0][1][k], res[1][1][k])


def test_transfer_capacity_keeps_first_in_index_order(orc):
    st = _adaptive_state(orc, seed=5)
    s = orc.settings_from({**_defaults(), "split": 0})
    fs_full = orc.FluidState(st)
    orc.neighborhood_green(fs_full, 1.0, (-4.0, -4.0, -4.0), (28.0, 28.0, 28.0), 3, 1 << 20)
    orc.update_transfers(fs_full, s, 10000)
    full = fs_full.transfers()
    k = max(full["source"].size // 2, 1)
    fs_cap = orc.FluidState(st)
    orc.neighborhood_green(fs_cap, 1.0, (-4.0, -4.0, -4.0), (28.0, 28.0, 28.0), 3, 1 << 20)
    orc.update_transfers(fs_cap, s, k)
    cap = fs_cap.transfers()
    assert np.array_equal(cap["source"], full["source"][:k])
    assert np.array_equal(cap["target"], full["target"][:k])
    assert int(np.sum(fs_cap.state()["transferring"])) == 2 * k
