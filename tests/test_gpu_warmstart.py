"""The learned warm start on the GPU: the BF16 tensor-core forward / backward /
Adam kernels against the FP64 network of the oracle, the samples a substep
records against the oracle's Jacobi passes, the learned first update against the
oracle's pass with the same lambda, and what a trained network saves."""
import numpy as np
import pytest

from apbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def _net_params(seed=0):
    from oracle import mlp_oracle as M

    rng = np.random.default_rng(seed)
    p = np.zeros(M.P_N, np.float32)
    p[M.P_MU:M.P_MU + 5] = rng.normal(size=5)
    p[M.P_IS:M.P_IS + 5] = rng.uniform(0.5, 2.0, size=5)
    p[M.P_W1:M.P_B1] = rng.normal(size=M.H * M.F) * 0.6
    p[M.P_W1:M.P_B1].reshape(M.H, M.F)[:, 5:] = 0.0
    p[M.P_B1:M.P_W2] = rng.normal(size=M.H) * 0.1
    p[M.P_W2:M.P_B2] = rng.normal(size=M.H * M.H) * 0.2
    p[M.P_B2:M.P_W3] = rng.normal(size=M.H) * 0.1
    p[M.P_W3:M.P_B3] = rng.normal(size=M.H) * 0.2
    p[M.P_B3] = 0.3
    p[M.P_YS] = 2.0
    p[M.P_YM] = -1.0
    return p


def _features(n, seed=1):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, 8), np.float32)
    X[:, :5] = rng.normal(size=(n, 5))
    return X


def _net(p):
    from apbf_gb300.warmstart import WarmStartNet

    net = WarmStartNet()
    net.load_state(p)
    return net


@pytest.mark.parametrize("n", [1, 127, 1000, 70001])
def test_forward_matches_oracle(n):
    import torch
    from oracle import mlp_oracle as M

    p = _net_params()
    X = _features(n)
    y = _net(p).forward(torch.from_numpy(X).cuda()).cpu().numpy().astype(np.float64)
    ref_q = M.predict(p, X, bf16=True)    # same BF16 operand rounding, FP64 accumulation
    ref = M.predict(p, X, bf16=False)     # the exact network
    scale = np.abs(ref).max() + 1.0
    err = np.abs(y - ref_q)
    # FP32 vs FP64 hidden activations can round to neighbouring BF16 values (a rare
    # flip of 2^-8 relative in one of 64 inputs): tight for 99.9 %, bounded for all
    assert np.percentile(err, 99.9) <= 1e-4 * scale, np.percentile(err, 99.9)
    assert err.max() <= 2e-3 * scale, err.max()
    assert np.all(np.abs(y - ref) <= 3e-2 * scale), np.abs(y - ref).max()


@pytest.mark.parametrize("n,over", [(96, 1.0), (1000, 1.0), (4099, 1.0), (1000, 8.0)])
def test_gradient_matches_oracle(n, over):
    import torch
    from oracle import mlp_oracle as M

    p = _net_params(2)
    X = _features(n, 3)
    T = np.tanh(X[:, 0]) + 0.5 * X[:, 3] - 0.2 * X[:, 1] * X[:, 2]
    loss, g = _net(p).gradient(torch.from_numpy(X).cuda(), torch.from_numpy(T.astype(np.float32)).cuda(), over)
    g = g.cpu().numpy().astype(np.float64)
    l_q, g_q = M.loss_and_grad(p, X, T, bf16=True, over_weight=over)
    l_x, g_x = M.loss_and_grad(p, X, T, bf16=False, over_weight=over)
    assert loss == pytest.approx(l_q, rel=1e-4)
    assert loss == pytest.approx(l_x, rel=2e-2)
    blocks = {"W1": (M.P_W1, M.P_B1), "b1": (M.P_B1, M.P_W2), "W2": (M.P_W2, M.P_B2), "b2": (M.P_B2, M.P_W3),
              "w3": (M.P_W3, M.P_B3), "b3": (M.P_B3, M.P_B3 + 1)}
    for name, (a, b) in blocks.items():
        sc = np.abs(g_q[a:b]).max()
        err = np.abs(g[a:b] - g_q[a:b]).max()
        assert err <= 2e-3 * sc + 1e-7, (name, err, sc)
        # against the exact network: BF16 operands cost a few per cent at most
        cos = np.dot(g[a:b], g_x[a:b]) / (np.linalg.norm(g[a:b]) * np.linalg.norm(g_x[a:b]) + 1e-30)
        assert cos > 0.995, (name, cos)
    assert np.all(g[:M.P_W1] == 0) and np.all(g[M.P_B3 + 1:] == 0)


def test_adam_step_matches_oracle():
    import torch
    from oracle import mlp_oracle as M

    p = _net_params(4)
    X = _features(2000, 5)
    T = (np.sin(X[:, 0]) + X[:, 4]).astype(np.float32)
    net = _net(p)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    _, g0 = net.gradient(Xd, Td)
    net.train_step(Xd, Td, 1e-3)
    got = net.state().astype(np.float64)
    # Adam from the device gradient in FP64: step 0, so m = 0.1 g, v = 0.001 g^2
    ref = p.astype(np.float64).copy()
    m = np.zeros(M.P_N)
    v = np.zeros(M.P_N)
    M.adam(ref, m, v, g0.cpu().numpy().astype(np.float64), 1e-3, 0)
    assert np.allclose(got, ref, rtol=1e-5, atol=2e-6), np.abs(got - ref).max()
    assert np.array_equal(got[:M.P_W1], p[:M.P_W1]) and np.array_equal(got[M.P_B3 + 1:], p[M.P_B3 + 1:])


def test_training_fits_a_smooth_target():
    import torch

    from apbf_gb300.warmstart import WarmStartNet

    X = _features(200_000, 6)
    T = (np.tanh(X[:, 0]) * X[:, 3] + 0.3 * X[:, 1]).astype(np.float32)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    net = WarmStartNet(seed=1)
    net.set_normalization(Xd, Td)
    hist = net.fit(Xd, Td, epochs=6, batch=8192, lr=3e-3, lr_final=3e-4)
    assert np.all(np.isfinite(hist))
    assert hist[-1] < 0.07 * hist[0] and hist[-1] < 0.045, hist
    pred = net.forward(Xd).cpu().numpy()
    assert np.sqrt(np.mean((pred - T) ** 2)) < 0.22 * np.std(T)


# ----------------------------------------------------------------- solver hooks
def _free_block(n_side=10, seed=0, iterations=3):
    from dataclasses import replace

    spec = scenes.dam_break(n_side=n_side, seed=seed, iterations=iterations)
    rng = np.random.default_rng(seed)
    pos = scenes.lattice([20, 20, 20], [n_side] * 3, 1.8, 0.2, rng)
    st = scenes.make_state(pos)
    # a random velocity field (velocity_handling infers v from position - backup over last_dt = 1)
    v = rng.normal(size=(pos.shape[0], 3)) * 2.0
    st["pos_backup"][:, :3] = st["position"][:, :3] - np.trunc(v * 262144.0).astype(np.int32)
    return replace(spec, state=st, box_min=np.zeros((0, 4), np.float32), box_max=np.zeros((0, 4), np.float32))


def _ctx(spec, iterations):
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=spec.n, max_neighbors=128, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1, solver_iterations=iterations)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    return ctx


def _oracle_first_pass(orc, spec, ctx):
    fs = orc.FluidState(spec.state)
    orc.velocity_handling(fs, np.float32(spec.dt), np.float32(1.0), spec.acceleration)
    orc.neighborhood_green(fs, 1.0, spec.grid_min, spec.grid_max, spec.log2res, 1 << 22)
    return fs, orc.settings_from(ctx.settings)


def test_recorded_samples_match_oracle(orc):
    import torch

    from apbf_gb300.warmstart import SampleBuffer
    from test_gpu_solver import _lambda_tolerance

    spec = _free_block()
    K = 3
    ctx = _ctx(spec, K)
    buf = SampleBuffer.allocate(spec.n + 100)
    buf.count.fill_(100)  # appends after existing samples
    ctx.record_samples(K, buf.features, buf.targets, buf.count)
    ctx.substep(spec.dt)
    ctx.check_status()
    assert buf.size() == spec.n + 100
    X = buf.features[100:].cpu().numpy()
    T = buf.targets[100:].cpu().numpy()
    assert np.all(buf.features[:100].cpu().numpy() == 0)

    fs, s = _oracle_first_pass(orc, spec, ctx)
    before = fs.state()
    rows = fs.rows()
    outs = [orc.incompressibility(fs, s)]
    for _ in range(K - 1):
        outs.append(orc.incompressibility(fs, s))
    r = before["radius"].astype(np.float64)
    im = before["inverse_mass"].astype(np.float64)
    ird = (2.0 * r) ** 3 * im
    dens = outs[0]["density"].astype(np.float64) / 262144.0
    assert np.array_equal(X[:, 0], np.array([len(x) for x in rows], np.float32))
    assert np.all(np.abs(X[:, 1] - (dens * ird - 1.0)) <= 1e-5 + 8.0 / 262144.0 * ird)
    assert np.array_equal(X[:, 2], before["kernel_width"] / before["radius"])
    lam0 = outs[0]["lambda"].astype(np.float64)
    tol0 = _lambda_tolerance(before, outs[0], rows)
    assert np.all(np.abs(X[:, 3] - lam0) <= tol0)
    div = outs[0]["divergence"].astype(np.float64) / dens
    dsc = np.abs(div).max()
    assert np.all(np.abs(X[:, 4] - div) <= 1e-4 * np.abs(div) + 1e-4 * dsc), np.abs(X[:, 4] - div).max()
    assert np.all(X[:, 5:] == 0)  # no lambda history before the first substep (f5, f6), f7 unused
    tgt = sum(np.minimum(o["lambda"].astype(np.float64), 0.0) for o in outs)
    tsc = np.abs(tgt).max()
    assert tsc > 0
    err = np.abs(T - tgt)
    # passes 2..K start from FP32 vs FP64 positions that differ by truncations
    assert np.percentile(err, 99) <= 2e-3 * tsc and err.max() <= 2e-2 * tsc, (np.percentile(err, 99), err.max(), tsc)
    ctx.close()


def test_previous_substep_lambda_feature():
    """f5 of a substep is the sum of the lambdas applied to the particle in the
    previous substep, carried through that substep's sort: with K = all passes
    (no early stop) the recorded target of substep 1 is the same multiset of
    values as f5 of substep 2."""
    from apbf_gb300.warmstart import SampleBuffer

    spec = _free_block(n_side=9, seed=3)
    ctx = _ctx(spec, 4)
    buf = SampleBuffer.allocate(2 * spec.n)
    for _ in range(2):
        ctx.record_samples(4, buf.features, buf.targets, buf.count)
        ctx.substep(spec.dt)
    ctx.check_status()
    assert buf.size() == 2 * spec.n
    X = buf.features.cpu().numpy()
    T = buf.targets.cpu().numpy()
    assert np.all(X[:spec.n, 5] == 0)
    assert np.any(T[:spec.n] < 0)
    assert np.array_equal(np.sort(X[spec.n:, 5]), np.sort(T[:spec.n]))
    # f6: the mean of f5 over the particle's neighbours (rows of the second substep)
    rows = ctx.download_rows()
    X2 = X[spec.n:]
    want = np.array([X2[r, 5].astype(np.float64).mean() if len(r) else 0.0 for r in rows])
    assert np.allclose(X2[:, 6], want, rtol=1e-5, atol=1e-6 * np.abs(want).max())
    assert np.any(want != 0)
    ctx.close()


def test_record_capacity_is_respected(orc):
    from apbf_gb300.warmstart import SampleBuffer

    spec = _free_block(n_side=8)
    ctx = _ctx(spec, 2)
    buf = SampleBuffer.allocate(spec.n + spec.n // 2)
    for _ in range(2):
        ctx.record_samples(2, buf.features, buf.targets, buf.count)
        ctx.substep(spec.dt)
    ctx.substep(spec.dt)  # not armed: appends nothing
    ctx.check_status()
    assert buf.size() == spec.n + spec.n // 2
    ctx.close()


def test_learned_first_update_matches_oracle(orc):
    """A network whose output is a constant c: the first position update of the
    substep uses lambda = c for every particle (self shift and neighbour shifts),
    exactly like the oracle's pass with lambda_in = c."""
    import torch
    from oracle import mlp_oracle as M

    spec = _free_block(seed=1)
    ctx = _ctx(spec, 1)
    fs, s = _oracle_first_pass(orc, spec, ctx)
    plain = orc.FluidState(fs.state())
    orc.set_rows(plain, fs.rows())
    lam = orc.incompressibility(plain, s)["lambda"]  # the plain first update, for contrast
    c = float(np.float32(0.6 * np.median(lam)))
    assert c < 0
    p = np.zeros(M.P_N, np.float32)
    p[M.P_YS] = 1.0
    p[M.P_YM] = c
    ctx.mlp_load(torch.from_numpy(p).cuda())
    ctx.set_warm_start(True)
    ctx.substep(spec.dt)
    ctx.check_status()
    g, _ = ctx.download()
    before = fs.state()
    orc.incompressibility(fs, s, lambda_in=np.full(spec.n, c, np.float32))
    o = fs.state()
    x = g["position"][:, :3].astype(np.int64)
    xo = o["position"][:, :3].astype(np.int64)
    assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), np.abs(x - xo).max()
    assert np.abs(plain.state()["position"][:, :3].astype(np.int64) - xo).max() > 1000
    assert np.abs(xo - before["position"][:, :3]).max() > 1000
    ctx.close()


def test_learned_first_update_over_relaxation_clamp(orc):
    """omega_max > 0: the learned lambda is clamped to [omega_max * lambda0, lambda0]
    where the plain lambda0 of the pass is negative, 0 elsewhere."""
    import torch
    from oracle import mlp_oracle as M

    spec = _free_block(seed=2)
    ctx = _ctx(spec, 1)
    fs, s = _oracle_first_pass(orc, spec, ctx)
    plain = orc.FluidState(fs.state())
    orc.set_rows(plain, fs.rows())
    lam0 = orc.incompressibility(plain, s)["lambda"].astype(np.float64)
    assert np.any(lam0 < 0) and np.any(lam0 >= 0)
    c = float(np.float32(4.0 * np.median(lam0[lam0 < 0])))
    om = 2.0
    p = np.zeros(M.P_N, np.float32)
    p[M.P_YS] = 1.0
    p[M.P_YM] = c
    p[M.P_OMEGA] = om
    ctx.mlp_load(torch.from_numpy(p).cuda())
    ctx.set_warm_start(True)
    ctx.substep(spec.dt)
    ctx.check_status()
    g, _ = ctx.download()
    lam_in = np.where(lam0 < 0, np.clip(c, om * lam0, lam0), 0.0).astype(np.float32)
    assert np.any(lam_in == np.float32(c)) or np.any(lam_in > c)
    orc.incompressibility(fs, s, lambda_in=lam_in)
    x = g["position"][:, :3].astype(np.int64)
    xo = fs.state()["position"][:, :3].astype(np.int64)
    assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), np.abs(x - xo).max()
    ctx.close()


def test_learned_first_update_neighbour_gate(orc):
    """min_neighbors: particles with fewer neighbours keep the plain lambda in the
    learned update, the others take the network's."""
    import torch
    from oracle import mlp_oracle as M

    spec = _free_block(seed=5)
    ctx = _ctx(spec, 1)
    fs, s = _oracle_first_pass(orc, spec, ctx)
    counts = np.array([len(r) for r in fs.rows()])
    plain = orc.FluidState(fs.state())
    orc.set_rows(plain, fs.rows())
    lam0 = orc.incompressibility(plain, s)["lambda"].astype(np.float64)
    nmin = float(np.median(counts))
    c = float(np.float32(2.0 * np.median(lam0[lam0 < 0])))
    p = np.zeros(M.P_N, np.float32)
    p[M.P_YS] = 1.0
    p[M.P_YM] = c
    p[M.P_NMIN] = nmin
    ctx.mlp_load(torch.from_numpy(p).cuda())
    ctx.set_warm_start(True)
    ctx.substep(spec.dt)
    ctx.check_status()
    g, _ = ctx.download()
    gated = counts < nmin
    assert 0.2 < gated.mean() < 0.8
    lam_in = np.where(gated, np.minimum(lam0, 0.0), c).astype(np.float32)
    orc.incompressibility(fs, s, lambda_in=lam_in)
    x = g["position"][:, :3].astype(np.int64)
    xo = fs.state()["position"][:, :3].astype(np.int64)
    assert np.all(np.abs(x - xo) <= 1e-5 * np.abs(xo) + 64), np.abs(x - xo).max()
    ctx.close()


def test_projected_passes_match_oracle(orc):
    """A learned first update that over-pushes (a constant lambda 3x the median
    plain one), then two projected passes: where a particle ends up under-dense
    after being pushed, the pass pulls it back by up to the substep's push sum --
    the same rule as the oracle's projected pass."""
    import torch
    from oracle import mlp_oracle as M

    spec = _free_block(seed=4)
    ctx = _ctx(spec, 3)
    fs, s = _oracle_first_pass(orc, spec, ctx)
    plain = orc.FluidState(fs.state())
    orc.set_rows(plain, fs.rows())
    lam0 = orc.incompressibility(plain, s)["lambda"].astype(np.float64)
    c = float(np.float32(3.0 * np.median(lam0[lam0 < 0])))
    p = np.zeros(M.P_N, np.float32)
    p[M.P_YS] = 1.0
    p[M.P_YM] = c
    ctx.mlp_load(torch.from_numpy(p).cuda())
    ctx.set_warm_start(True)
    ctx.substep(spec.dt)
    ctx.check_status()
    g, _ = ctx.download()
    acc = np.full(spec.n, c, np.float32)
    orc.incompressibility(fs, s, lambda_in=acc)
    pulled = 0
    for _ in range(2):
        out = orc.incompressibility(fs, s, projected_acc=acc)
        pulled += int(np.sum(out["applied"] > 0))
        acc = acc + out["applied"]
    assert pulled > 0 and np.all(acc <= 0)
    x = g["position"][:, :3].astype(np.int64)
    xo = fs.state()["position"][:, :3].astype(np.int64)
    assert np.all(np.abs(x - xo) <= 3e-5 * np.abs(xo) + 256), np.abs(x - xo).max()
    ctx.close()


def test_warm_start_needs_parameters():
    from apbf_gb300._native import ApbfError

    spec = _free_block(n_side=6)
    ctx = _ctx(spec, 1)
    with pytest.raises(ApbfError):
        ctx.set_warm_start(True)
    ctx.close()


# ----------------------------------------------------------------- what it gains
def _drop(seed):
    from apbf_gb300.api import Context

    spec = scenes.water_drop(total=60_000, seed=seed, basic_pbf=True)
    ctx = Context(int(spec.n * 1.25) + 1024, max_neighbors=192, max_log2res=max(spec.log2res, 3))
    ctx.set_settings(basic_pbf=1, solver_iterations=100, density_error_target=1e-3)
    ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
    ctx.set_boxes(spec.box_min, spec.box_max)
    ctx.upload(spec.state)
    return spec, ctx


def test_trained_network_saves_passes_on_held_out_seed():
    """Train on projected-rule rollouts of two water drops (seeds 1, 2), then run a
    third (seed 0, never seen) after impact: at the same 0.1 % target every
    substep converges in each form, and the learned first update needs fewer
    density passes than the same solve without it and than the reference rule.
    The validation that picks the network and its over-relaxation bound on a
    fourth seed (3) is reproducible and keeps to its kinetic-energy rule."""
    from apbf_gb300 import _native as N
    from apbf_gb300.warmstart import SampleBuffer, ValidationCase, WarmStartNet, record_rollout, select_warm_start

    make = _drop
    buf = SampleBuffer.allocate(12_000_000)
    for seed in (1, 2):
        spec, ctx = make(seed)
        ctx.set_warm_start(N.WARM_PROJECTED)
        record_rollout(ctx, spec.dt, spec.meta["presteps"] + 40, buf, iterations=100, every=2)
        ctx.check_status()
        ctx.close()
    X, T = buf.view()
    net = WarmStartNet(seed=0)
    net.set_normalization(X, T)
    hist = net.fit(X, T, epochs=3, batch=32768)
    assert hist[-1] < hist[0]
    net.min_neighbors = 16.0
    net.omega_max = 2.0

    def evaluate(mode):
        spec, ctx = make(0)
        if mode & N.WARM_LEARNED:
            ctx.mlp_load(net.params)
        if mode:
            ctx.set_warm_start(mode)
        for _ in range(spec.meta["presteps"]):
            ctx.substep(spec.dt)
        ctx.check_status()
        for _ in range(30):
            ctx.substep(spec.dt)
        info = ctx.check_status()
        ctx.close()
        return info.density_passes / 30.0, info.converged_substeps

    learned = evaluate(N.WARM_LEARNED | N.WARM_PROJECTED)
    projected = evaluate(N.WARM_PROJECTED)
    reference = evaluate(0)
    assert learned[1] == projected[1] == reference[1] == 30, (learned, projected, reference)
    assert learned[0] < 0.8 * projected[0], (learned, projected)
    assert learned[0] < reference[0], (learned, reference)

    # network and bound by validation on seed 3: every run starts from the scene's
    # start, so the table repeats exactly; the winner is admissible and has the
    # fewest passes among the admissible; with no energy allowance nothing is
    def vmake(mode, params):
        spec, ctx = make(3)
        if params is not None:
            ctx.mlp_load(params)
        if mode:
            ctx.set_warm_start(mode)
        return ctx

    vspec = scenes.water_drop(total=60_000, seed=3, basic_pbf=True)
    case = ValidationCase(make=vmake, dt=vspec.dt, before=vspec.meta["presteps"], counted=12)
    nets = {"a": net}
    choice, table = select_warm_start(nets, [case], (1.5, 2.0, 4.0))
    again, table2 = select_warm_start(nets, [case], (1.5, 2.0, 4.0))
    assert table2 == table
    cands = table["candidates"]
    admissible = {k: v for k, v in cands.items() if v["admissible"]}
    if choice is None:
        assert not admissible and again is None
    else:
        assert again["omega_max"] == choice["omega_max"]
        assert (net.omega_max, net.min_neighbors) == (choice["omega_max"], choice["min_neighbors"])
        assert cands[f"a / omega {choice['omega_max']:g}"]["admissible"]
        assert cands[f"a / omega {choice['omega_max']:g}"]["passes"] == min(v["passes"] for v in admissible.values())
        ref = table["plain"][0]["reference_rule"]
        assert all(r <= table["energy_bound"][0] / max(ref["mean_v2"], 1e-30) + 1e-3
                   for v in admissible.values() for r in v["energy_ratio"])
        assert all(r <= table["height_bound"][0] / max(ref["y_p99"], 1e-30) + 1e-3
                   for v in admissible.values() for r in v["height_ratio"])
        chosen = evaluate(N.WARM_LEARNED | N.WARM_PROJECTED)
        assert chosen[1] == 30
    none, _ = select_warm_start(nets, [case], (2.0,), energy_slack=1e-9)
    assert none is None
