"""Throughput benchmark of the adaptive PBF substep on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

A "step" is one substep (pool::update, source/pool.cpp:67-106) of the workload's
scene.  `value` is whole-job particle-substeps/s with the state resident in HBM;
`e2e` is the same metric through the C ABI with the particle state coming from
and going back to pinned host buffers every step.  Multi-GPU runs are replicas:
every rank simulates its own copy of the scene (seeded by rank), no collective on
the data path ("scaling": "weak").

--impl reference times the CPU restatement of the reference's shader math (the
oracle, single-threaded C) on every host core at once, as independent replicas of
a bounded sample of the same scene.

Rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path
from types import SimpleNamespace

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-substeps/s at <=0.1% density error: learned warm-start vs plain"
UNIT = "particle-substeps/s"

WORKLOADS = {
    # name: (scene factory, description)
    # the 250 k water drop with split/merge and kernel widths spread across neighbours (the
    # spread_kernel_width path, pool.cpp:87-89, taken when the widths do not come from
    # the boundary distance); target radii from 1 at the surface to 2 at the pool's
    # floor (volume ratios 1x-8x): scale factor 1/40 per radius of boundary distance
    "water_drop_250k": ("water_drop", dict(total=250_000, basic_pbf=False, max_neighbors=2048,
                                           settings={"base_kernel_width_on_boundary_distance": 0,
                                                     "target_radius_scale_factor": 0.025})),
    "water_drop_250k_plain": ("water_drop", dict(total=250_000, basic_pbf=True)),
    "dam_break_32k": ("dam_break", dict(n_side=32)),
    # 384k particles pre-filled + 2000/substep from the emitter: ~1M after 300 substeps
    "waterfall_1m": ("waterfall", dict(initial=384_000, basic_pbf=False)),
    # 64 independent scenes, log-uniform 4k-200k particles, one graph launch per substep
    "batch64": ("batch", dict(scenes=64, lo=4_000, hi=200_000)),
}
DEFAULT_WORKLOAD = "waterfall_1m"


def make_spec(name: str, seed: int = 0, scale: float = 1.0):
    from apbf_gb300 import scenes

    factory, kw = WORKLOADS[name]
    kw = dict(kw)
    if "total" in kw:
        kw["total"] = int(kw["total"] * scale)
    if factory == "dam_break":  # a cube of n_side^3 particles: scale its side
        kw["n_side"] = max(4, int(round(kw["n_side"] * scale ** (1.0 / 3.0))))
        return scenes.dam_break(seed=seed, **kw)
    if factory == "waterfall":
        spec = scenes.waterfall(initial=int(kw["initial"] * scale), seed=seed, basic_pbf=kw["basic_pbf"],
                                scale=scale ** (1.0 / 3.0), per_substep=int(round(2000 * scale ** (2.0 / 3.0))))
        spec.meta["presteps"] = 300  # the emitter has brought the count to ~1M
        return spec
    basic = kw.pop("basic_pbf")
    settings = kw.pop("settings", None)
    maxn = kw.pop("max_neighbors", None)
    spec = scenes.water_drop(seed=seed, basic_pbf=basic, **kw)
    if settings:
        spec.meta["settings"] = dict(settings)
    if maxn:
        spec.meta["max_neighbors"] = maxn
    return spec


def settings_dict(spec) -> dict:
    """The oracle's settings for a workload: the reference's defaults (restated in the
    oracle, so this loads nothing of the product), iterated to the error target."""
    from oracle.oracle import DEFAULT_SETTINGS

    s = dict(DEFAULT_SETTINGS)
    s.update(spec.meta.get("settings", {}))
    s["basic_pbf"] = 1 if spec.basic_pbf else 0
    s["solver_iterations"] = 100
    s["density_error_target"] = 0.001
    return s


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- roofline
def algorithmic_bytes(kernel: str, n: int, pairs: int) -> float | None:
    """Compulsory HBM bytes of one launch (inputs read once, outputs written once,
    neighbour data counted once per particle, rows as 4 bytes per pair)."""
    if kernel == "k_density_lambda":
        return 28.0 * n + 4.0 * pairs  # 4N + 4P + 12N pos + 8N (invMass, kw) + 4N lambda
    if kernel == "k_delta":
        return 40.0 * n + 4.0 * pairs  # 4N + 4P + 12N + 4N lambda + 8N + 12N pos out
    if kernel == "k_build_rows":
        return 16.0 * n + 4.0 * n + 4.0 * pairs  # pos + range in, counts + rows out
    return None


def _l2_resident(n: float, pairs: int) -> bool:
    """Whether one Jacobi pass's working set (per particle: position and packed record,
    solve record, self shift, widths; rows at 4 bytes per pair) fits the GPU's L2, in
    which case an HBM roofline fraction says little about the kernel."""
    try:
        import torch

        l2 = torch.cuda.get_device_properties(torch.cuda.current_device()).L2_cache_size
    except (RuntimeError, AttributeError, AssertionError):
        l2 = 126 * 1024 * 1024
    return bool(80.0 * n + 8.0 * pairs < l2)


def measured_peak() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(kernel: str, n: int, pairs: int) -> float | None:
    """DRAM bytes per launch from the committed ncu summary (scaled to this launch's size)."""
    p = ROOT / "profiles" / "ncu_traffic.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        f = [x.strip() for x in line.strip().strip("|").split("|")]
        if len(f) >= 5 and f[0] == kernel:
            try:
                bytes_, n0, p0 = float(f[1]), float(f[2]), float(f[3])
            except ValueError:
                continue
            a0 = algorithmic_bytes(kernel, int(n0), int(p0))
            a1 = algorithmic_bytes(kernel, n, pairs)
            return bytes_ * (a1 / a0) if a0 and a1 else None
    return None


# ----------------------------------------------------------------------------- CPU baseline
def oracle_boxes(spec) -> tuple:
    """The scene's boxes for the oracle: axis-aligned ones plus the oriented ones with
    their rotation rows computed as apbf_set_oriented_boxes computes them."""
    if spec.meta.get("oriented_boxes") is None:
        return (spec.box_min, spec.box_max)
    c, h, q = spec.meta["oriented_boxes"]
    rot = np.zeros((len(spec.box_min) + len(c), 3, 4), np.float32)
    for k, qq in enumerate(np.asarray(q, np.float64)):
        x, y, z, w = qq / np.linalg.norm(qq)
        m = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)],
                      [2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)],
                      [2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)]])
        rot[len(spec.box_min) + k, :, :3] = m.astype(np.float32)
        rot[len(spec.box_min) + k, 0, 3] = 1.0
    return (np.concatenate([spec.box_min, c]), np.concatenate([spec.box_max, h]), rot)


def cpu_sample(workload: str, budget_s: float = 15.0) -> dict:
    """The single-threaded oracle on a bounded sample: the same scene at 1/8 of the
    particle count (every length halved), substeps until the budget is spent.  The
    oracle library is the FP64 oracle, or its FP32 build when the process was
    started with APBF_ORACLE_VARIANT=f32."""
    from oracle import oracle as orc

    spec = make_spec(workload, scale=1.0 / 8.0)
    cap = max(spec.n, int(spec.meta.get("capacity", 0) // 8)) + 4096
    fs = orc.FluidState(spec.state, cap=cap)
    sc = orc.make_scene(orc.settings_from(settings_dict(spec)), spec.grid_min, spec.grid_max, spec.log2res,
                        spec.acceleration)
    boxes = oracle_boxes(spec)
    est = np.zeros(2, np.float64)
    em = spec.meta.get("emitter")
    steps, processed, t0 = 0, 0, time.perf_counter()
    while True:
        if em:
            orc.emit(fs, SimpleNamespace(**em, max_particles=0, enabled=1), est, np.float32(spec.dt),
                     np.float32(sc.last_dt))
        orc.substep(fs, sc, boxes, np.float32(spec.dt), int(cap * 64))
        steps += 1
        processed += fs.n
        if time.perf_counter() - t0 > budget_s or steps >= 20:
            break
    el = time.perf_counter() - t0
    return {"value": processed / el, "steps": steps, "particles": int(spec.n), "seconds": round(el, 1),
            "library": orc.LIB.name}


def cpu_baseline(workload: str, budget_s: float = 15.0) -> dict:
    """The oracle timed on this host: the FP64 oracle in this process, then the FP32
    build of the same code in a child process (same sample, same single thread)."""
    r64 = cpu_sample(workload, budget_s)
    env = dict(os.environ, APBF_ORACLE_VARIANT="f32")
    code = (f"import sys, json; sys.path.insert(0, {str(ROOT)!r}); import bench; "
            f"print(json.dumps(bench.cpu_sample({workload!r}, {budget_s!r})))")
    fp32 = None
    try:
        out = subprocess.run([sys.executable, "-c", code], env=env, cwd=str(ROOT), capture_output=True, text=True,
                             timeout=budget_s * 10 + 120, check=True)
        r32 = json.loads(out.stdout.strip().splitlines()[-1])
        fp32 = {"value": r32["value"], "unit": UNIT, "cores": 1, "library": r32["library"],
                "sample": f"the same sample, {r32['steps']} substep(s), {r32['seconds']} s"}
    except (subprocess.SubprocessError, ValueError, IndexError) as e:
        fp32 = {"unavailable": f"{type(e).__name__}: {str(e)[:200]}"}
    s = settings_dict(make_spec(workload, scale=1.0 / 8.0))
    return {"value": r64["value"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{r64['steps']} substep(s) from the start of the {r64['particles']}-particle (1/8 scale) "
                      f"version of the scene, reference Jacobi rule until {s['density_error_target']} "
                      f"(max {s['solver_iterations']} passes), single-threaded FP64 oracle, {r64['seconds']} s",
            "fp32": fp32}


def _product_library_mapped() -> bool:
    """Whether this process has mapped the library under test (Linux /proc)."""
    try:
        with open("/proc/self/maps") as f:
            return any("libapbf_gb300" in line for line in f)
    except OSError:
        return False


def _replica_loop(conn, name, scale, seed, presteps):
    """One replica of the reference arm: builds its scene, brings it to the phase the
    GPU arm times (the scene's untimed substeps, with the scene's fixed iteration
    count, the reference's own way of running: settings.cpp:31, pool.cpp:91-95), then
    advances it by the requested number of substeps per command (iterating to the
    error target like the timed GPU arms) and answers with its particle count.  An
    emitter adds particles every substep, as on the GPU."""
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as orc

    spec = make_spec(name, seed=seed, scale=scale)
    cap = max(spec.n, int(spec.meta.get("capacity", 0) * scale)) + 4096
    fs = orc.FluidState(spec.state, cap=cap)
    sc = orc.make_scene(orc.settings_from(settings_dict(spec)), spec.grid_min, spec.grid_max, spec.log2res,
                        spec.acceleration)
    boxes = oracle_boxes(spec)
    em = spec.meta.get("emitter")
    est = np.zeros(2, np.float64)

    def advance():
        if em:
            orc.emit(fs, SimpleNamespace(**em, max_particles=0, enabled=1), est, np.float32(spec.dt),
                     np.float32(sc.last_dt))
        orc.substep(fs, sc, boxes, np.float32(spec.dt), int(cap * 64))

    target, iters = sc.settings.density_error_target, sc.settings.solver_iterations
    sc.settings.density_error_target, sc.settings.solver_iterations = 0.0, spec.iterations
    for _ in range(presteps):
        advance()
    sc.settings.density_error_target, sc.settings.solver_iterations = target, iters
    conn.send((int(fs.n), orc.LIB.name, _product_library_mapped()))
    while True:
        k = conn.recv()
        if k is None:
            break
        for _ in range(k):
            advance()
        conn.send(int(fs.n))
    conn.close()


def run_reference(args) -> None:
    """The reference arm: the CPU restatement of the reference's shader math (the
    reference has no CPU path of its own and cannot be built here) on every host core,
    as independent replicas of a bounded sample of the scene (1/8 of its particles).
    By default the replicas run the oracle's FP32 build (the reference's shaders
    compute in FP32, and it is the faster CPU form); --oracle-variant f64 runs the
    FP64 oracle.  Each replica builds its scene once; a step is one substep of every
    replica, timed from the command to the last answer."""
    import multiprocessing as mp

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    full = make_spec(args.workload, scale=1.0)
    # a sample whose timed substep takes a few seconds per core: 1/8 of the water drops,
    # 1/256 of the waterfall (whose reference rule runs its 100-pass cap every substep)
    scale = 1.0 / 8.0 if full.n <= 300_000 else 1.0 / 256.0
    presteps = args.presteps if args.presteps >= 0 else full.meta.get("presteps", 0)
    ctx = mp.get_context("spawn")
    pipes, procs = [], []
    saved = os.environ.get("APBF_ORACLE_VARIANT")
    os.environ["APBF_ORACLE_VARIANT"] = args.oracle_variant  # inherited by the spawned replicas
    try:
        for s in range(cores):
            a, b = ctx.Pipe()
            p = ctx.Process(target=_replica_loop, args=(b, args.workload, scale, s, presteps), daemon=True)
            p.start()
            pipes.append(a)
            procs.append(p)
    finally:
        if saved is None:
            os.environ.pop("APBF_ORACLE_VARIANT", None)
        else:
            os.environ["APBF_ORACLE_VARIANT"] = saved
    built = [c.recv() for c in pipes]  # (particles, oracle library) once the scenes are built
    counts = [b[0] for b in built]
    libraries = sorted({b[1] for b in built})
    product_mapped = _product_library_mapped() or any(b[2] for b in built)

    def step():
        for c in pipes:
            c.send(1)
        return sum(c.recv() for c in pipes)

    for _ in range(args.warmup):
        step()
    processed = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        processed += step()
    wall = time.perf_counter() - t0
    for c in pipes:
        c.send(None)
    for p in procs:
        p.join(timeout=10)
    value = processed / wall
    n_sample = counts[0]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.oracle_variant == "f32" else "f64",
        "data": "synthetic (seeded scene generator)",
        "config": {"workload": args.workload, "sample_particles": n_sample, "sample_scale": scale,
                   "replicas": cores, "presteps": presteps, "oracle_build": args.oracle_variant,
                   "oracle_library": libraries, "product_library_mapped": product_mapped,
                   "iterations": "until mean density error <= 0.001 (max 100), reference Jacobi rule"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} independent replicas of the {scale:g}-scale version of the scene "
                                   f"({n_sample} particles at the start of the timed steps), each built once and "
                                   f"brought through the GPU arm's {presteps} untimed substeps, one substep of every "
                                   f"replica per step (the reference has no CPU implementation and cannot be built "
                                   f"here; the "
                                   f"oracle restates its shader math, here its "
                                   f"{'FP32 build' if args.oracle_variant == 'f32' else 'FP64 oracle'})"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- ours
def _make_ctx(spec, args, local, mode: int = 0, net=None):
    from apbf_gb300.api import Context

    cap = max(int(spec.n * 1.25) + 1024, int(spec.meta.get("capacity", 0) * 1.15))
    maxn = args.max_neighbors if spec.basic_pbf else max(args.max_neighbors, 256)
    maxn = max(maxn, spec.meta.get("max_neighbors", 0))
    # the search tuner may try grids up to search_levels finer than the scene's
    levels = min(9, max(spec.log2res, 3) + max(0, getattr(args, "search_levels", 0)))
    ctx = Context(particle_capacity=cap, max_neighbors=maxn, max_log2res=levels, device=local)
    # iterate every substep until the mean density error is at most the target
    ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=args.max_iterations,
                     density_error_target=args.error_target, **spec.meta.get("settings", {}))
    ctx.load_scene(spec)
    ctx.set_solve_graph(args.graph_mode)
    if getattr(args, "persistent", False):
        ctx.set_persistent_solve(True)
    if net is not None:
        ctx.mlp_load(net.params if hasattr(net, "params") else net)
    if mode:
        ctx.set_warm_start(mode)
    return ctx


VALIDATION_SUBSTEPS = 40  # counted substeps of each validation scene per warm-start candidate


def _ws_choices(args) -> tuple[tuple, tuple]:
    """Loss weights of the networks to train and over-relaxation bounds to compare
    (one of each when given on the command line)."""
    from apbf_gb300.warmstart import OMEGA_CANDIDATES

    ows = (args.ws_over_weight,) if args.ws_over_weight is not None else (4.0, 8.0, 16.0)
    oms = (args.ws_omega,) if args.ws_omega is not None else OMEGA_CANDIDATES
    return ows, oms


def _fit_nets(X, T, args, local: int, over_weights) -> dict:
    from apbf_gb300.warmstart import WarmStartNet

    nets = {}
    for ow in over_weights:
        net = WarmStartNet(device=local, seed=0)
        net.set_normalization(X, T)
        hist = net.fit(X, T, epochs=args.ws_epochs, batch=32768, lr=2e-3, lr_final=2e-4, over_weight=ow)
        nets[f"over_weight {ow:g}"] = (net, hist)
    return nets


def _selection_info(choice, table, seeds, args) -> dict:
    return {
        "chosen": ({k: v for k, v in choice.items() if k != "params"} if choice else
                   "none within the kinetic-energy bound: the reference Jacobi rule runs"),
        "selection": (None if table is None else
                      {"validation_seeds": seeds, "counted_substeps": VALIDATION_SUBSTEPS,
                       "energy_slack": args.ws_energy_slack, "height_slack": args.ws_height_slack,
                       "rule": "fewest passes among candidates that converge in every counted substep and end "
                               "with mean |v|^2 and the 99th-percentile height within the slacks x the largest "
                               "of the converging plain rules",
                       "plain": table["plain"], "candidates": table["candidates"]})}


# The warm start's training mixture: rollouts of the dam break (32 k), the adaptive
# water drop with spread kernel widths (250 k) and the adaptive waterfall (to ~1 M),
# two seeds each, that neither a timed scene (seed = rank), a validation scene
# (1000 + ...) nor an evaluation scene of the per-workload report (3000 + ...) uses.
MIXTURE = ("dam_break_32k", "water_drop_250k", "waterfall_1m")
MIXTURE_SAMPLES = 60_000_000  # about the same share from each rollout


def training_rollouts(rank: int) -> list[tuple]:
    """(workload, seed, substeps, every, particles at the end) of the mixture's
    rollouts: each runs from the scene's start through its untimed presteps plus 60
    substeps (the timed window and more; a scene timed from its start runs its own
    length) and records every `every`-th substep, so that each contributes about
    MIXTURE_SAMPLES / 6 samples (a growing scene counted at its mean size)."""
    per = MIXTURE_SAMPLES / (2 * len(MIXTURE))
    out = []
    for w in MIXTURE:
        for k in (0, 1):
            seed = 2000 + 10 * rank + k
            sp = make_spec(w, seed=seed)
            pre = sp.meta.get("presteps", 0)
            steps = pre + 60 if pre else sp.substeps
            n_end = sp.n + sp.meta.get("per_substep", 0) * steps
            every = max(1, int(round(steps * 0.5 * (sp.n + n_end) / per)))
            out.append((w, seed, steps, every, n_end))
    return out


def train_mixture(args, local: int, rank: int) -> tuple[dict, dict]:
    """Untimed: samples from projected-rule rollouts of the mixture (the plain solve;
    the target is the lambda sum a substep's passes apply), then minibatch Adam with
    the project's kernels, one network per overshoot weight of the loss."""
    import torch

    from apbf_gb300 import _native as N
    from apbf_gb300.warmstart import SampleBuffer, record_rollout

    t0 = time.perf_counter()
    plan = training_rollouts(rank)
    cap = int(sum(max(n_end, make_spec(w).n) * (steps // every + 1) for w, _, steps, every, n_end in plan) * 1.1)
    buf = SampleBuffer.allocate(min(cap, 160_000_000), device=local)
    counts = []
    for w, seed, steps, every, _ in plan:
        sp = make_spec(w, seed=seed)
        ctx = _make_ctx(sp, args, local, N.WARM_PROJECTED)
        before = buf.size()
        record_rollout(ctx, sp.dt, steps, buf, iterations=args.max_iterations, every=every)
        try:
            ctx.check_status()
        except Exception as e:
            raise RuntimeError(f"training rollout {w} seed {seed}: {e}") from e
        ctx.close()
        print(f"rollout {w} seed {seed}: {buf.size() - before} samples", file=sys.stderr, flush=True)
        counts.append({"workload": w, "seed": seed, "substeps": steps, "every": every,
                       "samples": buf.size() - before})
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    X, T = buf.view()
    n_samples = int(X.shape[0])
    ows, _ = _ws_choices(args)
    trained = _fit_nets(X, T, args, local, ows)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    del buf, X, T
    torch.cuda.empty_cache()
    info = {"samples": n_samples, "rollouts": counts,
            "target": "sum of the lambdas applied over all passes of a projected-rule substep",
            "epochs": args.ws_epochs,
            "loss_per_epoch": {k: [round(h, 5) for h in v[1]] for k, v in trained.items()},
            "collect_s": round(t1 - t0, 3), "train_s": round(t2 - t1, 3)}
    return {k: v[0] for k, v in trained.items()}, info


def select_for_workload(nets: dict, args, local: int, rank: int, workload: str) -> tuple:
    """Chooses the network and over-relaxation bound for `workload` on one or two of
    its seeds that training and the timed scene do not use (fewest passes within the
    plain solve's kinetic energy).  Returns (net or None, selection info)."""
    from apbf_gb300.warmstart import ValidationCase, select_warm_start

    t0 = time.perf_counter()
    _, oms = _ws_choices(args)
    nmin = args.ws_min_neighbors if args.ws_min_neighbors is not None else 16.0
    # seeds of the validation: a candidate must stay within the slacks on every one, so
    # more seeds keep a candidate at the edge of a slack from passing by chance (with
    # two seeds, the water drop admitted splashes of 1.2x that reached 1.34-1.51x on
    # other seeds)
    large = make_spec(workload).n >= 500_000 or workload.startswith("waterfall")
    vseeds = [1000 + 10 * rank + k for k in ((3, 4) if large else (3, 4, 5, 6))]
    table = None
    if len(nets) * len(oms) > 1:
        cases = []
        for vs in vseeds:
            vspec = make_spec(workload, seed=vs)
            before = (args.presteps if args.presteps >= 0 else vspec.meta.get("presteps", 0)) + args.warmup
            cases.append(ValidationCase(
                make=lambda mode, params, vspec=vspec: _make_ctx(vspec, args, local, mode, params),
                dt=vspec.dt, before=before, counted=VALIDATION_SUBSTEPS))
        choice, table = select_warm_start(nets, cases, oms, nmin, args.ws_energy_slack, args.ws_height_slack)
    else:
        key = next(iter(nets))
        nets[key].omega_max, nets[key].min_neighbors = oms[0], nmin
        choice = {"net": key, "omega_max": oms[0], "min_neighbors": nmin}
    info = {"select_s": round(time.perf_counter() - t0, 3), **_selection_info(choice, table, vseeds, args)}
    return (nets[choice["net"]] if choice else None), info


def train_warm_start(args, local: int, rank: int) -> tuple[object, dict]:
    """Untimed: one network set trained on the mixture, then the network and bound for
    the timed workload chosen on seeds of it that neither training nor the timed scene
    uses.  Returns (None, info) when no candidate passes: the headline then runs the
    reference Jacobi rule."""
    nets, info = train_mixture(args, local, rank)
    net, sel = select_for_workload(nets, args, local, rank, args.workload)
    return net, {**info, **sel}


def _state_summary(ctx) -> dict:
    g, _ = ctx.download()
    v = g["velocity"][:, :3].astype(np.float64)
    y = g["position"][:, 1].astype(np.float64) / 262144.0
    red = ctx.reduce_fp64()
    return {"mean_v2": round(float(np.mean(np.sum(v * v, axis=1))), 1), "y_p99": round(float(np.percentile(y, 99)), 1),
            "mean_abs_density_error": round(float(red[3]), 4), "last_density_error": float(red[2])}


def run_arm(spec, args, local, mode: int, net, dist, headline: bool) -> tuple[dict, object]:
    """Presteps and warm-up untimed, then `steps` substeps timed with CUDA events on
    the launching stream, L2 flushed (256 MB write) before each."""
    import torch

    ctx = _make_ctx(spec, args, local, mode, net)
    stream = torch.cuda.current_stream()
    presteps = args.presteps if args.presteps >= 0 else spec.meta.get("presteps", 0)
    for _ in range(presteps):  # untimed: bring the scene into its violent regime (after impact)
        ctx.substep(spec.dt)
    if not args.no_autotune:  # untimed, state restored
        search_tuning = ctx.autotune_search() if spec.meta.get("glue") is None else None
        tuning = ctx.autotune()
        tuning["search"] = search_tuning
    else:
        tuning = ctx.tuning()
    for _ in range(args.warmup):
        ctx.substep(spec.dt)
    ctx.check_status()
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    window = _window_snapshot(ctx) if headline else None  # the e2e run replays this window
    n_start, _ = ctx.lengths()
    ctx.check_status()  # clears the pass and convergence counters
    launches0 = ctx.launch_count()
    clocks = ClockSampler(local) if headline else None
    if clocks:
        clocks.start()
        time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if headline:
        torch.cuda.nvtx.range_push("timed")  # lets ncu select the timed substeps (--nvtx-include timed/)
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        ctx.substep(spec.dt)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if headline:
        torch.cuda.nvtx.range_pop()
    if dist:
        dist.barrier()
    clk = clocks.stop() if clocks else None
    launches = ctx.launch_count() - launches0
    total_ms = float(np.sum([a.elapsed_time(b) for a, b in ev]))
    info = ctx.check_status()
    n_end, _ = ctx.lengths()
    # the end state of the timed window, before the traced substeps below: every arm
    # (headline and plain) is compared at the same substep
    state_after = _state_summary(ctx)
    prof, dropped = {}, 0
    if headline and args.prof_steps > 0:
        # per-kernel CUDA events on a few more substeps with the same pass count and
        # no early stop (every launch a full pass), for the kernel shares and the
        # roofline of the dominant kernel; tracing uses one launch pair per pass
        passes = max(2, int(round(info.density_passes / args.steps)))
        ctx.set_settings(solver_iterations=passes, density_error_target=0.0)
        ctx.profile_enable(True, 65536)
        ctx.profile_read()
        for _ in range(args.prof_steps):
            flush.zero_()
            # a few ms of GPU time first: the host enqueues the substep's launches (each
            # with its two events) ahead of the GPU, so the events time the kernels and
            # not the gaps between host launches
            if hasattr(torch.cuda, "_sleep"):
                torch.cuda._sleep(6_000_000)
            ctx.substep(spec.dt)
        prof, dropped = ctx.profile_read()
        ctx.profile_enable(False, 0)
        ctx.set_settings(solver_iterations=args.max_iterations, density_error_target=args.error_target)
        ctx.check_status()
    n_mean = 0.5 * (n_start + n_end)  # particles per timed substep (an emitter adds some every substep)
    r = {"ms_per_step": total_ms / args.steps, "value": n_mean * args.steps / (total_ms / 1000.0),
         "particles_before": int(n_start), "particles_mean": n_mean,
         "density_passes_per_substep": info.density_passes / args.steps,
         "converged_substeps": f"{info.converged_substeps}/{args.steps}", "pairs": int(info.pairs),
         "particles_after": int(n_end), "presteps": presteps, "total_ms": total_ms, "gpu_launches": int(launches),
         "tuning": tuning,
         "state_after": state_after}
    if headline:
        r["_prof"], r["_dropped"], r["_clocks"], r["_window"] = prof, dropped, clk, window
    return r, ctx


def run_warm_start_report(args) -> None:
    """Passes saved per workload by one network set trained on the mixture.  For each
    workload of the mixture: the network and bound chosen on its validation seeds,
    then the reference rule, the projected rule and the learned form run on an
    evaluation seed (3000) that neither training nor validation uses, each timed like
    the headline (presteps and warm-up untimed, `steps` substeps with CUDA events, L2
    flushed): passes per substep and particle-substeps/s at the same error target.
    Prints one JSON line."""
    import torch

    from apbf_gb300 import _native as N

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    nets, info = train_mixture(args, local, 0)
    keep = ("value", "ms_per_step", "density_passes_per_substep", "converged_substeps", "particles_mean",
            "presteps", "state_after")
    per = {}
    for w in MIXTURE:
        net, sel = select_for_workload(nets, args, local, 0, w)
        spec = make_spec(w, seed=3000)
        arms = {}
        forms = [("reference_rule", 0, None), ("projected_rule", N.WARM_PROJECTED, None)]
        if net is not None:
            forms.append(("learned", N.WARM_LEARNED | N.WARM_PROJECTED, net))
        for name, mode, nn in forms:
            r, c = run_arm(spec, args, local, mode, nn, None, headline=False)
            c.close()
            arms[name] = {k: r[k] for k in keep}
        row = {"chosen": sel["chosen"], "select_s": sel["select_s"], "selection": sel["selection"], "arms": arms}
        if net is not None:
            lp = arms["learned"]["density_passes_per_substep"]
            for k in ("reference_rule", "projected_rule"):
                row[f"passes_saved_vs_{k}"] = round(arms[k]["density_passes_per_substep"] - lp, 2)
                row[f"rate_over_{k}"] = round(arms["learned"]["value"] / max(arms[k]["value"], 1e-30), 3)
        per[w] = row
        print(json.dumps({"workload": w, **{k: v for k, v in row.items() if k != "selection"}}), flush=True)
    print(json.dumps({"report": "warm start trained on the mixture, per workload", "metric": METRIC, "unit": UNIT,
                      "error_target": args.error_target, "max_iterations": args.max_iterations,
                      "evaluation_seed": 3000, "steps": args.steps, "warmup": args.warmup,
                      "training": info, "per_workload": per}), flush=True)


def _device_pairs(ctx, n: int) -> np.ndarray:
    """The device's neighbour rows as sorted (i << 32 | j) keys, one per directed pair."""
    nb = ctx.neighbors_view()
    cnt = nb["count"][:n].cpu().numpy().view(np.uint32).astype(np.int64)
    m = int(cnt.max()) if n else 0
    idx = nb["index"][:m, :n].cpu().numpy().view(np.uint32).astype(np.int64)
    live = np.arange(m)[:, None] < cnt[None, :]
    ii = np.broadcast_to(np.arange(n, dtype=np.int64)[None, :], (m, n))[live]
    return np.sort((ii << 32) | idx[live])


def oracle_check(ctx, spec) -> dict:
    """Parity of the final state of the timed run against the FP64 oracle: the state is
    downloaded and searched by the device and by the oracle with the substep's own
    range scale (1 for basic PBF or kernel widths from the boundary distance, else 1.5:
    source/pool.cpp:83) on the scene grid.  Reported: Morton keys and sort permutation
    bit for bit, neighbour sets (every directed pair) bit for bit, and the mean
    compression error of one density pass over those rows, FP32 on the device against
    FP64 in the oracle."""
    from apbf_gb300.api import incompressibility, neighborhood_green
    from oracle import oracle as orc

    s = ctx.settings
    scale = 1.0 if (s.basic_pbf or s.base_kernel_width_on_boundary_distance) else 1.5
    st, _ = ctx.download()
    n = int(st["position"].shape[0])
    t0 = time.perf_counter()
    neighborhood_green().set_data(ctx).set_range_scale(scale).set_position_range(
        spec.grid_min, spec.grid_max, spec.log2res).apply()
    perm_d, keys_d = ctx.debug_sort()
    pairs_d = _device_pairs(ctx, n)
    incompressibility().set_data(ctx).apply()
    e_dev = float(ctx.reduce_fp64()[2])
    t1 = time.perf_counter()
    fs = orc.FluidState(st)
    perm_o, keys_o, tot = orc.neighborhood_green(fs, scale, spec.grid_min, spec.grid_max, spec.log2res,
                                                 max(n * 160, 1024))
    off = fs.nb_off[:n + 1].astype(np.int64)
    pairs_o = (np.repeat(np.arange(n, dtype=np.int64), np.diff(off)) << 32) | fs.nb_idx[:tot].astype(np.int64)
    e_or = float(orc.density_error(fs, orc.settings_from(s))[0])
    same_sets = pairs_d.shape == pairs_o.shape and bool(np.array_equal(pairs_d, np.sort(pairs_o)))
    return {"particles": n, "range_scale": scale, "grid_log2res": spec.log2res,
            "morton_keys_bit_exact": bool(np.array_equal(keys_d, keys_o)),
            "sort_permutation_bit_exact": bool(np.array_equal(perm_d, perm_o)),
            "neighbor_sets_equal": same_sets, "pairs_device": int(pairs_d.size), "pairs_oracle": int(tot),
            "density_error_device_fp32": e_dev, "density_error_oracle_fp64": e_or, "abs_diff": abs(e_dev - e_or),
            "device_s": round(t1 - t0, 2), "oracle_s": round(time.perf_counter() - t1, 2),
            "what": "the final state searched again by both (keys, permutation, every directed pair) and one density "
                    "pass over those new rows (mean compression error; rows rebuilt after the solve's last pass, so "
                    "this is not the solve's own error, which config.density_error_last_pass reports)"}


def reduce_over_ranks(total_ms: float, processed: float, dist, device) -> tuple[float, float]:
    """Whole-job figures of independent replicas: the slowest rank's timed milliseconds
    and the particle-substeps of all ranks (no collective on the data path; these two
    numbers are the only exchange).  dist=None: one process, unchanged."""
    import torch

    if dist is None:
        return total_ms, processed
    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    p = torch.tensor([processed], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(t[0]), float(p[0])


def run_ours(args) -> None:
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    from apbf_gb300 import _native as N

    spec = make_spec(args.workload, seed=rank)
    n = spec.n
    wants_learned = not args.no_warm_start and args.solve == "learned"
    net, train_info = train_warm_start(args, local, rank) if wants_learned else (None, None)
    learned = net is not None  # no admissible warm start: the reference rule is the headline
    head_mode = (N.WARM_LEARNED | N.WARM_PROJECTED) if learned else 0
    if args.solve == "projected":
        head_mode = N.WARM_PROJECTED

    # the plain forms first (same scene, same seed), then the headline form
    plain = {}
    if wants_learned and not args.no_plain:
        for name, mode in (("reference_rule", 0), ("projected_rule", N.WARM_PROJECTED)):
            r, c = run_arm(spec, args, local, mode, None, dist, headline=False)
            c.close()
            plain[name] = {k: v for k, v in r.items() if not k.startswith("_")}
    head, ctx = run_arm(spec, args, local, head_mode, net, dist, headline=True)
    total_ms = head["total_ms"]
    n = head["particles_mean"]  # particles per timed substep
    particles_processed = n * args.steps
    total_ms, particles_processed = reduce_over_ranks(total_ms, particles_processed, dist, f"cuda:{local}")
    value = particles_processed / (total_ms / 1000.0)

    # roofline of the dominant kernel (largest share of the timed kernel time)
    prof = head.pop("_prof")
    dropped = head.pop("_dropped")
    clk = head.pop("_clocks")
    window = head.pop("_window")
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else None
    roof = None
    if dom:
        name, (cnt, ms) = dom
        per_launch_s = ms / cnt / 1000.0
        n_prof = head["particles_after"]  # the traced substeps follow the timed ones
        alg = algorithmic_bytes(name, n_prof, head["pairs"])
        peak, peak_kind = measured_peak()
        if alg:
            ach = alg / per_launch_s / 1e9
            roof = {"kernel": name, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                    "frac": ach / peak, "peak_source": peak_kind,
                    "traffic": traffic_from_profiles(name, n_prof, head["pairs"]),
                    "algorithmic_bytes": alg, "launch_us": per_launch_s * 1e6}
    kernel_share = {k: round(v[1] / max(sum(x[1] for x in prof.values()), 1e-9), 4) for k, v in prof.items()}
    kernel_us = {k: round(v[1] / max(v[0], 1) * 1000.0, 2) for k, v in prof.items()}  # mean per launch

    # e2e: the same substep driven from pinned host buffers through the C ABI
    e2e = run_e2e(ctx, spec, args, window)
    check = oracle_check(ctx, spec) if rank == 0 and not args.no_oracle_check else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload)

    if rank == 0:
        solver = ("learned warm start (BF16 MLP first update) + projected Jacobi passes" if learned
                  else "projected Jacobi rule (no network)" if args.solve == "projected"
                  else "reference Jacobi rule" + (" (no warm start within the kinetic-energy bound)"
                                                  if wants_learned else ""))
        # the plain forms of the same scene, seed and timed window, for the learned-vs-plain comparison
        vs_plain = {k: {"value": v["value"], "ms_per_step": round(v["ms_per_step"], 4),
                        "density_passes_per_substep": v["density_passes_per_substep"],
                        "converged_substeps": v["converged_substeps"],
                        "headline_over_this": round(value / v["value"], 3) if v["value"] else None}
                    for k, v in plain.items()} if plain else None
        parity = None
        if check:
            parity = {k: check[k] for k in ("morton_keys_bit_exact", "sort_permutation_bit_exact",
                                             "neighbor_sets_equal", "density_error_device_fp32",
                                             "density_error_oracle_fp64", "what")}
        fidelity = None
        if plain and head.get("state_after"):
            e = head["state_after"]["mean_v2"]
            hy = head["state_after"]["y_p99"]
            fidelity = {}
            for k, v in plain.items():
                if v.get("state_after"):
                    fidelity[f"mean_v2_vs_{k}"] = round(e / max(v["state_after"]["mean_v2"], 1e-30), 3)
                    fidelity[f"y_p99_vs_{k}"] = round(hy / max(v["state_after"]["y_p99"], 1e-30), 3)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (int32 fixed-point positions and sums; bf16 MLP)",
            "data": "synthetic (seeded scene generator)",
            "config": {"workload": args.workload, "particles": n, "particles_before": head["particles_before"],
                       "particles_after": head["particles_after"],
                       "solver": solver,
                       "iterations": f"until mean density error <= {args.error_target} (max {args.max_iterations})",
                       "density_passes_per_substep": head["density_passes_per_substep"],
                       "converged_substeps": head["converged_substeps"], "presteps": head["presteps"],
                       "dt": spec.dt, "adaptive": not spec.basic_pbf, "pairs": head["pairs"],
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{world}",
                       "graph_mode": args.graph_mode, "persistent_solve": bool(args.persistent),
                       "density_error_last_pass": head["state_after"]["last_density_error"],
                       "vs_plain": vs_plain, "parity_vs_fp64_oracle": parity,
                       "l2_resident": _l2_resident(n, head["pairs"]),
                       "tuning": head["tuning"]},
            "state_after": head["state_after"], "fidelity": fidelity,
            "plain": plain or None,
            "warm_start_training": train_info,
            "roofline": roof, "kernel_share": kernel_share, "kernel_us": kernel_us,
            "gpu_launches": head["gpu_launches"],
            "profiler_dropped": int(dropped), "clocks": clk, "e2e": e2e, "cpu_baseline": cpu,
            "oracle_check": check,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def batch_whole_job(seq_ms: float, seq_particles: float, e2e_s: float, e2e_particles: float, scenes: int,
                    particles: int, dist, device) -> dict:
    """Whole-job figures of the batch's comparison runs on N ranks, as for the headline:
    the slowest rank's time and the particle-substeps and scenes of all ranks."""
    seq_ms, seq_particles = reduce_over_ranks(seq_ms, seq_particles, dist, device)
    e2e_s, e2e_particles = reduce_over_ranks(e2e_s, e2e_particles, dist, device)
    _, scenes = reduce_over_ranks(0.0, float(scenes), dist, device)
    _, particles = reduce_over_ranks(0.0, float(particles), dist, device)
    return {"sequential_ms": seq_ms, "sequential_value": seq_particles / (seq_ms / 1000.0),
            "e2e_value": e2e_particles / e2e_s, "scenes": int(scenes), "particles_total": int(particles)}


# ----------------------------------------------------------------------------- batch
def batch_specs(n_scenes: int, lo: int, hi: int, seed: int = 7) -> list:
    """Seeded scene table: particle counts log-uniform in [lo, hi]; every other scene a
    dam break (single kernel width), the rest water drops, half of them adaptive."""
    from apbf_gb300 import scenes

    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_scenes)).astype(int)
    out = []
    for k, c in enumerate(counts):
        if k % 2 == 0:
            out.append(scenes.dam_break(n_side=max(8, int(round(c ** (1.0 / 3.0)))), seed=k))
        else:
            out.append(scenes.water_drop(total=int(c), seed=k, basic_pbf=(k % 4 == 1)))
    return out


def run_batch(args) -> None:
    """Batch throughput: many independent scenes of uneven sizes advanced by
    one graph launch per substep (their substeps are the graph's parallel branches),
    against the same scenes advanced one after the other."""
    import torch

    from apbf_gb300 import _native as N
    from apbf_gb300.api import Batch, Context
    from apbf_gb300.warmstart import SampleBuffer, ValidationCase, record_rollout, select_warm_start

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:  # replicas: every rank its own table of scenes
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    _, kw = WORKLOADS[args.workload]
    specs = batch_specs(kw["scenes"], kw["lo"], kw["hi"], seed=7 + rank)
    dt = 1.0 / 240.0  # one time step for the whole batch

    def make(spec, mode=0, net=None):
        maxn = 160 if spec.basic_pbf and spec.name == "dam_break" else (192 if spec.basic_pbf else 256)
        ctx = Context(particle_capacity=int(spec.n * 1.3) + 1024, max_neighbors=maxn,
                      max_log2res=max(spec.log2res, 3), device=local)
        ctx.set_settings(basic_pbf=1 if spec.basic_pbf else 0, solver_iterations=args.max_iterations,
                         density_error_target=args.error_target)
        ctx.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
        ctx.set_boxes(spec.box_min, spec.box_max)
        ctx.upload(spec.state)
        ctx.set_solve_graph(2)
        if net is not None:
            ctx.mlp_load(net if isinstance(net, torch.Tensor) else net.params)
        if mode:
            ctx.set_warm_start(mode)
        return ctx

    # warm start: one network for the mixture, trained on projected-rule rollouts of
    # small scenes of each kind with seeds the batch does not use
    t0 = time.perf_counter()
    from apbf_gb300 import scenes as S

    train = [S.dam_break(n_side=24, seed=901), S.water_drop(total=40_000, seed=902, basic_pbf=True),
             S.water_drop(total=40_000, seed=903, basic_pbf=False)]
    buf = SampleBuffer.allocate(12_000_000, device=local)
    for sp in train:
        c = make(sp, N.WARM_PROJECTED)
        record_rollout(c, dt, 120, buf, iterations=args.max_iterations, every=2)
        c.check_status()
        c.close()
    X, T = buf.view()
    n_samples = int(X.shape[0])
    ows, oms = _ws_choices(args)
    nets = {k: v[0] for k, v in _fit_nets(X, T, args, local, ows).items()}
    del buf, X, T
    torch.cuda.empty_cache()
    nmin = args.ws_min_neighbors if args.ws_min_neighbors is not None else 16.0

    # one set of networks for the mixture; the network and bound per scene kind (each
    # context loads its own parameter vector), chosen on a held-out scene of the kind
    def kind(sp):
        return f"{sp.name}{'' if sp.basic_pbf else ' adaptive'}"

    val = [(911, S.dam_break(n_side=24, seed=911)), (912, S.water_drop(total=40_000, seed=912, basic_pbf=True)),
           (913, S.water_drop(total=40_000, seed=913, basic_pbf=False))]
    kind_params, selections = {}, {}
    for vseed, sp in val:
        if len(nets) * len(oms) > 1:
            case = ValidationCase(make=lambda mode, params, sp=sp: make(sp, mode, params), dt=dt,
                                  before=args.presteps if args.presteps >= 0 else 40, counted=VALIDATION_SUBSTEPS)
            choice, table = select_warm_start(nets, [case], oms, nmin, args.ws_energy_slack,
                                              args.ws_height_slack)
        else:
            key = next(iter(nets))
            nets[key].omega_max, nets[key].min_neighbors = oms[0], nmin
            choice, table = {"net": key, "omega_max": oms[0], "min_neighbors": nmin,
                             "params": nets[key].params.clone()}, None
        kind_params[kind(sp)] = choice["params"] if choice else None
        selections[kind(sp)] = _selection_info(choice, table, [vseed], args)
    train_s = time.perf_counter() - t0

    learned_mode = N.WARM_LEARNED | N.WARM_PROJECTED
    ctxs = [make(sp, learned_mode if kind_params[kind(sp)] is not None else 0, kind_params[kind(sp)])
            for sp in specs]
    batch = Batch(ctxs)
    batch.set_persistent_solve(args.batch_persistent)
    for _ in range(args.presteps if args.presteps >= 0 else 40):
        batch.substep(dt)
    for c in ctxs:
        c.autotune()
    for _ in range(args.warmup):
        batch.substep(dt)
    for c in ctxs:
        c.check_status()
    windows = [_window_snapshot(c) for c in ctxs]  # the sequential and e2e runs replay this window
    n_total = sum(sp.n for sp in specs)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    l0 = sum(c.launch_count() for c in ctxs)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        batch.substep(dt)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = sum(c.launch_count() for c in ctxs) - l0
    total_ms = float(np.sum([a.elapsed_time(b) for a, b in ev]))
    infos = [c.check_status() for c in ctxs]
    errs = [float(c.reduce_fp64()[2]) for c in ctxs]
    passes = sum(i.density_passes for i in infos) / (len(ctxs) * args.steps)
    conv = sum(i.converged_substeps for i in infos)
    if dist:
        dist.barrier()
    total_ms, processed = reduce_over_ranks(total_ms, float(n_total * args.steps), dist, f"cuda:{local}")
    value = processed / (total_ms / 1000.0)

    # the same scenes one after the other (each a whole-substep graph), the same
    # window replayed from its start state
    for c, w in zip(ctxs, windows):
        _restore_window(c, w)
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        ev2[k][0].record(stream)
        for c in ctxs:
            c.substep(dt)
        ev2[k][1].record(stream)
    torch.cuda.synchronize()
    seq_ms = float(np.sum([a.elapsed_time(b) for a, b in ev2]))
    seq_passes = sum(c.check_status().density_passes for c in ctxs) / (len(ctxs) * args.steps)

    # per-scene density error: the device's FP64 value against the oracle's FP64
    # recomputation on the same (downloaded) state, for every 8th scene
    e2e = run_batch_e2e(batch, ctxs, args, dt, windows)
    whole = batch_whole_job(seq_ms, float(n_total * args.steps), e2e.pop("_seconds"), e2e.pop("_particles"),
                            len(specs), n_total, dist, f"cuda:{local}")
    e2e["value"] = whole["e2e_value"]
    check = []
    if rank == 0 and not args.no_cpu_baseline:
        from apbf_gb300.api import incompressibility, neighborhood_green
        from oracle import oracle as orc

        # every 8th scene, alternating dam breaks, plain and adaptive water drops
        for k in [8 * i + (0, 1, 3)[i % 3] for i in range(len(ctxs) // 8)]:
            c, sp = ctxs[k], specs[k]
            scale = 1.0 if sp.basic_pbf else 1.5
            st, _ = c.download()
            # device: neighbour search + one density pass on this state (FP32 sums, FP64 mean)
            neighborhood_green().set_data(c).set_range_scale(scale).set_position_range(
                sp.grid_min, sp.grid_max, sp.log2res).apply()
            incompressibility().set_data(c).apply()
            e_dev = float(c.reduce_fp64()[2])
            # oracle: the same state in FP64
            fs = orc.FluidState(st)
            orc.neighborhood_green(fs, scale, sp.grid_min, sp.grid_max, sp.log2res, int(st["position"].shape[0] * 160))
            e_or = float(orc.density_error(fs, orc.settings_from(c.settings))[0])
            check.append({"scene": k, "particles": int(st["position"].shape[0]), "adaptive": not sp.basic_pbf,
                          "device": e_dev, "oracle_fp64": e_or, "abs_diff": abs(e_dev - e_or)})
    batch.close()
    for c in ctxs:
        c.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (int32 fixed-point positions and sums; bf16 MLP)",
            "data": "synthetic (seeded scene table)",
            "config": {"workload": args.workload, "scenes": whole["scenes"], "particles_total": whole["particles_total"],
                       "per_rank_fields": (None if world == 1 else
                                           "rank 0's own scene table: particles_min/max, adaptive_scenes, passes, "
                                           "convergence, scene errors, oracle check, warm-start selection"),
                       "particles_min": int(min(sp.n for sp in specs)), "particles_max": int(max(sp.n for sp in specs)),
                       "adaptive_scenes": int(sum(not sp.basic_pbf for sp in specs)), "dt": dt,
                       "solver": ("learned warm start + projected Jacobi passes, per-scene convergence; "
                                  "kinds without an admissible warm start: reference Jacobi rule: " +
                                  (", ".join(k for k, v in kind_params.items() if v is None) or "none")),
                       "iterations": f"until mean density error <= {args.error_target} (max {args.max_iterations})",
                       "density_passes_per_scene_substep": passes,
                       "converged_scene_substeps": f"{conv}/{len(ctxs) * args.steps}",
                       "launch": ("one CUDA graph per substep, scenes as parallel branches" +
                                  (" around one persistent cooperative launch of every scene's Jacobi passes 1.."
                                   if args.batch_persistent else "")),
                       "l2": "flushed between timed steps (256 MB write)"},
            "sequential": {"ms_per_step": whole["sequential_ms"] / args.steps,
                           "value": whole["sequential_value"],
                           "density_passes_per_scene_substep": seq_passes,
                           "note": "the same window of the same scenes replayed, one whole-substep graph launch "
                                   "each, one after the other"},
            "scene_density_error_last_pass": {"min": min(errs), "max": max(errs), "mean": float(np.mean(errs))},
            "oracle_density_error_check": check,
            "warm_start_training": {"samples": n_samples, "seconds": round(train_s, 2),
                                    "per_scene_kind": selections},
            "roofline": None, "gpu_launches": int(launches), "clocks": clk, "e2e": e2e,
            "cpu_baseline": None,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_batch_e2e(batch, ctxs, args, dt, windows) -> dict:
    """The batch's timed window again, driven from host memory, through the C ABI's
    host-buffer calls for every scene: apbf_fluid_write of the scene's full particle
    state from pinned host memory, one batched substep (one graph launch), each
    scene's new particle count, and apbf_fluid_read of every full state back, then a
    stream synchronisation.  Warm-up and timed steps each start from the window's
    start state."""
    import torch

    stream = torch.cuda.current_stream()
    hosts = [_host_lists(c) for c in ctxs]
    counts = [torch.zeros(1, dtype=torch.int32).pin_memory() for _ in ctxs]
    per_particle = sum(t[0].numel() * t.element_size() for t in hosts[0].values())

    def step(ns):
        for c, h, n in zip(ctxs, hosts, ns):
            c.fluid_write(h, n)
        batch.substep(dt)
        out = []
        for c, h, cnt in zip(ctxs, hosts, counts):
            m, _ = c.lengths()
            c.fluid_read(h, m, cnt)
            out.append(m)
        stream.synchronize()
        return out

    def restart():
        for c, w, h in zip(ctxs, windows, hosts):
            _restore_window(c, w, h)
        return [w["n"] for w in windows]

    steps = args.steps
    ns = restart()
    for _ in range(min(args.warmup, steps)):
        ns = step(ns)
    ns = restart()
    for c in ctxs:
        c.check_status()
    h2d = d2h = total = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        h2d += sum(ns) * per_particle
        ns = step(ns)
        d2h += sum(ns) * per_particle + 4 * len(ns)
        total += sum(ns)
    el = time.perf_counter() - t0
    infos = [c.check_status() for c in ctxs]
    return {"value": total / el, "_seconds": el, "_particles": float(total), "unit": UNIT, "h2d_bytes_per_step": int(h2d / steps),
            "d2h_bytes_per_step": int(d2h / steps), "steps": steps, "warmup": min(args.warmup, steps),
            "density_passes_per_scene_substep": sum(i.density_passes for i in infos) / (len(ctxs) * steps),
            "window": "the device-resident timed window replayed from its start state",
            "api": "per scene apbf_fluid_write, one batched substep, per scene apbf_get_lengths + apbf_fluid_read "
                   "(C ABI, pinned host buffers)"}


def _host_lists(ctx) -> dict:
    """Pinned host arrays for every particle list of `ctx` (capacity rows) and the
    carried lambda sums: the layout apbf_fluid_write / apbf_fluid_read take."""
    import torch

    from apbf_gb300.api import FLUID_FIELDS

    h = {k: torch.empty((ctx.capacity, c) if c > 1 else (ctx.capacity,), dtype=d).pin_memory()
         for k, (d, c) in FLUID_FIELDS.items()}
    h["lambda_prev"] = torch.empty(ctx.capacity, dtype=torch.float32).pin_memory()
    return h


def _window_snapshot(ctx) -> dict:
    """Everything a substep carries to the next (the particle lists with the carried
    lambda sums in pinned host memory, the transfer list on the device), taken at the
    start of the timed window.  An emitter's phase is not part of it."""
    import torch

    n, nt = ctx.lengths()
    host = _host_lists(ctx)
    cnt = torch.zeros(1, dtype=torch.int32).pin_memory()
    ctx.fluid_read(host, n, cnt)
    tv = ctx.transfers_view()
    tr = {k: tv[k][:nt].clone() for k in ("source", "target", "time_left")}
    torch.cuda.synchronize()
    return {"host": host, "n": n, "nt": nt, "transfers": tr}


def _restore_window(ctx, w: dict, work: dict | None = None) -> None:
    """Puts the transfer list back on the device and the snapshot's particle lists
    into the caller's host arrays (`work`), or with work=None straight into the
    device lists; untimed setup."""
    import torch

    tv = ctx.transfers_view()
    for k, v in w["transfers"].items():
        tv[k][:w["nt"]].copy_(v)
    ctx.set_lengths(w["n"], w["nt"])
    if work is None:
        ctx.fluid_write(w["host"], w["n"])
    else:
        for k, v in w["host"].items():
            work[k].copy_(v)
    torch.cuda.synchronize()


def run_e2e(ctx, spec, args, window: dict) -> dict:
    """The timed window again, driven from host memory: per step, through the C ABI,
    apbf_fluid_write of the full particle state (the ten lists and the warm start's
    lambda history) from pinned host memory, one apbf_substep, the new particle count
    (an emitter or split/merge changes it), apbf_fluid_read of the full resulting state
    back into pinned host memory, then a stream synchronisation.  Warm-up and timed
    steps each start from the state at the start of the device-resident timed window,
    so both measurements time the same substeps (same pass counts, reported)."""
    import torch

    host = _host_lists(ctx)
    per_particle = sum(t[0].numel() * t.element_size() for t in host.values())
    count = torch.zeros(1, dtype=torch.int32).pin_memory()
    stream = torch.cuda.current_stream()
    steps = args.steps

    def step(n):
        ctx.fluid_write(host, n)
        ctx.substep(spec.dt)
        m, _ = ctx.lengths()  # synchronises: the count the read needs
        ctx.fluid_read(host, m, count)
        stream.synchronize()
        return m

    _restore_window(ctx, window, host)
    n = window["n"]
    for _ in range(min(args.warmup, steps)):  # untimed
        n = step(n)
    _restore_window(ctx, window, host)
    n = window["n"]
    ctx.check_status()  # clears the counters
    h2d = d2h = 0
    done = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        h2d += n * per_particle
        n = step(n)
        d2h += n * per_particle + 4
        done += n
    el = time.perf_counter() - t0
    info = ctx.check_status()
    return {"value": done / el, "unit": UNIT, "h2d_bytes_per_step": int(h2d / steps),
            "d2h_bytes_per_step": int(d2h / steps), "steps": steps, "warmup": min(args.warmup, steps),
            "density_passes_per_substep": info.density_passes / steps,
            "converged_substeps": f"{info.converged_substeps}/{steps}",
            "window": "the device-resident timed window replayed from its start state",
            "api": "apbf_fluid_write + apbf_substep + apbf_get_lengths + apbf_fluid_read (C ABI, pinned host buffers)"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--max-iterations", type=int, default=100)
    ap.add_argument("--error-target", type=float, default=0.001)
    ap.add_argument("--presteps", type=int, default=-1, help="untimed substeps before warm-up (-1: scene default)")
    ap.add_argument("--max-neighbors", type=int, default=192)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle-check", action="store_true", help="skip the FP64 oracle check of the final state")
    ap.add_argument("--no-warm-start", action="store_true", help="headline = the reference Jacobi rule")
    ap.add_argument("--no-plain", action="store_true", help="skip the two plain-solver comparison runs")
    ap.add_argument("--solve", choices=("learned", "reference", "projected"), default="learned",
                    help="headline solve: the learned warm start (default), or one plain rule without a network")
    ap.add_argument("--ws-epochs", type=int, default=3)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--oracle-variant", choices=("f32", "f64"), default="f32",
                    help="reference arm: the oracle's FP32 build (default) or the FP64 oracle")
    ap.add_argument("--search-levels", type=int, default=1,
                    help="finer search grids than the scene's that the search tuner may try")
    ap.add_argument("--graph-mode", type=int, default=2, choices=(0, 1, 2),
                    help="0 per-kernel launches, 1 solve loop as a graph, 2 whole substep as a graph")
    ap.add_argument("--prof-steps", type=int, default=8, help="traced substeps after the timed ones (kernel shares)")
    ap.add_argument("--batch-persistent", action="store_true",
                    help="batch64: every scene's Jacobi passes 1.. in one persistent cooperative launch")
    ap.add_argument("--persistent", action="store_true",
                    help="Jacobi passes 1.. as one persistent cooperative kernel (apbf_set_persistent_solve)")
    ap.add_argument("--ws-min-neighbors", type=float, default=None,
                    help="warm-start guard: particles with fewer neighbours keep the plain lambda (default 16)")
    ap.add_argument("--ws-omega", type=float, default=None,
                    help="warm-start over-relaxation bound (default: chosen by validation on held-out seeds)")
    ap.add_argument("--ws-over-weight", type=float, default=None,
                    help="overshoot weight of the training loss (default: networks for 4, 8, 16, chosen by validation)")
    ap.add_argument("--ws-energy-slack", type=float, default=1.05,
                    help="validation admits a warm start whose final mean |v|^2 is at most this times the plain "
                         "rule's (<= 0: no energy condition)")
    ap.add_argument("--ws-height-slack", type=float, default=1.25,
                    help="validation admits a warm start whose final 99th-percentile particle height is at most "
                         "this times the plain rule's (<= 0: no height condition)")
    ap.add_argument("--warm-start-report", action="store_true",
                    help="train one warm start on the mixture and report passes saved on each of its workloads")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.warm_start_report:
        run_warm_start_report(args)
    elif args.impl == "reference":
        run_reference(args)
    elif WORKLOADS[args.workload][0] == "batch":
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
