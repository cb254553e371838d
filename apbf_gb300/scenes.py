"""Seeded synthetic scenes in the reference's units.

Length unit = radius of the smallest particle (the reference's scenes use radius
1, source/main.cpp:63-68); kernel width 4 radii (KERNEL_SCALE,
cpu_gpu_shared_config.h:14); rest density 1, so a particle of radius r has
inverse mass 1 / (2r)^3 (source/initialize.cpp:25).  Scenes stated in metres
are converted by dividing lengths by the particle radius in metres; time is
unchanged, so gravity becomes g / r_m.

Particles are laid out like initialize_box.comp:38-45 (lattice spacing 2r, first
particle at min + r), with a seeded uniform jitter.  Walls follow pool.cpp:30-40
(four-radius-thick boxes around the container).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

FIX = 262144.0  # POS_RESOLUTION, cpu_gpu_shared_config.h:7


@dataclass
class SceneSpec:
    name: str
    state: dict                 # numpy arrays, one entry per particle
    box_min: np.ndarray         # (nb, 4) float32
    box_max: np.ndarray
    grid_min: tuple
    grid_max: tuple
    log2res: int
    acceleration: tuple
    dt: float
    iterations: int
    substeps: int
    basic_pbf: bool
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.state["position"].shape[0])


def _to_fixed(p: np.ndarray) -> np.ndarray:
    out = np.zeros((p.shape[0], 4), dtype=np.int32)
    out[:, :3] = np.trunc(p * np.float32(FIX)).astype(np.int32)
    return out


def make_state(pos: np.ndarray, radius: float = 1.0) -> dict:
    """Per-particle state as initialize_box.comp writes it plus the fluid defaults of pool.cpp:22-25."""
    n = pos.shape[0]
    ipos = _to_fixed(pos.astype(np.float32))
    r = np.float32(radius)
    return {
        "position": ipos,
        "velocity": np.zeros((n, 4), np.float32),
        "inverse_mass": np.full(n, np.float32(1.0) / np.float32((2.0 * r) ** 3), np.float32),
        "radius": np.full(n, r, np.float32),
        "pos_backup": ipos.copy(),
        "transferring": np.zeros(n, np.uint32),
        "target_radius": np.full(n, r, np.float32),
        "kernel_width": np.full(n, r * np.float32(4.0), np.float32),
        "boundariness": np.ones(n, np.float32),
        "boundary_distance": np.full(n, np.uint32(r * FIX), np.uint32),
    }


def wall_boxes(a_min, a_max, radius: float = 1.0, lid: bool = True, thickness: float = 4.0):
    """pool.cpp:30-40: walls of thickness 4 around [a_min, a_max + (0, 2r, 0)].

    box_collision pushes a particle out through the nearest face of a box
    (box_collision.comp:45-57), so a particle that moves more than half the wall
    thickness into a wall in one substep leaves through the far side; scenes with
    fast impacts pass a larger thickness."""
    t = float(thickness)
    wmin = np.asarray(a_min, np.float64) - t
    wmax = np.asarray(a_max, np.float64) + t + np.array([0.0, 2.0 * radius, 0.0])
    boxes = [
        (wmin, [wmin[0] + t, wmax[1], wmax[2]]),
        (wmin, [wmax[0], wmin[1] + t, wmax[2]]),
        ([wmax[0] - t, wmin[1], wmin[2]], wmax),
    ]
    if lid:
        boxes.append(([wmin[0], wmax[1] - t, wmin[2]], wmax))
    boxes.append((wmin, [wmax[0], wmax[1], wmin[2] + t]))
    boxes.append(([wmin[0], wmin[1], wmax[2] - t], wmax))
    bmin = np.zeros((len(boxes), 4), np.float32)
    bmax = np.zeros((len(boxes), 4), np.float32)
    for k, (lo, hi) in enumerate(boxes):
        bmin[k, :3] = lo
        bmax[k, :3] = hi
    return bmin, bmax


def lattice(origin, counts, spacing: float, jitter: float, rng: np.random.Generator) -> np.ndarray:
    ii, jj, kk = np.meshgrid(np.arange(counts[0]), np.arange(counts[1]), np.arange(counts[2]), indexing="ij")
    p = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64) * spacing
    p += np.asarray(origin, np.float64)
    if jitter > 0:
        p += rng.uniform(-jitter, jitter, size=p.shape)
    return p


def _grid_for(lo, hi, kernel_width: float = 4.0, max_log2res: int = 8):
    """Cubic Morton grid covering [lo, hi] with the coarsest resolution whose cells
    are at most one kernel width wide: a search then visits about (2h/c + 1)^3
    cells of c^3/8 particles each, which keeps candidates per particle near
    150-250 instead of the ~900 of cells twice as wide."""
    lo = np.asarray(lo, np.float64) - 4.0
    hi = np.asarray(hi, np.float64) + 4.0
    side = float(np.max(hi - lo))
    L = 1
    while L < max_log2res and side / (1 << L) > kernel_width:
        L += 1
    return tuple(lo.tolist()), tuple((lo + side).tolist()), L


def dam_break(n_side: int = 32, seed: int = 0, substeps: int = 200, iterations: int = 4) -> SceneSpec:
    """Plain PBF dam break: n_side^3 particles, lattice 0.05 m (= 2r, r = 0.025 m),
    jitter +/-0.005 m, in a 3.2 x 1.6 x 1.6 m box; h = 0.1 m; g = -9.81; dt = 1/120."""
    r_m = 0.025
    rng = np.random.default_rng(seed)
    box = np.array([3.2, 1.6, 1.6]) / r_m  # 128 x 64 x 64
    pos = lattice([1.0, 1.0, 1.0], [n_side] * 3, 2.0, 0.005 / r_m, rng)
    st = make_state(pos)
    # the front reaches ~2 radii per substep: 16-radius walls keep it inside
    bmin, bmax = wall_boxes([0, 0, 0], box, thickness=16.0)
    gmin, gmax, L = _grid_for([0, 0, 0], box)
    return SceneSpec("dam_break", st, bmin, bmax, gmin, gmax, L, (0.0, -9.81 / r_m, 0.0), 1.0 / 120.0, iterations,
                     substeps, True, {"r_m": r_m, "box": box.tolist()})


def water_drop(total: int = 250_000, seed: int = 0, substeps: int = 500, iterations: int = 6,
               basic_pbf: bool = False) -> SceneSpec:
    """Water drop: a sphere of radius 0.3 m (lattice 0.01 m = 2r, r = 0.005 m) whose
    centre starts 1.0 m above the pool floor, over a 2 x 2 x 0.5 m pool filled to the
    height that brings the total to `total` particles; dt = 1/240, 6 iterations.
    For totals other than 250 000 every length is scaled by (total / 250 000)^(1/3)
    at the same particle spacing, so the scene keeps its shape."""
    r_m = 0.005
    g = (total / 250_000.0) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    box = np.array([2.0, 0.5, 2.0]) / r_m * g  # x, y (up), z: 400 x 100 x 400 at 250k
    R = 0.3 / r_m * g
    centre = np.array([box[0] / 2, 1.0 / r_m * g, box[2] / 2])
    m = int(np.ceil(R))
    sp = lattice(centre - 2 * m, [m * 2 + 1] * 3, 2.0, 0.0, rng)
    sp = sp[np.sum((sp - centre) ** 2, axis=1) <= R * R]
    sp += rng.uniform(-0.2, 0.2, size=sp.shape)
    nx, nz = int(box[0] // 2), int(box[2] // 2)
    per_layer = nx * nz
    remaining = max(total - sp.shape[0], 0)
    layers = remaining // per_layer
    pool = lattice([1.0, 1.0, 1.0], [nx, max(layers, 0), nz], 2.0, 0.2, rng) if layers > 0 else np.zeros((0, 3))
    extra = remaining - pool.shape[0]
    if extra > 0:  # a partial top layer, taken in a seeded order
        top = lattice([1.0, 1.0 + 2.0 * layers, 1.0], [nx, 1, nz], 2.0, 0.2, rng)
        top = top[rng.permutation(top.shape[0])[:extra]]
        pool = np.concatenate([pool, top], axis=0)
    pos = np.concatenate([pool, sp], axis=0)
    st = make_state(pos)
    hi = np.maximum(box, centre + R + 2)
    # the drop hits the floor at ~3 radii per substep: 32-radius walls, as high as
    # the drop's start and closed by a lid there, so that the splash stays inside the
    # search grid (particles outside it are clamped into its border cells)
    bmin, bmax = wall_boxes([0, 0, 0], [box[0], hi[1], box[2]], lid=True, thickness=32.0)
    gmin, gmax, L = _grid_for([0, 0, 0], hi)
    # free fall of the drop onto the pool surface: (1.0 m - 0.3 m - fill) / (g/2) -> ~90 substeps at 250k
    fall = max(centre[1] - R - 2.0 * (layers + 1), 0.0) * r_m
    impact = int(np.sqrt(2.0 * fall / 9.81) * 240.0)
    return SceneSpec("water_drop", st, bmin, bmax, gmin, gmax, L, (0.0, -9.81 / r_m, 0.0), 1.0 / 240.0, iterations,
                     substeps, basic_pbf, {"r_m": r_m, "box": box.tolist(), "sphere": int(sp.shape[0]),
                                           "presteps": impact + 20})


def block(n: int, seed: int = 0, iterations: int = 4, dt: float = 1.0 / 120.0) -> SceneSpec:
    """A settled-size cube of about n particles in a closed pool (plain PBF), used for
    scaling runs at sizes between the named scenes."""
    side = max(2, int(round(n ** (1.0 / 3.0))))
    rng = np.random.default_rng(seed)
    pos = lattice([1.0, 1.0, 1.0], [side] * 3, 2.0, 0.2, rng)[:n]
    box = np.array([2.0 * side + 2, 2.0 * side + 2, 2.0 * side + 2])
    st = make_state(pos)
    bmin, bmax = wall_boxes([0, 0, 0], box)
    gmin, gmax, L = _grid_for([0, 0, 0], box)
    return SceneSpec("block", st, bmin, bmax, gmin, gmax, L, (0.0, -392.4, 0.0), dt, iterations, 1, True,
                     {"side": side})


def waterfall(initial: int = 384_000, seed: int = 0, substeps: int = 300, iterations: int = 6,
              basic_pbf: bool = False, per_substep: int = 2000, scale: float = 1.0) -> SceneSpec:
    """Waterfall: a seeded inflow of `per_substep` particles per substep (radius
    0.0025 m) from a 0.2 x 0.2 m emitter falls 1.5 m onto a sloped box (30 degrees,
    0.05 m thick) and runs into a 2 x 1 x 0.6 m tank pre-filled with `initial`
    particles; dt = 1/240.  The emitter's stream speed follows from the rate:
    per_substep particles per dt through 40 x 40 lattice cells of spacing 2r.
    `scale` < 1 shrinks every length (tank, slope, drop, emitter) for tests."""
    r_m = 0.0025
    rng = np.random.default_rng(seed)
    s = float(scale)
    box = np.array([800.0, 960.0, 240.0]) * s          # x, y (up), z in radii
    nx_fill, nz_fill = int(box[0] // 2), int(box[2] // 2)
    layers = max(1, int(round(initial / (nx_fill * nz_fill)))) if initial > 0 else 0
    pos = lattice([1.0, 1.0, 1.0], [nx_fill, layers, nz_fill], 2.0, 0.2, rng) if layers else np.zeros((0, 3))
    st = make_state(pos)
    bmin, bmax = wall_boxes([0, 0, 0], box, lid=True, thickness=32.0)
    # the slope: descends towards +x; its upper end under the emitter
    theta = -np.pi / 6.0
    centre = np.array([300.0, 200.0, 120.0]) * s
    half = np.array([200.0, 20.0, 100.0]) * s
    quat = np.array([0.0, 0.0, np.sin(theta / 2.0), np.cos(theta / 2.0)])
    upper = centre + np.array([np.cos(theta), np.sin(theta), 0.0]) * (-half[0])
    cells = max(2, int(round(40 * s)))  # emitter lattice cells per side (0.2 m at full size)
    dt = 1.0 / 240.0
    speed = per_substep / float(cells * cells) * 2.0 / dt  # radii per second
    emit_y = upper[1] + half[1] + 600.0 * s                # 1.5 m above the slope's top
    emitter = dict(origin=(float(upper[0] - cells), float(emit_y), float(centre[2] - cells)), radius=1.0,
                   nx=cells, nz=cells, speed=float(speed), jitter=0.2, seed=seed + 17)
    gmin, gmax, L = _grid_for([0, 0, 0], box)
    return SceneSpec("waterfall", st, bmin, bmax, gmin, gmax, L, (0.0, -9.81 / r_m, 0.0), dt, iterations, substeps,
                     basic_pbf, {"r_m": r_m, "box": box.tolist(), "emitter": emitter,
                                 "oriented_boxes": (np.array([[*centre, 0.0]], np.float32),
                                                    np.array([[*half, 0.0]], np.float32),
                                                    np.array([quat], np.float32)),
                                 "capacity": int(initial + per_substep * substeps * 1.05) + 4096, "presteps": 0,
                                 "per_substep": per_substep})
