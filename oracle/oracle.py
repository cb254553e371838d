"""ctypes wrapper of the oracle library (oracle/_build/libapbf_oracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py as the reference for parity and the timed CPU restatement.  The product
(apbf_gb300) never imports this module.

APBF_ORACLE_VARIANT=f32 in the environment (read when the library is first
loaded) selects libapbf_oracle_f32.so instead: the same code with the kernels and
the incompressibility passes in FP32, timed as a CPU baseline and checked against
the FP64 library, never used as the parity reference.

States are dicts of numpy arrays in the layout of apbf_gb300.scenes.make_state.
Every function copies its inputs, so callers keep their arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / ("libapbf_oracle_f32.so" if os.environ.get("APBF_ORACLE_VARIANT") == "f32"
                         else "libapbf_oracle.so")

_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_f32p = C.POINTER(C.c_float)


class OrSettings(C.Structure):
    _fields_ = [
        ("height_kernel_id", C.c_int32),
        ("gradient_kernel_id", C.c_int32),
        ("merge", C.c_int32),
        ("split", C.c_int32),
        ("base_kernel_width_on_target_radius", C.c_int32),
        ("base_kernel_width_on_boundary_distance", C.c_int32),
        ("update_target_radius", C.c_int32),
        ("update_boundariness", C.c_int32),
        ("boundariness_calculation_method", C.c_int32),
        ("basic_pbf", C.c_int32),
        ("solver_iterations", C.c_int32),
        ("pad0", C.c_int32),
        ("boundariness_adaption_speed", C.c_float),
        ("kernel_width_adaption_speed", C.c_float),
        ("boundariness_self_grad_length_factor", C.c_float),
        ("boundariness_underpressure_factor", C.c_float),
        ("merge_duration", C.c_float),
        ("split_duration", C.c_float),
        ("smallest_target_radius", C.c_float),
        ("target_radius_offset", C.c_float),
        ("target_radius_scale_factor", C.c_float),
        ("density_error_target", C.c_float),
        ("pad1", C.c_float * 2),
    ]


class OrFluid(C.Structure):
    _fields_ = [
        ("n", C.c_uint32),
        ("cap", C.c_uint32),
        ("pos", _i32p),
        ("vel", _f32p),
        ("inv_mass", _f32p),
        ("radius", _f32p),
        ("pos_backup", _i32p),
        ("transferring", _u32p),
        ("target_radius", _f32p),
        ("kernel_width", _f32p),
        ("boundariness", _f32p),
        ("boundary_distance", _u32p),
    ]


class OrTransfers(C.Structure):
    _fields_ = [("n", C.c_uint32), ("cap", C.c_uint32), ("source", _u32p), ("target", _u32p), ("time_left", _f32p)]


class OrNeighbors(C.Structure):
    _fields_ = [("n", C.c_uint32), ("cap", C.c_uint32), ("offsets", _u32p), ("idx", _u32p)]


class OrBoxes(C.Structure):
    _fields_ = [("n", C.c_uint32), ("bmin", _f32p), ("bmax", _f32p), ("rot", _f32p)]


def _boxes(boxes) -> tuple:
    """(bmin, bmax) or (bmin, bmax, rot) -> OrBoxes and the arrays it points into."""
    lo = np.ascontiguousarray(boxes[0], np.float32)
    hi = np.ascontiguousarray(boxes[1], np.float32)
    rot = np.ascontiguousarray(boxes[2], np.float32).reshape(-1) if len(boxes) > 2 and boxes[2] is not None else None
    b = OrBoxes(lo.shape[0], _p(lo, _f32p), _p(hi, _f32p), _p(rot, _f32p) if rot is not None else None)
    return b, (lo, hi, rot)


class OrIncompOut(C.Structure):
    _fields_ = [("density", _u32p), ("grad_sum", _i32p), ("sq_grad_sum", _u32p), ("lambda_", _f32p),
                ("divergence", _f32p), ("lambda_in", _f32p), ("projected_acc", _f32p), ("applied", _f32p)]


class OrScene(C.Structure):
    _fields_ = [
        ("settings", OrSettings),
        ("minp", C.c_float * 3),
        ("maxp", C.c_float * 3),
        ("log2res", C.c_uint32),
        ("accel", C.c_float * 3),
        ("last_dt", C.c_float),
        ("max_transfers", C.c_uint32),
        ("search_method", C.c_uint32),
    ]


_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.or_range_fixed.restype = C.c_int64
        L.or_range_fixed.argtypes = [C.c_float, C.c_float]
        L.or_neighbors_build.restype = C.c_uint64
        L.or_neighbors_brute.restype = C.c_uint64
        L.or_neighborhood_green.restype = C.c_uint64
        L.or_neighborhood_binary_search.restype = C.c_uint64
        L.or_neighbors_binary_search.restype = C.c_uint64
        L.or_substep.restype = C.c_uint64
        L.or_cell_coord.restype = C.c_uint32
        L.or_cell_coord.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_uint32]
        L.or_morton.restype = C.c_uint32
        L.or_delete_edit_list.restype = C.c_uint32
        L.or_kernel_height.restype = C.c_double
        L.or_glue_generate.restype = C.c_uint32
        L.or_emit.restype = C.c_uint32
        L.or_kernel_height.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_double]
        L.or_kernel_gradient.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


# pbd::settings defaults (source/settings.cpp:5-31), restated for the oracle so that
# callers that time or check the oracle need not load the product library.
DEFAULT_SETTINGS = {
    "height_kernel_id": 1, "gradient_kernel_id": 1, "merge": 1, "split": 1,
    "base_kernel_width_on_target_radius": 1, "base_kernel_width_on_boundary_distance": 1,
    "update_target_radius": 1, "update_boundariness": 1, "boundariness_calculation_method": 2, "basic_pbf": 0,
    "solver_iterations": 3, "boundariness_adaption_speed": 0.5, "kernel_width_adaption_speed": 0.01,
    "boundariness_self_grad_length_factor": 2.0, "boundariness_underpressure_factor": 4.0, "merge_duration": 2.0,
    "split_duration": 0.0, "smallest_target_radius": 1.0, "target_radius_offset": 10.0,
    "target_radius_scale_factor": 0.3, "density_error_target": 0.0,
}


def settings_from(src) -> OrSettings:
    """Copies a settings struct with the same field names (apbf_gb300 Settings or dict)."""
    s = OrSettings()
    for name, _ in OrSettings._fields_:
        if name.startswith("pad"):
            continue
        v = src.get(name, 0) if isinstance(src, dict) else getattr(src, name)
        setattr(s, name, v)
    return s


class FluidState:
    """Owns numpy arrays (with spare capacity) and the OrFluid struct pointing at them."""

    FIELDS = [
        ("position", np.int32, 4), ("velocity", np.float32, 4), ("inverse_mass", np.float32, 1),
        ("radius", np.float32, 1), ("pos_backup", np.int32, 4), ("transferring", np.uint32, 1),
        ("target_radius", np.float32, 1), ("kernel_width", np.float32, 1), ("boundariness", np.float32, 1),
        ("boundary_distance", np.uint32, 1),
    ]

    def __init__(self, state: dict, cap: int | None = None, transfers: dict | None = None, tcap: int = 10000):
        n = int(state["position"].shape[0])
        cap = max(cap or n, n, 1)
        self.arrays = {}
        for name, dt, comp in self.FIELDS:
            a = np.zeros((cap, comp) if comp > 1 else (cap,), dtype=dt)
            a[:n] = np.asarray(state[name]).view(dt).reshape(a[:n].shape)
            self.arrays[name] = a
        A = self.arrays
        self.f = OrFluid(n, cap, _p(A["position"], _i32p), _p(A["velocity"], _f32p), _p(A["inverse_mass"], _f32p),
                         _p(A["radius"], _f32p), _p(A["pos_backup"], _i32p), _p(A["transferring"], _u32p),
                         _p(A["target_radius"], _f32p), _p(A["kernel_width"], _f32p), _p(A["boundariness"], _f32p),
                         _p(A["boundary_distance"], _u32p))
        self.tsrc = np.zeros(tcap, np.uint32)
        self.ttgt = np.zeros(tcap, np.uint32)
        self.tttl = np.zeros(tcap, np.float32)
        nt = 0
        if transfers is not None:
            nt = int(transfers["source"].shape[0])
            self.tsrc[:nt] = transfers["source"]
            self.ttgt[:nt] = transfers["target"]
            self.tttl[:nt] = transfers["time_left"]
        self.t = OrTransfers(nt, tcap, _p(self.tsrc, _u32p), _p(self.ttgt, _u32p), _p(self.tttl, _f32p))
        self.nb = None

    @property
    def n(self) -> int:
        return int(self.f.n)

    def state(self) -> dict:
        n = self.n
        return {k: v[:n].copy() for k, v in self.arrays.items()}

    def transfers(self) -> dict:
        nt = int(self.t.n)
        return {"source": self.tsrc[:nt].copy(), "target": self.ttgt[:nt].copy(), "time_left": self.tttl[:nt].copy()}

    def alloc_neighbors(self, cap_pairs: int) -> OrNeighbors:
        self.nb_off = np.zeros(self.f.cap + 1, np.uint32)
        self.nb_idx = np.zeros(max(cap_pairs, 1), np.uint32)
        self.nb = OrNeighbors(0, cap_pairs, _p(self.nb_off, _u32p), _p(self.nb_idx, _u32p))
        return self.nb

    def rows(self) -> list:
        off = self.nb_off
        return [self.nb_idx[off[i]:off[i + 1]].astype(np.int64) for i in range(self.n)]


# ---------------------------------------------------------------- primitives
def prefix_sum(values: np.ndarray) -> np.ndarray:
    v = np.ascontiguousarray(values, np.uint32)
    out = np.zeros_like(v)
    lib().or_prefix_sum_inclusive(_p(v, _u32p), _p(out, _u32p), C.c_size_t(v.size))
    return out


def sort_pairs(keys: np.ndarray, vals: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    k = np.ascontiguousarray(keys, np.uint32)
    v = np.ascontiguousarray(vals, np.uint32)
    ok, ov = np.zeros_like(k), np.zeros_like(v)
    lib().or_sort_pairs_stable(_p(k, _u32p), _p(v, _u32p), C.c_size_t(k.size), _p(ok, _u32p), _p(ov, _u32p))
    return ok, ov


def apply_edit(src: np.ndarray, edit: np.ndarray, stride_words: int = 1) -> np.ndarray:
    s = np.ascontiguousarray(src, np.uint32).ravel()
    e = np.ascontiguousarray(edit, np.uint32)
    out = np.zeros(e.size * stride_words, np.uint32)
    lib().or_apply_edit_u32(_p(s, _u32p), _p(e, _u32p), C.c_size_t(e.size), stride_words, _p(out, _u32p))
    return out


def delete_edit_list(n_hidden: int, deleted: np.ndarray) -> np.ndarray:
    d = np.ascontiguousarray(deleted, np.uint32)
    edit = np.zeros(max(n_hidden, 1), np.uint32)
    m = lib().or_delete_edit_list(n_hidden, _p(d, _u32p), d.size, _p(edit, _u32p))
    return edit[:m]


def remap_index_list(lst: np.ndarray, edit: np.ndarray, n_hidden_old: int) -> tuple[np.ndarray, np.ndarray]:
    l_ = np.ascontiguousarray(lst, np.uint32)
    e = np.ascontiguousarray(edit, np.uint32)
    # exact output size: one entry per (edit entry, equal index-list entry)
    valid_l = l_[l_ < n_hidden_old]
    cnt = np.bincount(valid_l, minlength=max(n_hidden_old, 1)) if valid_l.size else np.zeros(max(n_hidden_old, 1), int)
    valid_e = e[e < n_hidden_old]
    cap = max(int(cnt[valid_e].sum()) if valid_e.size else 0, 1)
    out = np.zeros(cap, np.uint32)
    ne = np.zeros(cap, np.uint32)
    lib().or_remap_index_list.restype = C.c_uint32
    m = lib().or_remap_index_list(_p(l_, _u32p), l_.size, _p(e, _u32p), e.size, n_hidden_old, _p(out, _u32p),
                                  _p(ne, _u32p), cap)
    return out[:m], ne[:m]


# ---------------------------------------------------------------- neighbourhood
def position_keys(pos4: np.ndarray, minp, maxp, log2res: int) -> np.ndarray:
    p = np.ascontiguousarray(pos4, np.int32)
    keys = np.zeros(p.shape[0], np.uint32)
    lib().or_position_keys(_p(p, _i32p), C.c_size_t(p.shape[0]), (C.c_float * 3)(*minp), (C.c_float * 3)(*maxp),
                           log2res, _p(keys, _u32p))
    return keys


def neighbors_brute(pos4: np.ndarray, rng: np.ndarray, scale: float, cap_pairs: int = 1 << 22) -> list:
    p = np.ascontiguousarray(pos4, np.int32)
    r = np.ascontiguousarray(rng, np.float32)
    n = p.shape[0]
    off = np.zeros(n + 1, np.uint32)
    idx = np.zeros(cap_pairs, np.uint32)
    nb = OrNeighbors(0, cap_pairs, _p(off, _u32p), _p(idx, _u32p))
    tot = lib().or_neighbors_brute(_p(p, _i32p), _p(r, _f32p), C.c_float(scale), C.c_size_t(n), C.byref(nb))
    assert tot <= cap_pairs
    return [idx[off[i]:off[i + 1]].astype(np.int64) for i in range(n)]


def neighborhood_green(fs: FluidState, range_scale: float, minp, maxp, log2res: int, cap_pairs: int):
    nb = fs.alloc_neighbors(cap_pairs)
    perm = np.zeros(max(fs.n, 1), np.uint32)
    keys = np.zeros(max(fs.n, 1), np.uint32)
    tot = lib().or_neighborhood_green(C.byref(fs.f), C.byref(fs.t), C.c_float(range_scale), (C.c_float * 3)(*minp),
                                      (C.c_float * 3)(*maxp), log2res, C.byref(nb), _p(perm, _u32p), _p(keys, _u32p))
    if tot > cap_pairs:
        raise RuntimeError(f"oracle neighbour capacity {cap_pairs} < {tot}")
    return perm[:fs.n], keys[:fs.n], int(tot)


def position_codes(pos4: np.ndarray) -> np.ndarray:
    """The 96-bit position code of every particle as 3 uint32 words (least significant first)."""
    p = np.ascontiguousarray(pos4, np.int32)
    out = np.zeros((p.shape[0], 3), np.uint32)
    for i in range(p.shape[0]):
        lib().or_position_code96(_p(p[i], _i32p), _p(out[i], _u32p))
    return out


def neighborhood_binary_search(fs: FluidState, range_scale: float, cap_pairs: int):
    """neighborhood_binary_search::apply on the oracle state: (permutation, sorted
    codes (n x 3 words), pair count); the rows land in the state."""
    nb = fs.alloc_neighbors(cap_pairs)
    perm = np.zeros(max(fs.n, 1), np.uint32)
    codes = np.zeros((max(fs.n, 1), 3), np.uint32)
    tot = lib().or_neighborhood_binary_search(C.byref(fs.f), C.byref(fs.t), C.c_float(range_scale), C.byref(nb),
                                              _p(perm, _u32p), _p(codes, _u32p))
    if tot > cap_pairs:
        raise RuntimeError(f"oracle neighbour capacity {cap_pairs} < {tot}")
    return perm[:fs.n], codes[:fs.n], int(tot)


def set_rows(fs: FluidState, rows: list) -> None:
    """Installs neighbour rows (e.g. the device's, for lockstep stage checks)."""
    total = sum(len(r) for r in rows)
    nb = fs.alloc_neighbors(total)
    off = 0
    for i, r in enumerate(rows):
        fs.nb_idx[off:off + len(r)] = r
        off += len(r)
        fs.nb_off[i + 1] = off
    nb.n = fs.n


# ---------------------------------------------------------------- stages
def incompressibility(fs: FluidState, settings: OrSettings, lambda_in: np.ndarray | None = None,
                      projected_acc: np.ndarray | None = None) -> dict:
    """One Jacobi pass.  lambda_in (optional): the lambda that the position update
    uses instead of the computed one (the learned warm start's first update);
    projected_acc (optional): the lambdas applied earlier in the substep, enabling
    the pull-back of a projected pass.  out["lambda"] is always the computed one,
    out["applied"] the one the update used."""
    n = fs.n
    out = {"density": np.zeros(n, np.uint32), "grad_sum": np.zeros((n, 3), np.int32),
           "sq_grad_sum": np.zeros(n, np.uint32), "lambda": np.zeros(n, np.float32),
           "divergence": np.zeros(n, np.float32), "applied": np.zeros(n, np.float32)}
    lin = None if lambda_in is None else np.ascontiguousarray(lambda_in, np.float32)
    acc = None if projected_acc is None else np.ascontiguousarray(projected_acc, np.float32)
    o = OrIncompOut(_p(out["density"], _u32p), _p(out["grad_sum"], _i32p), _p(out["sq_grad_sum"], _u32p),
                    _p(out["lambda"], _f32p), _p(out["divergence"], _f32p),
                    _p(lin, _f32p) if lin is not None else None, _p(acc, _f32p) if acc is not None else None,
                    _p(out["applied"], _f32p))
    lib().or_incompressibility_apply(C.byref(fs.f), C.byref(fs.nb), C.byref(settings), C.byref(o))
    return out


def box_collision(fs: FluidState, bmin: np.ndarray, bmax: np.ndarray, rot: np.ndarray | None = None) -> None:
    """rot: None (axis-aligned boxes) or 12 floats per box (rotation rows; see OrBoxes)."""
    b, keep = _boxes((bmin, bmax, rot))
    fs._boxes_keep = keep
    lib().or_box_collision(C.byref(fs.f), C.byref(b))


def sphere_collision(fs: FluidState, center, radius: float, hollow: bool) -> None:
    lib().or_sphere_collision(C.byref(fs.f), (C.c_float * 3)(*center), C.c_float(radius), C.c_int(1 if hollow else 0))


def inter_particle_collision(fs: FluidState) -> None:
    lib().or_inter_particle_collision(C.byref(fs.f), C.byref(fs.nb))


def glue_generate(fs: FluidState, cap: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    g0 = np.zeros(cap, np.uint32)
    g1 = np.zeros(cap, np.uint32)
    gd = np.zeros(cap, np.uint32)
    m = lib().or_glue_generate(C.byref(fs.f), C.byref(fs.nb), _p(g0, _u32p), _p(g1, _u32p), _p(gd, _u32p), cap)
    m = min(int(m), cap)
    return g0[:m].copy(), g1[:m].copy(), gd[:m].copy()


def glue_apply(fs: FluidState, g0: np.ndarray, g1: np.ndarray, gd: np.ndarray, stability: float) -> None:
    a, b, d = (np.ascontiguousarray(x, np.uint32) for x in (g0, g1, gd))
    lib().or_glue_apply(C.byref(fs.f), _p(a, _u32p), _p(b, _u32p), _p(d, _u32p), C.c_uint32(a.size),
                        C.c_float(stability))


class OrEmitter(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("radius", C.c_float), ("nx", C.c_uint32), ("nz", C.c_uint32),
                ("speed", C.c_float), ("jitter", C.c_float), ("seed", C.c_uint32), ("max_particles", C.c_uint32),
                ("enabled", C.c_uint32), ("pad", C.c_uint32)]


def emit(fs: FluidState, emitter, state: np.ndarray, dt: float, last_dt: float) -> tuple[int, bool]:
    """Appends the emitter's particles for one substep (the device's first stage);
    `emitter` has the fields of apbf_emitter, `state` is a float64[2] the caller keeps."""
    e = OrEmitter((C.c_float * 3)(*emitter.origin), emitter.radius, emitter.nx, emitter.nz, emitter.speed,
                  emitter.jitter, emitter.seed, emitter.max_particles, emitter.enabled, 0)
    ov = C.c_int(0)
    k = lib().or_emit(C.byref(fs.f), C.byref(e), state.ctypes.data_as(C.POINTER(C.c_double)), C.c_float(dt),
                      C.c_float(last_dt), C.byref(ov))
    return int(k), bool(ov.value)


def velocity_handling(fs: FluidState, dt: float, last_dt: float, accel) -> None:
    lib().or_velocity_handling(C.byref(fs.f), C.c_float(dt), C.c_float(last_dt), (C.c_float * 3)(*accel))


def kernel_width_from_boundary_distance(fs: FluidState, settings: OrSettings) -> None:
    lib().or_kernel_width_from_boundary_distance(C.byref(fs.f), C.byref(settings))


def spread_kernel_width(fs: FluidState, settings: OrSettings) -> None:
    lib().or_spread_kernel_width(C.byref(fs.f), C.byref(fs.nb), C.byref(settings))


def update_transfers(fs: FluidState, settings: OrSettings, max_transfers: int = 10000) -> None:
    lib().or_update_transfers(C.byref(fs.f), C.byref(fs.nb), C.byref(fs.t), C.byref(settings), max_transfers)


def particle_transfer(fs: FluidState, dt: float) -> None:
    lib().or_particle_transfer(C.byref(fs.f), C.byref(fs.t), C.c_float(dt))


def density_error(fs: FluidState, settings: OrSettings) -> tuple[float, float]:
    out = (C.c_double * 2)()
    lib().or_density_error(C.byref(fs.f), C.byref(fs.nb), C.byref(settings), out)
    return out[0], out[1]


def reduce(fs: FluidState) -> np.ndarray:
    out = (C.c_double * 3)()
    lib().or_reduce(C.byref(fs.f), out)
    return np.array(list(out))


def substep(fs: FluidState, scene: OrScene, boxes: tuple, dt: float, cap_pairs: int) -> int:
    if fs.nb is None or fs.nb.cap < cap_pairs:
        fs.alloc_neighbors(cap_pairs)
    b, keep = _boxes(boxes)
    tot = lib().or_substep(C.byref(fs.f), C.byref(fs.t), C.byref(fs.nb), C.byref(b), C.byref(scene), C.c_float(dt))
    if tot > fs.nb.cap:
        raise RuntimeError(f"oracle neighbour capacity {fs.nb.cap} < {tot}")
    return int(tot)


def make_scene(settings: OrSettings, minp, maxp, log2res: int, accel, max_transfers: int = 10000,
               search_method: int = 1) -> OrScene:
    sc = OrScene()
    sc.search_method = search_method
    sc.settings = settings
    sc.minp = (C.c_float * 3)(*minp)
    sc.maxp = (C.c_float * 3)(*maxp)
    sc.log2res = log2res
    sc.accel = (C.c_float * 3)(*accel)
    sc.last_dt = 1.0
    sc.max_transfers = max_transfers
    return sc
