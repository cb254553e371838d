"""Host-side mirror of the reference's stage objects over the C ABI.

The reference's scene code (source/pool.cpp) owns lists and stage objects and
calls, once per frame:

    mVelocityHandling.apply(dt); mParticleTransfer.apply(dt);
    mNeighborhoodFluid.set_range_scale(s).apply(); mSpreadKernelWidth.apply();
    for i < solverIterations: mBoxCollision.apply(); mIncompressibility.apply();
    mUpdateTransfers.apply();

This module offers the same objects with the same method names
(set_data / set_range_scale / set_position_range / apply), backed by one
apbf_ctx that owns the device lists (the reference's gpu_list / indexed_list
buffers).  Device memory is handed out as torch tensors that alias the
context's buffers (valid until the next call that edits the lists, like
gpu_list::buffer()).  torch is used only for device memory and streams.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N

_TYPESTR = {torch.int32: "<i4", torch.float32: "<f4", torch.int64: "<i8", torch.uint8: "|u1"}


class _CudaArray:
    def __init__(self, ptr: int, shape: tuple, typestr: str):
        self.__cuda_array_interface__ = {
            "shape": shape,
            "typestr": typestr,
            "data": (int(ptr), False),
            "version": 2,
            "strides": None,
        }


def device_tensor(ptr: int, shape: tuple, dtype: torch.dtype, device: int = 0) -> torch.Tensor:
    """A torch tensor aliasing device memory owned by the context (no copy)."""
    if not ptr:
        raise ValueError("null device pointer")
    return torch.as_tensor(_CudaArray(ptr, tuple(shape), _TYPESTR[dtype]), device=f"cuda:{device}")


def _stream_handle(stream) -> C.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def default_settings() -> N.Settings:
    s = N.Settings()
    N.load().apbf_default_settings(C.byref(s))
    return s


FLUID_FIELDS = {
    # name: (dtype, components)
    "position": (torch.int32, 4),
    "velocity": (torch.float32, 4),
    "inverse_mass": (torch.float32, 1),
    "radius": (torch.float32, 1),
    "pos_backup": (torch.int32, 4),
    "transferring": (torch.int32, 1),
    "target_radius": (torch.float32, 1),
    "kernel_width": (torch.float32, 1),
    "boundariness": (torch.float32, 1),
    "boundary_distance": (torch.int32, 1),
}


@dataclass
class CallerLists:
    """Device lists owned by the caller (torch tensors), for Context.bind_lists: two
    buffer sets of the particle lists and of the transfer list, one length word per
    list, and the neighbour rows (column-major, row_stride as the context reports)."""

    capacity: int
    transfer_capacity: int
    row_stride: int
    max_neighbors: int
    device: int = 0

    def __post_init__(self):
        dev = f"cuda:{self.device}"
        self.fluid = [{name: torch.zeros((self.capacity, comps) if comps > 1 else (self.capacity,), dtype=dt,
                                         device=dev) for name, (dt, comps) in FLUID_FIELDS.items()} for _ in range(2)]
        self.transfers = [{"source": torch.zeros(self.transfer_capacity, dtype=torch.int32, device=dev),
                           "target": torch.zeros(self.transfer_capacity, dtype=torch.int32, device=dev),
                           "time_left": torch.zeros(self.transfer_capacity, dtype=torch.float32, device=dev)}
                          for _ in range(2)]
        self.len_particles = torch.zeros(1, dtype=torch.int32, device=dev)
        self.len_transfers = torch.zeros(1, dtype=torch.int32, device=dev)
        self.count = torch.zeros(self.capacity, dtype=torch.int32, device=dev)
        self.index = torch.zeros((self.max_neighbors, self.row_stride), dtype=torch.int32, device=dev)

    @classmethod
    def for_context(cls, ctx: "Context") -> "CallerLists":
        return cls(ctx.capacity, ctx.transfer_capacity, ctx.neighbors_view()["row_stride"], ctx.max_neighbors,
                   ctx.device)


class Context:
    """One apbf_ctx: the device lists of one scene plus the solver's scratch memory."""

    def __init__(self, particle_capacity: int, max_neighbors: int = 96, transfer_capacity: int = N.MAX_TRANSFERS,
                 max_log2res: int = 7, device: int = 0):
        self.lib = N.load()
        self.device = device
        torch.cuda.init()
        cfg = N.Config(particle_capacity, max_neighbors, transfer_capacity, max_log2res, device)
        h = C.c_void_p()
        N.check(self.lib.apbf_create(C.byref(cfg), C.byref(h)), "apbf_create")
        self.handle = h
        self.capacity = particle_capacity
        self.max_neighbors = max_neighbors
        self.transfer_capacity = transfer_capacity
        self.settings = default_settings()

    # ---- lifetime ----
    def close(self) -> None:
        if getattr(self, "handle", None):
            torch.cuda.synchronize(self.device)
            self.lib.apbf_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- configuration ----
    def set_settings(self, settings: N.Settings | None = None, **kw) -> "Context":
        s = settings if settings is not None else self.settings
        for k, v in kw.items():
            if not hasattr(s, k):
                raise AttributeError(k)
            setattr(s, k, v)
        N.check(self.lib.apbf_set_settings(self.handle, C.byref(s)), "apbf_set_settings")
        self.settings = s
        return self

    def set_scene(self, min_pos, max_pos, log2res: int, acceleration=(0.0, 0.0, 0.0)) -> "Context":
        sc = N.Scene(N.f3(min_pos), N.f3(max_pos), log2res, N.f3(acceleration))
        N.check(self.lib.apbf_set_scene(self.handle, C.byref(sc)), "apbf_set_scene")
        self.scene = (tuple(min_pos), tuple(max_pos), log2res, tuple(acceleration))
        return self

    def set_boxes(self, box_min: np.ndarray, box_max: np.ndarray) -> "Context":
        bmin = np.ascontiguousarray(box_min, dtype=np.float32).reshape(-1, 4)
        bmax = np.ascontiguousarray(box_max, dtype=np.float32).reshape(-1, 4)
        n = bmin.shape[0]
        N.check(self.lib.apbf_set_boxes(self.handle, bmin.ctypes.data_as(N._F3), bmax.ctypes.data_as(N._F3), n),
                "apbf_set_boxes")
        return self

    def load_scene(self, spec) -> "Context":
        """Scene range, boxes (axis-aligned and oriented), emitter and particle state of a
        scenes.SceneSpec."""
        self.set_scene(spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration)
        self.set_boxes(spec.box_min, spec.box_max)
        if spec.meta.get("oriented_boxes") is not None:
            self.set_oriented_boxes(*spec.meta["oriented_boxes"])
        if spec.meta.get("emitter"):
            self.set_emitter(**spec.meta["emitter"])
        self.upload(spec.state)
        return self

    def set_oriented_boxes(self, center: np.ndarray, half: np.ndarray, quat: np.ndarray) -> "Context":
        """Oriented boxes after the axis-aligned ones (centre, half extents, quaternion x y z w)."""
        c = np.ascontiguousarray(center, dtype=np.float32).reshape(-1, 4)
        h = np.ascontiguousarray(half, dtype=np.float32).reshape(-1, 4)
        q = np.ascontiguousarray(quat, dtype=np.float32).reshape(-1, 4)
        N.check(self.lib.apbf_set_oriented_boxes(self.handle, c.ctypes.data_as(N._F3), h.ctypes.data_as(N._F3),
                                                 q.ctypes.data_as(N._F3), c.shape[0]), "apbf_set_oriented_boxes")
        return self

    def box_rotations(self, n: int) -> np.ndarray:
        """Rotation rows of the first n boxes as the device uses them (n x 3 x 4 floats)."""
        out = np.zeros((n, 3, 4), np.float32)
        N.check(self.lib.apbf_get_box_rotations(self.handle, out.ctypes.data_as(N._F3), n), "apbf_get_box_rotations")
        return out

    def set_emitter(self, origin, radius: float, nx: int, nz: int, speed: float, jitter: float = 0.2,
                    seed: int = 0, max_particles: int = 0, enabled: bool = True) -> "Context":
        e = N.Emitter((C.c_float * 3)(*origin), radius, nx, nz, speed, jitter, seed, max_particles,
                      1 if enabled else 0, 0)
        N.check(self.lib.apbf_set_emitter(self.handle, C.byref(e)), "apbf_set_emitter")
        self.emitter = e
        return self

    def save_particle_info(self, folder: str, center=(0.0, 10.0, -60.0), stream=None) -> None:
        """save_particle_info::apply: the reference's particle-info text files in `folder`."""
        N.check(self.lib.apbf_save_particle_info(self.handle, str(folder).encode(), (C.c_float * 3)(*center),
                                                 _stream_handle(stream)), "apbf_save_particle_info")

    def bind_lists(self, lists: "CallerLists") -> None:
        """apbf_bind_lists: the stages run on the caller's device lists from now on."""
        fv = (N.FluidView * 2)()
        tv = (N.TransfersView * 2)()
        for k in range(2):
            f, t = lists.fluid[k], lists.transfers[k]
            fv[k] = N.FluidView(lists.capacity, lists.len_particles.data_ptr(),
                                *[f[name].data_ptr() for name in FLUID_FIELDS])
            tv[k] = N.TransfersView(lists.transfer_capacity, lists.len_transfers.data_ptr(), t["source"].data_ptr(),
                                    t["target"].data_ptr(), t["time_left"].data_ptr())
        nv = N.NeighborsView(lists.row_stride, lists.max_neighbors, lists.count.data_ptr(), lists.index.data_ptr(),
                             None)
        N.check(self.lib.apbf_bind_lists(self.handle, fv, tv, C.byref(nv)), "apbf_bind_lists")
        self.bound = lists

    def unbind_lists(self) -> None:
        N.check(self.lib.apbf_unbind_lists(self.handle), "apbf_unbind_lists")
        self.bound = None

    def set_wait_limit(self, limit: int = 0, inject: bool = False) -> None:
        """apbf_set_wait_limit: spins of the device-side waits before they give up (0:
        defaults); inject makes every wait run out (failure-path tests)."""
        N.check(self.lib.apbf_set_wait_limit(self.handle, limit, 1 if inject else 0), "apbf_set_wait_limit")

    def set_debug(self, enable: bool) -> None:
        N.check(self.lib.apbf_set_debug(self.handle, 1 if enable else 0), "apbf_set_debug")

    def tuning(self) -> dict:
        t = N.Tuning()
        N.check(self.lib.apbf_get_tuning(self.handle, C.byref(t)), "apbf_get_tuning")
        return {"gather_lanes": t.gather_lanes, "pass_block": t.pass_block,
                "pass_blocks_per_sm": t.pass_blocks_per_sm,
                "filter_in_density": t.filter_in_density, "sort_digit_bits": t.sort_digit_bits,
                "search_log2res": t.search_log2res}

    def set_neighborhood_search(self, method: int | str) -> None:
        """The neighbour search of substep(): "green" (the default) or "binary_search",
        or the NEIGHBORHOOD_TYPE number (shaders/cpu_gpu_shared_config.h:5)."""
        m = {"green": N.NEIGHBORHOOD_GREEN, "binary_search": N.NEIGHBORHOOD_BINARY_SEARCH}.get(method, method)
        N.check(self.lib.apbf_set_neighborhood_search(self.handle, int(m)), "apbf_set_neighborhood_search")

    def position_codes(self, index_list: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """calculate_position_code for the three code sections: (n, 3) uint32 words of
        the 96-bit code of every particle (of index_list[k] when given), least
        significant word first."""
        n, _ = self.lengths()
        dev = f"cuda:{self.device}"
        out = torch.zeros((3, max(n, 1)), dtype=torch.int32, device=dev)
        idx = None
        if index_list is not None:
            idx = index_list.to(device=dev, dtype=torch.int32).contiguous()
        for w in range(3):
            N.check(self.lib.apbf_calculate_position_code(self.handle, idx.data_ptr() if idx is not None else None, w,
                                                          out[w].data_ptr(), _stream_handle(stream)),
                    "apbf_calculate_position_code")
        torch.cuda.synchronize(self.device)
        return out[:, :n].t().contiguous()

    def set_tuning(self, gather_lanes: int | None = None, pass_block: int | None = None,
                   pass_blocks_per_sm: int | None = None,
                   filter_in_density: int | None = None, sort_digit_bits: int | None = None,
                   search_log2res: int | None = None) -> None:
        t = N.Tuning()
        N.check(self.lib.apbf_get_tuning(self.handle, C.byref(t)), "apbf_get_tuning")
        if gather_lanes is not None:
            t.gather_lanes = gather_lanes
        if pass_block is not None:
            t.pass_block = pass_block
        if pass_blocks_per_sm is not None:
            t.pass_blocks_per_sm = pass_blocks_per_sm
        if filter_in_density is not None:
            t.filter_in_density = filter_in_density
        if sort_digit_bits is not None:
            t.sort_digit_bits = sort_digit_bits
        if search_log2res is not None:
            t.search_log2res = search_log2res
        N.check(self.lib.apbf_set_tuning(self.handle, C.byref(t)), "apbf_set_tuning")

    def autotune(self, stream=None) -> dict:
        """Times every launch-shape candidate on the current state (restored afterwards)
        and keeps the fastest; returns the choice and the per-pass times (ms)."""
        t = N.Tuning()
        ms = (C.c_float * 24)()
        N.check(self.lib.apbf_autotune(self.handle, _stream_handle(stream), C.byref(t), ms), "apbf_autotune")
        keys = [f"L{l}/B{b}/S{p}" for l in (1, 2, 4, 8) for b in (128, 256) for p in (2, 4, 8)]
        return {"gather_lanes": t.gather_lanes, "pass_block": t.pass_block,
                "pass_blocks_per_sm": t.pass_blocks_per_sm,
                "filter_in_density": t.filter_in_density, "sort_digit_bits": t.sort_digit_bits,
                "search_log2res": t.search_log2res,
                "pass_ms": {k: round(float(v), 5) for k, v in zip(keys, ms)}}

    def autotune_search(self, stream=None) -> dict:
        """apbf_autotune_search: the sort digit width and the search grid of substep()
        from timed candidates (state restored); returns the choice and the times (ms)."""
        t = N.Tuning()
        ms = (C.c_float * 6)()
        N.check(self.lib.apbf_autotune_search(self.handle, _stream_handle(stream), C.byref(t), ms),
                "apbf_autotune_search")
        return {"sort_digit_bits": t.sort_digit_bits, "search_log2res": t.search_log2res,
                "sort_ms": {f"{b} bits": round(float(ms[i]), 5) for i, b in enumerate((6, 7, 8))},
                "search_ms": {f"L{d:+d}": round(float(ms[3 + i]), 5) for i, d in enumerate((-1, 0, 1))}}

    def set_solve_graph(self, mode: int | bool) -> None:
        """0: per-kernel launches; 1 (default): the Jacobi passes 1.. as one graph launch with a
        device-side loop; 2: the whole substep as one graph launch."""
        N.check(self.lib.apbf_set_solve_graph(self.handle, int(mode)), "apbf_set_solve_graph")

    def set_persistent_solve(self, enable: bool = True) -> None:
        """Jacobi passes 1.. of a substep as one persistent cooperative kernel (same
        results; used where it applies, see apbf_set_persistent_solve)."""
        N.check(self.lib.apbf_set_persistent_solve(self.handle, 1 if enable else 0), "apbf_set_persistent_solve")

    # ---- lists ----
    def fluid_view(self) -> dict:
        v = N.FluidView()
        N.check(self.lib.apbf_fluid_get_view(self.handle, C.byref(v)), "apbf_fluid_get_view")
        out = {}
        for name, (dt, comp) in FLUID_FIELDS.items():
            shape = (v.capacity, comp) if comp > 1 else (v.capacity,)
            out[name] = device_tensor(getattr(v, name), shape, dt, self.device)
        out["length"] = device_tensor(v.d_length, (1,), torch.int32, self.device)
        return out

    def transfers_view(self) -> dict:
        v = N.TransfersView()
        N.check(self.lib.apbf_transfers_get_view(self.handle, C.byref(v)), "apbf_transfers_get_view")
        return {
            "source": device_tensor(v.source, (v.capacity,), torch.int32, self.device),
            "target": device_tensor(v.target, (v.capacity,), torch.int32, self.device),
            "time_left": device_tensor(v.time_left, (v.capacity,), torch.float32, self.device),
            "length": device_tensor(v.d_length, (1,), torch.int32, self.device),
        }

    def neighbors_view(self) -> dict:
        v = N.NeighborsView()
        N.check(self.lib.apbf_neighbors_get_view(self.handle, C.byref(v)), "apbf_neighbors_get_view")
        return {
            "count": device_tensor(v.count, (self.capacity,), torch.int32, self.device),
            "index": device_tensor(v.index, (v.max_per_row, v.row_stride), torch.int32, self.device),
            "row_stride": v.row_stride,
        }

    def reverse_neighbors_view(self, stream=None) -> dict:
        """The rows the position update gathers over (apbf_neighbors_get_reverse_view):
        kind 2 symmetric (the forward rows serve), 1 union rows, 0 transposed rows."""
        v = N.NeighborsView()
        kind = C.c_uint32()
        N.check(self.lib.apbf_neighbors_get_reverse_view(self.handle, C.byref(v), C.byref(kind),
                                                         _stream_handle(stream)), "apbf_neighbors_get_reverse_view")
        return {
            "count": device_tensor(v.count, (self.capacity,), torch.int32, self.device),
            "index": device_tensor(v.index, (v.max_per_row, v.row_stride), torch.int32, self.device),
            "row_stride": v.row_stride, "kind": int(kind.value),
        }

    def set_lengths(self, n_particles: int, n_transfers: int = 0, stream=None) -> None:
        N.check(self.lib.apbf_set_lengths(self.handle, n_particles, n_transfers, _stream_handle(stream)),
                "apbf_set_lengths")

    def lengths(self, stream=None) -> tuple[int, int]:
        a, b = C.c_uint32(), C.c_uint32()
        N.check(self.lib.apbf_get_lengths(self.handle, C.byref(a), C.byref(b), _stream_handle(stream)),
                "apbf_get_lengths")
        return a.value, b.value

    def upload(self, state: dict, transfers: dict | None = None, stream=None) -> None:
        """Copies a host scene state (numpy arrays, see scenes.py) into the lists."""
        n = int(state["position"].shape[0])
        if n > self.capacity:
            raise ValueError(f"{n} particles exceed the capacity {self.capacity}")
        v = self.fluid_view()
        for name, (dt, comp) in FLUID_FIELDS.items():
            if name not in state:
                continue
            src = torch.from_numpy(np.ascontiguousarray(state[name]).view(
                np.int32 if dt == torch.int32 else np.float32))
            v[name][:n].copy_(src.reshape(v[name][:n].shape), non_blocking=False)
        nt = 0
        if transfers is not None:
            nt = int(transfers["source"].shape[0])
            tv = self.transfers_view()
            for k in ("source", "target"):
                tv[k][:nt].copy_(torch.from_numpy(np.ascontiguousarray(transfers[k]).view(np.int32)))
            tv["time_left"][:nt].copy_(torch.from_numpy(np.ascontiguousarray(transfers["time_left"], np.float32)))
        torch.cuda.synchronize(self.device)
        self.set_lengths(n, nt, stream)

    @staticmethod
    def _host_fluid(host: dict) -> N.HostFluid:
        hf = N.HostFluid()
        for name, _ in N.HostFluid._fields_:
            a = host.get(name)
            if a is None:
                continue
            if isinstance(a, torch.Tensor):
                if a.is_cuda or not a.is_contiguous():
                    raise ValueError(f"{name}: a contiguous host tensor is needed")
                setattr(hf, name, a.data_ptr())
            else:
                if not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"{name}: a C-contiguous array is needed")
                setattr(hf, name, a.ctypes.data)
        return hf

    def fluid_write(self, host: dict, count: int, stream=None) -> None:
        """apbf_fluid_write: `count` particles from host arrays (the FLUID_FIELDS layout,
        plus an optional 'lambda_prev'; numpy arrays or host tensors, pinned for
        asynchronous copies) into the lists, and the particle length; absent fields keep
        their device values.  Stream-ordered: keep the arrays alive until it has run."""
        hf = self._host_fluid(host)
        N.check(self.lib.apbf_fluid_write(self.handle, C.byref(hf), int(count), _stream_handle(stream)),
                "apbf_fluid_write")

    def fluid_read(self, host: dict, max_count: int, count_out, stream=None) -> None:
        """apbf_fluid_read: enqueues the copy of the particle length into count_out (a
        one-element int32 host tensor) and of up to max_count particles into the given
        host arrays.  Valid after the stream is synchronised."""
        hf = self._host_fluid(host)
        N.check(self.lib.apbf_fluid_read(self.handle, C.byref(hf), int(max_count), C.c_void_p(count_out.data_ptr()),
                                         _stream_handle(stream)), "apbf_fluid_read")

    def download(self, stream=None) -> tuple[dict, dict]:
        """Host copy of the current lists (numpy), lengths applied."""
        n, nt = self.lengths(stream)
        v = self.fluid_view()
        out = {}
        for name, (dt, comp) in FLUID_FIELDS.items():
            a = v[name][:n].cpu().numpy()
            if name in ("transferring", "boundary_distance"):
                a = a.view(np.uint32)
            out[name] = a.copy()
            if name in ("position", "pos_backup"):
                out[name][:, 3] = 0  # w is the library's scratch lane, not particle state
        tv = self.transfers_view()
        tr = {
            "source": tv["source"][:nt].cpu().numpy().view(np.uint32).copy(),
            "target": tv["target"][:nt].cpu().numpy().view(np.uint32).copy(),
            "time_left": tv["time_left"][:nt].cpu().numpy().copy(),
        }
        return out, tr

    def download_rows(self, stream=None) -> list[np.ndarray]:
        """Neighbour rows of the last search as sorted numpy arrays (test helper)."""
        n, _ = self.lengths(stream)
        nb = self.neighbors_view()
        cnt = nb["count"][:n].cpu().numpy()
        idx = nb["index"][:, :n].cpu().numpy()
        return [np.sort(idx[: cnt[i], i].astype(np.int64)) for i in range(n)]

    # ---- results ----
    def status(self, clear: bool = True, stream=None) -> N.StatusInfo:
        info = N.StatusInfo()
        self.last_status_code = self.lib.apbf_get_status(self.handle, C.byref(info), 1 if clear else 0,
                                                         _stream_handle(stream))
        return info

    def check_status(self, stream=None) -> N.StatusInfo:
        info = N.StatusInfo()
        code = self.lib.apbf_get_status(self.handle, C.byref(info), 1, _stream_handle(stream))
        N.check(code, f"device status (flags=0x{info.flags:x}, required_neighbors={info.required_neighbors})")
        return info

    def reduce_fp64(self, stream=None) -> np.ndarray:
        out = (C.c_double * 4)()
        N.check(self.lib.apbf_reduce_fp64(self.handle, out, _stream_handle(stream)), "apbf_reduce_fp64")
        return np.array(list(out))

    def profile_enable(self, enable: bool = True, capacity: int = 65536) -> None:
        N.check(self.lib.apbf_profile_enable(self.handle, 1 if enable else 0, capacity), "apbf_profile_enable")

    def profile_read(self, stream=None) -> tuple[dict, int]:
        """{kernel name: (launches, total ms)} of the launches since the last read."""
        cap = 64
        arr = (N.KernelTime * cap)()
        n = C.c_uint32()
        dropped = C.c_ulonglong()
        N.check(self.lib.apbf_profile_read(self.handle, arr, cap, C.byref(n), C.byref(dropped),
                                           _stream_handle(stream)), "apbf_profile_read")
        return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms) for i in range(n.value)}, dropped.value

    def launch_count(self) -> int:
        v = C.c_ulonglong()
        N.check(self.lib.apbf_launch_count(self.handle, C.byref(v)), "apbf_launch_count")
        return v.value

    def substep(self, dt: float, stream=None) -> None:
        N.check(self.lib.apbf_substep(self.handle, C.c_float(dt), _stream_handle(stream)), "apbf_substep")

    # ---- learned warm start (no reference counterpart) ----
    def mlp_load(self, params: torch.Tensor, stream=None) -> None:
        """Copies a device parameter vector (apbf_mlp_param_count() floats) into the context."""
        if params.dtype != torch.float32 or not params.is_cuda or params.numel() != N.MLP_PARAMS:
            raise ValueError("params must be a CUDA float32 tensor of %d floats" % N.MLP_PARAMS)
        N.check(self.lib.apbf_mlp_load(self.handle, C.c_void_p(params.data_ptr()), _stream_handle(stream)),
                "apbf_mlp_load")

    def set_warm_start(self, mode: int | bool) -> None:
        """N.WARM_LEARNED | N.WARM_PROJECTED bits (True = both); 0 / False = the reference's solve."""
        m = (N.WARM_LEARNED | N.WARM_PROJECTED) if mode is True else int(mode)
        N.check(self.lib.apbf_set_warm_start(self.handle, m), "apbf_set_warm_start")

    def record_samples(self, iterations: int, features: torch.Tensor, targets: torch.Tensor,
                       count: torch.Tensor) -> None:
        """Arms the next substep to append (features, sum of min(0, lambda) over its first
        `iterations` plain iterations) of every particle to the device buffers."""
        cap = targets.numel()
        if features.numel() < cap * 8 or count.dtype != torch.int32:
            raise ValueError("features needs 8 floats per sample and count one int32")
        N.check(self.lib.apbf_record_samples(self.handle, iterations, C.c_void_p(features.data_ptr()),
                                             C.c_void_p(targets.data_ptr()), cap, C.c_void_p(count.data_ptr())),
                "apbf_record_samples")

    def debug_incompressibility(self, stream=None) -> dict:
        n, _ = self.lengths(stream)
        d = torch.empty(self.capacity, dtype=torch.int32, device=f"cuda:{self.device}")
        g = torch.empty((self.capacity, 4), dtype=torch.int32, device=f"cuda:{self.device}")
        q = torch.empty(self.capacity, dtype=torch.int32, device=f"cuda:{self.device}")
        lam = torch.empty(self.capacity, dtype=torch.float32, device=f"cuda:{self.device}")
        N.check(self.lib.apbf_debug_incompressibility(self.handle, C.c_void_p(d.data_ptr()), C.c_void_p(g.data_ptr()),
                                                      C.c_void_p(q.data_ptr()), C.c_void_p(lam.data_ptr()),
                                                      _stream_handle(stream)), "apbf_debug_incompressibility")
        torch.cuda.synchronize(self.device)
        return {
            "density": d[:n].cpu().numpy().view(np.uint32),
            "grad_sum": g[:n, :3].cpu().numpy(),
            "sq_grad_sum": q[:n].cpu().numpy().view(np.uint32),
            "lambda": lam[:n].cpu().numpy(),
        }

    def debug_sort(self, stream=None) -> tuple[np.ndarray, np.ndarray]:
        n, _ = self.lengths(stream)
        p = torch.empty(self.capacity, dtype=torch.int32, device=f"cuda:{self.device}")
        k = torch.empty(self.capacity, dtype=torch.int32, device=f"cuda:{self.device}")
        N.check(self.lib.apbf_debug_sort(self.handle, C.c_void_p(p.data_ptr()), C.c_void_p(k.data_ptr()),
                                         _stream_handle(stream)), "apbf_debug_sort")
        torch.cuda.synchronize(self.device)
        return p[:n].cpu().numpy().view(np.uint32), k[:n].cpu().numpy().view(np.uint32)

    def export_pairs(self, capacity: int, stream=None) -> np.ndarray:
        pairs = torch.empty((capacity, 2), dtype=torch.int32, device=f"cuda:{self.device}")
        ln = torch.zeros(1, dtype=torch.int32, device=f"cuda:{self.device}")
        N.check(self.lib.apbf_export_pairs(self.handle, C.c_void_p(pairs.data_ptr()), capacity,
                                           C.c_void_p(ln.data_ptr()), _stream_handle(stream)), "apbf_export_pairs")
        torch.cuda.synchronize(self.device)
        m = min(int(ln.item()), capacity)
        return pairs[:m].cpu().numpy().view(np.uint32)


# ---------------------------------------------------------------------------
# Stage objects with the reference's method names.
# ---------------------------------------------------------------------------


class velocity_handling:
    """pbd::velocity_handling (source/velocity_handling.h, velocity_handling.cpp:15-31)."""

    def set_data(self, ctx: Context) -> "velocity_handling":
        self.ctx = ctx
        return self

    def set_acceleration(self, a) -> "velocity_handling":
        self.acc = N.f3(a)
        return self

    def apply(self, dt: float, stream=None) -> None:
        N.check(self.ctx.lib.apbf_velocity_handling_apply(self.ctx.handle, C.c_float(dt), self.acc,
                                                          _stream_handle(stream)), "velocity_handling.apply")


class neighborhood_green:
    """pbd::neighborhood_green (source/neighborhood_green.h:8-23)."""

    def __init__(self):
        self.range_scale = 1.0

    def set_data(self, ctx: Context) -> "neighborhood_green":
        self.ctx = ctx
        return self

    def set_range_scale(self, scale: float) -> "neighborhood_green":
        self.range_scale = float(scale)
        return self

    def set_position_range(self, min_pos, max_pos, resolution_log2: int) -> "neighborhood_green":
        self.min_pos, self.max_pos, self.log2res = N.f3(min_pos), N.f3(max_pos), int(resolution_log2)
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_neighborhood_green_apply(self.ctx.handle, C.c_float(self.range_scale), self.min_pos,
                                                           self.max_pos, self.log2res, _stream_handle(stream)),
                "neighborhood_green.apply")


class neighborhood_binary_search:
    """pbd::neighborhood_binary_search (source/neighborhood_binary_search.h:8-21)."""

    def __init__(self):
        self.range_scale = 1.0

    def set_data(self, ctx: Context) -> "neighborhood_binary_search":
        self.ctx = ctx
        return self

    def set_range_scale(self, scale: float) -> "neighborhood_binary_search":
        self.range_scale = float(scale)
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_neighborhood_binary_search_apply(self.ctx.handle, C.c_float(self.range_scale),
                                                                   _stream_handle(stream)),
                "neighborhood_binary_search.apply")


class box_collision:
    """pbd::box_collision (source/box_collision.h, box_collision.cpp:12-24)."""

    def set_data(self, ctx: Context, box_min=None, box_max=None) -> "box_collision":
        self.ctx = ctx
        if box_min is not None:
            ctx.set_boxes(box_min, box_max)
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_box_collision_apply(self.ctx.handle, _stream_handle(stream)), "box_collision.apply")


class incompressibility:
    """pbd::incompressibility (source/incompressibility.h:7-17)."""

    def set_data(self, ctx: Context) -> "incompressibility":
        self.ctx = ctx
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_incompressibility_apply(self.ctx.handle, _stream_handle(stream)),
                "incompressibility.apply")


class spread_kernel_width:
    """pbd::spread_kernel_width (source/spread_kernel_width.h, spread_kernel_width.cpp:12-26)."""

    def set_data(self, ctx: Context) -> "spread_kernel_width":
        self.ctx = ctx
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_spread_kernel_width_apply(self.ctx.handle, _stream_handle(stream)),
                "spread_kernel_width.apply")


class kernel_width_from_boundary_distance:
    """shader_provider::uint_to_float_with_indexed_lower_bound as called at source/pool.cpp:77-80."""

    def set_data(self, ctx: Context) -> "kernel_width_from_boundary_distance":
        self.ctx = ctx
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_kernel_width_from_boundary_distance_apply(self.ctx.handle, _stream_handle(stream)),
                "kernel_width_from_boundary_distance.apply")


class update_transfers:
    """pbd::update_transfers (source/update_transfers.h, update_transfers.cpp:14-71)."""

    def set_data(self, ctx: Context) -> "update_transfers":
        self.ctx = ctx
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_update_transfers_apply(self.ctx.handle, _stream_handle(stream)),
                "update_transfers.apply")


class particle_transfer:
    """pbd::particle_transfer (source/particle_transfer.h, particle_transfer.cpp:10-28)."""

    def set_data(self, ctx: Context) -> "particle_transfer":
        self.ctx = ctx
        return self

    def apply(self, dt: float, stream=None) -> None:
        N.check(self.ctx.lib.apbf_particle_transfer_apply(self.ctx.handle, C.c_float(dt), _stream_handle(stream)),
                "particle_transfer.apply")


class lists:
    """The list-edit services (gpu_list / indexed_list, source/gpu_list.h, indexed_list.h) on
    device tensors of 32-bit words with device lengths."""

    @staticmethod
    def _u32(n: int, device: int) -> torch.Tensor:
        return torch.zeros(max(n, 1), dtype=torch.int32, device=f"cuda:{device}")

    @staticmethod
    def apply_edit(src: torch.Tensor, edit: torch.Tensor, edit_len: torch.Tensor | None = None,
                   stride_words: int = 1, stream=None) -> torch.Tensor:
        """gpu_list::apply_edit: dst[k] = src[edit[k]] (elements of stride_words words)."""
        lib = N.load()
        m = edit.numel()
        dst = torch.zeros(max(m * stride_words, 1), dtype=src.dtype, device=src.device)
        N.check(lib.apbf_list_apply_edit(C.c_void_p(src.data_ptr()), stride_words, C.c_void_p(edit.data_ptr()),
                                         C.c_void_p(edit_len.data_ptr() if edit_len is not None else 0), m,
                                         C.c_void_p(dst.data_ptr()), _stream_handle(stream)), "lists.apply_edit")
        return dst[:m * stride_words]

    @staticmethod
    def delete_edit(ctx: "Context", deleted: torch.Tensor, n_hidden: int, stream=None) -> torch.Tensor:
        """indexed_list::delete_these: the edit list of the surviving hidden ids."""
        d_len = torch.tensor([deleted.numel()], dtype=torch.int32, device=deleted.device)
        edit = lists._u32(n_hidden, ctx.device)
        e_len = lists._u32(1, ctx.device)
        N.check(ctx.lib.apbf_list_delete_edit(ctx.handle, C.c_void_p(deleted.data_ptr()), C.c_void_p(d_len.data_ptr()),
                                              deleted.numel(), n_hidden, C.c_void_p(edit.data_ptr()),
                                              C.c_void_p(e_len.data_ptr()), _stream_handle(stream)),
                "lists.delete_edit")
        return edit[:int(e_len.item())]

    @staticmethod
    def remap_index(ctx: "Context", index_list: torch.Tensor, edit: torch.Tensor, n_hidden_old: int,
                    out_cap: int | None = None, stream=None) -> tuple[torch.Tensor, torch.Tensor, int]:
        """indexed_list::apply_hidden_edit: (new index list, old position of each entry, full count)."""
        dev = ctx.device
        l_len = torch.tensor([index_list.numel()], dtype=torch.int32, device=f"cuda:{dev}")
        e_len = torch.tensor([edit.numel()], dtype=torch.int32, device=f"cuda:{dev}")
        cap = out_cap if out_cap is not None else max(1, 4 * index_list.numel() + edit.numel())
        out, new_edit = lists._u32(cap, dev), lists._u32(cap, dev)
        o_len, req = lists._u32(1, dev), lists._u32(1, dev)
        lst = index_list if index_list.numel() else lists._u32(1, dev)
        ed = edit if edit.numel() else lists._u32(1, dev)
        N.check(ctx.lib.apbf_list_remap_index(ctx.handle, C.c_void_p(lst.data_ptr()), C.c_void_p(l_len.data_ptr()),
                                              index_list.numel(), C.c_void_p(ed.data_ptr()),
                                              C.c_void_p(e_len.data_ptr()), edit.numel(), n_hidden_old,
                                              C.c_void_p(out.data_ptr()), C.c_void_p(new_edit.data_ptr()), cap,
                                              C.c_void_p(o_len.data_ptr()), C.c_void_p(req.data_ptr()),
                                              _stream_handle(stream)), "lists.remap_index")
        m = int(o_len.item())
        return out[:m], new_edit[:m], int(req.item())

    @staticmethod
    def append(dst: torch.Tensor, dst_len: torch.Tensor, src: torch.Tensor, src_len: torch.Tensor,
               stride_words: int = 1, stream=None) -> None:
        """gpu_list::operator+=: appends src after the dst_len elements of dst (capacity: dst's size)."""
        lib = N.load()
        scratch = torch.zeros(1, dtype=torch.int32, device=dst.device)
        N.check(lib.apbf_list_append(C.c_void_p(dst.data_ptr()), C.c_void_p(dst_len.data_ptr()),
                                     dst.numel() // stride_words, C.c_void_p(src.data_ptr()),
                                     C.c_void_p(src_len.data_ptr()), src.numel() // stride_words, stride_words,
                                     C.c_void_p(scratch.data_ptr()), _stream_handle(stream)), "lists.append")
        torch.cuda.current_stream().synchronize()


class sphere_collision:
    """pbd::sphere_collision (source/sphere_collision.h)."""

    def set_data(self, ctx: Context) -> "sphere_collision":
        self.ctx = ctx
        return self

    def set_sphere(self, center, radius: float, hollow: bool) -> "sphere_collision":
        self.center, self.radius, self.hollow = tuple(center), float(radius), bool(hollow)
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_sphere_collision_apply(self.ctx.handle, (C.c_float * 3)(*self.center),
                                                         C.c_float(self.radius), 1 if self.hollow else 0,
                                                         _stream_handle(stream)), "sphere_collision.apply")


class inter_particle_collision:
    """pbd::inter_particle_collision (source/inter_particle_collision.h)."""

    def set_data(self, ctx: Context) -> "inter_particle_collision":
        self.ctx = ctx
        return self

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_inter_particle_collision_apply(self.ctx.handle, _stream_handle(stream)),
                "inter_particle_collision.apply")


class glue:
    """pbd::glue (source/glue.h): applyNewGlue() builds the glue list, apply() enforces it."""

    def __init__(self):
        self.stability, self.elasticity, self.capacity = 1.0, 0.0, 1 << 20

    def set_data(self, ctx: Context, capacity: int = 1 << 20) -> "glue":
        self.ctx, self.capacity = ctx, capacity
        return self

    def set_stability(self, s: float) -> "glue":
        self.stability = float(s)
        return self

    def set_elasticity(self, e: float) -> "glue":
        self.elasticity = float(e)
        return self

    def applyNewGlue(self, stream=None) -> None:  # noqa: N802 (the reference's name)
        N.check(self.ctx.lib.apbf_glue_generate(self.ctx.handle, self.capacity, _stream_handle(stream)),
                "glue.applyNewGlue")

    def apply(self, stream=None) -> None:
        N.check(self.ctx.lib.apbf_glue_apply(self.ctx.handle, C.c_float(self.stability), C.c_float(self.elasticity),
                                             _stream_handle(stream)), "glue.apply")

    def view(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        p0, p1, d, ln = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        cap = C.c_uint32()
        N.check(self.ctx.lib.apbf_glue_get_view(self.ctx.handle, C.byref(p0), C.byref(p1), C.byref(d), C.byref(ln),
                                                C.byref(cap)), "apbf_glue_get_view")
        m = int(device_tensor(ln.value, (1,), torch.int32, self.ctx.device).item())
        out = []
        for ptr in (p0, p1, d):
            out.append(device_tensor(ptr.value, (cap.value,), torch.int32, self.ctx.device)[:m].cpu().numpy()
                       .view(np.uint32).copy())
        return tuple(out)


class algorithms:
    """pbd::algorithms (source/algorithms.h:12-17) on device tensors."""

    @staticmethod
    def sort(ctx: Context, keys: torch.Tensor, values: torch.Tensor, count: torch.Tensor, max_count: int,
             out_keys: torch.Tensor, out_values: torch.Tensor, value_upper_bound: int = 0xFFFFFFFF,
             stream=None) -> None:
        N.check(ctx.lib.apbf_sort_pairs(ctx.handle, C.c_void_p(keys.data_ptr()), C.c_void_p(values.data_ptr()),
                                        C.c_void_p(count.data_ptr()), max_count, value_upper_bound,
                                        C.c_void_p(out_keys.data_ptr()), C.c_void_p(out_values.data_ptr()),
                                        _stream_handle(stream)), "algorithms.sort")

    @staticmethod
    def prefix_sum(ctx: Context, values: torch.Tensor, count: torch.Tensor, max_count: int, stream=None) -> None:
        N.check(ctx.lib.apbf_prefix_sum(ctx.handle, C.c_void_p(values.data_ptr()), C.c_void_p(count.data_ptr()),
                                        max_count, _stream_handle(stream)), "algorithms.prefix_sum")


class Batch:
    """Independent scenes (contexts) advanced together: one graph launch per substep
    whose parallel branches are the contexts' substeps (optionally around one batched
    persistent solve of their Jacobi passes after the first)."""

    def __init__(self, contexts: list):
        self.contexts = list(contexts)
        self.lib = N.load()
        arr = (C.c_void_p * len(self.contexts))(*[c.handle.value for c in self.contexts])
        h = C.c_void_p()
        N.check(self.lib.apbf_batch_create(arr, len(self.contexts), C.byref(h)), "apbf_batch_create")
        self.handle = h

    def substep(self, dt: float, stream=None) -> None:
        N.check(self.lib.apbf_batch_substep(self.handle, C.c_float(dt), _stream_handle(stream)),
                "apbf_batch_substep")

    def set_persistent_solve(self, enable: bool = True) -> None:
        """True: the batched persistent solve; False (default): each scene's solve loop in its branch."""
        N.check(self.lib.apbf_batch_set_persistent_solve(self.handle, 1 if enable else 0),
                "apbf_batch_set_persistent_solve")

    def close(self) -> None:
        if getattr(self, "handle", None):
            torch.cuda.synchronize()
            self.lib.apbf_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class SubstepStages:
    """The stage objects of one scene, wired as pool::pool wires them (source/pool.cpp:27-46)."""

    ctx: Context

    def __post_init__(self):
        self.velocity = velocity_handling().set_data(self.ctx)
        self.neighborhood = neighborhood_green().set_data(self.ctx)
        self.boxes = box_collision().set_data(self.ctx)
        self.incompressibility = incompressibility().set_data(self.ctx)
        self.spread = spread_kernel_width().set_data(self.ctx)
        self.kw_bd = kernel_width_from_boundary_distance().set_data(self.ctx)
        self.update_transfers = update_transfers().set_data(self.ctx)
        self.particle_transfer = particle_transfer().set_data(self.ctx)

    def update(self, dt: float, stream=None) -> None:
        """One substep as pool::update runs it (source/pool.cpp:67-106), stage by stage:
        velocity handling; with adaptivity, particle transfer and the kernel width from the
        boundary distance (or its spreading after the search); the neighbourhood; then
        solver_iterations x (box collision, one incompressibility iteration); with
        adaptivity, update_transfers.  The scene's range, resolution and acceleration come
        from Context.set_scene.  apbf_substep runs the same stages with the box passes fused
        into the kernels before them and gives the same state (no emitter, no error
        target, no warm start)."""
        s = self.ctx.settings
        min_pos, max_pos, log2res, acc = self.ctx.scene
        adaptive = not s.basic_pbf
        self.velocity.set_acceleration(acc).apply(dt, stream)
        if adaptive and (s.merge or s.split):
            self.particle_transfer.apply(dt, stream)
        if adaptive and s.base_kernel_width_on_boundary_distance:
            self.kw_bd.apply(stream)
        scale = 1.0 if (s.basic_pbf or s.base_kernel_width_on_boundary_distance) else 1.5
        self.neighborhood.set_range_scale(scale).set_position_range(min_pos, max_pos, log2res).apply(stream)
        if adaptive and not s.base_kernel_width_on_boundary_distance:
            self.spread.apply(stream)
        for _ in range(s.solver_iterations):
            self.boxes.apply(stream)
            self.incompressibility.apply(stream)
        if adaptive:
            self.update_transfers.apply(stream)


# ---- save_particle_info files read back (host only) ----
PARTICLE_INFO_LISTS = ("centerDist", "radius", "neighborCount", "kernelWidth", "targetRadius", "boundaryDistance")
PARTICLE_INFO_COLUMNS = ("center distance", "boundary distance", "kernel width", "neighbor count", "radius",
                         "target radius", "inverse mass", "x", "y", "z")


def load_particle_info(folder) -> dict:
    """Reads the files of save_particle_info (source/save_particle_info.cpp:22-125, as
    Context.save_particle_info writes them): every ';'-separated list present, as
    float64 arrays in particle order (neighborCount as int64), and data.csv's columns
    (rows sorted by the distance to the centre) under "data"."""
    from pathlib import Path

    d = Path(folder)
    out: dict = {}
    for name in PARTICLE_INFO_LISTS:
        p = d / f"{name}.txt"
        if p.exists():
            vals = [x for x in p.read_text().split(";") if x.strip()]
            out[name] = np.array(vals, dtype=np.int64 if name == "neighborCount" else np.float64)
    p = d / "data.csv"
    if p.exists():
        lines = p.read_text().strip().splitlines()
        head = tuple(h.strip() for h in lines[0].split(","))
        if head != PARTICLE_INFO_COLUMNS:
            raise ValueError(f"{p}: unexpected columns {head}")
        rows = np.array([[float(x) for x in ln.split(",")] for ln in lines[1:]], np.float64).reshape(-1, len(head))
        out["data"] = {h: rows[:, k] for k, h in enumerate(head)}
    return out


def state_from_particle_info(folder) -> dict:
    """A particle state for Context.upload from a save_particle_info data.csv (in its row
    order): positions, radii, target radii, inverse masses, kernel widths and boundary
    distances as written (six significant digits), velocities zero, the backup
    position equal to the position, no transfers, boundariness zero."""
    cols = load_particle_info(folder)["data"]
    n = cols["x"].shape[0]
    pos = np.zeros((n, 4), np.int32)
    for k, a in enumerate(("x", "y", "z")):
        pos[:, k] = np.rint(cols[a] * 262144.0).astype(np.int32)
    f32 = lambda a: np.ascontiguousarray(cols[a], dtype=np.float32)  # noqa: E731
    return {
        "position": pos,
        "velocity": np.zeros((n, 4), np.float32),
        "inverse_mass": f32("inverse mass"),
        "radius": f32("radius"),
        "pos_backup": pos.copy(),
        "transferring": np.zeros(n, np.uint32),
        "target_radius": f32("target radius"),
        "kernel_width": f32("kernel width"),
        "boundariness": np.zeros(n, np.float32),
        "boundary_distance": np.rint(cols["boundary distance"] * 262144.0).astype(np.uint32),
    }
