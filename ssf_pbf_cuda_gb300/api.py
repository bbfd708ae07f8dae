"""Python mirror of the reference simulator's solver interface.

Names follow yodaplusplus/ssf_pbf_cuda (``pbf_particle``, ``pbf_boundary``,
``pbf::one_step``; src/pbf/pbf_type.h:74-100, src/pbf/pbf_boundary.h:4-19,
src/pbf/solver/pbf_solve.h:57-70) and call straight through the C ABI of
``libpbf103.so``.  Host arrays are numpy ``(n, 3) float32`` (the reference's
``dom_dim``); device arrays are torch CUDA tensors of the same shape.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from ._lib import (PBF_ARRANGE_CYLINDER, PBF_ARRANGE_LINE, PBF_ARRANGE_RECTANGLE, PBF_ARRANGE_VOLUME, PbfArrangement,
                   PbfParams, check, load)

_PARAM_KEYS = [f[0] for f in PbfParams._fields_]


def params_to_dict(s: PbfParams) -> dict:
    d = {}
    for k in _PARAM_KEYS:
        v = getattr(s, k)
        d[k] = list(v) if hasattr(v, "__len__") else v
    return d


def dict_to_params(d: dict) -> PbfParams:
    s = PbfParams()
    check(load().pbf_params_init(ctypes.byref(s)), "pbf_params_init")
    for k, v in d.items():
        if k not in _PARAM_KEYS:
            raise KeyError(f"unknown parameter {k}")
        if k in ("body_force", "grid_size"):
            arr = getattr(s, k)
            for c in range(3):
                arr[c] = v[c]
        else:
            setattr(s, k, v)
    return s


def default_params(**overrides) -> dict:
    """Reference-mode defaults (pbf_params_init) with overrides."""
    s = PbfParams()
    check(load().pbf_params_init(ctypes.byref(s)), "pbf_params_init")
    d = params_to_dict(s)
    d.update(overrides)
    d["cell_width"] = d["cell_width"] or d["smoothing_length"]
    return d


def config_params(**overrides) -> dict:
    """Physics of the benchmark configs: textbook s_corr (k 0.1, n 4, dq 0.2h),
    XSPH c 0.01 and textbook vorticity confinement eps 0.0005, both over the
    step's neighbour list."""
    d = default_params(tensile_mode=L.PBF_TENSILE_TEXTBOOK, scorr_k=0.1, scorr_n=4, scorr_dq=0.2,
                       xsph_mode=L.PBF_XSPH_LIST, xsph_parameter=0.01, vorticity_mode=L.PBF_VORTICITY_TEXTBOOK,
                       vc_parameter=0.0005)
    d.update(overrides)
    return d


def _f3(a) -> ctypes.Array:
    a = np.asarray(a, np.float32).reshape(3)
    return (ctypes.c_float * 3)(*[float(t) for t in a])


def calc_grid_size(cell_size: float, domain_end) -> tuple:
    g = (ctypes.c_uint32 * 3)()
    check(load().pbf_calc_grid_size(float(cell_size), _f3(domain_end), g), "pbf_calc_grid_size")
    return tuple(g)


def resolve_grid(params: dict, domain_end) -> tuple:
    if all(params["grid_size"]):
        return tuple(params["grid_size"])
    return calc_grid_size(2.0 * (params["cell_width"] or params["smoothing_length"]), domain_end)


def scene_bytes(params: dict, capacity: int, domain_end) -> int:
    out = ctypes.c_uint64()
    check(load().pbf_scene_bytes(ctypes.byref(dict_to_params(params)), capacity, _f3(domain_end),
                                 ctypes.byref(out)), "pbf_scene_bytes")
    return out.value


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def _host3(a):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, 3))
    return a


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and a.is_cuda


def _ptr(a):
    if a is None:
        return None
    if _is_device(a):
        return a.data_ptr()
    return a.ctypes.data


_AXES = {"x": 0, "y": 1, "z": 2}


def arrangement(kind: str, *, origin=(0.0, 0.0, 0.0), end=(0.0, 0.0, 0.0), space: float, axis: str = "x",
                axis_value: float = 0.0, radius: float = 0.0, height: float = 0.0) -> PbfArrangement:
    """The reference's arrangement generators (src/pbf/util/pbf_arrangement.h):
    kind "volume" (cartesian_volume(origin, end, space)), "rectangle"
    (cartesian_rectangle(axis, axis_value, origin[:2], end[:2], space)), "line"
    (cartesian_line_inclusive(origin, end, space)) or "cylinder"
    (cartesian_cylinder(axis, axis_value, origin[:2], radius, height, space))."""
    kinds = {"volume": PBF_ARRANGE_VOLUME, "rectangle": PBF_ARRANGE_RECTANGLE, "line": PBF_ARRANGE_LINE,
             "cylinder": PBF_ARRANGE_CYLINDER}
    a = PbfArrangement()
    a.kind = kinds[kind]
    a.axis = _AXES[axis]
    o = list(origin) + [0.0] * (3 - len(origin))
    e = list(end) + [0.0] * (3 - len(end))
    for c in range(3):
        a.origin[c] = o[c]
        a.end[c] = e[c]
    a.axis_value, a.radius, a.height, a.space = axis_value, radius, height, space
    return a


def arrangement_count(a: PbfArrangement) -> int:
    n = ctypes.c_uint32()
    check(load().pbf_arrangement_count(ctypes.byref(a), ctypes.byref(n)), "pbf_arrangement_count")
    return n.value


class Emitter:
    """A fixed set of particles resident on a device, appended by
    PbfParticle.emit / Batch.emit (the sphere scene's jet,
    src/simulator/sphere/pbf_sphere_sim.cpp:20-82)."""

    def __init__(self, x=None, v=None, *, arrangement: PbfArrangement | None = None, velocity=(0.0, 0.0, 0.0),
                 device: int = 0):
        h = ctypes.c_void_p()
        if arrangement is not None:
            check(load().pbf_emitter_create_arrangement(device, ctypes.byref(arrangement), _f3(velocity),
                                                        ctypes.byref(h)), "pbf_emitter_create_arrangement")
        else:
            dev = _is_device(x)
            if not dev:
                x, v = _host3(x), _host3(v)
            check(load().pbf_emitter_create(device, _ptr(x), _ptr(v), x.shape[0], 1 if dev else 0,
                                            ctypes.byref(h)), "pbf_emitter_create")
        self.handle = h.value
        self.device = device

    @property
    def size(self) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_emitter_size(self.handle, ctypes.byref(n)), "pbf_emitter_size")
        return n.value

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                load().pbf_emitter_destroy(h)
            except Exception:
                pass


def _scatter_out(fn, args, n_out: int, stream, what: str):
    x = np.zeros((n_out, 3), np.float32)
    v = np.zeros((n_out, 3), np.float32)
    x[:] = np.nan
    v[:] = np.nan
    check(fn(*args, x.ctypes.data, v.ctypes.data, int(n_out), 0, _stream(stream)), what)
    return x, v


class Boundary:
    """pbf_boundary (src/pbf/pbf_boundary.h:4-19): inner spheres keep particles
    inside, outer spheres (routed through the inner routine, as the reference
    does), and planes given by a point and an inward normal."""

    def __init__(self, inner_spheres=(), outer_spheres=(), points_on_planes=(), normals_on_planes=()):
        self._inner = np.ascontiguousarray(np.asarray(inner_spheres, np.float32).reshape(-1, 4))
        self._outer = np.ascontiguousarray(np.asarray(outer_spheres, np.float32).reshape(-1, 4))
        self._pp = np.ascontiguousarray(np.asarray(points_on_planes, np.float32).reshape(-1, 3))
        self._pn = np.ascontiguousarray(np.asarray(normals_on_planes, np.float32).reshape(-1, 3))
        if self._pp.shape != self._pn.shape:
            raise ValueError("points_on_planes and normals_on_planes differ in length")
        fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))  # noqa: E731
        h = ctypes.c_void_p()
        check(load().pbf_boundary_create(fp(self._inner), len(self._inner), fp(self._outer), len(self._outer),
                                         fp(self._pp), fp(self._pn), len(self._pp), ctypes.byref(h)),
              "pbf_boundary_create")
        self.handle = h.value

    @property
    def inner_spheres(self):
        return self._inner

    @property
    def outer_spheres(self):
        return self._outer

    @property
    def points_on_planes(self):
        return self._pp

    @property
    def normals_on_planes(self):
        return self._pn

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                load().pbf_boundary_destroy(h)
            except Exception:
                pass


class PbfParticle:
    """pbf_particle + pbf_buffer on one GPU (src/pbf/pbf_type.h:74-100):
    ``allocate(num, domain_end)`` happens in the constructor."""

    def __init__(self, params: dict, capacity: int, domain_end, device: int = 0):
        self.params = dict(params)
        self.capacity = int(capacity)
        self.domain_end = tuple(float(t) for t in np.asarray(domain_end, np.float32).reshape(3))
        h = ctypes.c_void_p()
        check(load().pbf_create(ctypes.byref(dict_to_params(self.params)), self.capacity, _f3(self.domain_end),
                                device, ctypes.byref(h)), "pbf_create")
        self.handle = h.value
        self.device = device

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                load().pbf_destroy(h)
            except Exception:
                pass

    # -- state
    def set_particles(self, x, v=None, stream=None):
        dev = _is_device(x)
        if not dev:
            x, v = _host3(x), _host3(v)
        n = x.shape[0]
        check(load().pbf_set_particles(self.handle, _ptr(x), _ptr(v), n, 1 if dev else 0, _stream(stream)),
              "pbf_set_particles")

    def add_particles(self, x, v=None, stream=None):
        """cuda::addParticle (src/pbf/util/cuda/pbf_add.cu:12-28)."""
        dev = _is_device(x)
        if not dev:
            x, v = _host3(x), _host3(v)
        check(load().pbf_add_particles(self.handle, _ptr(x), _ptr(v), x.shape[0], 1 if dev else 0,
                                       _stream(stream)), "pbf_add_particles")

    @property
    def num(self) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_get_num(self.handle, ctypes.byref(n)), "pbf_get_num")
        return n.value

    def get_particles(self, stream=None):
        n = self.num
        x = np.zeros((n, 3), np.float32)
        v = np.zeros((n, 3), np.float32)
        if n:
            check(load().pbf_get_particles(self.handle, x.ctypes.data, v.ctypes.data, 0, _stream(stream)),
                  "pbf_get_particles")
        return x, v

    def get_particles_device(self, x_out, v_out, stream=None):
        check(load().pbf_get_particles(self.handle, _ptr(x_out), _ptr(v_out), 1, _stream(stream)),
              "pbf_get_particles")

    def set_params(self, params: dict):
        check(load().pbf_set_params(self.handle, ctypes.byref(dict_to_params(params))), "pbf_set_params")
        self.params = dict(params)

    def flags(self, clear: bool = False) -> int:
        f = ctypes.c_uint32()
        check(load().pbf_get_flags(self.handle, ctypes.byref(f), 1 if clear else 0), "pbf_get_flags")
        return f.value

    @property
    def grid(self) -> tuple:
        g = (ctypes.c_uint32 * 3)()
        cw = ctypes.c_float()
        check(load().pbf_get_grid(self.handle, g, ctypes.byref(cw)), "pbf_get_grid")
        return tuple(g)

    def set_graph_mode(self, on: bool):
        check(load().pbf_set_graph_mode(self.handle, 1 if on else 0), "pbf_set_graph_mode")

    @property
    def launches(self) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_last_launches(self.handle, ctypes.byref(n)), "pbf_last_launches")
        return n.value

    # -- ids, order restore, device-side appends
    def particle_ids(self, stream=None) -> np.ndarray:
        """Id of each particle in its current (sorted) order."""
        n = self.num
        ids = np.zeros(n, np.uint32)
        if n:
            check(load().pbf_get_particle_ids(self.handle, ids.ctypes.data, 0, _stream(stream)),
                  "pbf_get_particle_ids")
        return ids

    def restore_order(self, n_out: int, stream=None):
        """restoreOrder: positions / velocities in the order of the last
        step's input (rows without a live particle are NaN)."""
        return _scatter_out(load().pbf_restore_order, (self.handle,), n_out, stream, "pbf_restore_order")

    def particles_by_id(self, n_out: int, stream=None):
        """Row k = the particle with id k (NaN where no live particle has it)."""
        return _scatter_out(load().pbf_get_particles_by_id, (self.handle,), n_out, stream,
                            "pbf_get_particles_by_id")

    def generate(self, a: PbfArrangement, velocity=(0.0, 0.0, 0.0), stream=None) -> int:
        """Append an arrangement's points on the device; returns its point count."""
        n = ctypes.c_uint32()
        check(load().pbf_generate(self.handle, ctypes.byref(a), _f3(velocity), _stream(stream), ctypes.byref(n)),
              "pbf_generate")
        return n.value

    def emit(self, emitter: Emitter, max_fill: float = 0.8, stream=None):
        """Append the emitter's particles iff num < max_fill * capacity, decided on the device."""
        check(load().pbf_emit(self.handle, emitter.handle, float(max_fill), _stream(stream)), "pbf_emit")

    def neighbor_debug(self) -> dict:
        """Integer intermediates of the last step in the reference's layouts
        (neighbor_search getters, src/pbf/interaction/pbf_neighbor_search.h:49-56)."""
        g = self.grid
        C = g[0] * g[1] * g[2]
        cap = self.params["max_pair_particle_num"]
        n_in = ctypes.c_uint32()
        check(load().pbf_get_neighbor_debug(self.handle, None, None, None, None, None, ctypes.byref(n_in)),
              "pbf_get_neighbor_debug")
        n = n_in.value
        live = self.num
        sh = np.zeros(max(n, 1), np.uint32)
        pm = np.zeros(max(n, 1), np.uint32)
        cs = np.zeros(C, np.uint32)
        ce = np.zeros(C, np.uint32)
        nl = np.zeros(max((live + 31) // 32 * 32 * cap, 1), np.uint32)
        check(load().pbf_get_neighbor_debug(self.handle, sh.ctypes.data, pm.ctypes.data, cs.ctypes.data,
                                            ce.ctypes.data, nl.ctypes.data, ctypes.byref(n_in)),
              "pbf_get_neighbor_debug")
        return {"sorted_hash": sh[:n], "perm": pm[:n], "cell_start": cs, "cell_end": ce,
                "neighbor_list": nl, "n_in": n, "num": live}


def one_step(simulatee: PbfParticle, boundary: Boundary | None, simulation_area, num_solver_iteration: int,
             stream=None):
    """pbf::one_step (src/pbf/solver/pbf_solve.cpp:147-216).  ``boundary=None``
    is the overload without a boundary argument (fixed sphere at (3,3,3), r=3).
    ``simulation_area`` = (min, max); particles leaving it are deleted."""
    amin, amax = simulation_area
    check(load().pbf_one_step(simulatee.handle, boundary.handle if boundary else None, _f3(amin), _f3(amax),
                              int(num_solver_iteration), _stream(stream)), "pbf_one_step")


def profile_step(simulatee: PbfParticle, boundary: Boundary | None, simulation_area, num_solver_iteration: int,
                 stream=None) -> list:
    """one_step without a CUDA graph, timing each kernel with CUDA events:
    returns [(kernel name, milliseconds)] in launch order."""
    amin, amax = simulation_area
    names = (ctypes.c_char * (64 * 64))()
    ms = (ctypes.c_float * 64)()
    n = ctypes.c_uint32()
    check(load().pbf_profile_step(simulatee.handle, boundary.handle if boundary else None, _f3(amin), _f3(amax),
                                  int(num_solver_iteration), _stream(stream), ms, names, 64, ctypes.byref(n)),
          "pbf_profile_step")
    raw = bytes(names)
    return [(raw[64 * k:64 * k + 64].split(b"\0")[0].decode(), float(ms[k])) for k in range(n.value)]


def one_step_external(simulatee: PbfParticle, x_device, boundary: Boundary | None, simulation_area,
                      num_solver_iteration: int, stream=None):
    """one_step with positions in a borrowed device buffer (AoS float3), as the
    reference's simulators do with a GL-mapped buffer (pbf_dam_sim.cpp:53-66)."""
    amin, amax = simulation_area
    check(load().pbf_one_step_external(simulatee.handle, _ptr(x_device), boundary.handle if boundary else None,
                                       _f3(amin), _f3(amax), int(num_solver_iteration), _stream(stream)),
          "pbf_one_step_external")


class Batch:
    """Many independent scenes advanced together, one launch per kernel per step."""

    def __init__(self, max_scenes: int, max_particles: int, max_cells: int, max_pair: int = 30, device: int = 0):
        h = ctypes.c_void_p()
        check(load().pbf_batch_create(max_scenes, max_particles, max_cells, max_pair, device, ctypes.byref(h)),
              "pbf_batch_create")
        self.handle = h.value
        self._keep = {}

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                load().pbf_batch_destroy(h)
            except Exception:
                pass

    def add_scene(self, params: dict, capacity: int, domain_end, boundary: Boundary | None, simulation_area, x,
                  v=None, stream=None) -> int:
        dev = _is_device(x)
        if not dev:
            x, v = _host3(x), _host3(v)
        sid = ctypes.c_uint32()
        amin, amax = simulation_area
        check(load().pbf_batch_add_scene(self.handle, ctypes.byref(dict_to_params(params)), int(capacity),
                                         _f3(domain_end), boundary.handle if boundary else None, _f3(amin),
                                         _f3(amax), _ptr(x), _ptr(v), x.shape[0], 1 if dev else 0,
                                         _stream(stream), ctypes.byref(sid)), "pbf_batch_add_scene")
        self._keep[sid.value] = boundary
        return sid.value

    def remove_scene(self, sid: int):
        check(load().pbf_batch_remove_scene(self.handle, sid), "pbf_batch_remove_scene")
        self._keep.pop(sid, None)

    @property
    def num_scenes(self) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_batch_num_scenes(self.handle, ctypes.byref(n)), "pbf_batch_num_scenes")
        return n.value

    def step(self, iters: int, stream=None):
        check(load().pbf_batch_step(self.handle, int(iters), _stream(stream)), "pbf_batch_step")

    def get_scene(self, sid: int, stream=None):
        n = ctypes.c_uint32()
        check(load().pbf_batch_get_scene(self.handle, sid, None, None, ctypes.byref(n), 0, _stream(stream)),
              "pbf_batch_get_scene")
        x = np.zeros((n.value, 3), np.float32)
        v = np.zeros((n.value, 3), np.float32)
        check(load().pbf_batch_get_scene(self.handle, sid, x.ctypes.data, v.ctypes.data, ctypes.byref(n), 0,
                                         _stream(stream)), "pbf_batch_get_scene")
        return x, v

    def get_scene_device(self, sid: int, x_out, v_out, stream=None) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_batch_get_scene(self.handle, sid, _ptr(x_out), _ptr(v_out), ctypes.byref(n), 1,
                                         _stream(stream)), "pbf_batch_get_scene")
        return n.value

    def particle_ids(self, sid: int, stream=None) -> np.ndarray:
        n = ctypes.c_uint32()
        check(load().pbf_batch_get_particle_ids(self.handle, sid, None, ctypes.byref(n), 0, _stream(stream)),
              "pbf_batch_get_particle_ids")
        ids = np.zeros(n.value, np.uint32)
        if n.value:
            check(load().pbf_batch_get_particle_ids(self.handle, sid, ids.ctypes.data, ctypes.byref(n), 0,
                                                    _stream(stream)), "pbf_batch_get_particle_ids")
        return ids[:n.value]

    def restore_order(self, sid: int, n_out: int, stream=None):
        return _scatter_out(load().pbf_batch_restore_order, (self.handle, sid), n_out, stream,
                            "pbf_batch_restore_order")

    def particles_by_id(self, sid: int, n_out: int, stream=None):
        return _scatter_out(load().pbf_batch_get_particles_by_id, (self.handle, sid), n_out, stream,
                            "pbf_batch_get_particles_by_id")

    def generate(self, sid: int, a: PbfArrangement, velocity=(0.0, 0.0, 0.0), stream=None) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_batch_generate(self.handle, sid, ctypes.byref(a), _f3(velocity), _stream(stream),
                                        ctypes.byref(n)), "pbf_batch_generate")
        return n.value

    def emit(self, sid: int, emitter: Emitter, max_fill: float = 0.8, stream=None):
        check(load().pbf_batch_emit(self.handle, sid, emitter.handle, float(max_fill), _stream(stream)),
              "pbf_batch_emit")

    def flags(self, sid: int, clear: bool = False) -> int:
        f = ctypes.c_uint32()
        check(load().pbf_batch_get_flags(self.handle, sid, ctypes.byref(f), 1 if clear else 0),
              "pbf_batch_get_flags")
        return f.value

    def scene_ids(self) -> list:
        n = ctypes.c_uint32()
        check(load().pbf_batch_scene_ids(self.handle, None, 0, ctypes.byref(n)), "pbf_batch_scene_ids")
        ids = (ctypes.c_uint32 * max(n.value, 1))()
        check(load().pbf_batch_scene_ids(self.handle, ids, n.value, ctypes.byref(n)), "pbf_batch_scene_ids")
        return list(ids[:n.value])

    def set_all(self, x, v=None, counts=None, stream=None):
        """Upload every active scene from one packed (N, 3) buffer (scene-id order).
        Host buffers must stay alive until the stream has consumed them."""
        dev = _is_device(x)
        if not dev:
            x, v = _host3(x), _host3(v)
        c = None
        if counts is not None:
            c = np.ascontiguousarray(np.asarray(counts, np.uint32))
            self._counts_keep = c
        check(load().pbf_batch_set_all(self.handle, c.ctypes.data if c is not None else None, _ptr(x), _ptr(v),
                                       1 if dev else 0, _stream(stream)), "pbf_batch_set_all")

    def live_counts(self, stream=None) -> np.ndarray:
        """Live particles of every active scene (scene-id order); waits for the stream."""
        n = len(self.scene_ids())
        counts = np.zeros(max(n, 1), np.uint32)
        check(load().pbf_batch_get_all(self.handle, counts.ctypes.data, None, None, 0, _stream(stream)),
              "pbf_batch_get_all")
        return counts[:n]

    def get_all(self, x_out=None, v_out=None, stream=None):
        """Download every active scene into packed buffers; returns counts.
        With x_out None, numpy arrays are allocated and returned as (counts, x, v)."""
        ids = self.scene_ids()
        counts = np.zeros(max(len(ids), 1), np.uint32)
        if x_out is None:
            check(load().pbf_batch_get_all(self.handle, counts.ctypes.data, None, None, 0, _stream(stream)),
                  "pbf_batch_get_all")
            tot = int(counts[:len(ids)].sum())
            x_out = np.zeros((tot, 3), np.float32)
            v_out = np.zeros((tot, 3), np.float32)
        dev = _is_device(x_out)
        check(load().pbf_batch_get_all(self.handle, counts.ctypes.data, _ptr(x_out), _ptr(v_out), 1 if dev else 0,
                                       _stream(stream)), "pbf_batch_get_all")
        return counts[:len(ids)], x_out, v_out

    def step_packed(self, iters: int, x_dev, v_dev=None, counts=None, stream=None):
        """set_all from device buffers and step in one call, the step reading
        the packed input where it lies (no unpack pass)."""
        c = None
        if counts is not None:
            c = np.ascontiguousarray(np.asarray(counts, np.uint32))
            self._counts_keep = c
        check(load().pbf_batch_step_packed(self.handle, int(iters), c.ctypes.data if c is not None else None,
                                           _ptr(x_dev), _ptr(v_dev), _stream(stream)), "pbf_batch_step_packed")

    def get_all_async(self, counts_dev, x_dev=None, v_dev=None, stream=None):
        """Download every active scene into device buffers (packed as get_all)
        without waiting for the stream: counts_dev (device uint32, one per
        active scene) receives the live counts once the stream gets there."""
        check(load().pbf_batch_get_all_async(self.handle, _ptr(counts_dev), _ptr(x_dev), _ptr(v_dev),
                                             _stream(stream)), "pbf_batch_get_all_async")

    def profile_step(self, iters: int, stream=None) -> list:
        """One step without a graph, with CUDA events between kernels; returns
        [(kernel name, milliseconds)] in launch order."""
        names = (ctypes.c_char * (64 * 64))()
        ms = (ctypes.c_float * 64)()
        n = ctypes.c_uint32()
        check(load().pbf_batch_profile_step(self.handle, int(iters), _stream(stream), ms, names, 64,
                                            ctypes.byref(n)), "pbf_batch_profile_step")
        raw = bytes(names)
        return [(raw[64 * k:64 * k + 64].split(b"\0")[0].decode(), float(ms[k])) for k in range(n.value)]

    def autotune(self, iters: int, stream=None) -> int:
        t = ctypes.c_uint32()
        check(load().pbf_batch_autotune(self.handle, int(iters), _stream(stream), ctypes.byref(t)),
              "pbf_batch_autotune")
        return t.value

    def set_tile(self, tile: int):
        check(load().pbf_batch_set_tile(self.handle, int(tile)), "pbf_batch_set_tile")

    def set_chunk(self, chunk: int):
        """Neighbour indices requested ahead per thread in the lambda / delta-p passes (4 or 8)."""
        check(load().pbf_batch_set_chunk(self.handle, int(chunk)), "pbf_batch_set_chunk")

    def set_cell_tile(self, cells: int):
        """Cells per CTA of the per-cell stable rank of large steps (64, 128, 256 or 512)."""
        check(load().pbf_batch_set_cell_tile(self.handle, int(cells)), "pbf_batch_set_cell_tile")

    def launch_shape(self) -> dict:
        t, c, ct = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        check(load().pbf_batch_get_launch_shape(self.handle, ctypes.byref(t), ctypes.byref(c)),
              "pbf_batch_get_launch_shape")
        check(load().pbf_batch_get_cell_tile(self.handle, ctypes.byref(ct)), "pbf_batch_get_cell_tile")
        return {"tile": t.value, "chunk": c.value, "cell_tile": ct.value}

    def set_graph_mode(self, on: bool):
        check(load().pbf_batch_set_graph_mode(self.handle, 1 if on else 0), "pbf_batch_set_graph_mode")

    @property
    def launches(self) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_batch_last_launches(self.handle, ctypes.byref(n)), "pbf_batch_last_launches")
        return n.value


class Server:
    """Continuous-batching request server (pbf_server_* in include/pbf103.h)."""

    def __init__(self, hbm_budget_bytes: int, max_scenes: int, max_particles: int, max_cells: int,
                 iters: int = 4, max_pair: int = 30, device: int = 0, tile: int = 256):
        cfg = L.PbfServerConfig(hbm_budget_bytes, max_scenes, max_particles, max_cells, max_pair, iters, device,
                                tile)
        h = ctypes.c_void_p()
        check(load().pbf_server_create(ctypes.byref(cfg), ctypes.byref(h)), "pbf_server_create")
        self.handle = h.value

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                load().pbf_server_destroy(h)
            except Exception:
                pass

    def submit(self, params: dict, domain_end, simulation_area, x, v=None, horizon_steps: int = 60,
               planes=None, capacity: int = 0) -> int:
        d = L.PbfRequestDesc()
        d.params = dict_to_params(params)
        for c in range(3):
            d.domain_end[c] = float(domain_end[c])
            d.area_min[c] = float(simulation_area[0][c])
            d.area_max[c] = float(simulation_area[1][c])
        if planes is not None:
            pts, nrm = planes
            pts = np.asarray(pts, np.float32).reshape(-1, 3)
            nrm = np.asarray(nrm, np.float32).reshape(-1, 3)
            d.n_planes = len(pts)
            for k in range(len(pts)):
                for c in range(3):
                    d.plane_points[k][c] = pts[k, c]
                    d.plane_normals[k][c] = nrm[k, c]
        d.capacity = capacity
        d.horizon_steps = horizon_steps
        x = _host3(x)
        v = _host3(v) if v is not None else None
        rid = ctypes.c_uint64()
        check(load().pbf_server_submit(self.handle, ctypes.byref(d), x.ctypes.data,
                                       v.ctypes.data if v is not None else None, x.shape[0], ctypes.byref(rid)),
              "pbf_server_submit")
        return rid.value

    def start(self):
        check(load().pbf_server_start(self.handle), "pbf_server_start")

    def stop(self, drain: bool = True):
        check(load().pbf_server_stop(self.handle, 1 if drain else 0), "pbf_server_stop")

    def run_until_idle(self):
        check(load().pbf_server_run_until_idle(self.handle), "pbf_server_run_until_idle")

    def poll(self, max_items: int = 4096) -> list:
        buf = (L.PbfCompletion * max_items)()
        n = ctypes.c_uint32()
        check(load().pbf_server_poll(self.handle, buf, max_items, ctypes.byref(n)), "pbf_server_poll")
        return [{"request_id": c.request_id, "num": c.num, "steps": c.steps, "flags": c.flags,
                 "arrival_s": c.arrival_s, "admit_s": c.admit_s, "complete_s": c.complete_s}
                for c in buf[:n.value]]

    def result(self, rid: int):
        n = ctypes.c_uint32()
        check(load().pbf_server_result(self.handle, rid, None, None, ctypes.byref(n)), "pbf_server_result")
        x = np.zeros((n.value, 3), np.float32)
        v = np.zeros((n.value, 3), np.float32)
        check(load().pbf_server_result(self.handle, rid, x.ctypes.data, v.ctypes.data, ctypes.byref(n)),
              "pbf_server_result")
        return x, v

    def release(self, rid: int):
        check(load().pbf_server_release(self.handle, rid), "pbf_server_release")

    def stats(self) -> dict:
        s = L.PbfServerStats()
        check(load().pbf_server_get_stats(self.handle, ctypes.byref(s)), "pbf_server_get_stats")
        return {k: getattr(s, k) for k, _ in L.PbfServerStats._fields_}

    def clock(self) -> float:
        return load().pbf_server_clock(self.handle)


# ------------------------------------------------------------- rendering --

# image name -> (PBF_SSF_* id, dtype, channels)
SSF_IMAGES = {
    "depth": (L.PBF_SSF_DEPTH, np.float32, 1),
    "blurred": (L.PBF_SSF_BLURRED, np.float32, 1),
    "blur_input": (L.PBF_SSF_BLUR_INPUT, np.float32, 1),
    "normal": (L.PBF_SSF_NORMAL, np.float32, 4),
    "color": (L.PBF_SSF_COLOR, np.float32, 4),
    "rgba8": (L.PBF_SSF_RGBA8, np.uint8, 4),
}
_SSF_ARRAYS = {"projection": 16, "view": 16, "clear_color": 4}


def ssf_default_params(**overrides) -> dict:
    """The reference's first rendered frame: 1280 x 720 (src/main.cpp:32),
    the camera of src/common/controls.cpp:12-110, point radius 0.18
    (main.cpp:388), blur radius 5.5e-6 and three blur passes
    (main.cpp:189, 430-509); see ``pbf_ssf_params_init``."""
    s = L.PbfSsfParams()
    check(load().pbf_ssf_params_init(ctypes.byref(s)), "pbf_ssf_params_init")
    d = {}
    for k, _ in L.PbfSsfParams._fields_:
        v = getattr(s, k)
        d[k] = np.array(v[:], np.float32) if k in _SSF_ARRAYS else v
    h0 = d["height"]
    for k, v in overrides.items():
        if k not in d:
            raise KeyError(k)
        d[k] = v
    # both scales are proportional to the target height (main.cpp:445;
    # pixels per unit at unit distance); follow an overridden height
    if d["height"] != h0:
        for k in ("blur_scale", "point_scale"):
            if k not in overrides:
                d[k] = float(np.float32(d[k]) * np.float32(d["height"]) / np.float32(h0))
    return d


def _ssf_struct(d: dict) -> L.PbfSsfParams:
    s = L.PbfSsfParams()
    for k, _ in L.PbfSsfParams._fields_:
        v = d[k]
        if k in _SSF_ARRAYS:
            a = np.asarray(v, np.float32).reshape(-1)
            getattr(s, k)[:] = [float(t) for t in a]
        else:
            setattr(s, k, v)
    return s


class SsfRenderer:
    """Headless screen-space fluid renderer: the reference's per-frame GL
    passes (src/main.cpp:372-564) as CUDA kernels into device images.
    Images come back as numpy arrays with row 0 at the bottom."""

    def __init__(self, params: dict | None = None, device: int = 0, **overrides):
        self.params = dict(params) if params is not None else ssf_default_params()
        self.params.update(overrides)
        h = ctypes.c_void_p()
        check(load().pbf_ssf_create(device, ctypes.byref(_ssf_struct(self.params)), ctypes.byref(h)),
              "pbf_ssf_create")
        self.handle = h.value
        self.device = device
        self.width, self.height = int(self.params["width"]), int(self.params["height"])

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                load().pbf_ssf_destroy(h)
            except Exception:
                pass

    def render(self, x, stream=None):
        """One frame of n positions: a torch CUDA tensor (n, 3) float32, or a
        host array (copied to the device first)."""
        if not _is_device(x):
            import torch
            x = torch.from_numpy(_host3(x)).to(f"cuda:{self.device}")
        x = x.contiguous()
        check(load().pbf_ssf_render(self.handle, x.data_ptr(), x.shape[0], _stream(stream)), "pbf_ssf_render")
        self._keep = x  # the frame reads x until the stream reaches its end

    def render_particles(self, part: "PbfParticle", stream=None):
        check(load().pbf_ssf_render_particles(self.handle, part.handle, _stream(stream)), "pbf_ssf_render_particles")

    def render_scene(self, batch: "Batch", sid: int, stream=None):
        check(load().pbf_ssf_render_scene(self.handle, batch.handle, sid, _stream(stream)), "pbf_ssf_render_scene")

    def image(self, which: str = "rgba8", stream=None) -> np.ndarray:
        kind, dt, ch = SSF_IMAGES[which]
        shape = (self.height, self.width) if ch == 1 else (self.height, self.width, ch)
        out = np.zeros(shape, dt)
        check(load().pbf_ssf_get_image(self.handle, kind, out.ctypes.data, 0, _stream(stream)), "pbf_ssf_get_image")
        return out

    def image_device(self, which: str) -> tuple:
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_uint64()
        check(load().pbf_ssf_image_device(self.handle, SSF_IMAGES[which][0], ctypes.byref(ptr), ctypes.byref(nbytes)),
              "pbf_ssf_image_device")
        return ptr.value, nbytes.value

    def frame_constants(self) -> tuple:
        inv = (ctypes.c_float * 16)()
        inc = (ctypes.c_float * 3)()
        check(load().pbf_ssf_frame_constants(self.handle, inv, inc), "pbf_ssf_frame_constants")
        return np.array(inv[:], np.float32), np.array(inc[:], np.float32)

    @property
    def launches(self) -> int:
        n = ctypes.c_uint32()
        check(load().pbf_ssf_last_launches(self.handle, ctypes.byref(n)), "pbf_ssf_last_launches")
        return n.value

    def save_ppm(self, path: str, stream=None):
        """The composited frame as a binary PPM (top row first)."""
        img = self.image("rgba8", stream)[::-1, :, :3]
        with open(path, "wb") as fh:
            fh.write(f"P6\n{self.width} {self.height}\n255\n".encode())
            fh.write(np.ascontiguousarray(img).tobytes())
