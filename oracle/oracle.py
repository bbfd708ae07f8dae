"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

The oracle (``pbf_oracle.c``) restates the reference simulator's step
(yodaplusplus/ssf_pbf_cuda, ``pbf::one_step``, src/pbf/solver/pbf_solve.cpp:182-216)
on the CPU.  It is the checker for the CUDA path: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s cpu_baseline / reference arm
load it.  Nothing in ``ssf_pbf_cuda_gb300`` imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpbf_oracle.so")
SOURCES = [os.path.join(HERE, "pbf_oracle.c"), os.path.join(HERE, "ssf_oracle.c")]
DEPS = SOURCES + [os.path.join(HERE, "pbf_oracle.h"), os.path.join(HERE, "pbf_oracle_solve.inc")]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP, no FP contraction)."""
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= lib_m for d in DEPS):
            return LIB_PATH
    cmd = ["gcc", "-O2", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", *SOURCES, "-o", LIB_PATH + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class OraParams(ctypes.Structure):
    _fields_ = [
        ("rest_density", ctypes.c_float),
        ("particle_mass", ctypes.c_float),
        ("smoothing_length", ctypes.c_float),
        ("time_step", ctypes.c_float),
        ("relaxation", ctypes.c_float),
        ("xsph_c", ctypes.c_float),
        ("vorticity_eps", ctypes.c_float),
        ("body_force", ctypes.c_float * 3),
        ("cell_width", ctypes.c_float),
        ("grid", ctypes.c_uint32 * 3),
        ("max_pair", ctypes.c_uint32),
        ("tensile_mode", ctypes.c_int32),
        ("scorr_k", ctypes.c_float),
        ("scorr_n", ctypes.c_int32),
        ("scorr_dq", ctypes.c_float),
        ("xsph_mode", ctypes.c_int32),
        ("vorticity_mode", ctypes.c_int32),
        ("max_collision_passes", ctypes.c_uint32),
    ]


class OraBoundary(ctypes.Structure):
    _fields_ = [
        ("n_inner", ctypes.c_uint32),
        ("n_outer", ctypes.c_uint32),
        ("n_planes", ctypes.c_uint32),
        ("inner", ctypes.POINTER(ctypes.c_float)),
        ("outer", ctypes.POINTER(ctypes.c_float)),
        ("plane_pts", ctypes.POINTER(ctypes.c_float)),
        ("plane_nrm", ctypes.POINTER(ctypes.c_float)),
        ("use_builtin_sphere", ctypes.c_int32),
    ]


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        f = ctypes.c_float
        u32 = ctypes.c_uint32
        lib.ora_step.restype = ctypes.c_int
        lib.ora_step.argtypes = [P(OraParams), P(OraBoundary), P(f), P(f), ctypes.c_int, ctypes.c_int,
                                 u32, P(f), P(f), P(f), P(f), P(u32), P(u32), P(u32), P(u32), P(u32),
                                 P(ctypes.c_uint8), P(f)]
        lib.ora_hash_sort.restype = None
        lib.ora_hash_sort.argtypes = [u32, P(f), f, P(u32), P(f), P(f), ctypes.c_int, P(u32), P(u32), P(u32)]
        lib.ora_wpoly6.restype = f
        lib.ora_wpoly6.argtypes = [f, f]
        lib.ora_wspiky_deriv.restype = f
        lib.ora_wspiky_deriv.argtypes = [f, f]
        lib.ora_calc_grid_size.restype = ctypes.c_int
        lib.ora_calc_grid_size.argtypes = [ctypes.c_double, P(f), P(u32)]
        lib.ora_num_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _up(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def _f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


def make_params(p: dict) -> OraParams:
    """Build the oracle parameter struct from the package's parameter dict
    (the same keys as ``ssf_pbf_cuda_gb300.params``)."""
    o = OraParams()
    o.rest_density = p["stable_density"]
    o.particle_mass = p["particle_mass"]
    o.smoothing_length = p["smoothing_length"]
    o.time_step = p["time_step"]
    o.relaxation = p["relaxation"]
    o.xsph_c = p["xsph_parameter"]
    o.vorticity_eps = p["vc_parameter"]
    for c in range(3):
        o.body_force[c] = p["body_force"][c]
        o.grid[c] = p["grid_size"][c]
    o.cell_width = p["cell_width"]
    o.max_pair = p["max_pair_particle_num"]
    o.tensile_mode = p["tensile_mode"]
    o.scorr_k = p["scorr_k"]
    o.scorr_n = p["scorr_n"]
    o.scorr_dq = p["scorr_dq"]
    o.xsph_mode = p["xsph_mode"]
    o.vorticity_mode = p["vorticity_mode"]
    o.max_collision_passes = p["max_collision_passes"]
    return o


class Boundary:
    """Boundary primitives kept alive for the duration of an oracle call."""

    def __init__(self, inner=None, outer=None, plane_pts=None, plane_nrm=None, builtin_sphere=False):
        self.inner = _f32(inner if inner is not None else np.zeros((0, 4)), (-1, 4))
        self.outer = _f32(outer if outer is not None else np.zeros((0, 4)), (-1, 4))
        self.pp = _f32(plane_pts if plane_pts is not None else np.zeros((0, 3)), (-1, 3))
        self.pn = _f32(plane_nrm if plane_nrm is not None else np.zeros((0, 3)), (-1, 3))
        self.s = OraBoundary()
        self.s.n_inner = self.inner.shape[0]
        self.s.n_outer = self.outer.shape[0]
        self.s.n_planes = self.pp.shape[0]
        self.s.inner = _fp(self.inner)
        self.s.outer = _fp(self.outer)
        self.s.plane_pts = _fp(self.pp)
        self.s.plane_nrm = _fp(self.pn)
        self.s.use_builtin_sphere = 1 if builtin_sphere else 0


def step(params: dict, boundary: Boundary | None, area_min, area_max, iters: int, x, v, f64: bool = False):
    """One oracle step.  x, v: (n, 3) float32 in any order.  Returns a dict
    with sorted-order outputs and the integer intermediates."""
    lib = load()
    P = make_params(params)
    x = _f32(x, (-1, 3))
    v = _f32(v, (-1, 3))
    n = x.shape[0]
    C = int(P.grid[0]) * int(P.grid[1]) * int(P.grid[2])
    cap = int(P.max_pair) - 1
    x_out = np.zeros((n, 3), np.float32)
    v_out = np.zeros((n, 3), np.float32)
    num = np.zeros(1, np.uint32)
    keys = np.zeros(n, np.uint32)
    perm = np.zeros(n, np.uint32)
    offsets = np.zeros(C + 2, np.uint32)
    nbr = np.full((max(n, 1), cap), 0xFFFFFFFF, np.uint32)
    nnb = np.zeros(max(n, 1), np.uint8)
    lam0 = np.zeros(max(n, 1), np.float32)
    amin = _f32(area_min, (3,))
    amax = _f32(area_max, (3,))
    bptr = ctypes.byref(boundary.s) if boundary is not None else None
    rc = lib.ora_step(ctypes.byref(P), bptr, _fp(amin), _fp(amax), int(iters), 1 if f64 else 0,
                      n, _fp(x), _fp(v), _fp(x_out), _fp(v_out), _up(num), _up(keys), _up(perm),
                      _up(offsets), _up(nbr), nnb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _fp(lam0))
    live = int(num[0])
    return {
        "x": x_out[:live], "v": v_out[:live], "num": live, "keys": keys, "perm": perm,
        "offsets": offsets, "nbr": nbr[:live], "nnb": nnb[:live], "lambda0": lam0[:live],
        "collision_passes": rc,
    }


def hash_sort(xs, cell_width, grid, area_min=None, area_max=None):
    """Cell hash + stable counting sort of positions xs (n, 3)."""
    lib = load()
    xs = _f32(xs, (-1, 3))
    n = xs.shape[0]
    g = np.asarray(grid, np.uint32)
    C = int(g[0]) * int(g[1]) * int(g[2])
    keys = np.zeros(n, np.uint32)
    perm = np.zeros(n, np.uint32)
    offsets = np.zeros(C + 2, np.uint32)
    check = area_min is not None
    amin = _f32(area_min if check else [0, 0, 0], (3,))
    amax = _f32(area_max if check else [0, 0, 0], (3,))
    lib.ora_hash_sort(n, _fp(xs), float(cell_width), _up(g), _fp(amin), _fp(amax), 1 if check else 0,
                      _up(keys), _up(perm), _up(offsets))
    return keys, perm, offsets


def calc_grid_size(cell_size: float, sim_end) -> tuple:
    lib = load()
    e = _f32(sim_end, (3,))
    g = np.zeros(3, np.uint32)
    rc = lib.ora_calc_grid_size(float(cell_size), _fp(e), _up(g))
    if rc != 0:
        raise ValueError("grid_size is too large")
    return tuple(int(t) for t in g)


def wpoly6(r: float, inv_h: float) -> float:
    return load().ora_wpoly6(r, inv_h)


def wspiky_deriv(r: float, inv_h: float) -> float:
    return load().ora_wspiky_deriv(r, inv_h)


def num_threads() -> int:
    return load().ora_num_threads()
