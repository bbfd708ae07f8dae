"""ctypes front end of the screen-space fluid oracle — TEST INFRASTRUCTURE ONLY.

``ssf_oracle.c`` restates the reference's per-frame GL passes
(yodaplusplus/ssf_pbf_cuda, cuda_pbf_with_ssf/src/main.cpp:372-564) on the
CPU; this module feeds it.  ``reference_camera`` restates the camera the
reference builds on its first frame (src/common/controls.cpp:12-110 with the
vendored GLM 0.9.7: gtc/matrix_transform.inl perspectiveRH :233-247 and
lookAtRH :484-510, detail/func_geometric.inl normalize :154-159, cross
:134-142) in numpy float32, independently of the library's C version.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import oracle as _O

P = ctypes.POINTER
f32 = np.float32


class OraSsf(ctypes.Structure):
    _fields_ = [
        ("w", ctypes.c_uint32), ("h", ctypes.c_uint32), ("mode", ctypes.c_uint32), ("pad", ctypes.c_uint32),
        ("proj", ctypes.c_float * 16), ("view", ctypes.c_float * 16), ("inv_proj", ctypes.c_float * 16),
        ("radius", ctypes.c_float), ("point_scale", ctypes.c_float), ("znear", ctypes.c_float),
        ("zfar", ctypes.c_float), ("blur_radius", ctypes.c_float), ("blur_scale", ctypes.c_float),
        ("thickness", ctypes.c_float), ("pad1", ctypes.c_float), ("clear", ctypes.c_float * 4),
        ("incident", ctypes.c_float * 3),
    ]


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        lib = _O.load()
        fp = P(ctypes.c_float)
        lib.ora_ssf_splat.restype = None
        lib.ora_ssf_splat.argtypes = [P(OraSsf), fp, ctypes.c_uint32, ctypes.c_int, fp]
        lib.ora_ssf_blur.restype = None
        lib.ora_ssf_blur.argtypes = [P(OraSsf), fp, fp]
        lib.ora_ssf_normal.restype = None
        lib.ora_ssf_normal.argtypes = [P(OraSsf), fp, fp]
        lib.ora_ssf_shade.restype = None
        lib.ora_ssf_shade.argtypes = [P(OraSsf), fp, fp, fp, P(ctypes.c_uint8)]
        _lib = lib
    return _lib


def _fp(a):
    return a.ctypes.data_as(P(ctypes.c_float))


def inverse(m16) -> np.ndarray:
    """Inverse of a column-major 4x4, in float64, rounded to float32."""
    m = np.asarray(m16, np.float64).reshape(4, 4).T  # rows
    return np.linalg.inv(m).T.reshape(16).astype(f32)


def _normalize(v):
    v = np.asarray(v, f32)
    d = f32(v[0] * v[0]) + f32(v[1] * v[1])
    d = f32(d + f32(v[2] * v[2]))
    inv = f32(f32(1.0) / np.sqrt(d, dtype=f32))
    return (v * inv).astype(f32)


def _cross(a, b):
    a, b = np.asarray(a, f32), np.asarray(b, f32)
    return np.array([f32(a[1] * b[2]) - f32(b[1] * a[2]), f32(a[2] * b[0]) - f32(b[2] * a[0]),
                     f32(a[0] * b[1]) - f32(b[0] * a[1])], f32)


def _dot(a, b):
    p = np.asarray(a, f32) * np.asarray(b, f32)
    return f32(f32(p[0] + p[1]) + p[2])


def incident(view16) -> np.ndarray:
    """normalize((View * World * vec4(1, 4, 1, 0)).xyz), ssf_shading.frag:39, 52."""
    V = np.asarray(view16, f32)
    l = [f32(f32(f32(V[r] * f32(1)) + f32(V[4 + r] * f32(4))) + f32(V[8 + r] * f32(1))) + f32(V[12 + r] * f32(0))
         for r in range(3)]
    return _normalize(l)


def reference_camera(width: int = 1280, height: int = 720) -> dict:
    """Projection, view and blur scale of the reference's first frame."""
    pi = f32(np.pi)
    h_ang, v_ang = pi, f32(pi * f32(-0.1))
    cv, sv, sh, ch = np.cos(v_ang), np.sin(v_ang), np.sin(h_ang), np.cos(h_ang)
    direction = np.array([f32(cv * sh), sv, f32(cv * ch)], f32)
    a = f32(h_ang - f32(f32(3.14) / f32(2.0)))
    right = np.array([np.sin(a), 0, np.cos(a)], f32)
    up = _cross(right, direction)
    znear, zfar = f32(0.1), f32(50.0)
    tan_half = np.tan(f32(f32(45.0) / f32(2.0)), dtype=f32)
    aspect = f32(f32(4.0) / f32(3.0))
    proj = np.zeros(16, f32)
    proj[0] = f32(1) / f32(aspect * tan_half)
    proj[5] = f32(1) / tan_half
    proj[10] = f32(-f32(zfar + znear)) / f32(zfar - znear)
    proj[11] = -1
    proj[14] = f32(-f32(f32(f32(2) * zfar) * znear)) / f32(zfar - znear)
    eye = np.array([2, 4, 10], f32)
    center = (eye + direction).astype(f32)
    fw = _normalize(center - eye)
    s = _normalize(_cross(fw, up))
    u = _cross(s, fw)
    view = np.zeros(16, f32)
    view[[0, 4, 8]] = s
    view[[1, 5, 9]] = u
    view[[2, 6, 10]] = -fw
    view[12], view[13], view[14], view[15] = -_dot(s, eye), -_dot(u, eye), _dot(fw, eye), 1
    deg = f32(f32(f32(f32(45.0) * f32(0.5)) * f32(3.1415)) / f32(180.0))
    blur_scale = f32(f32(height) / np.tan(deg, dtype=f32))
    return {"projection": proj, "view": view, "blur_scale": blur_scale,
            "point_scale": f32(proj[5] * f32(f32(height) * f32(0.5)))}


def frame(params: dict, inv_proj=None, inc=None) -> OraSsf:
    """The passes' constants from renderer parameters (the keys of
    ``ssf_default_params``); the inverse projection and light direction are
    computed here unless given."""
    f = OraSsf()
    f.w, f.h, f.mode = int(params["width"]), int(params["height"]), int(params["splat_mode"])
    f.proj[:] = [float(t) for t in np.asarray(params["projection"], f32)]
    f.view[:] = [float(t) for t in np.asarray(params["view"], f32)]
    f.inv_proj[:] = [float(t) for t in (inverse(params["projection"]) if inv_proj is None else inv_proj)]
    f.radius, f.point_scale = params["point_radius"], params["point_scale"]
    f.znear, f.zfar = params["near_plane"], params["far_plane"]
    f.blur_radius, f.blur_scale, f.thickness = params["blur_radius"], params["blur_scale"], params["thickness"]
    f.clear[:] = [float(t) for t in np.asarray(params["clear_color"], f32)]
    f.incident[:] = [float(t) for t in (incident(params["view"]) if inc is None else inc)]
    return f


def splat(f: OraSsf, x) -> np.ndarray:
    x = np.ascontiguousarray(np.asarray(x, f32))
    stride = x.shape[1] if x.ndim == 2 else 3
    out = np.empty((f.h, f.w), f32)
    load().ora_ssf_splat(ctypes.byref(f), _fp(x), x.shape[0] if x.ndim == 2 else 0, stride, _fp(out))
    return out


def blur(f: OraSsf, depth) -> np.ndarray:
    d = np.ascontiguousarray(depth, f32)
    out = np.empty_like(d)
    load().ora_ssf_blur(ctypes.byref(f), _fp(d), _fp(out))
    return out


def normal(f: OraSsf, depth) -> np.ndarray:
    d = np.ascontiguousarray(depth, f32)
    out = np.empty((f.h, f.w, 4), f32)
    load().ora_ssf_normal(ctypes.byref(f), _fp(d), _fp(out))
    return out


def shade(f: OraSsf, depth, normals) -> tuple:
    d = np.ascontiguousarray(depth, f32)
    n = np.ascontiguousarray(normals, f32)
    c = np.empty((f.h, f.w, 4), f32)
    c8 = np.empty((f.h, f.w, 4), np.uint8)
    load().ora_ssf_shade(ctypes.byref(f), _fp(d), _fp(n), _fp(c), c8.ctypes.data_as(P(ctypes.c_uint8)))
    return c, c8


def render(f: OraSsf, x, blur_passes: int = 3) -> dict:
    """Every image of one frame, as the CUDA renderer keeps them."""
    depth = splat(f, x)
    src, prev = depth, depth
    for _ in range(blur_passes):
        prev, src = src, blur(f, src)
    nrm = normal(f, src)
    color, rgba8 = shade(f, depth, nrm)
    return {"depth": depth, "blur_input": prev, "blurred": src, "normal": nrm, "color": color, "rgba8": rgba8}
