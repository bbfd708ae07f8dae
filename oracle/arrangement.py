"""CPU restatement of the reference's arrangement generators — TEST INFRASTRUCTURE ONLY.

Follows src/pbf/util/pbf_arrangement.h of yodaplusplus/ssf_pbf_cuda (with GLM
0.9.7's length / normalize / dot, external/include/glm/detail/
func_geometric.inl:95-159): every float operation is a numpy float32
operation in the reference's order, every double one a Python float, so the
points are bit-exact for volume, rectangle and line.  The cylinder uses
cos / sin, whose last bit differs between libraries; its ring and point
counts are exact.  Used only by tests/ as the checker of the device
generators (pbf_generate, pbf_emitter_create_arrangement).
"""
from __future__ import annotations

import math
import sys

import numpy as np

F = np.float32
EPS10 = sys.float_info.epsilon * 10.0
PI_F = F(3.14159265358979323846264338327950288)


def _axis_count(rng: np.float32, space: np.float32) -> int:
    """static_cast<int>(range / space + epsilon * 10.0) + 1 (pbf_arrangement.h:85-90)."""
    q = F(rng) / F(space)
    return int(float(q) + EPS10) + 1


def volume(origin, end, space) -> np.ndarray:
    """cartesian_volume, pbf_arrangement.h:82-99 (z outer, x inner)."""
    o = np.asarray(origin, F)
    e = np.asarray(end, F)
    s = F(space)
    n = [_axis_count(e[c] - o[c], s) for c in range(3)]
    if min(n) <= 0:
        return np.zeros((0, 3), F)
    z, y, x = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    pts = np.stack([o[0] + s * x.astype(F).ravel(), o[1] + s * y.astype(F).ravel(),
                    o[2] + s * z.astype(F).ravel()], axis=1)
    return pts.astype(F)


def rectangle(axis: str, axis_value, origin2, end2, space) -> np.ndarray:
    """cartesian_rectangle, pbf_arrangement.h:123-163."""
    o = np.asarray(origin2, F)
    e = np.asarray(end2, F)
    s = F(space)
    av = F(axis_value)
    c0 = _axis_count(e[0] - o[0], s)
    c1 = _axis_count(e[1] - o[1], s)
    out = []
    if axis == "x":  # (av, o.x, o.y) + (0, s*y, s*z); z outer (c1), y inner (c0)
        for z in range(c1):
            for y in range(c0):
                out.append((av + F(0), o[0] + s * F(y), o[1] + s * F(z)))
    elif axis == "y":  # (o.y, av, o.x) + (s*x, 0, s*z); z outer (c0), x inner (c1)
        for z in range(c0):
            for x in range(c1):
                out.append((o[1] + s * F(x), av + F(0), o[0] + s * F(z)))
    elif axis == "z":  # (o.x, o.y, av) + (s*x, s*y, 0); x outer (c0), y inner (c1)
        for x in range(c0):
            for y in range(c1):
                out.append((o[0] + s * F(x), o[1] + s * F(y), av + F(0)))
    else:
        raise ValueError(axis)
    return np.asarray(out, F).reshape(-1, 3)


def line_inclusive(origin, end, space) -> np.ndarray:
    """cartesian_line_inclusive, pbf_arrangement.h:8-18."""
    o = np.asarray(origin, F)
    e = np.asarray(end, F)
    s = F(space)
    d = (e - o).astype(F)
    dot = F(F(d[0] * d[0]) + F(d[1] * d[1])) + F(d[2] * d[2])
    length = np.sqrt(dot, dtype=F)
    inv = F(1) / np.sqrt(dot, dtype=F)
    direction = ((d * inv).astype(F) * s).astype(F)
    n = int(np.floor(F(length / s))) + 1
    return np.asarray([o + direction * F(i) for i in range(n)], F).reshape(-1, 3)


def cylinder(axis: str, axis_value, origin2, radius, height, space) -> np.ndarray:
    """cartesian_cylinder, pbf_arrangement.h:212-244."""
    s = F(space)
    r = F(radius)
    o = np.asarray(origin2, F)
    av = F(axis_value)
    theta = F(2.0 * math.asin(float(s) / (2.0 * float(r))))
    n = F(math.floor(2.0 * float(PI_F) / float(theta)))
    theta_hat = F(2.0 * float(PI_F) / float(n))
    out = []
    h = F(0)
    while h < F(height):
        i = F(0)
        while i < n:
            ang = F(i * theta_hat)
            c, sn = F(r * np.cos(ang, dtype=F)), F(r * np.sin(ang, dtype=F))
            if axis == "x":
                out.append((av + h, o[0] + c, o[1] + sn))
            elif axis == "y":
                out.append((o[1] + sn, av + h, o[0] + c))
            elif axis == "z":
                out.append((o[0] + c, o[1] + sn, av + h))
            else:
                raise ValueError(axis)
            i = F(float(i) + 1.0)
        h = F(h + s)
    return np.asarray(out, F).reshape(-1, 3)


def generate(kind: str, **kw) -> np.ndarray:
    return {"volume": volume, "rectangle": rectangle, "line": line_inclusive, "cylinder": cylinder}[kind](**kw)
