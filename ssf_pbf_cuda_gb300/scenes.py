"""Seeded synthetic scenes for the five benchmark workloads.

No dataset is involved: every workload is a generated particle block.
Seeds: master 0x5EED2026; per scene splitmix64(master ^ (scene_id * 0x9E3779B97F4A7C15)),
driving numpy's PCG64 (platform independent).  Jitter is i.i.d. U[-0.01h, +0.01h]
per component.  Lattices are generated z-outer, y, x-inner like the
reference's cartesian_volume (src/pbf/util/pbf_arrangement.h:82-121).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MASTER_SEED = 0x5EED2026
GOLDEN = 0x9E3779B97F4A7C15
MASK64 = (1 << 64) - 1
H = 0.1          # smoothing length, m
SPACING = 0.05   # 0.5 h


def splitmix64(x: int) -> int:
    x = (x + GOLDEN) & MASK64
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def scene_seed(scene_id: int, master: int = MASTER_SEED) -> int:
    return splitmix64(master ^ ((scene_id * GOLDEN) & MASK64))


def rng_for(scene_id: int, master: int = MASTER_SEED) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(scene_seed(scene_id, master)))


def lattice(nx: int, ny: int, nz: int, spacing: float, origin) -> np.ndarray:
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float64) * spacing
    return (pts + np.asarray(origin, np.float64)).astype(np.float32)


def box_planes(box) -> tuple:
    """Six inward planes through the faces of [0, box]."""
    bx, by, bz = (float(t) for t in box)
    pts = np.array([[0, 0, 0], [0, by, 0], [0, 0, 0], [bx, 0, 0], [0, 0, 0], [0, 0, bz]], np.float32)
    nrm = np.array([[0, 1, 0], [0, -1, 0], [1, 0, 0], [-1, 0, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    return pts, nrm


@dataclass
class Scene:
    x: np.ndarray
    v: np.ndarray
    domain_end: tuple
    area: tuple                      # (min, max)
    planes: tuple                    # (points, normals)
    grid: tuple | None = None        # explicit hash grid, or None for calcGridSize
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def params(self, base: dict) -> dict:
        p = dict(base)
        if self.grid is not None:
            p["grid_size"] = list(self.grid)
        return p


def dam_break(nx: int, ny: int, nz: int, box, scene_id: int = 0, grid=None, origin=None, h: float = H,
              spacing: float = SPACING, jitter: float = 0.01, n_keep: int | None = None) -> Scene:
    rng = rng_for(scene_id)
    org = origin if origin is not None else (spacing, spacing, spacing)
    x = lattice(nx, ny, nz, spacing, org)
    if n_keep is not None:
        x = x[:n_keep]
    x = (x + rng.uniform(-jitter * h, jitter * h, size=x.shape)).astype(np.float32)
    v = np.zeros_like(x)
    box = tuple(float(t) for t in box)
    area = (tuple(-h for _ in range(3)), tuple(b + h for b in box))
    return Scene(x, v, box, area, box_planes(box), grid, {"lattice": (nx, ny, nz), "scene_id": scene_id})


def config1() -> Scene:
    """Plain dam break: 32x32x32 = 32,768 particles in a 4 x 2 x 2 m box."""
    return dam_break(32, 32, 32, (4.0, 2.0, 2.0), scene_id=0)


def config2() -> Scene:
    """Single large scene: 128x128x64 = 1,048,576 particles in a 16 x 8 x 8 m box,
    hash table fixed at 2^21 cells (256 x 128 x 64)."""
    return dam_break(128, 128, 64, (16.0, 8.0, 8.0), scene_id=1, grid=(256, 128, 64))


def config3(kind: str = "uniform", n: int = 4194304, seed_id: int = 3) -> tuple:
    """Neighbour-search micro-benchmark positions: (a) uniform in a cube of side
    n^(1/3)*spacing, (b) 64 Gaussian blobs (sigma 5h) clamped to the cube.
    Returns (positions, grid (256,128,128) = 2^22 cells, cell width h)."""
    rng = rng_for(seed_id if kind == "uniform" else seed_id + 1)
    L = n ** (1.0 / 3.0) * SPACING
    if kind == "uniform":
        x = rng.uniform(0.0, L, size=(n, 3))
    elif kind == "blobs":
        centers = rng.uniform(0.0, L, size=(64, 3))
        per = n // 64
        x = np.concatenate([c + rng.normal(0.0, 5 * H, size=(per, 3)) for c in centers], axis=0)
        x = np.clip(x, 0.0, L)
    else:
        raise ValueError(kind)
    return x.astype(np.float32), (256, 128, 128), H


def _random_scene(rng: np.random.Generator, scene_id: int, n: int, h: float = H, spacing: float = SPACING) -> Scene:
    aspect = rng.uniform(1.0, 3.0, size=3)
    vol = 4.0 * n * spacing ** 3
    box = aspect * (vol / float(np.prod(aspect))) ** (1.0 / 3.0)
    # the most cubic lattice >= n that fits the box with 1h clearance
    max_dim = np.maximum(1, np.floor((box - 2 * h) / spacing).astype(int) + 1)
    k = int(math.ceil(n ** (1.0 / 3.0)))
    dims = np.minimum(np.array([k, k, k]), max_dim)
    while int(np.prod(dims)) < n:
        room = max_dim - dims
        if room.max() <= 0:
            box = box * 1.1
            max_dim = np.maximum(1, np.floor((box - 2 * h) / spacing).astype(int) + 1)
            continue
        dims[int(np.argmax(room))] += 1
    extent = (dims - 1) * spacing
    lo = np.full(3, h)
    hi = np.maximum(lo, box - h - extent)
    origin = rng.uniform(lo, hi)
    sc = dam_break(int(dims[0]), int(dims[1]), int(dims[2]), tuple(box), scene_id=scene_id,
                   origin=tuple(origin), n_keep=n)
    sc.meta["aspect"] = tuple(aspect)
    return sc


def config4(n_scenes: int = 256, scale: float = 1.0) -> list:
    """Batched workload: n_scenes scenes, N log-uniform in [4096, 65536]."""
    rng = rng_for(4)
    scenes = []
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(4096), math.log(65536))) * scale))
        scenes.append(_random_scene(rng, 1000 + s, max(n, 1)))
    return scenes


def config5_requests(n_requests: int, rate_hz: float, seed_id: int = 5, min_n: int = 8192,
                     max_n: int = 262144, min_h: int = 60, max_h: int = 600) -> list:
    """Served stream: Poisson arrivals at rate_hz; N log-uniform in [min_n, max_n];
    horizons uniform in {min_h..max_h}.  Returns [(arrival_s, Scene, horizon)]."""
    rng = rng_for(seed_id)
    t = 0.0
    out = []
    for r in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        n = int(round(math.exp(rng.uniform(math.log(min_n), math.log(max_n)))))
        horizon = int(rng.integers(min_h, max_h + 1))
        out.append((t, _random_scene(rng, 100000 + r, n), horizon))
    return out
