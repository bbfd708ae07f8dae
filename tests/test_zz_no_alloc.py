"""pbf_cell_sort_noalloc: the neighbour-search sort for callers that cannot
allocate device memory (code under CUDA-graph capture, plug-ins whose host
owns all device allocations, real-time paths).

Its output must equal what the allocating path produces: pbf_one_step with
zero velocity and gravity and no iterations predicts x* = x, and its debug
getter returns the same stable permutation and cell ranges.  Two calls in a
row check that the shared fixed scratch starts clean on every call.  This
file is collected last so a failure here comes after every other test ran.
"""
import ctypes

import numpy as np
import pytest

from ssf_pbf_cuda_gb300 import api
from ssf_pbf_cuda_gb300._lib import check

pytestmark = pytest.mark.gpu


def allocating_sort(x, grid, cw):
    p = api.default_params(body_force=[0.0, 0.0, 0.0], grid_size=list(grid), cell_width=cw,
                           smoothing_length=cw)
    part = api.PbfParticle(p, len(x), (1.0, 1.0, 1.0))
    part.set_particles(x, np.zeros_like(x))
    big = 1e30
    api.one_step(part, None, ((-big,) * 3, (big,) * 3), 0)
    d = part.neighbor_debug()
    return d["perm"], d["cell_start"], d["cell_end"]


def noalloc_sort(lib, x, grid, cw):
    import torch
    n = len(x)
    C = int(np.prod(grid))
    xd = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    perm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    cs = torch.empty(C, dtype=torch.int32, device="cuda")
    ce = torch.empty(C, dtype=torch.int32, device="cuda")
    g = (ctypes.c_uint32 * 3)(*grid)
    stream = torch.cuda.current_stream().cuda_stream
    check(lib.pbf_cell_sort_noalloc(xd.data_ptr(), n, float(cw), g, perm.data_ptr(), cs.data_ptr(), ce.data_ptr(),
                                    stream), "pbf_cell_sort_noalloc")
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
    return u(perm)[:n], u(cs), u(ce)


def test_noalloc_sort_matches_allocating_path_twice(lib, gpu):
    rng = np.random.default_rng(2026)
    pile = rng.uniform(0.0, 1.6, size=(60000, 3)).astype(np.float32)
    pile[:30000] = rng.uniform(0.81, 0.89, size=(30000, 3))  # one bucket of 30,000 (> 4,096) entries
    cases = [
        (rng.uniform(-0.2, 1.8, size=(20000, 3)).astype(np.float32), (16, 16, 8), 0.1),
        (rng.normal(0.6, 0.2, size=(7777, 3)).astype(np.float32), (32, 16, 16), 0.07),
        (pile, (16, 16, 16), 0.1),
    ]
    for x, grid, cw in cases:  # two calls in a row on the shared scratch
        want = allocating_sort(x, grid, cw)
        got = noalloc_sort(lib, x, grid, cw)
        for a, b in zip(got, want):
            assert np.array_equal(a, np.asarray(b, np.uint32))


def test_noalloc_rejects_sizes_beyond_the_scratch(lib, gpu):
    g = (ctypes.c_uint32 * 3)(1024, 1024, 1)  # 2^20 cells > the fixed maximum
    assert lib.pbf_cell_sort_noalloc(None, 0, 0.1, g, None, ctypes.c_void_p(1), ctypes.c_void_p(1), None) == 4
    g = (ctypes.c_uint32 * 3)(8, 8, 8)
    assert lib.pbf_cell_sort_noalloc(ctypes.c_void_p(1), 262145, 0.1, g, ctypes.c_void_p(1), ctypes.c_void_p(1),
                                     ctypes.c_void_p(1), None) == 4
