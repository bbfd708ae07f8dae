"""The reference's own CUDA step (yodaplusplus/ssf_pbf_cuda, built from its
sources by oracle/ref_build.py) timed on this GPU beside the plain step of
this library, on identical inputs and parameters, and its outputs compared
with this library's at these sizes (32,768 and 1,048,576 particles): the
reference's IEEE build's step against this library's step from the same
input, as the golden fixtures are compared (sort-invariant integers,
neighbour sets and positions by particle id, 1e-5 relative).  Runs only
where the reference's sources were prepared (oracle/_ref/src); scenes are
checked against the reference's hazards first (tests/golden/make_golden.py)."""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import ref_build
from ssf_pbf_cuda_gb300 import api, scenes
from tests import helpers as H
from tests.golden import make_golden as MG

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.path.isdir(ref_build.SRC), reason="reference sources not prepared here")]

REPS = 20


def ref_params(grid=None):
    p = MG.reflike()
    if grid is not None:
        p["grid_size"] = list(grid)
    return p


CASES = [
    # the reference's dam-break parameters (h = 1.4 s) on config 1's lattice and on config 2's;
    # grids by the reference's own calcGridSize (its driver derives them from domain_end)
    ("dam_32k", lambda: scenes.dam_break(32, 32, 32, (4.0, 2.0, 2.0), scene_id=601, h=0.07, spacing=0.05), None),
    ("dam_1m", lambda: scenes.dam_break(128, 128, 64, (16.0, 8.0, 8.0), scene_id=602, h=0.07, spacing=0.05), None),
]


@pytest.fixture(scope="module")
def ref_exe():
    return ref_build.build("fast")  # the shipped flags


@pytest.fixture(scope="module")
def ref_exe_ieee():
    return ref_build.build("ieee")  # IEEE division and square root: the parity build


@pytest.mark.parametrize("name,make,grid", CASES, ids=[c[0] for c in CASES])
def test_reference_gpu_step_time(tmp_path, gpu, ref_exe, ref_exe_ieee, name, make, grid):
    import torch
    sc = make()
    p = ref_params(grid)
    if grid is None:
        p["grid_size"] = list(api.calc_grid_size(2.0 * p["smoothing_length"], sc.domain_end))
    MG.check_hazards(sc, p, "planes", 4)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    MG.write_input(inp, sc, p, "planes", 4, sc.n)
    out = subprocess.run([ref_exe, inp, outp, str(REPS)], check=True, timeout=600, capture_output=True, text=True)
    ref_ms = float(re.search(r"ms_per_step ([0-9.eE+-]+)", out.stdout).group(1))
    ref_fast = MG.read_output(outp)
    subprocess.run([ref_exe_ieee, inp, outp], check=True, timeout=600)
    ref = MG.read_output(outp)

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    p["cell_width"] = p["smoothing_length"]
    part = api.PbfParticle(p, sc.n, sc.domain_end)
    b = api.Boundary(points_on_planes=sc.planes[0], normals_on_planes=sc.planes[1])
    xd, vd = torch.from_numpy(sc.x).to(dev), torch.from_numpy(sc.v).to(dev)
    for _ in range(3):
        part.set_particles(xd, vd, stream)
        api.one_step(part, b, sc.area, 4, stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(REPS):
        part.set_particles(xd, vd, stream)
        api.one_step(part, b, sc.area, 4, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ours_ms = e0.elapsed_time(e1) / REPS
    assert part.num == ref["num"] == ref_fast["num"]
    # the last timed step ran from the input: compare its outputs in full
    x, v = part.get_particles()
    ours = part.neighbor_debug()
    ours.update(x=x, v=v)
    rep = H.compare_to_reference(ours, ref, int(np.prod(p["grid_size"])))
    print(f"\n{name}: {sc.n} particles, 4 iterations: reference {ref_ms:.4f} ms/step "
          f"({sc.n / ref_ms / 1e3:.1f} M particle-steps/s), this library {ours_ms:.4f} ms/step "
          f"({sc.n / ours_ms / 1e3:.1f} M particle-steps/s), {ref_ms / ours_ms:.2f}x; against the reference's "
          f"outputs: {rep}")
    assert rep["neighbor_set_mismatches"] == 0
    assert rep["pos_rel_err"] <= H.POS_RTOL, rep
    assert rep["vel_abs_err"] <= H.vel_abs_tol(p["time_step"], ref["x"]), rep
    assert ours_ms < ref_ms
