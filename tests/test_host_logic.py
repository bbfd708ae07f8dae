"""Host-side logic without a GPU: scene generators, replica sharding (with a
2-rank gloo process group), parameter plumbing."""
import os
import socket

import numpy as np
import pytest

from ssf_pbf_cuda_gb300 import replicas, scenes


def test_splitmix_and_seeds_are_stable():
    assert scenes.splitmix64(0) == 0xE220A8397B1DCDAF
    assert scenes.scene_seed(0) != scenes.scene_seed(1)
    a = scenes.rng_for(5).uniform(size=4)
    b = scenes.rng_for(5).uniform(size=4)
    assert np.array_equal(a, b)


def test_config1_shape_and_jitter():
    sc = scenes.config1()
    assert sc.n == 32768 and sc.domain_end == (4.0, 2.0, 2.0)
    lat = scenes.lattice(32, 32, 32, 0.05, (0.05, 0.05, 0.05))
    d = np.abs(sc.x - lat)
    assert d.max() <= 0.01 * scenes.H + 1e-6 and d.max() > 0.005 * scenes.H
    assert sc.area == ((-0.1, -0.1, -0.1), (4.1, 2.1, 2.1))


def test_config2_and_config3_sizes():
    sc = scenes.config2()
    assert sc.n == 1048576 and sc.grid == (256, 128, 64)
    x, grid, cw = scenes.config3("blobs", n=64 * 1024)
    assert x.shape == (64 * 1024, 3) and grid == (256, 128, 128) and cw == scenes.H
    L = (64 * 1024) ** (1 / 3) * scenes.SPACING
    assert x.min() >= 0 and x.max() <= L + 1e-5


def test_config4_distribution_and_clearance():
    scs = scenes.config4(32)
    ns = np.array([s.n for s in scs])
    assert ns.min() >= 4096 and ns.max() <= 65536
    for s in scs:
        box = np.array(s.domain_end)
        assert (s.x.min(axis=0) >= scenes.H - 0.01 * scenes.H - 1e-5).all()
        assert (s.x.max(axis=0) <= box - scenes.H + 0.01 * scenes.H + 1e-5).all()
    assert scenes.config4(32)[7].x.tobytes() == scs[7].x.tobytes()


def test_config5_requests_poisson():
    reqs = scenes.config5_requests(50, rate_hz=100.0, max_n=20000, min_n=8192)
    t = np.array([r[0] for r in reqs])
    assert np.all(np.diff(t) > 0)
    hz = np.array([r[2] for r in reqs])
    assert hz.min() >= 60 and hz.max() <= 600


def test_assign_scenes_balances():
    sizes = [5, 9, 1, 7, 3, 8, 2, 6]
    parts = replicas.assign_scenes(sizes, 3)
    assert sorted(i for p in parts for i in p) == list(range(8))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)


def test_job_throughput_uses_slowest_rank():
    assert replicas.job_throughput([100, 100], 10, [1.0, 2.0]) == pytest.approx(2000 / 2e-3)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    scs = replicas.rank_scenes(4, rank, world)
    n = torch.tensor([float(sum(s.n for s in scs))])
    first = torch.tensor([float(scs[0].x[0, 0])])
    ms = torch.tensor([10.0 + rank])
    allv = [torch.zeros(1) for _ in range(world)]
    dist.all_gather(allv, first)
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    tot = n.clone()
    dist.all_reduce(tot)
    dist.barrier()
    q.put((rank, float(n), [float(a) for a in allv], float(ms), float(tot)))
    dist.destroy_process_group()


def test_replicas_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, n0, firsts, ms0, tot0), (r1, n1, _, ms1, tot1) = res
    assert firsts[0] != firsts[1]            # ranks run different scenes
    assert ms0 == ms1 == 11.0                # max over ranks
    assert tot0 == tot1 == n0 + n1           # whole-job particle count
    assert n0 == sum(s.n for s in replicas.rank_scenes(4, 0, 2))


def test_oracle_side_params_equal_the_librarys(oracle, lib):
    """The benchmark's CPU reference arm builds its parameters in oracle/params.py
    so that it never loads the product library; they must be the library's
    (pbf_params_init, config overrides, calcGridSize) field for field."""
    from oracle import params as OP
    from ssf_pbf_cuda_gb300 import api
    a, b = OP.config_params(), api.config_params()
    assert sorted(a) == sorted(b)
    for k in a:
        assert np.allclose(np.float32(a[k]), np.float32(b[k])), k
    for sc in scenes.config4(12) + [scenes.config1(), scenes.config2()]:
        p_lib = sc.params(api.config_params())
        p_lib["grid_size"] = list(api.resolve_grid(p_lib, sc.domain_end))
        assert OP.scene_params(sc)["grid_size"] == p_lib["grid_size"]


def test_reference_arm_does_not_load_the_library(tmp_path):
    """bench.py --impl reference runs the oracle only: after a (tiny) run the
    process has no mapping of libpbf103.so."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import argparse, bench; "
            "bench.run_reference(argparse.Namespace(scenes=2, steps=1, warmup=1, gpus=1)); "
            "maps = open('/proc/self/maps').read(); "
            "print('LIB' if 'libpbf103' in maps else 'CLEAN', 'ORACLE' if 'libpbf_oracle' in maps else '')")
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert out.returncode == 0, out.stderr[-2000:]
    last = out.stdout.strip().splitlines()[-1]
    assert last.split() == ["CLEAN", "ORACLE"], out.stdout[-2000:]
    import json
    line = json.loads(out.stdout.strip().splitlines()[-2])
    assert line["impl"] == "reference" and line["config"]["particles_per_gpu"] > 0
