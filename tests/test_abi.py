"""The C-ABI library loads and exports every function include/pbf103.h
declares; the ctypes structs match the C layouts (no GPU needed: no compute
calls are made)."""
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pbf103.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(pbf_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_the_reference_surface():
    names = declared_functions()
    for must in ("pbf_create", "pbf_destroy", "pbf_one_step", "pbf_set_particles", "pbf_add_particles",
                 "pbf_get_particles", "pbf_get_num", "pbf_boundary_create", "pbf_get_neighbor_debug",
                 "pbf_one_step_external", "pbf_batch_step", "pbf_server_submit"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_symbol():
    from ssf_pbf_cuda_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_status_strings_and_version(lib):
    assert lib.pbf_abi_version() == 1
    assert lib.pbf_status_string(0) == b"success"
    assert lib.pbf_status_string(5) == b"grid_size is too large"


def test_grid_size_and_params_without_gpu(lib):
    import ctypes

    from ssf_pbf_cuda_gb300 import _lib
    g = (ctypes.c_uint32 * 3)()
    assert lib.pbf_calc_grid_size(0.2, (ctypes.c_float * 3)(4, 2, 2), g) == 0
    assert tuple(g) == (32, 16, 16)
    assert lib.pbf_calc_grid_size(0.001, (ctypes.c_float * 3)(7, 7, 7), g) == 5
    p = _lib.PbfParams()
    assert lib.pbf_params_init(ctypes.byref(p)) == 0
    assert p.max_pair_particle_num == 30 and p.tensile_mode == 0
    out = ctypes.c_uint64()
    assert lib.pbf_scene_bytes(ctypes.byref(p), 1000, (ctypes.c_float * 3)(4, 2, 2), ctypes.byref(out)) == 0
    assert out.value > 1000 * 100


def test_create_without_device_fails_cleanly(lib):
    import ctypes

    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from ssf_pbf_cuda_gb300 import _lib
    p = _lib.PbfParams()
    lib.pbf_params_init(ctypes.byref(p))
    h = ctypes.c_void_p()
    assert lib.pbf_create(ctypes.byref(p), 10, (ctypes.c_float * 3)(1, 1, 1), 0, ctypes.byref(h)) == 9


STRUCTS = {
    "pbf_params": ("PbfParams", ["stable_density", "body_force", "max_pair_particle_num", "tensile_mode",
                                 "max_collision_passes", "cell_width", "grid_size"]),
    "pbf_server_config": ("PbfServerConfig", ["hbm_budget_bytes", "max_scenes", "max_particles", "iters", "tile"]),
    "pbf_request_desc": ("PbfRequestDesc", ["params", "domain_end", "n_planes", "plane_normals", "capacity",
                                            "horizon_steps"]),
    "pbf_completion": ("PbfCompletion", ["request_id", "num", "flags", "arrival_s", "complete_s"]),
    "pbf_server_stats": ("PbfServerStats", ["submitted", "particle_steps", "resident_scenes", "busy_s",
                                            "elapsed_s"]),
    "pbf_arrangement": ("PbfArrangement", ["kind", "axis", "origin", "end", "axis_value", "radius", "height",
                                           "space"]),
    "pbf_ssf_params": ("PbfSsfParams", ["width", "height", "projection", "view", "point_radius", "point_scale",
                                        "near_plane", "far_plane", "blur_radius", "blur_scale", "blur_passes",
                                        "splat_mode", "thickness", "clear_color"]),
}


def test_struct_layouts_match_c():
    from ssf_pbf_cuda_gb300 import _lib
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(c, "w").write("\n".join(lines))
        subprocess.run(["gcc", c, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    got = dict(line.split() for line in out.strip().splitlines())
    import ctypes
    for cname, (pyname, fields) in STRUCTS.items():
        cls = getattr(_lib, pyname)
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for f in fields:
            assert int(got[f"{cname}.{f}"]) == getattr(cls, f).offset, (cname, f)
