"""The C ABI: struct layouts match include/povgpu.h, the library loads and
exports every declared entry point, and scene validation (host logic that
runs before any device call) rejects what the GPU path does not support."""
import ctypes as C
import os
import re
import subprocess

import pytest

from povray_gb300 import abi, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "povgpu.h")


def _declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(pov_gpu_\w+)\s*\(", text, re.M)))


def test_header_declares_the_exports():
    assert _declared_functions() == sorted(abi.EXPORTS)


def test_library_exports_every_declared_symbol(gpu_lib):
    for name in _declared_functions():
        assert hasattr(gpu_lib, name), name
    assert gpu_lib.pov_gpu_abi_version() == abi.POV_GPU_ABI_VERSION


def test_error_strings(gpu_lib):
    for code in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert gpu_lib.pov_gpu_error_string(code)
    assert gpu_lib.pov_gpu_error_string(-99) == b"unknown status"


def test_struct_layout_matches_header(tmp_path):
    """sizeof/offsetof of every field, as gcc sees the header, equal the ctypes mirror."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "povgpu.h"', "int main(void){"]
    for sname, cls in abi.STRUCTS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (sname, sname))
        for fname, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (sname, fname, sname, fname))
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    got = dict(l.split() for l in out if l.strip())
    for sname, cls in abi.STRUCTS.items():
        assert int(got[sname]) == C.sizeof(cls), sname
        for fname, _ in cls._fields_:
            assert int(got["%s.%s" % (sname, fname)]) == getattr(cls, fname).offset, (sname, fname)


def _create(lib, desc):
    h = C.c_void_p()
    bad = C.c_int32(-1)
    st = lib.pov_gpu_scene_create(C.byref(desc), C.byref(h), C.byref(bad))
    if st == 0:
        lib.pov_gpu_scene_destroy(h)
    return st, bad.value


def test_unsupported_object_is_rejected_at_setup(gpu_lib):
    s = scenes.spheres_plane(32, 24, n_spheres=4)
    desc, keep = s.desc()
    desc.objects[2].type = 99          # an object type outside the GPU path
    st, bad = _create(gpu_lib, desc)
    assert st == abi.POV_GPU_E_INVALID and bad == 2


def test_transformed_primitive_is_unsupported(gpu_lib):
    s = scenes.spheres_plane(32, 24, n_spheres=4)
    desc, keep = s.desc()
    desc.objects[1].flags |= abi.POV_FLAG_HAS_TRANS
    st, bad = _create(gpu_lib, desc)
    assert st == abi.POV_GPU_E_UNSUPPORTED and bad == 1


def test_transparent_pigment_is_unsupported(gpu_lib):
    s = scenes.spheres_plane(32, 24, n_spheres=4)
    desc, keep = s.desc()
    desc.materials[0].pigment[4] = 0.5    # transmit: needs refraction
    st, _ = _create(gpu_lib, desc)
    assert st == abi.POV_GPU_E_UNSUPPORTED


def test_bad_mesh_index_is_invalid(gpu_lib):
    s = scenes.mesh_spheres(32, 18, mesh_n=4, n_spheres=2)
    desc, keep = s.desc()
    keep[0].faces[0, 0] = 10 ** 6
    st, _ = _create(gpu_lib, desc)
    assert st == abi.POV_GPU_E_INVALID


def test_wrong_abi_version_is_invalid(gpu_lib):
    s = scenes.spheres_plane(32, 24, n_spheres=4)
    desc, keep = s.desc()
    desc.abi_version = 999
    st, _ = _create(gpu_lib, desc)
    assert st == abi.POV_GPU_E_INVALID


def test_null_arguments(gpu_lib):
    assert gpu_lib.pov_gpu_scene_create(None, None, None) == abi.POV_GPU_E_INVALID
    assert gpu_lib.pov_gpu_trace_blocks(None, None, 0, None, None, None) == abi.POV_GPU_E_INVALID
    assert gpu_lib.pov_gpu_trace_rays(None, None, None, 0, None) == abi.POV_GPU_E_INVALID
    assert gpu_lib.pov_gpu_trace_rays_static(None, None, None, 0, None) == abi.POV_GPU_E_INVALID
    gpu_lib.pov_gpu_scene_destroy(None)


def test_csg_validation(gpu_lib):
    """CSG: leaf children only; a mesh child or nested CSG is unsupported."""
    s = scenes.csg_torus_grid(32, 18, n=2, antialias=None)
    desc, keep = s.desc()
    assert desc.objects[0].type == abi.POV_OBJ_INTERSECTION and desc.objects[1].parent == 0
    desc.objects[1].type = abi.POV_OBJ_MESH
    desc.objects[1].mesh = 0
    st, bad = _create(gpu_lib, desc)
    assert st in (abi.POV_GPU_E_INVALID, abi.POV_GPU_E_UNSUPPORTED)
    desc, keep = s.desc()
    desc.objects[2].parent = 5           # child pointing at the wrong parent
    st, bad = _create(gpu_lib, desc)
    assert st == abi.POV_GPU_E_INVALID


def test_torus_requires_its_transform(gpu_lib):
    s = scenes.csg_torus_grid(32, 18, n=2, antialias=None)
    desc, keep = s.desc()
    tor = [i for i in range(desc.num_objects) if desc.objects[i].type == abi.POV_OBJ_TORUS][0]
    desc.objects[tor].flags &= ~abi.POV_FLAG_HAS_TRANS
    st, bad = _create(gpu_lib, desc)
    assert st == abi.POV_GPU_E_UNSUPPORTED and bad == tor
