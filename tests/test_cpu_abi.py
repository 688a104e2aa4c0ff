"""The C ABI: struct layouts match include/povgpu.h, the library loads and
exports every declared entry point, and scene validation (host logic that
runs before any device call) rejects what the GPU path does not support."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
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


def test_transparency_validation(gpu_lib):
    """Transparent surfaces: a plain pigment that filters or transmits
    (reflection beside it, fresnel or not, with or without
    conserve_energy), interiors without dispersion or caustics, no
    radiosity or area lights in the scene, the camera inside no object;
    fresnel reflection and conserve_energy on transparent surfaces only.
    Rejected before any device work."""
    ok = (abi.POV_GPU_OK, abi.POV_GPU_E_NODEVICE, abi.POV_GPU_E_CUDA)

    def fresh():
        return scenes.glass_spheres(32, 24).desc()
    desc, keep = fresh()
    assert _create(gpu_lib, desc)[0] in ok
    glass = [i for i in range(desc.num_materials) if desc.materials[i].pigment[3] > 0.0][0]
    desc, keep = fresh()
    desc.materials[glass].reflection_max[0] = 0.2        # a second secondary ray
    desc.materials[glass].reflection_fresnel = 1
    desc.materials[glass].conserve_energy = 1
    assert _create(gpu_lib, desc)[0] in ok
    opaque = [i for i in range(desc.num_materials) if desc.materials[i].pigment[3] == 0.0
              and desc.materials[i].pigment[4] == 0.0][0]
    for field in ("reflection_fresnel", "conserve_energy"):   # they need the surface's interior
        desc, keep = fresh()
        setattr(desc.materials[opaque], field, 1)
        assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED, field
    desc, keep = fresh()
    desc.interiors[0].dispersion = 1.02
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.interiors[0].caustics = 0.5
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    rdesc, rkeep = scenes.radiosity_room(32, 24, n_spheres=4).desc()
    desc.radiosity = rdesc.radiosity                     # valid radiosity settings
    assert desc.radiosity.enabled == 1
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.lights[0].kind = abi.POV_LIGHT_AREA
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.object_interior[3] = desc.num_interiors + 1     # no such interior
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_INVALID
    desc, keep = fresh()
    sph = [i for i in range(desc.num_objects) if desc.objects[i].type == abi.POV_OBJ_SPHERE
           and desc.objects[i].parent < 0][0]
    for k in range(3):
        desc.camera.location[k] = desc.objects[sph].p[k]  # the camera inside a sphere
    assert _create(gpu_lib, desc) == (abi.POV_GPU_E_UNSUPPORTED, sph)
    # an opaque scene is not held to these rules
    desc, keep = scenes.spheres_plane(32, 24, n_spheres=4).desc()
    for k in range(3):
        desc.camera.location[k] = desc.objects[1].p[k]
    assert _create(gpu_lib, desc)[0] in ok


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


def test_media_container_validation(gpu_lib):
    """Media containers: hollow boxes whose surface only transmits, method 3
    without jitter, intervals and AA level within the GPU path's limits,
    point lights only, camera outside; rejected before any device work."""
    def fresh():
        return scenes.media_spheres(32, 24, n_spheres=2).desc()
    desc, keep = fresh()
    box = [i for i in range(desc.num_objects) if desc.objects[i].media > 0][0]
    assert _create(gpu_lib, desc)[0] in (abi.POV_GPU_OK, abi.POV_GPU_E_NODEVICE, abi.POV_GPU_E_CUDA)
    desc, keep = fresh()
    desc.objects[box].flags &= ~abi.POV_FLAG_HOLLOW     # a media object that is not hollow
    assert _create(gpu_lib, desc) == (abi.POV_GPU_E_UNSUPPORTED, box)
    desc, keep = fresh()
    desc.medias[0].jitter = 0.5                          # jitter draws on the reference's RNG
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.medias[0].intervals = 1000                      # above the per-segment slots
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.medias[0].method = 2
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.camera.location[0], desc.camera.location[1], desc.camera.location[2] = 0.0, 0.0, 0.0   # inside the box
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.objects[box].media = 5                          # no such media
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_INVALID


def test_pattern_validation(gpu_lib):
    """Pattern pigments: known pattern types, 1..16 ascending colour map
    entries (checker exactly 2), noise generators 1..3, material indices in
    range."""
    def fresh():
        return scenes.textured_spheres(32, 24, n_spheres=4).desc()
    desc, keep = fresh()
    desc.patterns[0].type = 42
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.patterns[1].noise_generator = 7
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.patterns[1].values[0], desc.patterns[1].values[1] = 0.8, 0.2   # descending map
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_INVALID
    desc, keep = fresh()
    desc.patterns[0].num_entries = 3                      # checker takes two colours
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.materials[0].pattern = desc.num_patterns + 1
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_INVALID


def test_normal_validation(gpu_lib):
    """Normal perturbations: a pattern index in range whose pattern is not a
    checker, a positive delta, a finite amount; material indices in range; a
    pigment may not read a normal-only pattern."""
    def fresh():
        return scenes.bumpy_spheres(32, 24, n_spheres=4).desc()
    desc, keep = fresh()
    assert desc.num_normals == 5 and desc.materials[1].normal == 2
    desc.normals[1].pattern = desc.num_patterns + 1
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_INVALID
    desc, keep = fresh()
    desc.normals[1].delta = 0.0
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.normals[1].amount = float("nan")
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.patterns[desc.normals[1].pattern - 1].type = abi.POV_PATTERN_CHECKER
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.materials[0].normal = desc.num_normals + 1
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_INVALID
    desc, keep = fresh()
    desc.materials[0].pattern = desc.normals[0].pattern   # a pigment reading bumps
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED


def test_discrete_pattern_validation(gpu_lib):
    """Colour lists: square takes 4 entries, triangular and cubic 6,
    hexagon 3; a normal cannot read a discrete pattern (the reference
    parses those as normal maps)."""
    def fresh():
        return scenes.shaped_spheres(32, 24, n_spheres=11).desc()
    desc, keep = fresh()
    kinds = {desc.patterns[i].type: i for i in range(desc.num_patterns)}
    for t, n in ((abi.POV_PATTERN_SQUARE, 4), (abi.POV_PATTERN_TRIANGULAR, 6), (abi.POV_PATTERN_CUBIC, 6),
                 (abi.POV_PATTERN_HEXAGON, 3)):
        assert desc.patterns[kinds[t]].num_entries == n
        desc, keep = fresh()
        desc.patterns[kinds[t]].num_entries = n - 1
        assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED, t
    desc, keep = fresh()
    desc.normals[0].pattern = kinds[abi.POV_PATTERN_HEXAGON] + 1
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED


def test_normal_sdl_and_desc_agree():
    """The normal's SDL carries the amount right after the pattern and its
    modifiers after; the descriptor's forward matrix and the pattern's
    inverse are each other's inverse."""
    s = scenes.bumpy_spheres(32, 24, n_spheres=12)
    sdl = s.sdl()
    assert "normal { bumps, 0.3 scale <0.5,0.5,0.5> }" in sdl
    assert "no_bump_scale" in sdl and "accuracy 0.05" in sdl
    desc, keep = s.desc()
    for i in range(desc.num_normals):
        nm = desc.normals[i]
        pt = desc.patterns[nm.pattern - 1]
        fwd = np.array(nm.matrix[:]).reshape(4, 4)
        inv = np.array(pt.inverse[:]).reshape(4, 4)
        assert np.allclose(fwd @ inv, np.eye(4), atol=1e-12)


def test_light_source_validation(gpu_lib):
    """Light sources: Light_Type 0-4 and kind point/area (else invalid); a
    spotlight, cylinder or parallel light needs point_at away from its
    centre; area lights take no parallel beam; scenes with media containers
    take plain point lights only.  The oracle applies the same rules."""
    from oracle.pyoracle import Oracle
    ok = (abi.POV_GPU_OK, abi.POV_GPU_E_NODEVICE, abi.POV_GPU_E_CUDA)
    spot, cyl, par, fill, area = range(5)

    def fresh():
        return scenes.light_types(32, 24).desc()
    desc, keep = fresh()
    assert [desc.lights[i].light_type for i in range(5)] == [abi.POV_LIGHT_TYPE_SPOT, abi.POV_LIGHT_TYPE_CYLINDER,
                                                               abi.POV_LIGHT_TYPE_POINT, abi.POV_LIGHT_TYPE_SHADOWLESS,
                                                               abi.POV_LIGHT_TYPE_SPOT]
    assert desc.lights[cyl].parallel == 1 and desc.lights[par].parallel == 1
    assert _create(gpu_lib, desc)[0] in ok
    desc, keep = fresh()
    desc.lights[fill].light_type = 5
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_INVALID
    desc, keep = fresh()
    desc.lights[spot].points_at[:] = list(desc.lights[spot].center)
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.lights[area].light_type = abi.POV_LIGHT_TYPE_CYLINDER
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    desc, keep = fresh()
    desc.lights[area].parallel = 1
    assert _create(gpu_lib, desc)[0] == abi.POV_GPU_E_UNSUPPORTED
    Oracle(scenes.light_types(32, 24))
    for change in (dict(beam="spotlight", point_at=(0.0, 0.0, 0.0)), dict(fade_distance=5.0, fade_power=2.0),
                   dict(shadowless=True)):
        m = scenes.media_spheres(32, 24, n_spheres=4)
        m.lights[0].update(change)
        d, k = m.desc()
        assert _create(gpu_lib, d)[0] == abi.POV_GPU_E_UNSUPPORTED, change
        with pytest.raises(abi.PovGpuError):
            Oracle(m)
    bad = scenes.light_types(32, 24)
    bad.lights[area]["beam"] = "cylinder"
    with pytest.raises(abi.PovGpuError):
        Oracle(bad)


def test_object_ray_kind_flags_are_refused(gpu_lib):
    """no_shadow, no_reflection and no_image objects are refused at create
    (the GPU path does not filter objects by ray kind), with the object's
    index; the other flags pass."""
    ok = (abi.POV_GPU_OK, abi.POV_GPU_E_NODEVICE, abi.POV_GPU_E_CUDA)
    for flag in (abi.POV_FLAG_NO_SHADOW, abi.POV_FLAG_NO_REFLECTION, abi.POV_FLAG_NO_IMAGE):
        desc, keep = scenes.spheres_plane(32, 24, n_spheres=4).desc()
        desc.objects[2].flags |= flag
        assert _create(gpu_lib, desc) == (abi.POV_GPU_E_UNSUPPORTED, 2), flag
    desc, keep = scenes.spheres_plane(32, 24, n_spheres=4).desc()
    desc.objects[2].flags |= abi.POV_FLAG_DOUBLE_ILLUM
    assert _create(gpu_lib, desc)[0] in ok


def test_oracle_rejects_the_same_scenes():
    """The oracle applies the same rules as the library."""
    from oracle.pyoracle import Oracle
    s = scenes.textured_spheres(32, 24, n_spheres=4)
    Oracle(s)     # accepted
    bad = scenes.textured_spheres(32, 24, n_spheres=4)
    bad.materials[1].pattern.kind = "checker"   # a checker with a three-entry map
    with pytest.raises(abi.PovGpuError):
        Oracle(bad)
    Oracle(scenes.bumpy_spheres(32, 24, n_spheres=4))
    bad = scenes.bumpy_spheres(32, 24, n_spheres=4)
    bad.materials[1].normal.accuracy = 0.0           # the slope's delta must be positive
    with pytest.raises(abi.PovGpuError):
        Oracle(bad)


def test_timeout_argument_validation(gpu_lib):
    """pov_gpu_set_timeout validates on the host before touching the device:
    no scene, a negative or a non-finite limit are POV_GPU_E_INVALID."""
    assert gpu_lib.pov_gpu_set_timeout(None, 1.0) == abi.POV_GPU_E_INVALID
    assert gpu_lib.pov_gpu_set_timeout(None, -1.0) == abi.POV_GPU_E_INVALID
    assert gpu_lib.pov_gpu_set_timeout(None, float("nan")) == abi.POV_GPU_E_INVALID
    assert b"wait limit" in gpu_lib.pov_gpu_error_string(abi.POV_GPU_E_TIMEOUT)
