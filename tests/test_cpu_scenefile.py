"""The drop-in boundary from the reference side: the reference's own parse
of each golden scene, flattened into the C ABI's scene description by the
reference-side flattener (oracle/refbuild/pov_flatten.cpp, compiled against
the reference's headers; dumped by tests/golden/make_golden.py as
<case>.pgsf.gz), against the description the project's scene generator
(povray_gb300/scenes.py) builds for the same SDL, field by field.

Tolerances (written here, applied below):
  ids, counts, types, flags, links   exact
  camera vectors                     1e-15 relative (the parser's FP64 math)
  object parameters, transforms      1e-12
  material, light and media floats   1e-7 (single-precision fields)
  patterns and normals               by content: ids exact, matrices 1e-12,
                                     single-precision parameters and
                                     colour maps 1e-7
  mesh vertices and indices          exact; normals 1e-6 (the parser
                                     normalises normal_vectors in FP64 and
                                     stores them as floats)
Materials are compared per object after resolving inheritance (a CSG
child without a texture takes its parent's, Parser::Post_Process,
parser.cpp:9025-9030), because the two sides number shared textures
differently.
"""
import ctypes as C
import os
import struct

import numpy as np
import pytest

from povray_gb300 import abi
from povray_gb300.scenefile import ParsedScene
from tests.golden.make_golden import SCENE_FILE_CASES, cases, radiosity_cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _scenes():
    allc = dict((k, v[0]) for k, v in cases().items())
    allc.update(radiosity_cases())
    return allc


def _close(tag, x, y, tol, skip=()):
    for name, _ in x._fields_:
        if name in skip:
            continue
        a, b = getattr(x, name), getattr(y, name)
        if isinstance(a, C._Pointer):
            continue
        av = np.array(a[:] if hasattr(a, "__len__") else a, dtype=float)
        bv = np.array(b[:] if hasattr(b, "__len__") else b, dtype=float)
        assert av.shape == bv.shape and np.allclose(av, bv, rtol=tol, atol=tol), (tag, name, av, bv)


def _pattern_close(i, pa, pb):
    """A pattern record: ids and counts exact, matrices and FP64 parameters
    1e-12, the single-precision ones (wave, turbulence omega/lambda,
    agate_turb, colour map) 1e-7."""
    from povray_gb300 import abi
    for k in ("type", "noise_generator", "num_entries", "wave_type", "has_turbulence"):
        assert getattr(pa, k) == getattr(pb, k), (i, k, getattr(pa, k), getattr(pb, k))
    # the kind's own fields only where the kind reads them
    skip = ["type", "noise_generator", "num_entries", "wave_type", "octaves", "has_turbulence", "values", "colours",
            "frequency", "phase", "exponent", "omega", "lambda", "agate_turb", "turbulence"]
    if pa.type != abi.POV_PATTERN_GRADIENT:
        skip.append("gradient")
    if pa.type != abi.POV_PATTERN_BRICK:
        skip += ["brick_size", "mortar"]
    if pa.type not in (abi.POV_PATTERN_SPIRAL1, abi.POV_PATTERN_SPIRAL2):
        skip.append("arms")
    if pa.type != abi.POV_PATTERN_CRACKLE:
        skip += ["crackle_form", "crackle_metric", "crackle_offset", "crackle_solid"]
    if pa.type != abi.POV_PATTERN_QUILTED:
        skip += ["control0", "control1"]
    _close("pattern of object %d" % i, pa, pb, 1e-12, skip=tuple(skip))
    single = ["frequency", "phase", "exponent"]
    if pa.has_turbulence:
        assert pa.octaves == pb.octaves, i
        assert np.allclose(pa.turbulence[:], pb.turbulence[:], rtol=1e-12, atol=1e-12), i
        single += ["omega", "lambda"]
    if pa.type == abi.POV_PATTERN_AGATE:
        single.append("agate_turb")
    for k in single:
        assert abs(getattr(pa, k) - getattr(pb, k)) <= 1e-7 * max(1.0, abs(getattr(pa, k))), (i, k)
    n = pa.num_entries
    assert np.allclose(pa.values[:n], pb.values[:n], atol=1e-7), i
    assert np.allclose(np.array(pa.colours[:n]), np.array(pb.colours[:n]), atol=1e-7), i


def _material_of(d, i):
    o = d.objects[i]
    while o.material < 0 and o.parent >= 0:
        o = d.objects[o.parent]
    return o.material


@pytest.mark.parametrize("case", SCENE_FILE_CASES)
def test_reference_flattened_scene_equals_generator_desc(case):
    scene = _scenes()[case]
    a, _keep = scene.desc()
    ps = ParsedScene(os.path.join(GOLDEN, case + ".pgsf.gz"), scene.width, scene.height)
    b, _keep2 = ps.desc()
    _close("camera", a.camera, b.camera, 1e-15)
    for k in ("max_trace_level", "language_version", "num_objects", "num_lights", "num_meshes", "num_medias",
              "num_patterns", "num_normals"):
        assert getattr(a, k) == getattr(b, k), k
    assert abs(a.adc_bailout - b.adc_bailout) <= 1e-9
    assert list(a.background) == list(b.background)
    assert list(a.ambient_light) == list(b.ambient_light)
    assert a.radiosity.enabled == b.radiosity.enabled
    if a.radiosity.enabled:
        _close("radiosity", a.radiosity, b.radiosity, 1e-12)
    for i in range(a.num_objects):
        oa, ob = a.objects[i], b.objects[i]
        for k in ("type", "flags", "parent", "first_child", "num_children", "mesh", "media"):
            assert getattr(oa, k) == getattr(ob, k), (i, k, getattr(oa, k), getattr(ob, k))
        assert np.allclose(oa.p[:], ob.p[:], rtol=1e-12, atol=1e-12), (i, oa.p[:], ob.p[:])
        assert np.allclose(oa.trans[:], ob.trans[:], rtol=1e-12, atol=1e-12), i
        ma, mb = _material_of(a, i), _material_of(b, i)
        assert (ma >= 0) == (mb >= 0), i
        if ma >= 0:
            A, Bm = a.materials[ma], b.materials[mb]
            assert (A.pattern > 0) == (Bm.pattern > 0) and (A.normal > 0) == (Bm.normal > 0), i
            # pattern and normal records are compared by content (the two
            # sides number them in different orders); a pattern pigment's
            # own colour is unused
            skip = ("pattern", "normal") + (("pigment",) if A.pattern > 0 else ())
            _close("material of object %d" % i, A, Bm, 1e-7, skip=skip)
            if A.pattern > 0:
                _pattern_close(i, a.patterns[A.pattern - 1], b.patterns[Bm.pattern - 1])
            if A.normal > 0:
                na, nb = a.normals[A.normal - 1], b.normals[Bm.normal - 1]
                _close("normal of object %d" % i, na, nb, 1e-12, skip=("pattern", "amount", "delta"))
                assert abs(na.amount - nb.amount) <= 1e-7 and abs(na.delta - nb.delta) <= 1e-7, i
                _pattern_close(i, a.patterns[na.pattern - 1], b.patterns[nb.pattern - 1])
    # interiors: the same content per object, and the same sharing (which
    # objects have one interior between them)
    assert abs(a.atmosphere_ior - b.atmosphere_ior) == 0.0
    for i in range(a.num_objects):
        ia, ib = a.object_interior[i], b.object_interior[i]
        assert ia > 0 and ib > 0, i
        _close("interior of object %d" % i, a.interiors[ia - 1], b.interiors[ib - 1], 1e-7)
        for j in range(i):
            assert (a.object_interior[j] == ia) == (b.object_interior[j] == ib), (i, j)
    for i in range(a.num_lights):
        _close("light %d" % i, a.lights[i], b.lights[i], 1e-7)
    for i in range(a.num_medias):
        _close("media %d" % i, a.medias[i], b.medias[i], 1e-7)
    for i, m in enumerate(scene.meshes):
        pm = ps.meshes[i]
        assert np.array_equal(m.vertices.ravel(), pm["vertices"])
        assert np.array_equal(m.faces.ravel(), pm["faces"])
        if m.normals is not None:
            assert np.allclose(m.normals.ravel(), pm["normals"], atol=1e-6)
            assert np.array_equal(m.faces.ravel(), pm["normal_indices"])


def test_scene_file_rejects_damage(tmp_path):
    src = os.path.join(GOLDEN, "spheres_plane_320x240.pgsf.gz")
    import gzip
    data = gzip.open(src, "rb").read()
    bad = tmp_path / "bad.pgsf"
    bad.write_bytes(data[:-5])
    with pytest.raises(ValueError):
        ParsedScene(str(bad), 320, 240)
    bad.write_bytes(b"XXXX" + data[4:])
    with pytest.raises(ValueError):
        ParsedScene(str(bad), 320, 240)
    # a file written for another layout of the C structs
    bad.write_bytes(data[:8] + struct.pack("<I", abi.POV_GPU_ABI_VERSION + 1) + data[12:])
    with pytest.raises(ValueError):
        ParsedScene(str(bad), 320, 240)
