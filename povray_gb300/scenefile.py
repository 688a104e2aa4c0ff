"""Scene files: a PovGpuSceneDesc with all its arrays, as written by the
reference-side flattener (oracle/refbuild/pov_flatten.cpp, which walks the
SceneData the reference's parser built) -- so that a scene the reference
parsed renders through libpovgpu unchanged, without the project's own scene
generator in between.

Files may be gzip-compressed (name ending in .gz).  Format (little-endian, the C structs of include/povgpu.h laid out as the C
compiler lays them out on a 64-bit target):

    char[4]  "PGSF";  uint32 format version (2);  uint32 ABI version
    PovGpuCamera camera
    float background[4];  float ambient_light[3]
    int32 max_trace_level;  float adc_bailout;  int32 language_version
    PovGpuRadiosity radiosity
    for objects, materials, lights, medias, patterns, normals, interiors in
    that order: uint32 count, then count records of the struct
    uint32 count, then that many int32: each object's 1-based interior
    double atmosphere_ior
    uint32 mesh count, then per mesh:
        int32 num_vertices, num_normals, num_triangles, has_normal_indices
        float vertices[3 * num_vertices];  float normals[3 * num_normals]
        int32 face_indices[3 * num_triangles]
        int32 normal_indices[3 * num_triangles] (when has_normal_indices)
"""
import ctypes as C
import gzip
import struct

import numpy as np

from . import abi

MAGIC = b"PGSF"
VERSION = 2


class _Reader:
    def __init__(self, data):
        self.data = data
        self.pos = 0

    def take(self, n):
        if self.pos + n > len(self.data):
            raise ValueError("scene file truncated")
        b = self.data[self.pos:self.pos + n]
        self.pos += n
        return b

    def u32(self):
        return struct.unpack("<I", self.take(4))[0]

    def i32(self):
        return struct.unpack("<i", self.take(4))[0]

    def f32(self):
        return struct.unpack("<f", self.take(4))[0]

    def record(self, ctype):
        return ctype.from_buffer_copy(self.take(C.sizeof(ctype)))

    def records(self, ctype):
        n = self.u32()
        arr = (ctype * max(n, 1))()
        if n:
            C.memmove(arr, self.take(C.sizeof(ctype) * n), C.sizeof(ctype) * n)
        return n, arr

    def array(self, dtype, n):
        return np.frombuffer(self.take(np.dtype(dtype).itemsize * n), dtype=dtype).copy()


class ParsedScene:
    """A scene read from a scene file: what GpuScene needs from a scene
    (desc(), render_params(), width/height, radiosity) for a scene the
    reference parsed.  `width` / `height` are the image size to render at,
    which the scene file does not hold (the camera's right vector carries
    the aspect ratio the parser was given)."""

    def __init__(self, path, width, height, antialias=None):
        self.path = path
        self.width, self.height = int(width), int(height)
        self.antialias = antialias
        data = (gzip.open if str(path).endswith(".gz") else open)(path, "rb").read()
        r = _Reader(data)
        if r.take(4) != MAGIC:
            raise ValueError("not a scene file: %s" % path)
        if r.u32() != VERSION:
            raise ValueError("scene file version")
        if r.u32() != abi.POV_GPU_ABI_VERSION:
            raise ValueError("scene file written for another ABI version")
        self.camera = r.record(abi.PovGpuCamera)
        self.background = [r.f32() for _ in range(4)]
        self.ambient_light = [r.f32() for _ in range(3)]
        self.max_trace_level = r.i32()
        self.adc_bailout = r.f32()
        self.language_version = r.i32()
        self.radiosity_desc = r.record(abi.PovGpuRadiosity)
        self.num_objects, self.objects = r.records(abi.PovGpuObject)
        self.num_materials, self.materials = r.records(abi.PovGpuMaterial)
        self.num_lights, self.lights = r.records(abi.PovGpuLight)
        self.num_medias, self.medias = r.records(abi.PovGpuMedia)
        self.num_patterns, self.patterns = r.records(abi.PovGpuPattern)
        self.num_normals, self.normals = r.records(abi.PovGpuNormal)
        self.num_interiors, self.interiors = r.records(abi.PovGpuInterior)
        no = r.u32()
        self.object_interior = (C.c_int32 * max(no, 1))(*[r.i32() for _ in range(no)])
        self.atmosphere_ior = struct.unpack("<d", r.take(8))[0]
        self.meshes = []
        for _ in range(r.u32()):
            nv, nn, nt, has_ni = r.i32(), r.i32(), r.i32(), r.i32()
            v = r.array("<f4", 3 * nv)
            n = r.array("<f4", 3 * nn)
            f = r.array("<i4", 3 * nt)
            ni = r.array("<i4", 3 * nt) if has_ni else None
            self.meshes.append(dict(vertices=v, normals=n if nn else None, faces=f, normal_indices=ni,
                                    num_vertices=nv, num_normals=nn, num_triangles=nt))
        if r.pos != len(data):
            raise ValueError("trailing bytes in scene file")
        # GpuScene runs the radiosity pretrace when this is not None
        self.radiosity = {"error_bound": self.radiosity_desc.error_bound} if self.radiosity_desc.enabled else None

    def radiosity_settings(self):
        rd = self.radiosity_desc
        return dict(count=rd.count, recursion_limit=rd.recursion_limit, error_bound=rd.error_bound)

    def desc(self):
        keep = [self.objects, self.materials, self.lights, self.medias, self.patterns, self.normals,
                self.interiors, self.object_interior]
        meshes = (abi.PovGpuMesh * max(len(self.meshes), 1))()
        for i, m in enumerate(self.meshes):
            meshes[i].vertices = m["vertices"].ctypes.data_as(C.POINTER(C.c_float))
            meshes[i].num_vertices = m["num_vertices"]
            if m["normals"] is not None:
                meshes[i].normals = m["normals"].ctypes.data_as(C.POINTER(C.c_float))
                meshes[i].num_normals = m["num_normals"]
            if m["normal_indices"] is not None:
                meshes[i].normal_indices = m["normal_indices"].ctypes.data_as(C.POINTER(C.c_int32))
            meshes[i].face_indices = m["faces"].ctypes.data_as(C.POINTER(C.c_int32))
            meshes[i].num_triangles = m["num_triangles"]
        keep += [meshes, self.meshes]
        d = abi.PovGpuSceneDesc()
        d.abi_version = abi.POV_GPU_ABI_VERSION
        d.num_objects, d.objects = self.num_objects, self.objects
        d.num_materials, d.materials = self.num_materials, self.materials
        d.num_lights, d.lights = self.num_lights, self.lights
        d.num_meshes, d.meshes = len(self.meshes), meshes
        d.camera = self.camera
        d.background[:] = self.background
        d.ambient_light[:] = self.ambient_light
        d.max_trace_level = self.max_trace_level
        d.adc_bailout = self.adc_bailout
        d.language_version = self.language_version
        d.radiosity = self.radiosity_desc
        d.num_medias, d.medias = self.num_medias, self.medias
        d.num_patterns, d.patterns = self.num_patterns, self.patterns
        d.num_normals, d.normals = self.num_normals, self.normals
        d.num_interiors, d.interiors = self.num_interiors, self.interiors
        d.object_interior = self.object_interior
        d.atmosphere_ior = self.atmosphere_ior
        return d, keep

    def render_params(self):
        p = abi.PovGpuRenderParams()
        p.width, p.height = self.width, self.height
        if self.antialias is not None:
            p.antialias, p.sampling_method = 1, 2
            p.aa_threshold, p.aa_depth = self.antialias
        else:
            p.antialias, p.sampling_method = 0, 1
        p.quality = 9
        return p
