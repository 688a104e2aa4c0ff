"""ctypes mirror of include/povgpu.h and the loader of libpovgpu.so.

The structures here must stay byte-identical to the C header; the
``-m "not gpu"`` tests check every size against the compiled library.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpovgpu.so")

POV_GPU_ABI_VERSION = 3

POV_GPU_OK = 0
POV_GPU_E_INVALID = -1
POV_GPU_E_UNSUPPORTED = -2
POV_GPU_E_CUDA = -3
POV_GPU_E_TIMEOUT = -4
POV_GPU_E_NOMEM = -5
POV_GPU_E_DEVICE = -6
POV_GPU_E_NODEVICE = -7
POV_GPU_E_CAPACITY = -8

POV_GPU_STATIC_MAX_RAYS = 65536

POV_OBJ_SPHERE = 1
POV_OBJ_PLANE = 2
POV_OBJ_BOX = 3
POV_OBJ_MESH = 4
POV_OBJ_TORUS = 5
POV_OBJ_UNION = 6
POV_OBJ_INTERSECTION = 7
POV_OBJ_MERGE = 8

POV_FLAG_INVERTED = 0x0001
POV_FLAG_NO_SHADOW = 0x0002
POV_FLAG_HAS_TRANS = 0x0004
POV_FLAG_INFINITE = 0x0008
POV_FLAG_DOUBLE_ILLUM = 0x0010
POV_FLAG_NO_REFLECTION = 0x0020
POV_FLAG_NO_IMAGE = 0x0040
POV_FLAG_HOLLOW = 0x0080

POV_LIGHT_POINT = 0
POV_LIGHT_AREA = 1
POV_LIGHT_TYPE_POINT = 1
POV_LIGHT_TYPE_SPOT = 2
POV_LIGHT_TYPE_SHADOWLESS = 3
POV_LIGHT_TYPE_CYLINDER = 4


class PovGpuObject(C.Structure):
    _fields_ = [("type", C.c_int32), ("flags", C.c_int32), ("material", C.c_int32),
                ("parent", C.c_int32), ("first_child", C.c_int32),
                ("num_children", C.c_int32), ("mesh", C.c_int32), ("media", C.c_int32),
                ("p", C.c_double * 8), ("trans", C.c_double * 32)]


class PovGpuMaterial(C.Structure):
    _fields_ = [("pigment", C.c_float * 5), ("ambient", C.c_float * 3),
                ("emission", C.c_float * 3), ("diffuse", C.c_float),
                ("diffuse_back", C.c_float), ("brilliance", C.c_float),
                ("brilliance_adjust", C.c_float), ("brilliance_adjust_rad", C.c_float),
                ("phong", C.c_float), ("phong_size", C.c_float), ("specular", C.c_float),
                ("roughness", C.c_float), ("metallic", C.c_float),
                ("reflection_max", C.c_float * 3), ("reflection_min", C.c_float * 3),
                ("reflection_falloff", C.c_float), ("reflect_exp", C.c_float),
                ("reflect_metallic", C.c_float), ("reflection_fresnel", C.c_int32),
                ("conserve_energy", C.c_int32), ("fresnel", C.c_float),
                ("crand", C.c_float), ("irid", C.c_float), ("pattern", C.c_int32),
                ("normal", C.c_int32)]


POV_PATTERN_CHECKER = 1
POV_PATTERN_GRADIENT = 2
POV_PATTERN_BOZO = 3
POV_PATTERN_GRANITE = 4
POV_PATTERN_MARBLE = 5
POV_PATTERN_WOOD = 6
POV_PATTERN_AGATE = 7
POV_PATTERN_ONION = 8
POV_PATTERN_LEOPARD = 9
POV_PATTERN_BUMPS = 10
POV_PATTERN_DENTS = 11
POV_PATTERN_WRINKLES = 12
POV_PATTERN_RIPPLES = 13
POV_PATTERN_WAVES = 14
POV_PATTERN_RADIAL = 15
POV_PATTERN_PLANAR = 16
POV_PATTERN_SPHERICAL = 17
POV_PATTERN_CYLINDRICAL = 18
POV_PATTERN_BOXED = 19
POV_PATTERN_SQUARE = 20
POV_PATTERN_TRIANGULAR = 21
POV_PATTERN_CUBIC = 22
POV_PATTERN_HEXAGON = 23
POV_PATTERN_BRICK = 24
POV_PATTERN_SPIRAL1 = 25
POV_PATTERN_SPIRAL2 = 26
POV_PATTERN_CELLS = 27
POV_PATTERN_CRACKLE = 28
POV_PATTERN_QUILTED = 29
POV_WAVES = {"ramp": 0, "sine": 1, "triangle": 2, "scallop": 3, "cubic": 4, "poly": 5}
POV_PATTERN_MAX_ENTRIES = 16


class PovGpuPattern(C.Structure):
    _fields_ = [("type", C.c_int32), ("noise_generator", C.c_int32), ("num_entries", C.c_int32),
                ("wave_type", C.c_int32), ("inverse", C.c_double * 16), ("gradient", C.c_double * 3),
                ("frequency", C.c_double), ("phase", C.c_double), ("exponent", C.c_double),
                ("turbulence", C.c_double * 3), ("omega", C.c_double), ("lambda", C.c_double),
                ("agate_turb", C.c_double), ("octaves", C.c_int32), ("has_turbulence", C.c_int32),
                ("values", C.c_float * POV_PATTERN_MAX_ENTRIES),
                ("colours", (C.c_float * 3) * POV_PATTERN_MAX_ENTRIES),
                ("brick_size", C.c_double * 3), ("mortar", C.c_double), ("arms", C.c_int32),
                ("crackle_solid", C.c_int32), ("crackle_form", C.c_double * 3), ("crackle_metric", C.c_double),
                ("crackle_offset", C.c_double), ("control0", C.c_double), ("control1", C.c_double),
                ("filters", C.c_float * POV_PATTERN_MAX_ENTRIES), ("transmits", C.c_float * POV_PATTERN_MAX_ENTRIES)]


class PovGpuLight(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("colour", C.c_float * 3), ("kind", C.c_int32),
                ("axis1", C.c_double * 3), ("axis2", C.c_double * 3),
                ("area_size1", C.c_int32), ("area_size2", C.c_int32),
                ("adaptive_level", C.c_int32), ("jitter", C.c_int32),
                ("circular", C.c_int32), ("orient", C.c_int32),
                ("fade_distance", C.c_double), ("fade_power", C.c_double),
                ("light_type", C.c_int32), ("parallel", C.c_int32), ("points_at", C.c_double * 3),
                ("radius", C.c_double), ("falloff", C.c_double), ("tightness", C.c_double)]


class PovGpuNormal(C.Structure):
    _fields_ = [("pattern", C.c_int32), ("dont_scale_bumps", C.c_int32), ("amount", C.c_float),
                ("delta", C.c_float), ("matrix", C.c_double * 16)]


class PovGpuMesh(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("face_indices", C.POINTER(C.c_int32)), ("normal_indices", C.POINTER(C.c_int32)),
                ("num_vertices", C.c_int32), ("num_normals", C.c_int32),
                ("num_triangles", C.c_int32), ("reserved", C.c_int32)]


class PovGpuCamera(C.Structure):
    _fields_ = [("location", C.c_double * 3), ("direction", C.c_double * 3),
                ("right", C.c_double * 3), ("up", C.c_double * 3),
                ("type", C.c_int32), ("reserved", C.c_int32)]


class PovGpuRadiosity(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("count", C.c_int32), ("recursion_limit", C.c_int32),
                ("nearest_count", C.c_int32), ("error_bound", C.c_double),
                ("low_error_factor", C.c_double), ("gray_threshold", C.c_double),
                ("minimum_reuse", C.c_double), ("maximum_reuse", C.c_double),
                ("brightness", C.c_double), ("pretrace_start", C.c_double),
                ("pretrace_end", C.c_double), ("adc_bailout", C.c_double),
                ("always_sample", C.c_int32), ("normal", C.c_int32), ("media", C.c_int32),
                ("reserved", C.c_int32)]


class PovGpuMedia(C.Structure):
    _fields_ = [("scattering_type", C.c_int32), ("method", C.c_int32), ("intervals", C.c_int32),
                ("min_samples", C.c_int32), ("max_samples", C.c_int32), ("aa_level", C.c_int32),
                ("aa_threshold", C.c_float), ("jitter", C.c_float), ("absorption", C.c_float * 3),
                ("emission", C.c_float * 3), ("scattering", C.c_float * 3), ("extinction", C.c_float * 3),
                ("eccentricity", C.c_float), ("reserved", C.c_int32)]


class PovGpuInterior(C.Structure):
    _fields_ = [("ior", C.c_double), ("dispersion", C.c_double), ("caustics", C.c_double),
                ("fade_distance", C.c_double), ("fade_power", C.c_double), ("fade_colour", C.c_float * 3),
                ("old_refract", C.c_float)]


class PovGpuSceneDesc(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("num_objects", C.c_int32),
                ("objects", C.POINTER(PovGpuObject)), ("num_materials", C.c_int32),
                ("materials", C.POINTER(PovGpuMaterial)), ("num_lights", C.c_int32),
                ("lights", C.POINTER(PovGpuLight)), ("num_meshes", C.c_int32),
                ("meshes", C.POINTER(PovGpuMesh)), ("camera", PovGpuCamera),
                ("background", C.c_float * 4), ("ambient_light", C.c_float * 3),
                ("max_trace_level", C.c_int32), ("adc_bailout", C.c_float),
                ("language_version", C.c_int32), ("radiosity", PovGpuRadiosity),
                ("num_medias", C.c_int32), ("medias", C.POINTER(PovGpuMedia)),
                ("num_patterns", C.c_int32), ("patterns", C.POINTER(PovGpuPattern)),
                ("num_normals", C.c_int32), ("normals", C.POINTER(PovGpuNormal)),
                ("num_interiors", C.c_int32), ("interiors", C.POINTER(PovGpuInterior)),
                ("object_interior", C.POINTER(C.c_int32)), ("atmosphere_ior", C.c_double)]


class PovGpuBlock(C.Structure):
    _fields_ = [("left", C.c_int32), ("top", C.c_int32), ("right", C.c_int32),
                ("bottom", C.c_int32), ("serial", C.c_uint32), ("reserved", C.c_uint32)]


class PovGpuRenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("antialias", C.c_int32),
                ("sampling_method", C.c_int32), ("aa_threshold", C.c_float),
                ("aa_depth", C.c_int32), ("jitter", C.c_int32), ("jitter_amount", C.c_float),
                ("quality", C.c_int32), ("high_reproducibility", C.c_int32)]


class PovGpuStats(C.Structure):
    _fields_ = [("number_of_rays", C.c_uint64), ("shadow_ray_tests", C.c_uint64),
                ("shadow_rays_succeeded", C.c_uint64), ("reflected_rays", C.c_uint64),
                ("number_of_pixels", C.c_uint64), ("number_of_samples", C.c_uint64),
                ("radiosity_gathers", C.c_uint64), ("radiosity_reuse", C.c_uint64),
                ("device_error", C.c_uint64), ("radiosity_rays", C.c_uint64),
                ("radiosity_gathers_d0", C.c_uint64), ("radiosity_gathers_d1", C.c_uint64),
                ("nic_answers", C.c_uint64), ("nic_val_error_ppm", C.c_uint64),
                ("transmitted_rays", C.c_uint64), ("media_samples", C.c_uint64),
                ("refracted_rays", C.c_uint64), ("internal_reflected_rays", C.c_uint64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_ if k != "reserved"}


class PovGpuNeuralCache(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("steps", C.c_int32), ("batch", C.c_int32),
                ("learning_rate", C.c_float), ("gate", C.c_float), ("seed", C.c_uint32), ("shared", C.c_int32)]


POV_GPU_NIC_PARAMS = 20752


class PovGpuHit(C.Structure):
    _fields_ = [("object", C.c_int32), ("triangle", C.c_int32), ("t", C.c_double)]


POV_GPU_CURVE_SRGB = 0
POV_GPU_CURVE_BT709 = 1
POV_GPU_STAGES = 9
STAGE_NAMES = ["camera", "trace_closest", "shade", "trace_shadow", "resolve", "finalize", "area_shadow", "radiosity",
               "media"]
POV_GPU_PROFILE_TIMES = 1
POV_GPU_PROFILE_WORK = 2


class PovGpuTimings(C.Structure):
    _fields_ = [("stage_ms", C.c_float * POV_GPU_STAGES), ("stage_launches", C.c_uint32 * POV_GPU_STAGES),
                ("node_visits", C.c_uint64 * 2), ("prim_tests", C.c_uint64 * 2),
                ("tri_tests", C.c_uint64 * 2), ("rays_traced", C.c_uint64 * 2),
                ("kernel_launches", C.c_uint32), ("reserved", C.c_uint32)]


class PovGpuLaunchConfig(C.Structure):
    _fields_ = [("trace_blocks_per_sm", C.c_int32), ("trace_block", C.c_int32), ("trace_occupancy", C.c_int32),
                ("shade_blocks_per_sm", C.c_int32), ("bounding_tree", C.c_int32), ("reserved", C.c_int32 * 3)]


class PovGpuTreeInfo(C.Structure):
    _fields_ = [("bounding_tree", C.c_int32), ("nodes", C.c_int32), ("depth", C.c_int32),
                ("ref_top_nodes", C.c_int32), ("ref_mesh_nodes", C.c_int32), ("reserved", C.c_int32 * 3)]


STRUCTS = {
    "PovGpuLaunchConfig": PovGpuLaunchConfig, "PovGpuTreeInfo": PovGpuTreeInfo, "PovGpuNormal": PovGpuNormal,
    "PovGpuInterior": PovGpuInterior,
    "PovGpuObject": PovGpuObject, "PovGpuMaterial": PovGpuMaterial,
    "PovGpuLight": PovGpuLight, "PovGpuMesh": PovGpuMesh, "PovGpuCamera": PovGpuCamera,
    "PovGpuRadiosity": PovGpuRadiosity, "PovGpuSceneDesc": PovGpuSceneDesc,
    "PovGpuBlock": PovGpuBlock, "PovGpuRenderParams": PovGpuRenderParams,
    "PovGpuStats": PovGpuStats, "PovGpuHit": PovGpuHit, "PovGpuTimings": PovGpuTimings,
    "PovGpuNeuralCache": PovGpuNeuralCache, "PovGpuMedia": PovGpuMedia, "PovGpuPattern": PovGpuPattern,
}

# Entry points that include/povgpu.h declares (checked by the CPU tests).
EXPORTS = ["pov_gpu_scene_create", "pov_gpu_trace_blocks", "pov_gpu_trace_rays",
           "pov_gpu_scene_destroy", "pov_gpu_error_string", "pov_gpu_abi_version",
           "pov_gpu_scene_set_stream", "pov_gpu_set_profiling", "pov_gpu_get_timings",
           "pov_gpu_trace_rays_static", "pov_gpu_radiosity_pretrace", "pov_gpu_set_pretrace_jitter",
           "pov_gpu_set_neural_cache", "pov_gpu_nic_eval", "pov_gpu_set_camera", "pov_gpu_encode_u8",
           "pov_gpu_set_timeout", "pov_gpu_cache_save", "pov_gpu_cache_load", "pov_gpu_set_launch_config",
           "pov_gpu_get_tree_info"]


class PovGpuError(RuntimeError):
    def __init__(self, status, what, bad_index=-1):
        self.status = status
        self.bad_index = bad_index
        super().__init__(f"{what}: status {status}" + (f" (object {bad_index})" if bad_index >= 0 else ""))


_lib = None


def load_library(path=None):
    """Loads libpovgpu.so.  Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libpovgpu.so not built at {p}; run __graft_entry__.build()")
    lib = C.CDLL(p)
    lib.pov_gpu_scene_create.argtypes = [C.POINTER(PovGpuSceneDesc), C.POINTER(C.c_void_p),
                                         C.POINTER(C.c_int32)]
    lib.pov_gpu_scene_create.restype = C.c_int
    lib.pov_gpu_trace_blocks.argtypes = [C.c_void_p, C.POINTER(PovGpuBlock), C.c_int32,
                                         C.POINTER(PovGpuRenderParams), C.c_void_p,
                                         C.POINTER(PovGpuStats)]
    lib.pov_gpu_trace_blocks.restype = C.c_int
    lib.pov_gpu_trace_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                       C.POINTER(PovGpuHit)]
    lib.pov_gpu_trace_rays.restype = C.c_int
    lib.pov_gpu_trace_rays_static.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                              C.POINTER(PovGpuHit)]
    lib.pov_gpu_trace_rays_static.restype = C.c_int
    lib.pov_gpu_radiosity_pretrace.argtypes = [C.c_void_p, C.POINTER(PovGpuBlock), C.c_int32,
                                               C.POINTER(PovGpuRenderParams), C.POINTER(PovGpuStats)]
    lib.pov_gpu_radiosity_pretrace.restype = C.c_int
    lib.pov_gpu_set_pretrace_jitter.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
    lib.pov_gpu_set_pretrace_jitter.restype = C.c_int
    lib.pov_gpu_set_neural_cache.argtypes = [C.c_void_p, C.POINTER(PovGpuNeuralCache)]
    lib.pov_gpu_set_neural_cache.restype = C.c_int
    lib.pov_gpu_nic_eval.argtypes = [C.c_void_p] * 5 + [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.pov_gpu_nic_eval.restype = C.c_int
    lib.pov_gpu_scene_destroy.argtypes = [C.c_void_p]
    lib.pov_gpu_scene_destroy.restype = None
    lib.pov_gpu_error_string.argtypes = [C.c_int]
    lib.pov_gpu_error_string.restype = C.c_char_p
    lib.pov_gpu_abi_version.argtypes = []
    lib.pov_gpu_abi_version.restype = C.c_int
    lib.pov_gpu_encode_u8.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]
    lib.pov_gpu_encode_u8.restype = C.c_int
    lib.pov_gpu_set_camera.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.pov_gpu_set_camera.restype = C.c_int
    lib.pov_gpu_set_launch_config.argtypes = [C.c_void_p, C.POINTER(PovGpuLaunchConfig)]
    lib.pov_gpu_set_launch_config.restype = C.c_int
    lib.pov_gpu_get_tree_info.argtypes = [C.c_void_p, C.POINTER(PovGpuTreeInfo)]
    lib.pov_gpu_get_tree_info.restype = C.c_int
    lib.pov_gpu_cache_save.argtypes = [C.c_void_p, C.c_char_p]
    lib.pov_gpu_cache_save.restype = C.c_int
    lib.pov_gpu_cache_load.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_int32)]
    lib.pov_gpu_cache_load.restype = C.c_int
    lib.pov_gpu_set_timeout.argtypes = [C.c_void_p, C.c_double]
    lib.pov_gpu_set_timeout.restype = C.c_int
    lib.pov_gpu_scene_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    lib.pov_gpu_scene_set_stream.restype = C.c_int
    lib.pov_gpu_set_profiling.argtypes = [C.c_void_p, C.c_int]
    lib.pov_gpu_set_profiling.restype = C.c_int
    lib.pov_gpu_get_timings.argtypes = [C.c_void_p, C.POINTER(PovGpuTimings)]
    lib.pov_gpu_get_timings.restype = C.c_int
    if path is None:
        _lib = lib
    return lib
