"""ctypes loader of the oracle (oracle/povoracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the povray_gb300 package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libpovoracle.so")
SRC = os.path.join(HERE, "povoracle.c")


def build(force=False):
    """Compiles the oracle with gcc (portable flags: runs on x86 and Arm)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    subprocess.check_call(["gcc", "-O2", "-std=c99", "-shared", "-fPIC", "-o", LIB, SRC,
                           "-lm", "-lpthread"])
    return LIB


_lib = None
JITTER_TABLE = os.path.join(os.path.dirname(HERE), "tests", "golden", "pretrace_jitter.npy")


def lib():
    global _lib
    if _lib is None:
        from povray_gb300 import abi
        build()
        L = C.CDLL(LIB)
        L.pov_oracle_create.argtypes = [C.POINTER(abi.PovGpuSceneDesc), C.POINTER(C.c_void_p),
                                        C.POINTER(C.c_int32)]
        L.pov_oracle_create.restype = C.c_int
        L.pov_oracle_destroy.argtypes = [C.c_void_p]
        L.pov_oracle_destroy.restype = None
        L.pov_oracle_trace_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                            C.POINTER(abi.PovGpuHit)]
        L.pov_oracle_trace_rays.restype = C.c_int
        L.pov_oracle_render.argtypes = [C.c_void_p, C.POINTER(abi.PovGpuRenderParams), C.c_int32,
                                        C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                        C.POINTER(abi.PovGpuStats)]
        L.pov_oracle_render.restype = C.c_int
        L.pov_oracle_count_work.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                            C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.pov_oracle_count_work.restype = C.c_int
        L.pov_oracle_render_converged.argtypes = [C.c_void_p, C.POINTER(abi.PovGpuRenderParams), C.c_void_p,
                                                  C.c_int32, C.c_void_p, C.c_int32, C.c_uint64, C.c_int32,
                                                  C.c_void_p, C.POINTER(abi.PovGpuStats)]
        L.pov_oracle_render_converged.restype = C.c_int
        L.pov_oracle_set_pretrace_jitter.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
        L.pov_oracle_set_pretrace_jitter.restype = C.c_int
        L.pov_oracle_tree_info.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.pov_oracle_tree_info.restype = None
        L.pov_oracle_pattern_rand.argtypes = [C.c_int32]
        L.pov_oracle_pattern_rand.restype = C.c_double
        _lib = L
    return _lib


class Oracle:
    """One oracle scene built from a povray_gb300.scenes.Scene."""

    def __init__(self, scene, jitter=None):
        from povray_gb300 import abi
        self.scene = scene
        self.desc, self._keep = scene.desc()
        h = C.c_void_p()
        bad = C.c_int32(-1)
        st = lib().pov_oracle_create(C.byref(self.desc), C.byref(h), C.byref(bad))
        if st != 0:
            raise abi.PovGpuError(st, "pov_oracle_create", bad.value)
        self.h = h
        if scene.radiosity is not None:
            # the reference's pretrace jitter table, dumped from it by
            # tests/golden/make_golden.py
            table = np.load(JITTER_TABLE) if jitter is None else jitter
            self._jitter = np.ascontiguousarray(table, dtype=np.float64)
            lib().pov_oracle_set_pretrace_jitter(self.h, self._jitter.ctypes.data, len(self._jitter))

    def close(self):
        if self.h:
            lib().pov_oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace_rays(self, origins, directions):
        from povray_gb300 import abi
        o = np.ascontiguousarray(origins, dtype=np.float64)
        d = np.ascontiguousarray(directions, dtype=np.float64)
        n = o.shape[0]
        hits = (abi.PovGpuHit * max(n, 1))()
        st = lib().pov_oracle_trace_rays(self.h, o.ctypes.data, d.ctypes.data, n, hits)
        if st != 0:
            raise abi.PovGpuError(st, "pov_oracle_trace_rays")
        arr = np.frombuffer(hits, dtype=np.dtype([("object", "<i4"), ("triangle", "<i4"), ("t", "<f8")]),
                            count=n)
        return arr.copy()

    def render(self, x0=0, y0=0, x1=None, y1=None, threads=0, params=None):
        from povray_gb300 import abi
        p = params or self.scene.render_params()
        x1 = p.width if x1 is None else x1
        y1 = p.height if y1 is None else y1
        out = np.zeros(((y1 - y0), (x1 - x0), 4), dtype=np.float32)
        stats = abi.PovGpuStats()
        st = lib().pov_oracle_render(self.h, C.byref(p), x0, y0, x1, y1, threads, out.ctypes.data,
                                     C.byref(stats))
        if st != 0:
            raise abi.PovGpuError(st, "pov_oracle_render")
        return out, stats.as_dict()

    def render_converged(self, pixels, counts, seed=1, threads=0, params=None):
        """Converged radiosity (the FP64 ground truth): RGBT of the given
        pixels ((n, 2) int array of x, y in the full image), every radiosity
        query answered without the cache by counts[d] stratified
        cosine-weighted rays at bounce depth d.  Returns ((n, 4) float32,
        stats)."""
        from povray_gb300 import abi
        p = params or self.scene.render_params()
        px = np.ascontiguousarray(pixels, dtype=np.int32).reshape(-1, 2)
        cn = np.ascontiguousarray(counts, dtype=np.int32)
        out = np.zeros((px.shape[0], 4), dtype=np.float32)
        stats = abi.PovGpuStats()
        st = lib().pov_oracle_render_converged(self.h, C.byref(p), px.ctypes.data, px.shape[0], cn.ctypes.data,
                                               len(cn), int(seed), threads, out.ctypes.data, C.byref(stats))
        if st != 0:
            raise abi.PovGpuError(st, "pov_oracle_render_converged")
        return out, stats.as_dict()

    def tree_info(self):
        """Composite nodes of the oracle's bounding trees: (top tree, all mesh
        trees) -- the reference's Build_BBox_Tree restated."""
        t, m = C.c_int32(0), C.c_int32(0)
        lib().pov_oracle_tree_info(self.h, C.byref(t), C.byref(m))
        return t.value, m.value

    def count_work(self, origins, directions):
        o = np.ascontiguousarray(origins, dtype=np.float64)
        d = np.ascontiguousarray(directions, dtype=np.float64)
        boxes, prims = C.c_uint64(), C.c_uint64()
        lib().pov_oracle_count_work(self.h, o.ctypes.data, d.ctypes.data, o.shape[0],
                                    C.byref(boxes), C.byref(prims))
        return int(boxes.value), int(prims.value)


def pattern_rand(i):
    """Entry i of the pattern random table the cells pattern reads."""
    return float(lib().pov_oracle_pattern_rand(int(i)))
