"""Host-side driver over the C ABI, shaped like the reference's view/task
pair: a GpuScene is what View::StartRender builds once per view, and
GpuTraceTask.run() is TraceTask::Run -- it pulls render blocks from a
ViewData-like block source (GetNextRectangle), traces them in batches on the
GPU and hands each finished block back (CompletedRectangle).

There is no CPU path here: every call goes through libpovgpu.so and fails
loudly if the library or a device is missing.
"""
import ctypes as C

import numpy as np

from . import abi
from . import scenes as _scenes

HIT_DTYPE = np.dtype([("object", "<i4"), ("triangle", "<i4"), ("t", "<f8")])


def _check(st, what, bad=-1):
    if st != abi.POV_GPU_OK:
        raise abi.PovGpuError(st, what, bad)


class GpuScene:
    """Device copy of one parsed scene (pov_gpu_scene_create)."""

    def __init__(self, scene):
        self.lib = abi.load_library()
        self.scene = scene
        self.desc, self._keep = scene.desc()
        h = C.c_void_p()
        bad = C.c_int32(-1)
        st = self.lib.pov_gpu_scene_create(C.byref(self.desc), C.byref(h), C.byref(bad))
        _check(st, "pov_gpu_scene_create", bad.value)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.pov_gpu_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace_blocks(self, blocks, params=None, out=None):
        """Traces `blocks` (list of (left, top, right, bottom, serial), or a
        scenes.BlockBatch packed once).

        `out` may be None (a host array is returned), a host float32 array,
        or an integer device pointer (e.g. torch tensor .data_ptr()).
        Returns (rgbt or None, stats dict)."""
        p = params or self.scene.render_params()
        bb = _scenes.block_batch(blocks)
        arr, npix = bb.arr, bb.npix
        stats = abi.PovGpuStats()
        host = None
        if out is None:
            host = np.empty((npix, 4), dtype=np.float32)
            ptr = host.ctypes.data
        elif isinstance(out, np.ndarray):
            assert out.dtype == np.float32 and out.size >= npix * 4 and out.flags.c_contiguous
            host = out
            ptr = out.ctypes.data
        else:
            ptr = int(out)
        st = self.lib.pov_gpu_trace_blocks(self.h, arr, len(bb), C.byref(p), C.c_void_p(ptr),
                                           C.byref(stats))
        _check(st, "pov_gpu_trace_blocks")
        return host, stats.as_dict()

    def radiosity_pretrace(self, blocks, params=None):
        """RadiosityTask: empties the sample cache and runs every pretrace
        pass over `blocks`.  Returns the pass's stats dict."""
        p = params or self.scene.render_params()
        bb = _scenes.block_batch(blocks)
        stats = abi.PovGpuStats()
        _check(self.lib.pov_gpu_radiosity_pretrace(self.h, bb.arr, len(bb), C.byref(p), C.byref(stats)),
               "pov_gpu_radiosity_pretrace")
        return stats.as_dict()

    def set_neural_cache(self, enabled=True, steps=64, batch=None, learning_rate=1e-2, gate=None, seed=1,
                         shared=False):
        """Neural irradiance cache (pov_gpu_set_neural_cache): trained at the
        end of each pretrace; answers uncovered final-trace queries when its
        held-out relative RMSE is at most `gate` (None: the scene's radiosity
        error_bound).  `batch` None: one 128-sample tile per SM of the
        device.  `shared`: one network for all views, each pretrace training
        it further."""
        if gate is None:
            rs = self.scene.radiosity_settings() if self.scene.radiosity is not None else {"error_bound": 0.5}
            gate = rs["error_bound"]
        if batch is None:
            batch = 0
        c = abi.PovGpuNeuralCache(int(enabled), int(steps), int(batch), float(learning_rate), float(gate), int(seed),
                                  int(shared))
        _check(self.lib.pov_gpu_set_neural_cache(self.h, C.byref(c)), "pov_gpu_set_neural_cache")

    def set_camera(self, location, look_at, angle, width, height, sky=(0.0, 1.0, 0.0)):
        """The view's camera (pov_gpu_set_camera): ``camera { perspective
        location L right x*width/height up y look_at A angle a }`` for a view
        of width x height pixels, the look_at applied by the library the way
        View::StartRender applies it."""
        right_len = float(width) / float(height)
        dl = right_len / np.tan(float(angle) * _scenes.M_PI_360) / 2.0   # Parse_Camera's "angle"
        cam = abi.PovGpuCamera()
        for k in range(3):
            cam.location[k] = float(location[k])
        cam.direction[:] = (0.0, 0.0, dl)
        cam.right[:] = (right_len, 0.0, 0.0)
        cam.up[:] = (0.0, 1.0, 0.0)
        la = (C.c_double * 3)(*map(float, look_at))
        sk = (C.c_double * 3)(*map(float, sky))
        _check(self.lib.pov_gpu_set_camera(self.h, C.byref(cam), la, sk), "pov_gpu_set_camera")

    def encode_u8(self, rgbt_device_ptr, npix, curve="srgb", out=None):
        """8-bit RGB of `npix` linear RGBT pixels already in device memory
        (pov_gpu_encode_u8).  `out`: None (a host array is returned), a host
        uint8 array, or an integer device pointer."""
        c = {"srgb": abi.POV_GPU_CURVE_SRGB, "bt709": abi.POV_GPU_CURVE_BT709}[curve]
        host = None
        if out is None:
            host = np.empty((npix, 3), dtype=np.uint8)
            ptr = host.ctypes.data
        elif isinstance(out, np.ndarray):
            assert out.dtype == np.uint8 and out.size >= npix * 3 and out.flags.c_contiguous
            host, ptr = out, out.ctypes.data
        else:
            ptr = int(out)
        _check(self.lib.pov_gpu_encode_u8(self.h, C.c_void_p(int(rgbt_device_ptr)), int(npix), c, C.c_void_p(ptr)),
               "pov_gpu_encode_u8")
        return host

    def set_pretrace_jitter(self, table):
        """The reference's pretrace jitter table (RadiosityTask's
        RandomDoubleSequence(-1, 1, 2047) values)."""
        t = np.ascontiguousarray(table, dtype=np.float64)
        _check(self.lib.pov_gpu_set_pretrace_jitter(self.h, t.ctypes.data, len(t)), "pov_gpu_set_pretrace_jitter")

    def render(self, params=None, block=32):
        """Whole image (H, W, 4) through the block interface; with radiosity
        the pretrace runs over all blocks first and the returned stats add
        its counters (pixels, rays, shadow rays, radiosity samples)."""
        p = params or self.scene.render_params()
        blocks = _scenes.blocks_for(p.width, p.height, block)
        pre = None
        if self.scene.radiosity is not None:
            pre = self.radiosity_pretrace(blocks, p)
        rgbt, stats = self.trace_blocks(blocks, p)
        if pre is not None:
            # counters add up; the error word and the network's held-out
            # error (reported by both calls) do not
            merge = {"device_error": lambda a, b: a | b, "nic_val_error_ppm": max}
            stats = {k: merge.get(k, lambda a, b: a + b)(stats[k], pre[k]) for k in stats}
        return _scenes.unblock(rgbt, blocks, p.width, p.height), stats

    def set_launch_config(self, trace_blocks_per_sm=0, trace_block=0, trace_occupancy=0, shade_blocks_per_sm=0,
                          bounding_tree=0):
        """Launch shapes of the trace path's kernels (pov_gpu_set_launch_config;
        0 = the library's default), e.g. an entry of the autotuner's table;
        bounding_tree=1 traces the reference's own bounding tree."""
        c = abi.PovGpuLaunchConfig(int(trace_blocks_per_sm), int(trace_block), int(trace_occupancy),
                                   int(shade_blocks_per_sm), int(bounding_tree))
        _check(self.lib.pov_gpu_set_launch_config(self.h, C.byref(c)), "pov_gpu_set_launch_config")

    def tree_info(self):
        """The traversal tree in use (pov_gpu_get_tree_info) as a dict."""
        t = abi.PovGpuTreeInfo()
        _check(self.lib.pov_gpu_get_tree_info(self.h, C.byref(t)), "pov_gpu_get_tree_info")
        return {k: getattr(t, k) for k, _ in t._fields_ if k != "reserved"}

    def cache_save(self, path):
        """Writes the radiosity sample cache as a .rca file (pov_gpu_cache_save)."""
        _check(self.lib.pov_gpu_cache_save(self.h, str(path).encode()), "pov_gpu_cache_save")

    def cache_load(self, path):
        """Loads a .rca file (pov_gpu_cache_load); its samples start every
        following frame's cache.  None forgets a loaded file.  Returns the
        number of samples read."""
        n = C.c_int32(0)
        _check(self.lib.pov_gpu_cache_load(self.h, None if path is None else str(path).encode(), C.byref(n)),
               "pov_gpu_cache_load")
        return n.value

    def set_timeout(self, seconds):
        """Host wait limit of this scene's calls (pov_gpu_set_timeout); a
        call that runs out raises PovGpuError with POV_GPU_E_TIMEOUT."""
        _check(self.lib.pov_gpu_set_timeout(self.h, float(seconds)), "pov_gpu_set_timeout")

    def set_stream(self, stream_handle):
        """Launch on a caller-owned cudaStream_t (int handle, 0 = own stream)."""
        _check(self.lib.pov_gpu_scene_set_stream(self.h, C.c_void_p(int(stream_handle) or None)),
               "pov_gpu_scene_set_stream")

    def set_profiling(self, times=False, work=False):
        flags = (abi.POV_GPU_PROFILE_TIMES if times else 0) | (abi.POV_GPU_PROFILE_WORK if work else 0)
        _check(self.lib.pov_gpu_set_profiling(self.h, flags), "pov_gpu_set_profiling")

    def timings(self):
        t = abi.PovGpuTimings()
        _check(self.lib.pov_gpu_get_timings(self.h, C.byref(t)), "pov_gpu_get_timings")
        return {
            "stage_ms": {abi.STAGE_NAMES[i]: float(t.stage_ms[i]) for i in range(abi.POV_GPU_STAGES)},
            "stage_launches": {abi.STAGE_NAMES[i]: int(t.stage_launches[i]) for i in range(abi.POV_GPU_STAGES)},
            "node_visits": [int(x) for x in t.node_visits], "prim_tests": [int(x) for x in t.prim_tests],
            "tri_tests": [int(x) for x in t.tri_tests], "rays_traced": [int(x) for x in t.rays_traced],
            "kernel_launches": int(t.kernel_launches),
        }

    def trace_rays(self, origins, directions):
        o = np.ascontiguousarray(origins, dtype=np.float64)
        d = np.ascontiguousarray(directions, dtype=np.float64)
        n = o.shape[0]
        hits = (abi.PovGpuHit * max(n, 1))()
        st = self.lib.pov_gpu_trace_rays(self.h, o.ctypes.data, d.ctypes.data, n, hits)
        _check(st, "pov_gpu_trace_rays")
        return np.frombuffer(hits, dtype=HIT_DTYPE, count=n).copy()


class BlockSource:
    """ViewData's block dispenser: GetNextRectangle hands out the 32x32 grid
    in serial order (source/backend/scene/view.cpp:236-271), skipping blocks
    listed as already done (continue-trace skip list, view.cpp:240-252);
    CompletedRectangle receives the finished pixels (view.cpp:405)."""

    def __init__(self, width, height, block=32, skip=()):
        self.width, self.height = width, height
        self.blocks = [b for b in _scenes.blocks_for(width, height, block) if b[4] not in set(skip)]
        self.next = 0
        self.image = np.zeros((height, width, 4), dtype=np.float32)
        self.completed = []

    def get_next_rectangle(self):
        if self.next >= len(self.blocks):
            return None
        b = self.blocks[self.next]
        self.next += 1
        return b

    def completed_rectangle(self, rect, pixels):
        l, t, r, b, s = rect
        self.image[t:b + 1, l:r + 1] = pixels.reshape(b - t + 1, r - l + 1, 4)
        self.completed.append(s)


class GpuTraceTask:
    """TraceTask::Run with SimpleSamplingM0 (source/backend/render/
    tracetask.cpp:287,403): drains the block source in batches of
    `batch` blocks per device call."""

    def __init__(self, gpu_scene, source, params=None, batch=4096):
        self.gpu = gpu_scene
        self.source = source
        self.params = params or gpu_scene.scene.render_params()
        self.batch = batch
        self.stats = {}

    def run(self):
        while True:
            rects = []
            while len(rects) < self.batch:
                r = self.source.get_next_rectangle()
                if r is None:
                    break
                rects.append(r)
            if not rects:
                break
            rgbt, st = self.gpu.trace_blocks(rects, self.params)
            for k, v in st.items():
                self.stats[k] = self.stats.get(k, 0) + v
            off = 0
            for rect in rects:
                l, t, r, b, _s = rect
                n = (r - l + 1) * (b - t + 1)
                self.source.completed_rectangle(rect, rgbt[off:off + n])
                off += n
        return self.stats


def nic_eval(params, bounds, points, normals, targets=None):
    """pov_gpu_nic_eval: the neural cache's forward pass on (points, normals)
    and, with targets, the gradient and loss of its training objective.
    Returns (pred (n,3), grad or None, loss or None)."""
    lib = abi.load_library()
    p = np.ascontiguousarray(params, dtype=np.float32)
    assert p.size == abi.POV_GPU_NIC_PARAMS
    b = np.ascontiguousarray(bounds, dtype=np.float32)
    x = np.ascontiguousarray(points, dtype=np.float32)
    nrm = np.ascontiguousarray(normals, dtype=np.float32)
    n = x.shape[0]
    out = np.zeros((n, 3), dtype=np.float32)
    grad = loss = None
    tg = None
    if targets is not None:
        tg = np.ascontiguousarray(targets, dtype=np.float32)
        grad = np.zeros(abi.POV_GPU_NIC_PARAMS, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
    st = lib.pov_gpu_nic_eval(p.ctypes.data, b.ctypes.data, x.ctypes.data, nrm.ctypes.data,
                              tg.ctypes.data if tg is not None else None, n, out.ctypes.data,
                              grad.ctypes.data if grad is not None else None,
                              loss.ctypes.data if loss is not None else None)
    _check(st, "pov_gpu_nic_eval")
    return out, grad, (float(loss[0]) if loss is not None else None)
