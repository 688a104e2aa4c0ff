"""pov_gpu_trace_rays_static (the allocation-free closest-hit query) against
pov_gpu_trace_rays on the same rays, called through the C-ABI.

Named to be collected last, so that it runs both after every other test
(device memory already used by other scenes) and alone.  Besides the
results, it checks the property the entry exists for: the device's free
memory does not change across its calls.

Tolerances: object and triangle ids exact; depths within 1e-5 relative
(the parity tests' depth tolerance).
"""
import ctypes as C

import numpy as np
import pytest

from povray_gb300 import GpuScene, abi, scenes
from povray_gb300.render import HIT_DTYPE

pytestmark = pytest.mark.gpu

T_TOL = 1e-5


def _rays(scene, n_random, seed):
    """Camera rays plus rays from random points towards random points of the
    objects' region (these reach surfaces from every side, and some start
    inside objects)."""
    o, d = scene.camera_rays()
    rng = np.random.default_rng(seed)
    ro = rng.uniform(-20.0, 20.0, size=(n_random, 3))
    target = rng.uniform(-3.5, 3.5, size=(n_random, 3))
    rd = target - ro
    rd /= np.linalg.norm(rd, axis=1)[:, None]
    return (np.ascontiguousarray(np.concatenate([o, ro])),
            np.ascontiguousarray(np.concatenate([d, rd])))


def _static(gpu, o, d):
    n = o.shape[0]
    hits = (abi.PovGpuHit * max(n, 1))()
    st = gpu.lib.pov_gpu_trace_rays_static(gpu.h, o.ctypes.data, d.ctypes.data, n, hits)
    assert st == abi.POV_GPU_OK, gpu.lib.pov_gpu_error_string(st)
    return np.frombuffer(hits, dtype=HIT_DTYPE, count=n).copy()


def _same(got, ref):
    assert np.array_equal(got["object"], ref["object"])
    assert np.array_equal(got["triangle"], ref["triangle"])
    hit = ref["object"] >= 0
    rel = np.abs(got["t"][hit] - ref["t"][hit]) / np.maximum(np.abs(ref["t"][hit]), 1e-12)
    assert rel.size == 0 or rel.max() <= T_TOL, float(rel.max())
    assert np.all(got["t"][~hit] == 0.0)


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("make", [
    lambda: scenes.csg_torus_grid(96, 54, n=4, antialias=None),   # sphere, plane, box, torus, CSG
    lambda: scenes.mesh_spheres(96, 54, mesh_n=24, n_spheres=8),   # triangles
], ids=["csg_torus_grid", "mesh_spheres"])
def test_static_matches_trace_rays_twice(make):
    """The fixed-scratch query runs before any pov_gpu_trace_rays call on the
    scene (so it cannot lean on that call's buffers), leaves the device's
    free memory unchanged across two calls, and agrees with
    pov_gpu_trace_rays on both."""
    scene = make()
    gpu = GpuScene(scene)
    # one-time set-up on this device (n = 0 does only that)
    assert gpu.lib.pov_gpu_trace_rays_static(gpu.h, None, None, 0, None) == abi.POV_GPU_OK
    o, d = _rays(scene, 20000, seed=7)
    _static(gpu, o[:64], d[:64])   # first launches of its kernels (CUDA loads them lazily)
    free0 = _free_bytes()
    first = _static(gpu, o, d)
    second = _static(gpu, o, d)
    assert _free_bytes() == free0
    ref = gpu.trace_rays(o, d)
    assert (ref["object"] >= 0).sum() > 0.2 * len(ref)
    _same(first, ref)
    _same(second, ref)


def test_static_full_capacity_and_rejection():
    scene = scenes.csg_torus_grid(64, 36, n=3, antialias=None)
    gpu = GpuScene(scene)
    cap = abi.POV_GPU_STATIC_MAX_RAYS
    o, d = _rays(scene, cap - 64 * 36, seed=11)
    assert o.shape[0] == cap
    ref = gpu.trace_rays(o, d)
    _same(_static(gpu, o, d), ref)
    # one ray more than the scratch holds: rejected with the capacity status
    o2 = np.ascontiguousarray(np.concatenate([o, o[:1]]))
    d2 = np.ascontiguousarray(np.concatenate([d, d[:1]]))
    hits = (abi.PovGpuHit * (cap + 1))()
    st = gpu.lib.pov_gpu_trace_rays_static(gpu.h, o2.ctypes.data, d2.ctypes.data, cap + 1, hits)
    assert st == abi.POV_GPU_E_CAPACITY
    assert b"capacity" in gpu.lib.pov_gpu_error_string(st)
    # a smaller call after the rejected one still agrees with trace_rays
    _same(_static(gpu, o[:1000], d[:1000]), ref[:1000])
