"""Radiosity renders of the 1280x720 room against its FP64 converged truth,
plain GPU form and neural-cache form side by side.

The truth (tests/golden/radiosity_room_converged_1280x720.npz, made by
tests/golden/make_converged.py) is the oracle's converged mode: every
radiosity query gathered without the sample cache, 4096 / 16 stratified
cosine-weighted rays at bounce depth 0 / 1, summed in FP64; its own sampling
noise is 0.27% relative RMSE.  Renders are compared on its 14,400 pixels (an
8x8 grid), in linear radiance: relative RMSE = RMS(render - truth) /
mean(truth).

The neural-cache form trains the network at the end of the pretrace
(the library's defaults: 64 Adam steps of one 128-sample tile per SM) and,
when its held-out relative error is at most the scene's error_bound (0.5),
answers the final trace's uncovered queries instead of gathering.

Measured on a GB300 (several runs): plain 5.1-5.2% RMSE, mean ratio
1.000-1.002; neural cache 10.8-11.0% RMSE, mean ratio 1.00-1.01; the
neural cache's final trace 6.5 ms against the plain 25 ms.  Bounds, with
margin over those (the samples, and so the network, vary from run to run):
  plain          RMSE <= 7%, mean within 1.5%
  neural cache   RMSE <= 16%, mean within 4% (when its gate passes)
  gain           the neural cache's final trace shoots at most half the
                 plain final trace's radiosity rays and takes at most half
                 its time
"""
import json
import os

import numpy as np
import pytest
import torch

from povray_gb300 import GpuScene, scenes

pytestmark = pytest.mark.gpu

TRUTH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "radiosity_room_converged_1280x720.npz")


def _frame(gpu, scene):
    """One frame (pretrace + final trace) on torch's stream; returns the image
    and, per call, its statistics and CUDA-event milliseconds."""
    p = scene.render_params()
    blocks = scenes.blocks_for(p.width, p.height)
    stream = torch.cuda.current_stream()
    gpu.set_stream(stream.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(stream)
    pre = gpu.radiosity_pretrace(blocks, p)
    ev[1].record(stream)
    rgbt, fin = gpu.trace_blocks(blocks, p)
    ev[2].record(stream)
    torch.cuda.synchronize()
    img = scenes.unblock(rgbt, blocks, p.width, p.height)
    return img, pre, fin, ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])


@pytest.fixture(scope="module")
def truth():
    t = np.load(TRUTH)
    return t["pixels"], t["rgb"]


def _err(img, truth):
    px, rgb = truth
    a = img[px[:, 1], px[:, 0], :3]
    return float(np.sqrt(((a - rgb) ** 2).mean()) / rgb.mean()), float(a.mean() / rgb.mean())


@pytest.fixture(scope="module")
def plain(truth):
    scene = scenes.radiosity_room(1280, 720)
    gpu = GpuScene(scene)
    _frame(gpu, scene)   # warm-up
    img, pre, fin, pre_ms, fin_ms = _frame(gpu, scene)
    rmse, mean = _err(img, truth)
    return dict(rmse=rmse, mean=mean, pre_ms=pre_ms, fin_ms=fin_ms, fin_rays=fin["radiosity_rays"],
                device_error=pre["device_error"] | fin["device_error"])


def test_plain_radiosity_against_fp64_truth(plain):
    info = json.dumps(plain)
    print("plain radiosity vs FP64 truth:", info)
    assert plain["device_error"] == 0, info
    assert plain["rmse"] <= 0.07, info
    assert abs(plain["mean"] - 1.0) <= 0.015, info


def test_neural_cache_against_fp64_truth_and_its_gain(plain, truth):
    scene = scenes.radiosity_room(1280, 720)
    gpu = GpuScene(scene)
    gpu.set_neural_cache(True)           # gate = error_bound 0.5
    _frame(gpu, scene)   # warm-up
    img, pre, fin, pre_ms, fin_ms = _frame(gpu, scene)
    rmse, mean = _err(img, truth)
    rec = dict(rmse=rmse, mean=mean, pre_ms=pre_ms, fin_ms=fin_ms, frame_ms=pre_ms + fin_ms,
               plain_frame_ms=plain["pre_ms"] + plain["fin_ms"],
               frame_speedup=(plain["pre_ms"] + plain["fin_ms"]) / (pre_ms + fin_ms),
               held_out=fin["nic_val_error_ppm"] / 1e6, answers=fin["nic_answers"], fin_rays=fin["radiosity_rays"],
               plain=plain)
    info = json.dumps(rec)
    print("neural cache vs FP64 truth:", info)
    assert pre["device_error"] == 0 and fin["device_error"] == 0, info
    assert 0 < rec["held_out"] < 1.0, info
    if rec["held_out"] > 0.5:
        # the gate keeps the plain gather: no answers, the plain form's image
        assert rec["answers"] == 0, info
        assert rmse <= 0.07, info
        return
    assert rec["answers"] > 0, info
    assert rmse <= 0.16, info
    assert abs(mean - 1.0) <= 0.04, info
    assert rec["fin_rays"] <= 0.5 * plain["fin_rays"], info
    assert fin_ms <= 0.5 * plain["fin_ms"], info
