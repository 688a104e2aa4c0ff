"""GPU radiosity against the reference's own radiosity render and against
the oracle.

The reference samples its cache one query at a time; the GPU answers a
batch of queries in rounds, so the two place different samples and the
comparison is statistical.  Tolerances (written here, applied below):
  mean linear radiance           within 2% of the reference
  relative RMSE (linear RGB)     at most 1.5x the distance between the
                                 reference's own 1-thread and 8-thread
                                 renders of the same scene
  samples gathered / rays shot   within 35% of the reference's counts
"""
import json
import os

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from povray_gb300 import GpuScene, scenes
from tests.golden.make_golden import radiosity_cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
JITTER = np.load(os.path.join(GOLDEN, "pretrace_jitter.npy"))


def _rel_rmse(a, b):
    return float(np.sqrt(((a - b) ** 2).mean()) / b.mean())


def _render(scene, jitter=True):
    gpu = GpuScene(scene)
    if jitter:
        gpu.set_pretrace_jitter(JITTER)
    img, st = gpu.render()
    return img[..., :3], st


def test_radiosity_room_matches_reference_render():
    scene = radiosity_cases()["radiosity_room_160x90"]
    g = np.load(os.path.join(GOLDEN, "radiosity_room_160x90.npz"))
    img, st = _render(scene)
    ref = g["rad_pixels_wt1"]
    floor = _rel_rmse(g["rad_pixels_wt8"], ref)
    rel = _rel_rmse(img, ref)
    rs = json.loads(str(g["rad_stats_wt1"]))
    info = json.dumps(dict(rel=rel, floor=floor, mean=float(img.mean()), ref_mean=float(ref.mean()), gpu=st, ref=rs))
    assert st["device_error"] == 0, info
    assert abs(img.mean() / ref.mean() - 1.0) < 0.02, info
    assert rel <= 1.5 * floor, info
    assert abs(st["radiosity_gathers"] / rs["samples"] - 1.0) < 0.35, info
    assert abs(st["radiosity_rays"] / rs["rays_shot"] - 1.0) < 0.35, info
    assert st["number_of_pixels"] == rs["number_of_pixels"], info


def test_radiosity_room_matches_oracle_mid_size():
    """320x180, 200 spheres, count 100: GPU vs the oracle's single-thread
    restatement (the reference's order).  The noise floor is the oracle
    against itself with another valid pretrace jitter (the table rotated)."""
    scene = scenes.radiosity_room(320, 180, count=100)
    img, st = _render(scene)
    ref, rst = Oracle(scene).render(threads=1)
    alt, _ = Oracle(scene, jitter=np.roll(JITTER, 1000)).render(threads=1)
    ref, alt = ref[..., :3], alt[..., :3]
    rel = _rel_rmse(img, ref)
    floor = _rel_rmse(alt, ref)
    info = json.dumps(dict(rel=rel, floor=floor, mean=float(img.mean()), ref_mean=float(ref.mean()), gpu=st,
                           oracle=rst))
    assert st["device_error"] == 0, info
    assert abs(img.mean() / ref.mean() - 1.0) < 0.02, info
    assert rel <= 1.5 * floor, info
    assert abs(st["radiosity_gathers"] / rst["radiosity_gathers"] - 1.0) < 0.35, info


def test_radiosity_without_reference_jitter_is_statistically_equal():
    """The pretrace jitter is a sampling detail: the GPU's own jitter gives
    the same image statistics."""
    scene = radiosity_cases()["radiosity_room_160x90"]
    a, _ = _render(scene, jitter=True)
    b, _ = _render(scene, jitter=False)
    assert abs(a.mean() / b.mean() - 1.0) < 0.02
    assert _rel_rmse(b, a) < 0.06


def test_radiosity_pretrace_requires_radiosity():
    scene = scenes.radiosity_room(64, 36, n_spheres=8, radiosity=False)
    gpu = GpuScene(scene)
    with pytest.raises(Exception):
        gpu.radiosity_pretrace(scenes.blocks_for(64, 36))
