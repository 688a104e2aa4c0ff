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


def _read_rca(path):
    """The .rca lines as (depth, point, illuminance, hmd, nearest) floats and
    the packed normal / direction bytes."""
    rows, packed = [], []
    for line in open(path):
        if not line.startswith("C"):
            continue
        f = line[1:].split()
        rows.append([float(x) for x in (f[0], f[1], f[2], f[3], f[5], f[6], f[7], f[8], f[9])])
        packed.append([int(f[4][i:i + 2], 16) for i in (0, 2, 4)] + [int(f[10][i:i + 2], 16) for i in (0, 2, 4)])
    return np.array(rows), np.array(packed)


def test_cache_file_round_trip_and_final_trace_on_it(tmp_path):
    """pov_gpu_cache_save / pov_gpu_cache_load in the reference's .rca text
    format.  A pretrace's cache saved, loaded into a new scene and saved
    again: the same samples (depth, point, illuminance and distances as
    written; the packed unit vectors within one step, as the reference's own
    unpack-normalise-repack gives).  A final trace on the loaded cache alone
    (no pretrace) renders the pretraced scene's image: mean within 2%,
    relative RMSE within the 160x90 room's sampling floor (6%)."""
    scene = radiosity_cases()["radiosity_room_160x90"]
    p = scene.render_params()
    blocks = scenes.blocks_for(p.width, p.height)
    a = GpuScene(scene)
    a.set_pretrace_jitter(JITTER)
    a.radiosity_pretrace(blocks, p)
    f1, f2 = tmp_path / "a.rca", tmp_path / "b.rca"
    a.cache_save(f1)
    img_a, st_a = a.trace_blocks(blocks, p)
    b = GpuScene(scene)
    n = b.cache_load(f1)
    rows1, packed1 = _read_rca(f1)
    assert n == len(rows1) > 100
    b.cache_save(f2)
    rows2, packed2 = _read_rca(f2)
    assert np.array_equal(rows1, rows2)
    assert np.abs(packed1 - packed2).max() <= 1
    img_b, st_b = b.trace_blocks(blocks, p)
    ia = scenes.unblock(img_a, blocks, p.width, p.height)[..., :3]
    ib = scenes.unblock(img_b, blocks, p.width, p.height)[..., :3]
    info = json.dumps(dict(rel=_rel_rmse(ib, ia), mean=float(ib.mean() / ia.mean()), a=st_a, b=st_b))
    assert st_b["device_error"] == 0, info
    assert abs(ib.mean() / ia.mean() - 1.0) < 0.02, info
    assert _rel_rmse(ib, ia) < 0.06, info
    # forgetting the file: an empty cache again
    assert b.cache_load(None) == 0


def test_reference_cache_file_loads_and_renders_its_image(tmp_path):
    """The reference CLI's own cache file of the golden room (+RFO, one
    thread: every sample its pretrace and final trace took) loaded into the
    GPU cache: its 5,653 samples read, and the final trace on them alone
    renders the reference's image -- mean within 2%, relative RMSE at most
    1.5x the reference's own 1- vs 8-thread distance -- while gathering
    under a fifth of the samples the reference gathered."""
    import gzip
    scene = radiosity_cases()["radiosity_room_160x90"]
    g = np.load(os.path.join(GOLDEN, "radiosity_room_160x90.npz"))
    rca = tmp_path / "ref.rca"
    rca.write_bytes(gzip.open(os.path.join(GOLDEN, "radiosity_room_160x90.rca.gz"), "rb").read())
    gpu = GpuScene(scene)
    assert gpu.cache_load(rca) == 5653
    p = scene.render_params()
    blocks = scenes.blocks_for(p.width, p.height)
    rgbt, st = gpu.trace_blocks(blocks, p)
    img = scenes.unblock(rgbt, blocks, p.width, p.height)[..., :3]
    ref = g["rad_pixels_wt1"]
    floor = _rel_rmse(g["rad_pixels_wt8"], ref)
    rs = json.loads(str(g["rad_stats_wt1"]))
    info = json.dumps(dict(rel=_rel_rmse(img, ref), floor=floor, mean=float(img.mean() / ref.mean()), gpu=st))
    assert st["device_error"] == 0, info
    assert abs(img.mean() / ref.mean() - 1.0) < 0.02, info
    assert _rel_rmse(img, ref) <= 1.5 * floor, info
    assert st["radiosity_gathers"] < 0.2 * rs["samples"], info
