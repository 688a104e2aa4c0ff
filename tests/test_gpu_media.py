"""Media containers and views on the GPU against the oracle.

The reference's own fixture (media_spheres 160x120) is checked in
test_gpu_parity.py; here the same scene is seen from other cameras through
pov_gpu_set_camera (View::StartRender's camera change without parsing) and
compared with the oracle rendering a scene built with that camera.

Tolerances (written here, applied below):
  8-bit pixels      >= 99.9% of channels within 1 LSB
  rays              Number_Of_Rays, Transmitted_Rays, Reflected_Rays exact
  media samples     within 1.5% (FP32 segment lengths decide the padding
                    interval differently from FP64 ones)
  shadow counters   within 1% of the shadow tests
"""
import json

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from povray_gb300 import GpuScene, abi, scenes
from tests.parity import compare_pixels

pytestmark = pytest.mark.gpu

VIEWS = [((25.0, 6.0, 0.0), (0.0, 0.0, 0.0), 96, 72),
         ((-18.0, 2.0, -18.0), (1.0, -1.0, 0.0), 64, 64),
         ((0.0, 20.0, 22.0), (0.0, 0.0, 0.0), 120, 68)]


def _no_aa(scene):
    p = scene.render_params()
    p.antialias = 0
    p.sampling_method = 1
    return p


def _close(got, ref):
    info = json.dumps(dict(gpu=got, oracle=ref))
    for k in ("number_of_rays", "transmitted_rays", "reflected_rays"):
        assert got[k] == ref[k], (k, info)
    assert abs(got["media_samples"] - ref["media_samples"]) <= 0.015 * ref["media_samples"], info
    for k in ("shadow_ray_tests", "shadow_rays_succeeded"):
        assert abs(got[k] - ref[k]) <= 0.01 * ref["shadow_ray_tests"], (k, info)


def test_views_through_set_camera_match_oracle():
    base = scenes.media_spheres(64, 48)
    gpu = GpuScene(base)
    for loc, at, w, h in VIEWS:
        view = scenes.view_of(base, loc, at, w, h)
        gpu.set_camera(loc, at, base.angle, w, h)
        img, st = gpu.render(params=_no_aa(view))
        ref, rst = Oracle(view).render(threads=8, params=_no_aa(view))
        c = compare_pixels(img, ref)
        assert c["within_1lsb"] >= 0.999, (loc, c)
        assert st["media_samples"] > 0
        _close(st, rst)


def test_set_camera_equals_a_scene_built_with_that_camera():
    """The library's look_at (View::StartRender) gives the parser's camera
    vectors: the images agree to FP32 rounding of the vectors."""
    base = scenes.media_spheres(64, 48)
    loc, at, w, h = VIEWS[0]
    a = GpuScene(base)
    a.set_camera(loc, at, base.angle, w, h)
    img_a, st_a = a.render(params=_no_aa(scenes.view_of(base, loc, at, w, h)))
    view = scenes.view_of(base, loc, at, w, h)
    img_b, st_b = GpuScene(view).render(params=_no_aa(view))
    assert np.abs(img_a - img_b).max() <= 1e-5
    assert st_a["number_of_rays"] == st_b["number_of_rays"]


def test_set_camera_rejects_bad_cameras():
    base = scenes.media_spheres(32, 24)
    gpu = GpuScene(base)
    with pytest.raises(abi.PovGpuError) as e:          # inside the media box
        gpu.set_camera((0.0, 0.0, 0.0), (0.0, 0.0, 5.0), base.angle, 32, 24)
    assert e.value.status == abi.POV_GPU_E_UNSUPPORTED
    with pytest.raises(abi.PovGpuError) as e:          # look_at at the location
        gpu.set_camera((0.0, 4.0, -25.0), (0.0, 4.0, -25.0), base.angle, 32, 24)
    assert e.value.status == abi.POV_GPU_E_INVALID
    # the camera it had still renders
    img, st = gpu.render(params=_no_aa(base))
    assert st["device_error"] == 0 and img.shape == (24, 32, 4)
