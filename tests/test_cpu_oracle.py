"""The oracle is pinned against the reference: the golden fixtures were
dumped by the reference renderer itself (tests/golden/make_golden.py) for
the same SDL scenes, and the oracle must reproduce them."""
import json
import os

import numpy as np
import pytest

from oracle.pyoracle import Oracle
from povray_gb300 import scenes
from tests.golden.make_golden import cases
from tests.parity import compare_hits, compare_pixels
from povray_gb300.encode import to_u8

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = cases()


def _load(case):
    return np.load(os.path.join(GOLDEN, case + ".npz"))


@pytest.mark.parametrize("case", sorted(CASES))
def test_camera_vectors_match_the_parser(case):
    scene = CASES[case][0]
    g = _load(case)
    d, r, u = scene.camera()
    assert np.array_equal(g["camera"][0], np.array(scene.location))
    assert np.array_equal(g["camera"][1], np.array(d))
    assert np.array_equal(g["camera"][2], np.array(r))
    assert np.array_equal(g["camera"][3], np.array(u))


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_hits_match_reference(case):
    scene = CASES[case][0]
    g = _load(case)
    o = Oracle(scene)
    h = o.trace_rays(g["ray_org"], g["ray_dir"])
    r = compare_hits(h["object"], h["triangle"], h["t"], g["hit_object"], g["hit_triangle"], g["hit_t"],
                     oracle=o, org=g["ray_org"], dirs=g["ray_dir"], t_tol=1e-12)
    assert r["mismatch"] == 0, r
    assert r["t_max_rel"] <= 1e-12, r


def no_aa(scene):
    p = scene.render_params()
    p.antialias = 0
    p.sampling_method = 1
    return p


def _has_area_light(scene):
    return any(l["kind"] == 1 for l in scene.lights)


def _has_media(scene):
    return bool(getattr(scene, "medias", None))


def _reflects_through_glass(scene):
    """A transparent surface that also reflects (a hit traces two rays)."""
    return any((m.filter or m.transmit) and m.reflection for m in scene.materials)


def check_branching_counters(st, rs):
    """Counters of scenes whose transparent surfaces also reflect.  The
    refraction counters are exact.  Two count-only effects are bounded
    (pixels are unaffected):
    * Fresnel reflectance at a relative ior of exactly 1 (leaving the inner
      of two nested interiors, trace.cpp:2611-2618) is zero in exact
      arithmetic; computed, it is the residue of (1 + cos^2) - 1 - cos^2,
      zero or not by the last bit of the cosine, and a non-zero one traces
      (and counts) a reflection ray that bails at the ADC bailout at once:
      rays and reflected rays differ by the same few, either way.
    * The shadow cache (trace.cpp:1990-2023): a cached opaque object behind
      a transparent one ends the reference's shadow ray in one counted
      test where the full test counts the transparent surface too; the
      oracle and the GPU never take the shortcut: one test and one success
      more, never fewer."""
    for k in ("transmitted_rays", "refracted_rays", "internal_reflected_rays"):
        assert st[k] == rs[k], (k, st[k], rs[k])
    dr = st["number_of_rays"] - rs["number_of_rays"]
    assert dr == st["reflected_rays"] - rs["reflected_rays"], (st, rs)
    assert abs(dr) <= 1e-3 * rs["number_of_rays"], (st, rs)
    dt = st["shadow_ray_tests"] - rs["shadow_ray_tests"]
    assert dt == st["shadow_rays_succeeded"] - rs["shadow_rays_succeeded"], (st, rs)
    assert 0 <= dt <= 1e-3 * rs["shadow_ray_tests"], (st, rs)


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_pixels_and_counters_match_reference(case):
    """Exact, except where the reference's light-source shadow cache decides
    a shadow ray: its test of the cached object accepts hits in
    [MIN_ISECT_DEPTH, depth) (trace.cpp:1999, 346-390) where the full test
    needs (SHADOW_TOLERANCE, depth - SHADOW_TOLERANCE) (trace.cpp:2034-2037),
    and which object is cached depends on render order.  With area lights
    (many shadow rays per point) a few samples of a point whose shadow ray
    passes within 1e-3 of another surface flip: bounded here at 0.01% of the
    shadow rays, less than 1/255 linear per pixel and 99.9% of 8-bit
    channels within one step.  Inside a media container the cached object
    can lie beyond the container wall, which the full test counts as a hit
    of its own: one test and one success fewer in the reference (bounded
    the same way); media samples are counted exactly."""
    scene = CASES[case][0]
    g = _load(case)
    img, st = Oracle(scene).render(threads=4, params=no_aa(scene))
    ref = g["pixels"]
    rs = json.loads(str(g["stats"]))
    diff = np.abs(img - ref).max(axis=2)
    if _has_media(scene):
        assert diff.max() <= 1e-5, float(diff.max())
        for k in ("number_of_rays", "reflected_rays", "transmitted_rays", "media_samples"):
            assert st[k] == rs[k], (k, st[k], rs[k])
        # at most one test and one success per shadow ray that starts inside
        # the container: 1e-4 of the shadow tests where the media samples'
        # own shadow rays dominate, 1% of the rays without scattering
        bound = max(1e-4 * rs["shadow_ray_tests"], 0.01 * rs["number_of_rays"])
        for k in ("shadow_ray_tests", "shadow_rays_succeeded"):
            assert 0 <= st[k] - rs[k] <= bound, (k, st[k], rs[k])
        assert compare_pixels(img, ref)["max_lsb"] <= 1
    elif _reflects_through_glass(scene):
        # one pixel in 10^4 may take another path at a grazing hit
        assert diff.max() < 1.0 / 255.0 and (diff <= 1e-5).mean() >= 0.9999, float(diff.max())
        check_branching_counters(st, rs)
        assert compare_pixels(img, ref)["max_lsb"] <= 1
    elif _has_area_light(scene):
        assert diff.max() < 1.0 / 255.0 and (diff <= 1e-5).mean() >= 0.999, float(diff.max())
        for k in ("shadow_ray_tests", "shadow_rays_succeeded"):
            assert abs(st[k] - rs[k]) <= 1e-4 * rs["shadow_ray_tests"], (k, st[k], rs[k])
        assert st["number_of_rays"] == rs["number_of_rays"]
        assert compare_pixels(img, ref)["within_1lsb"] >= 0.999
    else:
        assert diff.max() <= 1e-5
        for k in ("number_of_rays", "shadow_ray_tests", "shadow_rays_succeeded", "reflected_rays"):
            assert st[k] == rs[k], (k, st[k], rs[k])
        if "refracted_rays" in rs:   # transparent scenes: the refraction counters too
            for k in ("transmitted_rays", "refracted_rays", "internal_reflected_rays"):
                assert st[k] == rs[k], (k, st[k], rs[k])
        assert compare_pixels(img, ref)["max_lsb"] <= 1


@pytest.mark.parametrize("case", sorted(c for c in CASES if CASES[c][0].antialias is not None))
def test_oracle_adaptive_aa_matches_reference_cli(case):
    """AdaptiveSupersamplingM2 restated: the reference CLI's PPM within 1 LSB
    and every counter of its statistics printout exact."""
    scene = CASES[case][0]
    g = _load(case)
    img, st = Oracle(scene).render(threads=4)
    got = to_u8(img, "bt709").astype(int)
    d = np.abs(got - g["aa_u8"].astype(int))
    assert d.max() <= 1 and (d == 0).mean() > 0.999
    rs = json.loads(str(g["aa_stats"]))
    for k in ("number_of_pixels", "number_of_samples", "number_of_rays", "shadow_ray_tests",
              "shadow_rays_succeeded", "reflected_rays"):
        assert st[k] == rs[k], (k, st[k], rs[k])


def test_oracle_is_thread_count_invariant():
    s = scenes.mesh_spheres(96, 54, mesh_n=12, n_spheres=32)
    o = Oracle(s)
    a, sa = o.render(threads=1)
    b, sb = o.render(threads=5)
    assert np.array_equal(a, b)
    assert sa == sb


def test_oracle_subrectangle_equals_full_render():
    s = scenes.spheres_plane(64, 48, n_spheres=16)
    o = Oracle(s)
    full, _ = o.render(threads=2)
    part, _ = o.render(x0=10, y0=7, x1=41, y1=30, threads=2)
    assert np.array_equal(full[7:30, 10:41], part)


def test_oracle_radiosity_matches_reference_single_thread_render():
    """Radiosity (pretrace passes + final trace, octree-addressed sample
    cache, Halton gather directions) restated in the reference's
    single-thread order: every radiosity counter of the reference CLI's
    statistics printout equal, and its +FH image within the RGBE format's
    own precision (relative RMSE well under the 8-thread render's distance
    from the 1-thread one)."""
    from tests.golden.make_golden import radiosity_cases
    scene = radiosity_cases()["radiosity_room_160x90"]
    g = _load("radiosity_room_160x90")
    img, st = Oracle(scene).render(threads=1)
    rs = json.loads(str(g["rad_stats_wt1"]))
    assert st["radiosity_gathers"] == rs["samples"]
    assert st["radiosity_reuse"] == rs["reused"]
    assert st["radiosity_rays"] == rs["rays_shot"]
    assert [st["radiosity_gathers_d0"], st["radiosity_gathers_d1"]] == rs["pass_total"]
    assert st["number_of_rays"] == rs["number_of_rays"]
    assert st["number_of_pixels"] == rs["number_of_pixels"]
    # the shadow cache may decide a few shadow rays (see above)
    assert abs(st["shadow_ray_tests"] - rs["shadow_ray_tests"]) <= 1e-4 * rs["shadow_ray_tests"]
    assert abs(st["shadow_rays_succeeded"] - rs["shadow_rays_succeeded"]) <= 1e-4 * rs["shadow_ray_tests"]
    ref = g["rad_pixels_wt1"]
    a = img[..., :3]
    rel = np.sqrt(((a - ref) ** 2).mean()) / ref.mean()
    floor = np.sqrt(((g["rad_pixels_wt8"] - ref) ** 2).mean()) / ref.mean()
    assert rel < 0.005 and rel < 0.2 * floor, (rel, floor)
    assert np.abs(a - ref).max() < 0.01


def _grid(width, height, stride):
    ys, xs = np.mgrid[stride // 2:height:stride, stride // 2:width:stride]
    return np.stack([xs.ravel(), ys.ravel()], 1)


def test_converged_radiosity_agrees_with_reference_render():
    """The oracle's converged mode (every radiosity query gathered without
    the cache, 256 / 16 stratified rays at depth 0 / 1, FP64 sums) against
    the reference's own one-thread radiosity render of the golden room:
    the means agree within 1%, and the converged image is closer to the
    reference's render than the reference's own 8-thread render is (the
    reference's sampling-and-reuse error is the larger one)."""
    from tests.golden.make_golden import radiosity_cases
    scene = radiosity_cases()["radiosity_room_160x90"]
    g = _load("radiosity_room_160x90")
    px = _grid(scene.width, scene.height, 4)
    out, _ = Oracle(scene).render_converged(px, (256, 16), seed=1)
    a = out[:, :3]
    r1 = g["rad_pixels_wt1"][px[:, 1], px[:, 0]]
    r8 = g["rad_pixels_wt8"][px[:, 1], px[:, 0]]

    def rel(x, y):
        return float(np.sqrt(((x - y) ** 2).mean()) / y.mean())
    info = dict(mean_ratio=float(a.mean() / r1.mean()), gt_ref1=rel(r1, a), ref8_ref1=rel(r8, r1))
    assert abs(a.mean() / r1.mean() - 1.0) < 0.01, info
    assert rel(r1, a) < rel(r8, r1), info


def test_converged_radiosity_is_thread_count_invariant():
    scene = scenes.radiosity_room(64, 36, n_spheres=20, count=50)
    px = _grid(64, 36, 6)
    o = Oracle(scene)
    a, _ = o.render_converged(px, (64, 4), seed=3, threads=1)
    b, _ = o.render_converged(px, (64, 4), seed=3, threads=4)
    c, _ = o.render_converged(px, (64, 4), seed=4, threads=4)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)


def test_converged_truth_fixture_reproduces():
    """A few pixels of the committed FP64 truth of the 1280x720 room
    (tests/golden/make_converged.py) rendered again: the same values (the
    per-pixel random sequences depend only on the seed and the pixel)."""
    t = np.load(os.path.join(GOLDEN, "radiosity_room_converged_1280x720.npz"))
    info = json.loads(str(t["info"]))
    scene = scenes.radiosity_room(1280, 720)
    pick = np.arange(0, len(t["pixels"]), 997)
    out, _ = Oracle(scene).render_converged(t["pixels"][pick], info["counts"], seed=info["seed"])
    assert np.allclose(out[:, :3], t["rgb"][pick], rtol=1e-5, atol=1e-7)
    assert info["noise_rel_rmse"] < 0.005


def test_pattern_random_table_matches_reference():
    """The cells pattern's random table (gPatternRands: boost's mt19937 at
    its default seed through uniform_real, restated in the oracle and the
    library) against the reference's own RandomDoubleSequence output: the
    pretrace jitter table is the same generator's first 2047 values mapped
    to [-1, 1), bit for bit."""
    from oracle.pyoracle import pattern_rand
    jitter = np.load(os.path.join(GOLDEN, "pretrace_jitter.npy"))
    table = np.array([pattern_rand(i) for i in range(len(jitter))])
    assert np.array_equal(table * 2.0 - 1.0, jitter)
    assert all(0.0 <= pattern_rand(i) < 1.0 for i in range(0, 4096, 97))
