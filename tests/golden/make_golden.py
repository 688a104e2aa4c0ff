"""Generates the golden fixtures of this directory from the reference itself.

Runs only where the reference sources are present (it drives
oracle/_ref/pov_oracle and oracle/_ref/povray_ref, built from them by
oracle/refbuild/Makefile):

    python tests/golden/make_golden.py [case ...]

For every case it writes the scene's SDL to a temporary directory, has the
reference parse and render it, and stores in <case>.npz:
  pixels       float32 (H, W, 4) linear RGBT from TracePixel::operator()
               at pixel centres (no antialiasing)
  stats        JSON of Number_Of_Rays / Shadow_Ray_Tests / ... counters
  ray_org/dir  float64 probe rays (strided camera rays + random rays)
  hit_object, hit_triangle, hit_t   Trace::FindIntersection of each probe
  camera       the camera vectors after Parse_Camera
and, for cases rendered with adaptive antialiasing, the reference CLI's own
output (+AM2, jitter off):
  aa_u8        uint8 (H, W, 3), the PPM it writes (BT.709 transfer curve)
  aa_stats     JSON of its statistics printout (Pixels, Samples, Rays,
               Shadow Ray Tests, Succeeded)
Radiosity cases (radiosity_cases) hold the reference CLI's own radiosity
renders instead (run_radiosity), and pretrace_jitter.npy the pretrace jitter
table of the reference's radiosity task.  <case>.pgsf.gz (SCENE_FILE_CASES)
is the reference parser's SceneData of the case flattened into the C ABI's
scene description (write_scene_files; format in povray_gb300/scenefile.py),
and radiosity_room_160x90.rca.gz the reference CLI's own radiosity cache
file of that room (write_radiosity_cache_file, +RFO).
The cases are small so the fixtures stay around a megabyte.
"""
import json
import os
import re
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from povray_gb300 import scenes  # noqa: E402
from povray_gb300.encode import read_ppm  # noqa: E402

POV_ORACLE = os.path.join(ROOT, "oracle", "_ref", "pov_oracle")
POVRAY_REF = os.path.join(ROOT, "oracle", "_ref", "povray_ref")


def cases():
    """name -> (scene, probe stride, random-origin half-extent)."""
    return {
        "spheres_plane_320x240": (scenes.spheres_plane(320, 240), 4, 12.0),
        "mesh_spheres_small_160x90": (scenes.mesh_spheres(160, 90, mesh_n=24, n_spheres=64), 2, 12.0),
        "csg_torus_grid_160x90": (scenes.csg_torus_grid(160, 90, n=16), 2, 16.0),
        "area_room_160x90": (scenes.radiosity_room(160, 90, n_spheres=40, radiosity=False), 2, 9.0),
        "area_room_adaptive_160x90": (scenes.radiosity_room(160, 90, n_spheres=40, radiosity=False, area=(5, 5),
                                                            adaptive=1, orient=True), 2, 9.0),
        "light_types_160x120": (scenes.light_types(160, 120), 2, 9.0),
        "glass_reflective_160x120": (scenes.glass_reflective(160, 120), 2, 8.0),
        "patterned_spheres_160x120": (scenes.patterned_spheres(160, 120), 2, 8.0),
        "glass_patterns_160x120": (scenes.glass_patterns(160, 120), 2, 8.0),
        "backlit_sheets_160x120": (scenes.backlit_sheets(160, 120), 2, 6.0),
        "metal_spheres_160x120": (scenes.metal_spheres(160, 120), 2, 6.0),
        "media_spheres_160x120": (scenes.media_spheres(160, 120), 2, 9.0),
        "media_hazy_160x120": (scenes.media_spheres(160, 120, scattering_type=2), 4, 9.0),
        "media_murky_160x120": (scenes.media_spheres(160, 120, scattering_type=3), 4, 9.0),
        "media_rayleigh_160x120": (scenes.media_spheres(160, 120, scattering_type=4), 4, 9.0),
        "media_hg_160x120": (scenes.media_spheres(160, 120, scattering_type=5, eccentricity=0.6), 4, 9.0),
        "media_sphere_160x120": (scenes.media_spheres(160, 120, container="sphere", scattering_type=5,
                                                      eccentricity=-0.3), 4, 9.0),
        "media_glow_160x120": (scenes.media_spheres(160, 120, scattering=0.0, absorption=(0.06, 0.03, 0.01),
                                                    emission=(0.02, 0.01, 0.03)), 4, 9.0),
        "textured_spheres_160x120": (scenes.textured_spheres(160, 120), 2, 8.0),
        "textured_perlin_160x120": (scenes.textured_spheres(160, 120, noise_generator=3), 2, 8.0),
        "textured_original_160x120": (scenes.textured_spheres(160, 120, noise_generator=1), 2, 8.0),
        "textured_turbulent_160x120": (scenes.textured_spheres(160, 120, n_spheres=16, turbulent=True), 2, 8.0),
        "textured_turbulent_perlin_160x120": (scenes.textured_spheres(160, 120, n_spheres=16, turbulent=True,
                                                                      noise_generator=3), 2, 8.0),
        "bumpy_spheres_160x120": (scenes.bumpy_spheres(160, 120), 2, 8.0),
        "bumpy_perlin_160x120": (scenes.bumpy_spheres(160, 120, noise_generator=3), 2, 8.0),
        "bumpy_waves_160x120": (scenes.bumpy_spheres(160, 120, waves=True), 2, 8.0),
        "shaped_spheres_160x120": (scenes.shaped_spheres(160, 120, n_spheres=22), 2, 8.0),
        "glass_spheres_160x120": (scenes.glass_spheres(160, 120), 2, 8.0),
    }


def radiosity_cases():
    """name -> scene, rendered by the reference CLI with radiosity."""
    return {
        "radiosity_room_160x90": scenes.radiosity_room(160, 90, n_spheres=40, count=50),
    }


def probe_rays(scene, stride, extent=12.0, n_random=2000, seed=11):
    hh, ww = np.mgrid[0:scene.height:stride, 0:scene.width:stride]
    o, d = scene.camera_rays(ww.ravel(), hh.ravel())
    rng = np.random.Generator(np.random.PCG64(seed))
    ro = rng.uniform(-extent, extent, size=(n_random, 3))
    rd = rng.normal(size=(n_random, 3))
    rd /= np.linalg.norm(rd, axis=1)[:, None]
    return np.concatenate([o, ro]), np.concatenate([d, rd])


def read_hdr(path):
    """Radiance RGBE file (+FH output) -> float32 (H, W, 3); new-style
    run-length scanlines and flat scanlines."""
    data = open(path, "rb").read()
    pos = 0
    while True:                                  # header up to the blank line
        end = data.index(b"\n", pos)
        line = data[pos:end]
        pos = end + 1
        if line == b"":
            break
    end = data.index(b"\n", pos)
    dims = data[pos:end].split()
    pos = end + 1
    h, w = int(dims[1]), int(dims[3])
    out = np.zeros((h, w, 4), dtype=np.uint8)
    for y in range(h):
        if data[pos] == 2 and data[pos + 1] == 2 and (data[pos + 2] << 8 | data[pos + 3]) == w:
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        out[y, x:x + n - 128, c] = data[pos]
                        pos += 1
                        x += n - 128
                    else:
                        out[y, x:x + n, c] = np.frombuffer(data[pos:pos + n], dtype=np.uint8)
                        pos += n
                        x += n
        else:
            out[y] = np.frombuffer(data[pos:pos + 4 * w], dtype=np.uint8).reshape(w, 4)
            pos += 4 * w
    e = out[..., 3].astype(np.int32)
    f = np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)
    return ((out[..., :3].astype(np.float64) + 0.5) * f[..., None] * (e > 0)[..., None]).astype(np.float32)


def radiosity_stats(text):
    """Radiosity counters of the reference's statistics printout
    (renderfrontend.cpp): samples per pass and depth, reuse, rays shot."""
    out = {}
    m = re.search(r"Radiosity samples calculated:\s+(\d+)", text)
    out["samples"] = int(m.group(1)) if m else 0
    m = re.search(r"Radiosity samples reused:\s+(\d+)", text)
    out["reused"] = int(m.group(1)) if m else 0
    m = re.search(r"Radiosity sample rays shot:\s+(\d+)", text)
    out["rays_shot"] = int(m.group(1)) if m else 0
    for row in re.finditer(r"^\s+(\d+|Final|Total)\s+(\d+)\s+(\d+)\s+(\d+)\s*$", text, re.M):
        out["pass_" + row.group(1).lower()] = [int(row.group(2)), int(row.group(3))]
    return out


def cli_stats(text):
    """Counters of the reference's statistics printout (renderfrontend.cpp:1834-1933)."""
    out = {}
    pats = {"number_of_pixels": r"Pixels:\s+(\d+)", "number_of_samples": r"Samples:\s+(\d+)",
            "number_of_rays": r"Rays:\s+(\d+)", "shadow_ray_tests": r"Shadow Ray Tests:\s+(\d+)",
            "shadow_rays_succeeded": r"Succeeded:\s+(\d+)\s*\n", "reflected_rays": r"Reflected Rays:\s+(\d+)"}
    for k, p in pats.items():
        m = re.search(p, text)
        out[k] = int(m.group(1)) if m else 0
    return out


def run(case, scene, stride, extent, tmp):
    pov = os.path.join(tmp, case + ".pov")
    with open(pov, "w") as f:
        f.write(scene.sdl())
    w, h = str(scene.width), str(scene.height)
    rgbt = os.path.join(tmp, case + ".rgbt")
    out = subprocess.run([POV_ORACLE, pov, w, h, "pixels", rgbt], check=True, capture_output=True, text=True)
    stats = json.loads(out.stdout.strip().splitlines()[-1])
    pixels = np.fromfile(rgbt, dtype=np.float32).reshape(scene.height, scene.width, 4)
    o, d = probe_rays(scene, stride, extent)
    rays = os.path.join(tmp, case + ".rays")
    with open(rays, "wb") as f:
        f.write(struct.pack("<i", o.shape[0]))
        f.write(np.concatenate([o, d], axis=1).astype("<f8").tobytes())
    hits = os.path.join(tmp, case + ".hits")
    subprocess.run([POV_ORACLE, pov, w, h, "rays", rays, hits], check=True, capture_output=True)
    hr = np.fromfile(hits, dtype=np.dtype([("object", "<i4"), ("triangle", "<i4"), ("t", "<f8")]))
    # the camera vectors the reference's parser produced
    dump = os.path.join(tmp, case + ".scene.txt")
    subprocess.run([POV_ORACLE, pov, w, h, "scene", dump], check=True, capture_output=True)
    cam = {}
    with open(dump) as f:
        for line in f:
            k, *v = line.split()
            if k in ("location", "direction", "right", "up"):
                cam[k] = [float(x) for x in v]
    camera = np.array([cam["location"], cam["direction"], cam["right"], cam["up"]], dtype=np.float64)
    extra = {}
    if scene.antialias is not None:
        thr, depth = scene.antialias
        ppm = os.path.join(tmp, case + "_aa.ppm")
        r = subprocess.run([POVRAY_REF, "+I" + pov, "+W" + w, "+H" + h, "-D", "+FP", "+A%g" % thr, "+AM2",
                            "+R%d" % depth, "-J", "+WT4", "+O" + ppm], capture_output=True, text=True, cwd=tmp)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:])
        extra["aa_u8"] = read_ppm(ppm)
        extra["aa_stats"] = json.dumps(cli_stats(r.stdout + r.stderr))
    np.savez_compressed(os.path.join(HERE, case + ".npz"), pixels=pixels, stats=json.dumps(stats),
                        ray_org=o, ray_dir=d, hit_object=hr["object"], hit_triangle=hr["triangle"],
                        hit_t=hr["t"], camera=camera, **extra)
    print(case, stats, extra.get("aa_stats", ""), "hits", int((hr["object"] >= 0).sum()), "/", len(hr))


def run_radiosity(case, scene, tmp):
    """The reference CLI renders the scene with radiosity, once with one
    render thread (a fixed sample order: the oracle restates that order) and
    once with eight (another valid order: their difference is the sampling
    noise floor).  Stores linear RGB from the +FH (RGBE) output and the
    statistics printout."""
    pov = os.path.join(tmp, case + ".pov")
    with open(pov, "w") as f:
        f.write(scene.sdl())
    w, h = str(scene.width), str(scene.height)
    out = {}
    for threads in (1, 8):
        hdr = os.path.join(tmp, "%s_wt%d.hdr" % (case, threads))
        r = subprocess.run([POVRAY_REF, "+I" + pov, "+W" + w, "+H" + h, "-D", "+FH", "-A", "+WT%d" % threads,
                            "+O" + hdr], capture_output=True, text=True, cwd=tmp)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:])
        text = r.stdout + r.stderr
        out["rad_pixels_wt%d" % threads] = read_hdr(hdr)
        out["rad_stats_wt%d" % threads] = json.dumps(dict(radiosity_stats(text), **cli_stats(text)))
    np.savez_compressed(os.path.join(HERE, case + ".npz"), **out)
    print(case, out["rad_stats_wt1"])


def write_radiosity_cache_file(tmp, case="radiosity_room_160x90"):
    """The reference CLI's own radiosity cache file (+RFO, one thread) of
    the golden room -> <case>.rca.gz: every sample its pretrace and final
    trace gathered, in the .rca text format (ot_write_block,
    source/core/support/octree.cpp:1345-1370)."""
    import gzip
    scene = radiosity_cases()[case]
    pov = os.path.join(tmp, case + ".pov")
    with open(pov, "w") as f:
        f.write(scene.sdl())
    rca = os.path.join(tmp, case + ".rca")
    hdr = os.path.join(tmp, case + "_rfo.hdr")
    r = subprocess.run([POVRAY_REF, "+I" + pov, "+W%d" % scene.width, "+H%d" % scene.height, "-D", "+FH", "-A",
                        "+WT1", "+RFO", "+RF" + rca, "+O" + hdr], capture_output=True, text=True, cwd=tmp)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-2000:])
    with open(rca, "rb") as f, gzip.GzipFile(os.path.join(HERE, case + ".rca.gz"), "wb", mtime=0) as g:
        data = f.read()
        g.write(data)
    print(case, "cache file:", data.count(b"\nC") + data.startswith(b"C"), "samples")


SCENE_FILE_CASES = ("spheres_plane_320x240", "mesh_spheres_small_160x90", "csg_torus_grid_160x90",
                    "area_room_160x90", "media_spheres_160x120", "radiosity_room_160x90",
                    "textured_spheres_160x120", "textured_turbulent_perlin_160x120", "bumpy_spheres_160x120",
                    "bumpy_waves_160x120", "shaped_spheres_160x120", "glass_spheres_160x120",
                    "media_sphere_160x120", "media_hg_160x120", "light_types_160x120",
                    "glass_reflective_160x120", "patterned_spheres_160x120",
                    "glass_patterns_160x120")


def write_scene_files(tmp):
    """The reference's parse of each case flattened into the C ABI's scene
    description (pov_oracle ... desc: oracle/refbuild/pov_flatten.cpp walks
    the SceneData the reference's parser built) -> <case>.pgsf.gz."""
    import gzip
    allc = dict((k, v[0]) for k, v in cases().items())
    allc.update(radiosity_cases())
    for case in SCENE_FILE_CASES:
        scene = allc[case]
        pov = os.path.join(tmp, case + ".pov")
        with open(pov, "w") as f:
            f.write(scene.sdl())
        raw = os.path.join(tmp, case + ".pgsf")
        subprocess.run([POV_ORACLE, pov, str(scene.width), str(scene.height), "desc", raw], check=True,
                       capture_output=True)
        with open(raw, "rb") as f, gzip.GzipFile(os.path.join(HERE, case + ".pgsf.gz"), "wb", mtime=0) as g:
            g.write(f.read())
        print(case, "scene file")


def write_jitter_table():
    """RadiosityTask's pretrace jitter table (RandomDoubleSequence(-1,1,2047),
    radiositytask.cpp:99) as the reference generates it."""
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "jitter.bin")
        subprocess.run([POV_ORACLE, "-", "0", "0", "jitter", path], check=True)
        np.save(os.path.join(HERE, "pretrace_jitter.npy"), np.fromfile(path, dtype="<f8"))


def main():
    if not os.path.exists(POV_ORACLE):
        sys.exit("build the reference first: make -C oracle/refbuild")
    if len(sys.argv) == 1 or "pretrace_jitter" in sys.argv[1:]:
        write_jitter_table()
    if len(sys.argv) == 1 or "scene_files" in sys.argv[1:]:
        with tempfile.TemporaryDirectory() as tmp:
            write_scene_files(tmp)
    if len(sys.argv) == 1 or "radiosity_cache_file" in sys.argv[1:]:
        with tempfile.TemporaryDirectory() as tmp:
            write_radiosity_cache_file(tmp)
    with tempfile.TemporaryDirectory() as tmp:
        for case, scene in radiosity_cases().items():
            if len(sys.argv) > 1 and case not in sys.argv[1:]:
                continue
            run_radiosity(case, scene, tmp)
        for case, (scene, stride, extent) in cases().items():
            if len(sys.argv) > 1 and case not in sys.argv[1:]:
                continue
            run(case, scene, stride, extent, tmp)


if __name__ == "__main__":
    main()
