"""Benchmark of the GPU trace path on the 1M-triangle workload.

Workload (one "step" = one full frame through the C ABI):
  mesh_spheres: 1920x1080, 1 spp, no AA; a 1,051,392-triangle displaced
  sphere mesh2 (radius 8, smooth normals) + 1024 spheres + plane y=-9; one
  point light with shadows; reflection 0.3 on every surface;
  max_trace_level 3.  Synthetic, seeded (PCG64 seed 2).

Metric: Mrays/s (primary+shadow) = (Number_Of_Rays + Shadow_Ray_Tests) of
the frame / frame time -- the reference's own counters ("Rays" and "Shadow
Ray Tests" of its statistics printout).

  value  frame time by CUDA events on the launch stream, scene resident in
         HBM, image written to device memory; L2 flushed (256 MiB write)
         between frames, outside the timed events.
  e2e    the same frame with host buffers: block list H2D, RGBT image D2H
         into pinned host memory, all inside the timed region.

`--impl reference` times the CPU implementation of the path (the oracle
restatement of the reference, all host threads) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "mesh_spheres": "mesh_spheres: %dx%d 1spp, 1,051,392-tri displaced-sphere mesh2 + 1024 spheres + plane, "
                    "1 point light w/ shadows, reflection 0.3, max_trace_level 3",
    "csg_torus_grid": "csg_torus_grid: %dx%d, 4096 objects (difference/intersection/merge CSG + FP64 tori), "
                      "adaptive AA method 2 thr 0.1 depth 3, 2 lights w/ shadows, reflection 0.2, max_trace_level 4",
    "spheres_plane": "spheres_plane: %dx%d 1spp, 64 spheres + plane, 2 lights w/ shadows, phong 0.5",
    "radiosity_room": "radiosity_room: %dx%d 1spp, 6-plane room + 200 spheres, 4x4 area light, radiosity count 200 "
                      "recursion_limit 2 error_bound 0.5 (pretrace + final trace per frame)",
    "media_spheres": "media_spheres: %dx%d 1spp, 24 spheres + plane in a scattering media box (rgb 0.05, "
                     "intervals 10, samples 10), 1 point light, reflection 0.2, max_trace_level 3",
    "multiview_media": "multiview_media: 64 views on a circle r=30 y=5 at 256x256/640x480/1280x720/1920x1080 "
                       "(seed 5) of the 1,051,392-tri mesh2 + 10,000 spheres + plane inside a scattering media box "
                       "(rgb 0.05, intervals 10, samples 10), radiosity count 200 recursion_limit 2 error_bound 0.5 "
                       "(pretrace + final trace per view), one step = the next view",
    "bumpy_spheres": "bumpy_spheres: %dx%d 1spp, 12 spheres + plane with bumps/dents/wrinkles/slope normals "
                     "and bozo pigments, phong + specular + reflection 0.25, 1 point light, max_trace_level 3",
}
MULTIVIEW = ("multiview_media",)


def make_scene(args):
    from povray_gb300 import scenes
    if args.workload in MULTIVIEW:
        return scenes.WORKLOADS[args.workload]()
    return scenes.WORKLOADS[args.workload](args.width, args.height)


def workload_name(args):
    if args.workload in MULTIVIEW:
        return WORKLOADS[args.workload]
    return WORKLOADS[args.workload] % (args.width, args.height)


METRIC = "Mrays/s (primary+shadow)"
L2_NOTE = ("GPU arm: L2 flushed between steps (256 MiB write, outside the timed events); "
           "CPU arm: host caches as they are")


def bench_config(args):
    """The config object both arms print (identical, so that the two lines
    describe the same workload)."""
    return {"workload": workload_name(args), "l2": L2_NOTE}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--workload", default="mesh_spheres", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the short lines of the reference's other configurations")
    ap.add_argument("--radiosity-sweep", action="store_true",
                    help="radiosity_room at 1280x720: frame time and RMSE against the FP64 truth over radiosity "
                         "count / error_bound, plain and neural-cache forms (one JSON line each; not the bench line)")
    ap.add_argument("--bounding-tree", default=None, choices=["sah", "reference"],
                    help="the traversal's tree: the library's binned-SAH tree or the reference's bounding tree "
                         "(Build_BBox_Tree, each mesh2's own tree); default: the launch table's choice")
    return ap.parse_args()


def job_totals(times, units, dist=None, device="cpu"):
    """Whole-job figures of a replica run: each time the largest over the
    ranks (the job ends with its slowest rank), each unit count summed over
    the ranks (every replica renders its own frames).  No data-path
    collective: this is the one reduction of the run, after the timed
    region."""
    if dist is None:
        return [float(t) for t in times], [int(u) for u in units]
    import torch
    t = torch.tensor([float(x) for x in times], dtype=torch.float64, device=device)
    u = torch.tensor([int(x) for x in units], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.tolist()], [int(x) for x in u.tolist()]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(scene, cpu_seconds_target=20.0, crop=None):
    """The oracle port (FP64 restatement of the reference), all host threads,
    on a band of rows of the same frame (or a `crop` square at the centre);
    Mrays/s by its own counters."""
    from oracle.pyoracle import Oracle
    # radiosity renders run on one thread in the reference's sample order
    cores = 1 if scene.radiosity is not None else (os.cpu_count() or 1)
    t0 = time.time()
    orc = Oracle(scene)
    build_s = time.time() - t0
    if crop:
        x0, y0 = (scene.width - crop) // 2, (scene.height - crop) // 2
        t = time.time()
        _, st = orc.render(x0, y0, x0 + crop, y0 + crop, threads=0)
        dt = time.time() - t
        return {"value": (st["number_of_rays"] + st["shadow_ray_tests"]) / dt / 1e6, "unit": "Mrays/s",
                "cores": cores, "kind": "port",
                "sample": "oracle restatement, %dx%d px at the centre of a %dx%d view (pretrace over the crop, "
                          "then the final trace), %.1f s wall, tree build %.1f s excluded"
                          % (crop, crop, scene.width, scene.height, dt, build_s)}
    if scene.radiosity is None:
        # the whole frame, as the GPU renders it
        t = time.time()
        _, st = orc.render(0, 0, scene.width, scene.height, threads=0)
        dt = time.time() - t
        return {"value": (st["number_of_rays"] + st["shadow_ray_tests"]) / dt / 1e6, "unit": "Mrays/s",
                "cores": cores, "kind": "port",
                "sample": "oracle restatement, the whole %dx%d frame, %.1f s wall, tree build %.1f s excluded"
                          % (scene.width, scene.height, dt, build_s)}
    rows = 8
    y0 = scene.height // 2
    total_rays, total_t = 0, 0.0
    while total_t < cpu_seconds_target / cores and y0 + rows <= scene.height:
        t = time.time()
        _, st = orc.render(0, y0, scene.width, y0 + rows, threads=0)
        total_t += time.time() - t
        total_rays += st["number_of_rays"] + st["shadow_ray_tests"]
        y0 += rows
        rows *= 2
    rows_done = y0 - scene.height // 2
    return {"value": total_rays / total_t / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
            "sample": "oracle restatement, %d rows x %d px of the frame (rows %d..%d), %.1f s wall, "
                      "tree build %.1f s excluded" % (rows_done, scene.width, scene.height // 2,
                                                        scene.height // 2 + rows_done, total_t, build_s)}


def run_reference(args, rank, world):
    """CPU reference arm: the oracle port of the reference's trace path."""
    if rank != 0:
        return
    from oracle.pyoracle import Oracle
    from povray_gb300 import scenes
    s = make_scene(args)
    if args.workload in MULTIVIEW:
        # a 16x16 crop at the centre of the first view per step: radiosity
        # and media make every pixel of this scene cost milliseconds on a CPU
        loc, at, w, h = scenes.circle_views()[0]
        s = scenes.view_of(s, loc, at, w, h)
        args.width, args.height = w, h
    orc = Oracle(s)
    # the whole frame per step, as the GPU arm renders it; radiosity frames
    # (one thread, the reference's sample order) take a band of rows
    band = args.height if s.radiosity is None else max(8, args.height // 10)
    def step(i):
        t = time.time()
        if args.workload in MULTIVIEW:
            x0, y0 = (args.width - 16) // 2, (args.height - 16) // 2
            _, st = orc.render(x0, y0, x0 + 16, y0 + 16, threads=0)
        else:
            y0 = (i * band) % max(1, args.height - band)
            _, st = orc.render(0, y0, args.width, y0 + band, threads=0)
        return time.time() - t, st["number_of_rays"] + st["shadow_ray_tests"]
    for i in range(args.warmup):
        step(i)
    tt, rr = 0.0, 0
    for i in range(args.steps):
        dt, r = step(args.warmup + i)
        tt += dt
        rr += r
    v = rr / tt / 1e6
    cores = 1 if s.radiosity is not None else (os.cpu_count() or 1)
    if band == args.height:
        sample = "oracle restatement of the reference (FP64 C, pthreads), the whole %dx%d frame per step" % (
            args.width, args.height)
    else:
        sample = "oracle restatement of the reference (FP64 C, one thread: radiosity), %d-row band of the %dx%d " \
                 "frame per step" % (band, args.width, args.height)
    if args.workload in MULTIVIEW:
        sample = "oracle restatement of the reference (FP64 C, one thread: radiosity), 16x16 px at the centre of " \
                 "the first %dx%d view per step (pretrace over the crop, then the final trace)" % (args.width,
                                                                                                   args.height)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args), "rays_per_step": rr // max(1, args.steps),
        "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


TRUTH = os.path.join(ROOT, "tests", "golden", "radiosity_room_converged_1280x720.npz")


def radiosity_forms(args, scene, gpu, stream, params, blocks, dev_out, flush, plain_ms):
    """The radiosity half of the metric: frame time of the plain GPU form
    (the timed frames above) and of the neural-cache form (the network
    trained at the end of each pretrace answers the final trace's uncovered
    queries, gated by its held-out error against error_bound), each with its
    linear-radiance relative RMSE against the FP64 converged truth of this
    scene (tests/golden, the oracle with 4096 / 16 rays per query and no
    reuse) on the truth's pixel grid."""
    import torch
    from povray_gb300 import GpuScene, scenes
    if (args.width, args.height) != (1280, 720) or not os.path.exists(TRUTH):
        return None
    t = np.load(TRUTH)
    px, truth = t["pixels"], t["rgb"]

    def rmse_of_last():
        img = scenes.unblock(dev_out.cpu().numpy(), blocks, args.width, args.height)
        a = img[px[:, 1], px[:, 0], :3]
        return float(np.sqrt(((a - truth) ** 2).mean()) / truth.mean()), float(a.mean() / truth.mean())

    rmse_plain, mean_plain = rmse_of_last()
    nic = GpuScene(scene)
    nic.set_stream(stream.cuda_stream)
    nic.set_neural_cache(True)   # the library's defaults, gate = error_bound
    for _ in range(args.warmup):
        nic.radiosity_pretrace(blocks, params)
        nic.trace_blocks(blocks, params, out=dev_out.data_ptr())
    torch.cuda.synchronize()
    ms, answers, val = [], 0, 0
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        nic.radiosity_pretrace(blocks, params)
        st = nic.trace_blocks(blocks, params, out=dev_out.data_ptr())[1]
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        answers, val = st["nic_answers"], st["nic_val_error_ppm"]
    rmse_nic, mean_nic = rmse_of_last()
    nic_ms = sum(ms) / len(ms)
    return {"plain": {"frame_ms": plain_ms, "rmse_vs_fp64": rmse_plain, "mean_vs_fp64": mean_plain},
            "neural_cache": {"frame_ms": nic_ms, "rmse_vs_fp64": rmse_nic, "mean_vs_fp64": mean_nic,
                             "nic_answers": answers, "held_out_error": val / 1e6},
            "speedup": plain_ms / nic_ms,
            "truth": "oracle converged radiosity (FP64 sums, 4096 / 16 stratified rays per query at depth 0 / 1, "
                     "no reuse) on %d pixels (8x8 grid), own noise %.4f" % (len(px), json.loads(str(t["info"]))
                                                                          ["noise_rel_rmse"])}


def radiosity_sweep():
    """Frame time at fixed RMSE: the 1280x720 room over radiosity count and
    error_bound, plain and with the neural cache, each frame (pretrace +
    final trace) the median of 3 after one, its linear-radiance relative RMSE
    against the FP64 converged truth on the truth's pixels."""
    import torch
    from povray_gb300 import GpuScene, scenes
    t = np.load(TRUTH)
    px, truth = t["pixels"], t["rgb"]
    stream = torch.cuda.current_stream()
    runs = [("plain", c, e) for c, e in [(50, 1.0), (100, 0.8), (200, 0.5), (200, 0.3), (400, 0.3), (400, 0.2),
                                          (800, 0.2), (800, 0.1), (1600, 0.1), (1600, 0.05)]]
    runs += [("neural_cache", c, e) for c, e in [(200, 0.5), (400, 0.3), (800, 0.2)]]
    for form, count, eb in runs:
        s = scenes.radiosity_room(1280, 720, count=count, error_bound=eb)
        g = GpuScene(s)
        g.set_stream(stream.cuda_stream)
        if form == "neural_cache":
            g.set_neural_cache(True)
        p = s.render_params()
        blocks = scenes.BlockBatch(scenes.blocks_for(p.width, p.height))
        out = torch.empty((p.width * p.height, 4), dtype=torch.float32, device="cuda")
        ms = []
        for r in range(4):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            g.radiosity_pretrace(blocks, p)
            g.trace_blocks(blocks, p, out=out.data_ptr())
            e1.record(stream)
            torch.cuda.synchronize()
            if r > 0:
                ms.append(e0.elapsed_time(e1))
        img = scenes.unblock(out.cpu().numpy(), blocks, p.width, p.height)
        a = img[px[:, 1], px[:, 0], :3]
        print(json.dumps({"form": form, "count": count, "error_bound": eb, "frame_ms": float(np.median(ms)),
                          "rmse_vs_fp64": float(np.sqrt(((a - truth) ** 2).mean()) / truth.mean()),
                          "mean_vs_fp64": float(a.mean() / truth.mean())}), flush=True)
        del g


# The reference's other benchmark workloads (64 spheres at 320x240; the
# CSG/torus grid at 1080p with AA; the radiosity room at 720p; the
# multi-view media scene), each timed briefly in the same run beside the
# main line.
OTHER_CONFIGS = (("spheres_plane", 320, 240), ("csg_torus_grid", 1920, 1080), ("radiosity_room", 1280, 720),
                 ("multiview_media", 0, 0))


def other_configs(args, stream, flush, steps=3, warmup=2):
    """One compact line per other configuration: frames by CUDA events on the
    launch stream, L2 flushed between them, scene resident, image in device
    memory; rays (primary + shadow) per second of the timed frames; the
    launch table's shape; radiosity frames include the pretrace, the
    multi-view steps are consecutive views."""
    import torch
    from povray_gb300 import GpuScene, autotune, scenes
    out = []
    for wl, w, h in OTHER_CONFIGS:
        if wl == args.workload:
            continue
        try:
            multiview = wl in MULTIVIEW
            s = scenes.WORKLOADS[wl]() if multiview else scenes.WORKLOADS[wl](w, h)
            gpu = GpuScene(s)
            gpu.set_stream(stream.cuda_stream)
            cfg = None if multiview else autotune.tuned_config(wl, w, h)
            if cfg:
                gpu.set_launch_config(**cfg)
            views = scenes.circle_views() if multiview else None
            if multiview:
                gpu.set_neural_cache(True, shared=True)
            npix = max(vw * vh for _, _, vw, vh in views) if multiview else w * h
            dev = torch.empty((npix, 4), dtype=torch.float32, device="cuda")

            packed = {}

            def batch(vw, vh):
                if (vw, vh) not in packed:
                    packed[(vw, vh)] = scenes.BlockBatch(scenes.blocks_for(vw, vh))
                return packed[(vw, vh)]

            def frame(i):
                if multiview:
                    loc, at, vw, vh = views[i % len(views)]
                    gpu.set_camera(loc, at, s.angle, vw, vh)
                    p, bl = scenes.view_of(s, loc, at, vw, vh).render_params(), batch(vw, vh)
                else:
                    p, bl = s.render_params(), batch(w, h)
                st_pre = gpu.radiosity_pretrace(bl, p) if s.radiosity is not None else None
                st = gpu.trace_blocks(bl, p, out=dev.data_ptr())[1]
                r = st["number_of_rays"] + st["shadow_ray_tests"]
                if st_pre is not None:
                    r += st_pre["number_of_rays"] + st_pre["shadow_ray_tests"]
                return r

            for i in range(warmup):
                frame(i)
            ms, rays = [], 0
            for i in range(steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                rays += frame(warmup + i)
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            desc = WORKLOADS[wl] if multiview else WORKLOADS[wl] % (w, h)
            out.append({"workload": desc, "value": rays / (sum(ms) / 1e3) / 1e6, "unit": "Mrays/s",
                        "ms_per_step": sum(ms) / len(ms), "steps": steps, "warmup": warmup,
                        "launch_config": cfg or "library defaults"})
            del gpu, dev
        except Exception as e:   # a failing extra line must not lose the main one
            out.append({"workload": wl, "error": str(e)[:300]})
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.radiosity_sweep:
        if rank == 0:
            import torch
            torch.cuda.set_device(local)
            radiosity_sweep()
        return
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from povray_gb300 import GpuScene, scenes
    from povray_gb300.abi import STAGE_NAMES  # noqa: F401

    s = make_scene(args)
    gpu = GpuScene(s)
    # the autotuner's launch shape for this workload, when it recorded one
    from povray_gb300 import autotune
    launch_cfg = None if args.workload in MULTIVIEW else autotune.tuned_config(args.workload, args.width, args.height)
    if args.bounding_tree is not None:
        launch_cfg = dict(launch_cfg or {}, bounding_tree=1 if args.bounding_tree == "reference" else 0)
    if launch_cfg:
        gpu.set_launch_config(**launch_cfg)
    stream = torch.cuda.current_stream()
    gpu.set_stream(stream.cuda_stream)
    multiview = args.workload in MULTIVIEW
    views = scenes.circle_views() if multiview else None
    params = s.render_params()
    # render blocks packed for the C ABI once per resolution (the reference's
    # render task passes its block array the same way)
    packed = {}

    def batch(w, h):
        if (w, h) not in packed:
            packed[(w, h)] = scenes.BlockBatch(scenes.blocks_for(w, h))
        return packed[(w, h)]

    blocks = batch(args.width, args.height)
    npix = max(w * h for _, _, w, h in views) if multiview else args.width * args.height
    dev_out = torch.empty((npix, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    radiosity = s.radiosity is not None
    if multiview and radiosity:
        # the neural cache shared across the views, each pretrace training it on
        gpu.set_neural_cache(True, shared=True)

    def view(i):
        """Render params and blocks of step i: the frame, or the next view
        (its camera set without re-parsing)."""
        if not multiview:
            return params, blocks
        loc, at, w, h = views[i % len(views)]
        gpu.set_camera(loc, at, s.angle, w, h)
        return scenes.view_of(s, loc, at, w, h).render_params(), batch(w, h)

    def frame_device(i=0, out_ptr=None):
        """One frame: with radiosity the pretrace over all blocks, then the
        final trace.  Returns the frame's counters, per-call timings and the
        block count and pixels of the frame."""
        p, bl = view(i)
        st_all, tims = None, []
        if radiosity:
            st_all = gpu.radiosity_pretrace(bl, p)
            tims.append(gpu.timings())
        st = gpu.trace_blocks(bl, p, out=out_ptr or dev_out.data_ptr())[1]
        tims.append(gpu.timings())
        if st_all is not None:
            st = {k: st[k] + st_all[k] for k in st if k != "device_error"}
        return st, tims, len(bl), p.width * p.height

    # one profiling frame (outside the timed region): traversal work counts
    gpu.set_profiling(times=False, work=True)
    _, wt, _, _ = frame_device(args.warmup)   # the first timed frame (view)
    work = {k: [sum(t[k][j] for t in wt) for j in range(2)] for k in ("node_visits", "prim_tests", "tri_tests",
                                                                          "rays_traced")}
    # per-stage CUDA-event times and launch counts of the same frames, from
    # profiled frames outside the timed region (stage events keep a plain
    # frame off its captured graph)
    gpu.set_profiling(times=True, work=False)
    for i in range(args.warmup):
        frame_device(i)
    stage_ms = {}
    stage_launches = {}
    for i in range(args.steps):
        flush.zero_()
        _, tims, _, _ = frame_device(args.warmup + i)
        for t in tims:
            for k, v in t["stage_ms"].items():
                stage_ms[k] = stage_ms.get(k, 0.0) + v
            for k, v in t["stage_launches"].items():
                stage_launches[k] = stage_launches.get(k, 0) + v

    # the timed frames: the production path (a plain frame replays its
    # captured graph after its first two calls)
    gpu.set_profiling(times=False, work=False)
    for i in range(args.warmup):
        frame_device(i)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches = 0
    rays = 0
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        st, tims, _, _ = frame_device(args.warmup + i)
        ev[i][1].record(stream)
        launches += sum(t["kernel_launches"] for t in tims)
        rays += st["number_of_rays"] + st["shadow_ray_tests"]
    torch.cuda.synchronize()
    clocks = sampler.stop()
    frame_ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(frame_ms) / 1e3

    # e2e: host buffers through the public call (pinned output)
    host_out = torch.empty((npix, 4), dtype=torch.float32, pin_memory=True)
    for i in range(max(1, args.warmup // 2)):
        frame_device(i, host_out.data_ptr())
    torch.cuda.synchronize()
    e2e_rays, h2d, d2h = 0, 0, 0
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        st, _, nb, npx = frame_device(args.warmup + i, host_out.data_ptr())
        e2e_rays += st["number_of_rays"] + st["shadow_ray_tests"]
        h2d += nb * 16 + (nb + 1) * 4
        d2h += npx * 16
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_wall = time.perf_counter() - t0
    e2e_t = max(e2e_wall, e0.elapsed_time(e1) / 1e3)

    # max over ranks of the times, rays summed over the replicas
    (t_total, e2e_t), (job_rays, job_e2e_rays) = job_totals([t_total, e2e_t], [rays, e2e_rays], dist, "cuda")
    value = job_rays / t_total / 1e6
    e2e_value = job_e2e_rays / e2e_t / 1e6
    # roofline of the dominant kernel (closest-hit traversal): algorithmic
    # bytes = 32 B ray + 16 B hit per ray + 112 B per node visit (the four
    # child boxes and links of a four-wide node) + 48 B per triangle test +
    # 16 B per sphere test
    nv, pt, tt_, rt = work["node_visits"], work["prim_tests"], work["tri_tests"], work["rays_traced"]
    k = 0 if stage_ms.get("trace_closest", 0) >= stage_ms.get("trace_shadow", 0) else 1
    if rt[k] == 0:   # shadow rays through media containers run outside the counted any-hit kernel
        k = 0
    kname = ["trace_closest", "trace_shadow"][k]
    bytes_per_frame = rt[k] * (32 + (16 if k == 0 else 1)) + nv[k] * 112 + tt_[k] * 48 + (pt[k] - tt_[k]) * 16
    kernel_s = stage_ms[kname] / 1e3 / args.steps
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = bytes_per_frame / kernel_s / 1e9
    launches_per_frame = max(1.0, stage_launches.get(kname, args.steps) / args.steps)
    # DRAM bytes of this kernel on this workload from an ncu capture
    # (profiles/traffic.json, keyed by workload, then kernel stage)
    prof = {}
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(args.workload, {}).get(kname, {})
    except Exception:
        pass
    dram_frame = prof.get("dram_bytes_per_frame")
    out = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fp64 grazing re-solve, fp64 camera)",
        "data": "synthetic",
        "config": bench_config(args),
        "rays_per_frame": rays // args.steps, "parallelism": "replica per GPU" if world > 1 else "1 GPU",
        **({"radiosity": {k: st[k] for k in ("radiosity_gathers", "radiosity_reuse", "radiosity_rays",
                                             "radiosity_gathers_d0", "radiosity_gathers_d1")}}
           if radiosity else {}),
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": h2d // args.steps,
                "d2h_bytes_per_step": d2h // args.steps},
        "roofline": {"bound": "hbm", "kernel": "k_trace<%s>" % ("closest" if k == 0 else "any"),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (dram_frame / prof.get("launches_per_frame", launches_per_frame)
                                 if dram_frame else None),
                     "peak_source": "measured" if peaks else "fallback",
                     "algorithmic_bytes_per_launch": bytes_per_frame / launches_per_frame,
                     "launches_per_frame": launches_per_frame,
                     # the byte model charges every node and primitive fetch
                     # as if it came from HBM; ncu's DRAM bytes give the
                     # fraction of HBM the kernel really uses
                     "dram_gbs": dram_frame / kernel_s / 1e9 if dram_frame else None,
                     "dram_frac": dram_frame / kernel_s / 1e9 / peak if dram_frame else None,
                     "l2_hit_rate": prof.get("l2_hit_rate"),
                     "traffic_source": prof.get("source")},
        "stage_ms_per_frame": {k2: v / args.steps for k2, v in stage_ms.items() if v > 0},
        "stage_note": "stage times from the same number of profiled frames outside the timed region",
        "launch_config": launch_cfg or "library defaults (no tuned entry)",
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if radiosity and not multiview:
        out["radiosity_forms"] = radiosity_forms(args, s, gpu, stream, params, blocks, dev_out, flush,
                                                 t_total / args.steps * 1e3)
    if rank == 0 and world == 1 and not args.no_other_configs:
        out["other_configs"] = other_configs(args, stream, flush)
    if rank == 0 and not args.no_cpu_baseline:
        if multiview:
            loc, at, w, h = views[0]
            out["cpu_baseline"] = cpu_baseline(scenes.view_of(s, loc, at, w, h), crop=16)
        else:
            out["cpu_baseline"] = cpu_baseline(s)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
