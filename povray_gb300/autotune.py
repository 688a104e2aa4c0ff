"""Autotuner of the trace path's launch shapes.

The traversal and queue kernels are persistent over device-resident ray
queues (warps claim rays with one atomic), so how many blocks run, how many
threads each has and how many registers a thread may keep decide how well
the node and triangle loads are hidden.  The best shape depends on the
scene and the device, so it is measured: this module times one frame of a
workload (CUDA events on the launch stream, L2 flushed between frames, the
median of several frames) for candidate PovGpuLaunchConfig values, searching
coordinate by coordinate from the library's defaults, and records the best
per workload and image size in launch_table.json beside this file.
bench.py and callers apply the recorded entry with
GpuScene.set_launch_config(**entry["config"]).

The tree itself is one of the choices: the library's binned-SAH tree or
the reference's own bounding tree (objects as single leaves with their
Compute_BBox boxes, each mesh2's tree under its leaf), which suits scenes of
few expensive objects (CSG, tori) better than leaves of up to eight.

The traversal stack depth is not a tuning knob: it is set from the depth of
the scene's tree so that no push can overflow (a smaller one would not be
correct, a larger one only costs shared memory).

    python -m povray_gb300.autotune --workload mesh_spheres --write
"""
import argparse
import json
import os
import statistics

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "launch_table.json")

DEFAULT = {"trace_blocks_per_sm": 8, "trace_block": 128, "trace_occupancy": 0, "shade_blocks_per_sm": 16,
           "bounding_tree": 0}
SPACE = {
    "bounding_tree": [0, 1],
    "trace_blocks_per_sm": [4, 6, 8, 12, 16],
    "trace_block": [64, 128],
    "trace_occupancy": [0, 1],
    "shade_blocks_per_sm": [8, 16, 32],
}


def table_key(workload, width, height):
    return "%s %dx%d" % (workload, width, height)


def load_table(path=TABLE):
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def tuned_config(workload, width, height, path=TABLE):
    """The recorded launch shape of a workload at an image size, or None."""
    e = load_table(path).get(table_key(workload, width, height))
    return dict(e["config"]) if e else None


def _frame_timer(scene, gpu):
    import torch
    from . import scenes
    stream = torch.cuda.current_stream()
    gpu.set_stream(stream.cuda_stream)
    params = scene.render_params()
    blocks = scenes.blocks_for(params.width, params.height)
    out = torch.empty((params.width * params.height, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def frame_ms(frames):
        ms = []
        for _ in range(frames):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if scene.radiosity is not None:
                gpu.radiosity_pretrace(blocks, params)
            gpu.trace_blocks(blocks, params, out=out.data_ptr())
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)
    return frame_ms


def tune(scene, frames=5, warmup=2, rounds=2, log=None):
    """Coordinate search over SPACE from DEFAULT on `scene`.  Returns
    (best config, its frame ms, the default's frame ms, shapes timed)."""
    from .render import GpuScene
    gpu = GpuScene(scene)
    frame_ms = _frame_timer(scene, gpu)
    cache = {}

    def measure(cfg):
        k = tuple(sorted(cfg.items()))
        if k not in cache:
            gpu.set_launch_config(**cfg)
            frame_ms(warmup)
            cache[k] = frame_ms(frames)
            if log:
                log("%s %.3f ms" % (json.dumps(cfg), cache[k]))
        return cache[k]

    best = dict(DEFAULT)
    best_ms = default_ms = measure(best)
    for _ in range(rounds):
        changed = False
        for name, values in SPACE.items():
            for v in values:
                cand = dict(best, **{name: v})
                ms = measure(cand)
                if ms < best_ms * 0.995:   # a change must beat the noise
                    best, best_ms, changed = cand, ms, True
        if not changed:
            break
    return best, best_ms, default_ms, len(cache)


def main():
    from . import scenes
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="mesh_spheres", choices=sorted(scenes.WORKLOADS))
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--frames", type=int, default=5)
    ap.add_argument("--write", action="store_true", help="record the result in the table")
    ap.add_argument("--table", default=TABLE, help="the table file (default: launch_table.json beside this module)")
    args = ap.parse_args()
    import torch
    scene = scenes.WORKLOADS[args.workload](args.width, args.height)
    best, best_ms, default_ms, n = tune(scene, frames=args.frames, log=print)
    entry = {"config": best, "frame_ms": round(best_ms, 4), "default_frame_ms": round(default_ms, 4),
             "shapes_timed": n, "device": torch.cuda.get_device_name(0),
             "method": "coordinate search from the defaults, median of %d frames per shape, L2 flushed" % args.frames}
    print(json.dumps({table_key(args.workload, args.width, args.height): entry}))
    if args.write:
        t = load_table(args.table)
        t[table_key(args.workload, args.width, args.height)] = entry
        with open(args.table, "w") as f:
            json.dump(t, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main()
