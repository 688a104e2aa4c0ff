"""Generates the converged radiosity fixture of this directory: the FP64
ground truth of the radiosity room (1280x720, 200 spheres, 4x4 area light,
radiosity count 200, recursion_limit 2, error_bound 0.5).

Rendered by the oracle's converged mode (oracle/povoracle.c,
pov_oracle_render_converged): every radiosity query is answered without
the sample cache by 4096 stratified cosine-weighted rays at bounce depth 0
and 16 at depth 1, summed in FP64; direct light, shadows and shading are the
oracle's restatement of the reference.  Pixels: the centres of an 8x8 grid
of the image, (8i+4, 8j+4), 14,400 of them.  A second render of every 25th
of those pixels with another seed measures the fixture's own sampling noise.

    python tests/golden/make_converged.py          (about 5 minutes on 8 cores)
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import Oracle  # noqa: E402
from povray_gb300 import scenes  # noqa: E402

NAME = "radiosity_room_converged_1280x720.npz"
COUNTS = (4096, 16)
STRIDE = 8


def grid_pixels(width, height, stride=STRIDE):
    ys, xs = np.mgrid[stride // 2:height:stride, stride // 2:width:stride]
    return np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)


def main():
    s = scenes.radiosity_room(1280, 720)
    o = Oracle(s)
    px = grid_pixels(s.width, s.height)
    t = time.time()
    rgbt, st = o.render_converged(px, COUNTS, seed=1)
    dt = time.time() - t
    sub = np.arange(0, len(px), 25)
    alt, _ = o.render_converged(px[sub], COUNTS, seed=2)
    a, b = rgbt[sub, :3], alt[:, :3]
    noise = float(np.sqrt(((a - b) ** 2).mean()) / a.mean() / np.sqrt(2.0))
    info = dict(counts=list(COUNTS), seed=1, stride=STRIDE, seconds=round(dt, 1), rays=st["number_of_rays"],
                noise_rel_rmse=noise, scene="radiosity_room(1280, 720)")
    np.savez_compressed(os.path.join(HERE, NAME), pixels=px, rgb=rgbt[:, :3].astype(np.float32),
                        info=json.dumps(info))
    print(NAME, info)


if __name__ == "__main__":
    main()
