"""Image output on the device (pov_gpu_encode_u8) against the host
restatement of IntEncode (povray_gb300/encode.py) on the same pixels.

Tolerance (written here, applied below): both sides take the floor of the
encoded value with their own powf, which may differ by one unit in the last
place, so a value within one rounding of a level boundary may land one
level apart: at least 99.99% of channels equal, none more than 1 apart.
"""
import numpy as np
import pytest
import torch

from povray_gb300 import GpuScene, scenes
from povray_gb300.encode import int_encode, to_u8

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    return GpuScene(scenes.spheres_plane(32, 24))


def _pixels(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.1, 1.2, size=(n, 4)).astype(np.float32)
    # edge values: zero, one, the smallest normal, tiny, exact level values
    edge = np.array([0.0, 1.0, 1e-38, 1e-7, 0.0031308, 0.018, 0.5, 1.5, -1.0], dtype=np.float32)
    x[:len(edge), 0] = edge
    x[:255, 1] = (np.arange(255, dtype=np.float32) / 255.0) ** 2.2
    return x


@pytest.mark.parametrize("curve", ["srgb", "bt709"])
def test_encode_matches_host_restatement(gpu, curve):
    x = _pixels(200_000, 7)
    dev = torch.tensor(x, device="cuda")
    got = gpu.encode_u8(dev.data_ptr(), len(x), curve)
    ref = int_encode(x[:, :3], curve)
    d = np.abs(got.astype(int) - ref.astype(int))
    assert d.max() <= 1, int(d.max())
    assert (d == 0).mean() >= 0.9999, float((d == 0).mean())


def test_encode_into_device_memory_and_of_a_render(gpu):
    s = scenes.spheres_plane(64, 48)
    g = GpuScene(s)
    img, _ = g.render()
    dev = torch.tensor(img.reshape(-1, 4), device="cuda")
    out = torch.empty((dev.shape[0], 3), dtype=torch.uint8, device="cuda")
    assert g.encode_u8(dev.data_ptr(), dev.shape[0], "srgb", out=out.data_ptr()) is None
    got = out.cpu().numpy().reshape(48, 64, 3)
    d = np.abs(got.astype(int) - to_u8(img).astype(int))
    assert d.max() <= 1 and (d == 0).mean() >= 0.9999
