"""Host-side logic that needs no GPU: the block dispenser, the block-batching
task driver (with a stand-in for the device scene), scene generators and the
8-bit encoder."""
import numpy as np

from povray_gb300 import scenes
from povray_gb300.encode import int_encode_srgb, to_u8
from povray_gb300.render import BlockSource, GpuTraceTask


class FakeGpu:
    """Returns each pixel's (x, y) so block bookkeeping can be checked."""

    def __init__(self, scene):
        self.scene = scene
        self.calls = 0

    def trace_blocks(self, blocks, params):
        self.calls += 1
        out = []
        for (l, t, r, b, _s) in blocks:
            yy, xx = np.mgrid[t:b + 1, l:r + 1]
            px = np.stack([xx, yy, np.zeros_like(xx), np.ones_like(xx)], axis=-1).reshape(-1, 4)
            out.append(px.astype(np.float32))
        return np.concatenate(out), {"number_of_pixels": sum(len(o) for o in out)}


def test_block_grid_covers_image_once():
    for w, h in [(320, 240), (100, 37), (1, 1), (33, 65)]:
        cover = np.zeros((h, w), dtype=np.int32)
        for (l, t, r, b, _s) in scenes.blocks_for(w, h):
            cover[t:b + 1, l:r + 1] += 1
        assert (cover == 1).all()


def test_trace_task_assembles_image_in_batches():
    s = scenes.spheres_plane(100, 70, n_spheres=2)
    src = BlockSource(100, 70)
    fake = FakeGpu(s)
    st = GpuTraceTask(fake, src, params=s.render_params(), batch=3).run()
    yy, xx = np.mgrid[0:70, 0:100]
    assert np.array_equal(src.image[..., 0], xx) and np.array_equal(src.image[..., 1], yy)
    assert fake.calls == -(-len(src.blocks) // 3)
    assert st["number_of_pixels"] == 100 * 70


def test_skip_list_is_honoured():
    src = BlockSource(96, 64, skip=[0, 4])
    s = scenes.spheres_plane(96, 64, n_spheres=2)
    GpuTraceTask(FakeGpu(s), src, params=s.render_params()).run()
    assert sorted(src.completed) == [1, 2, 3, 5]
    assert (src.image[0:32, 0:32] == 0).all()


def test_unblock_inverts_block_order():
    blocks = scenes.blocks_for(70, 40)
    img = np.random.default_rng(0).random((40, 70, 4)).astype(np.float32)
    flat = np.concatenate([img[t:b + 1, l:r + 1].reshape(-1, 4) for (l, t, r, b, _s) in blocks])
    assert np.array_equal(scenes.unblock(flat, blocks, 70, 40), img)


def test_generators_are_deterministic():
    a = scenes.mesh_spheres(64, 36, mesh_n=8, n_spheres=16)
    b = scenes.mesh_spheres(64, 36, mesh_n=8, n_spheres=16)
    assert a.sdl() == b.sdl()
    assert np.array_equal(a.meshes[0].vertices, b.meshes[0].vertices)


def test_full_mesh_has_a_million_triangles():
    m = scenes.displaced_sphere_mesh(n=296)
    assert m.num_triangles == 1051392
    assert np.isfinite(m.vertices).all()
    r = np.linalg.norm(m.vertices, axis=1)
    assert r.min() > 8 * 0.8 and r.max() < 8 * 1.2
    assert np.allclose(np.linalg.norm(m.normals, axis=1), 1.0, atol=1e-5)


def test_int_encode_endpoints_and_monotone():
    x = np.linspace(-0.1, 1.2, 5001, dtype=np.float32)
    v = int_encode_srgb(x)
    assert v[0] == 0 and v[-1] == 255
    assert (np.diff(v.astype(int)) >= 0).all()
    assert to_u8(np.ones((2, 2, 4), np.float32)).shape == (2, 2, 3)
