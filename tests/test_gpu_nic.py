"""Neural irradiance cache kernels (tcgen05 forward and backward) against a
plain PyTorch fp32 reference of the same model.

The reference rounds to BF16 exactly where the kernels do (input features,
weights, hidden activations) and computes everything else in FP32; the
gradient reference is fp32 autograd without BF16 rounding of the backward
signals.  Tolerances (written here, applied below):
  forward    relative L2 error of the predictions <= 1e-2
  gradient   relative L2 error of the parameter gradient <= 5e-2,
             loss within 1e-3 relative
"""
import json

import numpy as np
import pytest
import torch

from povray_gb300 import abi
from povray_gb300.render import nic_eval

pytestmark = pytest.mark.gpu

K1, HID, NO, FEAT = 112, 64, 16, 102
SIZES = [("W1", HID * K1), ("b1", HID), ("W2", HID * HID), ("b2", HID), ("W3", HID * HID), ("b3", HID),
         ("W4", HID * HID), ("b4", HID), ("W5", NO * HID), ("b5", NO)]


def _unpack(p):
    out, o = {}, 0
    for name, n in SIZES:
        out[name] = p[o:o + n]
        o += n
    assert o == abi.POV_GPU_NIC_PARAMS
    out["W1"] = out["W1"].reshape(HID, K1)
    for k in ("W2", "W3", "W4"):
        out[k] = out[k].reshape(HID, HID)
    out["W5"] = out["W5"].reshape(NO, HID)
    return out


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(abi.POV_GPU_NIC_PARAMS, dtype=np.float32)
    o = 0
    for name, n in SIZES:
        if name.startswith("W"):
            cols = K1 if name == "W1" else HID
            v = rng.uniform(-1, 1, n).astype(np.float32) * np.sqrt(6.0 / cols)
            if name == "W1":
                v = v.reshape(HID, K1)
                v[:, FEAT:] = 0
                v = v.ravel()
            if name == "W5":
                v = v.reshape(NO, HID)
                v[3:] = 0
                v = v.ravel()
        else:
            v = rng.uniform(-0.1, 0.1, n).astype(np.float32)
            if name == "b5":
                v[3:] = 0
        p[o:o + n] = v
        o += n
    return p


def _features(points, normals, bounds):
    lo = bounds[:3]
    scale = 2.0 / np.maximum(bounds[3:] - bounds[:3], 1e-6)
    c6 = np.concatenate([np.clip((points - lo) * scale - 1.0, -1, 1), normals], axis=1)
    c6 = torch.tensor(c6, dtype=torch.float32)
    feats = [c6]
    for c in range(6):
        for k in range(8):
            a = np.pi * (2 ** k) / 8 * c6[:, c]
            feats.append(torch.stack([torch.sin(a), torch.cos(a)], dim=1))
    f = torch.cat(feats, dim=1)
    return torch.cat([f, torch.zeros(f.shape[0], K1 - FEAT)], dim=1)


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float32)


def _reference(params, points, normals, bounds, bf16_backward=False):
    P = {k: torch.tensor(v, dtype=torch.float32) for k, v in _unpack(params).items()}
    for k in ("W1", "W2", "W3", "W4", "W5"):
        P[k] = _bf(P[k]).requires_grad_(True)
    for k in ("b1", "b2", "b3", "b4", "b5"):
        P[k] = P[k].requires_grad_(True)
    h = _bf(_features(points, normals, bounds))
    for i in range(1, 5):
        z = h @ P["W%d" % i].T + P["b%d" % i]
        a = torch.relu(z)
        # forward values rounded like the kernel's BF16 activations; the
        # gradient flows through unrounded (straight-through)
        h = a + (_bf(a) - a).detach()
    y = h @ P["W5"].T + P["b5"]
    return y, P


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(5)
    n = 1000   # not a multiple of the 128-sample tile: a ragged last tile
    pts = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    bounds = np.array([-10, -10, -10, 10, 10, 10], dtype=np.float32)
    tgt = np.abs(np.sin(pts * 0.3) * 0.5 + 0.3).astype(np.float32)
    return pts, nrm, bounds, tgt


def test_forward_matches_torch(data):
    pts, nrm, bounds, _ = data
    params = _params(1)
    got, _, _ = nic_eval(params, bounds, pts, nrm)
    ref, _ = _reference(params, pts, nrm, bounds)
    ref = ref[:, :3].detach().numpy()
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel <= 1e-2, rel


def test_gradient_matches_torch_autograd(data):
    pts, nrm, bounds, tgt = data
    params = _params(2)
    _, grad, loss = nic_eval(params, bounds, pts, nrm, tgt)
    y, P = _reference(params, pts, nrm, bounds)
    p = y[:, :3]
    t = torch.tensor(tgt)
    L = ((p - t) ** 2 / (p.detach() ** 2 + 0.01)).sum() / len(pts)
    L.backward()
    ref = torch.cat([P[name].grad.reshape(-1) for name, _ in SIZES]).numpy()
    # the padded rows carry no gradient that matters
    w5 = slice(sum(n for _, n in SIZES[:8]), sum(n for _, n in SIZES[:9]))
    mask = np.ones_like(ref, dtype=bool)
    w5m = mask[w5].reshape(NO, HID)
    w5m[3:] = False
    mask[-NO + 3:] = False
    rel = np.linalg.norm(grad[mask] - ref[mask]) / np.linalg.norm(ref[mask])
    info = json.dumps(dict(rel=float(rel), loss=loss, ref_loss=float(L.detach())))
    assert abs(loss / float(L.detach()) - 1) < 1e-3, info
    assert rel <= 5e-2, info


def test_gradient_is_reproducible(data):
    """Each CTA keeps its own gradient slice and the slices are summed in a
    fixed order: the same samples give bit-identical gradients and loss."""
    pts, nrm, bounds, tgt = data
    params = _params(3)
    _, g1, l1 = nic_eval(params, bounds, pts, nrm, tgt)
    _, g2, l2 = nic_eval(params, bounds, pts, nrm, tgt)
    assert np.array_equal(g1, g2)
    assert l1 == l2
