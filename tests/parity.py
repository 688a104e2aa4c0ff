"""Comparison helpers of the parity tests.

Hit parity: object ids (and mesh triangle ids) must agree bit-exactly on
non-grazing rays; depths within 1e-5 relative.  A ray counts as grazing when
the FP64 oracle's own answer is unstable under a 1e-5 rad perturbation of its
direction (silhouettes, shared edges) or when two surfaces lie within 1e-5
relative depth of each other (ties).

Pixel parity: at least 99.9% of 8-bit sRGB channels within 1 LSB.
"""
import numpy as np

from povray_gb300.encode import to_u8

T_REL_TOL = 1e-5
PERTURB = 1e-5


def _perturbed(d, k):
    # two directions orthogonal to d
    a = np.where(np.abs(d[:, :1]) < 0.9, np.array([[1.0, 0.0, 0.0]]), np.array([[0.0, 1.0, 0.0]]))
    u = np.cross(d, a)
    u /= np.linalg.norm(u, axis=1)[:, None]
    v = np.cross(d, u)
    s = [(1, 0), (-1, 0), (0, 1), (0, -1)][k]
    p = d + PERTURB * (s[0] * u + s[1] * v)
    return p / np.linalg.norm(p, axis=1)[:, None]


def grazing_mask(oracle, org, dirs, ref_obj, ref_tri, ref_t, idx):
    """For rays `idx`, True where the oracle's answer changes under small
    perturbations of the direction (silhouette/edge) -- such rays are
    excluded from the bit-exact check."""
    if len(idx) == 0:
        return np.zeros(0, dtype=bool)
    o, d = org[idx], dirs[idx]
    g = np.zeros(len(idx), dtype=bool)
    for k in range(4):
        h = oracle.trace_rays(o, _perturbed(d, k))
        g |= (h["object"] != ref_obj[idx]) | (h["triangle"] != ref_tri[idx])
    return g


def compare_hits(got_obj, got_tri, got_t, ref_obj, ref_tri, ref_t, oracle=None, org=None, dirs=None,
                 t_tol=T_REL_TOL):
    """Returns a dict of counts; 'bad' must be 0 for parity."""
    got_obj, ref_obj = np.asarray(got_obj), np.asarray(ref_obj)
    mism = (got_obj != ref_obj) | (np.asarray(got_tri) != np.asarray(ref_tri))
    idx = np.nonzero(mism)[0]
    graz = np.zeros(len(idx), dtype=bool)
    if oracle is not None and len(idx):
        graz = grazing_mask(oracle, org, dirs, ref_obj, np.asarray(ref_tri), np.asarray(ref_t), idx)
        # depth ties: both surfaces within t_tol relative of each other
        both = (got_obj[idx] >= 0) & (ref_obj[idx] >= 0)
        tie = both & (np.abs(np.asarray(got_t)[idx] - np.asarray(ref_t)[idx]) <=
                      10 * t_tol * np.abs(np.asarray(ref_t)[idx]))
        graz |= tie
    same = ~mism & (ref_obj >= 0)
    rel = np.abs(np.asarray(got_t)[same] - np.asarray(ref_t)[same]) / np.maximum(np.abs(np.asarray(ref_t)[same]), 1e-12)
    worst = []
    if rel.size:
        sidx = np.nonzero(same)[0]
        for k in np.argsort(-rel)[:8]:
            if rel[k] > t_tol:
                j = int(sidx[k])
                worst.append((j, int(ref_obj[j]), float(np.asarray(ref_t)[j]), float(np.asarray(got_t)[j])))
    return {
        "rays": int(len(ref_obj)),
        "mismatch": int(len(idx)),
        "grazing": int(graz.sum()),
        "bad": int((~graz).sum()),
        "t_max_rel": float(rel.max()) if rel.size else 0.0,
        "t_bad": int((rel > t_tol).sum()),
        "worst_t": worst,   # (ray, object, reference t, got t)
    }


def compare_pixels(got, ref):
    """Fraction of 8-bit channels within 1 LSB, and the max LSB difference."""
    a = to_u8(got).astype(np.int32)
    b = to_u8(ref).astype(np.int32)
    diff = np.abs(a - b)
    return {"within_1lsb": float((diff <= 1).mean()), "max_lsb": int(diff.max()),
            "max_abs_linear": float(np.abs(np.asarray(got)[..., :3] - np.asarray(ref)[..., :3]).max())}
