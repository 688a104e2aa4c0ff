"""8-bit output encoding of linear RGBT pixels, as the reference's image
writers do it: clip to [0,1], apply the file's transfer curve, then the
rounding of IntEncode(gamma, x, 255) without dithering
(source/base/image/encoding.cpp:67-91).  Curves (source/base/image/
colourspace.cpp): sRGB (:181-191, the default of most formats) and ITU-R
BT.709 (:211-222, the default of the PPM writer, source/base/image/ppm.cpp:132).
The same function quantises both sides of the 1-LSB parity checks."""
import numpy as np

F = np.float32


def srgb_encode(x):
    x = np.asarray(x, dtype=F)
    return np.where(x <= F(0.0031308), x * F(12.92),
                    F(1.055) * np.power(np.maximum(x, 0), F(1.0 / 2.4)) - F(0.055)).astype(F)


def srgb_decode(x):
    x = np.asarray(x, dtype=F)
    return np.where(x < F(0.04045), x / F(12.92),
                    np.power((x + F(0.055)) / F(1.055), F(2.4))).astype(F)


def bt709_encode(x):
    x = np.asarray(x, dtype=F)
    return np.where(x < F(0.018), x * F(4.5), F(1.099) * np.power(np.maximum(x, 0), F(0.45)) - F(0.099)).astype(F)


def bt709_decode(x):
    x = np.asarray(x, dtype=F)
    return np.where(x < F(0.081), x / F(4.5), np.power((x + F(0.099)) / F(1.099), F(1.0 / 0.45))).astype(F)


CURVES = {"srgb": (srgb_encode, srgb_decode), "bt709": (bt709_encode, bt709_decode)}


def int_encode(x, curve="srgb", maxv=255):
    """IntEncode(g, x, max) with qOff = 0 and no error diffusion."""
    enc, dec = CURVES[curve]
    xe = np.clip(np.asarray(x, dtype=F), 0.0, 1.0)
    v = np.clip(np.floor(enc(xe) * F(maxv)), 0, maxv).astype(np.int32)
    lo = dec(v.astype(F) / F(maxv))
    up = dec(np.minimum(v + 1, maxv).astype(F) / F(maxv))
    thr = F(0.5) * lo + F(0.5) * up
    bump = (v < maxv) & (xe > thr)
    return (v + bump).astype(np.uint8)


def int_encode_srgb(x, maxv=255):
    return int_encode(x, "srgb", maxv)


def to_u8(rgbt, curve="srgb"):
    """(H, W, 4) linear RGBT -> (H, W, 3) uint8."""
    return int_encode(np.asarray(rgbt)[..., :3], curve)


def write_ppm(path, rgbt, curve="bt709"):
    img = to_u8(rgbt, curve)
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(img.tobytes())


def read_ppm(path):
    """8-bit binary PPM (P6) as written by the reference CLI (comments allowed)."""
    data = open(path, "rb").read()
    toks, i = [], 0
    while len(toks) < 4:
        while data[i:i + 1].isspace():
            i += 1
        if data[i:i + 1] == b"#":
            while data[i:i + 1] != b"\n":
                i += 1
            continue
        j = i
        while not data[j:j + 1].isspace():
            j += 1
        toks.append(data[i:j])
        i = j
    i += 1
    w, h = int(toks[1]), int(toks[2])
    return np.frombuffer(data[i:i + w * h * 3], dtype=np.uint8).reshape(h, w, 3).copy()
