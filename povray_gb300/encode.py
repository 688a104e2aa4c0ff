"""8-bit output encoding of linear RGBT pixels, as the reference's image
writer does it: clip to [0,1], sRGB gamma curve, then the rounding of
IntEncode(gamma, x, 255) without dithering (source/base/image/encoding.cpp:67-91,
sRGB curve source/base/image/colourspace.cpp:181-191).  The same function
quantises both sides of the 1-LSB parity check."""
import numpy as np


def srgb_encode(x):
    x = np.asarray(x, dtype=np.float32)
    return np.where(x <= np.float32(0.0031308), x * np.float32(12.92),
                    np.float32(1.055) * np.power(np.maximum(x, 0), np.float32(1.0 / 2.4)) - np.float32(0.055)
                    ).astype(np.float32)


def srgb_decode(x):
    x = np.asarray(x, dtype=np.float32)
    return np.where(x < np.float32(0.04045), x / np.float32(12.92),
                    np.power((x + np.float32(0.055)) / np.float32(1.055), np.float32(2.4))).astype(np.float32)


def int_encode_srgb(x, maxv=255):
    """IntEncode(g=sRGB, x, max) with qOff = 0 and no error diffusion."""
    xe = np.clip(np.asarray(x, dtype=np.float32), 0.0, 1.0)
    v = np.clip(np.floor(srgb_encode(xe) * np.float32(maxv)), 0, maxv).astype(np.int32)
    dec = srgb_decode(v.astype(np.float32) / np.float32(maxv))
    up = srgb_decode(np.minimum(v + 1, maxv).astype(np.float32) / np.float32(maxv))
    thr = np.float32(0.5) * dec + np.float32(0.5) * up
    bump = (v < maxv) & (xe > thr)
    return (v + bump).astype(np.uint8)


def to_u8(rgbt):
    """(H, W, 4) linear RGBT -> (H, W, 3) uint8."""
    return int_encode_srgb(np.asarray(rgbt)[..., :3])


def write_ppm(path, rgbt):
    img = to_u8(rgbt)
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(img.tobytes())
