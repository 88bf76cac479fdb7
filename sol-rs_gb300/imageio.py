"""Image output replacing the swapchain blit of examples/5-pathtrace.rs:360-366.

write_png / write_ppm store the RGBA8 render image (row 0 = gl_LaunchIDEXT.y
= 0 at the top, as presented by the reference). Tonemaps of
assets/glsl/postprocess.glsl:5-36 are offered for HDR accumulation buffers.
"""
import struct
import zlib

import numpy as np


def write_png(path, rgba8):
    a = np.ascontiguousarray(rgba8, dtype=np.uint8)
    h, w, c = a.shape
    if c not in (3, 4):
        raise ValueError("expected RGB or RGBA")
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n"
    png += chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6 if c == 4 else 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6))
    png += chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def write_ppm(path, rgba8):
    a = np.ascontiguousarray(rgba8, dtype=np.uint8)[..., :3]
    h, w, _ = a.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(a.tobytes())


def gamma_correct(c, power=2.2):
    """postprocess.glsl:38-41"""
    return np.power(np.maximum(c, 0.0), np.float32(1.0) / np.float32(power))


def tonemap_uncharted2(c):
    """postprocess.glsl:5-22 (Hable's filmic curve, exposure bias 2, white 11.2)."""
    A, B, C, D, E, F = 0.15, 0.50, 0.10, 0.20, 0.02, 0.30

    def curve(x):
        return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F

    return curve(2.0 * c) * (1.0 / curve(np.float32(11.2)))


def tonemap_aces(c):
    """postprocess.glsl:24-31 (Narkowicz's ACES fit)."""
    a, b, cc, d, e = 2.51, 0.03, 2.43, 0.59, 0.14
    return np.clip((c * (a * c + b)) / (c * (cc * c + d) + e), 0.0, 1.0)


def to_rgba8(rgb, tonemap=None):
    x = np.asarray(rgb, np.float32)[..., :3]
    if tonemap == "aces":
        x = tonemap_aces(x)
    elif tonemap == "uncharted2":
        x = tonemap_uncharted2(x)
    x = gamma_correct(x)
    out = np.empty(x.shape[:-1] + (4,), np.uint8)
    out[..., :3] = (np.clip(x, 0, 1) * 255.0 + 0.5).astype(np.uint8)
    out[..., 3] = 255
    return out
