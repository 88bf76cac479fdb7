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


_F = np.float32


def tonemap_uncharted2(c):
    """postprocess.glsl:5-22 (Hable's filmic curve, exposure bias 2, white
    11.2), in FP32 with the shader's operation order: constant products are
    single-precision products (C*B, D*E, D*F, E/F), then
    ((x*(A*x+CB)+DE)/(x*(A*x+B)+DF))-EF of 2*c, times 1/curve(11.2)."""
    A, B, C, D, E, F = _F(0.15), _F(0.50), _F(0.10), _F(0.20), _F(0.02), _F(0.30)
    CB, DE, DF, EF = C * B, D * E, D * F, E / F

    def curve(x):
        return ((x * (A * x + CB) + DE) / (x * (A * x + B) + DF)) - EF

    x = np.asarray(c, _F)
    white = _F(1.0) / curve(_F(11.2))
    return curve(_F(2.0) * x) * white


def tonemap_aces(c):
    """postprocess.glsl:24-31 (Narkowicz's ACES fit) in FP32:
    clamp((x*(a*x+b))/(x*(c*x+d)+e), 0, 1)."""
    a, b, cc, d, e = _F(2.51), _F(0.03), _F(2.43), _F(0.59), _F(0.14)
    x = np.asarray(c, _F)
    return np.minimum(np.maximum((x * (a * x + b)) / (x * (cc * x + d) + e), _F(0.0)), _F(1.0))


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


def read_png(path):
    """Non-interlaced 8- or 16-bit PNG (grey, grey+alpha, RGB, RGBA) ->
    (h, w, 4) uint8 RGBA, rows in file order; e.g. the blue-noise texture
    the AO example loads (examples/4-ray-ao.rs:198-201; src/texture.rs:489-492
    converts it with to_rgba8). 16-bit samples v become round(v * 255 /
    65535) = (v + 128) // 257."""
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos + 8 <= len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + n
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    chans = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if depth not in (8, 16) or chans is None or interlace != 0:
        raise ValueError("unsupported PNG (need 8/16-bit non-interlaced grey/RGB/RGBA)")
    bpp = chans * depth // 8                     # bytes per pixel (filter unit)
    stride = w * bpp
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(h, 1 + stride)
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.uint8)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:]
        if f == 0:
            cur = line.copy()
        elif f == 2:
            cur = (line.astype(np.uint16) + prev).astype(np.uint8)
        else:
            cur = np.zeros_like(line)
            for x in range(stride):        # sub / average / paeth depend on the left neighbour
                a = int(cur[x - bpp]) if x >= bpp else 0
                c = int(prev[x - bpp]) if x >= bpp else 0
                b = int(prev[x])
                if f == 1:
                    pred = a
                elif f == 3:
                    pred = (a + b) // 2
                elif f == 4:
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                else:
                    raise ValueError("bad PNG filter %d" % f)
                cur[x] = (int(line[x]) + pred) & 0xFF
        out[y] = cur
        prev = cur
    if depth == 16:
        v = out.reshape(h, w * chans, 2).astype(np.uint32)
        px = (((v[..., 0] << 8) | v[..., 1]) + 128) // 257
        px = px.astype(np.uint8).reshape(h, w, chans)
    else:
        px = out.reshape(h, w, chans)
    rgba = np.zeros((h, w, 4), np.uint8)
    if chans in (1, 2):
        rgba[..., :3] = px[..., :1]
        rgba[..., 3] = px[..., 1] if chans == 2 else 255
    else:
        rgba[..., :3] = px[..., :3]
        rgba[..., 3] = px[..., 3] if chans == 4 else 255
    return rgba
