"""Writes tests/golden/color_ramps_ref.npz from the reference's own output image
(run: python tests/golden/make_ramp_golden.py PATH/TO/doc/customColorMaps.png,
the image as it lies in a checkout of the reference; or set
SPHUGO_COLOR_RAMP_PNG to that path).

doc/customColorMaps.png in the reference is the output of its example
examples/color-ramp/color-ramp.go: four 20-pixel-wide strips (RainbowRamp,
ParaRamp, HeatRamp, ToxicRamp from gx/graphics.go), row 255 - i painted with
colour index i. The middle column of each strip gives the 256 colours of each
ramp as the reference computed them; the frame rasteriser's ParaRamp is pinned
against them.
"""
import os
import struct
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

def source_png():
    import sys
    if len(sys.argv) > 1:
        return sys.argv[1]
    path = os.environ.get("SPHUGO_COLOR_RAMP_PNG")
    if not path:
        raise SystemExit("usage: make_ramp_golden.py PATH/TO/doc/customColorMaps.png "
                         "(or set SPHUGO_COLOR_RAMP_PNG)")
    return path


def decode_png_rgb(path):
    """8-bit RGB, non-interlaced PNG (what Go's image/png writes for an opaque image)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        ln = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if tag == b"IHDR":
            w, h, bd, ct, _, _, il = struct.unpack(">IIBBBBB", body)
            assert (bd, ct, il) == (8, 2, 0)
        elif tag == b"IDAT":
            idat += body
    raw = zlib.decompress(idat)
    bpp, stride = 3, w * 3
    img = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    o = 0
    for y in range(h):
        f = raw[o]
        line = np.frombuffer(raw[o + 1:o + 1 + stride], np.uint8).astype(np.int32)
        o += 1 + stride
        out = np.zeros(stride, np.int32)
        for x in range(stride):
            a = out[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) // 2
            else:  # Paeth
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out[x] = (line[x] + p) & 255
        img[y] = out
        prev = out
    return img.reshape(h, w, 3)


def main():
    img = decode_png_rgb(source_png())
    assert img.shape == (256, 80, 3)
    names = ["rainbow", "para", "heat", "toxic"]
    ramps = {nm: img[255 - np.arange(256), 20 * j + 10].copy() for j, nm in enumerate(names)}
    np.savez_compressed(os.path.join(HERE, "color_ramps_ref.npz"), **ramps)
    print("wrote", os.path.join(HERE, "color_ramps_ref.npz"))


if __name__ == "__main__":
    main()
