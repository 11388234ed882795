"""Writes tests/golden/blue_noise_64x64.npy: the reference's 64x64 blue-noise
jitter tile (data/BlueNoise/64_64/HDR_L_0.png, CC0, 16-bit greyscale), as the
uint16 texels the reference uploads into its GL_R16 texture
(src/Base/src/Textures.cpp:21-25): row y of the file is texel row y, read by
texelFetch(blue_noise, pos & 63) (VolumetricCloudRender.comp:168) as
value / 65535.

Run here, where the reference is mounted:
    python tests/golden/make_blue_noise.py [path/to/reference]
The PNG is decoded with zlib and the five PNG row filters (no image library).
"""
from __future__ import annotations

import struct
import sys
import zlib
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "blue_noise_64x64.npy"


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def decode_gray16(data: bytes) -> np.ndarray:
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG file"
    i, idat, hdr = 8, b"", None
    while i < len(data):
        n = struct.unpack(">I", data[i:i + 4])[0]
        kind, body = data[i + 4:i + 8], data[i + 8:i + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        i += 12 + n
    w, h, depth, color, _, _, interlace = hdr
    assert depth == 16 and color == 0 and interlace == 0, "expects 16-bit greyscale, not interlaced"
    raw = zlib.decompress(idat)
    bpp, stride = 2, 2 * w
    rows, prev = [], bytearray(stride)
    for y in range(h):
        f, line = raw[y * (stride + 1)], bytearray(raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)])
        for x in range(stride):
            a = line[x - bpp] if x >= bpp else 0
            b, c = prev[x], prev[x - bpp] if x >= bpp else 0
            line[x] = (line[x] + (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]) & 0xFF
        rows.append(bytes(line))
        prev = line
    return np.frombuffer(b"".join(rows), dtype=">u2").reshape(h, w).astype(np.uint16)


def main(reference: str = "/root/reference") -> None:
    png = Path(reference) / "data" / "BlueNoise" / "64_64" / "HDR_L_0.png"
    tile = decode_gray16(png.read_bytes())
    assert tile.shape == (64, 64)
    np.save(OUT, tile)
    print(f"{OUT}: {tile.shape} uint16, min {tile.min()} max {tile.max()} mean {tile.mean():.1f}")


if __name__ == "__main__":
    main(*sys.argv[1:])
