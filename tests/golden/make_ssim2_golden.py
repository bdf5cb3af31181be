"""Regenerate tests/golden/ssim2_pairs.npz from the reference's SSIMULACRA2 verification pairs.

Source: fixtures/ssim2/*.png and fixtures/ssim2/expected.csv of rust-compress (54 pairs, 8-bit RGB PNGs,
scores from the py-ssimulacra2 port; the reference checks itself against them at 1e-4 in
cli/tests/ssimulacra2.rs:8-29). The PNGs are decoded here with a minimal PNG reader (zlib + the five
scanline filters, 8-bit RGB/RGBA/Gray, non-interlaced: all the fixtures are 8-bit RGB) and stored as raw
uint8 arrays so the tests need neither the reference tree nor an image library.

Usage: python tests/golden/make_ssim2_golden.py <path to the reference's fixtures/ssim2>
"""

import csv
import os
import struct
import sys
import zlib

import numpy as np


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", path
    pos = 8
    idat = b""
    width = height = depth = ctype = interlace = None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos : pos + 4])
        kind = data[pos + 4 : pos + 8]
        body = data[pos + 8 : pos + 8 + length]
        pos += 12 + length
        if kind == b"IHDR":
            width, height, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
    assert depth == 8 and interlace == 0 and ctype in (0, 2, 6), (path, depth, ctype, interlace)
    bpp = {0: 1, 2: 3, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = width * bpp
    out = np.zeros((height, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    p = 0
    for y in range(height):
        ftype = raw[p]
        line = np.frombuffer(raw[p + 1 : p + 1 + stride], dtype=np.uint8).astype(np.int32)
        p += 1 + stride
        cur = np.zeros(stride, dtype=np.int32)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if ftype == 0:
                v = line[x]
            elif ftype == 1:
                v = line[x] + a
            elif ftype == 2:
                v = line[x] + b
            elif ftype == 3:
                v = line[x] + ((a + b) >> 1)
            elif ftype == 4:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                v = line[x] + pred
            else:
                raise ValueError(f"bad filter {ftype} in {path}")
            cur[x] = v & 0xFF
        out[y] = cur
        prev = cur
    img = out.reshape(height, width, bpp)
    if bpp == 1:
        img = np.repeat(img, 3, axis=2)
    elif bpp == 4:
        img = img[:, :, :3]
    return img


def main():
    src = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    rows = list(csv.reader(open(os.path.join(src, "expected.csv"))))
    arrays = {}
    names, refs, dists, scores = [], [], [], []
    for r in rows:
        if not r:
            continue
        name, ref, dist, score = r
        for f in (ref, dist):
            if f not in arrays:
                arrays[f] = read_png(os.path.join(src, f))
        names.append(name)
        refs.append(ref)
        dists.append(dist)
        scores.append(score)
    payload = {f"img:{k}": v for k, v in arrays.items()}
    payload["names"] = np.array(names)
    payload["refs"] = np.array(refs)
    payload["dists"] = np.array(dists)
    # Scores kept as the exact decimal strings of expected.csv (17 significant digits).
    payload["scores"] = np.array(scores)
    np.savez_compressed(os.path.join(here, "ssim2_pairs.npz"), **payload)
    print(f"{len(names)} pairs, {len(arrays)} images")


if __name__ == "__main__":
    main()
