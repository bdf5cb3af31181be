"""Collect the reference's Huffman JPEG fixtures as decoder test inputs (tests/golden/jpeg_fixtures.npz).

Reads rust-compress's fixtures/ directory (the path is the first argument), keeps the files the oracle's Huffman
decoder accepts (the reference's own test images written by libjpeg/libjpeg-turbo: baseline, optimized tables,
gray, 4:4:4 and 4:2:0, ICC-tagged, progressive with successive approximation (rgb8_prog.jpg), and the sequential
Huffman twins of the arithmetic-coding fixtures), and stores each file's bytes with the SHA-256 of the
coefficients the oracle decodes from it.

    python tests/golden/make_jpeg_fixtures.py /path/to/rust-compress/fixtures
"""

import glob
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import oracle  # noqa: E402


def main(src):
    names, blobs, shas = [], [], []
    for path in sorted(glob.glob(os.path.join(src, "*.jpg"))):
        data = open(path, "rb").read()
        try:
            g, _ = oracle.decode_sequential(data)
        except ValueError:
            continue
        names.append(os.path.basename(path))
        blobs.append(np.frombuffer(data, np.uint8))
        shas.append(hashlib.sha256(g.coefs.tobytes()).hexdigest())
    offsets = np.cumsum([0] + [b.size for b in blobs])
    np.savez_compressed(os.path.join(HERE, "jpeg_fixtures.npz"), names=np.array(names), shas=np.array(shas),
                        offsets=offsets, data=np.concatenate(blobs))
    print(f"{len(names)} fixtures, {offsets[-1]} bytes")


if __name__ == "__main__":
    main(sys.argv[1])
