"""Seeded synthetic RGB8 test images for the quality search (no dataset: the inputs are generated).

Content, as the workload definition asks: the sum of 3 random linear colour gradients, 2-octave value noise of
amplitude 24, and 6 random axis-aligned flat-colour rectangles with hard edges, clamped to u8; optionally plus
Gaussian sensor noise.

Randomness is SplitMix64 (Steele, Lea, Flood 2014) used as a counter-based generator: draw i of stream `s` under
`seed` is mix64(seed*2^32 + s*2^24 ... ) -- precisely mix64(base + (i + 1) * 0x9E3779B97F4A7C15) with
base = (seed * 0x100000001B3 + stream * 0xC2B2AE3D27D4EB4F) mod 2^64 -- and a uniform in [0, 1) is
(draw >> 11) * 2^-53. Streams: 0 gradients, 1 rectangles, 2 + octave*3 + channel noise lattices, 16 sensor noise.
Everything is vectorised numpy (a 4000x3000 image takes a few seconds); many images are generated in parallel by
`images()` with a spawn process pool.
"""

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def _mix64(z):
    z = z.copy()
    z ^= z >> np.uint64(30)
    z *= M1
    z ^= z >> np.uint64(27)
    z *= M2
    z ^= z >> np.uint64(31)
    return z


def uniforms(seed, stream, n):
    """n uniforms in [0, 1) from stream `stream` of `seed` (float64)."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed * 0x100000001B3 + stream * 0xC2B2AE3D27D4EB4F) % (1 << 64))
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = _mix64(base + i * GAMMA)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def _smooth(t):
    return t * t * (3.0 - 2.0 * t)


def _value_noise(seed, stream, w, h, cell):
    """Value noise in [-1, 1]: a lattice of uniforms every `cell` pixels, smoothstep-bilinear in between."""
    gw, gh = w // cell + 2, h // cell + 2
    lat = (uniforms(seed, stream, gw * gh).reshape(gh, gw) * 2.0 - 1.0).astype(np.float32)
    xs = (np.arange(w, dtype=np.float32) + 0.5) / cell
    ys = (np.arange(h, dtype=np.float32) + 0.5) / cell
    xi = np.floor(xs).astype(np.int64)
    yi = np.floor(ys).astype(np.int64)
    tx = _smooth(xs - xi).astype(np.float32)
    ty = _smooth(ys - yi).astype(np.float32)
    a = lat[yi][:, xi]
    b = lat[yi][:, xi + 1]
    c = lat[yi + 1][:, xi]
    d = lat[yi + 1][:, xi + 1]
    top = a + (b - a) * tx[None, :]
    bot = c + (d - c) * tx[None, :]
    return top + (bot - top) * ty[:, None]


def image(w, h, seed, sensor_sigma=0.0):
    """A (h, w, 3) uint8 image as described in the module docstring."""
    g = uniforms(seed, 0, 3 * 7)
    xs = (np.arange(w, dtype=np.float32) + 0.5) / w - 0.5
    ys = (np.arange(h, dtype=np.float32) + 0.5) / h - 0.5
    # 3 linear colour gradients: channel ch = sum_k (c0[k,ch] + (c1-c0)[k,ch] * t_k) / 3, t_k a clamped ramp
    ts = []
    for k in range(3):
        th = g[k * 7 + 6] * 2.0 * np.pi
        t = xs[None, :] * np.float32(np.cos(th)) + ys[:, None] * np.float32(np.sin(th))
        t += np.float32(0.5)
        np.clip(t, 0.0, 1.0, out=t)
        ts.append(t)
    img = np.empty((h, w, 3), dtype=np.float32)
    for ch in range(3):
        acc = np.full((h, w), np.float32(sum(g[k * 7 + ch] * 255.0 for k in range(3)) / 3.0), dtype=np.float32)
        for k in range(3):
            c0, c1 = g[k * 7 + ch] * 255.0, g[k * 7 + 3 + ch] * 255.0
            acc += np.float32((c1 - c0) / 3.0) * ts[k]
        # 2-octave value noise, amplitude 24 (16 + 8), independent per channel
        cell0 = max(8, min(w, h) // 16)
        for octave, amp in ((0, 16.0), (1, 8.0)):
            cell = max(4, cell0 >> octave)
            acc += np.float32(amp) * _value_noise(seed, 2 + octave * 3 + ch, w, h, cell)
        img[:, :, ch] = acc
    del ts
    # 6 flat rectangles with hard edges, drawn over the rest
    r = uniforms(seed, 1, 6 * 7)
    for k in range(6):
        x0 = int(r[k * 7] * w)
        y0 = int(r[k * 7 + 1] * h)
        rw = max(1, int((0.05 + 0.25 * r[k * 7 + 2]) * w))
        rh = max(1, int((0.05 + 0.25 * r[k * 7 + 3]) * h))
        col = r[k * 7 + 4: k * 7 + 7] * 255.0
        img[y0: y0 + rh, x0: x0 + rw, :] = col.astype(np.float32)[None, None, :]
    if sensor_sigma > 0:
        # Gaussian sensor noise by Box-Muller, both outputs of each pair used: n/2 pairs of uniforms
        n = h * w * 3
        m = (n + 1) // 2
        u1 = uniforms(seed, 16, m)
        u2 = uniforms(seed, 17, m)
        rad = np.sqrt(-2.0 * np.log1p(-u1)).astype(np.float32)  # 1-u1 is in (0, 1]
        ang = (2.0 * np.pi * u2).astype(np.float32)
        z = np.empty(2 * m, dtype=np.float32)
        z[0::2] = rad * np.cos(ang)
        z[1::2] = rad * np.sin(ang)
        img += np.float32(sensor_sigma) * z[:n].reshape(h, w, 3)
    np.rint(img, out=img)
    np.clip(img, 0, 255, out=img)
    return img.astype(np.uint8)


def log_uniform_sizes(seed, n, lo=(640, 480), hi=(6000, 4000)):
    """Mixed image sizes: log-uniform area between lo and hi, aspect ratio from {4:3, 3:2, 16:9, 1:1}."""
    u = uniforms(seed, 32, 2 * n)
    aspects = [4 / 3, 3 / 2, 16 / 9, 1.0]
    a_lo, a_hi = np.log(lo[0] * lo[1]), np.log(hi[0] * hi[1])
    out = []
    for i in range(n):
        area = np.exp(a_lo + (a_hi - a_lo) * u[2 * i])
        asp = aspects[min(3, int(u[2 * i + 1] * 4))]
        w = int(round(np.sqrt(area * asp)))
        h = int(round(w / asp))
        out.append((max(8, w), max(8, h)))
    return out


def _image_args(args):
    return image(*args)


def images(specs, workers=None):
    """[(w, h, seed, sensor_sigma), ...] -> list of images, generated in a spawn process pool."""
    import multiprocessing as mp
    import os

    workers = workers or min(len(specs), os.cpu_count() or 1, 16)
    if workers <= 1 or len(specs) <= 1:
        return [image(*s) for s in specs]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_image_args, specs, chunksize=1)
