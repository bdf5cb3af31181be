"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs, where it is
the checker (or the timed CPU restatement of the reference), never the measured product.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P, i32 = ctypes.c_void_p, ctypes.c_int
        pd = ctypes.POINTER(ctypes.c_double)
        pi = ctypes.POINTER(ctypes.c_int)
        L.orc_ssimulacra2.argtypes = [P, P, i32, i32, i32, i32, pd, P, pi]
        L.orc_ssimulacra2_fp64.argtypes = [P, P, i32, i32, i32, i32, pd, P, pi]
        L.orc_build_coefs.argtypes = [P, i32, i32, i32, i32, i32, i32, P, P, P]
        L.orc_coef_layout.argtypes = [i32, i32, i32, i32, i32, pi, P, P, P, P]
        L.orc_reconstruct.argtypes = [i32, i32, i32, P, P, P, P, P, P, P, pi]
        L.orc_ac_code_lengths.argtypes = [i32, i32, i32, P, P, P, P, P, P, P]
        L.orc_search.argtypes = [P, i32, i32, i32, ctypes.c_double, i32, i32, i32, pi, pd, P, P, P, P, pi, i32, P]
        for name in ("orc_ssim", "orc_psnr"):
            getattr(L, name).argtypes = [P, P, i32, i32, i32]
            getattr(L, name).restype = ctypes.c_double
        L.orc_ms_ssim.argtypes = [P, P, i32, i32, i32, P]
        for name in ("orc_score64", "orc_grad64"):
            getattr(L, name).restype = ctypes.c_double
        L.orc_score64.argtypes = [P, P, i32, i32]
        L.orc_grad64.argtypes = [P, P, i32, i32, P]
        L.orc_ms_ssim.restype = ctypes.c_double
        L.orc_write_best.argtypes = [i32, i32, i32, P, P, P, P, P, P, P, ctypes.c_long, pi]
        L.orc_write_best.restype = ctypes.c_long
        L.orc_requantize.argtypes = [i32, i32, i32, P, P, P, P, P, P, P, P, i32, i32, P, P, P, P]
        L.orc_reconstruct_tq.argtypes = [i32, i32, i32, P, P, P, P, P, P, P, P, P, pi]
        L.orc_search_requantize.argtypes = [i32, i32, i32, P, P, P, P, P, P, P, P, ctypes.c_double, i32, i32, pi, pd,
                                            P, P, P, P, P, P, pi, i32]
        L.orc_write_best_tq.argtypes = [i32, i32, i32, P, P, P, P, P, P, P, P, P, ctypes.c_long, pi]
        L.orc_write_best_tq.restype = ctypes.c_long
        pu64 = ctypes.POINTER(ctypes.c_uint64)
        L.orc_decode_sequential.argtypes = [P, ctypes.c_long, pi, pi, pi, P, P, P, P, P, P, P, P, P]
        L.orc_write_jpeg_variant.argtypes = [i32, i32, i32, P, P, P, P, P, P, P, P, i32, i32, P, ctypes.c_long]
        L.orc_write_jpeg_variant.restype = ctypes.c_long
        L.orc_emit_script.argtypes = [i32, i32, i32, P, P, P, P, P, P, i32, P, ctypes.c_long]
        L.orc_emit_script.restype = ctypes.c_long
        L.orc_script_count.argtypes = [i32]
        L.orc_script_count.restype = i32
        L.orc_plan.argtypes = [i32, i32, i32, P, P, P, P, P, pu64, pu64, pi, P, pi, P, P]
        L.orc_round_f32.argtypes = [ctypes.c_float]
        L.orc_round_f32.restype = ctypes.c_int32
        L.orc_fdct.argtypes = [P]
        L.orc_idct.argtypes = [P]
        L.orc_aan.restype = ctypes.POINTER(ctypes.c_float)
        L.orc_scale_table.argtypes = [i32, P]
        L.orc_rdo_quantize_ac.argtypes = [P, ctypes.c_float, P, P, P]
        L.orc_build_lengths.argtypes = [P, i32, i32, P]
        L.orc_optimal_sizes.argtypes = [P, P]
        L.orc_set_threads.argtypes = [i32]
        L.orc_max_threads.restype = i32
        _lib = L
    return _lib


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return int(lib().orc_max_threads())


def _img(a):
    a = np.ascontiguousarray(a)
    if a.ndim == 2:
        a = a[:, :, None]
    h, w, c = a.shape
    depth = 8
    if a.dtype == np.uint16:
        depth = 16
        a = np.ascontiguousarray(a.astype(">u2"))
    return a, w, h, c, depth


def ssimulacra2(ref, dist, fp64=False, per_scale=False):
    a, w, h, c, d = _img(ref)
    b, _, _, _, _ = _img(dist)
    out = ctypes.c_double()
    ps = np.zeros((6, 3, 6), dtype=np.float64)
    ns = ctypes.c_int()
    f = lib().orc_ssimulacra2_fp64 if fp64 else lib().orc_ssimulacra2
    rc = f(a.ctypes.data, b.ctypes.data, w, h, c, d, ctypes.byref(out), ps.ctypes.data, ctypes.byref(ns))
    if rc != 0:
        raise ValueError("invalid input for SSIMULACRA 2")
    if per_scale:
        return out.value, ps[: ns.value]
    return out.value


def layout(w, h, channels, quality, subsampling):
    nc = ctypes.c_int()
    hs, vs, bws, bhs = (np.zeros(3, dtype=np.int32) for _ in range(4))
    rc = lib().orc_coef_layout(w, h, channels, quality, int(subsampling), ctypes.byref(nc), hs.ctypes.data,
                               vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data)
    if rc != 0:
        raise ValueError("bad layout")
    n = nc.value
    return dict(ncomp=n, h=hs[:n].copy(), v=vs[:n].copy(), blocks_w=bws[:n].copy(), blocks_h=bhs[:n].copy(),
                ncoefs=int(sum(bws[i] * bhs[i] for i in range(n)) * 64))


def _weights(weights, ncoefs):
    """The perceptual trellis's per-coefficient weights (f32, coefficient layout) or None for the plain trellis."""
    if weights is None:
        return None, None
    wt = np.ascontiguousarray(weights, dtype=np.float32)
    if wt.size != ncoefs:
        raise ValueError("weights do not match the coefficient layout")
    return wt, wt.ctypes.data


def build_coefs(src, quality, subsampling, trellis=True, weights=None):
    a, w, h, c, _ = _img(src)
    lay = layout(w, h, c, quality, subsampling)
    coefs = np.zeros(lay["ncoefs"], dtype=np.int16)
    qt = np.zeros((2, 64), dtype=np.uint8)
    wt, wp = _weights(weights, lay["ncoefs"])
    rc = lib().orc_build_coefs(a.ctypes.data, w, h, c, quality, int(subsampling), 1 if trellis else 0,
                               coefs.ctypes.data, qt.ctypes.data, wp)
    if rc != 0:
        raise ValueError("bad input")
    return coefs, qt, lay


def _lay_arrays(lay):
    n = lay["ncomp"]
    pad = lambda x: np.ascontiguousarray(np.pad(np.asarray(x, dtype=np.int32), (0, 3 - n)))
    return n, pad(lay["h"]), pad(lay["v"]), pad(lay["blocks_w"]), pad(lay["blocks_h"])


def reconstruct(w, h, lay, qt, coefs):
    n, hs, vs, bws, bhs = _lay_arrays(lay)
    qt = np.ascontiguousarray(qt, dtype=np.uint8)
    coefs = np.ascontiguousarray(coefs, dtype=np.int16)
    out = np.zeros((h, w, n), dtype=np.uint8)
    oc = ctypes.c_int()
    lib().orc_reconstruct(w, h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data, qt.ctypes.data,
                          coefs.ctypes.data, out.ctypes.data, ctypes.byref(oc))
    return out[:, :, 0] if n == 1 else out


def ac_code_lengths(w, h, lay, qt, coefs):
    n, hs, vs, bws, bhs = _lay_arrays(lay)
    out = np.zeros((2, 256), dtype=np.uint8)
    qt = np.ascontiguousarray(qt, dtype=np.uint8)
    coefs = np.ascontiguousarray(coefs, dtype=np.int16)
    lib().orc_ac_code_lengths(w, h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data,
                              qt.ctypes.data, coefs.ctypes.data, out.ctypes.data)
    return out


METRIC_SSIMULACRA2, METRIC_SSIM = 0, 1


def search(src, target, max_quality=100, subsampling=0, trellis=True, metric=METRIC_SSIMULACRA2, weights=None):
    """find_quality_with; `weights` (explicit subsampling only) switches every candidate's trellis to the
    perceptual mode."""
    a, w, h, c, _ = _img(src)
    q = ctypes.c_int()
    s = ctypes.c_double()
    tq = np.zeros(16, dtype=np.int32)
    ts = np.zeros(16, dtype=np.float64)
    nt = ctypes.c_int()
    # layout depends on the found quality under Auto: size for the largest
    cap = max(layout(w, h, c, qq, subsampling)["ncoefs"] for qq in (1, 89, 90, 100))
    coefs = np.zeros(cap, dtype=np.int16)
    qt = np.zeros((2, 64), dtype=np.uint8)
    if weights is not None and int(subsampling) == 0 and c == 3:
        raise ValueError("perceptual weights need an explicit subsampling")
    wt, wp = (None, None) if weights is None else _weights(weights, layout(w, h, c, 50, subsampling)["ncoefs"])
    rc = lib().orc_search(a.ctypes.data, w, h, c, float(target), int(max_quality), int(subsampling),
                          1 if trellis else 0, ctypes.byref(q), ctypes.byref(s), coefs.ctypes.data, qt.ctypes.data,
                          tq.ctypes.data, ts.ctypes.data, ctypes.byref(nt), int(metric), wp)
    if rc != 0:
        raise ValueError("bad input")
    lay = layout(w, h, c, q.value, subsampling)
    trace = [(int(tq[i]), float(ts[i])) for i in range(nt.value)]
    return q.value, s.value, coefs[: lay["ncoefs"]].copy(), qt, lay, trace


def write_best(w, h, lay, qt, coefs):
    n, hs, vs, bws, bhs = _lay_arrays(lay)
    qt = np.ascontiguousarray(qt, dtype=np.uint8)
    coefs = np.ascontiguousarray(coefs, dtype=np.int16)
    prog = ctypes.c_int()
    size = lib().orc_write_best(w, h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data,
                                qt.ctypes.data, coefs.ctypes.data, None, 0, ctypes.byref(prog))
    out = np.zeros(size, dtype=np.uint8)
    lib().orc_write_best(w, h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data, qt.ctypes.data,
                         coefs.ctypes.data, out.ctypes.data, size, ctypes.byref(prog))
    return out.tobytes(), bool(prog.value)


class GeneralCoefs:
    """A general flat CoefImage: layout, per-component table slot tq, four table slots (has_q marks present ones)."""

    def __init__(self, w, h, lay, tq, qtables4, has_q, coefs):
        self.w, self.h, self.lay = w, h, lay
        self.tq = np.ascontiguousarray(np.pad(np.asarray(tq, np.int32), (0, 3 - len(tq))))
        self.qtables4 = np.ascontiguousarray(np.asarray(qtables4, np.uint8).reshape(4, 64))
        self.has_q = np.ascontiguousarray(np.asarray(has_q, np.uint8).reshape(4))
        self.coefs = np.ascontiguousarray(coefs, dtype=np.int16)

    def args(self):
        n, hs, vs, bws, bhs = _lay_arrays(self.lay)
        self._keep = (hs, vs, bws, bhs)
        return (self.w, self.h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data,
                self.tq.ctypes.data, self.qtables4.ctypes.data, self.has_q.ctypes.data, self.coefs.ctypes.data)


def general_from_encoder(w, h, lay, qt, coefs):
    """The encoder's CoefImage in general form: tq = [0, 1, 1], slots 0 (luma) and 1 (chroma)."""
    n = lay["ncomp"]
    q4 = np.zeros((4, 64), np.uint8)
    q4[0] = qt[0]
    has = np.zeros(4, np.uint8)
    has[0] = 1
    if n > 1:
        q4[1] = qt[1]
        has[1] = 1
    return GeneralCoefs(w, h, lay, [0] + [1] * (n - 1), q4, has, coefs)


def requantize(g, quality, trellis=True):
    out = np.zeros_like(g.coefs)
    tq = np.zeros(3, np.int32)
    q4 = np.zeros((4, 64), np.uint8)
    has = np.zeros(4, np.uint8)
    rc = lib().orc_requantize(*g.args(), int(quality), 1 if trellis else 0, out.ctypes.data, tq.ctypes.data,
                              q4.ctypes.data, has.ctypes.data)
    if rc:
        raise ValueError("unsupported component count")
    return GeneralCoefs(g.w, g.h, g.lay, tq[: g.lay["ncomp"]], q4, has, out)


def reconstruct_general(g):
    n = g.lay["ncomp"]
    out = np.zeros((g.h, g.w, n), np.uint8)
    oc = ctypes.c_int()
    lib().orc_reconstruct_tq(*g.args(), out.ctypes.data, ctypes.byref(oc))
    return out[:, :, 0] if n == 1 else out


def search_requantize(g, target, max_quality=100, trellis=True, metric=METRIC_SSIMULACRA2):
    q = ctypes.c_int()
    s = ctypes.c_double()
    out = np.zeros_like(g.coefs)
    tq = np.zeros(3, np.int32)
    q4 = np.zeros((4, 64), np.uint8)
    has = np.zeros(4, np.uint8)
    tqs = np.zeros(16, np.int32)
    ts = np.zeros(16, np.float64)
    nt = ctypes.c_int()
    rc = lib().orc_search_requantize(*g.args(), float(target), int(max_quality), 1 if trellis else 0,
                                     ctypes.byref(q), ctypes.byref(s), out.ctypes.data, tq.ctypes.data,
                                     q4.ctypes.data, has.ctypes.data, tqs.ctypes.data, ts.ctypes.data,
                                     ctypes.byref(nt), int(metric))
    if rc:
        raise ValueError("unsupported component count")
    trace = [(int(tqs[i]), float(ts[i])) for i in range(nt.value)]
    return q.value, s.value, GeneralCoefs(g.w, g.h, g.lay, tq[: g.lay["ncomp"]], q4, has, out), trace


def write_best_general(g):
    prog = ctypes.c_int()
    size = lib().orc_write_best_tq(*g.args(), None, 0, ctypes.byref(prog))
    out = np.zeros(size, dtype=np.uint8)
    lib().orc_write_best_tq(*g.args(), out.ctypes.data, size, ctypes.byref(prog))
    return out.tobytes(), bool(prog.value)


def plan(w, h, lay, coefs):
    """write_best's plan: (progressive estimate, baseline estimate, best script, [(scan, cost)] of distinct scans).
    A scan is (comps tuple, ss, se, ah, al)."""
    n, hs, vs, bws, bhs = _lay_arrays(lay)
    coefs = np.ascontiguousarray(coefs, dtype=np.int16)
    pe, be = ctypes.c_uint64(), ctypes.c_uint64()
    ns, nd = ctypes.c_int(), ctypes.c_int()
    scans = np.zeros(16 * 8, np.int32)
    dist = np.zeros(48 * 8, np.int32)
    costs = np.zeros(48, np.uint64)
    lib().orc_plan(w, h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data, coefs.ctypes.data,
                   ctypes.byref(pe), ctypes.byref(be), ctypes.byref(ns), scans.ctypes.data, ctypes.byref(nd),
                   dist.ctypes.data, costs.ctypes.data)

    def scan(a):
        return (tuple(int(x) for x in a[1: 1 + a[0]]), int(a[5]), int(a[6]), int(a[7]) >> 4, int(a[7]) & 15)

    best = [scan(scans[8 * i: 8 * i + 8]) for i in range(ns.value)]
    distinct = [(scan(dist[8 * i: 8 * i + 8]), int(costs[i])) for i in range(nd.value)]
    return int(pe.value), int(be.value), best, distinct


def _pair(a, b):
    a = np.ascontiguousarray(a, dtype=np.uint8)
    b = np.ascontiguousarray(b, dtype=np.uint8)
    if a.shape != b.shape:
        raise ValueError("images differ in shape")
    h, w = a.shape[:2]
    ch = 1 if a.ndim == 2 else a.shape[2]
    return a, b, w, h, ch


def ssim(a, b):
    """core/src/metrics.rs:13 (8-bit, every channel including alpha)."""
    a, b, w, h, ch = _pair(a, b)
    return lib().orc_ssim(a.ctypes.data, b.ctypes.data, w, h, ch)


def psnr(a, b):
    """core/src/metrics.rs:67."""
    a, b, w, h, ch = _pair(a, b)
    return lib().orc_psnr(a.ctypes.data, b.ctypes.data, w, h, ch)


def ms_ssim(a, b, per_scale=False):
    """core/src/metrics.rs:111; with per_scale, also the five clamped luma SSIM values."""
    a, b, w, h, ch = _pair(a, b)
    ps = np.zeros(5, np.float64)
    v = lib().orc_ms_ssim(a.ctypes.data, b.ctypes.data, w, h, ch, ps.ctypes.data)
    return (v, ps) if per_scale else v


def decode_sequential(data):
    """parse(data)?.into_coefs() for sequential and progressive Huffman JPEGs: (GeneralCoefs, ids) or raises
    ValueError with "invalid" / "unsupported". (The name predates progressive support; decode_huffman is the same.)"""
    data = np.frombuffer(bytes(data), np.uint8)
    w, h, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    hs, vs, bws, bhs = (np.zeros(4, np.int32) for _ in range(4))
    ids = np.zeros(4, np.uint8)
    args = lambda *rest: (data.ctypes.data, data.size, ctypes.byref(w), ctypes.byref(h), ctypes.byref(n),
                          hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data, ids.ctypes.data) + rest
    rc = lib().orc_decode_sequential(*args(None, None, None, None))
    if rc:
        raise ValueError("invalid" if rc == 1 else "unsupported")
    k = n.value
    lay = dict(ncomp=k, h=hs[:k].copy(), v=vs[:k].copy(), blocks_w=bws[:k].copy(), blocks_h=bhs[:k].copy(),
               ncoefs=int(sum(bws[i] * bhs[i] for i in range(k)) * 64))
    coefs = np.zeros(lay["ncoefs"], np.int16)
    tq = np.zeros(4, np.int32)
    q4 = np.zeros((4, 64), np.uint8)
    has = np.zeros(4, np.uint8)
    lib().orc_decode_sequential(*args(coefs.ctypes.data, tq.ctypes.data, q4.ctypes.data, has.ctypes.data))
    return GeneralCoefs(w.value, h.value, lay, tq[:k], q4, has, coefs), bytes(ids[:k])


decode_huffman = decode_sequential


def script_count(ncomp):
    """Candidate progressive scripts (jpeg/src/progressive.rs:242-295) for ncomp components."""
    return int(lib().orc_script_count(int(ncomp)))


def emit_script(w, h, lay, qt, coefs, index):
    """The progressive JPEG of a flat CoefImage written with candidate script `index` (progressive::emit)."""
    n, hs, vs, bws, bhs = _lay_arrays(lay)
    qt = np.ascontiguousarray(qt, dtype=np.uint8)
    coefs = np.ascontiguousarray(coefs, dtype=np.int16)
    size = lib().orc_emit_script(w, h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data,
                                 qt.ctypes.data, coefs.ctypes.data, int(index), None, 0)
    if size < 0:
        raise ValueError("bad script index")
    out = np.zeros(size, np.uint8)
    lib().orc_emit_script(w, h, n, hs.ctypes.data, vs.ctypes.data, bws.ctypes.data, bhs.ctypes.data,
                          qt.ctypes.data, coefs.ctypes.data, int(index), out.ctypes.data, size)
    return out.tobytes()


def write_jpeg_variant(g, restart_interval=0, per_component=False):
    """Baseline JPEG of a GeneralCoefs with a restart interval and/or one scan per component (decoder tests)."""
    size = lib().orc_write_jpeg_variant(*g.args(), int(restart_interval), 1 if per_component else 0, None, 0)
    out = np.zeros(size, np.uint8)
    lib().orc_write_jpeg_variant(*g.args(), int(restart_interval), 1 if per_component else 0, out.ctypes.data, size)
    return out.tobytes()


def score64(ref, dist):
    """FP64 SSIMULACRA2 with the distorted RGB image as continuous values (float array (h, w, 3) in [0, 255])."""
    r = np.ascontiguousarray(ref, dtype=np.float64)
    d = np.ascontiguousarray(dist, dtype=np.float64)
    h, w = r.shape[:2]
    return lib().orc_score64(r.ctypes.data, d.ctypes.data, w, h)


def grad64(ref, dist):
    """(score, d score / d dist) of score64, the gradient as a float64 (h, w, 3) array."""
    r = np.ascontiguousarray(ref, dtype=np.float64)
    d = np.ascontiguousarray(dist, dtype=np.float64)
    h, w = r.shape[:2]
    g = np.zeros((h, w, 3), np.float64)
    s = lib().orc_grad64(r.ctypes.data, d.ctypes.data, w, h, g.ctypes.data)
    return s, g



# ------------------------------------------------------------------------------------------------ perceptual trellis
# The adjoint of the decoder's linear part, restated in numpy (f64). Forward: orthonormal 8x8 IDCT per block
# (jpeg/src/dct.rs:67-119 with the multipliers of jpeg/src/decode.rs:1316-1321), triangle-filter chroma upsampling
# (jpeg/src/decode.rs:1768-1828: 3/4 near + 1/4 far per axis, far index clamped), fixed-point YCbCr->RGB
# (jpeg/src/decode.rs:1438-1441); roundings and clamps dropped. The weights are the perceptual mode's rule (no
# reference counterpart): W[b][k] = strength * clamp((s_b / mean_c s)^gamma, w_min, w_max), s_b the RMS of the blocks'
# gradient energies over a (2 radius + 1)^2 edge-replicated neighbourhood.

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                   13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52,
                   45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])  # jpeg/src/lib.rs:14-19
DCT8 = np.array([[(np.sqrt(1 / 8) if u == 0 else 0.5) * np.cos((2 * x + 1) * u * np.pi / 16) for x in range(8)]
                 for u in range(8)])
# d(R, G, B) / d(Y, Cb, Cr) of jpeg/src/decode.rs:1438-1441 without rounding
YCC_TO_RGB = np.array([[1.0, 0.0, 91881 / 65536], [1.0, -22554 / 65536, -46802 / 65536], [1.0, 116130 / 65536, 0.0]])


def _upsample_matrix(n_full, n_c, f):
    """[n_full, n_c] weights of one axis of the upsampler (identity for f == 1)."""
    m = np.zeros((n_full, n_c))
    if f == 1:
        m[np.arange(n_full), np.arange(n_full)] = 1.0
        return m
    x = np.arange(n_full)
    near = x // 2
    far = np.where(x % 2 == 0, np.maximum(near - 1, 0), np.minimum(near + 1, n_c - 1))
    np.add.at(m, (x, near), 0.75)
    np.add.at(m, (x, far), 0.25)
    return m


def _comp_geometry(w, h, lay, c):
    hmax, vmax = max(lay["h"]), max(lay["v"])
    fx, fy = hmax // lay["h"][c], vmax // lay["v"][c]
    cw, ch = (w * lay["h"][c] + hmax - 1) // hmax, (h * lay["v"][c] + vmax - 1) // vmax
    return fx, fy, cw, ch


def component_gradients(grad, w, h, lay):
    """d score / d component sample per component (padded block grid, f64), from d score / d RGB (h, w, 3)."""
    g = np.asarray(grad, dtype=np.float64)
    if lay["ncomp"] == 1:
        planes = [g.sum(2)]
    else:
        planes = [np.tensordot(g, YCC_TO_RGB[:, c], axes=([2], [0])) for c in range(3)]
    out = []
    for c in range(lay["ncomp"]):
        fx, fy, cw, ch = _comp_geometry(w, h, lay, c)
        ux, uy = _upsample_matrix(w, cw, fx), _upsample_matrix(h, ch, fy)
        gc = uy.T @ planes[c] @ ux
        P = np.zeros((lay["blocks_h"][c] * 8, lay["blocks_w"][c] * 8))
        P[:ch, :cw] = gc
        out.append(P)
    return out


def coef_gradient(grad, w, h, lay):
    """d score / d coefficient (dequantized units), coefficient layout (64 zigzag entries per block), f64."""
    res = []
    for c, P in enumerate(component_gradients(grad, w, h, lay)):
        bw, bh = lay["blocks_w"][c], lay["blocks_h"][c]
        B = P.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
        G = np.einsum("vy,abyx,ux->abvu", DCT8, B, DCT8).reshape(bh * bw, 64)
        res.append(G[:, ZIGZAG].reshape(-1))
    return np.concatenate(res)


def decode_linear(coef_f, w, h, lay):
    """The forward map whose adjoint coef_gradient is: dequantized coefficients (coefficient layout) -> RGB (h, w, 3)
    (or Gray replicated), without level shift, roundings or clamps."""
    comps, off = [], 0
    for c in range(lay["ncomp"]):
        bw, bh = lay["blocks_w"][c], lay["blocks_h"][c]
        F = np.zeros((bh * bw, 64))
        F[:, ZIGZAG] = coef_f[off * 64:(off + bw * bh) * 64].reshape(-1, 64)
        off += bw * bh
        B = np.einsum("vy,abvu,ux->abyx", DCT8, F.reshape(bh, bw, 8, 8), DCT8)
        P = B.transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8)
        fx, fy, cw, ch = _comp_geometry(w, h, lay, c)
        comps.append(_upsample_matrix(h, ch, fy) @ P[:ch, :cw] @ _upsample_matrix(w, cw, fx).T)
    if lay["ncomp"] == 1:
        return np.repeat(comps[0][:, :, None], 3, 2)
    return np.stack([sum(YCC_TO_RGB[k, c] * comps[c] for c in range(3)) for k in range(3)], 2)


def perceptual_weights(grad, w, h, lay, strength=0.35, gamma=0.5, w_min=0.25, w_max=4.0, radius=1):
    """The perceptual trellis weights (f32, coefficient layout) from d score / d RGB."""
    res = []
    for c, P in enumerate(component_gradients(grad, w, h, lay)):
        bw, bh = lay["blocks_w"][c], lay["blocks_h"][c]
        e = (P.reshape(bh, 8, bw, 8) ** 2).sum((1, 3))
        p = np.pad(e, radius, mode="edge")
        acc = np.zeros_like(e)
        for dy in range(2 * radius + 1):
            for dx in range(2 * radius + 1):
                acc += p[dy:dy + bh, dx:dx + bw]
        s = np.sqrt(acc / (2 * radius + 1) ** 2).reshape(-1)
        m = s.mean()
        r = s / m if m > 0 else np.ones_like(s)
        wv = (np.clip(r ** gamma, w_min, w_max) * strength).astype(np.float32)
        res.append(np.repeat(wv, 64))
    return np.concatenate(res)
