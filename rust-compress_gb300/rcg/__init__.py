"""Python host side of rcg: the reference's JPEG quality-search interface over the C ABI in include/rcg.h.

Names and argument meaning follow rust-compress:
  ssimulacra2(reference, distorted) -> float            core/src/ssimulacra2.rs:471
  build_coefs(src, EncodeOptions) -> CoefImage          jpeg/src/encode.rs:426
  reconstruct(CoefImage) -> Image                        jpeg/src/decode.rs:334
  find_quality_ssimulacra2(reference, target, max_q, opts) -> Found
      = jpeg::target::find_quality_with (jpeg/src/target.rs:29) with make = build_coefs and
        metric = ssimulacra2(..).unwrap_or(f64::MIN) (cli/src/pipeline.rs:207-222)
Errors surface as RcgError carrying the C status (Invalid / Unsupported like rc_core::error::Error).

Images are numpy uint8 arrays: (h, w, 3) for Rgb, (h, w) or (h, w, 1) for Gray; the scorer also takes
(h, w, 2|4) with alpha and uint16 arrays (16-bit samples). The library is loaded from this directory on first use
(creating a Context, or lib()), so importing the package or rcg.synth maps no GPU code; there is no fallback: if
librcg.so is missing or cannot be loaded, that first use raises.
"""

import ctypes
import enum
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "librcg.so")

RCG_OK, RCG_INVALID, RCG_UNSUPPORTED, RCG_CUDA_ERROR, RCG_TIMEOUT, RCG_NO_MEMORY = range(6)
_STATUS_NAMES = {1: "Invalid", 2: "Unsupported", 3: "CudaError", 4: "Timeout", 5: "NoMemory"}


METRIC_SSIMULACRA2, METRIC_SSIM, METRIC_PSNR, METRIC_MS_SSIM = 0, 1, 2, 3


class RcgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


class Subsampling(enum.IntEnum):
    """jpeg::encode::Subsampling (jpeg/src/encode.rs:12-20)."""

    Auto = 0
    S444 = 1
    S422 = 2
    S420 = 3


@dataclass
class EncodeOptions:
    """jpeg::encode::EncodeOptions (jpeg/src/encode.rs:22-37); alpha must be flattened by the caller."""

    quality: int = 80
    subsampling: Subsampling = Subsampling.Auto
    trellis: bool = True


class _Opts(ctypes.Structure):
    _fields_ = [("quality", ctypes.c_int32), ("subsampling", ctypes.c_int32), ("trellis", ctypes.c_int32)]


class _Layout(ctypes.Structure):
    _fields_ = [
        ("ncomp", ctypes.c_int32),
        ("h", ctypes.c_int32 * 3),
        ("v", ctypes.c_int32 * 3),
        ("blocks_w", ctypes.c_int32 * 3),
        ("blocks_h", ctypes.c_int32 * 3),
        ("ncoefs", ctypes.c_int64),
    ]


class _Found(ctypes.Structure):
    _fields_ = [
        ("quality", ctypes.c_int32),
        ("score", ctypes.c_double),
        ("nsteps", ctypes.c_int32),
        ("trace_q", ctypes.c_int32 * 16),
        ("trace_score", ctypes.c_double * 16),
    ]


class _QTables(ctypes.Structure):
    _fields_ = [("tq", ctypes.c_int32 * 3), ("qtables", (ctypes.c_uint8 * 64) * 4), ("present", ctypes.c_int32 * 4)]


class _JpegInfo(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("ids", ctypes.c_uint8 * 4),
                ("scans", ctypes.c_int32), ("sync_rounds", ctypes.c_int32)]


class _Scan(ctypes.Structure):
    _fields_ = [("ncomps", ctypes.c_int32), ("comps", ctypes.c_int32 * 4), ("ss", ctypes.c_int32),
                ("se", ctypes.c_int32), ("ah", ctypes.c_int32), ("al", ctypes.c_int32)]


class _PlanResult(ctypes.Structure):
    _fields_ = [("progressive_bytes", ctypes.c_uint64), ("baseline_bytes", ctypes.c_uint64),
                ("progressive", ctypes.c_int32), ("nscans", ctypes.c_int32), ("scans", _Scan * 16),
                ("ndistinct", ctypes.c_int32), ("distinct", _Scan * 48), ("distinct_bytes", ctypes.c_uint64 * 48)]


class _PerceptualOpts(ctypes.Structure):
    _fields_ = [("strength", ctypes.c_double), ("gamma", ctypes.c_double), ("w_min", ctypes.c_double),
                ("w_max", ctypes.c_double), ("radius", ctypes.c_int32), ("keep_smaller", ctypes.c_int32),
                ("gradient_fp64", ctypes.c_int32), ("strength_by_quality", ctypes.c_int32)]


@dataclass
class PerceptualOptions:
    """Options of the perceptual trellis (rcg_perceptual_options): W[b][k] = strength * clamp((s_b / mean s)^gamma,
    w_min, w_max) with s_b the RMS coefficient-gradient energy over the (2 radius + 1)^2 blocks around block b; the
    gradient from the FP32 adjoint unless gradient_fp64."""

    strength: float = 0.35
    gamma: float = 0.5
    w_min: float = 0.25
    w_max: float = 4.0
    radius: int = 1
    keep_smaller: bool = True
    gradient_fp64: bool = False  # the FP64 adjoint instead of its FP32 instantiation
    strength_by_quality: bool = True  # find_quality_perceptual: strength from the plain result's quality

    def _c(self):
        return _PerceptualOpts(float(self.strength), float(self.gamma), float(self.w_min), float(self.w_max),
                               int(self.radius), 1 if self.keep_smaller else 0, 1 if self.gradient_fp64 else 0,
                               1 if self.strength_by_quality else 0)

    def strength_for(self, quality):
        """The strength find_quality_perceptual uses after a plain search found `quality`."""
        o = self._c()
        return float(_lib.rcg_perceptual_strength(ctypes.byref(o), int(quality)))


@dataclass
class PerceptualFound:
    """rcg_search_perceptual: the plain search's result, the returned result (the weighted search's, or the plain
    one when it plans smaller and keep_smaller is set), both planned sizes and the weights."""

    plain: "Found"
    found: "Found"
    plain_bytes: int
    perceptual_bytes: int
    chose_perceptual: bool
    weights: np.ndarray


@dataclass
class Plan:
    """write_best's decision (jpeg/src/encode.rs:543-565): the estimated sizes, whether the progressive script wins,
    the script (scans as (comps, ss, se, ah, al)) and every distinct candidate scan with its cost."""

    progressive_bytes: int
    baseline_bytes: int
    progressive: bool
    scans: list
    distinct: list


def _scan_tuple(sc):
    return (tuple(int(sc.comps[i]) for i in range(sc.ncomps)), int(sc.ss), int(sc.se), int(sc.ah), int(sc.al))


def _plan(r):
    return Plan(int(r.progressive_bytes), int(r.baseline_bytes), bool(r.progressive),
                [_scan_tuple(r.scans[i]) for i in range(r.nscans)],
                [(_scan_tuple(r.distinct[i]), int(r.distinct_bytes[i])) for i in range(r.ndistinct)])


@dataclass
class CoefComponent:
    """jpeg::encode::CoefComponent (jpeg/src/encode.rs:56-69)."""

    id: int
    h: int
    v: int
    tq: int
    blocks_w: int
    blocks_h: int
    coefs: np.ndarray  # int16, (blocks_h * blocks_w * 64,), zigzag order per block


@dataclass
class CoefImage:
    """jpeg::encode::CoefImage (jpeg/src/encode.rs:71-83), restricted to what the pixel path produces."""

    width: int
    height: int
    comps: list
    # uint8 natural order. Encoder form: (2, 64), slot 0 luma and slot 1 chroma, `present` None. General form
    # (requantized images, jpeg/src/encode.rs:77): (4, 64) by slot, `present` marks the slots that hold a table.
    qtables: np.ndarray
    present: np.ndarray = None

    def flat(self):
        return np.concatenate([c.coefs for c in self.comps]).astype(np.int16, copy=False)

    def layout(self):
        lay = _Layout()
        lay.ncomp = len(self.comps)
        for i, c in enumerate(self.comps):
            lay.h[i], lay.v[i] = c.h, c.v
            lay.blocks_w[i], lay.blocks_h[i] = c.blocks_w, c.blocks_h
        lay.ncoefs = sum(c.coefs.size for c in self.comps)
        return lay

    def table_slots(self):
        """The general table assignment (tq per component, four slots)."""
        t = _QTables()
        for i, c in enumerate(self.comps):
            t.tq[i] = c.tq
        q = np.asarray(self.qtables, np.uint8)
        present = [1, 1, 0, 0] if self.present is None else [int(x) for x in self.present]
        if self.present is None and len(self.comps) == 1:
            present = [1, 0, 0, 0]
        for sl in range(4):
            t.present[sl] = present[sl]
            if present[sl] and sl < q.shape[0]:
                ctypes.memmove(t.qtables[sl], q[sl].ctypes.data, 64)
        return t


@dataclass
class Found:
    """jpeg::target::Found (jpeg/src/target.rs:12-18) plus the evaluated (quality, score) trace."""

    quality: int
    score: float
    coefs: CoefImage
    trace: list = field(default_factory=list)


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() (no CPU fallback exists)")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    u32, i32, sz = ctypes.c_uint32, ctypes.c_int, ctypes.c_size_t
    sig = {
        "rcg_ctx_create": (i32, [i32, ctypes.POINTER(P)]),
        "rcg_ctx_destroy": (None, [P]),
        "rcg_last_error": (ctypes.c_char_p, [P]),
        "rcg_ctx_set_stream": (i32, [P, P]),
        "rcg_ctx_stream": (P, [P]),
        "rcg_ctx_synchronize": (i32, [P]),
        "rcg_ctx_launch_count": (ctypes.c_uint64, [P]),
        "rcg_ctx_set_profiling": (i32, [P, i32]),
        "rcg_ctx_set_graphs": (i32, [P, i32]),
        "rcg_ssimulacra2_batch": (i32, [P, i32, P, P, P, P, P, P, P]),
        "rcg_ssimulacra2_batch_device": (i32, [P, i32, P, P, P, P, P, P, P]),
        "rcg_sweep_qualities": (i32, [P, i32, P, P, P, P, i32, P, ctypes.POINTER(_Opts), P]),
        "rcg_ctx_graph_stats": (i32, [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
        "rcg_ctx_kernel_time": (i32, [P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64),
                                      ctypes.POINTER(ctypes.c_double)]),
        "rcg_coef_layout_for": (i32, [u32, u32, i32, ctypes.POINTER(_Opts), ctypes.POINTER(_Layout)]),
        "rcg_ssimulacra2": (i32, [P, P, P, u32, u32, i32, i32, ctypes.POINTER(ctypes.c_double)]),
        "rcg_ssimulacra2_device": (i32, [P, P, P, u32, u32, i32, ctypes.POINTER(ctypes.c_double)]),
        "rcg_ssimulacra2_exact": (i32, [P, P, P, u32, u32, i32, i32, ctypes.POINTER(ctypes.c_double)]),
        "rcg_ctx_set_tie_band": (i32, [P, ctypes.c_double]),
        "rcg_ctx_tie_rescores": (ctypes.c_uint64, [P]),
        "rcg_ctx_set_band_chunks": (i32, [P, i32]),
        "rcg_ctx_band_chunks": (i32, [P, u32, u32]),
        "rcg_ctx_set_ref_cache": (i32, [P, i32]),
        "rcg_ssimulacra2_device_noalloc": (i32, [P, P, u32, u32, i32, P, P]),
        "rcg_build_coefs": (i32, [P, P, u32, u32, i32, ctypes.POINTER(_Opts), P, sz, P]),
        "rcg_reconstruct": (i32, [P, u32, u32, ctypes.POINTER(_Layout), P, P, P, sz]),
        "rcg_search": (i32, [P, P, u32, u32, i32, ctypes.c_double, i32, ctypes.POINTER(_Opts),
                             ctypes.POINTER(_Found), P, sz, P]),
        "rcg_search_device": (i32, [P, P, u32, u32, i32, ctypes.c_double, i32, ctypes.POINTER(_Opts),
                                    ctypes.POINTER(_Found), P, sz, P]),
        "rcg_reconstruct_tables": (i32, [P, u32, u32, ctypes.POINTER(_Layout), ctypes.POINTER(_QTables), P, P, sz]),
        "rcg_requantize": (i32, [P, u32, u32, ctypes.POINTER(_Layout), ctypes.POINTER(_QTables), P, i32, i32, P, sz,
                                 ctypes.POINTER(_QTables)]),
        "rcg_search_requantize": (i32, [P, u32, u32, ctypes.POINTER(_Layout), ctypes.POINTER(_QTables), P, i32,
                                        ctypes.c_double, i32, i32, ctypes.POINTER(_Found), P, sz,
                                        ctypes.POINTER(_QTables)]),
        "rcg_metric_score": (i32, [P, i32, P, P, u32, u32, i32, ctypes.POINTER(ctypes.c_double)]),
        "rcg_metric_score_device": (i32, [P, i32, P, P, u32, u32, i32, ctypes.POINTER(ctypes.c_double)]),
        "rcg_search_metric": (i32, [P, P, u32, u32, i32, i32, ctypes.c_double, i32, ctypes.POINTER(_Opts),
                                    ctypes.POINTER(_Found), P, sz, P]),
        "rcg_decode_coefs": (i32, [P, P, sz, ctypes.POINTER(_JpegInfo), ctypes.POINTER(_Layout),
                                   ctypes.POINTER(_QTables), P, sz]),
        "rcg_decode_coefs_device": (i32, [P, P, sz, ctypes.POINTER(_JpegInfo), ctypes.POINTER(_Layout),
                                          ctypes.POINTER(_QTables), P, sz]),
        "rcg_search_requantize_device": (i32, [P, u32, u32, ctypes.POINTER(_Layout), ctypes.POINTER(_QTables), P,
                                               i32, ctypes.c_double, i32, i32, ctypes.POINTER(_Found), P, sz,
                                               ctypes.POINTER(_QTables)]),
        "rcg_ssimulacra2_grad": (i32, [P, P, P, u32, u32, ctypes.POINTER(ctypes.c_double), P]),
        "rcg_ssimulacra2_grad_device": (i32, [P, P, P, u32, u32, ctypes.POINTER(ctypes.c_double), P]),
        "rcg_plan": (i32, [P, u32, u32, ctypes.POINTER(_Layout), P, sz, ctypes.POINTER(_PlanResult)]),
        "rcg_plan_device": (i32, [P, u32, u32, ctypes.POINTER(_Layout), P, ctypes.POINTER(_PlanResult)]),
        "rcg_search_batch": (i32, [P, i32, P, P, P, P, P, i32, ctypes.POINTER(_Opts), i32, P, P, P, P]),
        "rcg_search_batch_lockstep": (i32, [P, i32, P, P, P, P, P, i32, ctypes.POINTER(_Opts), P, P, P, P]),
        "rcg_perceptual_defaults": (None, [ctypes.POINTER(_PerceptualOpts)]),
        "rcg_perceptual_strength": (ctypes.c_double, [ctypes.POINTER(_PerceptualOpts), i32]),
        "rcg_coef_gradient": (i32, [P, P, P, u32, u32, i32, ctypes.POINTER(_Layout),
                                    ctypes.POINTER(ctypes.c_double), P, sz]),
        "rcg_perceptual_weights": (i32, [P, P, P, u32, u32, i32, ctypes.POINTER(_Layout),
                                         ctypes.POINTER(_PerceptualOpts), ctypes.POINTER(ctypes.c_double), P, sz]),
        "rcg_build_coefs_weighted": (i32, [P, P, u32, u32, i32, ctypes.POINTER(_Opts), P, sz, P, sz, P]),
        "rcg_search_weighted": (i32, [P, P, u32, u32, i32, ctypes.c_double, i32, ctypes.POINTER(_Opts), P, sz,
                                      ctypes.POINTER(_Found), P, sz, P]),
        "rcg_search_perceptual": (i32, [P, P, u32, u32, i32, ctypes.c_double, i32, ctypes.POINTER(_Opts),
                                        ctypes.POINTER(_PerceptualOpts), ctypes.POINTER(_Found),
                                        ctypes.POINTER(_Found), P, ctypes.POINTER(ctypes.c_int), P, sz, P, P, sz]),
        "rcg_search_perceptual_fast": (i32, [P, P, u32, u32, i32, ctypes.c_double, i32, ctypes.POINTER(_Opts),
                                             ctypes.POINTER(_PerceptualOpts), ctypes.POINTER(_Found),
                                             ctypes.POINTER(_Found), P, sz, P, P, sz]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


class _LazyLib:
    """librcg.so, loaded (and its signatures declared) on the first attribute access."""

    _real = None

    def get(self):
        if _LazyLib._real is None:
            _LazyLib._real = _load()
        return _LazyLib._real

    def __getattr__(self, name):
        return getattr(self.get(), name)


_lib = _LazyLib()
EXPORTED = (
    "rcg_ctx_create rcg_ctx_destroy rcg_last_error rcg_ctx_set_stream rcg_ctx_stream rcg_ctx_synchronize "
    "rcg_ctx_launch_count rcg_ctx_set_profiling rcg_ctx_kernel_time rcg_coef_layout_for rcg_ssimulacra2 "
    "rcg_ssimulacra2_device rcg_ssimulacra2_device_noalloc rcg_build_coefs rcg_reconstruct rcg_search rcg_search_device "
    "rcg_search_batch rcg_reconstruct_tables rcg_requantize rcg_search_requantize rcg_plan rcg_plan_device "
    "rcg_metric_score rcg_metric_score_device rcg_search_metric rcg_decode_coefs rcg_decode_coefs_device "
    "rcg_search_requantize_device rcg_ssimulacra2_grad rcg_ssimulacra2_grad_device rcg_perceptual_defaults "
    "rcg_coef_gradient rcg_perceptual_weights rcg_build_coefs_weighted rcg_search_weighted rcg_search_perceptual "
    "rcg_perceptual_strength rcg_ctx_set_graphs rcg_ctx_graph_stats rcg_ssimulacra2_batch rcg_ssimulacra2_batch_device "
    "rcg_sweep_qualities rcg_ssimulacra2_exact rcg_ctx_set_tie_band rcg_ctx_tie_rescores "
    "rcg_ctx_set_band_chunks rcg_ctx_band_chunks rcg_search_batch_lockstep rcg_search_perceptual_fast "
    "rcg_ctx_set_ref_cache"
).split()


def lib():
    """The loaded librcg.so (loads it on first call; raises if it is missing)."""
    return _lib.get()


def _opts(o):
    return _Opts(int(o.quality), int(o.subsampling), 1 if o.trellis else 0)


def _out_buffer(arr, dtype, n):
    """A caller's reusable output array (checked) or a new one of n entries."""
    if arr is None:
        return np.zeros(n, dtype=dtype)
    if arr.dtype != dtype or arr.size < n or not arr.flags.c_contiguous:
        raise ValueError(f"the buffer must be a contiguous {np.dtype(dtype).name} array of at least {n} entries")
    return arr


def _image(img):
    """(data, w, h, channels, depth) of an image array, C-contiguous."""
    a = np.ascontiguousarray(img)
    if a.ndim == 2:
        a = a[:, :, None]
    if a.ndim != 3:
        raise ValueError("image must be (h, w) or (h, w, c)")
    h, w, c = a.shape
    if a.dtype == np.uint8:
        depth = 8
    elif a.dtype == np.uint16:
        depth = 16
        a = a.astype(">u2")  # the reference stores 16-bit samples big-endian (core/src/image.rs:103)
    else:
        raise ValueError("image samples must be uint8 or uint16")
    return np.ascontiguousarray(a), w, h, c, depth


class Context:
    """One rcg_ctx: a CUDA stream plus device workspace. Not thread-safe; use one per thread."""

    def __init__(self, device=0):
        self._ptr = ctypes.c_void_p()
        rc = _lib.rcg_ctx_create(int(device), ctypes.byref(self._ptr))
        if rc != RCG_OK:
            raise RcgError(rc, f"cannot create a context on CUDA device {device}")

    def close(self):
        if self._ptr:
            _lib.rcg_ctx_destroy(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._ptr

    def _check(self, rc):
        if rc != RCG_OK:
            raise RcgError(rc, _lib.rcg_last_error(self._ptr).decode())

    # ---- plumbing
    def set_stream(self, stream_ptr):
        self._check(_lib.rcg_ctx_set_stream(self._ptr, ctypes.c_void_p(stream_ptr or 0)))

    def stream(self):
        return _lib.rcg_ctx_stream(self._ptr)

    def synchronize(self):
        self._check(_lib.rcg_ctx_synchronize(self._ptr))

    def launch_count(self):
        return int(_lib.rcg_ctx_launch_count(self._ptr))

    def set_profiling(self, on):
        self._check(_lib.rcg_ctx_set_profiling(self._ptr, 1 if on else 0))

    def set_graphs(self, on):
        """CUDA graphs for the searches' step loops (on by default); results are the same either way."""
        self._check(_lib.rcg_ctx_set_graphs(self._ptr, 1 if on else 0))

    def graph_stats(self):
        """(step loops captured, graph launches) on this context so far."""
        c = ctypes.c_uint64()
        r = ctypes.c_uint64()
        self._check(_lib.rcg_ctx_graph_stats(self._ptr, ctypes.byref(c), ctypes.byref(r)))
        return int(c.value), int(r.value)

    def set_tie_band(self, band):
        """Near-tie band of the SSIMULACRA2 searches: candidates whose fast score lies within `band` of the target
        are decided on their reference-order FP64 score (default 1e-3; 0 never, math.inf always)."""
        self._check(_lib.rcg_ctx_set_tie_band(self._ptr, float(band)))

    def tie_rescores(self):
        """Candidates this context has decided on the reference-order FP64 score so far."""
        return int(_lib.rcg_ctx_tie_rescores(self._ptr))

    def set_band_chunks(self, chunks):
        """The fast scorer's band height in 32-row chunks: 0 autotunes per size class (default), 1..64 fixes it."""
        self._check(_lib.rcg_ctx_set_band_chunks(self._ptr, int(chunks)))

    def set_ref_cache(self, on):
        """The SSIMULACRA2 searches' stored reference moments (default on; the same scores either way)."""
        self._check(_lib.rcg_ctx_set_ref_cache(self._ptr, 1 if on else 0))

    def band_chunks(self, width, height):
        """Chunks per band used for a width x height image (autotuning its size class if needed)."""
        return int(_lib.rcg_ctx_band_chunks(self._ptr, int(width), int(height)))

    def kernel_time(self, name):
        n = ctypes.c_uint64()
        ms = ctypes.c_double()
        self._check(_lib.rcg_ctx_kernel_time(self._ptr, name.encode(), ctypes.byref(n), ctypes.byref(ms)))
        return int(n.value), float(ms.value)

    # ---- the path
    def ssimulacra2(self, reference, distorted):
        """core/src/ssimulacra2.rs:471: score of `distorted` against `reference` (RcgError on Invalid)."""
        a, w, h, c, d = _image(reference)
        b, w2, h2, c2, d2 = _image(distorted)
        if (w, h) != (w2, h2):
            raise RcgError(RCG_INVALID, "images differ in size")
        if (c, d) != (c2, d2):
            raise RcgError(RCG_INVALID, "images differ in colour type")
        out = ctypes.c_double()
        self._check(_lib.rcg_ssimulacra2(self._ptr, a.ctypes.data, b.ctypes.data, w, h, c, d, ctypes.byref(out)))
        return out.value

    def ssimulacra2_exact(self, reference, distorted):
        """The same score in the reference's own f64 arithmetic and order (rcg_ssimulacra2_exact): equal to
        core/src/ssimulacra2.rs:471's result up to the last bits of cbrt/pow; much slower than ssimulacra2."""
        a, w, h, c, d = _image(reference)
        b, w2, h2, c2, d2 = _image(distorted)
        if (w, h) != (w2, h2):
            raise RcgError(RCG_INVALID, "images differ in size")
        if (c, d) != (c2, d2):
            raise RcgError(RCG_INVALID, "images differ in colour type")
        out = ctypes.c_double()
        self._check(_lib.rcg_ssimulacra2_exact(self._ptr, a.ctypes.data, b.ctypes.data, w, h, c, d,
                                               ctypes.byref(out)))
        return out.value

    def ssimulacra2_batch(self, pairs):
        """Scores of many (reference, distorted) pairs of any sizes (rcg_ssimulacra2_batch); the same reference
        object given for several pairs is uploaded and converted once. Returns a float64 array."""
        n = len(pairs)
        conv, keep = {}, []

        def arr(img):
            if id(img) not in conv:
                conv[id(img)] = _image(img)
                keep.append(img)
            return conv[id(img)]

        P = ctypes.c_void_p * max(n, 1)
        refs, dists = P(), P()
        ws, hs, cs, ds = (ctypes.c_uint32 * max(n, 1))(), (ctypes.c_uint32 * max(n, 1))(), \
            (ctypes.c_int32 * max(n, 1))(), (ctypes.c_int32 * max(n, 1))()
        for i, (ref, dist) in enumerate(pairs):
            a, w, h, c, d = arr(ref)
            b, w2, h2, c2, d2 = arr(dist)
            if (w, h, c, d) != (w2, h2, c2, d2):
                raise RcgError(RCG_INVALID, f"pair {i}: images differ in size or colour type")
            refs[i], dists[i] = a.ctypes.data, b.ctypes.data
            ws[i], hs[i], cs[i], ds[i] = w, h, c, d
        out = np.zeros(max(n, 1), dtype=np.float64)
        self._check(_lib.rcg_ssimulacra2_batch(self._ptr, n, refs, dists, ws, hs, cs, ds, out.ctypes.data))
        return out[:n]

    def sweep_qualities(self, images, qualities, opts=None):
        """rcg_sweep_qualities: a (len(images), len(qualities)) float64 array of the SSIMULACRA2 score of each image
        against its candidate at each quality (build_coefs at that quality, reconstruct, ssimulacra2)."""
        opts = opts or EncodeOptions()
        n, nq = len(images), len(qualities)
        arrs = []
        for im in images:
            a, w, h, c, d = _image(im)
            if d != 8 or c not in (1, 3):
                raise RcgError(RCG_INVALID, "the sweep takes 8-bit Gray or Rgb")
            arrs.append((a, w, h, c))
        P = ctypes.c_void_p * max(n, 1)
        U = ctypes.c_uint32 * max(n, 1)
        I = ctypes.c_int32 * max(n, 1)
        q = (ctypes.c_int32 * nq)(*[int(x) for x in qualities])
        out = np.zeros((max(n, 1), nq), dtype=np.float64)
        o = _opts(opts)
        self._check(_lib.rcg_sweep_qualities(self._ptr, n, P(*[a.ctypes.data for a, _, _, _ in arrs]),
                                             U(*[w for _, w, _, _ in arrs]), U(*[h for _, _, h, _ in arrs]),
                                             I(*[c for _, _, _, c in arrs]), nq, q, ctypes.byref(o),
                                             out.ctypes.data))
        return out[:n]

    def ssimulacra2_batch_device(self, ref_ptrs, dist_ptrs, widths, heights, channels, depths=None):
        """rcg_ssimulacra2_batch_device: device images, per-pair sizes; returns a float64 array of scores."""
        n = len(ref_ptrs)
        P = ctypes.c_void_p * max(n, 1)
        U = ctypes.c_uint32 * max(n, 1)
        I = ctypes.c_int32 * max(n, 1)
        out = np.zeros(max(n, 1), dtype=np.float64)
        dp = I(*depths) if depths is not None else None
        self._check(_lib.rcg_ssimulacra2_batch_device(self._ptr, n, P(*ref_ptrs), P(*dist_ptrs), U(*widths),
                                                      U(*heights), I(*channels), dp, out.ctypes.data))
        return out[:n]

    def ssimulacra2_device(self, ref_ptr, dist_ptr, width, height, channels):
        out = ctypes.c_double()
        self._check(_lib.rcg_ssimulacra2_device(self._ptr, ctypes.c_void_p(ref_ptr), ctypes.c_void_p(dist_ptr),
                                                width, height, channels, ctypes.byref(out)))
        return out.value

    def ssimulacra2_grad(self, reference, distorted, score_only=False):
        """(FP64 score, d score / d distorted) of an 8-bit RGB reference and a float RGB distorted image (values in
        [0, 255], taken as continuous); the gradient as a float64 (h, w, 3) array (None with score_only)."""
        a = np.ascontiguousarray(reference, dtype=np.uint8)
        d = np.ascontiguousarray(distorted, dtype=np.float32)
        if a.ndim != 3 or a.shape[2] != 3 or d.shape != a.shape:
            raise ValueError("the gradient takes an RGB reference and an RGB float image of the same shape")
        h, w = a.shape[:2]
        g = None if score_only else np.zeros((h, w, 3), np.float64)
        s = ctypes.c_double()
        self._check(_lib.rcg_ssimulacra2_grad(self._ptr, a.ctypes.data, d.ctypes.data, w, h, ctypes.byref(s),
                                              None if g is None else g.ctypes.data))
        return s.value, g

    def metric(self, metric, reference, candidate):
        """score(reference, candidate, metric) (cli/src/pipeline.rs:130): 8-bit images with 1..=4 channels."""
        a, w, h, c, d = _image(reference)
        b, w2, h2, c2, d2 = _image(candidate)
        if (w, h, c, d) != (w2, h2, c2, d2) or d != 8:
            raise RcgError(RCG_INVALID, "the metrics take two 8-bit images of the same shape")
        out = ctypes.c_double()
        self._check(_lib.rcg_metric_score(self._ptr, int(metric), a.ctypes.data, b.ctypes.data, w, h, c,
                                          ctypes.byref(out)))
        return out.value

    def ssim(self, reference, candidate):
        """core/src/metrics.rs:13."""
        return self.metric(METRIC_SSIM, reference, candidate)

    def psnr(self, reference, candidate):
        """core/src/metrics.rs:67."""
        return self.metric(METRIC_PSNR, reference, candidate)

    def ms_ssim(self, reference, candidate):
        """core/src/metrics.rs:111."""
        return self.metric(METRIC_MS_SSIM, reference, candidate)

    def metric_device(self, metric, ref_ptr, cand_ptr, width, height, channels):
        out = ctypes.c_double()
        self._check(_lib.rcg_metric_score_device(self._ptr, int(metric), ctypes.c_void_p(ref_ptr),
                                                 ctypes.c_void_p(cand_ptr), width, height, channels,
                                                 ctypes.byref(out)))
        return out.value

    def coef_layout(self, width, height, channels, opts):
        lay = _Layout()
        o = _opts(opts)
        rc = _lib.rcg_coef_layout_for(width, height, channels, ctypes.byref(o), ctypes.byref(lay))
        if rc != RCG_OK:
            raise RcgError(rc, "bad layout request")
        return lay

    def build_coefs(self, src, opts):
        """jpeg/src/encode.rs:426: quantized DCT coefficients of an 8-bit Gray/Rgb image."""
        a, w, h, c, d = _image(src)
        if d != 8 or c not in (1, 3):
            raise RcgError(RCG_INVALID, "build_coefs takes 8-bit Gray or Rgb")
        lay = self.coef_layout(w, h, c, opts)
        coefs = np.zeros(lay.ncoefs, dtype=np.int16)
        qt = np.zeros((2, 64), dtype=np.uint8)
        o = _opts(opts)
        self._check(_lib.rcg_build_coefs(self._ptr, a.ctypes.data, w, h, c, ctypes.byref(o), coefs.ctypes.data,
                                         coefs.size, qt.ctypes.data))
        return _coef_image(w, h, lay, coefs, qt)

    def build_coefs_weighted(self, src, opts, weights):
        """build_coefs with the trellis pass in the perceptual mode (`weights`: f32, the layout's ncoefs entries)."""
        a, w, h, c, d = _image(src)
        if d != 8 or c not in (1, 3):
            raise RcgError(RCG_INVALID, "build_coefs takes 8-bit Gray or Rgb")
        lay = self.coef_layout(w, h, c, opts)
        wt = np.ascontiguousarray(weights, dtype=np.float32)
        coefs = np.zeros(lay.ncoefs, dtype=np.int16)
        qt = np.zeros((2, 64), dtype=np.uint8)
        o = _opts(opts)
        self._check(_lib.rcg_build_coefs_weighted(self._ptr, a.ctypes.data, w, h, c, ctypes.byref(o),
                                                  wt.ctypes.data, wt.size, coefs.ctypes.data, coefs.size,
                                                  qt.ctypes.data))
        return _coef_image(w, h, lay, coefs, qt)

    def _pullback_args(self, reference, decoded, layout):
        a, w, h, c, d = _image(reference)
        b, w2, h2, c2, d2 = _image(decoded)
        if (w, h, c, d) != (w2, h2, c2, d2) or d != 8:
            raise RcgError(RCG_INVALID, "reference and decoded must be 8-bit images of the same shape")
        return a, b, w, h, c

    def coef_gradient(self, reference, decoded, layout):
        """(score, d score / d coefficient) of a decoded image for the coefficient layout `layout` (_Layout):
        float64, 64 zigzag entries per block, dequantized units."""
        a, b, w, h, c = self._pullback_args(reference, decoded, layout)
        out = np.zeros(layout.ncoefs, dtype=np.float64)
        s = ctypes.c_double()
        self._check(_lib.rcg_coef_gradient(self._ptr, a.ctypes.data, b.ctypes.data, w, h, c, ctypes.byref(layout),
                                           ctypes.byref(s), out.ctypes.data, out.size))
        return s.value, out

    def perceptual_weights(self, reference, decoded, layout, popts=None):
        """(score, perceptual trellis weights) from the gradient at `decoded` for the layout `layout`."""
        popts = popts or PerceptualOptions()
        a, b, w, h, c = self._pullback_args(reference, decoded, layout)
        out = np.zeros(layout.ncoefs, dtype=np.float32)
        s = ctypes.c_double()
        po = popts._c()
        self._check(_lib.rcg_perceptual_weights(self._ptr, a.ctypes.data, b.ctypes.data, w, h, c,
                                                ctypes.byref(layout), ctypes.byref(po), ctypes.byref(s),
                                                out.ctypes.data, out.size))
        return s.value, out

    def find_quality_weighted(self, reference, target, weights, max_quality=100, opts=None):
        """The --target-ssimulacra2 search with every candidate's trellis in the perceptual mode."""
        opts = opts or EncodeOptions()
        a, w, h, c, d = _image(reference)
        lay = self.coef_layout(w, h, c, EncodeOptions(50, opts.subsampling, opts.trellis))
        wt = np.ascontiguousarray(weights, dtype=np.float32)
        coefs = np.zeros(lay.ncoefs, dtype=np.int16)
        qt = np.zeros((2, 64), dtype=np.uint8)
        f = _Found()
        o = _opts(opts)
        self._check(_lib.rcg_search_weighted(self._ptr, a.ctypes.data, w, h, c, float(target), int(max_quality),
                                             ctypes.byref(o), wt.ctypes.data, wt.size, ctypes.byref(f),
                                             coefs.ctypes.data, coefs.size, qt.ctypes.data))
        trace = [(int(f.trace_q[i]), float(f.trace_score[i])) for i in range(f.nsteps)]
        return Found(int(f.quality), float(f.score), _coef_image(w, h, lay, coefs, qt), trace)

    def find_quality_perceptual(self, reference, target, max_quality=100, opts=None, popts=None, out=None,
                                weights_out=None, want_weights=True):
        """rcg_search_perceptual: plain search, gradient at its result, weighted search, planned sizes of both.
        `out`, `weights_out` and `want_weights` as in find_quality_perceptual_fast."""
        opts = opts or EncodeOptions()
        popts = popts or PerceptualOptions()
        a, w, h, c, d = _image(reference)
        lay = self.coef_layout(w, h, c, EncodeOptions(50, opts.subsampling, opts.trellis))
        coefs = _out_buffer(out, np.int16, lay.ncoefs)
        wts = _out_buffer(weights_out, np.float32, lay.ncoefs) if want_weights else None
        qt = np.zeros((2, 64), dtype=np.uint8)
        fp, ff = _Found(), _Found()
        sizes = (ctypes.c_uint64 * 2)()
        chose = ctypes.c_int()
        o, po = _opts(opts), popts._c()
        self._check(_lib.rcg_search_perceptual(self._ptr, a.ctypes.data, w, h, c, float(target), int(max_quality),
                                               ctypes.byref(o), ctypes.byref(po), ctypes.byref(fp),
                                               ctypes.byref(ff), sizes, ctypes.byref(chose), coefs.ctypes.data,
                                               coefs.size, qt.ctypes.data, wts.ctypes.data if wts is not None else None,
                                               wts.size if wts is not None else 0))

        def found(f, ci):
            return Found(int(f.quality), float(f.score), ci,
                         [(int(f.trace_q[i]), float(f.trace_score[i])) for i in range(f.nsteps)])

        return PerceptualFound(found(fp, None), found(ff, _coef_image(w, h, lay, coefs[: lay.ncoefs], qt)),
                               int(sizes[0]), int(sizes[1]), bool(chose.value),
                               wts[: lay.ncoefs] if wts is not None else None)

    def find_quality_perceptual_fast(self, reference, target, max_quality=100, opts=None, popts=None, out=None,
                                     weights_out=None, want_weights=True):
        """rcg_search_perceptual_fast: a four-candidate plain probe, the gradient at its best candidate, one
        weighted search. Returns (probe Found without coefficients, weighted Found, weights).

        `out` / `weights_out` (optional): reusable int16 / float32 arrays of at least coef_capacity() entries that
        receive the coefficients / weights (the returned Found and weights are views of them); want_weights=False
        passes no weights buffer (the library then copies none back) and returns None for them."""
        opts = opts or EncodeOptions()
        popts = popts or PerceptualOptions()
        a, w, h, c, d = _image(reference)
        lay = self.coef_layout(w, h, c, EncodeOptions(50, opts.subsampling, opts.trellis))

        coefs = _out_buffer(out, np.int16, lay.ncoefs)
        wts = _out_buffer(weights_out, np.float32, lay.ncoefs) if want_weights else None
        qt = np.zeros((2, 64), dtype=np.uint8)
        fp, ff = _Found(), _Found()
        o, po = _opts(opts), popts._c()
        self._check(_lib.rcg_search_perceptual_fast(self._ptr, a.ctypes.data, w, h, c, float(target),
                                                    int(max_quality), ctypes.byref(o), ctypes.byref(po),
                                                    ctypes.byref(fp), ctypes.byref(ff), coefs.ctypes.data, coefs.size,
                                                    qt.ctypes.data, wts.ctypes.data if wts is not None else None,
                                                    wts.size if wts is not None else 0))

        def found(f, ci):
            return Found(int(f.quality), float(f.score), ci,
                         [(int(f.trace_q[i]), float(f.trace_score[i])) for i in range(f.nsteps)])

        return (found(fp, None), found(ff, _coef_image(w, h, lay, coefs[: lay.ncoefs], qt)),
                wts[: lay.ncoefs] if wts is not None else None)

    def reconstruct(self, ci):
        """jpeg/src/decode.rs:334: the pixels a viewer would show (Gray (h, w) or Rgb (h, w, 3) uint8)."""
        lay = ci.layout()
        flat = np.ascontiguousarray(ci.flat())
        nc = len(ci.comps)
        out = np.zeros((ci.height, ci.width, nc), dtype=np.uint8)
        if ci.present is None:
            qt = np.ascontiguousarray(ci.qtables, dtype=np.uint8)
            self._check(_lib.rcg_reconstruct(self._ptr, ci.width, ci.height, ctypes.byref(lay), qt.ctypes.data,
                                             flat.ctypes.data, out.ctypes.data, out.size))
        else:
            t = ci.table_slots()
            self._check(_lib.rcg_reconstruct_tables(self._ptr, ci.width, ci.height, ctypes.byref(lay),
                                                    ctypes.byref(t), flat.ctypes.data, out.ctypes.data, out.size))
        return out[:, :, 0] if nc == 1 else out

    def decode_coefs(self, data):
        """jpeg::decode::parse(data)?.into_coefs() (jpeg/src/decode.rs:397, :540) of a sequential Huffman JPEG, with
        the entropy-coded data decoded on the GPU. Returns a CoefImage (general table form; component ids kept)."""
        buf = np.frombuffer(bytes(data), dtype=np.uint8)
        info, lay, t = _JpegInfo(), _Layout(), _QTables()
        self._check(_lib.rcg_decode_coefs(self._ptr, buf.ctypes.data, buf.size, ctypes.byref(info), ctypes.byref(lay),
                                          ctypes.byref(t), None, 0))
        coefs = np.empty(lay.ncoefs, dtype=np.int16)
        self._check(_lib.rcg_decode_coefs(self._ptr, buf.ctypes.data, buf.size, ctypes.byref(info), ctypes.byref(lay),
                                          ctypes.byref(t), coefs.ctypes.data, coefs.size))
        self.last_decode_rounds = int(info.sync_rounds)
        comps, off = [], 0
        for i in range(lay.ncomp):
            n = lay.blocks_w[i] * lay.blocks_h[i] * 64
            comps.append(CoefComponent(int(info.ids[i]), lay.h[i], lay.v[i], int(t.tq[i]), lay.blocks_w[i],
                                       lay.blocks_h[i], coefs[off: off + n]))
            off += n
        q4 = np.array([list(t.qtables[sl]) for sl in range(4)], dtype=np.uint8)
        present = np.array([int(t.present[sl]) for sl in range(4)], dtype=np.uint8)
        return CoefImage(int(info.width), int(info.height), comps, q4, present)

    def decode_coefs_device(self, data, coefs_ptr, coefs_len):
        """rcg_decode_coefs_device: decode into device memory; returns (width, height, layout, tables, ids)."""
        buf = np.frombuffer(bytes(data), dtype=np.uint8)
        info, lay, t = _JpegInfo(), _Layout(), _QTables()
        self._check(_lib.rcg_decode_coefs_device(self._ptr, buf.ctypes.data, buf.size, ctypes.byref(info),
                                                 ctypes.byref(lay), ctypes.byref(t), ctypes.c_void_p(coefs_ptr),
                                                 coefs_len))
        self.last_decode_rounds = int(info.sync_rounds)
        return int(info.width), int(info.height), lay, t, bytes(info.ids[: lay.ncomp])

    def search_requantize_device(self, width, height, layout, tables, src_ptr, out_ptr, coefs_len, target,
                                 max_quality=100, trellis=True, metric=METRIC_SSIMULACRA2):
        """rcg_search_requantize_device: (quality, score, trace, output tables)."""
        f, t_out = _Found(), _QTables()
        self._check(_lib.rcg_search_requantize_device(self._ptr, width, height, ctypes.byref(layout),
                                                      ctypes.byref(tables), ctypes.c_void_p(src_ptr), int(metric),
                                                      float(target), int(max_quality), 1 if trellis else 0,
                                                      ctypes.byref(f), ctypes.c_void_p(out_ptr), coefs_len,
                                                      ctypes.byref(t_out)))
        trace = [(int(f.trace_q[i]), float(f.trace_score[i])) for i in range(f.nsteps)]
        return int(f.quality), float(f.score), trace, t_out

    def plan(self, ci):
        """write_best's plan of a CoefImage (jpeg/src/encode.rs:543-565): statistics, costs and choice on the GPU."""
        lay = ci.layout()
        flat = np.ascontiguousarray(ci.flat())
        r = _PlanResult()
        self._check(_lib.rcg_plan(self._ptr, ci.width, ci.height, ctypes.byref(lay), flat.ctypes.data, flat.size,
                                  ctypes.byref(r)))
        return _plan(r)

    def plan_device(self, width, height, layout, coefs_ptr):
        """rcg_plan_device: coefficients already on the device (layout: the _Layout of coef_layout())."""
        r = _PlanResult()
        self._check(_lib.rcg_plan_device(self._ptr, width, height, ctypes.byref(layout), ctypes.c_void_p(coefs_ptr),
                                         ctypes.byref(r)))
        return _plan(r)

    def requantize(self, ci, quality, trellis=True):
        """CoefImage::requantize (jpeg/src/encode.rs:111) of a copy of `ci`; returns the new CoefImage."""
        lay = ci.layout()
        flat = np.ascontiguousarray(ci.flat())
        out = np.empty_like(flat)
        t_in, t_out = ci.table_slots(), _QTables()
        self._check(_lib.rcg_requantize(self._ptr, ci.width, ci.height, ctypes.byref(lay), ctypes.byref(t_in),
                                        flat.ctypes.data, int(quality), 1 if trellis else 0, out.ctypes.data,
                                        out.size, ctypes.byref(t_out)))
        return _general_image(ci, out, t_out)

    def find_quality_requantize(self, ci, target, max_quality=100, trellis=True, metric=METRIC_SSIMULACRA2):
        """The JPEG -> JPEG --target-ssimulacra2 search (cli/src/pipeline.rs:369-386) over requantizations of `ci`."""
        lay = ci.layout()
        flat = np.ascontiguousarray(ci.flat())
        out = np.empty_like(flat)
        t_in, t_out = ci.table_slots(), _QTables()
        f = _Found()
        self._check(_lib.rcg_search_requantize(self._ptr, ci.width, ci.height, ctypes.byref(lay),
                                               ctypes.byref(t_in), flat.ctypes.data, int(metric), float(target),
                                               int(max_quality), 1 if trellis else 0, ctypes.byref(f),
                                               out.ctypes.data, out.size, ctypes.byref(t_out)))
        trace = [(int(f.trace_q[i]), float(f.trace_score[i])) for i in range(f.nsteps)]
        return Found(int(f.quality), float(f.score), _general_image(ci, out, t_out), trace)

    def coef_capacity(self, width, height, channels, opts):
        """int16 count that holds the search result for any quality (Auto switches layout at quality 90)."""
        return max(self.coef_layout(width, height, channels, EncodeOptions(q, opts.subsampling, opts.trellis)).ncoefs
                   for q in (1, 89, 90, 100))

    def find_quality_ssimulacra2(self, reference, target, max_quality=100, opts=None, out=None):
        """The --target-ssimulacra2 search (jpeg/src/target.rs:29 with cli/src/pipeline.rs:207-222), on device.

        `out` (optional): a reusable int16 array of at least coef_capacity() entries; the returned coefficients are
        views into it (valid until it is reused), which spares a fresh allocation per call."""
        return self._find_quality(reference, target, max_quality, opts, out, METRIC_SSIMULACRA2)

    def find_quality(self, reference, target, max_quality=100, opts=None, out=None):
        """The --target-ssim search (jpeg/src/target.rs:24, cli/src/pipeline.rs:213), on device."""
        return self._find_quality(reference, target, max_quality, opts, out, METRIC_SSIM)

    def _find_quality(self, reference, target, max_quality, opts, out, metric):
        opts = opts or EncodeOptions()
        a, w, h, c, d = _image(reference)
        if d != 8 or c not in (1, 3):
            raise RcgError(RCG_INVALID, "the search takes 8-bit Gray or Rgb")
        cap = self.coef_capacity(w, h, c, opts)
        if out is None:
            coefs = np.empty(cap, dtype=np.int16)
        else:
            if out.dtype != np.int16 or out.size < cap or not out.flags.c_contiguous:
                raise ValueError(f"out must be a contiguous int16 array of at least {cap} entries")
            coefs = out
        qt = np.zeros((2, 64), dtype=np.uint8)
        f = _Found()
        o = _opts(opts)
        self._check(_lib.rcg_search_metric(self._ptr, a.ctypes.data, w, h, c, int(metric), float(target),
                                           int(max_quality), ctypes.byref(o), ctypes.byref(f), coefs.ctypes.data,
                                           coefs.size, qt.ctypes.data))
        lay = self.coef_layout(w, h, c, EncodeOptions(f.quality, opts.subsampling, opts.trellis))
        ci = _coef_image(w, h, lay, coefs[: lay.ncoefs], qt)
        trace = [(int(f.trace_q[i]), float(f.trace_score[i])) for i in range(f.nsteps)]
        return Found(int(f.quality), float(f.score), ci, trace)

    def search_batch(self, images, targets, max_quality=100, opts=None, parallel=0, lockstep=False):
        """Independent searches over many images at once (rcg_search_batch on `parallel` worker streams, or with
        lockstep rcg_search_batch_lockstep: every step of every image in one work-list launch per stage); same
        results as one search each."""
        opts = opts or EncodeOptions()
        n = len(images)
        arrs = [_image(im) for im in images]
        for a, w, h, c, d in arrs:
            if d != 8 or c not in (1, 3):
                raise RcgError(RCG_INVALID, "the search takes 8-bit Gray or Rgb")
        srcs = (ctypes.c_void_p * n)(*[a.ctypes.data for a, *_ in arrs])
        ws = (ctypes.c_uint32 * n)(*[w for _, w, _, _, _ in arrs])
        hs = (ctypes.c_uint32 * n)(*[h for _, _, h, _, _ in arrs])
        cs = (ctypes.c_int * n)(*[c for _, _, _, c, _ in arrs])
        ts = (ctypes.c_double * n)(*[float(t) for t in targets])
        found = (_Found * n)()
        coefs, caps, qts = [], [], []
        for a, w, h, c, _ in arrs:
            cap = max(self.coef_layout(w, h, c, EncodeOptions(q, opts.subsampling, opts.trellis)).ncoefs
                      for q in (1, 89, 90, 100))
            coefs.append(np.zeros(cap, dtype=np.int16))
            caps.append(cap)
            qts.append(np.zeros((2, 64), dtype=np.uint8))
        cptr = (ctypes.c_void_p * n)(*[x.ctypes.data for x in coefs])
        clen = (ctypes.c_size_t * n)(*caps)
        qptr = (ctypes.c_void_p * n)(*[x.ctypes.data for x in qts])
        o = _opts(opts)
        if lockstep:
            self._check(_lib.rcg_search_batch_lockstep(self._ptr, n, srcs, ws, hs, cs, ts, int(max_quality),
                                                       ctypes.byref(o), found, cptr, clen, qptr))
        else:
            self._check(_lib.rcg_search_batch(self._ptr, n, srcs, ws, hs, cs, ts, int(max_quality), ctypes.byref(o),
                                              int(parallel), found, cptr, clen, qptr))
        out = []
        for i, (a, w, h, c, _) in enumerate(arrs):
            f = found[i]
            lay = self.coef_layout(w, h, c, EncodeOptions(f.quality, opts.subsampling, opts.trellis))
            ci = _coef_image(w, h, lay, coefs[i][: lay.ncoefs], qts[i])  # each image has its own buffer
            trace = [(int(f.trace_q[k]), float(f.trace_score[k])) for k in range(f.nsteps)]
            out.append(Found(int(f.quality), float(f.score), ci, trace))
        return out

    def search_device(self, src_ptr, width, height, channels, target, max_quality, opts, coefs_ptr=0,
                      coefs_len=0, qt_ptr=0):
        """rcg_search_device: image and outputs already on the device; returns (quality, score, trace)."""
        f = _Found()
        o = _opts(opts)
        self._check(_lib.rcg_search_device(self._ptr, ctypes.c_void_p(src_ptr), width, height, channels,
                                           float(target), int(max_quality), ctypes.byref(o), ctypes.byref(f),
                                           ctypes.c_void_p(coefs_ptr or 0), coefs_len, ctypes.c_void_p(qt_ptr or 0)))
        trace = [(int(f.trace_q[i]), float(f.trace_score[i])) for i in range(f.nsteps)]
        return int(f.quality), float(f.score), trace


def _coef_image(w, h, lay, coefs, qt):
    comps = []
    off = 0
    for i in range(lay.ncomp):
        n = lay.blocks_w[i] * lay.blocks_h[i] * 64
        comps.append(CoefComponent(i + 1, lay.h[i], lay.v[i], min(i, 1), lay.blocks_w[i], lay.blocks_h[i],
                                   coefs[off: off + n]))
        off += n
    return CoefImage(w, h, comps, qt if lay.ncomp > 1 else qt[:1].repeat(2, axis=0))


def _general_image(src, flat, t):
    """A CoefImage shaped like `src` holding `flat` with the table assignment `t` (general form)."""
    comps = []
    off = 0
    for i, c in enumerate(src.comps):
        n = c.coefs.size
        comps.append(CoefComponent(c.id, c.h, c.v, int(t.tq[i]), c.blocks_w, c.blocks_h, flat[off: off + n]))
        off += n
    q4 = np.array([list(t.qtables[sl]) for sl in range(4)], dtype=np.uint8)
    present = np.array([int(t.present[sl]) for sl in range(4)], dtype=np.uint8)
    return CoefImage(src.width, src.height, comps, q4, present)


_default = None


def default_context():
    global _default
    if _default is None:
        _default = Context(0)
    return _default


def ssimulacra2(reference, distorted):
    return default_context().ssimulacra2(reference, distorted)


def build_coefs(src, opts):
    return default_context().build_coefs(src, opts)


def reconstruct(ci):
    return default_context().reconstruct(ci)


def find_quality_ssimulacra2(reference, target, max_quality=100, opts=None):
    return default_context().find_quality_ssimulacra2(reference, target, max_quality, opts)
