"""The allocation-free scorer entry point against the allocating one, through the C ABI.

rcg_ssimulacra2_device_noalloc serves callers that cannot let a library call cudaMalloc (a host whose caching
allocator owns a fixed device budget, or a latency-critical loop where cudaMalloc/cudaFree would synchronize the
whole device). It keeps its scratch in one fixed array inside the library, so this file runs last: if it fails, a run
that stops at the first failure has already run every other test. It must pass on its own in a fresh process too,
which is why each test sets up what it needs (the entry point configures the device on its first call).
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PIXELS = 512 * 512


def _noalloc():
    import rcg

    return rcg.lib().rcg_ssimulacra2_device_noalloc


def _pair(w, h, seed, channels=3):
    import rcg.synth as synth

    ref = synth.image(w, h, seed)
    dist = synth.image(w, h, seed, sensor_sigma=5.0)
    if channels == 1:
        ref, dist = np.ascontiguousarray(ref[:, :, 1]), np.ascontiguousarray(dist[:, :, 1])
    return ref, dist


def test_noalloc_matches_the_allocating_entry_point_on_two_calls_in_a_row():
    import torch

    import rcg

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    ctx = rcg.Context(0)
    f = _noalloc()
    stream = torch.cuda.current_stream(dev)
    # Two calls in a row on different inputs (the second one overwrites the first one's scratch).
    for (w, h, seed, ch) in [(320, 240, 21, 3), (512, 512, 22, 3), (300, 200, 23, 1)]:
        ref, dist = _pair(w, h, seed, ch)
        d_ref = torch.from_numpy(ref).to(dev)
        d_dist = torch.from_numpy(dist).to(dev)
        d_score = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = f(ctypes.c_void_p(d_ref.data_ptr()), ctypes.c_void_p(d_dist.data_ptr()), w, h, ch,
               ctypes.c_void_p(d_score.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == rcg.RCG_OK
        torch.cuda.synchronize()
        got = float(d_score.item())
        want = ctx.ssimulacra2_device(d_ref.data_ptr(), d_dist.data_ptr(), w, h, ch)
        # the same kernels in the same order on the same inputs: the same bits
        assert got == want, (w, h, got, want)
    # Identical images still score exactly 100 after the scratch held another pair.
    d_score = torch.zeros(1, dtype=torch.float64, device=dev)
    rc = f(ctypes.c_void_p(d_ref.data_ptr()), ctypes.c_void_p(d_ref.data_ptr()), w, h, ch,
           ctypes.c_void_p(d_score.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == rcg.RCG_OK
    torch.cuda.synchronize()
    assert float(d_score.item()) == 100.0
    ctx.close()


def test_noalloc_rejects_what_it_cannot_hold():
    import torch

    import rcg

    dev = torch.device("cuda", 0)
    f = _noalloc()
    big = torch.zeros(1024 * 1024 * 3, dtype=torch.uint8, device=dev)
    d_score = torch.zeros(1, dtype=torch.float64, device=dev)
    p = ctypes.c_void_p(big.data_ptr())
    s = ctypes.c_void_p(d_score.data_ptr())
    assert f(p, p, 513, 512, 3, s, None) == rcg.RCG_INVALID  # over the pixel limit
    assert f(p, p, 7, 100, 3, s, None) == rcg.RCG_INVALID  # sides < 8
    assert f(p, p, 64, 64, 4, s, None) == rcg.RCG_INVALID  # only Gray or Rgb
    assert f(None, p, 64, 64, 3, s, None) == rcg.RCG_INVALID
    assert f(p, p, 512, 512, 3, s, None) == rcg.RCG_OK  # exactly at the limit
    torch.cuda.synchronize()
    assert float(d_score.item()) == 100.0


def test_noalloc_allocates_nothing_after_set_up():
    """After the first call on a device has set it up, a call at a size this process has not scored yet leaves the
    device's free memory unchanged (every buffer the call needs is the fixed array)."""
    import torch

    import rcg

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    f = _noalloc()
    stream = torch.cuda.current_stream(dev)
    ref, dist = _pair(64, 64, 30)
    d_ref, d_dist = torch.from_numpy(ref).to(dev), torch.from_numpy(dist).to(dev)
    d_score = torch.zeros(1, dtype=torch.float64, device=dev)
    args = (ctypes.c_void_p(d_score.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert f(ctypes.c_void_p(d_ref.data_ptr()), ctypes.c_void_p(d_dist.data_ptr()), 64, 64, 3, *args) == rcg.RCG_OK
    torch.cuda.synchronize()
    ref2, dist2 = _pair(411, 333, 31)  # a size no other test here scores
    e_ref, e_dist = torch.from_numpy(ref2).to(dev), torch.from_numpy(dist2).to(dev)
    torch.cuda.synchronize()
    unchanged = False
    for _ in range(3):  # the free figure is device-wide: retry once or twice should anything else move it
        free0 = torch.cuda.mem_get_info(0)[0]
        rc = f(ctypes.c_void_p(e_ref.data_ptr()), ctypes.c_void_p(e_dist.data_ptr()), 411, 333, 3, *args)
        assert rc == rcg.RCG_OK
        torch.cuda.synchronize()
        if torch.cuda.mem_get_info(0)[0] == free0:
            unchanged = True
            break
    assert unchanged, "device free memory changed across an allocation-free call"
    assert np.isfinite(float(d_score.item()))
