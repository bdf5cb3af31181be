"""The SSIMULACRA2 adjoint on the GPU (FP64): d score / d distorted RGB samples.

A 1024x1024 image: the GPU gradient against the FP64 CPU reference gradient at every sample, and against FP64 central
differences (h = 1e-3, the perturbed samples as the f32 values actually used) at 256 random samples. The
differences come from the central difference's own truncation and rounding error, so the bound is relative with an
absolute floor far below the gradient's typical size.
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu


def _pair(oracle, w, h, seed, q=50):
    """The reference and its decoded JPEG as float samples, nudged by a seeded +-0.25: where a decoded region equals
    the reference exactly (flat areas), the edge maps sit on the kink of |.| and the derivative is one-sided, picked
    by rounding; the nudge keeps the comparison to points where the score is differentiable."""
    ref = synth.image(w, h, seed)
    coefs, qt, lay = oracle.build_coefs(ref, q, 3, True)
    dist = oracle.reconstruct(w, h, lay, qt, coefs).astype(np.float32)
    rng = np.random.default_rng(seed)
    dist = np.clip(dist + rng.uniform(-0.25, 0.25, dist.shape).astype(np.float32), 0.0, 255.0).astype(np.float32)
    return ref, dist


def test_gradient_matches_the_fp64_cpu_gradient(ctx, oracle):
    ref, dist = _pair(oracle, 1024, 1024, 80)
    d32 = dist
    s_gpu, g_gpu = ctx.ssimulacra2_grad(ref, d32)
    s_cpu, g_cpu = oracle.grad64(ref.astype(np.float64), d32.astype(np.float64))
    assert abs(s_gpu - s_cpu) < 1e-9
    # on integer samples the continuous score is the FP64 scorer
    d8 = np.rint(dist).astype(np.uint8)
    assert abs(ctx.ssimulacra2_grad(ref, d8.astype(np.float32), score_only=True)[0] -
               oracle.ssimulacra2(ref, d8, fp64=True)) < 1e-9
    # Everywhere but at the samples whose maps sit on a kink of max(., 0) or |.| (a 1e-16 rounding difference picks
    # the other one-sided derivative there) the two FP64 gradients agree to rounding.
    scale = np.abs(g_cpu).max()
    err = np.abs(g_gpu - g_cpu)
    off = err > 1e-12 * scale + 1e-9 * np.abs(g_cpu)
    print(f"max |grad| {scale:.3e}, max |gpu - cpu| {err.max():.3e}, off the rounding bound: {off.sum()} of {off.size}")
    assert off.mean() <= 1e-5
    assert err.max() <= 1e-6 * scale


def test_gradient_matches_central_differences(ctx, oracle):
    ref, dist = _pair(oracle, 1024, 1024, 81)
    d32 = dist
    _, g = ctx.ssimulacra2_grad(ref, d32)
    rng = np.random.default_rng(4)
    h = 1e-3
    worst = 0.0
    for _ in range(256):
        y, x, c = int(rng.integers(0, 1024)), int(rng.integers(0, 1024)), int(rng.integers(0, 3))
        dp, dm = d32.copy(), d32.copy()
        dp[y, x, c] = np.float32(d32[y, x, c] + h)
        dm[y, x, c] = np.float32(d32[y, x, c] - h)
        sp, _ = ctx.ssimulacra2_grad(ref, dp, score_only=True)
        sm, _ = ctx.ssimulacra2_grad(ref, dm, score_only=True)
        fd = (sp - sm) / (float(dp[y, x, c]) - float(dm[y, x, c]))
        worst = max(worst, abs(fd - g[y, x, c]) / (abs(fd) + 1e-7))
        assert abs(fd - g[y, x, c]) <= 1e-8 + 2e-3 * abs(fd), (y, x, c, fd, g[y, x, c])
    print(f"worst relative difference {worst:.2e}")


def test_gradient_of_identical_images_and_small_sizes(ctx, oracle):
    ref = synth.image(64, 48, 82)
    s, g = ctx.ssimulacra2_grad(ref, ref.astype(np.float32))
    assert s == 100.0 and not np.any(g)  # the maximum: every map is zero, the final mapping is constant
    for w, h in ((8, 8), (9, 13), (37, 21)):
        ref, dist = _pair(oracle, w, h, 83, q=30)
        d32 = dist
        s_gpu, g_gpu = ctx.ssimulacra2_grad(ref, d32)
        s_cpu, g_cpu = oracle.grad64(ref.astype(np.float64), d32.astype(np.float64))
        assert abs(s_gpu - s_cpu) < 1e-9
        assert np.abs(g_gpu - g_cpu).max() <= 1e-5 * max(np.abs(g_cpu).max(), 1e-30)
    with pytest.raises(rcg.RcgError):
        ctx.ssimulacra2_grad(ref[:7], d32[:7])
