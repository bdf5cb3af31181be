"""SSIM, PSNR and MS-SSIM on the GPU (core/src/metrics.rs) and the `--target-ssim` searches, against the oracle.

The window sums are exact integers and the per-window formula runs in f64 with the reference's operations, so SSIM
matches the oracle to rounding of the final additions (asserted at 1e-12); PSNR's squared-error sum is exact;
MS-SSIM combines five such SSIMs with pow (1e-12). The searches must visit the same qualities, pick the same
candidate and return the same coefficients as the oracle's searches with SSIM as the metric.
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _pair(w, h, ch, seed, sigma=6.0):
    a = synth.image(max(w, 8), max(h, 8), seed)[:h, :w]
    b = synth.image(max(w, 8), max(h, 8), seed, sensor_sigma=sigma)[:h, :w]
    if ch == 1:
        return a[:, :, 0].copy(), b[:, :, 0].copy()
    if ch == 2:
        return a[:, :, :2].copy(), b[:, :, :2].copy()
    if ch == 4:
        return np.concatenate([a, a[:, :, :1]], 2), np.concatenate([b, b[:, :, 2:3]], 2)
    return a.copy(), b.copy()


@pytest.mark.parametrize("w,h", [(1, 1), (3, 2), (7, 30), (8, 8), (9, 13), (64, 9), (257, 255), (1000, 777),
                                 (4100, 12)])
@pytest.mark.parametrize("ch", [1, 2, 3, 4])
def test_ssim_and_psnr_match_the_oracle(ctx, oracle, w, h, ch):
    a, b = _pair(w, h, ch, 50 + w % 7)
    got, want = ctx.ssim(a, b), oracle.ssim(a, b)
    assert abs(got - want) <= TOL, (got, want)
    assert ctx.ssim(a, a) == oracle.ssim(a, a)
    got, want = ctx.psnr(a, b), oracle.psnr(a, b)
    assert got == want or abs(got - want) <= TOL * abs(want)
    assert ctx.psnr(a, a) == float("inf")


@pytest.mark.parametrize("w,h,ch", [(64, 64, 1), (333, 217, 3), (1920, 1080, 3), (20, 12, 4), (5, 40, 2),
                                    (31, 31, 3)])
def test_ms_ssim_matches_the_oracle(ctx, oracle, w, h, ch):
    a, b = _pair(w, h, ch, 60)
    got = ctx.ms_ssim(a, b)
    want = oracle.ms_ssim(a, b)
    assert abs(got - want) <= TOL, (got, want)
    assert abs(ctx.ms_ssim(a, a) - 1.0) <= TOL


def test_reference_metric_properties(ctx):
    """core/src/metrics.rs:141-175, through the GPU."""

    def img(w, h, f):
        y, x = np.mgrid[0:h, 0:w]
        return f(x, y).astype(np.uint8)

    a = img(40, 33, lambda x, y: x * 5 + y * 3)
    assert abs(ctx.ssim(a, a) - 1.0) < 1e-12
    a = img(64, 64, lambda x, y: (x * 7 + y * 5) % 256)
    s, hv = ctx.ssim(a, a // 8 * 8), ctx.ssim(a, a // 64 * 64)
    assert s > hv and s < 1.0 and hv > -1.0
    t = img(3, 2, lambda x, y: x + y)
    assert ctx.ssim(t, t) > 0.99
    a = img(32, 32, lambda x, y: (x * 3 + y * 5) % 256)
    p = ctx.psnr(a, (a + 8).astype(np.uint8))
    assert 20.0 < p < 40.0
    a = img(64, 64, lambda x, y: (x * 7 + y * 11) % 256)
    assert ctx.ms_ssim(a, a) > 0.99 and ctx.ms_ssim(a, a // 16 * 16) < ctx.ms_ssim(a, a)


def test_ssimulacra2_through_the_metric_entry_point(ctx, oracle):
    a, b = _pair(120, 90, 3, 61)
    assert ctx.metric(rcg.METRIC_SSIMULACRA2, a, b) == ctx.ssimulacra2(a, b)
    with pytest.raises(rcg.RcgError):
        ctx.metric(rcg.METRIC_SSIMULACRA2, a[:7], b[:7])
    with pytest.raises(rcg.RcgError):
        ctx.metric(9, a, b)


@pytest.mark.parametrize("target,sub,trellis", [(0.9, rcg.Subsampling.S420, True), (0.97, rcg.Subsampling.Auto, True),
                                                (0.8, rcg.Subsampling.S444, False), (0.999, rcg.Subsampling.S420, True),
                                                (0.2, rcg.Subsampling.S422, True)])
def test_target_ssim_search_matches_the_oracle(ctx, oracle, target, sub, trellis):
    img = synth.image(300, 200, 62, sensor_sigma=3.0)
    opts = rcg.EncodeOptions(90, sub, trellis)
    f = ctx.find_quality(img, target, 100, opts)
    q, s, coefs, qt, lay, trace = oracle.search(img, target, 100, int(sub), trellis, metric=oracle.METRIC_SSIM)
    assert [t[0] for t in f.trace] == [t[0] for t in trace]
    for (_, x), (_, y) in zip(f.trace, trace):
        assert abs(x - y) <= TOL
    assert f.quality == q and abs(f.score - s) <= TOL
    assert np.array_equal(f.coefs.flat(), coefs)


def test_target_ssim_search_gray_and_tiny(ctx, oracle):
    for w, h in ((96, 64), (5, 5), (3, 40)):
        img = synth.image(max(w, 8), max(h, 8), 63, sensor_sigma=4.0)[:h, :w, 1].copy()
        opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
        f = ctx.find_quality(img, 0.95, 100, opts)
        q, s, coefs, qt, lay, trace = oracle.search(img, 0.95, 100, 3, True, metric=oracle.METRIC_SSIM)
        assert [t[0] for t in f.trace] == [t[0] for t in trace], (w, h)
        assert f.quality == q and abs(f.score - s) <= TOL
        assert np.array_equal(f.coefs.flat(), coefs)
    # below 8x8 only SSIMULACRA2 refuses
    with pytest.raises(rcg.RcgError) as e:
        ctx.find_quality_ssimulacra2(synth.image(8, 8, 64)[:5, :5].copy(), 70.0)
    assert e.value.status == rcg.RCG_UNSUPPORTED


def test_requantize_search_with_ssim(ctx, oracle):
    from test_gpu_requantize import _source, _to_oracle, _assert_same

    img = synth.image(320, 213, 65, sensor_sigma=3.0)
    src, lay = _source(oracle, img, 95, rcg.Subsampling.S420)
    f = ctx.find_quality_requantize(src, 0.93, 100, True, metric=rcg.METRIC_SSIM)
    q, s, g, trace = oracle.search_requantize(_to_oracle(oracle, src, lay), 0.93, 100, True,
                                              metric=oracle.METRIC_SSIM)
    assert [t[0] for t in f.trace] == [t[0] for t in trace]
    assert f.quality == q and abs(f.score - s) <= TOL
    _assert_same(f.coefs, g, "ssim requantize search")
