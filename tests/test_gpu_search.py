"""The device-driven --target-ssimulacra2 search against the oracle's find_quality_with.

Per step the GPU and the oracle encode the same coefficients (bit-exact) and score them within 1e-3; a candidate
whose fast score lands within 1e-3 of the target is decided on its reference-order FP64 score (within 1e-9 of the
oracle's), so the bisection takes the oracle's path in every case. The chosen coefficients must be bit-exact with the
oracle's, and the bitstream written from them (the oracle's write_best, standing in for the Rust host's entropy
coder) byte-identical.
"""

import hashlib

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu


def _compare(ctx, oracle, img, target, sub, trellis=True, max_q=100):
    h, w = img.shape[:2]
    f = ctx.find_quality_ssimulacra2(img, target, max_q, rcg.EncodeOptions(90, sub, trellis))
    q, s, coefs, qt, lay, trace = oracle.search(img, target, max_q, int(sub), trellis)
    assert [t[0] for t in f.trace] == [t[0] for t in trace], (f.trace, trace)
    for (gq, gs), (oq, os_) in zip(f.trace, trace):
        assert abs(gs - os_) <= 1e-3, (gq, gs, os_)
    assert f.quality == q
    assert abs(f.score - s) <= 1e-3
    assert np.array_equal(f.coefs.flat(), coefs)
    a, _ = oracle.write_best(w, h, lay, f.coefs.qtables, f.coefs.flat())
    b, _ = oracle.write_best(w, h, lay, qt, coefs)
    assert hashlib.sha256(a).hexdigest() == hashlib.sha256(b).hexdigest()
    return f


@pytest.mark.parametrize("target", [50.0, 70.0, 85.0])
def test_search_matches_oracle_420(ctx, oracle, target):
    img = synth.image(512, 512, 0)
    _compare(ctx, oracle, img, target, rcg.Subsampling.S420)


def test_search_auto_subsampling_switches_layout(ctx, oracle):
    img = synth.image(300, 200, 2, sensor_sigma=3.0)
    f = _compare(ctx, oracle, img, 80.0, rcg.Subsampling.Auto)
    assert f.trace[0][0] == 100


@pytest.mark.parametrize("sub", [rcg.Subsampling.S444, rcg.Subsampling.S422])
def test_search_other_layouts(ctx, oracle, sub):
    _compare(ctx, oracle, synth.image(257, 129, 3), 75.0, sub)


def test_search_without_trellis_and_gray(ctx, oracle):
    img = synth.image(200, 160, 4)
    _compare(ctx, oracle, img, 65.0, rcg.Subsampling.S420, trellis=False)
    _compare(ctx, oracle, np.ascontiguousarray(img[:, :, 0]), 65.0, rcg.Subsampling.S420)


def test_unreachable_target_returns_max_quality(ctx, oracle):
    img = synth.image(96, 96, 5, sensor_sigma=8.0)
    f = ctx.find_quality_ssimulacra2(img, 99.9, 100, rcg.EncodeOptions(90, rcg.Subsampling.S420, True))
    assert f.quality == 100 and len(f.trace) == 1 and f.score < 99.9


def test_trivial_target_reaches_quality_1(ctx, oracle):
    img = synth.image(96, 96, 6)
    f = _compare(ctx, oracle, img, -1000.0, rcg.Subsampling.S420)
    assert f.quality == 1


def test_max_quality_below_100(ctx, oracle):
    img = synth.image(120, 90, 7)
    _compare(ctx, oracle, img, 60.0, rcg.Subsampling.S420, max_q=63)


def test_search_rejects_small_images(ctx):
    with pytest.raises(rcg.RcgError) as e:
        ctx.find_quality_ssimulacra2(np.zeros((7, 30, 3), np.uint8), 70.0)
    assert e.value.status == rcg.RCG_UNSUPPORTED


def test_repeated_searches_agree(ctx):
    img = synth.image(640, 480, 8, sensor_sigma=3.0)
    a = ctx.find_quality_ssimulacra2(img, 70.0)
    b = ctx.find_quality_ssimulacra2(img, 70.0)
    assert a.trace == b.trace and np.array_equal(a.coefs.flat(), b.coefs.flat())


@pytest.mark.parametrize("w,h", [(8, 8), (9, 13), (17, 33), (64, 48), (257, 9), (64, 33), (132, 67)])
def test_search_tiny_and_awkward_sizes(ctx, oracle, w, h):
    """Every column of these images is near the zero left/right border at some scale: the split scorer's border
    corrections and the per-scale tiling are exercised on each candidate. Widths that are a multiple of 4 take the
    fused upsampling + pyramid kernel (odd heights: a last chroma row with one output row; edge tiles)."""
    img = synth.image(max(w, 16), max(h, 16), 9, sensor_sigma=4.0)[:h, :w].copy()
    _compare(ctx, oracle, img, 60.0, rcg.Subsampling.S420)


def test_batch_matches_individual_searches(ctx):
    """rcg_search_batch (concurrent searches on worker streams) gives exactly each image's own search result."""
    sizes = [(96, 80), (300, 200), (640, 480), (17, 33), (1000, 700), (64, 64), (333, 111)]
    imgs = [synth.image(w, h, 20 + i, sensor_sigma=2.0) for i, (w, h) in enumerate(sizes)]
    imgs[5] = np.ascontiguousarray(imgs[5][:, :, 0])  # a gray image in the mix
    targets = [60.0, 70.0, 80.0, 65.0, 75.0, 55.0, 72.0]
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    for parallel in (1, 3, 8):
        res = ctx.search_batch(imgs, targets, 100, opts, parallel=parallel)
        for im, t, r in zip(imgs, targets, res):
            f = ctx.find_quality_ssimulacra2(im, t, 100, opts)
            assert r.quality == f.quality and r.trace == f.trace
            assert np.array_equal(r.coefs.flat(), f.coefs.flat())


def test_batch_reports_the_failing_image(ctx):
    imgs = [synth.image(64, 64, 1), np.zeros((4, 40, 3), np.uint8), synth.image(80, 64, 2)]
    with pytest.raises(rcg.RcgError) as e:
        ctx.search_batch(imgs, [60.0, 60.0, 60.0], 100, rcg.EncodeOptions(90, rcg.Subsampling.S420, True), 2)
    assert e.value.status == rcg.RCG_UNSUPPORTED and "image 1" in e.value.message


def test_batch_at_the_large_end_of_the_image_set(ctx, oracle):
    """The four largest images of the 64-image set (seeds 2..65, log-uniform 640x480..6000x4000, targets U(55,85))
    through rcg_search_batch, each against the oracle's search: same path, coefficients and file."""
    sizes = synth.log_uniform_sizes(2, 64)
    targets = [55.0 + 30.0 * u for u in synth.uniforms(2, 40, 64)]
    largest = sorted(range(64), key=lambda i: sizes[i][0] * sizes[i][1])[-4:]
    imgs = [synth.image(sizes[i][0], sizes[i][1], 2 + i) for i in largest]
    tgts = [targets[i] for i in largest]
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    res = ctx.search_batch(imgs, tgts, 100, opts, parallel=4)
    for img, t, r in zip(imgs, tgts, res):
        h, w = img.shape[:2]
        q, s, coefs, qt, lay, trace = oracle.search(img, t, 100, 3, True)
        assert [x[0] for x in r.trace] == [x[0] for x in trace], (w, h, r.trace, trace)
        assert r.quality == q and np.array_equal(r.coefs.flat(), coefs), (w, h)
        a, _ = oracle.write_best(w, h, lay, r.coefs.qtables, r.coefs.flat())
        b, _ = oracle.write_best(w, h, lay, qt, coefs)
        assert hashlib.sha256(a).hexdigest() == hashlib.sha256(b).hexdigest()


def test_lockstep_batch_matches_individual_searches(ctx):
    """rcg_search_batch_lockstep (every step of every image in one work-list launch per stage) gives exactly each
    image's own search result: sizes from tiny to 2 MP, gray, a target the max quality misses, Auto subsampling."""
    sizes = [(96, 80), (300, 200), (1600, 1200), (17, 33), (1000, 700), (64, 64), (333, 111), (8, 8)]
    imgs = [synth.image(max(w, 16), max(h, 16), 30 + i, sensor_sigma=2.0)[:h, :w].copy()
            for i, (w, h) in enumerate(sizes)]
    imgs[5] = np.ascontiguousarray(imgs[5][:, :, 0])
    targets = [60.0, 70.0, 80.0, 65.0, 99.5, 55.0, 72.0, 50.0]
    for sub in (rcg.Subsampling.S420, rcg.Subsampling.Auto):
        opts = rcg.EncodeOptions(90, sub, True)
        want = [ctx.find_quality_ssimulacra2(im, t, 100, opts) for im, t in zip(imgs, targets)]
        for _ in range(3):  # plain launches, then the captured graph, then its replay
            res = ctx.search_batch(imgs, targets, 100, opts, lockstep=True)
            for r, f in zip(res, want):
                assert r.quality == f.quality and r.trace == f.trace, (r.trace, f.trace)
                assert np.array_equal(r.coefs.flat(), f.coefs.flat())


def test_lockstep_batch_near_tie(ctx, oracle):
    """A target 1e-9 above a candidate's oracle score: the lockstep batch pauses that image, decides it on the exact
    score and finishes it on the oracle's path while the other images run on."""
    a = synth.image(512, 512, 0)
    b = synth.image(320, 240, 4, sensor_sigma=2.0)
    _, _, _, _, _, trace = oracle.search(a, 70.0, 100, 3, True)
    assert len(trace) >= 3
    t = trace[2][1] + 1e-9
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    n0 = ctx.tie_rescores()
    res = ctx.search_batch([a, b], [t, 70.0], 100, opts, lockstep=True)
    assert ctx.tie_rescores() > n0
    q, s, coefs, qt, lay, otrace = oracle.search(a, t, 100, 3, True)
    assert [x[0] for x in res[0].trace] == [x[0] for x in otrace]
    assert res[0].quality == q and np.array_equal(res[0].coefs.flat(), coefs)
    f = ctx.find_quality_ssimulacra2(b, 70.0, 100, opts)
    assert res[1].trace == f.trace and np.array_equal(res[1].coefs.flat(), f.coefs.flat())
