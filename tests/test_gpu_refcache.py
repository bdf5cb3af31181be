"""The SSIMULACRA2 searches' stored reference moments.

The scorer's offsets come from the reference image alone, so its blurred a' and a'^2 depend on the reference only: a
search's first candidate stores them and every later candidate reads them instead of blurring them. The blurred
moments are the same per-lane FMA chains either way, so a search must give the same bits with the cache on (the
default) and off: the same trace of qualities and scores, the same coefficients. Every other search test runs with
the cache on against the oracle.
"""

import math

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

OPTS = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)


def _pair_of_contexts():
    on, off = rcg.Context(0), rcg.Context(0)
    off.set_ref_cache(False)
    return on, off


def _same(a, b):
    assert a.quality == b.quality
    assert a.trace == b.trace  # qualities and scores, bit for bit
    if a.coefs is not None or b.coefs is not None:  # a perceptual probe returns no coefficients
        assert np.array_equal(a.coefs.flat(), b.coefs.flat())


@pytest.mark.parametrize("w,h,seed,sub,target", [
    (512, 512, 0, rcg.Subsampling.S420, 70.0),
    (1023, 767, 1, rcg.Subsampling.S444, 80.0),
    (1600, 1200, 2, rcg.Subsampling.S422, 60.0),
    (4000, 3000, 1, rcg.Subsampling.S420, 70.0),
])
def test_cache_on_and_off_give_the_same_search(w, h, seed, sub, target):
    img = synth.image(w, h, seed, 3.0)
    opts = rcg.EncodeOptions(90, sub, True)
    on, off = _pair_of_contexts()
    with on, off:
        for _ in range(3):  # plain launches, graph capture, replay
            _same(on.find_quality_ssimulacra2(img, target, 100, opts),
                  off.find_quality_ssimulacra2(img, target, 100, opts))


def test_cache_with_a_near_tie(oracle):
    """A target 1e-9 above an oracle candidate score: the search pauses there, is rescored exactly and resumes; the
    resumed steps read the moments the first candidate stored."""
    img = synth.image(512, 512, 0)
    _, _, _, _, _, trace = oracle.search(img, 70.0, 100, 3, True)
    on, off = _pair_of_contexts()
    with on, off:
        for s in (trace[0][1], trace[min(2, len(trace) - 1)][1]):
            t = s + 1e-9
            n0 = on.tie_rescores()
            a = on.find_quality_ssimulacra2(img, t, 100, OPTS)
            assert on.tie_rescores() > n0
            _same(a, off.find_quality_ssimulacra2(img, t, 100, OPTS))
            q, _, coefs, _, _, otrace = oracle.search(img, t, 100, 3, True)
            assert [x[0] for x in a.trace] == [x[0] for x in otrace]
            assert a.quality == q and np.array_equal(a.coefs.flat(), coefs)


def test_cache_in_the_requantize_search(oracle):
    img = synth.image(640, 480, 5)
    coefs, qt, lay = oracle.build_coefs(img, 95, 3, True)
    g = oracle.general_from_encoder(640, 480, lay, qt, coefs)
    on, off = _pair_of_contexts()
    with on, off:
        data = oracle.write_jpeg_variant(g, 0, False)
        a = on.find_quality_requantize(on.decode_coefs(data), 70.0)
        b = off.find_quality_requantize(off.decode_coefs(data), 70.0)
        _same(a, b)
        qr, _, gr, trace = oracle.search_requantize(g, 70.0)
        assert a.quality == qr and np.array_equal(a.coefs.flat(), gr.coefs)


def test_cache_in_batch_and_perceptual_searches():
    imgs = [synth.image(w, h, 30 + i, 2.0) for i, (w, h) in enumerate([(700, 500), (320, 240), (1200, 900)])]
    targets = [65.0, 75.0, 70.0]
    on, off = _pair_of_contexts()
    with on, off:
        ra = on.search_batch(imgs, targets, 100, OPTS, 2)
        rb = off.search_batch(imgs, targets, 100, OPTS, 2)
        for a, b in zip(ra, rb):
            _same(a, b)
        for _ in range(3):  # the lockstep batch: plain launches, capture, replay
            la = on.search_batch(imgs, targets, 100, OPTS, lockstep=True)
            lb = off.search_batch(imgs, targets, 100, OPTS, lockstep=True)
            for a, b, c in zip(la, lb, ra):
                _same(a, b)
                _same(a, c)
        pa, fa, wa = on.find_quality_perceptual_fast(imgs[2], 70.0, 100, OPTS)
        pb, fb, wb = off.find_quality_perceptual_fast(imgs[2], 70.0, 100, OPTS)
        _same(pa, pb)
        _same(fa, fb)
        assert np.array_equal(wa, wb)


def test_switching_the_cache_retires_captured_loops():
    """A context that captured its step loop with the cache on, switched off and on again: every search equals the
    first (the captured graphs of the old setting are not replayed)."""
    img = synth.image(800, 600, 7)
    with rcg.Context(0) as c:
        first = c.find_quality_ssimulacra2(img, 72.0, 100, OPTS)
        for on in (True, False, False, True, True):
            c.set_ref_cache(on)
            _same(c.find_quality_ssimulacra2(img, 72.0, 100, OPTS), first)
        assert math.isfinite(first.score)
