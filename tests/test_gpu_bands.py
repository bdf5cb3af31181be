"""The scorer's band shapes and their autotuner.

A CTA of the fast scorer walks a band of 32 columns and `chunks` x 32 rows; the rows two chunks share are converted
to XYB once and re-offset. Every band height must score within the usual 1e-3 of the oracle (the heights differ
from each other only by re-offset rounding, about 1e-9); for one shape the scores are the same bits on every call,
through every entry point (single, batch, search). Images of about 1 MP and more are autotuned per size class.
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

TOL = 1e-3


def _pair(w, h, seed):
    ref = synth.image(w, h, seed, sensor_sigma=2.0)
    dist = synth.image(w, h, seed, sensor_sigma=6.0)
    return ref, dist


@pytest.mark.parametrize("w,h", [(1600, 1199), (1333, 1000), (2000, 700)])
def test_every_band_height_matches_the_oracle(oracle, w, h):
    ref, dist = _pair(w, h, 40)
    want = oracle.ssimulacra2(ref, dist)
    scores = {}
    with rcg.Context(0) as c:
        for chunks in (1, 2, 3, 4, 8, 37):
            c.set_band_chunks(chunks)
            s = c.ssimulacra2(ref, dist)
            assert c.ssimulacra2(ref, dist) == s  # the same bits on every call
            assert abs(s - want) <= TOL, (chunks, s, want)
            scores[chunks] = s
    spread = max(scores.values()) - min(scores.values())
    print(f"{w}x{h}: oracle {want:.9f}, spread over band heights {spread:.2e}")
    assert spread <= 1e-6


def test_autotuned_shape_is_used_everywhere(oracle):
    """The tuned height is fixed per size class for the process: the single scorer, the batch scorer and a search on
    the same image give the same bits as each other."""
    w, h = 1800, 1200
    ref, dist = _pair(w, h, 41)
    with rcg.Context(0) as c:
        chunks = c.band_chunks(w, h)
        assert chunks in (1, 2, 4, 8)
        s = c.ssimulacra2(ref, dist)
        b = c.ssimulacra2_batch([(ref, dist), (dist, ref), (ref, dist)])
        assert b[0] == s and b[2] == s
        assert b[1] == c.ssimulacra2(dist, ref)
        assert c.band_chunks(w, h) == chunks
        # a second context agrees (the choice is per process and device)
        with rcg.Context(0) as d:
            assert d.band_chunks(w, h) == chunks and d.ssimulacra2(ref, dist) == s
        f = c.find_quality_ssimulacra2(ref, 70.0, 100, rcg.EncodeOptions(90, rcg.Subsampling.S420, True))
        q, _, coefs, _, _, trace = oracle.search(ref, 70.0, 100, 3, True)
        assert [t[0] for t in f.trace] == [t[0] for t in trace]
        assert f.quality == q and np.array_equal(f.coefs.flat(), coefs)


def test_small_images_keep_tiles_and_band_limits(ctx):
    assert ctx.band_chunks(512, 512) == 1
    assert ctx.band_chunks(7, 100) == 0
    with rcg.Context(0) as c:
        with pytest.raises(rcg.RcgError):
            c.set_band_chunks(-1)
        with pytest.raises(rcg.RcgError):
            c.set_band_chunks(65)
        c.set_band_chunks(4)
        assert c.band_chunks(64, 64) == 4


@pytest.mark.parametrize("w,h", [(65535, 16), (40, 6000), (33, 1000)])
def test_bands_on_thin_images(oracle, w, h):
    """Bands taller than the image, single-column bands, chunks past the bottom edge."""
    ref, dist = _pair(w, h, 42)
    want = oracle.ssimulacra2(ref, dist)
    with rcg.Context(0) as c:
        for chunks in (1, 4, 8):
            c.set_band_chunks(chunks)
            assert abs(c.ssimulacra2(ref, dist) - want) <= TOL, chunks
