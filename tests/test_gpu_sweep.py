"""Rate-quality sweeps (rcg_sweep_qualities) against one build_coefs -> reconstruct -> ssimulacra2 per quality.

The sweep runs the same kernels (one FDCT per image, the per-quality tables, quantization, trellis, decode) and scores
an image's candidates together with the work-list scorer, which gives the one-pair scorer's bits: every score must
equal the single calls' exactly, across subsampling modes (Auto switching layout at quality 90), quality 100 (no
trellis pass), gray images and odd sizes.
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu


def _single(ctx, img, q, sub, trellis):
    ci = ctx.build_coefs(img, rcg.EncodeOptions(q, sub, trellis))
    return ctx.ssimulacra2(img, ctx.reconstruct(ci))


@pytest.mark.parametrize("sub,trellis", [(rcg.Subsampling.S420, True), (rcg.Subsampling.Auto, True),
                                         (rcg.Subsampling.S422, False)])
def test_sweep_equals_single_calls(ctx, sub, trellis):
    images = [synth.image(331, 197, 71, sensor_sigma=3.0), synth.image(64, 48, 72)]
    qualities = [100, 95, 90, 89, 75, 50, 20, 1]
    got = ctx.sweep_qualities(images, qualities, rcg.EncodeOptions(90, sub, trellis))
    assert got.shape == (2, len(qualities))
    for i, img in enumerate(images):
        for k, q in enumerate(qualities):
            assert got[i, k] == _single(ctx, img, q, sub, trellis), (i, q)


def test_sweep_gray_and_repeat(ctx):
    gray = np.ascontiguousarray(synth.image(120, 90, 73)[:, :, 0])
    qs = [85, 60]
    a = ctx.sweep_qualities([gray], qs, rcg.EncodeOptions(90, rcg.Subsampling.S420, True))
    b = ctx.sweep_qualities([gray], qs, rcg.EncodeOptions(90, rcg.Subsampling.S420, True))
    assert np.array_equal(a, b)
    for k, q in enumerate(qs):
        assert a[0, k] == _single(ctx, gray, q, rcg.Subsampling.S420, True)
    # scores fall with quality on this image
    assert a[0, 0] > a[0, 1]


def test_sweep_errors(ctx):
    img = synth.image(32, 32, 74)
    with pytest.raises(rcg.RcgError):
        ctx.sweep_qualities([img], [0], rcg.EncodeOptions())
    with pytest.raises(rcg.RcgError):
        ctx.sweep_qualities([img[:7].copy()], [50], rcg.EncodeOptions())
    assert ctx.sweep_qualities([], [50], rcg.EncodeOptions()).shape == (0, 1)
