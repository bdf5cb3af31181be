"""JPEG encoder and decoder kernels against the CPU oracle: bit-exact coefficients and pixels.

build_coefs (jpeg/src/encode.rs:426) and reconstruct (jpeg/src/decode.rs:334) are integer/f32 pipelines with a fixed
operation order, so the bar is equality, for every subsampling, gray and colour, trellis on and off, odd and tiny
sizes (jpeg/tests/jpeg.rs:66-80) and qualities across the range including 100 (no trellis pass).
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

SUBS = [rcg.Subsampling.S420, rcg.Subsampling.S422, rcg.Subsampling.S444, rcg.Subsampling.Auto]


def _check_encode(ctx, oracle, img, q, sub, trellis):
    opts = rcg.EncodeOptions(q, sub, trellis)
    ci = ctx.build_coefs(img, opts)
    coefs, qt, lay = oracle.build_coefs(img, q, int(sub), trellis)
    got = ci.flat()
    assert got.shape == coefs.shape
    if not np.array_equal(got, coefs):
        bad = np.nonzero(got != coefs)[0]
        raise AssertionError(f"q{q} sub{int(sub)} trellis{trellis}: {bad.size} coefficients differ, first at "
                             f"{bad[0]} (block {bad[0] // 64}, k {bad[0] % 64}): {got[bad[0]]} vs {coefs[bad[0]]}")
    assert np.array_equal(ci.qtables[0], qt[0])
    return ci, (coefs, qt, lay)


@pytest.mark.parametrize("sub", SUBS)
@pytest.mark.parametrize("q", [1, 10, 30, 50, 75, 89, 90, 95, 100])
def test_build_coefs_bit_exact(ctx, oracle, sub, q):
    img = synth.image(203, 77, 3, sensor_sigma=3.0)
    for trellis in (True, False):
        _check_encode(ctx, oracle, img, q, sub, trellis)


@pytest.mark.parametrize("w,h", [(1, 1), (7, 9), (8, 8), (9, 9), (17, 1), (1, 17), (33, 31), (250, 3), (16, 16)])
def test_odd_and_tiny_sizes(ctx, oracle, w, h):
    img = synth.image(max(w, 8), max(h, 8), 4)[:h, :w].copy()
    for sub in SUBS[:3]:
        ci, (coefs, qt, lay) = _check_encode(ctx, oracle, img, 90, sub, True)
        rec = ctx.reconstruct(ci)
        want = oracle.reconstruct(w, h, lay, qt, coefs)
        assert np.array_equal(rec, want)


def test_gray(ctx, oracle):
    img = synth.image(130, 97, 5)[:, :, 1].copy()
    for q in (20, 75, 100):
        ci, (coefs, qt, lay) = _check_encode(ctx, oracle, img, q, rcg.Subsampling.S420, True)
        assert len(ci.comps) == 1
        rec = ctx.reconstruct(ci)
        assert rec.ndim == 2
        assert np.array_equal(rec, oracle.reconstruct(130, 97, lay, qt, coefs))


@pytest.mark.parametrize("sub", SUBS[:3])
def test_reconstruct_bit_exact(ctx, oracle, sub):
    img = synth.image(333, 211, 6, sensor_sigma=3.0)
    for q in (15, 60, 92):
        ci, (coefs, qt, lay) = _check_encode(ctx, oracle, img, q, sub, True)
        rec = ctx.reconstruct(ci)
        want = oracle.reconstruct(333, 211, lay, qt, coefs)
        assert np.array_equal(rec, want), (q, int(sub), np.abs(rec.astype(int) - want).max())


def test_reconstruct_of_arbitrary_coefficients(ctx, oracle):
    """The decoder takes any CoefImage with this layout, not only encoder output: random and extreme values."""
    rng = np.random.default_rng(7)
    img = synth.image(64, 48, 8)
    ci = ctx.build_coefs(img, rcg.EncodeOptions(50, rcg.Subsampling.S420, True))
    for scale in (3, 300, 2047):
        for c in ci.comps:
            c.coefs[:] = rng.integers(-scale, scale + 1, size=c.coefs.size).astype(np.int16)
        lay = dict(ncomp=3, h=[c.h for c in ci.comps], v=[c.v for c in ci.comps],
                   blocks_w=[c.blocks_w for c in ci.comps], blocks_h=[c.blocks_h for c in ci.comps])
        want = oracle.reconstruct(64, 48, lay, ci.qtables, ci.flat())
        assert np.array_equal(ctx.reconstruct(ci), want), scale


def test_encoder_rejects_bad_input(ctx):
    img = np.zeros((8, 8, 3), np.uint8)
    with pytest.raises(rcg.RcgError):
        ctx.build_coefs(img, rcg.EncodeOptions(0, rcg.Subsampling.S420, True))
    with pytest.raises(rcg.RcgError):
        ctx.build_coefs(img, rcg.EncodeOptions(101, rcg.Subsampling.S420, True))
    with pytest.raises(rcg.RcgError):
        ctx.build_coefs(np.zeros((8, 8, 4), np.uint8), rcg.EncodeOptions(50))
