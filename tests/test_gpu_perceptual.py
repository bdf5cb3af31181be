"""The perceptual trellis on the GPU: the coefficient pullback of the SSIMULACRA2 gradient, the weights, the weighted
trellis and the perceptual search, against the oracle.

- The coefficient gradient and the weights are f64 computations; the oracle restates them in numpy from the same
  pixel gradient (the GPU's FP64 adjoint, itself checked against the CPU gradient and central differences elsewhere):
  the coefficient gradient to 1e-12 of its largest entry, the f32 weights to 1e-6 relative. The default weights,
  from the FP32 adjoint, stay within a few 1e-3 of the FP64 ones.
- The weighted trellis is integer work given its weights: coefficients bit-exact with the oracle's trellis in the
  same mode (GPU weights passed to both), all-ones weights bit-exact with the plain trellis, and the weighted search
  visits the oracle's qualities and returns its coefficients.
- The perceptual search returns the plain search's result unchanged beside its own, and never a larger planned file
  than the plain one when keep_smaller is set.
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu


def _decoded(ctx, img, q, sub):
    ci = ctx.build_coefs(img, rcg.EncodeOptions(q, sub, True))
    return ctx.reconstruct(ci)


def _lay_dict(lay):
    n = lay.ncomp
    return {"ncomp": n, "h": list(lay.h[:n]), "v": list(lay.v[:n]), "blocks_w": list(lay.blocks_w[:n]),
            "blocks_h": list(lay.blocks_h[:n]), "ncoefs": int(lay.ncoefs)}


CASES = [(200, 150, 3, rcg.Subsampling.S420), (131, 77, 3, rcg.Subsampling.S422), (96, 72, 3, rcg.Subsampling.S444),
         (121, 90, 1, rcg.Subsampling.S420), (9, 8, 3, rcg.Subsampling.S420)]


@pytest.mark.parametrize("w,h,c,sub", CASES)
def test_coefficient_gradient_and_weights_match_the_oracle(ctx, oracle, w, h, c, sub):
    img = synth.image(max(w, 8), max(h, 8), 90)[:h, :w].copy()
    if c == 1:
        img = img[:, :, 0].copy()
    dec = _decoded(ctx, img, 45, sub)
    lay = ctx.coef_layout(w, h, c, rcg.EncodeOptions(45, sub, True))
    s, g = ctx.coef_gradient(img, dec, lay)
    rgb = lambda a: np.repeat(a[:, :, None], 3, 2) if a.ndim == 2 else a
    s_pix, gpix = ctx.ssimulacra2_grad(rgb(img), rgb(dec).astype(np.float32))
    assert s == s_pix
    want = oracle.coef_gradient(gpix, w, h, _lay_dict(lay))
    assert np.abs(g - want).max() <= 1e-12 * max(np.abs(want).max(), 1e-300)
    for popts in (rcg.PerceptualOptions(gradient_fp64=True), rcg.PerceptualOptions(1.0, 1.0, 0.1, 10.0, 2, True, True),
                  rcg.PerceptualOptions(0.5, 0.0, 0.25, 4.0, 0, True, True)):
        s2, wts = ctx.perceptual_weights(img, dec, lay, popts)
        assert s2 == s
        ref = oracle.perceptual_weights(gpix, w, h, _lay_dict(lay), popts.strength, popts.gamma, popts.w_min,
                                        popts.w_max, popts.radius)
        assert wts.dtype == np.float32 and wts.size == lay.ncoefs
        assert np.allclose(wts, ref, rtol=1e-6, atol=0), np.abs(wts / ref - 1).max()
    # The default weights come from the FP32 instantiation of the adjoint: the same rule on a gradient a few digits
    # from the FP64 one (measured: median 1e-4, worst 7e-3 relative). Its score carries the f32 cancellation of the
    # SSIM map (up to ~0.05 on flat gray content); the score only scales the whole gradient, which the weights'
    # per-component normalisation removes.
    s32, w32 = ctx.perceptual_weights(img, dec, lay)
    _, w64 = ctx.perceptual_weights(img, dec, lay, rcg.PerceptualOptions(gradient_fp64=True))
    rel = np.abs(w32.astype(np.float64) / w64 - 1.0)
    print(f"{w}x{h}: FP32 weights vs FP64: median {np.median(rel):.2e}, max {rel.max():.2e}; score {s32 - s:+.2e}")
    assert np.median(rel) < 1e-3 and rel.max() < 0.03
    assert abs(s32 - s) < 0.1


def test_all_ones_weights_are_the_plain_trellis(ctx):
    img = synth.image(333, 217, 91, sensor_sigma=3.0)
    for sub in (rcg.Subsampling.S420, rcg.Subsampling.S422, rcg.Subsampling.S444):
        for q in (20, 75, 99):
            opts = rcg.EncodeOptions(q, sub, True)
            plain = ctx.build_coefs(img, opts)
            ones = np.ones(plain.flat().size, dtype=np.float32)
            assert np.array_equal(ctx.build_coefs_weighted(img, opts, ones).flat(), plain.flat()), (sub, q)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    f = ctx.find_quality_ssimulacra2(img, 70.0, 100, opts)
    g = ctx.find_quality_weighted(img, 70.0, np.ones(f.coefs.flat().size, dtype=np.float32), 100, opts)
    assert (g.quality, g.score, g.trace) == (f.quality, f.score, f.trace)
    assert np.array_equal(g.coefs.flat(), f.coefs.flat())


@pytest.mark.parametrize("w,h,c,sub", [(245, 173, 3, rcg.Subsampling.S420), (160, 96, 3, rcg.Subsampling.S422),
                                       (100, 75, 3, rcg.Subsampling.S444), (99, 67, 1, rcg.Subsampling.S420)])
def test_weighted_trellis_matches_the_oracle(ctx, oracle, w, h, c, sub):
    img = synth.image(w, h, 92, sensor_sigma=3.0)
    if c == 1:
        img = img[:, :, 1].copy()
    rng = np.random.default_rng(w)
    lay = ctx.coef_layout(w, h, c, rcg.EncodeOptions(50, sub, True))
    # random weights with whole blocks and single coefficients far from 1
    wts = np.exp(rng.uniform(np.log(0.05), np.log(8.0), lay.ncoefs)).astype(np.float32)
    for q in (15, 60, 92):
        got = ctx.build_coefs_weighted(img, rcg.EncodeOptions(q, sub, True), wts)
        want, _, _ = oracle.build_coefs(img, q, int(sub), True, weights=wts)
        assert np.array_equal(got.flat(), want), (q, int(np.count_nonzero(got.flat() != want)))


def test_weighted_search_matches_the_oracle(ctx, oracle):
    img = synth.image(320, 240, 93, sensor_sigma=3.0)
    sub = rcg.Subsampling.S420
    opts = rcg.EncodeOptions(90, sub, True)
    plain = ctx.find_quality_ssimulacra2(img, 70.0, 100, opts)
    dec = ctx.reconstruct(plain.coefs)
    lay = ctx.coef_layout(320, 240, 3, rcg.EncodeOptions(50, sub, True))
    _, wts = ctx.perceptual_weights(img, dec, lay)
    f = ctx.find_quality_weighted(img, 70.0, wts, 100, opts)
    q, s, coefs, qt, olay, trace = oracle.search(img, 70.0, 100, int(sub), True, weights=wts)
    assert [t[0] for t in f.trace] == [t[0] for t in trace]
    for (_, x), (_, y) in zip(f.trace, trace):
        assert abs(x - y) <= 1e-3
    assert f.quality == q and abs(f.score - s) <= 1e-3
    assert np.array_equal(f.coefs.flat(), coefs)


def test_weighted_search_at_the_workload_size(ctx, oracle):
    """The perceptual trellis at the size it is specified for: 4000x3000 (seed 1, sensor noise sigma 3), target 70,
    4:2:0, the weights of the perceptual search's own schedule at the plain result; the weighted search visits the
    oracle's qualities and returns its coefficients bit for bit."""
    img = synth.image(4000, 3000, 1, 3.0)
    sub = rcg.Subsampling.S420
    opts = rcg.EncodeOptions(90, sub, True)
    plain = ctx.find_quality_ssimulacra2(img, 70.0, 100, opts)
    dec = ctx.reconstruct(plain.coefs)
    lay = ctx.coef_layout(4000, 3000, 3, rcg.EncodeOptions(50, sub, True))
    popts = rcg.PerceptualOptions()
    popts.strength = popts.strength_for(plain.quality)
    _, wts = ctx.perceptual_weights(img, dec, lay, popts)
    f = ctx.find_quality_weighted(img, 70.0, wts, 100, opts)
    q, s, coefs, qt, olay, trace = oracle.search(img, 70.0, 100, int(sub), True, weights=wts)
    assert [t[0] for t in f.trace] == [t[0] for t in trace], (f.trace, trace)
    for (_, x), (_, y) in zip(f.trace, trace):
        assert abs(x - y) <= 1e-3
    assert f.quality == q
    assert np.array_equal(f.coefs.flat(), coefs)


def test_perceptual_search(ctx):
    img = synth.image(640, 480, 94, sensor_sigma=3.0)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    plain = ctx.find_quality_ssimulacra2(img, 70.0, 100, opts)
    for keep in (True, False):
        popts = rcg.PerceptualOptions(keep_smaller=keep)
        r = ctx.find_quality_perceptual(img, 70.0, 100, opts, popts)
        assert (r.plain.quality, r.plain.score, r.plain.trace) == (plain.quality, plain.score, plain.trace)
        # the weights come from the gradient at the plain result's decoded image, with the strength the plain
        # result's quality selects
        strength = popts.strength_for(plain.quality)
        assert strength == (0.35 if plain.quality < 70 else (0.7 if plain.quality < 85 else 1.0))
        lay = ctx.coef_layout(640, 480, 3, rcg.EncodeOptions(50, rcg.Subsampling.S420, True))
        _, wts = ctx.perceptual_weights(img, ctx.reconstruct(plain.coefs), lay, rcg.PerceptualOptions(strength))
        assert np.array_equal(r.weights, wts)
        weighted = ctx.find_quality_weighted(img, 70.0, wts, 100, opts)
        p_plain, p_w = ctx.plan(plain.coefs), ctx.plan(weighted.coefs)
        assert r.plain_bytes == min(p_plain.progressive_bytes, p_plain.baseline_bytes)
        assert r.perceptual_bytes == min(p_w.progressive_bytes, p_w.baseline_bytes)
        expect_perc = (not keep) or r.perceptual_bytes <= r.plain_bytes
        assert r.chose_perceptual == expect_perc
        src = weighted if expect_perc else plain
        assert (r.found.quality, r.found.score) == (src.quality, src.score)
        assert np.array_equal(r.found.coefs.flat(), src.coefs.flat())
        assert r.found.score >= 70.0
        print(f"keep_smaller={keep}: plain q{plain.quality} {r.plain_bytes} B, weighted q{weighted.quality} "
              f"{weighted.score:.2f} {r.perceptual_bytes} B")


def test_perceptual_errors(ctx):
    img = synth.image(64, 48, 95)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    lay = ctx.coef_layout(64, 48, 3, opts)
    with pytest.raises(rcg.RcgError) as e:
        ctx.find_quality_perceptual(img, 70.0, 100, rcg.EncodeOptions(90, rcg.Subsampling.Auto, True))
    assert e.value.status == rcg.RCG_UNSUPPORTED
    with pytest.raises(rcg.RcgError) as e:
        ctx.find_quality_perceptual(img, 70.0, 100, rcg.EncodeOptions(90, rcg.Subsampling.S420, False))
    assert e.value.status == rcg.RCG_INVALID
    with pytest.raises(rcg.RcgError):
        ctx.find_quality_weighted(img, 70.0, np.ones(lay.ncoefs - 64, dtype=np.float32), 100, opts)
    for bad in (rcg.PerceptualOptions(strength=0.0), rcg.PerceptualOptions(gamma=-1.0),
                rcg.PerceptualOptions(w_min=2.0, w_max=1.0), rcg.PerceptualOptions(radius=-1)):
        with pytest.raises(rcg.RcgError) as e:
            ctx.find_quality_perceptual(img, 70.0, 100, opts, bad)
        assert e.value.status == rcg.RCG_INVALID
    with pytest.raises(rcg.RcgError):
        ctx.coef_gradient(img, img[:, :, :1].copy(), lay)


@pytest.mark.parametrize("c,sub", [(1, rcg.Subsampling.Auto), (3, rcg.Subsampling.S444), (3, rcg.Subsampling.S422)])
def test_perceptual_search_other_layouts(ctx, oracle, c, sub):
    """Gray (any subsampling: its layout never changes), 4:4:4 and 4:2:2: the weighted search follows the oracle's
    weighted search with the same weights, and the returned result is the smaller planned one."""
    img = synth.image(352, 264, 96, sensor_sigma=3.0)
    if c == 1:
        img = img[:, :, 2].copy()
    opts = rcg.EncodeOptions(90, sub, True)
    r = ctx.find_quality_perceptual(img, 65.0, 100, opts)
    q, s, coefs, _, _, trace = oracle.search(img, 65.0, 100, int(sub), True, weights=r.weights)
    weighted = ctx.find_quality_weighted(img, 65.0, r.weights, 100, opts)
    assert [t[0] for t in weighted.trace] == [t[0] for t in trace]
    assert weighted.quality == q and np.array_equal(weighted.coefs.flat(), coefs)
    assert r.chose_perceptual == (r.perceptual_bytes <= r.plain_bytes)
    assert r.found.quality == (weighted.quality if r.chose_perceptual else r.plain.quality)
    assert r.found.score >= 65.0


def test_fast_perceptual_search(ctx, oracle):
    """rcg_search_perceptual_fast: its probe is the plain bisection's first four candidates, its weights those of
    the gradient at the probe candidate scoring closest to the target, and its result the weighted search with those
    weights (and the oracle's weighted search)."""
    img = synth.image(640, 480, 95, sensor_sigma=3.0)
    sub = rcg.Subsampling.S420
    opts = rcg.EncodeOptions(90, sub, True)
    popts = rcg.PerceptualOptions()
    probe, res, wts = ctx.find_quality_perceptual_fast(img, 70.0, 100, opts, popts)
    plain = ctx.find_quality_ssimulacra2(img, 70.0, 100, opts)
    assert probe.trace == plain.trace[:4]
    closest = min(probe.trace, key=lambda qs: abs(qs[1] - 70.0))
    assert (probe.quality, probe.score) == closest
    ci = ctx.build_coefs(img, rcg.EncodeOptions(probe.quality, sub, True))
    lay = ctx.coef_layout(640, 480, 3, rcg.EncodeOptions(50, sub, True))
    po = rcg.PerceptualOptions()
    po.strength = popts.strength_for(probe.quality)
    _, want_w = ctx.perceptual_weights(img, ctx.reconstruct(ci), lay, po)
    assert np.array_equal(wts, want_w)
    f = ctx.find_quality_weighted(img, 70.0, wts, 100, opts)
    assert (res.quality, res.trace) == (f.quality, f.trace)
    assert np.array_equal(res.coefs.flat(), f.coefs.flat())
    q, s, coefs, qt, olay, trace = oracle.search(img, 70.0, 100, int(sub), True, weights=wts)
    assert res.quality == q and np.array_equal(res.coefs.flat(), coefs)
    assert res.score >= 70.0 or res.quality == 100
