"""The reference-order FP64 scorer and the searches' near-tie decisions.

rcg_ssimulacra2_exact computes SSIMULACRA2 in the reference's own arithmetic and order (core/src/ssimulacra2.rs:
f64 XYB, blurs, maps and per-96-row-stripe sums); against the oracle (the reference restated in C++) it may differ
only by the last bits of cbrt/pow, so the bar here is 1e-9 absolute where the fast scorer's is 1e-3.

A search accepts a candidate on score >= target (jpeg/src/target.rs:48). Targets placed 1e-9 either side of an
oracle candidate score make that decision a near tie, which the fast f32 scorer cannot settle; the search must then
decide on the exact score and take the oracle's path, with the same coefficients and the same file.
"""

import hashlib
import math

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

TOL_EXACT = 1e-9
TOL_FAST = 1e-3


def test_exact_scorer_on_the_golden_pairs(ctx, golden, oracle):
    worst_o = worst_g = 0.0
    for name, ref, dist, want in golden:
        got = ctx.ssimulacra2_exact(ref, dist)
        orc = oracle.ssimulacra2(ref, dist)
        worst_o = max(worst_o, abs(got - orc))
        worst_g = max(worst_g, abs(got - want))
        assert abs(got - orc) <= TOL_EXACT, f"{name}: exact {got!r} oracle {orc!r}"
        assert abs(got - want) <= 1e-4, f"{name}: exact {got} golden {want}"
    print(f"worst |exact-oracle| {worst_o:.3e}  worst |exact-golden| {worst_g:.3e}")


@pytest.mark.parametrize("w,h", [(8, 8), (9, 13), (11, 40), (17, 33), (257, 9), (300, 200), (97, 193)])
def test_exact_scorer_awkward_sizes(ctx, oracle, w, h):
    """Rows of <= 10 samples (every sample on the edge path), odd 2x2 edges, stripes that end mid-image."""
    ref = synth.image(max(w, 16), max(h, 16), 12)[:h, :w].copy()
    dist = synth.image(max(w, 16), max(h, 16), 12, sensor_sigma=7.0)[:h, :w].copy()
    got = ctx.ssimulacra2_exact(ref, dist)
    want = oracle.ssimulacra2(ref, dist)
    assert abs(got - want) <= TOL_EXACT, (w, h, got, want)


def test_exact_scorer_formats(ctx, oracle):
    """Gray, alpha and 16-bit samples go through the same linear planes as the fast scorer."""
    rng = np.random.default_rng(5)
    base = synth.image(120, 90, 13)
    noisy = synth.image(120, 90, 13, sensor_sigma=5.0)
    gray = (np.ascontiguousarray(base[:, :, 0]), np.ascontiguousarray(noisy[:, :, 0]))
    alpha = rng.integers(0, 256, (90, 120, 1), dtype=np.uint8)
    rgba = (np.concatenate([base, alpha], axis=2), np.concatenate([noisy, alpha], axis=2))
    b16 = (base.astype(np.uint16) * 257, noisy.astype(np.uint16) * 257 + 3)
    for a, b in (gray, rgba, b16):
        got = ctx.ssimulacra2_exact(a, b)
        want = oracle.ssimulacra2(a, b)
        assert abs(got - want) <= TOL_EXACT, (a.shape, a.dtype, got, want)


def test_exact_scorer_identical_images_and_errors(ctx):
    img = synth.image(64, 48, 14)
    assert ctx.ssimulacra2_exact(img, img) == 100.0
    with pytest.raises(rcg.RcgError) as e:
        ctx.ssimulacra2_exact(img[:7], img[:7])
    assert e.value.status == rcg.RCG_INVALID


def test_exact_scorer_workload_pair(ctx, oracle):
    """The scorer workload's 3840x2160 pair: the exact scorer, the fast one, the oracle and the FP64 oracle."""
    w, h = 3840, 2160
    ref = synth.image(w, h, 0)
    coefs, qt, lay = oracle.build_coefs(ref, 50, 3, True)
    dist = oracle.reconstruct(w, h, lay, qt, coefs)
    exact = ctx.ssimulacra2_exact(ref, dist)
    fast = ctx.ssimulacra2(ref, dist)
    want = oracle.ssimulacra2(ref, dist)
    want64 = oracle.ssimulacra2(ref, dist, fp64=True)
    print(f"exact {exact!r} fast {fast!r} oracle {want!r} fp64 {want64!r}")
    assert abs(exact - want) <= TOL_EXACT
    assert abs(fast - want) <= TOL_FAST and abs(fast - want64) <= TOL_FAST


def _file(w, h, lay, qt, coefs, oracle):
    data, _ = oracle.write_best(w, h, lay, qt, coefs)
    return hashlib.sha256(data).hexdigest()


def _same_search(ctx, oracle, img, target, sub=rcg.Subsampling.S420, max_q=100):
    """GPU and oracle searches for `target`; returns how many candidates the GPU decided on the exact score."""
    h, w = img.shape[:2]
    n0 = ctx.tie_rescores()
    f = ctx.find_quality_ssimulacra2(img, target, max_q, rcg.EncodeOptions(90, sub, True))
    q, s, coefs, qt, lay, trace = oracle.search(img, target, max_q, int(sub), True)
    ties = ctx.tie_rescores() - n0
    assert [t[0] for t in f.trace] == [t[0] for t in trace], (target, f.trace, trace)
    for (gq, gs), (oq, os_) in zip(f.trace, trace):
        tol = TOL_EXACT if abs(os_ - target) <= 1e-6 else TOL_FAST
        assert abs(gs - os_) <= tol, (target, gq, gs, os_)
    assert f.quality == q
    assert np.array_equal(f.coefs.flat(), coefs)
    assert _file(w, h, lay, f.coefs.qtables, f.coefs.flat(), oracle) == _file(w, h, lay, qt, coefs, oracle)
    return ties


def test_near_ties_take_the_oracle_path(ctx, oracle):
    """Targets 1e-9 above and below each candidate score of a search: every one is a near tie for the fast scorer,
    decided on the exact score; the path, the coefficients and the file equal the oracle's."""
    img = synth.image(512, 512, 0)
    _, _, _, _, _, trace = oracle.search(img, 70.0, 100, 3, True)
    exercised = 0
    for _, s in trace:
        for delta in (-1e-9, 1e-9):
            exercised += _same_search(ctx, oracle, img, s + delta) > 0
    # A candidate is re-evaluated under its shifted target whenever the score rises with quality along the path.
    assert exercised >= len(trace), (exercised, trace)
    print(f"{exercised} of {2 * len(trace)} shifted targets met their candidate as a near tie")


def test_near_tie_at_the_first_candidate(ctx, oracle):
    """The first candidate (max quality) ends the search when it misses: a target just above its score must end at
    quality 100, just below must go on bisecting."""
    img = synth.image(300, 200, 2, sensor_sigma=3.0)
    _, s100, _, _, _, trace = oracle.search(img, 50.0, 100, 3, True)
    assert trace[0][0] == 100
    s0 = trace[0][1]
    _same_search(ctx, oracle, img, s0 + 1e-9)
    f = ctx.find_quality_ssimulacra2(img, s0 + 1e-9, 100, rcg.EncodeOptions(90, rcg.Subsampling.S420, True))
    assert f.quality == 100 and len(f.trace) == 1
    _same_search(ctx, oracle, img, s0 - 1e-9)


def test_near_ties_with_graph_replays(oracle):
    """The same tie search three times on one context (plain launches, capture, replay): the pause and resume work
    from a replayed graph too, with the same results each time."""
    img = synth.image(256, 192, 3)
    _, _, _, _, _, trace = oracle.search(img, 65.0, 100, 3, True)
    target = trace[min(2, len(trace) - 1)][1] + 1e-9
    with rcg.Context(0) as c:
        results = []
        for _ in range(3):
            assert _same_search(c, oracle, img, target) >= 1
            results.append(c.find_quality_ssimulacra2(img, target, 100,
                                                      rcg.EncodeOptions(90, rcg.Subsampling.S420, True)))
        assert c.graph_stats()[1] >= 1
        for r in results[1:]:
            assert r.trace == results[0].trace and np.array_equal(r.coefs.flat(), results[0].coefs.flat())


def test_every_candidate_decided_exactly(oracle):
    """Band infinity: every candidate is decided on (and reports) its exact score, equal to the oracle's to 1e-9.
    Band 0: every candidate on the fast score, as before."""
    img = synth.image(320, 240, 4, sensor_sigma=2.0)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    q, s, coefs, qt, lay, trace = oracle.search(img, 72.0, 100, 3, True)
    with rcg.Context(0) as c:
        c.set_tie_band(math.inf)
        f = c.find_quality_ssimulacra2(img, 72.0, 100, opts)
        assert c.tie_rescores() == len(trace)
        assert [t[0] for t in f.trace] == [t[0] for t in trace]
        for (_, gs), (_, os_) in zip(f.trace, trace):
            assert abs(gs - os_) <= TOL_EXACT, (gs, os_)
        assert f.quality == q and np.array_equal(f.coefs.flat(), coefs)
        c.set_tie_band(0.0)
        f0 = c.find_quality_ssimulacra2(img, 72.0, 100, opts)
        assert c.tie_rescores() == len(trace)
        assert f0.quality == q
        with pytest.raises(rcg.RcgError):
            c.set_tie_band(-1.0)


def test_requantize_search_near_tie(oracle):
    """The JPEG -> JPEG search decides near ties the same way (every candidate exact under band infinity)."""
    img = synth.image(256, 256, 5)
    coefs, qt, lay = oracle.build_coefs(img, 95, 3, True)
    g = oracle.general_from_encoder(256, 256, lay, qt, coefs)
    qr, sr, gr, trace = oracle.search_requantize(g, 70.0)
    with rcg.Context(0) as c:
        src = c.decode_coefs(oracle.write_jpeg_variant(g, 0, False))
        c.set_tie_band(math.inf)
        f = c.find_quality_requantize(src, 70.0)
        assert [t[0] for t in f.trace] == [t[0] for t in trace]
        for (_, gs), (_, os_) in zip(f.trace, trace):
            assert abs(gs - os_) <= TOL_EXACT, (gs, os_)
        assert f.quality == qr and np.array_equal(f.coefs.flat(), gr.coefs)
        # a target just above a candidate's score: a near tie at the default band
        c.set_tie_band(1e-3)
        t = trace[min(1, len(trace) - 1)][1] + 1e-9
        qr2, _, gr2, trace2 = oracle.search_requantize(g, t)
        n0 = c.tie_rescores()
        f2 = c.find_quality_requantize(src, t)
        assert c.tie_rescores() > n0
        assert [x[0] for x in f2.trace] == [x[0] for x in trace2]
        assert f2.quality == qr2 and np.array_equal(f2.coefs.flat(), gr2.coefs)
