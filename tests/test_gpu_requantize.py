"""DCT-domain requantization and the JPEG -> JPEG quality search on the GPU against the CPU oracle.

CoefImage::requantize (jpeg/src/encode.rs:111-172) is integer/f32 work in a fixed order: the bar is equal
coefficients and equal table assignments, for sources with shared, distinct and absent table slots, gray and colour,
every sampling layout, trellis on and off. The search (cli/src/pipeline.rs:369-386) must visit the same qualities and
pick the same candidate as the oracle, its scores within 1e-3 of the oracle's (the reference scorer restated).
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

TOL = 1e-3


def _source(oracle, img, q, sub, trellis=True):
    """An encoder-produced CoefImage (rcg form) and its oracle twin."""
    coefs, qt, lay = oracle.build_coefs(img, q, int(sub), trellis)
    h, w = img.shape[:2]
    n = lay["ncomp"]
    comps, off = [], 0
    for i in range(n):
        k = int(lay["blocks_w"][i] * lay["blocks_h"][i] * 64)
        comps.append(rcg.CoefComponent(i + 1, int(lay["h"][i]), int(lay["v"][i]), min(i, 1), int(lay["blocks_w"][i]),
                                       int(lay["blocks_h"][i]), coefs[off: off + k].copy()))
        off += k
    q4 = np.zeros((4, 64), np.uint8)
    q4[0] = qt[0]
    present = np.zeros(4, np.uint8)
    present[0] = 1
    if n > 1:
        q4[1] = qt[1]
        present[1] = 1
    return rcg.CoefImage(w, h, comps, q4, present), lay


def _to_oracle(oracle, ci, lay):
    return oracle.GeneralCoefs(ci.width, ci.height, lay, [c.tq for c in ci.comps], ci.qtables, ci.present, ci.flat())


def _assert_same(ci, g, what):
    got = ci.flat()
    if not np.array_equal(got, g.coefs):
        bad = np.nonzero(got != g.coefs)[0]
        raise AssertionError(f"{what}: {bad.size} coefficients differ, first at {bad[0]} (block {bad[0] // 64}, "
                             f"k {bad[0] % 64}): {got[bad[0]]} vs {g.coefs[bad[0]]}")
    assert [c.tq for c in ci.comps] == [int(x) for x in g.tq[: len(ci.comps)]], what
    assert np.array_equal(ci.present.astype(bool), g.has_q.astype(bool)), what
    for sl in range(4):
        if g.has_q[sl]:
            assert np.array_equal(ci.qtables[sl], g.qtables4[sl]), (what, sl)


def _check(ctx, oracle, ci, lay, q, trellis):
    out = ctx.requantize(ci, q, trellis)
    want = oracle.requantize(_to_oracle(oracle, ci, lay), q, trellis)
    _assert_same(out, want, f"q{q} trellis{trellis}")
    return out, want


@pytest.mark.parametrize("sub", [rcg.Subsampling.S420, rcg.Subsampling.S422, rcg.Subsampling.S444])
@pytest.mark.parametrize("q", [5, 30, 60, 85, 95, 100])
def test_requantize_encoder_sources(ctx, oracle, sub, q):
    img = synth.image(203, 77, 21, sensor_sigma=3.0)
    src, lay = _source(oracle, img, 95, sub)
    for trellis in (True, False):
        _check(ctx, oracle, src, lay, q, trellis)


def test_requantize_distinct_shared_and_absent_slots(ctx, oracle):
    img = synth.image(150, 101, 22, sensor_sigma=2.0)
    src, lay = _source(oracle, img, 90, rcg.Subsampling.S444)
    # three components with three different tables in slots 2, 0, 3
    _, qt80, _ = oracle.build_coefs(img[:8, :8].copy(), 80, 3, False)
    q4 = np.zeros((4, 64), np.uint8)
    q4[2] = src.qtables[0]
    q4[0] = src.qtables[1]
    q4[3] = qt80[1]
    src3 = rcg.CoefImage(src.width, src.height, [
        rcg.CoefComponent(c.id, c.h, c.v, tq, c.blocks_w, c.blocks_h, c.coefs) for c, tq in zip(src.comps, (2, 0, 3))
    ], q4, np.array([1, 0, 1, 1], np.uint8))
    for q in (40, 75, 92):
        for trellis in (True, False):
            _check(ctx, oracle, src3, lay, q, trellis)
    # a component naming an empty slot reads an all-ones table (jpeg/src/encode.rs:121)
    absent = rcg.CoefImage(src.width, src.height, [
        rcg.CoefComponent(c.id, c.h, c.v, tq, c.blocks_w, c.blocks_h, c.coefs) for c, tq in zip(src.comps, (0, 1, 2))
    ], src.qtables, np.array([1, 1, 0, 0], np.uint8))
    for trellis in (True, False):
        _check(ctx, oracle, absent, lay, 70, trellis)


def test_requantize_gray_and_tiny(ctx, oracle):
    img = synth.image(99, 45, 23)[:, :, 2].copy()
    src, lay = _source(oracle, img, 100, rcg.Subsampling.S420)
    for q in (20, 90):
        out, _ = _check(ctx, oracle, src, lay, q, True)
        assert len(out.comps) == 1
    for w, h in ((1, 1), (7, 9), (17, 3)):
        img = synth.image(max(w, 8), max(h, 8), 24)[:h, :w].copy()
        src, lay = _source(oracle, img, 97, rcg.Subsampling.S420)
        _check(ctx, oracle, src, lay, 50, True)


def test_quality_100_changes_nothing(ctx, oracle):
    """Nothing is requantized to a finer table than the source had (cli/tests/cmyk.rs:40)."""
    img = synth.image(120, 64, 25, sensor_sigma=4.0)
    src, lay = _source(oracle, img, 60, rcg.Subsampling.S420)
    out = ctx.requantize(src, 100, True)
    assert np.array_equal(out.flat(), src.flat())
    for c_new, c_old in zip(out.comps, src.comps):  # equal tables now share one slot (jpeg/src/encode.rs:139-148)
        assert np.array_equal(out.qtables[c_new.tq], src.qtables[c_old.tq])
    # a coarser target moves every table up, never down
    out = ctx.requantize(src, 30, True)
    for c_new, c_old in zip(out.comps, src.comps):
        assert np.all(out.qtables[c_new.tq] >= src.qtables[c_old.tq])


def test_requantized_image_reconstructs_like_the_oracle(ctx, oracle):
    img = synth.image(131, 90, 26, sensor_sigma=3.0)
    src, lay = _source(oracle, img, 92, rcg.Subsampling.S420)
    out, want = _check(ctx, oracle, src, lay, 55, True)
    assert np.array_equal(ctx.reconstruct(out), oracle.reconstruct_general(want))
    assert np.array_equal(ctx.reconstruct(src), oracle.reconstruct_general(_to_oracle(oracle, src, lay)))


@pytest.mark.parametrize("target,max_q,trellis,sub", [
    (70.0, 100, True, rcg.Subsampling.S420),
    (85.0, 100, False, rcg.Subsampling.S444),
    (60.0, 75, True, rcg.Subsampling.S422),
    (99.0, 100, True, rcg.Subsampling.S420),  # above what any requantization reaches: the top quality is kept
    (10.0, 100, True, rcg.Subsampling.S420),
])
def test_search_requantize_matches_the_oracle(ctx, oracle, target, max_q, trellis, sub):
    img = synth.image(320, 213, 27, sensor_sigma=3.0)
    src, lay = _source(oracle, img, 95, sub)
    f = ctx.find_quality_requantize(src, target, max_q, trellis)
    q, s, g, trace = oracle.search_requantize(_to_oracle(oracle, src, lay), target, max_q, trellis)
    assert [t[0] for t in f.trace] == [t[0] for t in trace], (f.trace, trace)
    for (_, a), (_, b) in zip(f.trace, trace):
        assert abs(a - b) <= TOL
    assert f.quality == q
    assert abs(f.score - s) <= TOL
    _assert_same(f.coefs, g, "search result")
    # the chosen candidate writes the same file as the oracle's
    assert oracle.write_best_general(_to_oracle(oracle, f.coefs, lay)) == oracle.write_best_general(g)


def test_search_requantize_gray_and_errors(ctx, oracle):
    img = synth.image(96, 80, 28)[:, :, 0].copy()
    src, lay = _source(oracle, img, 98, rcg.Subsampling.S420)
    f = ctx.find_quality_requantize(src, 75.0)
    q, s, g, _ = oracle.search_requantize(_to_oracle(oracle, src, lay), 75.0)
    assert f.quality == q and abs(f.score - s) <= TOL
    _assert_same(f.coefs, g, "gray search")
    small, _ = _source(oracle, synth.image(8, 8, 29)[:7, :8].copy(), 90, rcg.Subsampling.S420)
    with pytest.raises(rcg.RcgError) as e:
        ctx.find_quality_requantize(small, 70.0)
    assert e.value.status == rcg.RCG_UNSUPPORTED
    bad = rcg.CoefImage(src.width, src.height, [
        rcg.CoefComponent(1, 1, 1, 0, src.comps[0].blocks_w - 1, src.comps[0].blocks_h,
                          src.comps[0].coefs[: (src.comps[0].blocks_w - 1) * src.comps[0].blocks_h * 64])
    ], src.qtables, src.present)
    with pytest.raises(rcg.RcgError) as e:
        ctx.requantize(bad, 50)
    assert e.value.status == rcg.RCG_INVALID


def test_search_requantize_larger_image(ctx, oracle):
    """A 2 MP 4:2:0 source: the oracle search takes seconds; same decision and coefficients."""
    img = synth.image(1600, 1200, 30, sensor_sigma=3.0)
    src, lay = _source(oracle, img, 93, rcg.Subsampling.S420)
    f = ctx.find_quality_requantize(src, 72.0)
    q, s, g, trace = oracle.search_requantize(_to_oracle(oracle, src, lay), 72.0)
    assert [t[0] for t in f.trace] == [t[0] for t in trace]
    assert f.quality == q and abs(f.score - s) <= TOL
    _assert_same(f.coefs, g, "2 MP search")
