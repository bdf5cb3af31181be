"""The work-list scorer (rcg_ssimulacra2_batch): many pairs of different sizes and formats in one launch per stage.

Each pair's score must equal, bit for bit, what the one-pair scorer gives for it (same kernels, same arithmetic,
same reduction order), and so meet the same bars: 1e-4 against the reference's golden vectors
(cli/tests/ssimulacra2.rs:8, the 54 fixture pairs scored here in a single call), 1e-3 against the oracle. Pairs that
share a reference buffer share one conversion of it; errors name the pair at fault.
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

TOL_ORACLE = 1e-3
TOL_GOLDEN = 1e-4


def test_all_golden_pairs_in_one_call(ctx, golden):
    got = ctx.ssimulacra2_batch([(ref, dist) for _, ref, dist, _ in golden])
    assert got.shape == (len(golden),)
    for (name, ref, dist, want), g in zip(golden, got):
        assert g == ctx.ssimulacra2(ref, dist), name
        assert abs(g - want) <= TOL_GOLDEN, (name, g, want)


def test_candidates_sharing_one_reference(ctx, oracle):
    """Several decoded qualities of one image against the same reference object (converted once)."""
    img = synth.image(333, 250, 51)
    pairs = []
    for q in (30, 50, 70, 90):
        coefs, qt, lay = oracle.build_coefs(img, q, int(rcg.Subsampling.S420), True)
        pairs.append((img, oracle.reconstruct(333, 250, lay, qt, coefs)))
    other = synth.image(64, 48, 52)
    pairs.insert(2, (other, np.ascontiguousarray(other[::-1])))  # a different reference in between
    got = ctx.ssimulacra2_batch(pairs)
    for (a, b), g in zip(pairs, got):
        assert g == ctx.ssimulacra2(a, b)
        assert abs(g - oracle.ssimulacra2(a, b)) <= TOL_ORACLE


def test_mixed_formats_and_awkward_sizes(ctx):
    rng = np.random.default_rng(53)
    pairs = []
    for (w, h, c, dt) in [(8, 8, 3, np.uint8), (9, 15, 1, np.uint8), (17, 8, 4, np.uint8), (129, 65, 2, np.uint8),
                          (40, 33, 3, np.uint16), (31, 47, 1, np.uint16), (300, 7 + 200, 3, np.uint8)]:
        hi = 256 if dt == np.uint8 else 65536
        a = rng.integers(0, hi, (h, w, c)).astype(dt)
        b = np.clip(a.astype(np.int64) + rng.integers(-hi // 16, hi // 16, a.shape), 0, hi - 1).astype(dt)
        pairs.append((a, b))
    got = ctx.ssimulacra2_batch(pairs)
    for (a, b), g in zip(pairs, got):
        assert g == ctx.ssimulacra2(a, b), a.shape


def test_identical_pairs_score_exactly_100(ctx, golden):
    _, ref, _, _ = golden[0]
    img = synth.image(96, 72, 54)
    got = ctx.ssimulacra2_batch([(ref, ref), (img, img.copy()), (img, img)])
    assert list(got) == [100.0, 100.0, 100.0]


def test_device_pairs_and_replay(ctx):
    torch = pytest.importorskip("torch")
    sizes = [(640, 480), (100, 75), (1024, 768), (8, 8), (257, 129)]
    refs = [synth.image(w, h, 60 + i) for i, (w, h) in enumerate(sizes)]
    dists = [np.ascontiguousarray(np.clip(r.astype(np.int16) + 9 - (r % 19), 0, 255).astype(np.uint8)) for r in refs]
    d_r = [torch.from_numpy(r).cuda() for r in refs]
    d_d = [torch.from_numpy(d).cuda() for d in dists]
    want = [ctx.ssimulacra2(r, d) for r, d in zip(refs, dists)]
    with rcg.Context(0) as g:
        for _ in range(3):  # plain launches, then a captured graph, then its replay: same bits
            got = g.ssimulacra2_batch_device([t.data_ptr() for t in d_r], [t.data_ptr() for t in d_d],
                                             [w for w, _ in sizes], [h for _, h in sizes], [3] * len(sizes))
            assert list(got) == want
        assert g.graph_stats() == (1, 2)
        # the same totals with other pairs replay the stored launches: the work-list carries the pairs
        got = g.ssimulacra2_batch_device([t.data_ptr() for t in d_d], [t.data_ptr() for t in d_r],
                                         [w for w, _ in sizes], [h for _, h in sizes], [3] * len(sizes))
        assert list(got) == [ctx.ssimulacra2(d, r) for r, d in zip(refs, dists)]
        assert g.graph_stats() == (1, 3)


def test_errors_name_the_pair(ctx):
    a = synth.image(16, 16, 55)
    small = a[:7, :8].copy()
    with pytest.raises(rcg.RcgError) as e:
        ctx.ssimulacra2_batch([(a, a), (small, small)])
    assert e.value.status == rcg.RCG_INVALID and "pair 1" in str(e.value)
    with pytest.raises(rcg.RcgError):
        ctx.ssimulacra2_batch([(a, a[:, :, :2].copy())])
    assert len(ctx.ssimulacra2_batch([])) == 0
