"""Parity at the benchmark's full size and at the largest JPEG dimension.

The 12 MP workload the bench times (4000x3000, seed 1, sensor noise sigma 3, target 70, 4:2:0, trellis) must take the
oracle's bisection path, choose bit-exact coefficients and write the same file, also with the target moved onto a
near tie. Strips 65535 pixels long (the
largest JPEG dimension, jpeg/src/encode.rs:417-418) in both orientations exercise the grids and the edge padding at
the size limit: coefficients and pixels bit-exact, scores within 1e-3 of the oracle.
"""

import hashlib

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu

TOL = 1e-3


def test_workload_search_matches_the_oracle(ctx, oracle):
    img = synth.image(4000, 3000, 1, 3.0)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    f = ctx.find_quality_ssimulacra2(img, 70.0, 100, opts)
    q, s, coefs, qt, lay, trace = oracle.search(img, 70.0, 100, int(rcg.Subsampling.S420), True)
    assert [t[0] for t in f.trace] == [t[0] for t in trace], (f.trace, trace)
    for (_, a), (_, b) in zip(f.trace, trace):
        assert abs(a - b) <= TOL
    assert f.quality == q
    assert np.array_equal(f.coefs.flat(), coefs)
    a, _ = oracle.write_best(4000, 3000, lay, f.coefs.qtables, f.coefs.flat())
    b, _ = oracle.write_best(4000, 3000, lay, qt, coefs)
    assert hashlib.sha256(a).hexdigest() == hashlib.sha256(b).hexdigest()


@pytest.mark.parametrize("w,h", [(65535, 16), (16, 65535)])
def test_largest_dimension_strips(ctx, oracle, w, h):
    img = synth.image(w, h, 81)
    for sub in (rcg.Subsampling.S420, rcg.Subsampling.S444):
        ci = ctx.build_coefs(img, rcg.EncodeOptions(75, sub, True))
        coefs, qt, lay = oracle.build_coefs(img, 75, int(sub), True)
        assert np.array_equal(ci.flat(), coefs), sub
        rec = ctx.reconstruct(ci)
        assert np.array_equal(rec, oracle.reconstruct(w, h, lay, qt, coefs)), sub
        assert abs(ctx.ssimulacra2(img, rec) - oracle.ssimulacra2(img, rec)) <= TOL
    f = ctx.find_quality_ssimulacra2(img, 75.0, 100, rcg.EncodeOptions(90, rcg.Subsampling.S420, True))
    q, _, oc, _, _, trace = oracle.search(img, 75.0, 100, int(rcg.Subsampling.S420), True)
    assert f.quality == q and np.array_equal(f.coefs.flat(), oc)


def test_workload_near_tie(ctx, oracle):
    """The 12 MP workload with the target moved 1e-9 above its third candidate's oracle score: a near tie the fast
    scorer cannot settle, decided on the exact score; same path, coefficients and file as the oracle."""
    img = synth.image(4000, 3000, 1, 3.0)
    _, _, _, _, _, trace0 = oracle.search(img, 70.0, 100, int(rcg.Subsampling.S420), True)
    target = trace0[2][1] + 1e-9
    n0 = ctx.tie_rescores()
    f = ctx.find_quality_ssimulacra2(img, target, 100, rcg.EncodeOptions(90, rcg.Subsampling.S420, True))
    q, s, coefs, qt, lay, trace = oracle.search(img, target, 100, int(rcg.Subsampling.S420), True)
    assert ctx.tie_rescores() > n0
    assert [t[0] for t in f.trace] == [t[0] for t in trace], (f.trace, trace)
    assert f.quality == q
    assert np.array_equal(f.coefs.flat(), coefs)
    a, _ = oracle.write_best(4000, 3000, lay, f.coefs.qtables, f.coefs.flat())
    b, _ = oracle.write_best(4000, 3000, lay, qt, coefs)
    assert hashlib.sha256(a).hexdigest() == hashlib.sha256(b).hexdigest()
