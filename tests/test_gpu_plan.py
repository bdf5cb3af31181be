"""write_best's plan on the GPU against the oracle (jpeg/src/encode.rs:543-565, jpeg/src/progressive.rs:191-351).

The plan is integer work: every distinct candidate scan must cost exactly what the reference's scan_cost gives, the
baseline estimate must match, and the chosen script must be the reference's (the first cheapest). Cases cover
encoder output at several qualities and layouts, gray, odd and tiny sizes, and synthetic coefficient images built to
stress the end-of-band runs: runs longer than 0x7FFF blocks, and refinement scans whose pending correction bits pass
the 937-bit limit many times inside one run (jpeg/src/progressive.rs:136, :184).
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu


def _coef_image(w, h, lay, coefs, qt=None):
    comps, off = [], 0
    for i in range(lay["ncomp"]):
        k = int(lay["blocks_w"][i] * lay["blocks_h"][i] * 64)
        comps.append(rcg.CoefComponent(i + 1, int(lay["h"][i]), int(lay["v"][i]), min(i, 1), int(lay["blocks_w"][i]),
                                       int(lay["blocks_h"][i]), np.ascontiguousarray(coefs[off: off + k])))
        off += k
    if qt is None:
        qt = np.ones((2, 64), np.uint8)
    return rcg.CoefImage(w, h, comps, qt)


def _check(ctx, oracle, w, h, lay, coefs):
    got = ctx.plan(_coef_image(w, h, lay, coefs))
    pe, be, best, distinct = oracle.plan(w, h, lay, coefs)
    assert [d for d, _ in got.distinct] == [d for d, _ in distinct]
    bad = [(d, a, b) for (d, a), (_, b) in zip(got.distinct, distinct) if a != b]
    assert not bad, f"scan costs differ: {bad[:5]}"
    assert got.baseline_bytes == be
    assert got.progressive_bytes == pe
    assert got.scans == best
    assert got.progressive == (be > pe)
    return got


@pytest.mark.parametrize("sub", [rcg.Subsampling.S420, rcg.Subsampling.S422, rcg.Subsampling.S444])
@pytest.mark.parametrize("q", [10, 50, 75, 90, 100])
def test_plan_of_encoder_output(ctx, oracle, sub, q):
    img = synth.image(333, 217, 41, sensor_sigma=3.0)
    coefs, qt, lay = oracle.build_coefs(img, q, int(sub), True)
    _check(ctx, oracle, 333, 217, lay, coefs)


@pytest.mark.parametrize("w,h", [(1, 1), (8, 8), (9, 7), (17, 33), (250, 3), (3, 250), (64, 48)])
def test_plan_tiny_and_odd_sizes(ctx, oracle, w, h):
    img = synth.image(max(w, 8), max(h, 8), 42, sensor_sigma=5.0)[:h, :w].copy()
    for sub in (rcg.Subsampling.S420, rcg.Subsampling.S444):
        coefs, qt, lay = oracle.build_coefs(img, 85, int(sub), True)
        _check(ctx, oracle, w, h, lay, coefs)
    coefs, qt, lay = oracle.build_coefs(img[:, :, 1].copy(), 85, 3, True)
    _check(ctx, oracle, w, h, lay, coefs)


def test_plan_gray(ctx, oracle):
    img = synth.image(400, 300, 43, sensor_sigma=4.0)[:, :, 0].copy()
    for q in (30, 95):
        coefs, qt, lay = oracle.build_coefs(img, q, 3, True)
        assert lay["ncomp"] == 1
        got = _check(ctx, oracle, 400, 300, lay, coefs)
        assert len(got.distinct) == 26


def _layout(oracle, w, h, ncomp, sub):
    return oracle.layout(w, h, ncomp, 75, int(sub))


def _random_coefs(rng, n_blocks, density, values):
    """n_blocks x 64 coefficients: each position nonzero with probability `density`, drawn from `values`."""
    c = np.zeros((n_blocks, 64), np.int16)
    mask = rng.random((n_blocks, 64)) < density
    c[mask] = rng.choice(np.asarray(values, np.int16), size=int(mask.sum()))
    return c.ravel()


def test_plan_long_end_of_band_runs(ctx, oracle):
    """A flat 2048x1536 picture: every AC band is empty, so each AC scan is one run of more than 0x7FFF blocks."""
    w, h = 2048, 1536
    lay = _layout(oracle, w, h, 3, rcg.Subsampling.S420)
    rng = np.random.default_rng(7)
    n = lay["ncoefs"] // 64
    coefs = np.zeros((n, 64), np.int16)
    coefs[:, 0] = rng.integers(-40, 40, n)
    coefs[rng.random(n) < 0.001, 5] = 3  # a few isolated symbols cut the runs at random places
    _check(ctx, oracle, w, h, lay, coefs.ravel())


def test_plan_pending_correction_bits(ctx, oracle):
    """Coefficients of magnitude 2..7 only (no magnitude 1): the al=0 refinement scans emit no symbol in most blocks,
    so correction bits pile up and the 937-bit limit cuts the runs; sparse 1s add symbol blocks in between."""
    w, h = 640, 480
    rng = np.random.default_rng(8)
    for sub in (rcg.Subsampling.S420, rcg.Subsampling.S444):
        lay = _layout(oracle, w, h, 3, sub)
        n = lay["ncoefs"] // 64
        coefs = _random_coefs(rng, n, 0.3, [-7, -5, -4, -3, -2, 2, 3, 4, 5, 6, 7]).reshape(n, 64)
        ones = rng.random((n, 64)) < 0.002
        coefs[ones] = 1
        coefs[:, 0] = rng.integers(-2047, 2048, n)
        _check(ctx, oracle, w, h, lay, coefs.ravel())


@pytest.mark.parametrize("density", [0.01, 0.1, 0.5, 0.95])
def test_plan_random_coefficients(ctx, oracle, density):
    w, h = 500, 380
    rng = np.random.default_rng(int(density * 1000))
    vals = np.concatenate([np.arange(-2047, 0), np.arange(1, 2048)])
    p = 1.0 / np.abs(vals).astype(np.float64) ** 2
    for ncomp, sub in ((3, rcg.Subsampling.S420), (3, rcg.Subsampling.S422), (1, rcg.Subsampling.S444)):
        lay = _layout(oracle, w, h, ncomp, sub)
        n = lay["ncoefs"] // 64
        c = np.zeros((n, 64), np.int16)
        mask = rng.random((n, 64)) < density
        c[mask] = rng.choice(vals, size=int(mask.sum()), p=p / p.sum())
        _check(ctx, oracle, w, h, lay, c.ravel())


def test_plan_device_entry_and_search_output(ctx, oracle):
    """rcg_plan_device on a search's device-resident result gives the same plan as the host entry."""
    import torch

    w, h = 720, 480
    img = synth.image(w, h, 44, sensor_sigma=3.0)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    f = ctx.find_quality_ssimulacra2(img, 70.0, 100, opts)
    lay = ctx.coef_layout(w, h, 3, rcg.EncodeOptions(f.quality, opts.subsampling, opts.trellis))
    d = torch.from_numpy(f.coefs.flat().copy()).to("cuda:0")
    torch.cuda.synchronize()
    got = ctx.plan_device(w, h, lay, d.data_ptr())
    want = ctx.plan(f.coefs)
    assert got == want
    lay_o = {"ncomp": 3, "h": [c.h for c in f.coefs.comps], "v": [c.v for c in f.coefs.comps],
             "blocks_w": [c.blocks_w for c in f.coefs.comps], "blocks_h": [c.blocks_h for c in f.coefs.comps]}
    _check(ctx, oracle, w, h, lay_o, f.coefs.flat())


def test_plan_errors(ctx):
    ci = rcg.CoefImage(16, 16, [rcg.CoefComponent(1, 1, 1, 0, 2, 2, np.zeros(4 * 64, np.int16))],
                       np.ones((2, 64), np.uint8))
    ctx.plan(ci)
    with pytest.raises(rcg.RcgError):
        ctx.plan(rcg.CoefImage(70000, 16, ci.comps, ci.qtables))
    short = rcg.CoefImage(17, 16, ci.comps, ci.qtables)  # needs a 3x2 block grid
    with pytest.raises(rcg.RcgError) as e:
        ctx.plan(short)
    assert e.value.status == rcg.RCG_INVALID
