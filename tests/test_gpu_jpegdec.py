"""GPU entropy decoding of Huffman JPEGs against the oracle's parse().into_coefs() restatement.

Integer work: the coefficients, the table assignment, the component ids and the error behaviour must match the
oracle exactly, for every sampling layout, gray, odd sizes, restart intervals (every MCU, and irregular ones),
one scan per component, a 12 MP file (tens of thousands of self-synchronizing subsequences), the reference's own
fixture files (tests/golden/jpeg_fixtures.npz, rgb8_prog.jpg among them), progressive files of every candidate
script of the restated progressive writer (DC and AC first scans, DC and AC refinement), corrupt and truncated files;
other frame kinds answer RCG_UNSUPPORTED.
"""

import hashlib

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu


def _same(ci, g, ids=None):
    assert (ci.width, ci.height) == (g.w, g.h)
    got = ci.flat()
    if not np.array_equal(got, g.coefs):
        bad = np.nonzero(got != g.coefs)[0]
        raise AssertionError(f"{bad.size} coefficients differ, first at {bad[0]} (block {bad[0] // 64}): "
                             f"{got[bad[0]]} vs {g.coefs[bad[0]]}")
    assert [c.tq for c in ci.comps] == [int(x) for x in g.tq[: len(ci.comps)]]
    for sl in range(4):
        assert bool(ci.present[sl]) == bool(g.has_q[sl])
        if g.has_q[sl]:
            assert np.array_equal(ci.qtables[sl], g.qtables4[sl])
    if ids is not None:
        assert bytes(c.id for c in ci.comps) == ids


def _check(ctx, oracle, data):
    try:
        g, ids = oracle.decode_sequential(data)
    except ValueError as e:
        with pytest.raises(rcg.RcgError) as err:
            ctx.decode_coefs(data)
        want = rcg.RCG_INVALID if str(e) == "invalid" else rcg.RCG_UNSUPPORTED
        assert err.value.status == want, (err.value, e)
        return None
    ci = ctx.decode_coefs(data)
    _same(ci, g, ids)
    return ci


def _encoded(oracle, img, q, sub):
    coefs, qt, lay = oracle.build_coefs(img, q, int(sub), True)
    h, w = img.shape[:2]
    return oracle.general_from_encoder(w, h, lay, qt, coefs)


@pytest.mark.parametrize("sub", [rcg.Subsampling.S444, rcg.Subsampling.S422, rcg.Subsampling.S420])
@pytest.mark.parametrize("ri,per_comp", [(0, False), (1, False), (7, False), (0, True), (3, True)])
def test_decode_matches_the_oracle(ctx, oracle, sub, ri, per_comp):
    img = synth.image(245, 173, 70, sensor_sigma=3.0)
    g = _encoded(oracle, img, 88, sub)
    ci = _check(ctx, oracle, oracle.write_jpeg_variant(g, ri, per_comp))
    if not per_comp:  # single-component scans code only the blocks that overlap the image (decode.rs:1255-1257)
        assert np.array_equal(ci.flat(), g.coefs)


@pytest.mark.parametrize("w,h", [(1, 1), (7, 9), (8, 8), (17, 33), (250, 3), (3, 250)])
def test_decode_small_and_gray(ctx, oracle, w, h):
    img = synth.image(max(w, 8), max(h, 8), 71, sensor_sigma=5.0)[:h, :w].copy()
    for src in (img, img[:, :, 2].copy()):
        g = _encoded(oracle, src, 93, rcg.Subsampling.S420)
        for ri in (0, 1, 2):
            _check(ctx, oracle, oracle.write_jpeg_variant(g, ri, False))


def test_decode_12mp(ctx, oracle):
    img = synth.image(4000, 3000, 72, sensor_sigma=3.0)
    for ri, q in ((0, 92), (0, 40), (250, 75)):
        g = _encoded(oracle, img, q, rcg.Subsampling.S420)
        data = oracle.write_jpeg_variant(g, ri, False)
        ci = ctx.decode_coefs(data)
        assert np.array_equal(ci.flat(), g.coefs), (ri, q)
        print(f"q{q} ri{ri}: {len(data)} bytes, {ctx.last_decode_rounds} synchronization rounds")


def test_decode_reference_fixtures(ctx, oracle):
    from test_oracle import _fixtures

    for name, data, sha in _fixtures():
        ci = ctx.decode_coefs(data)
        assert hashlib.sha256(ci.flat().tobytes()).hexdigest() == sha, name
        g, ids = oracle.decode_sequential(data)
        _same(ci, g, ids)


def test_decode_corrupt_and_truncated(ctx, oracle):
    from test_oracle import _fixtures

    rng = np.random.default_rng(11)
    sources = [d for _, d, _ in _fixtures()[:4]]
    g = _encoded(oracle, synth.image(160, 120, 73), 70, rcg.Subsampling.S420)
    sources.append(oracle.write_jpeg_variant(g, 4, False))
    for data in sources:
        for _ in range(40):
            m = bytearray(data)
            for i in rng.integers(2, len(m), 3):
                m[i] = int(rng.integers(0, 256))
            _check(ctx, oracle, bytes(m))
            _check(ctx, oracle, bytes(m[: int(rng.integers(0, len(m) + 1))]))


def test_decode_unsupported_kinds(ctx, oracle):
    g = _encoded(oracle, synth.image(64, 48, 74), 75, rcg.Subsampling.S420)
    data = bytearray(oracle.write_jpeg_variant(g, 0, False))
    sof = data.find(b"\xff\xc0")
    for marker in (0xC3, 0xC9, 0xCA):  # lossless, arithmetic sequential, arithmetic progressive frames
        data[sof + 1] = marker
        with pytest.raises(rcg.RcgError) as e:
            ctx.decode_coefs(bytes(data))
        assert e.value.status == rcg.RCG_UNSUPPORTED
    with pytest.raises(rcg.RcgError) as e:
        ctx.decode_coefs(b"not a jpeg")
    assert e.value.status == rcg.RCG_INVALID


@pytest.mark.parametrize("w,h,sub,gray,step", [(200, 152, 3, False, 1), (120, 90, 2, False, 7), (97, 65, 1, False, 7),
                                               (33, 17, 3, False, 11), (64, 48, 0, True, 1)])
def test_decode_progressive_scripts(ctx, oracle, w, h, sub, gray, step):
    """Every `step`-th candidate script of the restated progressive writer (jpeg/src/progressive.rs:242-295): DC first
    with and without a refinement, luma and chroma spectral splits, successive approximation down to al 0."""
    img = synth.image(max(w, 16), max(h, 16), 75, sensor_sigma=2.0)[:h, :w].copy()
    if gray:
        img = np.ascontiguousarray(img[:, :, 0])
    coefs, qt, lay = oracle.build_coefs(img, 80, sub, True)
    for i in range(0, oracle.script_count(lay["ncomp"]), step):
        _check(ctx, oracle, oracle.emit_script(w, h, lay, qt, coefs, i))


def test_decode_progressive_12mp(ctx, oracle):
    """A 12 MP progressive file with successive approximation in every band (the writer's last script: DC al 1, luma
    al 2 split at 8, chroma al 1 split at 5: refinement scans for all three components)."""
    import time

    img = synth.image(4000, 3000, 76, sensor_sigma=3.0)
    coefs, qt, lay = oracle.build_coefs(img, 80, 3, True)
    n = oracle.script_count(3)
    data = oracle.emit_script(4000, 3000, lay, qt, coefs, n - 1)
    g, ids = oracle.decode_huffman(data)
    ctx.decode_coefs(data)  # warm-up
    t0 = time.perf_counter()
    ci = ctx.decode_coefs(data)
    dt = time.perf_counter() - t0
    _same(ci, g, ids)
    print(f"12 MP progressive, {len(data)} bytes: {dt * 1e3:.1f} ms")


def test_decode_corrupt_progressive(ctx, oracle):
    from test_oracle import _fixtures

    rng = np.random.default_rng(12)
    prog = [d for name, d, _ in _fixtures() if name == "rgb8_prog.jpg"]
    img = synth.image(96, 80, 77)
    coefs, qt, lay = oracle.build_coefs(img, 70, 3, True)
    prog.append(oracle.emit_script(96, 80, lay, qt, coefs, oracle.script_count(3) - 1))
    for data in prog:
        for _ in range(60):
            m = bytearray(data)
            for i in rng.integers(2, len(m), 3):
                m[i] = int(rng.integers(0, 256))
            _check(ctx, oracle, bytes(m))
            _check(ctx, oracle, bytes(m[: int(rng.integers(0, len(m) + 1))]))


def test_decoded_source_feeds_the_requantize_search(ctx, oracle):
    """JPEG -> JPEG end to end on the GPU: decode, requantize search, plan; same as the oracle's chain."""
    from test_gpu_requantize import _assert_same

    img = synth.image(640, 480, 75, sensor_sigma=3.0)
    g = _encoded(oracle, img, 95, rcg.Subsampling.S420)
    data = oracle.write_jpeg_variant(g, 0, False)
    ci = ctx.decode_coefs(data)
    f = ctx.find_quality_requantize(ci, 72.0)
    q, s, want, _ = oracle.search_requantize(oracle.decode_sequential(data)[0], 72.0)
    assert f.quality == q and abs(f.score - s) <= 1e-3
    _assert_same(f.coefs, want, "decoded source")
    p = ctx.plan(f.coefs)
    lay = {"ncomp": 3, "h": [c.h for c in f.coefs.comps], "v": [c.v for c in f.coefs.comps],
           "blocks_w": [c.blocks_w for c in f.coefs.comps], "blocks_h": [c.blocks_h for c in f.coefs.comps]}
    pe, be, best, _ = oracle.plan(f.coefs.width, f.coefs.height, lay, f.coefs.flat())
    assert (p.progressive_bytes, p.baseline_bytes, p.scans) == (pe, be, best)


def test_device_resident_jpeg_to_jpeg_chain(ctx, oracle):
    """decode -> requantize search -> plan with the coefficients never leaving the device; same results as the
    host entry points."""
    import torch

    img = synth.image(800, 600, 76, sensor_sigma=3.0)
    g = _encoded(oracle, img, 94, rcg.Subsampling.S420)
    data = oracle.write_jpeg_variant(g, 0, False)
    ci = ctx.decode_coefs(data)
    n = ci.flat().size
    src = torch.empty(n, dtype=torch.int16, device="cuda:0")
    out = torch.empty(n, dtype=torch.int16, device="cuda:0")
    w, h, lay, tables, ids = ctx.decode_coefs_device(data, src.data_ptr(), n)
    torch.cuda.synchronize()
    assert (w, h) == (800, 600) and ids == bytes(c.id for c in ci.comps)
    assert np.array_equal(src.cpu().numpy(), ci.flat())
    q, s, trace, t_out = ctx.search_requantize_device(w, h, lay, tables, src.data_ptr(), out.data_ptr(), n, 70.0)
    f = ctx.find_quality_requantize(ci, 70.0)
    assert (q, s, trace) == (f.quality, f.score, f.trace)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), f.coefs.flat())
    assert ctx.plan_device(w, h, lay, out.data_ptr()) == ctx.plan(f.coefs)


def test_decode_progressive_to_device_any_alignment(ctx, oracle):
    """rcg_decode_coefs_device into aligned and unaligned device buffers gives the oracle's coefficients."""
    import torch

    img = synth.image(200, 150, 78, sensor_sigma=2.0)
    coefs, qt, lay = oracle.build_coefs(img, 80, 3, True)
    data = oracle.emit_script(200, 150, lay, qt, coefs, oracle.script_count(3) - 1)
    g, _ = oracle.decode_huffman(data)
    n = g.coefs.size
    buf = torch.zeros(n + 8, dtype=torch.int16, device="cuda")
    for off in (0, 1, 3):  # int16 offsets: 0, 2 and 6 bytes past a 256-byte boundary
        buf.zero_()
        ctx.decode_coefs_device(data, buf.data_ptr() + 2 * off, n)
        torch.cuda.synchronize()
        got = buf[off: off + n].cpu().numpy()
        assert np.array_equal(got, g.coefs), off
