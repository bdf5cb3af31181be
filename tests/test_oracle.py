"""The CPU oracle pinned against the reference's golden vectors and its own unit-test known answers.

The oracle is the checker of every GPU parity test, so it is checked first: SSIMULACRA2 against the 54 golden
pairs of fixtures/ssim2/expected.csv (cli/tests/ssimulacra2.rs:10-38), the DCT / rounding / trellis known answers of
jpeg/src/dct.rs:131-211 and jpeg/src/rdo.rs:122-162, and the scorer unit tests of core/src/ssimulacra2.rs:514-634.
"""

import ctypes
import math

import numpy as np
import pytest

# cli/tests/ssimulacra2.rs:8 allows 1e-4; the restatement reproduces the ~7e-6 the reference reports for its own scorer.
GOLDEN_TOL = 1e-5


def test_golden_pairs(oracle, golden):
    worst = 0.0
    for name, ref, dist, want in golden:
        got = oracle.ssimulacra2(ref, dist)
        assert math.isfinite(got)
        worst = max(worst, abs(got - want))
        assert abs(got - want) <= GOLDEN_TOL, f"{name}: {got} vs {want}"
    assert len(golden) == 54
    assert worst < GOLDEN_TOL


def test_golden_pairs_fp64_variant(oracle, golden):
    # The FP64 oracle keeps the planes in f64 like py-ssimulacra2: it agrees with the expected scores to ~1e-10.
    for name, ref, dist, want in golden:
        assert abs(oracle.ssimulacra2(ref, dist, fp64=True) - want) < 1e-8, name


def test_identical_is_exactly_100(oracle, golden):
    for name, ref, dist, want in golden:
        if name.startswith("identical") or name == "gray_identical":
            assert oracle.ssimulacra2(ref, ref) == 100.0
            assert want == 100.0


# ---- jpeg/src/dct.rs:131-211


def _random_block(seed):
    s = seed
    b = np.zeros((8, 8), dtype=np.float32)
    for y in range(8):
        for x in range(8):
            s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
            b[y, x] = float((s >> 24) - 128)
    return b


def _naive_dct(b):
    out = np.zeros((8, 8))
    for u in range(8):
        for v in range(8):
            s = 0.0
            for y in range(8):
                for x in range(8):
                    s += (b[y, x] * math.cos((2 * x + 1) * u * math.pi / 16.0)
                          * math.cos((2 * y + 1) * v * math.pi / 16.0))
            a = lambda k: 1 / math.sqrt(2) if k == 0 else 1.0
            out[u, v] = 0.25 * a(u) * a(v) * s
    return out


def test_fdct_matches_naive_dct(oracle):
    aan = np.ctypeslib.as_array(oracle.lib().orc_aan(), shape=(8,))
    for seed in range(20):
        b = _random_block(seed)
        want = _naive_dct(b)
        got = np.ascontiguousarray(b.copy())
        oracle.lib().orc_fdct(got.ctypes.data)
        for u in range(8):
            for v in range(8):
                g = got[u, v] / (8.0 * aan[u] * aan[v])
                assert abs(g - want[u, v]) < 1e-2


def test_idct_inverts_dct(oracle):
    aan = np.ctypeslib.as_array(oracle.lib().orc_aan(), shape=(8,))
    for seed in range(20):
        b = _random_block(seed + 100)
        c = _naive_dct(b)
        inp = np.zeros((8, 8), dtype=np.float32)
        for v in range(8):
            for u in range(8):
                inp[v, u] = c[u, v] * aan[u] * aan[v]
        inp = np.ascontiguousarray(inp)
        oracle.lib().orc_idct(inp.ctypes.data)
        assert np.all(np.abs(inp - b) < 1e-2)


def test_round_f32(oracle):
    r = oracle.lib().orc_round_f32
    assert r(2.4) == 2 and r(2.6) == 3 and r(-2.6) == -3 and r(-0.4) == 0
    assert r(2.5) == 2 and r(3.5) == 4 and r(-2.5) == -2  # ties to even


# ---- jpeg/src/rdo.rs:122-162


def _flat_sizes():
    s = np.array([4 + min(i >> 4, 8) + min(i & 15, 4) for i in range(256)], dtype=np.uint8)
    s[0] = 3
    s[0xF0] = 8
    return s


def _rdo(oracle, table, kappa, sizes, a):
    out = np.zeros(64, dtype=np.int16)
    a = np.ascontiguousarray(a, dtype=np.float32)
    oracle.lib().orc_rdo_quantize_ac(np.ascontiguousarray(table).ctypes.data, ctypes.c_float(kappa),
                                     np.ascontiguousarray(sizes).ctypes.data, a.ctypes.data, out.ctypes.data)
    return out


def test_zero_lambda_equals_plain_rounding(oracle):
    a = np.array([((k * np.float32(7.3)) % np.float32(5.0)) - np.float32(2.43) for k in range(64)], dtype=np.float32)
    out = _rdo(oracle, np.full(64, 10, np.uint8), 0.0, _flat_sizes(), a)
    for k in range(1, 64):
        want = int(np.trunc(a[k] + np.float32(0.5) * np.sign(a[k])))
        assert out[k] == want, (k, a[k])


def test_large_lambda_zeroes_marginal_coefficients(oracle):
    a = np.zeros(64, dtype=np.float32)
    a[5] = 0.6
    a[1] = 9.0
    out = _rdo(oracle, np.full(64, 10, np.uint8), 4.0, _flat_sizes(), a)
    assert out[5] == 0
    assert out[1] >= 8


# ---- core/src/util/huffman.rs:10-86


def _lengths(oracle, freqs, max_len=16):
    f = np.ascontiguousarray(freqs, dtype=np.uint32)
    out = np.zeros(len(f), dtype=np.uint8)
    oracle.lib().orc_build_lengths(f.ctypes.data, len(f), max_len, out.ctypes.data)
    return out


def test_build_lengths_properties(oracle):
    rng = np.random.default_rng(0)
    for trial in range(50):
        n = int(rng.integers(2, 257))
        f = rng.integers(0, 1000, size=n).astype(np.uint32)
        f[rng.integers(0, n)] = 1
        if trial % 5 == 0:
            f = (rng.pareto(0.5, size=n) * 10).astype(np.uint32)  # skewed: exercises the length limit
        L = _lengths(oracle, f)
        used = f > 0
        assert np.all((L > 0) == used) or used.sum() == 1
        assert L.max() <= 16
        if used.sum() > 1:
            kraft = sum(2.0 ** -int(l) for l in L[used])
            assert abs(kraft - 1.0) < 1e-12  # complete code


def test_build_lengths_edge_cases(oracle):
    assert list(_lengths(oracle, [0, 0, 0])) == [0, 0, 0]
    assert list(_lengths(oracle, [0, 5, 0])) == [0, 1, 0]
    L = _lengths(oracle, [1, 1])
    assert list(L) == [1, 1]


# ---- core/src/ssimulacra2.rs:514-634


def _noise(seed):
    seed[0] = (seed[0] * 1664525 + 1013904223) & 0xFFFFFFFF
    return seed[0] >> 24


def picture(w, h, amp, seed):
    """The reference's test picture (core/src/ssimulacra2.rs:524-539)."""
    s = [seed]
    out = np.zeros((h, w, 3), dtype=np.uint8)
    for y in range(h):
        for x in range(w):
            base = [x * 255 // max(w, 1), y * 255 // max(h, 1), (x + y) * 255 // max(w + h, 1)]
            for c, b in enumerate(base):
                n = 0 if amp == 0 else int((_noise(s) - 128) * amp / 128)
                out[y, x, c] = min(max(b + n, 0), 255)
    return out


def test_more_damage_scores_lower(oracle):
    r = picture(96, 80, 0, 3)
    scores = [oracle.ssimulacra2(r, picture(96, 80, amp, 3)) for amp in (4, 16, 48, 120)]
    assert all(a > b for a, b in zip(scores, scores[1:])), scores
    assert scores[0] < 100.0


def test_awkward_sizes_give_finite_scores(oracle):
    for w, h in [(8, 8), (9, 13), (8, 100), (100, 8), (17, 33), (255, 9), (57, 55), (300, 11)]:
        assert math.isfinite(oracle.ssimulacra2(picture(w, h, 0, 5), picture(w, h, 25, 5)))


def test_small_images_are_rejected(oracle):
    with pytest.raises(ValueError):
        oracle.ssimulacra2(picture(7, 32, 0, 4), picture(7, 32, 0, 4))
    with pytest.raises(ValueError):
        oracle.ssimulacra2(picture(32, 7, 0, 4), picture(32, 7, 0, 4))


def test_gray_is_scored_as_replicated_rgb(oracle):
    w, h = 48, 40
    s = [7]
    gray = np.array([((i % w) * 5 + _noise(s) // 8) & 0xFF for i in range(w * h)], dtype=np.uint8).reshape(h, w)
    s2 = [8]
    gray2 = np.array([min(255, int(v) + _noise(s2) // 16) for v in gray.ravel()], dtype=np.uint8).reshape(h, w)
    rgb = lambda g: np.repeat(g[:, :, None], 3, axis=2)
    assert oracle.ssimulacra2(gray, gray2) == oracle.ssimulacra2(rgb(gray), rgb(gray2))


def test_sixteen_bit_replicating_eight_bit_scores_identically(oracle):
    a, b = picture(50, 44, 0, 9), picture(50, 44, 30, 9)
    up = lambda i: i.astype(np.uint16) * 257
    assert oracle.ssimulacra2(a, b) == oracle.ssimulacra2(up(a), up(b))


def test_alpha_is_composited(oracle):
    w = h = 40

    def rgba(hidden):
        d = np.zeros((h, w, 4), dtype=np.uint8)
        d[:, :20] = [200, 100, 50, 255]
        d[:, 20:] = [hidden, hidden // 2, 255 - hidden, 0]
        return d

    assert oracle.ssimulacra2(rgba(0), rgba(255)) == 100.0
    rgb = picture(w, h, 0, 11)
    with_alpha = np.concatenate([rgb, np.full((h, w, 1), 255, np.uint8)], axis=2)
    other = picture(w, h, 40, 11)
    other_a = np.concatenate([other, np.full((h, w, 1), 255, np.uint8)], axis=2)
    assert oracle.ssimulacra2(rgb, other) == oracle.ssimulacra2(with_alpha, other_a)


def test_repeated_calls_agree_bit_for_bit(oracle):
    a, b = picture(130, 97, 0, 12), picture(130, 97, 20, 12)
    assert oracle.ssimulacra2(a, b) == oracle.ssimulacra2(a, b)


# ---- encoder / decoder / search restatement


def test_oracle_encode_decode_roundtrip(oracle):
    import rcg.synth as synth

    img = synth.image(96, 72, 0)
    for sub in (1, 2, 3, 0):
        for q in (30, 75, 95, 100):
            coefs, qt, lay = oracle.build_coefs(img, q, sub, True)
            rec = oracle.reconstruct(96, 72, lay, qt, coefs)
            assert rec.shape == img.shape
            err = np.abs(rec.astype(int) - img.astype(int)).mean()
            assert err < (12 if q < 50 else 6), (sub, q, err)


def test_oracle_threads_do_not_change_results(oracle):
    import rcg.synth as synth

    img = synth.image(200, 150, 3)
    oracle.set_threads(1)
    a = oracle.build_coefs(img, 60, 3, True)[0]
    s1 = oracle.ssimulacra2(img, synth.image(200, 150, 4))
    oracle.set_threads(max(2, oracle.max_threads()))
    b = oracle.build_coefs(img, 60, 3, True)[0]
    s2 = oracle.ssimulacra2(img, synth.image(200, 150, 4))
    assert np.array_equal(a, b) and s1 == s2


def test_oracle_search_follows_bisection(oracle):
    import rcg.synth as synth

    img = synth.image(128, 96, 5)
    for target in (40.0, 60.0, 99.0):
        q, s, coefs, qt, lay, trace = oracle.search(img, target, 100, 3, True)
        assert trace[0][0] == 100
        if trace[0][1] < target:  # even the maximum quality misses: best effort (jpeg/src/target.rs:35-37)
            assert len(trace) == 1 and q == 100
            continue
        lo, hi = 1, 100
        best = 100
        for qq, ss in trace[1:]:
            assert qq == lo + (hi - lo) // 2
            if ss >= target:
                hi, best = qq, qq
            else:
                lo = qq + 1
        assert lo == hi and q == best and s >= target


def test_write_best_produces_a_jpeg(oracle):
    import rcg.synth as synth

    img = synth.image(64, 48, 1)
    coefs, qt, lay = oracle.build_coefs(img, 75, 3, True)
    data, progressive = oracle.write_best(64, 48, lay, qt, coefs)
    assert data[:2] == b"\xff\xd8" and data[-2:] == b"\xff\xd9"
    sof = b"\xff\xc2" if progressive else b"\xff\xc0"
    i = data.index(sof)
    # SOF: precision 8, height, width, 3 components with 2x2 luma sampling (jpeg/src/encode.rs:664-671)
    assert data[i + 4] == 8 and int.from_bytes(data[i + 5: i + 7], "big") == 48
    assert int.from_bytes(data[i + 7: i + 9], "big") == 64 and data[i + 9] == 3 and data[i + 11] == 0x22


def _zigzag():
    """Natural index of each zigzag position (JPEG scan order): anti-diagonals, alternating direction."""
    order = []
    for d in range(15):
        cells = [(y, d - y) for y in range(8) if 0 <= d - y < 8]
        order += cells if d % 2 else cells[::-1]
    return [y * 8 + x for y, x in order]


ZIGZAG = _zigzag()


def _general(oracle, img, q, sub):
    coefs, qt, lay = oracle.build_coefs(img, q, sub, True)
    h, w = img.shape[:2]
    return oracle.general_from_encoder(w, h, lay, qt, coefs)


def test_oracle_requantize_plain_formula_and_monotone_tables(oracle):
    """CoefImage::requantize without trellis (jpeg/src/encode.rs:118-138) restated in numpy: new table =
    max(standard table, old), coefficient = round-half-even of the f32 product with old/new, clamped to +-2047."""
    import rcg.synth as synth

    img = synth.image(72, 40, 6, sensor_sigma=3.0)
    g = _general(oracle, img, 96, 3)
    zz = np.asarray(ZIGZAG)
    for q in (20, 70, 100):
        out = oracle.requantize(g, q, trellis=False)
        off = 0
        for c in range(3):
            old = g.qtables4[g.tq[c]]
            new = out.qtables4[out.tq[c]]
            assert np.all(new >= old)
            nb = int(g.lay["blocks_w"][c] * g.lay["blocks_h"][c])
            blk = g.coefs[off: off + nb * 64].reshape(nb, 64).astype(np.float32)
            ratio = old[zz].astype(np.float32) / new[zz].astype(np.float32)
            want = np.clip(np.rint(blk * ratio[None, :]), -2047, 2047).astype(np.int16)
            assert np.array_equal(out.coefs[off: off + nb * 64].reshape(nb, 64), want), (q, c)
            off += nb * 64
        if q == 100:  # never finer than the source (cli/tests/cmyk.rs:40)
            assert np.array_equal(out.coefs, g.coefs)


def test_oracle_requantize_trellis_keeps_dc_and_shrinks(oracle):
    import rcg.synth as synth

    img = synth.image(80, 64, 7, sensor_sigma=4.0)
    g = _general(oracle, img, 95, 3)
    plain = oracle.requantize(g, 50, trellis=False)
    rdo = oracle.requantize(g, 50, trellis=True)
    a, b = plain.coefs.reshape(-1, 64), rdo.coefs.reshape(-1, 64)
    assert np.array_equal(a[:, 0], b[:, 0])  # quantize_ac writes positions 1..63 only (jpeg/src/rdo.rs:109)
    assert np.abs(b[:, 1:]).sum() <= np.abs(a[:, 1:]).sum()
    assert (b[:, 1:] != 0).sum() <= (a[:, 1:] != 0).sum()
    # an unchanged table skips the trellis pass (jpeg/src/encode.rs:151)
    same = oracle.requantize(g, 100, trellis=True)
    assert np.array_equal(same.coefs, g.coefs)


def test_oracle_search_requantize_follows_bisection(oracle):
    import rcg.synth as synth

    img = synth.image(96, 72, 8, sensor_sigma=3.0)
    g = _general(oracle, img, 95, 3)
    for target in (50.0, 80.0):
        q, s, best, trace = oracle.search_requantize(g, target, 100, True)
        assert trace[0][0] == 100
        lo, hi, want = 1, 100, 100
        for qq, ss in trace[1:]:
            assert qq == lo + (hi - lo) // 2
            if ss >= target:
                hi, want = qq, qq
            else:
                lo = qq + 1
        assert q == want and s >= target
        ref = oracle.reconstruct_general(g)
        assert abs(oracle.ssimulacra2(ref, oracle.reconstruct_general(best)) - s) < 1e-12


def _np_ssim(a, b):
    """core/src/metrics.rs:13-62 restated with numpy: integer window sums from 4x4 group sums, the f64 formula in
    the reference's order, each row of windows summed left to right, rows added in order."""
    a = a.astype(np.int64)
    b = b.astype(np.int64)
    if a.ndim == 2:
        a, b = a[:, :, None], b[:, :, None]
    h, w, ch = a.shape
    c1, c2 = 6.5025, 58.5225

    def term(sx, sy, sxx, syy, sxy, n):
        mx, my = sx / n, sy / n
        vx, vy, cov = sxx / n - mx * mx, syy / n - my * my, sxy / n - mx * my
        return ((2.0 * mx * my + c1) * (2.0 * cov + c2)) / ((mx * mx + my * my + c1) * (vx + vy + c2))

    if w < 8 or h < 8:
        total = 0.0
        for c in range(ch):
            p, q = a[:, :, c], b[:, :, c]
            total += term(*(float(x.sum()) for x in (p, q, p * p, q * q, p * q)), float(w * h))
        return total / ch
    ny, nx = (h - 8) // 4 + 1, (w - 8) // 4 + 1
    gh, gw = ny + 1, nx + 1
    vals = np.zeros((ny, nx))
    for c in range(ch):
        p = a[: 4 * gh, : 4 * gw, c]
        q = b[: 4 * gh, : 4 * gw, c]
        sums = []
        for x in (p, q, p * p, q * q, p * q):
            g = x.reshape(gh, 4, gw, 4).sum(axis=(1, 3))
            sums.append((g[:-1, :-1] + g[:-1, 1:] + g[1:, :-1] + g[1:, 1:]).astype(np.float64))
        vals = vals + term(*sums, 64.0)
    vals = vals / ch
    rows = np.zeros(ny)
    for i in range(nx):
        rows = rows + vals[:, i]
    total = 0.0
    for j in range(ny):
        total += rows[j]
    return total / (ny * nx)


def test_oracle_metrics_against_numpy_and_reference_properties(oracle):
    import rcg.synth as synth

    def img(w, h, f):
        y, x = np.mgrid[0:h, 0:w]
        return f(x, y).astype(np.uint8)

    # core/src/metrics.rs:141-175 (the reference's own tests)
    a = img(40, 33, lambda x, y: x * 5 + y * 3)
    assert abs(oracle.ssim(a, a) - 1.0) < 1e-12
    a = img(64, 64, lambda x, y: (x * 7 + y * 5) % 256)
    s = oracle.ssim(a, a // 8 * 8)
    hv = oracle.ssim(a, a // 64 * 64)
    assert s > hv and s < 1.0 and hv > -1.0
    t = img(3, 2, lambda x, y: x + y)
    assert oracle.ssim(t, t) > 0.99
    a = img(32, 32, lambda x, y: (x * 3 + y * 5) % 256)
    assert oracle.psnr(a, a) == float("inf")
    p = oracle.psnr(a, (a + 8).astype(np.uint8))
    assert 20.0 < p < 40.0
    a = img(64, 64, lambda x, y: (x * 7 + y * 11) % 256)
    same, sl = oracle.ms_ssim(a, a), oracle.ms_ssim(a, a // 16 * 16)
    assert same > 0.99 and sl < same
    # independent numpy restatement: bit-exact SSIM, exact PSNR
    for w, h, ch in ((200, 150, 3), (37, 21, 1), (64, 9, 4), (7, 30, 3), (5, 5, 2)):
        ref = synth.image(max(w, 8), max(h, 8), 12)[:h, :w]
        dist = synth.image(max(w, 8), max(h, 8), 12, sensor_sigma=6.0)[:h, :w]
        if ch == 1:
            ref, dist = ref[:, :, 0].copy(), dist[:, :, 0].copy()
        elif ch == 2:
            ref, dist = ref[:, :, :2].copy(), dist[:, :, :2].copy()
        elif ch == 4:
            ref = np.concatenate([ref, ref[:, :, :1]], 2)
            dist = np.concatenate([dist, dist[:, :, 1:2]], 2)
        assert oracle.ssim(ref, dist) == _np_ssim(ref, dist), (w, h, ch)
        d = ref.astype(np.float64) - dist.astype(np.float64)
        mse = (d * d).sum() / d.size
        assert oracle.psnr(ref, dist) == 10.0 * np.log10(255.0 * 255.0 / mse)


def _fixtures():
    import os

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "jpeg_fixtures.npz"))
    off = z["offsets"]
    return [(str(n), z["data"][off[i]: off[i + 1]].tobytes(), str(s)) for i, (n, s) in enumerate(zip(z["names"],
                                                                                                      z["shas"]))]


def test_oracle_sequential_decoder_round_trips_and_fixtures(oracle):
    """parse().into_coefs() restated: the restated writer's baseline files (with restart intervals and per-component
    scans too) decode to the coefficients written, and the reference's Huffman fixture files (sequential and
    progressive) decode to pinned coefficients that survive a baseline re-encode unchanged
    (jpeg/tests/jpeg_decode.rs:95-110)."""
    import hashlib

    import rcg.synth as synth

    img = synth.image(123, 61, 9, sensor_sigma=3.0)
    for sub in (1, 2, 3):
        coefs, qt, lay = oracle.build_coefs(img, 85, sub, True)
        g = oracle.general_from_encoder(123, 61, lay, qt, coefs)
        for ri, pc in ((0, False), (1, False), (5, True), (13, False)):
            d, ids = oracle.decode_sequential(oracle.write_jpeg_variant(g, ri, pc))
            assert np.array_equal(d.coefs, g.coefs) and (d.w, d.h) == (123, 61)
    gray = img[:, :, 0].copy()
    coefs, qt, lay = oracle.build_coefs(gray, 60, 3, True)
    g = oracle.general_from_encoder(123, 61, lay, qt, coefs)
    d, _ = oracle.decode_sequential(oracle.write_jpeg_variant(g, 3, False))
    assert np.array_equal(d.coefs, g.coefs)
    fx = _fixtures()
    assert len(fx) >= 10
    assert any(name == "rgb8_prog.jpg" for name, _, _ in fx)  # libjpeg's progressive script with refinement scans
    for name, data, sha in fx:
        d, ids = oracle.decode_sequential(data)
        assert hashlib.sha256(d.coefs.tobytes()).hexdigest() == sha, name
        again, _ = oracle.decode_sequential(oracle.write_jpeg_variant(d, 0, False))
        assert np.array_equal(again.coefs, d.coefs), name
    # corrupt and truncated files end in an error or a decode, never a crash (jpeg/tests/jpeg_decode.rs:46-62)
    data = bytearray(fx[0][1])
    rng = np.random.default_rng(3)
    for _ in range(50):
        m = bytearray(data)
        for i in rng.integers(2, len(m), 3):
            m[i] = int(rng.integers(0, 256))
        for blob in (bytes(m), bytes(m[: int(rng.integers(0, len(m) + 1))])):
            try:
                oracle.decode_sequential(blob)
            except ValueError:
                pass


def _coded_coefs(w, h, lay, coefs):
    """The coefficients a progressive file carries: single-component AC scans code only the blocks that overlap the
    image (jpeg/src/decode.rs:1255-1257), so the AC of the MCU-padding blocks reads back as 0."""
    out = np.array(coefs, copy=True)
    n = lay["ncomp"]
    hmax, vmax = max(lay["h"][:n]), max(lay["v"][:n])
    off = 0
    for c in range(n):
        bw, bh = int(lay["blocks_w"][c]), int(lay["blocks_h"][c])
        rbw = ((w * lay["h"][c] + hmax - 1) // hmax + 7) // 8
        rbh = ((h * lay["v"][c] + vmax - 1) // vmax + 7) // 8
        blk = out[off: off + bw * bh * 64].reshape(bh, bw, 64)
        blk[:, rbw:, 1:] = 0
        blk[rbh:, :, 1:] = 0
        off += bw * bh * 64
    return out


def test_oracle_progressive_decoder_round_trips(oracle):
    """decode_dc_first / dc refinement / decode_ac_first / decode_ac_refine (jpeg/src/decode.rs:1509-1601) restated:
    every candidate script of the restated progressive writer (jpeg/src/progressive.rs:242-295: spectral splits and
    successive approximation of DC, luma and chroma) decodes back to the coefficients written, for 4:2:0, 4:2:2,
    4:4:4 and gray, odd sizes with MCU padding included."""
    import rcg.synth as synth

    for w, h, sub, gray in ((200, 152, 3, False), (120, 90, 2, False), (97, 65, 1, False), (33, 17, 3, False),
                            (64, 48, 0, True)):
        img = synth.image(max(w, 16), max(h, 16), 7)[:h, :w].copy()
        if gray:
            img = np.ascontiguousarray(img[:, :, 0])
        coefs, qt, lay = oracle.build_coefs(img, 70, sub, True)
        want = _coded_coefs(w, h, lay, coefs)
        n = oracle.script_count(lay["ncomp"])
        assert n == (24 if gray else 144)
        for i in range(n):
            d, _ = oracle.decode_huffman(oracle.emit_script(w, h, lay, qt, coefs, i))
            assert np.array_equal(d.coefs, want), (w, h, sub, i)


def test_oracle_fp64_gradient_matches_central_differences(oracle):
    """The FP64 reverse-mode gradient of SSIMULACRA2 against FP64 central differences (h = 1e-3), and the
    continuous-input forward against the FP64 scorer on integer samples."""
    import rcg.synth as synth

    w, h = 96, 80
    ref = synth.image(w, h, 5)
    coefs, qt, lay = oracle.build_coefs(ref, 60, 3, True)
    dist = oracle.reconstruct(w, h, lay, qt, coefs)
    r64, d64 = ref.astype(np.float64), dist.astype(np.float64)
    assert abs(oracle.score64(r64, d64) - oracle.ssimulacra2(ref, dist, fp64=True)) < 1e-9
    s, g = oracle.grad64(r64, d64)
    rng = np.random.default_rng(0)
    step = 1e-3
    for _ in range(48):
        y, x, c = int(rng.integers(0, h)), int(rng.integers(0, w)), int(rng.integers(0, 3))
        dp, dm = d64.copy(), d64.copy()
        dp[y, x, c] += step
        dm[y, x, c] -= step
        fd = (oracle.score64(r64, dp) - oracle.score64(r64, dm)) / (2 * step)
        assert abs(fd - g[y, x, c]) <= 1e-9 + 1e-4 * abs(fd), (y, x, c, fd, g[y, x, c])


def test_oracle_weighted_trellis(oracle):
    """The perceptual mode in the oracle's trellis: all-ones weights are the plain trellis bit for bit; larger
    weights keep more (or equal) nonzero coefficients, smaller ones fewer; weights are validated against the
    layout."""
    import rcg.synth as synth

    img = synth.image(120, 88, 6, sensor_sigma=3.0)
    for sub in (1, 2, 3):
        plain, qt, lay = oracle.build_coefs(img, 70, sub, True)
        ones = np.ones(lay["ncoefs"], dtype=np.float32)
        same, _, _ = oracle.build_coefs(img, 70, sub, True, weights=ones)
        assert np.array_equal(same, plain)
        heavy, _, _ = oracle.build_coefs(img, 70, sub, True, weights=ones * 16)
        light, _, _ = oracle.build_coefs(img, 70, sub, True, weights=ones / 16)
        nz = lambda c: int(np.count_nonzero(c))
        assert nz(light) < nz(plain) < nz(heavy)
    with pytest.raises(ValueError):
        oracle.build_coefs(img, 70, 3, True, weights=np.ones(5, dtype=np.float32))
    # the search with all-ones weights is the plain search
    small = synth.image(64, 48, 7)
    a = oracle.search(small, 70.0, 100, 3, True)
    b = oracle.search(small, 70.0, 100, 3, True, weights=np.ones(oracle.layout(64, 48, 3, 50, 3)["ncoefs"],
                                                                 dtype=np.float32))
    assert a[0] == b[0] and a[5] == b[5] and np.array_equal(a[2], b[2])


def test_oracle_pullback_is_the_adjoint_of_the_decoder(oracle):
    """coef_gradient is the exact adjoint of decode_linear (<g, L f> == <L^T g, f>), and decode_linear is the
    oracle decoder (jpeg/src/decode.rs:334) without its roundings: within the accumulated rounding of the IDCT,
    upsampling and colour steps on real coefficients, for every sampling layout and Gray."""
    import rcg.synth as synth

    rng = np.random.default_rng(1)
    for w, h, c, sub, q in ((97, 61, 3, 3, 80), (64, 40, 3, 1, 85), (45, 33, 3, 2, 75), (40, 24, 1, 3, 80)):
        lay = oracle.layout(w, h, c, q, sub)
        f = rng.standard_normal(lay["ncoefs"])
        g = rng.standard_normal((h, w, 3))
        lhs = (g * oracle.decode_linear(f, w, h, lay)).sum()
        rhs = (oracle.coef_gradient(g, w, h, lay) * f).sum()
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
        img = synth.image(max(w, 8), max(h, 8), 5)[:h, :w]
        if c == 1:
            img = img[:, :, 1].copy()
        coefs, qt, lay = oracle.build_coefs(img, q, sub, True)
        dec = oracle.reconstruct(w, h, lay, qt, coefs).astype(np.float64)
        deq, off = np.zeros(lay["ncoefs"]), 0
        for ci in range(lay["ncomp"]):
            n = lay["blocks_w"][ci] * lay["blocks_h"][ci]
            t = qt[0 if ci == 0 else 1][oracle.ZIGZAG].astype(np.float64)
            deq[off * 64:(off + n) * 64] = (coefs[off * 64:(off + n) * 64].reshape(n, 64) * t).reshape(-1)
            off += n
        lin = oracle.decode_linear(deq, w, h, lay) + 128.0  # level shift (chroma's cancels in the colour step)
        if c == 1:
            lin = lin[:, :, 0]
        err = np.abs(np.clip(lin, 0, 255) - dec)
        assert err.max() <= (0.5 if c == 1 else 2.5) and err.mean() < 0.6, (w, h, sub, err.max())


def test_oracle_perceptual_weights_rule(oracle):
    """A uniform gradient gives every block the clamp of ratio 1 (weight = strength); a gradient in one block
    raises that block and its neighbours (radius 1) and lowers the rest, within the clamp."""
    lay = oracle.layout(64, 48, 1, 50, 3)
    g = np.ones((48, 64, 3))
    wts = oracle.perceptual_weights(g, 64, 48, lay, strength=0.5)
    assert np.all(wts == np.float32(0.5))
    g = np.zeros((48, 64, 3))
    g[16:24, 24:32, :] = 1.0  # block (2, 3) of the 6 x 8 grid
    wts = oracle.perceptual_weights(g, 64, 48, lay, strength=1.0, gamma=1.0, w_min=0.25, w_max=4.0, radius=1)
    per_block = wts.reshape(6, 8, 64)[:, :, 0]
    assert np.all(per_block[1:4, 2:5] == per_block[2, 3]) and per_block[2, 3] > 1.0
    assert np.all(per_block[0] == np.float32(0.25))
    assert np.all(wts.reshape(-1, 64) == wts.reshape(-1, 64)[:, :1])
    # zero gradient everywhere: ratio 1 by definition
    assert np.all(oracle.perceptual_weights(np.zeros((48, 64, 3)), 64, 48, lay, strength=2.0) == 2.0)
