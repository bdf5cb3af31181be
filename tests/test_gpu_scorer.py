"""SSIMULACRA2 on the GPU (through the C ABI) against the reference's golden vectors and the CPU oracle.

Tolerances: the fast scorer's bound is 1e-3 absolute against the reference's scorer (the oracle); the golden pairs also
keep the reference's own 1e-4 against py-ssimulacra2 (cli/tests/ssimulacra2.rs:8). Identical images must give exactly
100 and repeated calls must agree bit for bit (core/src/ssimulacra2.rs:542, :630).
"""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_ORACLE = 1e-3
TOL_GOLDEN = 1e-4


def test_golden_pairs(ctx, golden, oracle):
    worst_g = worst_o = 0.0
    for name, ref, dist, want in golden:
        got = ctx.ssimulacra2(ref, dist)
        orc = oracle.ssimulacra2(ref, dist)
        worst_g = max(worst_g, abs(got - want))
        worst_o = max(worst_o, abs(got - orc))
        assert abs(got - want) <= TOL_GOLDEN, f"{name}: gpu {got} golden {want}"
        assert abs(got - orc) <= TOL_ORACLE, f"{name}: gpu {got} oracle {orc}"
    print(f"worst |gpu-golden| {worst_g:.3e}  worst |gpu-oracle| {worst_o:.3e}")


def test_identical_images_score_exactly_100(ctx, golden):
    for name, ref, dist, want in golden:
        assert ctx.ssimulacra2(ref, ref) == 100.0, name
        assert ctx.ssimulacra2(dist, dist) == 100.0, name


def test_repeated_calls_agree_bit_for_bit(ctx, golden):
    _, ref, dist, _ = golden[20]
    a = ctx.ssimulacra2(ref, dist)
    for _ in range(3):
        assert ctx.ssimulacra2(ref, dist) == a


def test_errors_match_the_reference(ctx):
    import rcg

    a = np.zeros((32, 7, 3), np.uint8)
    with pytest.raises(rcg.RcgError) as e:
        ctx.ssimulacra2(a, a)
    assert e.value.status == rcg.RCG_INVALID
    with pytest.raises(rcg.RcgError):
        ctx.ssimulacra2(np.zeros((7, 32, 3), np.uint8), np.zeros((7, 32, 3), np.uint8))
    with pytest.raises(rcg.RcgError):
        ctx.ssimulacra2(np.zeros((32, 32, 3), np.uint8), np.zeros((33, 32, 3), np.uint8))
    assert math.isfinite(ctx.ssimulacra2(np.zeros((8, 8, 3), np.uint8), np.full((8, 8, 3), 5, np.uint8)))


def test_gray_16bit_and_alpha_inputs(ctx, oracle):
    from test_oracle import picture

    a, b = picture(50, 44, 0, 9), picture(50, 44, 30, 9)
    s8 = ctx.ssimulacra2(a, b)
    assert ctx.ssimulacra2(a.astype(np.uint16) * 257, b.astype(np.uint16) * 257) == s8
    g1, g2 = a[:, :, 0].copy(), b[:, :, 1].copy()
    rgb = lambda g: np.repeat(g[:, :, None], 3, axis=2)
    assert ctx.ssimulacra2(g1, g2) == ctx.ssimulacra2(rgb(g1), rgb(g2))
    alpha = np.full((44, 50, 1), 255, np.uint8)
    assert ctx.ssimulacra2(np.concatenate([a, alpha], 2), np.concatenate([b, alpha], 2)) == s8
    half = alpha.copy()
    half[:, 25:] = 0
    x = np.concatenate([a, half], 2)
    y = np.concatenate([b, half], 2)
    assert abs(ctx.ssimulacra2(x, y) - oracle.ssimulacra2(x, y)) <= TOL_ORACLE
    # 16-bit samples that do not replicate 8-bit values go through the 65536-entry table
    r16 = (a.astype(np.uint16) * 257 + 77).astype(np.uint16)
    d16 = (b.astype(np.uint16) * 257 + 1000).clip(0, 65535).astype(np.uint16)
    assert abs(ctx.ssimulacra2(r16, d16) - oracle.ssimulacra2(r16, d16)) <= TOL_ORACLE


@pytest.mark.parametrize("w,h", [(8, 8), (9, 13), (8, 300), (300, 8), (17, 33), (255, 9), (257, 255), (300, 11),
                                 (513, 385), (1000, 777)])
def test_awkward_sizes_match_the_oracle(ctx, oracle, w, h):
    import rcg.synth as synth

    ref = synth.image(w, h, 11)
    dist = synth.image(w, h, 11, sensor_sigma=6.0)
    got = ctx.ssimulacra2(ref, dist)
    want = oracle.ssimulacra2(ref, dist)
    assert abs(got - want) <= TOL_ORACLE, (w, h, got, want)


def test_large_pair_vs_oracle_and_fp64(ctx, oracle):
    """The scorer workload itself: a 3840x2160 pair (synthetic seed 0 against its q50 4:2:0 round trip through the
    reference's JPEG path), with the error against the reference-exact oracle and the FP64 oracle printed."""
    import rcg.synth as synth

    w, h = 3840, 2160
    ref = synth.image(w, h, 0)
    coefs, qt, lay = oracle.build_coefs(ref, 50, 3, True)
    dist = oracle.reconstruct(w, h, lay, qt, coefs)
    got = ctx.ssimulacra2(ref, dist)
    want = oracle.ssimulacra2(ref, dist)
    want64 = oracle.ssimulacra2(ref, dist, fp64=True)
    print(f"gpu {got:.9f} oracle {want:.9f} fp64 {want64:.9f}: |gpu - oracle| {abs(got - want):.2e}, "
          f"|gpu - fp64| {abs(got - want64):.2e}")
    assert abs(got - want) <= TOL_ORACLE
    assert abs(got - want64) <= TOL_ORACLE


def test_device_entry_point_with_unaligned_pointers(ctx, oracle):
    """rcg_ssimulacra2_device takes any device pointer: odd offsets must give the same score (scalar path)."""
    import torch

    import rcg.synth as synth

    w, h = 131, 67
    ref = synth.image(w, h, 31)
    dist = synth.image(w, h, 31, sensor_sigma=4.0)
    dev = torch.device("cuda", 0)
    n = ref.size
    buf_a = torch.zeros(n + 3, dtype=torch.uint8, device=dev)
    buf_b = torch.zeros(n + 3, dtype=torch.uint8, device=dev)
    want = oracle.ssimulacra2(ref, dist)
    for off in (0, 1, 3):
        buf_a[off: off + n] = torch.from_numpy(ref.ravel()).to(dev)
        buf_b[off: off + n] = torch.from_numpy(dist.ravel()).to(dev)
        torch.cuda.synchronize()
        got = ctx.ssimulacra2_device(buf_a.data_ptr() + off, buf_b.data_ptr() + off, w, h, 3)
        assert abs(got - want) <= TOL_ORACLE, (off, got, want)
