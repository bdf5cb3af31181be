"""The device searches' step loops as CUDA graphs against the same searches issued as plain launches.

A search's bisection is decided on the device, so its launches depend only on the image shape, the options and the
context's buffers: the second search of a shape on a context is captured and later ones replay the graph. Replays
must give the same qualities, the same score bits and the same coefficients as plain launches, for any target (the
target lives in the device-side search state, not in the graph), and must count the same kernels.
"""

import numpy as np
import pytest

import rcg
import rcg.synth as synth

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a.quality == b.quality
    assert a.score == b.score  # same kernels, same order: the same bits
    assert a.trace == b.trace
    assert np.array_equal(a.coefs.flat(), b.coefs.flat())


def _counted(ctx, fn):
    l0 = ctx.launch_count()
    r = fn()
    return r, ctx.launch_count() - l0


def test_search_graph_replays_equal_plain_launches():
    img = synth.image(480, 352, 41, sensor_sigma=3.0)
    other = synth.image(200, 136, 42)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    with rcg.Context(0) as plain, rcg.Context(0) as g:
        plain.set_graphs(False)
        want = {t: _counted(plain, lambda: plain.find_quality_ssimulacra2(img, t, 100, opts)) for t in (70.0, 55.0)}
        want_other = plain.find_quality_ssimulacra2(other, 80.0, 100, opts)
        assert plain.graph_stats() == (0, 0)
        got = [_counted(g, lambda: g.find_quality_ssimulacra2(img, 70.0, 100, opts)) for _ in range(3)]
        # first search: plain launches; second: captured and launched; third: replayed
        assert g.graph_stats() == (1, 2)
        for f, n in got:
            _same(f, want[70.0][0])
            assert n == want[70.0][1]
        # another shape in between (plain launches: first sight), then a new target on the stored graph
        _same(g.find_quality_ssimulacra2(other, 80.0, 100, opts), want_other)
        f, n = _counted(g, lambda: g.find_quality_ssimulacra2(img, 55.0, 100, opts))
        _same(f, want[55.0][0])
        assert n == want[55.0][1]
        assert g.graph_stats() == (1, 3)


def test_ssim_goal_gray_and_weighted_searches_replay():
    img = synth.image(256, 200, 43)
    gray = np.ascontiguousarray(img[:, :, 0])
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    with rcg.Context(0) as plain, rcg.Context(0) as g:
        plain.set_graphs(False)
        lay = plain.coef_layout(256, 200, 3, rcg.EncodeOptions(50, opts.subsampling, opts.trellis))
        wts = np.random.default_rng(7).uniform(0.3, 3.0, lay.ncoefs).astype(np.float32)
        cases = [
            lambda c: c.find_quality(img, 0.97, 100, opts),
            lambda c: c.find_quality_ssimulacra2(gray, 65.0, 100, opts),
            lambda c: c.find_quality_weighted(img, 70.0, wts, 100, opts),
        ]
        for k, case in enumerate(cases):
            want = case(plain)
            for _ in range(3):
                _same(case(g), want)
            assert g.graph_stats()[0] == k + 1


def test_requantize_search_replays(oracle):
    img = synth.image(320, 213, 44, sensor_sigma=3.0)
    coefs, qt, lay = oracle.build_coefs(img, 95, int(rcg.Subsampling.S420), True)
    comps, off = [], 0
    for i in range(lay["ncomp"]):
        k = int(lay["blocks_w"][i] * lay["blocks_h"][i] * 64)
        comps.append(rcg.CoefComponent(i + 1, int(lay["h"][i]), int(lay["v"][i]), min(i, 1), int(lay["blocks_w"][i]),
                                       int(lay["blocks_h"][i]), coefs[off: off + k].copy()))
        off += k
    q4 = np.zeros((4, 64), np.uint8)
    q4[0], q4[1] = qt[0], qt[1]
    src = rcg.CoefImage(320, 213, comps, q4, np.array([1, 1, 0, 0], np.uint8))
    with rcg.Context(0) as plain, rcg.Context(0) as g:
        plain.set_graphs(False)
        for target in (70.0, 80.0):
            want = plain.find_quality_requantize(src, target)
            for _ in range(3):
                _same(g.find_quality_requantize(src, target), want)
        assert g.graph_stats() == (1, 5)


def test_graphs_off_and_profiling_use_plain_launches():
    img = synth.image(128, 96, 45)
    with rcg.Context(0) as g:
        g.set_profiling(True)
        for _ in range(3):
            g.find_quality_ssimulacra2(img, 70.0)
        g.set_profiling(False)
        assert g.graph_stats() == (0, 0)
        g.set_graphs(False)
        for _ in range(3):
            g.find_quality_ssimulacra2(img, 70.0)
        assert g.graph_stats() == (0, 0)


def test_perceptual_search_replays_both_loops():
    """The perceptual search runs a plain and a weighted step loop per call; both get their own graph."""
    img = synth.image(320, 240, 46, sensor_sigma=3.0)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    with rcg.Context(0) as plain, rcg.Context(0) as g:
        plain.set_graphs(False)
        want = plain.find_quality_perceptual(img, 70.0, 100, opts)
        for _ in range(4):
            got = g.find_quality_perceptual(img, 70.0, 100, opts)
            for a, b in ((got.plain, want.plain), (got.found, want.found)):
                assert (a.quality, a.score, a.trace) == (b.quality, b.score, b.trace)
            assert np.array_equal(got.found.coefs.flat(), want.found.coefs.flat())
            assert (got.plain_bytes, got.perceptual_bytes, got.chose_perceptual) == (
                want.plain_bytes, want.perceptual_bytes, want.chose_perceptual)
            assert np.array_equal(got.weights, want.weights)
        captures, replays = g.graph_stats()
        assert captures == 2 and replays >= 4


def test_graphs_on_a_caller_stream():
    """Captured and replayed on a stream the caller owns (the context's stream set to it), same results."""
    torch = pytest.importorskip("torch")
    img = synth.image(256, 160, 47)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    with rcg.Context(0) as plain, rcg.Context(0) as g:
        plain.set_graphs(False)
        want = plain.find_quality_ssimulacra2(img, 72.0, 100, opts)
        s = torch.cuda.Stream()
        g.set_stream(s.cuda_stream)
        for _ in range(3):
            _same(g.find_quality_ssimulacra2(img, 72.0, 100, opts), want)
        assert g.graph_stats() == (1, 2)
        g.set_stream(0)  # back to the context's own stream: the stored graph replays there too
        _same(g.find_quality_ssimulacra2(img, 72.0, 100, opts), want)
        assert g.graph_stats() == (1, 3)


def test_stream_switch_orders_work_queued_on_the_old_stream():
    """A stream switch orders the new stream after everything queued on the old one: an upload of the image queued
    on the old stream behind a long spin must land before a device search issued on the new stream reads it."""
    torch = pytest.importorskip("torch")
    w, h = 320, 240
    img = synth.image(w, h, 48)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    with rcg.Context(0) as plain, rcg.Context(0) as g:
        want = plain.find_quality_ssimulacra2(img, 72.0, 100, opts)
        lay = g.coef_layout(w, h, 3, rcg.EncodeOptions(100, rcg.Subsampling.S420, True))
        s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
        dev = torch.zeros(img.size, dtype=torch.uint8, device="cuda")
        coefs = torch.zeros(lay.ncoefs, dtype=torch.int16, device="cuda")
        host = torch.from_numpy(img.reshape(-1).copy()).pin_memory()
        torch.cuda.synchronize()
        for a, b in ((s1, s2), (s2, s1)):
            dev.zero_()
            torch.cuda.synchronize()
            g.set_stream(a.cuda_stream)
            with torch.cuda.stream(a):
                torch.cuda._sleep(100_000_000)  # tens of milliseconds of spinning ahead of the upload
                dev.copy_(host, non_blocking=True)
            g.set_stream(b.cuda_stream)
            q, s, trace = g.search_device(dev.data_ptr(), w, h, 3, 72.0, 100, opts, coefs.data_ptr(), lay.ncoefs)
            assert (q, s, trace) == (want.quality, want.score, want.trace)
        g.set_stream(0)
