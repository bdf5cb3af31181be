"""Benchmark of the --target-ssimulacra2 JPEG quality search on GB300.

Workload (one "step" = one complete search): a 4000x3000 RGB8 synthetic image (seed 1: gradients, value noise,
flat rectangles, plus Gaussian sensor noise sigma 3), target SSIMULACRA2 70, 4:2:0, trellis on, quality bisected over
1..100 (at most 8 candidates, each encoded, decoded and scored on the GPU; the bisection decision is on the device).

Reported:
  value   searches/s with the image already in HBM (rcg_search_device; output coefficients stay on the device)
  e2e     searches/s through the public C ABI with host buffers (rcg_search: 36 MB image in, the chosen
          coefficients and quantization tables out, inside the timed region)
  roofline  of the dominant kernel (ssim2_tiles) against measured HBM bandwidth, plus its FP32 view
  cpu_baseline  the CPU restatement of the reference (oracle/, OpenMP over all host cores) on one search
Timing: CUDA events on the library's stream around each step, L2 flushed (256 MB write) between steps, warm-up
steps untimed; max over ranks for N > 1 (replicas: each rank runs its own searches, no collective on the data path).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "rust-compress_gb300"))

W, H, SEED, SIGMA, TARGET = 4000, 3000, 1, 3.0, 70.0
WORKLOAD = {
    "workload": "target-ssimulacra2 search, 4000x3000 RGB8 synthetic (seed 1, sensor noise sigma 3), "
                "target 70, 4:2:0, trellis, max quality 100",
    "width": W,
    "height": H,
    "subsampling": "4:2:0",
    "target": TARGET,
    "l2": "flushed between timed steps (256 MB write)",
}
METRIC = "target-ssimulacra2 JPEG searches/s at 12MP"


def _set_size(w, h):
    global W, H
    W, H = w, h
    WORKLOAD["width"], WORKLOAD["height"] = w, h
    if (w, h) != (4000, 3000):
        WORKLOAD["workload"] = WORKLOAD["workload"].replace("4000x3000", f"{w}x{h}")


def _env_rank():
    from rcg import replicas

    return replicas.env_rank()


def _tile_capture(name="ssim2_tiles_12mp.csv"):
    """Per-launch figures of the scorer's tile kernel on the 12 MP workload, from the committed summary of its ncu
    capture (profiles/, metric,value rows); None if absent."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    out = {}
    for ln in open(path):
        k, _, v = ln.strip().partition(",")
        if k and v and k != "metric":
            out[k] = float(v)
    need = ("dram_read_bytes", "dram_write_bytes", "issue_active_pct", "fma_pipe_pct", "alu_pipe_pct", "ffma",
            "ffma2", "fadd", "fadd2", "fmul", "fmul2")
    return out if all(k in out for k in need) else None


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def run_reference(args):
    """The reference's path on the host cores: the CPU restatement (the reference cannot be built here)."""
    rank, world, _ = _env_rank()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import rcg.synth as synth

    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    img = synth.image(W, H, SEED, SIGMA)
    for _ in range(max(1, args.warmup if args.warmup < 2 else 1)):
        oracle.search(img, TARGET, 100, 3, True)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.search(img, TARGET, 100, 3, True)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = args.steps / total
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "searches/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/int16/f32 (f64 scorer)",
        "data": "synthetic", "config": WORKLOAD,
        "cpu_baseline": {"value": value, "unit": "searches/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full searches (one per step) of the workload"},
        "e2e": {"value": value, "unit": "searches/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Rust and cannot be compiled here; this times the line-by-line C++ restatement "
                "(oracle/oracle.cpp) with OpenMP in the reference's rayon shapes",
    }
    print(json.dumps(out), flush=True)


def scorer_alone(ctx, stream, timed, torch, dev, peaks, with_oracle=True, w=3840, h=2160, steps=20):
    """SSIMULACRA2 alone on a 3840x2160 pair: the original is the synthetic image (seed 0) at 4K, the distorted one
    its JPEG round trip at quality 50, 4:2:0, trellis (the bit-exact GPU codec). Images resident on the device;
    L2 flushed between calls. Reports Mpx/s, the roofline of the launch (6 B per pixel) and the error against the
    reference-exact and FP64 oracles."""
    import rcg
    import rcg.synth as synth

    ref = synth.image(w, h, 0)
    ci = ctx.build_coefs(ref, rcg.EncodeOptions(50, rcg.Subsampling.S420, True))
    dist_img = ctx.reconstruct(ci)
    d_ref = torch.from_numpy(ref).to(dev)
    d_dist = torch.from_numpy(dist_img).to(dev)
    torch.cuda.synchronize()

    def one():
        return ctx.ssimulacra2_device(d_ref.data_ptr(), d_dist.data_ptr(), w, h, 3)

    for _ in range(3):
        one()
    times, score = timed(one, steps)
    ms = sum(times) / len(times)
    ctx.set_profiling(True)
    for _ in range(5):
        one()
    n, tiles_ms = ctx.kernel_time("ssim2_tiles")
    ctx.set_profiling(False)
    tile_ms = tiles_ms / max(1, n)
    hbm = peaks.get("hbm_gbs") or 6800.0
    out = {
        "workload": "SSIMULACRA2 of a 3840x2160 RGB8 pair (synthetic seed 0 vs its q50 4:2:0 JPEG round trip)",
        "score": score, "ms_per_score": ms, "mpx_per_s": (w * h / 1e6) / (ms / 1000.0),
        "roofline": {"kernel": "ssim2_tiles", "bound": "hbm", "achieved": 6.0 * w * h / (tile_ms / 1000.0) / 1e9,
                     "peak": hbm, "unit": "GB/s", "frac": 6.0 * w * h / (tile_ms / 1000.0) / 1e9 / hbm,
                     "avg_launch_ms": tile_ms},
    }
    if with_oracle:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        oracle.set_threads(os.cpu_count() or 1)
        o = oracle.ssimulacra2(ref, dist_img)
        o64 = oracle.ssimulacra2(ref, dist_img, fp64=True)
        out.update({"oracle": o, "oracle_fp64": o64, "abs_err_vs_oracle": abs(score - o),
                    "abs_err_vs_fp64": abs(score - o64)})
    return out


def scorer_batch_workload(ctx, torch, dev, timed, n=64, steps=5):
    """SSIMULACRA2 of many pairs of uneven sizes: the batch workload's images (seeds 2..2+n-1, log-uniform
    640x480..6000x4000) against their q50 4:2:0 JPEG round trips (the bit-exact GPU codec). Device-resident pairs
    (inputs far larger than L2); one rcg_ssimulacra2_batch_device call against n rcg_ssimulacra2_device calls."""
    import rcg
    import rcg.synth as synth

    sizes = synth.log_uniform_sizes(2, n)
    imgs = synth.images([(w, h, 2 + i, 0.0) for i, (w, h) in enumerate(sizes)])
    o50 = rcg.EncodeOptions(50, rcg.Subsampling.S420, True)
    d_r = [torch.from_numpy(im).to(dev) for im in imgs]
    d_d = [torch.from_numpy(ctx.reconstruct(ctx.build_coefs(im, o50))).to(dev) for im in imgs]
    del imgs
    torch.cuda.synchronize()
    ws, hs = [w for w, _ in sizes], [h for _, h in sizes]
    rp, dp = [t.data_ptr() for t in d_r], [t.data_ptr() for t in d_d]

    def batch():
        return ctx.ssimulacra2_batch_device(rp, dp, ws, hs, [3] * n)

    def one_by_one():
        return [ctx.ssimulacra2_device(a, b, w, h, 3) for a, b, w, h in zip(rp, dp, ws, hs)]

    for _ in range(3):
        batch()
        one_by_one()
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    tb, sb = timed(batch, steps)
    tp, sp = timed(one_by_one, steps)
    clocks = sampler.stop()
    mpx = sum(w * h for w, h in sizes) / 1e6
    ctx.set_profiling(True)
    batch()
    kb = {k: ctx.kernel_time(k)[1] for k in ("to_linear_batch", "pyramid_batch", "ssim2_tiles_batch",
                                             "ssim2_reduce_batch")}
    ctx.set_profiling(False)
    ctx.set_profiling(True)
    one_by_one()
    kp = {k: ctx.kernel_time(k)[1] for k in ("to_linear", "pyramid", "ssim2_tiles", "ssim2_reduce")}
    ctx.set_profiling(False)
    del d_r, d_d
    torch.cuda.empty_cache()
    ms_b, ms_p = sum(tb) / len(tb), sum(tp) / len(tp)
    return {"workload": f"{n} pairs, log-uniform 640x480..6000x4000 ({mpx:.0f} MP), distorted = q50 4:2:0 round trip",
            "pairs": n, "megapixels": mpx, "batch_ms": ms_b, "one_by_one_ms": ms_p,
            "batch_mpx_per_s": mpx / (ms_b / 1000.0), "one_by_one_mpx_per_s": mpx / (ms_p / 1000.0),
            "batch_vs_one_by_one": ms_p / ms_b, "identical_scores": [float(x) for x in sb] == sp,
            "batch_kernels_ms": kb, "one_by_one_kernels_ms": kp, "launches_per_batch": 4,
            "launches_one_by_one": 6 * n, "clocks": clocks}


def sweep_workload(ctx, img, steps=3):
    """A rate-quality curve of the workload image (8 qualities, 4:2:0, trellis) through rcg_sweep_qualities (host
    image in, scores out) against the same curve from build_coefs + reconstruct + ssimulacra2 per quality."""
    import rcg

    qs = [95, 90, 85, 80, 75, 70, 60, 50]
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    ctx.sweep_qualities([img], qs, opts)
    t0 = time.perf_counter()
    for _ in range(steps):
        sw = ctx.sweep_qualities([img], qs, opts)[0]
    t_sweep = (time.perf_counter() - t0) / steps

    def singles():
        out = []
        for q in qs:
            ci = ctx.build_coefs(img, rcg.EncodeOptions(q, opts.subsampling, opts.trellis))
            out.append(ctx.ssimulacra2(img, ctx.reconstruct(ci)))
        return out

    singles()
    t0 = time.perf_counter()
    one = singles()
    t_single = time.perf_counter() - t0
    out = {"workload": f"rate-quality curve of the {W}x{H} workload image, qualities {qs}, 4:2:0, trellis, host buffers",
           "ms_per_curve": 1000.0 * t_sweep, "ms_per_curve_single_calls": 1000.0 * t_single,
           "speedup": t_single / t_sweep, "identical_scores": [float(x) for x in sw] == one,
           "scores": [round(float(x), 4) for x in sw]}
    # The batch workload's 64 images x the same 8 qualities: one call (images grouped, each group's 512 pairs
    # scored by one work-list launch) against one call per image.
    import rcg.synth as synth

    sizes = synth.log_uniform_sizes(2, 64)
    imgs = synth.images([(w, h, 2 + i, 0.0) for i, (w, h) in enumerate(sizes)])
    ctx.sweep_qualities(imgs[:2], qs, opts)
    t0 = time.perf_counter()
    allq = ctx.sweep_qualities(imgs, qs, opts)
    t_all = time.perf_counter() - t0
    t0 = time.perf_counter()
    per = [ctx.sweep_qualities([im], qs, opts)[0] for im in imgs]
    t_per = time.perf_counter() - t0
    mpx = sum(w * h for w, h in sizes) / 1e6
    out["image_set"] = {"workload": f"64 images (log-uniform 640x480..6000x4000, {mpx:.0f} MP) x {len(qs)} qualities",
                        "candidates": 64 * len(qs), "ms_one_call": 1000.0 * t_all, "ms_one_call_per_image": 1000.0 * t_per,
                        "candidates_per_s": 64 * len(qs) / t_all, "candidate_mpx_per_s": mpx * len(qs) / t_all,
                        "identical_scores": all(np_equal(a, b) for a, b in zip(allq, per))}
    return out


def np_equal(a, b):
    return len(a) == len(b) and all(float(x) == float(y) for x, y in zip(a, b))


def batch_workload(ctx, torch, n=64, parallel=8, steps=2, perceptual=True):
    """Many images of uneven sizes (seeds 2..2+n-1, log-uniform 640x480..6000x4000, aspect 4:3/3:2/16:9/1:1), each
    with its own target drawn uniformly from 55..85: plain searches one after another (rcg_search) against the
    concurrent rcg_search_batch. Host buffers (end to end through the C ABI); same results per image."""
    import rcg
    import rcg.synth as synth

    sizes = synth.log_uniform_sizes(2, n)
    targets = [55.0 + 30.0 * u for u in synth.uniforms(2, 40, n)]
    imgs = synth.images([(w, h, 2 + i, 0.0) for i, (w, h) in enumerate(sizes)])
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    mpx = sum(w * h for w, h in sizes) / 1e6
    ctx.search_batch(imgs, targets, 100, opts, parallel)  # warm-up: worker contexts and their workspaces
    t0 = time.perf_counter()
    for _ in range(steps):
        res_b = ctx.search_batch(imgs, targets, 100, opts, parallel)
    tb = (time.perf_counter() - t0) / steps
    # The lockstep batch: every step of every image in one work-list launch per stage (first call: plain launches,
    # second: capture, then replays).
    for _ in range(2):
        ctx.search_batch(imgs, targets, 100, opts, lockstep=True)
    t0 = time.perf_counter()
    for _ in range(steps):
        res_l = ctx.search_batch(imgs, targets, 100, opts, lockstep=True)
    tl = (time.perf_counter() - t0) / steps
    # One by one on this context: a first pass meets each shape for the first time (workspace, graph capture),
    # the second is timed.
    for im, t in zip(imgs, targets):
        ctx.find_quality_ssimulacra2(im, t, 100, opts)
    t0 = time.perf_counter()
    res_p = [ctx.find_quality_ssimulacra2(im, t, 100, opts) for im, t in zip(imgs, targets)]
    tp = time.perf_counter() - t0
    same = all(a.quality == b.quality and a.trace == b.trace for a, b in zip(res_b, res_p))
    same_l = all(a.quality == b.quality and a.trace == b.trace for a, b in zip(res_l, res_p))
    out = {"workload": f"{n} images, log-uniform 640x480..6000x4000 ({mpx:.0f} MP in all), targets U(55,85), "
                       "4:2:0, trellis", "images": n, "megapixels": mpx,
           "plain_searches_per_s": n / tp, "batch_searches_per_s": n / tb, "batch_parallel": parallel,
           "batch_vs_plain": tp / tb, "identical_results": same,
           "lockstep_searches_per_s": n / tl, "lockstep_vs_batch": tb / tl, "lockstep_identical": same_l,
           "mean_quality": sum(r.quality for r in res_b) / n}
    if perceptual:
        # The perceptual search on the same images and targets: planned file sizes of the plain result, of the
        # weighted search's result, and of what the search returns (the smaller of the two); all meet the target.
        t0 = time.perf_counter()
        res_w = [ctx.find_quality_perceptual(im, t, 100, opts) for im, t in zip(imgs, targets)]
        tw = time.perf_counter() - t0
        plain_b = [r.plain_bytes for r in res_w]
        weighted_b = [r.perceptual_bytes for r in res_w]
        returned_b = [r.perceptual_bytes if r.chose_perceptual else r.plain_bytes for r in res_w]
        mean = lambda v: sum(v) / len(v)
        out["perceptual"] = {
            "searches_per_s": n / tw,
            "mean_plain_bytes": mean(plain_b), "mean_weighted_bytes": mean(weighted_b),
            "mean_returned_bytes": mean(returned_b),
            "returned_vs_plain_pct": round(100.0 * (mean(returned_b) / mean(plain_b) - 1.0), 2),
            "weighted_vs_plain_pct": round(100.0 * (mean(weighted_b) / mean(plain_b) - 1.0), 2),
            "images_weighted_smaller": sum(1 for a, b in zip(plain_b, weighted_b) if b < a),
            "plain_same_as_batch": all(r.plain.quality == b.quality for r, b in zip(res_w, res_b)),
            # the reference returns the max quality below the target when even that misses (jpeg/src/target.rs:36-39)
            "returned_meets_target_when_plain_does": all(r.found.score >= t for r, t in zip(res_w, targets)
                                                         if r.plain.score >= t),
            "mean_returned_score_minus_plain": mean([r.found.score - r.plain.score for r in res_w])}
        # The single-search form: a four-candidate plain probe, the gradient at its best candidate, one weighted
        # search; its planned sizes against the plain results' above.
        t0 = time.perf_counter()
        res_f = [ctx.find_quality_perceptual_fast(im, t, 100, opts)[1] for im, t in zip(imgs, targets)]
        tf = time.perf_counter() - t0

        def planned(f):
            p = ctx.plan(f.coefs)
            return min(p.progressive_bytes, p.baseline_bytes)

        fast_b = [planned(f) for f in res_f]
        out["perceptual_fast"] = {
            "searches_per_s": n / tf, "vs_plain_searches_per_s": (n / tf) / out["plain_searches_per_s"],
            "mean_bytes": mean(fast_b),
            "vs_plain_pct": round(100.0 * (mean(fast_b) / mean(plain_b) - 1.0), 2),
            "images_smaller_than_plain": sum(1 for a, b in zip(plain_b, fast_b) if b < a),
            "meets_target_when_plain_does": all(f.score >= t for f, r, t in zip(res_f, res_w, targets)
                                                if r.plain.score >= t)}
    return out


def requantize_workload(ctx, img, timed, with_oracle=True, steps=5):
    """The JPEG -> JPEG search (cli/src/pipeline.rs:369-386) on the same 12 MP image: the source is its q95 4:2:0
    trellis encoding; target 70, trellis requantization. Host buffers through the public API (coefficients in,
    coefficients and tables out). CPU baseline: the oracle's search on all host threads, once."""
    import rcg

    src = ctx.build_coefs(img, rcg.EncodeOptions(95, rcg.Subsampling.S420, True))
    for _ in range(2):
        ctx.find_quality_requantize(src, TARGET)
    times, f = timed(lambda: ctx.find_quality_requantize(src, TARGET), steps)
    ms = sum(times) / len(times)
    out = {"workload": "JPEG->JPEG search: 4000x3000 seed 1 sigma 3 encoded at q95 4:2:0, target 70, trellis",
           "searches_per_s": 1000.0 / ms, "ms_per_search": ms, "quality": f.quality, "score": f.score,
           "candidates": len(f.trace)}
    if with_oracle:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        lay = {"ncomp": 3, "h": [c.h for c in src.comps], "v": [c.v for c in src.comps],
               "blocks_w": [c.blocks_w for c in src.comps], "blocks_h": [c.blocks_h for c in src.comps]}
        g = oracle.general_from_encoder(src.width, src.height, lay, src.qtables, src.flat())
        t0 = time.perf_counter()
        q, s, _, _ = oracle.search_requantize(g, TARGET)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "searches/s", "cores": threads, "kind": "port",
                               "sample": "one full search", "quality": q, "same_quality": q == f.quality}
    return out


def _pareto_bytes(curve, target):
    """Bytes at `target` on the upper-left frontier of (bytes, score) points: the cheapest size that reaches the
    score, interpolated linearly between frontier points."""
    front = []
    for b, s in sorted(curve):
        if not front or s > front[-1][1]:
            front.append((b, s))
    if front and front[0][1] >= target:
        return float(front[0][0])
    for (b0, s0), (b1, s1) in zip(front, front[1:]):
        if s0 < target <= s1:
            return b0 + (target - s0) / (s1 - s0) * (b1 - b0)
    return None


def perceptual_workload(ctx, img, timed, steps=3):
    """The perceptual trellis on the 12 MP workload, target 70, 4:2:0: the perceptual search (plain search ->
    SSIMULACRA2 gradient at its result -> coefficient weights -> weighted search -> planned sizes) through the
    public API with host buffers (a reusable coefficient buffer, no weights copied back), and the file size at equal
    score: rate-score curves (planned bytes, score) over
    qualities 50..95 for the plain trellis, the weighted trellis and a control with uniform weights of the same
    strength (no gradient), each read off its Pareto frontier at scores 60..80."""
    import numpy as np

    import rcg

    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    popts = rcg.PerceptualOptions()
    # Timed as a host that keeps one output buffer per worker and wants the encoded result only (no weights copied
    # back: the C ABI's weights argument is nullable); one more call returns the weights for the curves below.
    coefs_out = np.zeros(ctx.coef_capacity(W, H, 3, opts), dtype=np.int16)
    ctx.find_quality_perceptual(img, TARGET, 100, opts, popts, out=coefs_out, want_weights=False)
    times, _ = timed(lambda: ctx.find_quality_perceptual(img, TARGET, 100, opts, popts, out=coefs_out,
                                                         want_weights=False), steps)
    r = ctx.find_quality_perceptual(img, TARGET, 100, opts, popts)
    ms = sum(times) / len(times)
    strength = popts.strength_for(r.plain.quality)
    uniform = np.full_like(r.weights, np.float32(strength))

    def point(q, wts):
        o = rcg.EncodeOptions(q, opts.subsampling, True)
        ci = ctx.build_coefs(img, o) if wts is None else ctx.build_coefs_weighted(img, o, wts)
        s = ctx.ssimulacra2(img, ctx.reconstruct(ci))
        p = ctx.plan(ci)
        return min(p.progressive_bytes, p.baseline_bytes), s

    t0 = time.perf_counter()
    curves = {name: [point(q, wts) for q in range(50, 96)]
              for name, wts in (("plain", None), ("perceptual", r.weights), ("uniform_strength", uniform))}
    curve_s = time.perf_counter() - t0
    targets = [60.0, 65.0, 70.0, 75.0, 80.0]
    at = {name: [_pareto_bytes(c, t) for t in targets] for name, c in curves.items()}

    def change(name):
        pct = [round(100 * (b / a - 1.0), 2) if a and b else None for a, b in zip(at["plain"], at[name])]
        vals = [x for x in pct if x is not None]
        return {"per_target_pct": pct, "mean_pct": round(float(np.mean(vals)), 2) if vals else None}

    returned = r.perceptual_bytes if r.chose_perceptual else r.plain_bytes
    # the single-search form on the same image, timed the same way
    def fast():
        return ctx.find_quality_perceptual_fast(img, TARGET, 100, opts, popts, out=coefs_out, want_weights=False)

    fast()
    times_f, rf = timed(fast, steps)
    ms_f = sum(times_f) / len(times_f)
    pf = ctx.plan(rf[1].coefs)

    return {"workload": "perceptual trellis: 4000x3000 seed 1 sigma 3, target 70, 4:2:0, default options "
                        f"(strength {strength} for plain quality {r.plain.quality}, gamma {popts.gamma}, "
                        f"radius {popts.radius}, FP32 adjoint)",
            "ms_per_perceptual_search": ms, "searches_per_s": 1000.0 / ms,
            "fast": {"ms_per_search": ms_f, "searches_per_s": 1000.0 / ms_f, "probe_quality": rf[0].quality,
                     "quality": rf[1].quality, "score": rf[1].score,
                     "bytes": min(pf.progressive_bytes, pf.baseline_bytes)},
            "plain": {"quality": r.plain.quality, "score": r.plain.score, "bytes": r.plain_bytes},
            "weighted": {"bytes": r.perceptual_bytes},
            "returned": {"quality": r.found.quality, "score": r.found.score, "chose_perceptual": r.chose_perceptual,
                         "bytes": returned, "bytes_vs_plain_pct": round(100 * (returned / r.plain_bytes - 1.0), 2)},
            "equal_score": {"targets": targets, "plain_bytes": at["plain"],
                            "perceptual_vs_plain": change("perceptual"),
                            "uniform_strength_vs_plain": change("uniform_strength"),
                            "qualities": "50..95", "seconds": round(curve_s, 1)}}


def ssim_workload(ctx, img, timed, torch, dev, with_oracle=True, steps=5):
    """`--target-ssim` (jpeg/src/target.rs:24): the same 12 MP image, target SSIM 0.95, 4:2:0, trellis, host
    buffers; and SSIM alone on a device-resident 12 MP pair (the source vs its q50 round trip)."""
    import rcg

    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    for _ in range(2):
        ctx.find_quality(img, 0.95, 100, opts)
    times, f = timed(lambda: ctx.find_quality(img, 0.95, 100, opts), steps)
    ms = sum(times) / len(times)
    dist_img = ctx.reconstruct(ctx.build_coefs(img, rcg.EncodeOptions(50, rcg.Subsampling.S420, True)))
    d_a = torch.from_numpy(img).to(dev)
    d_b = torch.from_numpy(dist_img).to(dev)
    torch.cuda.synchronize()
    one = lambda: ctx.metric_device(rcg.METRIC_SSIM, d_a.data_ptr(), d_b.data_ptr(), W, H, 3)
    for _ in range(3):
        one()
    mt, score = timed(one, 10)
    out = {"workload": "--target-ssim 0.95 search of the 12 MP image (4:2:0, trellis), host buffers",
           "searches_per_s": 1000.0 / ms, "ms_per_search": ms, "quality": f.quality, "score": f.score,
           "candidates": len(f.trace), "ssim_alone_ms": sum(mt) / len(mt), "ssim_alone_score": score}
    if with_oracle:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        oracle.set_threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        o = oracle.ssim(img, dist_img)
        dt = time.perf_counter() - t0
        out["ssim_oracle"] = o
        out["ssim_abs_err"] = abs(o - score)
        out["cpu_baseline_ssim_ms"] = dt * 1000.0
    return out


def decode_workload(ctx, img, timed, torch, steps=10):
    """GPU entropy decoding of a 12 MP baseline JPEG (the workload image encoded at q90 4:2:0 with trellis, written
    with optimized Huffman tables and no restart markers) into device memory, against the oracle's sequential
    decoder on all host threads. The input file is written inside this CPU-baseline leg (the library has no JPEG
    writer), so the workload runs only when the CPU baseline does."""
    import numpy as np

    import rcg

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    coefs, qt, lay = oracle.build_coefs(img, 90, 3, True)
    g = oracle.general_from_encoder(W, H, lay, qt, coefs)
    data = oracle.write_jpeg_variant(g, 0, False)
    t0 = time.perf_counter()
    og, _ = oracle.decode_sequential(data)
    cpu_ms = (time.perf_counter() - t0) * 1000.0
    n = lay["ncoefs"]
    d_out = torch.empty(n, dtype=torch.int16, device="cuda")
    for _ in range(3):
        ctx.decode_coefs_device(data, d_out.data_ptr(), n)
    times, _ = timed(lambda: ctx.decode_coefs_device(data, d_out.data_ptr(), n), steps)
    ms = sum(times) / len(times)
    ctx.set_profiling(True)
    for _ in range(3):
        ctx.decode_coefs_device(data, d_out.data_ptr(), n)
    kern = {k: ctx.kernel_time(k)[1] / 3 for k in ("seq_sync", "seq_chain", "seq_prefix", "seq_write")}
    ctx.set_profiling(False)
    rounds = ctx.last_decode_rounds  # of the full decodes above (the header-only calls below run no rounds)
    t0 = time.perf_counter()
    for _ in range(5):
        ctx.decode_coefs_device(data, 0, 0)
    parse_ms = (time.perf_counter() - t0) * 200.0
    same = bool(np.array_equal(d_out.cpu().numpy(), og.coefs))
    return {"workload": "decode a 4000x3000 4:2:0 baseline JPEG (q90, trellis, optimized tables) to device coefficients",
            "jpeg_bytes": len(data), "ms_per_decode": ms, "mb_per_s": len(data) / 1e6 / (ms / 1000.0),
            "kernels_ms": kern, "host_parse_ms": parse_ms, "sync_rounds": rounds,
            "identical_to_oracle": same,
            "cpu_baseline": {"value": cpu_ms, "unit": "ms per decode", "cores": 1, "kind": "port",
                             "sample": "one decode of the same file (the restated sequential decoder is serial)"}}


def plan_workload(ctx, timed, d_coefs, lay, with_oracle=True, steps=10):
    """write_best's plan of the search result (device-resident coefficients of the 12 MP workload at the found
    quality): statistics of the 48 distinct candidate scans and the baseline scan, code lengths, costs, choice.
    CPU baseline: the oracle's plan + baseline estimate on all host threads."""
    for _ in range(3):
        ctx.plan_device(W, H, lay, d_coefs.data_ptr())
    times, r = timed(lambda: ctx.plan_device(W, H, lay, d_coefs.data_ptr()), steps)
    ms = sum(times) / len(times)
    ctx.set_profiling(True)
    for _ in range(3):
        ctx.plan_device(W, H, lay, d_coefs.data_ptr())
    kern = {}
    for k in ("plan_blocks", "plan_chunks", "plan_prefix", "plan_eobruns", "plan_tables", "plan_choose"):
        n, kms = ctx.kernel_time(k)
        kern[k] = kms / 3
    ctx.set_profiling(False)
    out = {"workload": "write_best plan of the 12 MP search result (48 candidate scans + baseline)",
           "ms_per_plan": ms, "kernels_ms": kern, "progressive": r.progressive,
           "progressive_bytes": r.progressive_bytes, "baseline_bytes": r.baseline_bytes, "scans": len(r.scans)}
    if with_oracle:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.build()
        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        flat = d_coefs[: lay.ncoefs].cpu().numpy()
        lay_o = {"ncomp": lay.ncomp, "h": list(lay.h)[: lay.ncomp], "v": list(lay.v)[: lay.ncomp],
                 "blocks_w": list(lay.blocks_w)[: lay.ncomp], "blocks_h": list(lay.blocks_h)[: lay.ncomp]}
        t0 = time.perf_counter()
        pe, be, best, _ = oracle.plan(W, H, lay_o, flat)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": dt * 1000.0, "unit": "ms per plan", "cores": threads, "kind": "port",
                               "sample": "one plan of the same coefficients",
                               "same_choice": (pe, be) == (r.progressive_bytes, r.baseline_bytes)}
    return out


def kernel_case(name):
    """A handful of launches of one workload on the W x H image (for ncu captures of a single kernel). The workload
    runs once untimed (first-use work: the scorer's band tuning, workspace), then again inside an NVTX range named
    "profiled", which `ncu --nvtx --nvtx-include profiled/` selects. Step loops run as plain launches."""
    import numpy as np
    import torch

    import rcg
    import rcg.synth as synth

    ctx = rcg.Context(0)
    ctx.set_graphs(False)
    img = synth.image(W, H, SEED, SIGMA)
    ci = ctx.build_coefs(img, rcg.EncodeOptions(70, rcg.Subsampling.S420, True))
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    dist = ctx.reconstruct(ci)
    pairs = [(img, dist)] + [(np.ascontiguousarray(img[: H // k, : W // k]),
                              np.ascontiguousarray(dist[: H // k, : W // k])) for k in (2, 3, 5)]

    def run(reps):
        for _ in range(reps):
            if name == "plan":
                ctx.plan(ci)
            elif name == "ssim2_batch":
                # the W x H pair plus three smaller crops of it, four times over, in one work-list call
                ctx.ssimulacra2_batch(pairs * 4)
            elif name == "perceptual":
                # one perceptual search (plain search, adjoint, pullback, weighted search, two plans)
                ctx.find_quality_perceptual(img, TARGET, 100, opts)
            elif name == "perceptual_fast":
                # one fast perceptual search (four-candidate probe, adjoint, pullback, weighted search)
                ctx.find_quality_perceptual_fast(img, TARGET, 100, opts)
            elif name == "search":
                # one search of the workload: every kernel of the timed step, once per candidate
                ctx.find_quality_ssimulacra2(img, TARGET, 100, opts)
            elif name == "ssim":
                ctx.ssim(img, dist)
            else:
                ctx.ssimulacra2(img, dist)
        ctx.synchronize()

    run(1)
    torch.cuda.nvtx.range_push("profiled")
    run(1 if name in ("perceptual", "perceptual_fast", "search") else 2)
    torch.cuda.nvtx.range_pop()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="rcg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-scorer", action="store_true", help="skip the scorer-alone measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the many-image batch measurement")
    ap.add_argument("--no-requant", action="store_true", help="skip the JPEG->JPEG search measurement")
    ap.add_argument("--no-perceptual", action="store_true", help="skip the perceptual trellis measurement")
    ap.add_argument("--kernel-case", choices=["plan", "ssim", "ssim2", "ssim2_batch", "perceptual", "perceptual_fast",
                                              "search"],
                    default=None,
                    help="profiling aid: run only a few calls of one workload at --width x --height, print nothing")
    ap.add_argument("--width", type=int, default=W, help="smaller cases for profiling only; the bench line uses 4000")
    ap.add_argument("--height", type=int, default=H)
    args = ap.parse_args()
    _set_size(args.width, args.height)
    if args.impl == "reference":
        return run_reference(args)
    if args.kernel_case:
        return kernel_case(args.kernel_case)

    import numpy as np
    import torch

    import rcg
    import rcg.synth as synth

    rank, world, local = _env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    img = synth.image(W, H, SEED, SIGMA)
    ctx = rcg.Context(local)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    opts = rcg.EncodeOptions(90, rcg.Subsampling.S420, True)
    lay = ctx.coef_layout(W, H, 3, opts)
    d_img = torch.from_numpy(img).to(dev)
    d_coefs = torch.empty(lay.ncoefs, dtype=torch.int16, device=dev)
    d_qt = torch.empty(128, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def step_device():
        return ctx.search_device(d_img.data_ptr(), W, H, 3, TARGET, 100, opts, d_coefs.data_ptr(), lay.ncoefs,
                                 d_qt.data_ptr())

    def timed(fn, k):
        times = []
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r = fn()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        return times, r

    for _ in range(args.warmup):
        step_device()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    l0 = ctx.launch_count()
    times, res = timed(step_device, args.steps)
    launches = ctx.launch_count() - l0
    clocks = sampler.stop()
    from rcg import replicas

    total_ms = replicas.max_over_ranks(sum(times), dist)
    if dist:
        dist.barrier()
    value = world * args.steps / (total_ms / 1000.0)

    # e2e: public API with host buffers (H2D image, D2H coefficients + tables) inside the timed region.
    pinned = torch.from_numpy(img).pin_memory()
    host_img = pinned.numpy()
    # The caller's reusable output buffer (a pipeline keeps one per worker): its pages stay resident, so the
    # device-to-host copy of the chosen coefficients runs at link speed.
    coefs_host = np.zeros(ctx.coef_capacity(W, H, 3, opts), dtype=np.int16)

    def step_e2e():
        return ctx.find_quality_ssimulacra2(host_img, TARGET, 100, opts, out=coefs_host)

    for _ in range(2):
        step_e2e()
    e2e_times, f = timed(step_e2e, max(3, args.steps // 2))
    e2e_ms = replicas.max_over_ranks(sum(e2e_times) / len(e2e_times), dist)
    e2e_value = world * 1000.0 / e2e_ms

    # Per-kernel times (CUDA events around every launch) over 3 more searches, for the roofline.
    ctx.set_profiling(True)
    for _ in range(3):
        step_device()
    prof = {}
    for k in ("ssim2_tiles_cached", "ssim2_tiles_store", "ssim2_tiles", "trellis", "quantize", "dequant_idct",
              "upsample_color", "pyramid", "upsample_pyramid", "ssim2_reduce", "rate_tables", "step_tables",
              "fdct_cache", "color_pad",
              "chroma_down", "to_linear"):
        n, ms = ctx.kernel_time(k)
        prof[k] = {"launches": n, "ms": ms}
    ctx.set_profiling(False)
    # The dominant kernel: the tile kernel reading the stored reference moments (every candidate after a search's
    # first; the first stores them), or the plain tile kernel when a context runs without the store.
    cached = prof["ssim2_tiles_cached"]["launches"] > 0
    tile_kernel = "ssim2_tiles_cached" if cached else "ssim2_tiles"
    tiles = prof[tile_kernel]
    peaks = _peaks()
    hbm = peaks.get("hbm_gbs")
    tile_ms = tiles["ms"] / max(1, tiles["launches"])
    alg_bytes = 6.0 * W * H  # two RGB8 images per score (full-resolution pixels)
    achieved = alg_bytes / (tile_ms / 1000.0) / 1e9
    # DRAM bytes and the compute view of one launch at this workload size, from the committed summary of an ncu
    # capture of the same kernel and workload (None for other sizes or without the summary).
    cap = (_tile_capture("ssim2_tiles_cached_12mp.csv" if cached else "ssim2_tiles_12mp.csv")
           if (W, H) == (4000, 3000) else None)
    roof = {"kernel": tile_kernel, "bound": "hbm", "achieved": achieved, "peak": hbm or 6800.0,
            "unit": "GB/s", "frac": achieved / (hbm or 6800.0),
            "traffic": cap["dram_read_bytes"] + cap["dram_write_bytes"] if cap else None,
            "peak_source": "measured" if hbm else "fallback",
            "avg_launch_ms": tile_ms,
            "note": "the scorer is FP32-ALU bound, far below the HBM roof; algorithmic bytes = 6 B per "
                    "full-resolution pixel (two RGB8 images)"}
    if cap:
        roof["traffic_source"] = (f"ncu capture of the same kernel and workload: {cap['dram_read_bytes'] / 1e6:.1f} MB "
                                  f"read + {cap['dram_write_bytes'] / 1e6:.1f} MB written per launch")
        # FP32 roof: flops per launch counted by the capture (FFMA 2, FFMA2 4, FADD/FMUL 1, FADD2/FMUL2 2 per thread
        # instruction) over the event-timed launch, against 152 SMs x 128 FP32 lanes x 2 flops x the median SM clock
        # seen while the bench ran.
        flops = (2 * cap["ffma"] + 4 * cap["ffma2"] + cap["fadd"] + 2 * cap["fadd2"] + cap["fmul"] +
                 2 * cap["fmul2"])
        mhz = (clocks or {}).get("sm_mhz") or 2070.0
        peak_fp32 = 152 * 128 * 2 * mhz * 1e6 / 1e12
        roof["compute_view"] = {
            "issue_active_pct": cap["issue_active_pct"], "fma_pipe_pct": cap["fma_pipe_pct"],
            "alu_pipe_pct": cap["alu_pipe_pct"], "fp32_gflop_per_launch": flops / 1e9,
            "fp32_tflops": flops / (tile_ms / 1000.0) / 1e12, "fp32_peak_tflops": peak_fp32,
            "fp32_frac": flops / (tile_ms / 1000.0) / 1e12 / peak_fp32,
            "fp32_peak_formula": "152 SMs x 128 lanes x 2 flops x median SM clock",
            "source": "ncu --set full of the same kernel and workload (committed summary)"}
    batch = None
    if rank == 0 and not args.no_batch:
        batch = batch_workload(ctx, torch, perceptual=not args.no_perceptual)
    scorer = None
    scorer_batch = None
    if rank == 0 and not args.no_scorer:
        scorer = scorer_alone(ctx, stream, timed, torch, dev, peaks, with_oracle=not args.no_cpu_baseline)
        scorer_batch = scorer_batch_workload(ctx, torch, dev, timed)
    plan = None
    if rank == 0:
        lay_found = ctx.coef_layout(W, H, 3, rcg.EncodeOptions(res[0], opts.subsampling, opts.trellis))
        step_device()  # leaves the last search's chosen coefficients in d_coefs
        plan = plan_workload(ctx, timed, d_coefs, lay_found, with_oracle=not args.no_cpu_baseline)
    ssim_w = None
    if rank == 0 and not args.no_requant:
        ssim_w = ssim_workload(ctx, img, timed, torch, dev, with_oracle=not args.no_cpu_baseline)
    decode = None
    if rank == 0 and not args.no_cpu_baseline and not args.no_requant:
        decode = decode_workload(ctx, img, timed, torch)
    requant = None
    if rank == 0 and not args.no_requant:
        requant = requantize_workload(ctx, img, timed, with_oracle=not args.no_cpu_baseline)
    perceptual = None
    if rank == 0 and not args.no_perceptual:
        perceptual = perceptual_workload(ctx, img, timed)
    sweep = None
    if rank == 0 and not args.no_scorer:
        sweep = sweep_workload(ctx, img)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle

            oracle.build()
            threads = os.cpu_count() or 1
            oracle.set_threads(threads)
            t0 = time.perf_counter()
            oracle.search(img, TARGET, 100, 3, True)
            dt = time.perf_counter() - t0
            cpu = {"value": 1.0 / dt, "unit": "searches/s", "cores": threads, "kind": "port",
                   "sample": "one full search of the workload"}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "searches/s", "cores": None, "kind": "port", "sample": f"failed: {e}"}
    if rank == 0:
        steps_ms = total_ms / args.steps
        out = {
            "metric": METRIC, "value": value, "unit": "searches/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": steps_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8/int16/f32 (integer+f32 codec, f32 scorer)", "data": "synthetic",
            "config": dict(WORKLOAD),
            "replicas": world,
            "e2e": {"value": e2e_value, "unit": "searches/s", "h2d_bytes_per_step": W * H * 3,
                    "d2h_bytes_per_step": int(f.coefs.flat().nbytes) + 128 + 312},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "result": {"quality": res[0], "score": res[1], "candidates": len(res[2])},
            "kernels_ms_per_search": {k: v["ms"] / 3 for k, v in prof.items() if v["launches"]},
            "scorer_mpx_per_s": (W * H / 1e6) / (tile_ms / 1000.0),
            "scorer_alone": scorer,
            "scorer_batch": scorer_batch,
            "quality_sweep": sweep,
            "batch": batch,
            "requantize": requant,
            "write_best_plan": plan,
            "target_ssim": ssim_w,
            "jpeg_decode": decode,
            "perceptual_trellis": perceptual,
        }
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
