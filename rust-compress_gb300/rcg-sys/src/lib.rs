//! Raw bindings to librcg (`include/rcg.h`): the pixel work of rust-compress's `--target-ssimulacra2` JPEG search
//! on one GB300 GPU -- `build_coefs` (jpeg/src/encode.rs:426), `reconstruct` (jpeg/src/decode.rs:334),
//! `ssimulacra2` (core/src/ssimulacra2.rs:471) and the bisection of `find_quality_with` (jpeg/src/target.rs:29) --
//! plus the JPEG -> JPEG search, `write_best`'s scan statistics, the entropy decode of sequential sources, the other
//! metrics and the opt-in perceptual trellis. Every function returns 0 or an `RCG_*` status and never aborts; the
//! message is `rcg_last_error(ctx)`. Buffers are owned by the caller; device memory by the opaque context. A context
//! is not thread-safe: give each rayon worker its own (cli/src/main.rs:57-60).
//!
//! The types mirror the header's structs field for field (`#[repr(C)]`); the header's comments give each field's
//! meaning and each function's contract.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const RCG_OK: c_int = 0;
pub const RCG_INVALID: c_int = 1;
pub const RCG_UNSUPPORTED: c_int = 2;
pub const RCG_CUDA_ERROR: c_int = 3;
pub const RCG_TIMEOUT: c_int = 4;
pub const RCG_NO_MEMORY: c_int = 5;

pub const RCG_SUB_AUTO: i32 = 0;
pub const RCG_SUB_444: i32 = 1;
pub const RCG_SUB_422: i32 = 2;
pub const RCG_SUB_420: i32 = 3;

pub const RCG_METRIC_SSIMULACRA2: c_int = 0;
pub const RCG_METRIC_SSIM: c_int = 1;
pub const RCG_METRIC_PSNR: c_int = 2;
pub const RCG_METRIC_MS_SSIM: c_int = 3;

/// Opaque context: a CUDA stream and the device workspace of one caller thread.
#[repr(C)]
pub struct RcgCtx {
    _private: [u8; 0],
}

/// jpeg::encode::EncodeOptions minus `background` (the caller flattens alpha first).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct RcgEncodeOptions {
    pub quality: i32,
    pub subsampling: i32,
    pub trellis: i32,
}

/// Block grids of the CoefImage build_coefs produces.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RcgCoefLayout {
    pub ncomp: i32,
    pub h: [i32; 3],
    pub v: [i32; 3],
    pub blocks_w: [i32; 3],
    pub blocks_h: [i32; 3],
    pub ncoefs: i64,
}

/// jpeg::target::Found plus the evaluated (quality, score) trace.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct RcgFound {
    pub quality: i32,
    pub score: f64,
    pub nsteps: i32,
    pub trace_q: [i32; 16],
    pub trace_score: [f64; 16],
}

/// Quantization tables of a general CoefImage: a slot per component, four slots.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct RcgQTables {
    pub tq: [i32; 3],
    pub qtables: [[u8; 64]; 4],
    pub present: [i32; 4],
}

/// One progressive scan (jpeg/src/progressive.rs:14-21).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RcgScan {
    pub ncomps: i32,
    pub comps: [i32; 4],
    pub ss: i32,
    pub se: i32,
    pub ah: i32,
    pub al: i32,
}

/// write_best's decision (jpeg/src/encode.rs:543-546).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct RcgPlanResult {
    pub progressive_bytes: u64,
    pub baseline_bytes: u64,
    pub progressive: i32,
    pub nscans: i32,
    pub scans: [RcgScan; 16],
    pub ndistinct: i32,
    pub distinct: [RcgScan; 48],
    pub distinct_bytes: [u64; 48],
}

/// What rcg_decode_coefs learned about a JPEG besides its coefficients.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RcgJpegInfo {
    pub width: u32,
    pub height: u32,
    pub ids: [u8; 4],
    pub scans: i32,
    pub sync_rounds: i32,
}

/// Options of the opt-in perceptual trellis.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct RcgPerceptualOptions {
    pub strength: f64,
    pub gamma: f64,
    pub w_min: f64,
    pub w_max: f64,
    pub radius: i32,
    pub keep_smaller: i32,
    pub gradient_fp64: i32,
    pub strength_by_quality: i32,
}

extern "C" {
    pub fn rcg_ctx_create(device: c_int, out: *mut *mut RcgCtx) -> c_int;
    pub fn rcg_ctx_destroy(ctx: *mut RcgCtx);
    pub fn rcg_last_error(ctx: *const RcgCtx) -> *const c_char;
    pub fn rcg_ctx_set_stream(ctx: *mut RcgCtx, stream: *mut c_void) -> c_int;
    pub fn rcg_ctx_stream(ctx: *const RcgCtx) -> *mut c_void;
    pub fn rcg_ctx_synchronize(ctx: *mut RcgCtx) -> c_int;
    pub fn rcg_ctx_set_tie_band(ctx: *mut RcgCtx, band: f64) -> c_int;
    pub fn rcg_ctx_tie_rescores(ctx: *const RcgCtx) -> u64;
    pub fn rcg_ctx_set_band_chunks(ctx: *mut RcgCtx, chunks: c_int) -> c_int;
    pub fn rcg_ctx_band_chunks(ctx: *mut RcgCtx, width: u32, height: u32) -> c_int;
    pub fn rcg_ctx_set_ref_cache(ctx: *mut RcgCtx, on: c_int) -> c_int;
    pub fn rcg_ctx_launch_count(ctx: *const RcgCtx) -> u64;
    pub fn rcg_ctx_set_profiling(ctx: *mut RcgCtx, on: c_int) -> c_int;
    pub fn rcg_ctx_kernel_time(ctx: *mut RcgCtx, name: *const c_char, launches: *mut u64,
        total_ms: *mut f64) -> c_int;
    pub fn rcg_ctx_set_graphs(ctx: *mut RcgCtx, on: c_int) -> c_int;
    pub fn rcg_ctx_graph_stats(ctx: *const RcgCtx, captures: *mut u64, replays: *mut u64) -> c_int;
    pub fn rcg_coef_layout_for(width: u32, height: u32, channels: c_int, opts: *const RcgEncodeOptions,
        out: *mut RcgCoefLayout) -> c_int;
    pub fn rcg_ssimulacra2(ctx: *mut RcgCtx, reference: *const u8, distorted: *const u8, width: u32, height: u32,
        channels: c_int, depth: c_int, score: *mut f64) -> c_int;
    pub fn rcg_ssimulacra2_device(ctx: *mut RcgCtx, d_reference: *const u8, d_distorted: *const u8, width: u32,
        height: u32, channels: c_int, score: *mut f64) -> c_int;
    pub fn rcg_ssimulacra2_exact(ctx: *mut RcgCtx, reference: *const u8, distorted: *const u8, width: u32,
        height: u32, channels: c_int, depth: c_int, score: *mut f64) -> c_int;
    pub fn rcg_ssimulacra2_batch(ctx: *mut RcgCtx, n: c_int, references: *const *const u8,
        distorted: *const *const u8, widths: *const u32, heights: *const u32, channels: *const c_int,
        depths: *const c_int, scores: *mut f64) -> c_int;
    pub fn rcg_sweep_qualities(ctx: *mut RcgCtx, n: c_int, images: *const *const u8, widths: *const u32,
        heights: *const u32, channels: *const c_int, nq: c_int, qualities: *const c_int,
        opts: *const RcgEncodeOptions, scores: *mut f64) -> c_int;
    pub fn rcg_ssimulacra2_batch_device(ctx: *mut RcgCtx, n: c_int, d_references: *const *const u8,
        d_distorted: *const *const u8, widths: *const u32, heights: *const u32, channels: *const c_int,
        depths: *const c_int, scores: *mut f64) -> c_int;
    pub fn rcg_ssimulacra2_device_noalloc(d_reference: *const u8, d_distorted: *const u8, width: u32, height: u32,
        channels: c_int, d_score: *mut f64, stream: *mut c_void) -> c_int;
    pub fn rcg_build_coefs(ctx: *mut RcgCtx, src: *const u8, width: u32, height: u32, channels: c_int,
        opts: *const RcgEncodeOptions, coefs: *mut i16, coefs_len: usize, qtables: *mut u8) -> c_int;
    pub fn rcg_reconstruct(ctx: *mut RcgCtx, width: u32, height: u32, layout: *const RcgCoefLayout,
        qtables: *const u8, coefs: *const i16, out: *mut u8, out_len: usize) -> c_int;
    pub fn rcg_search(ctx: *mut RcgCtx, src: *const u8, width: u32, height: u32, channels: c_int, target: f64,
        max_quality: c_int, opts: *const RcgEncodeOptions, found: *mut RcgFound, coefs: *mut i16, coefs_len: usize,
        qtables: *mut u8) -> c_int;
    pub fn rcg_search_device(ctx: *mut RcgCtx, d_src: *const u8, width: u32, height: u32, channels: c_int,
        target: f64, max_quality: c_int, opts: *const RcgEncodeOptions, found: *mut RcgFound, d_coefs: *mut i16,
        coefs_len: usize, d_qtables: *mut u8) -> c_int;
    pub fn rcg_reconstruct_tables(ctx: *mut RcgCtx, width: u32, height: u32, layout: *const RcgCoefLayout,
        tables: *const RcgQTables, coefs: *const i16, out: *mut u8, out_len: usize) -> c_int;
    pub fn rcg_metric_score(ctx: *mut RcgCtx, metric: c_int, reference: *const u8, candidate: *const u8, width: u32,
        height: u32, channels: c_int, score: *mut f64) -> c_int;
    pub fn rcg_metric_score_device(ctx: *mut RcgCtx, metric: c_int, d_reference: *const u8, d_candidate: *const u8,
        width: u32, height: u32, channels: c_int, score: *mut f64) -> c_int;
    pub fn rcg_ssimulacra2_grad(ctx: *mut RcgCtx, reference: *const u8, distorted: *const f32, width: u32,
        height: u32, score: *mut f64, grad: *mut f64) -> c_int;
    pub fn rcg_ssimulacra2_grad_device(ctx: *mut RcgCtx, d_reference: *const u8, d_distorted: *const f32, width: u32,
        height: u32, score: *mut f64, d_grad: *mut f64) -> c_int;
    pub fn rcg_search_metric(ctx: *mut RcgCtx, src: *const u8, width: u32, height: u32, channels: c_int,
        metric: c_int, target: f64, max_quality: c_int, opts: *const RcgEncodeOptions, found: *mut RcgFound,
        coefs: *mut i16, coefs_len: usize, qtables: *mut u8) -> c_int;
    pub fn rcg_decode_coefs(ctx: *mut RcgCtx, jpeg: *const u8, len: usize, info: *mut RcgJpegInfo,
        layout: *mut RcgCoefLayout, tables: *mut RcgQTables, coefs: *mut i16, coefs_len: usize) -> c_int;
    pub fn rcg_decode_coefs_device(ctx: *mut RcgCtx, jpeg: *const u8, len: usize, info: *mut RcgJpegInfo,
        layout: *mut RcgCoefLayout, tables: *mut RcgQTables, d_coefs: *mut i16, coefs_len: usize) -> c_int;
    pub fn rcg_search_requantize_device(ctx: *mut RcgCtx, width: u32, height: u32, layout: *const RcgCoefLayout,
        tables_in: *const RcgQTables, d_coefs_in: *const i16, metric: c_int, target: f64, max_quality: c_int,
        trellis: c_int, found: *mut RcgFound, d_coefs_out: *mut i16, coefs_len: usize,
        tables_out: *mut RcgQTables) -> c_int;
    pub fn rcg_plan(ctx: *mut RcgCtx, width: u32, height: u32, layout: *const RcgCoefLayout, coefs: *const i16,
        coefs_len: usize, result: *mut RcgPlanResult) -> c_int;
    pub fn rcg_plan_device(ctx: *mut RcgCtx, width: u32, height: u32, layout: *const RcgCoefLayout,
        d_coefs: *const i16, result: *mut RcgPlanResult) -> c_int;
    pub fn rcg_requantize(ctx: *mut RcgCtx, width: u32, height: u32, layout: *const RcgCoefLayout,
        tables_in: *const RcgQTables, coefs_in: *const i16, quality: c_int, trellis: c_int, coefs_out: *mut i16,
        coefs_len: usize, tables_out: *mut RcgQTables) -> c_int;
    pub fn rcg_search_requantize(ctx: *mut RcgCtx, width: u32, height: u32, layout: *const RcgCoefLayout,
        tables_in: *const RcgQTables, coefs_in: *const i16, metric: c_int, target: f64, max_quality: c_int,
        trellis: c_int, found: *mut RcgFound, coefs_out: *mut i16, coefs_len: usize,
        tables_out: *mut RcgQTables) -> c_int;
    pub fn rcg_search_batch(ctx: *mut RcgCtx, n: c_int, srcs: *const *const u8, widths: *const u32,
        heights: *const u32, channels: *const c_int, targets: *const f64, max_quality: c_int,
        opts: *const RcgEncodeOptions, parallel: c_int, found: *mut RcgFound, coefs: *const *mut i16,
        coefs_len: *const usize, qtables: *const *mut u8) -> c_int;
    pub fn rcg_search_batch_lockstep(ctx: *mut RcgCtx, n: c_int, srcs: *const *const u8, widths: *const u32,
        heights: *const u32, channels: *const c_int, targets: *const f64, max_quality: c_int,
        opts: *const RcgEncodeOptions, found: *mut RcgFound, coefs: *const *mut i16, coefs_len: *const usize,
        qtables: *const *mut u8) -> c_int;
    pub fn rcg_perceptual_defaults(opts: *mut RcgPerceptualOptions);
    pub fn rcg_perceptual_strength(opts: *const RcgPerceptualOptions, quality: c_int) -> f64;
    pub fn rcg_coef_gradient(ctx: *mut RcgCtx, reference: *const u8, decoded: *const u8, width: u32, height: u32,
        channels: c_int, layout: *const RcgCoefLayout, score: *mut f64, grad: *mut f64, grad_len: usize) -> c_int;
    pub fn rcg_perceptual_weights(ctx: *mut RcgCtx, reference: *const u8, decoded: *const u8, width: u32,
        height: u32, channels: c_int, layout: *const RcgCoefLayout, popts: *const RcgPerceptualOptions,
        score: *mut f64, weights: *mut f32, weights_len: usize) -> c_int;
    pub fn rcg_build_coefs_weighted(ctx: *mut RcgCtx, src: *const u8, width: u32, height: u32, channels: c_int,
        opts: *const RcgEncodeOptions, weights: *const f32, weights_len: usize, coefs: *mut i16, coefs_len: usize,
        qtables: *mut u8) -> c_int;
    pub fn rcg_search_weighted(ctx: *mut RcgCtx, src: *const u8, width: u32, height: u32, channels: c_int,
        target: f64, max_quality: c_int, opts: *const RcgEncodeOptions, weights: *const f32, weights_len: usize,
        found: *mut RcgFound, coefs: *mut i16, coefs_len: usize, qtables: *mut u8) -> c_int;
    pub fn rcg_search_perceptual(ctx: *mut RcgCtx, src: *const u8, width: u32, height: u32, channels: c_int,
        target: f64, max_quality: c_int, opts: *const RcgEncodeOptions, popts: *const RcgPerceptualOptions,
        plain: *mut RcgFound, found: *mut RcgFound, sizes: *mut u64, chose_perceptual: *mut c_int, coefs: *mut i16,
        coefs_len: usize, qtables: *mut u8, weights: *mut f32, weights_len: usize) -> c_int;
    pub fn rcg_search_perceptual_fast(ctx: *mut RcgCtx, src: *const u8, width: u32, height: u32, channels: c_int,
        target: f64, max_quality: c_int, opts: *const RcgEncodeOptions, popts: *const RcgPerceptualOptions,
        probe: *mut RcgFound, found: *mut RcgFound, coefs: *mut i16, coefs_len: usize, qtables: *mut u8,
        weights: *mut f32, weights_len: usize) -> c_int;
}
