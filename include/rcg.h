/*
 * rcg — GB300 (sm_103a) implementation of rust-compress's JPEG `--target-ssimulacra2` quality search.
 *
 * C ABI. Plain pointers and sizes only; every call returns an rcg_status and never aborts the process. Buffers
 * passed in are owned by the caller and never freed here. Device memory is owned by an opaque rcg_ctx. A context
 * holds its own CUDA stream and workspace and is not thread-safe: use one context per calling thread (the
 * reference runs one search per rayon worker, cli/src/main.rs:57-60). Contexts share no mutable state; the only
 * global state is the fixed scratch array of rcg_ssimulacra2_device_noalloc (see there).
 *
 * Image data: 8-bit samples, interleaved, row-major, no row padding (rc_core::image::Image, core/src/image.rs:103-113).
 * `channels` is 1 (Gray) or 3 (Rgb) for the encoder and the search (the reference encodes flattened 8-bit Gray/Rgb
 * images, jpeg/src/encode.rs:424-426); the scorer also takes 2 (GrayAlpha) and 4 (Rgba) and 16-bit samples
 * (big-endian), as core/src/ssimulacra2.rs:177-221 does.
 *
 * Coefficients: the flat form of jpeg::encode::CoefImage (jpeg/src/encode.rs:56-83). Components are stored back to
 * back (Y, then Cb, then Cr); each holds blocks_w*blocks_h blocks in raster order over the MCU-padded grid, 64
 * zigzag-ordered int16 per block. Quantization tables are natural order, slot 0 luma, slot 1 chroma.
 */
#ifndef RCG_H
#define RCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference's rc_core::error::Error::{Invalid, Unsupported} (core/src/error.rs:4-20) map to
 * RCG_INVALID and RCG_UNSUPPORTED; rcg_last_error() gives the message. */
typedef enum {
  RCG_OK = 0,
  RCG_INVALID = 1,      /* bad sizes, mismatched images, <8x8 for the scorer, null pointers, short buffers */
  RCG_UNSUPPORTED = 2,  /* a format the path does not handle (e.g. >65535 pixels for JPEG) */
  RCG_CUDA_ERROR = 3,   /* a CUDA runtime error; the context stays usable if the device does */
  RCG_TIMEOUT = 4,      /* a bounded device-side wait gave up */
  RCG_NO_MEMORY = 5     /* device allocation failed */
} rcg_status;

/* jpeg::encode::Subsampling (jpeg/src/encode.rs:12-20). AUTO is 4:2:0 below quality 90, else 4:4:4. */
typedef enum { RCG_SUB_AUTO = 0, RCG_SUB_444 = 1, RCG_SUB_422 = 2, RCG_SUB_420 = 3 } rcg_subsampling;

/* jpeg::encode::EncodeOptions (jpeg/src/encode.rs:22-37), minus `background`: the caller flattens alpha first, as
 * cli/src/pipeline.rs:236 does before the search. */
typedef struct {
  int32_t quality;     /* 1..=100 */
  int32_t subsampling; /* rcg_subsampling */
  int32_t trellis;     /* nonzero: rate-distortion optimized AC quantization (default on in the reference) */
} rcg_encode_options;

/* Block-grid layout of the CoefImage that build_coefs produces (jpeg/src/encode.rs:440-443, :511-513). */
typedef struct {
  int32_t ncomp;       /* 1 (Gray) or 3 (YCbCr) */
  int32_t h[3], v[3];  /* sampling factors per component */
  int32_t blocks_w[3]; /* block-grid width, padded to whole MCUs */
  int32_t blocks_h[3];
  int64_t ncoefs;      /* total int16 coefficients over all components (= 64 * total blocks) */
} rcg_coef_layout;

/* jpeg::target::Found (jpeg/src/target.rs:12-18) plus the trace of evaluated candidates. */
typedef struct {
  int32_t quality;
  double score;
  int32_t nsteps;         /* candidates evaluated (max quality first, then the bisection steps) */
  int32_t trace_q[16];    /* quality of each evaluated candidate, in order */
  double trace_score[16]; /* its SSIMULACRA2 score (-DBL_MAX when it could not be scored) */
} rcg_found;

/* Quantization tables of a general CoefImage (jpeg/src/encode.rs:63, :77-78): each component names a table slot. */
typedef struct {
  int32_t tq[3];          /* table slot of each component */
  uint8_t qtables[4][64]; /* natural order, by slot */
  int32_t present[4];     /* nonzero where the slot holds a table (an absent source table counts as all ones) */
} rcg_qtables;

/* Image metrics (cli/src/pipeline.rs:130-138). SSIMULACRA2 and SSIM are the JPEG search goals
 * (cli/src/pipeline.rs:197-222). */
typedef enum {
  RCG_METRIC_SSIMULACRA2 = 0, /* core/src/ssimulacra2.rs:471 */
  RCG_METRIC_SSIM = 1,        /* core/src/metrics.rs:13 */
  RCG_METRIC_PSNR = 2,        /* core/src/metrics.rs:67 */
  RCG_METRIC_MS_SSIM = 3      /* core/src/metrics.rs:111 */
} rcg_metric;

/* One progressive scan (jpeg/src/progressive.rs:14-21): components, spectral band ss..se, successive approximation
 * ah/al. */
typedef struct {
  int32_t ncomps;
  int32_t comps[4];
  int32_t ss, se, ah, al;
} rcg_scan;

/* write_best's decision (jpeg/src/encode.rs:543-546): progressive::plan (jpeg/src/progressive.rs:335-351) and
 * baseline_estimate (jpeg/src/encode.rs:548-565). */
typedef struct {
  uint64_t progressive_bytes; /* estimated size of the best script */
  uint64_t baseline_bytes;    /* estimated size of the baseline encoding */
  int32_t progressive;        /* 1: write the script (baseline_bytes > progressive_bytes); 0: write baseline */
  int32_t nscans;             /* the best script, in order */
  rcg_scan scans[16];
  int32_t ndistinct;          /* every distinct candidate scan, in first-appearance order, with its cost */
  rcg_scan distinct[48];
  uint64_t distinct_bytes[48];
} rcg_plan_result;

/* What rcg_decode_coefs learned about a JPEG besides its coefficients. */
typedef struct {
  uint32_t width, height;
  uint8_t ids[4]; /* component identifiers (SOF order) */
  int32_t scans;  /* scans decoded */
  int32_t sync_rounds; /* most synchronization rounds a scan needed (-1: a scan fell back to the serial chain) */
} rcg_jpeg_info;

typedef struct rcg_ctx rcg_ctx;

/* Context lifetime. `device` is a CUDA device ordinal. */
int rcg_ctx_create(int device, rcg_ctx** out);
void rcg_ctx_destroy(rcg_ctx* ctx);
/* Message of the last failed call on this context ("" if none). Valid until the next call on it. */
const char* rcg_last_error(const rcg_ctx* ctx);
/* Run the context's work on a caller stream (a cudaStream_t; NULL restores the context's own stream). The switch
 * is ordered on the device: later work on the new stream waits for everything queued on the old one (an event
 * recorded on the old stream, waited on by the new one), because both use the same context buffers. The host is
 * not blocked. When either stream is being captured into a graph, that ordering is the capturing caller's. */
int rcg_ctx_set_stream(rcg_ctx* ctx, void* stream);
void* rcg_ctx_stream(const rcg_ctx* ctx);
int rcg_ctx_synchronize(rcg_ctx* ctx);
/* Near-tie band of the SSIMULACRA2 searches (rcg_search*, rcg_search_requantize*, the weighted and perceptual
 * searches): jpeg/src/target.rs:48 accepts a candidate on score >= target, and the fast f32 scorer is within about
 * 1e-6 of the reference, so a candidate whose fast score lies within `band` of the target is decided on its
 * reference-order FP64 score (rcg_ssimulacra2_exact) instead, and that score is the one reported. Default 1e-3;
 * 0 decides every candidate on the fast score; INFINITY decides every candidate on the exact score. */
int rcg_ctx_set_tie_band(rcg_ctx* ctx, double band);
/* Candidates this context has decided on the exact score so far. */
uint64_t rcg_ctx_tie_rescores(const rcg_ctx* ctx);
/* The fast scorer's CTA shape. No counterpart option in the reference; its own shape parameter is the 96-row stripe
 * of core/src/ssimulacra2.rs:33. Each CTA walks a band 32 columns wide and `chunks` x 32 rows tall, computing the XYB
 * of the rows it shares between chunks once. 0 (the default) autotunes: the first image of each size class (scale-0
 * tiles in half-octave steps) on a device times the candidates 1, 2, 4 and 8 and the fastest is kept for the
 * process; images under about 1 MP always use 1 (plain 32x32 tiles). A fixed 1..64 applies to every image this
 * context scores. Scores move by about 1e-9 between shapes; for one shape they are the same bits every call. */
int rcg_ctx_set_band_chunks(rcg_ctx* ctx, int chunks);
/* The chunks per band this context uses for a width x height image (autotuning its size class first if needed);
 * 0 for sizes the scorer rejects. */
int rcg_ctx_band_chunks(rcg_ctx* ctx, uint32_t width, uint32_t height);
/* The SSIMULACRA2 searches' reference moments: 1 on (the default), 0 off. No counterpart in the reference, which
 * recomputes everything per candidate (core/src/ssimulacra2.rs:339-452 from jpeg/src/target.rs:29-56). The
 * scorer's blurred reference-only moments depend on the reference image alone, so a search's first candidate stores
 * them (24 KB per 32x32 chunk of the scorer's layout: about 2x the reference's f32 pyramid, 388 MB at 12 MP, in the
 * context's workspace) and the later candidates read them instead of blurring them: 547 against 585 us per 12 MP
 * candidate score, 613 for the first. Scores are the same bits either way. Off: nothing is stored or allocated. */
int rcg_ctx_set_ref_cache(rcg_ctx* ctx, int on);
/* Kernels this context has launched so far (each kernel launch counts once). */
uint64_t rcg_ctx_launch_count(const rcg_ctx* ctx);
/* Per-kernel timing with CUDA events around every launch, for profiling: 1 on, 0 off. Off by default. */
int rcg_ctx_set_profiling(rcg_ctx* ctx, int on);
/* Accumulated event time of kernel `name` since profiling was switched on. Synchronizes the context. */
int rcg_ctx_kernel_time(rcg_ctx* ctx, const char* name, uint64_t* launches, double* total_ms);
/* CUDA graphs for the device searches' step loops (rcg_search*, rcg_search_requantize*): 1 on (the default), 0 off.
 * The bisection is decided on the device, so a search's launches depend only on the image shape, the options and
 * the context's buffers. The second search of a shape on a context is captured; later ones replay it, one graph
 * launch per search. Results are the same either way. Graphs are not used while profiling is on, on the legacy
 * default stream, or while the caller captures the context's stream. Replaces nothing in the reference (a rayon
 * CPU loop has no launches to batch). Synchronizes the context. */
int rcg_ctx_set_graphs(rcg_ctx* ctx, int on);
/* Step loops captured into graphs, and graph launches, on this context so far (no reference counterpart). */
int rcg_ctx_graph_stats(const rcg_ctx* ctx, uint64_t* captures, uint64_t* replays);

/* Coefficient layout for an image and options. Replaces nothing in the reference: it sizes the caller-allocated
 * output buffers that a Rust `Vec<i16>` would otherwise grow (jpeg/src/encode.rs:440-517). */
int rcg_coef_layout_for(uint32_t width, uint32_t height, int channels, const rcg_encode_options* opts,
                        rcg_coef_layout* out);

/* rc_core::ssimulacra2::ssimulacra2(reference, distorted) -> Result<f64> (core/src/ssimulacra2.rs:471).
 * Host buffers of width*height*channels*(depth/8) bytes. Errors as the reference: RCG_INVALID for a size mismatch
 * (here: impossible, one size is passed), sides < 8, or a non-finite score. */
int rcg_ssimulacra2(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* distorted, uint32_t width,
                    uint32_t height, int channels, int depth, double* score);
/* The same on device buffers (8-bit Gray/Rgb only); no host<->device copies besides the 8-byte score. */
int rcg_ssimulacra2_device(rcg_ctx* ctx, const uint8_t* d_reference, const uint8_t* d_distorted, uint32_t width,
                           uint32_t height, int channels, double* score);
/* rc_core::ssimulacra2::ssimulacra2 (core/src/ssimulacra2.rs:471) in the reference's own arithmetic and order on the
 * GPU: f32 linear planes and pyramid (2x2 means summed in f64), f64 XYB, blurs and maps, and the per-96-row-stripe
 * sums added in the reference's order (:339-466), no FMA contraction. Equal to the reference's score up to the last
 * bits of cbrt/pow (the reference calls the platform libm). Much slower than rcg_ssimulacra2 (FP64 plus serial stripe
 * sums: tens of milliseconds at 12 MP); the searches use it to decide near ties (rcg_ctx_set_tie_band). Same
 * arguments and errors as rcg_ssimulacra2. */
int rcg_ssimulacra2_exact(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* distorted, uint32_t width,
                          uint32_t height, int channels, int depth, double* score);
/* n calls of rc_core::ssimulacra2::ssimulacra2 (core/src/ssimulacra2.rs:471), one per pair, as a caller scoring many
 * files or many candidates does (cli/tests/ssimulacra2.rs:12-31 loops over 54 fixture pairs of different sizes;
 * cli/src/pipeline.rs:130-138 scores each candidate of each file). Pairs may differ in size and format
 * (widths/heights/channels/depths per pair; depths NULL = all 8-bit). All pairs go through one launch per stage
 * over a work-list of every pair's tiles; pairs that pass the same reference buffer with the same size and format
 * share one conversion of it. scores[i] equals what rcg_ssimulacra2 gives for pair i. Errors as rcg_ssimulacra2,
 * naming the first pair at fault; scores of every pair are written even when one of them is not finite (NaN there,
 * RCG_INVALID returned). n = 0 does nothing. */
int rcg_ssimulacra2_batch(rcg_ctx* ctx, int n, const uint8_t* const* references, const uint8_t* const* distorted,
                          const uint32_t* widths, const uint32_t* heights, const int* channels, const int* depths,
                          double* scores);
/* A rate-quality curve: for each of n 8-bit Gray/Rgb host images and each of nq qualities (1..=100, any order), the
 * SSIMULACRA2 score of the image against its candidate at that quality, scores[i * nq + k] =
 * ssimulacra2(image_i, reconstruct(build_coefs(image_i, {qualities[k], opts->subsampling, opts->trellis}))), the
 * value jpeg::target::find_quality_with would get for that quality (jpeg/src/target.rs:29-56 evaluates them one at a
 * time; this has no single-call counterpart in the reference). Each image's FDCT is computed once; its candidates are
 * decoded on the device and scored together by the work-list scorer, sharing one conversion of the image. Errors as
 * rcg_search for the image (RCG_INVALID for sides < 8 or a non-finite score, naming the image). */
int rcg_sweep_qualities(rcg_ctx* ctx, int n, const uint8_t* const* images, const uint32_t* widths,
                        const uint32_t* heights, const int* channels, int nq, const int* qualities,
                        const rcg_encode_options* opts, double* scores);
/* The same with device images (arrays of device pointers, sizes and scores on the host). */
int rcg_ssimulacra2_batch_device(rcg_ctx* ctx, int n, const uint8_t* const* d_references,
                                 const uint8_t* const* d_distorted, const uint32_t* widths, const uint32_t* heights,
                                 const int* channels, const int* depths, double* scores);

/* SSIMULACRA 2 of two 8-bit Gray/Rgb images already on the device, for callers that cannot allocate device memory:
 * this call allocates nothing. No counterpart in the reference (which has no device memory at all); it exists for
 * hosts that own every device allocation themselves -- a framework whose caching allocator holds a fixed device
 * budget, or a latency-critical loop where cudaMalloc/cudaFree would synchronize the whole device -- and so cannot let
 * a library call cudaMalloc. It needs no rcg_ctx. Scratch lives in one fixed device array compiled into the library
 * (about 10 MB). CUDA loads a module's device arrays onto a device when the module is first used there, so the array
 * is reserved on every device where any scorer call (allocating or not) has run, until the process exits; images are limited to
 * width*height <= 262144 pixels (e.g. 512x512); larger ones return RCG_INVALID, as do sides < 8 and channels other than
 * 1 or 3. The score (f64; NaN if it is not finite) is written to the device pointer `d_score`; the work is queued on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) of the current device and the call returns without
 * waiting. The first call on a device sets up that device (looks up the scratch address and uploads constant tables),
 * so make it before any stream capture. Every call on a device shares the one scratch array: calls whose work overlaps
 * on the GPU (different streams, or other host threads) race and corrupt each other's results; serialize them. The
 * set-up is kept for the life of the process: calls after a cudaDeviceReset of that device are not supported. */
int rcg_ssimulacra2_device_noalloc(const uint8_t* d_reference, const uint8_t* d_distorted, uint32_t width,
                                   uint32_t height, int channels, double* d_score, void* stream);

/* jpeg::encode::build_coefs(src, opts) -> CoefImage (jpeg/src/encode.rs:426). `src` is 8-bit Gray/Rgb on the host.
 * `coefs` receives layout.ncoefs int16 (capacity `coefs_len`), `qtables` (nullable) 2*64 bytes. */
int rcg_build_coefs(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                    const rcg_encode_options* opts, int16_t* coefs, size_t coefs_len, uint8_t* qtables);

/* jpeg::decode::reconstruct(ci) -> Result<Image> (jpeg/src/decode.rs:334) for a CoefImage with this library's
 * layout. `out` receives width*height*ncomp bytes (Gray for 1 component, Rgb for 3). */
int rcg_reconstruct(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                    const uint8_t* qtables, const int16_t* coefs, uint8_t* out, size_t out_len);

/* The whole `--target-ssimulacra2` search: jpeg::target::find_quality_with(reference, target, max_quality, make,
 * metric) (jpeg/src/target.rs:29) with make = build_coefs at each quality (cli/src/pipeline.rs:238) and metric =
 * ssimulacra2(..).unwrap_or(f64::MIN) (cli/src/pipeline.rs:218). Every step (encode, decode, score, bisection
 * decision) runs on the device; the host only copies the image in and the chosen coefficients out.
 * `opts->quality` is ignored. `coefs`/`qtables` (nullable) receive the chosen candidate's CoefImage, sized by
 * rcg_coef_layout_for at the found quality (the layout depends on quality only with RCG_SUB_AUTO). */
int rcg_search(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels, double target,
               int max_quality, const rcg_encode_options* opts, rcg_found* found, int16_t* coefs, size_t coefs_len,
               uint8_t* qtables);
/* The same with the image already on the device; coefs/qtables (nullable) are device pointers. */
int rcg_search_device(rcg_ctx* ctx, const uint8_t* d_src, uint32_t width, uint32_t height, int channels,
                      double target, int max_quality, const rcg_encode_options* opts, rcg_found* found,
                      int16_t* d_coefs, size_t coefs_len, uint8_t* d_qtables);

/* reconstruct (jpeg/src/decode.rs:334) of a CoefImage with a general table assignment (requantized images: components
 * may share a slot or each have their own). */
int rcg_reconstruct_tables(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                           const rcg_qtables* tables, const int16_t* coefs, uint8_t* out, size_t out_len);

/* score(reference, candidate, metric) (cli/src/pipeline.rs:130-138) of two 8-bit interleaved images with 1..=4
 * channels (SSIM and PSNR count every channel, alpha included; MS-SSIM uses luma), host buffers. SSIMULACRA2 here is
 * rcg_ssimulacra2 at depth 8. PSNR of identical images is +infinity, as in the reference. */
int rcg_metric_score(rcg_ctx* ctx, int metric, const uint8_t* reference, const uint8_t* candidate, uint32_t width,
                     uint32_t height, int channels, double* score);
/* As rcg_metric_score with both images on the device. */
int rcg_metric_score_device(rcg_ctx* ctx, int metric, const uint8_t* d_reference, const uint8_t* d_candidate,
                            uint32_t width, uint32_t height, int channels, double* score);

/* The derivative of SSIMULACRA2 (core/src/ssimulacra2.rs:471) with respect to the distorted image, in FP64: the
 * reference is 8-bit RGB, the distorted image RGB float samples in [0, 255] taken as continuous values (linear light
 * by the sRGB curve itself, of which the scorer's 8-bit table is a sampling). Writes the FP64 score and
 * d score / d sample (w x h x 3 doubles, interleaved like the image; grad NULL: the score alone). Host buffers. */
int rcg_ssimulacra2_grad(rcg_ctx* ctx, const uint8_t* reference, const float* distorted, uint32_t width,
                         uint32_t height, double* score, double* grad);
/* As rcg_ssimulacra2_grad with all three images in device memory. */
int rcg_ssimulacra2_grad_device(rcg_ctx* ctx, const uint8_t* d_reference, const float* d_distorted, uint32_t width,
                                uint32_t height, double* score, double* d_grad);

/* The JPEG quality search for a goal metric (cli/src/pipeline.rs:207-222): RCG_METRIC_SSIMULACRA2 (as rcg_search) or
 * RCG_METRIC_SSIM (`--target-ssim`, jpeg/src/target.rs:24; any image size). */
int rcg_search_metric(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels, int metric,
                      double target, int max_quality, const rcg_encode_options* opts, rcg_found* found,
                      int16_t* coefs, size_t coefs_len, uint8_t* qtables);

/* jpeg::decode::parse(data)?.into_coefs() (jpeg/src/decode.rs:397, :540) for Huffman JPEGs, sequential (SOF0/SOF1)
 * and progressive (SOF2), 8-bit, 1 or 3 components, any sampling, restart intervals, any number of scans: markers on
 * the host, the entropy-coded data decoded on the GPU (sequential, DC-first and AC-first scans by self-synchronizing
 * spans in parallel, DC refinement one bit per block, AC refinement one thread per restart segment). Arithmetic,
 * lossless, hierarchical, 12-bit, RGB-coded and 4-component files answer RCG_UNSUPPORTED (decode them on the host).
 * With coefs == NULL only the header is parsed (info, layout, tables: size the buffer from layout.ncoefs). Metadata
 * segments are not returned. */
int rcg_decode_coefs(rcg_ctx* ctx, const uint8_t* jpeg, size_t len, rcg_jpeg_info* info, rcg_coef_layout* layout,
                     rcg_qtables* tables, int16_t* coefs, size_t coefs_len);
/* As rcg_decode_coefs with the coefficients written to device memory. */
int rcg_decode_coefs_device(rcg_ctx* ctx, const uint8_t* jpeg, size_t len, rcg_jpeg_info* info,
                            rcg_coef_layout* layout, rcg_qtables* tables, int16_t* d_coefs, size_t coefs_len);

/* As rcg_search_requantize with the source and output coefficients in device memory (16-byte aligned), e.g. from
 * rcg_decode_coefs_device: the JPEG -> JPEG search without host copies of the coefficients. */
int rcg_search_requantize_device(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                                 const rcg_qtables* in, const int16_t* d_coefs_in, int metric, double target,
                                 int max_quality, int trellis, rcg_found* found, int16_t* d_coefs_out,
                                 size_t coefs_len, rcg_qtables* out);

/* Plan write_best for a CoefImage (1 or 3 components): symbol statistics of every candidate scan and of the baseline
 * scan on the GPU, Huffman code lengths, costs and the cheapest script. The caller then writes baseline
 * (jpeg/src/encode.rs:571) or the script (jpeg/src/progressive.rs:380) as `result.progressive` says. */
int rcg_plan(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout, const int16_t* coefs,
             size_t coefs_len, rcg_plan_result* result);
/* As rcg_plan with the coefficients already on the device (16-byte aligned), e.g. a search's output. */
int rcg_plan_device(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                    const int16_t* d_coefs, rcg_plan_result* result);

/* jpeg::encode::CoefImage::requantize(quality, trellis) (jpeg/src/encode.rs:111): re-quantize existing coefficients
 * (1 or 3 components, any integral sampling layout) toward the quality's tables, never finer than the source's, with
 * the trellis pass when a table changed. Host buffers; `out` receives the new table assignment. */
int rcg_requantize(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                   const rcg_qtables* in, const int16_t* coefs_in, int quality, int trellis, int16_t* coefs_out,
                   size_t coefs_len, rcg_qtables* out);

/* The JPEG -> JPEG `--target-ssimulacra2` search (cli/src/pipeline.rs:369-386): the reference image is the source
 * reconstructed, each candidate the source requantized; bisection as rcg_search, on the device. `metric`:
 * RCG_METRIC_SSIMULACRA2 or RCG_METRIC_SSIM. */
int rcg_search_requantize(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                          const rcg_qtables* in, const int16_t* coefs_in, int metric, double target, int max_quality,
                          int trellis, rcg_found* found, int16_t* coefs_out, size_t coefs_len, rcg_qtables* out);

/* Many independent searches at once: the images (host buffers, each with its own size, channel count and target)
 * share max_quality and the options. Up to `parallel` searches (0: 4) run at the same time, each on its own stream and
 * workspace owned by `ctx`, so small images no longer leave the GPU idle between kernels. Results are exactly those of
 * rcg_search on each image: found[i], coefs[i] (capacity coefs_len[i]; the array or an entry may be NULL) and
 * qtables[i] (2*64 bytes; nullable). The cli's per-file loop over rayon workers (cli/src/main.rs:57-60) maps onto this
 * call; no single reference function corresponds to it. Returns the first failing image's status (the others still
 * run) with its index in the message. */
int rcg_search_batch(rcg_ctx* ctx, int n, const uint8_t* const* srcs, const uint32_t* widths,
                     const uint32_t* heights, const int* channels, const double* targets, int max_quality,
                     const rcg_encode_options* opts, int parallel, rcg_found* found, int16_t* const* coefs,
                     const size_t* coefs_len, uint8_t* const* qtables);

/* The same many searches in lockstep: every bisection step of every image is one launch per stage over a work-list
 * of all the images' CTAs (step tables, quantization, rate tables, trellis, dequantization + IDCT, upsampling,
 * pyramid, scorer tiles, reductions), the step loop captured as one CUDA graph per batch composition (the images'
 * sizes) and replayed for later batches of the same composition. Each image's set-up (upload, colour planes, FDCTs,
 * the reference pyramid) runs on its own stream first. Results are exactly those of rcg_search on each image (the
 * same kernels per image), near ties included; arguments as rcg_search_batch without `parallel`. All images' buffers
 * are resident at once (about 70 bytes per pixel). Like rcg_search_batch, no single reference function corresponds to
 * it: the cli runs find_quality_with per file (jpeg/src/target.rs:29-56) across rayon workers (cli/src/main.rs:57-60).
 */
int rcg_search_batch_lockstep(rcg_ctx* ctx, int n, const uint8_t* const* srcs, const uint32_t* widths,
                              const uint32_t* heights, const int* channels, const double* targets, int max_quality,
                              const rcg_encode_options* opts, rcg_found* found, int16_t* const* coefs,
                              const size_t* coefs_len, uint8_t* const* qtables);

/* ---- Perceptual trellis (opt-in; not a reference mode)
 *
 * The SSIMULACRA2 gradient of a decoded image, pulled back through the decoder's YCbCr->RGB conversion, chroma
 * upsampling and orthonormal IDCT, gives d score / d coefficient; the perceptual weights derived from it multiply the
 * trellis's distortion weight (jpeg/src/rdo.rs:41-43, (median / q)^1 per frequency) coefficient by coefficient. With
 * the weights absent every entry point below is the reference's plain MSE trellis; the plain calls above never read
 * weights. */
typedef struct {
  double strength; /* global scale of the weights (below 1: the trellis trades more distortion for rate) */
  double gamma;    /* exponent on the block's normalised gradient sensitivity (0: uniform weights) */
  double w_min;    /* clamp of the normalised, exponentiated sensitivity (before `strength`) */
  double w_max;
  int32_t radius;  /* sensitivity = RMS of the gradient energy over (2 radius + 1)^2 neighbouring blocks */
  int32_t keep_smaller; /* rcg_search_perceptual: return the plain result when its planned size is smaller */
  int32_t gradient_fp64; /* 1: the weights come from the FP64 adjoint; 0: from the same pass in FP32 (faster) */
  int32_t strength_by_quality; /* rcg_search_perceptual: the strength follows the plain result's quality (see
                                  rcg_perceptual_strength) instead of `strength` */
} rcg_perceptual_options;

/* The defaults: strength 0.35, gamma 0.5, w_min 0.25, w_max 4, radius 1, keep_smaller 1, gradient_fp64 0,
 * strength_by_quality 1. */
void rcg_perceptual_defaults(rcg_perceptual_options* opts);

/* The strength rcg_search_perceptual uses after a plain search found `quality`: `strength` unless
 * strength_by_quality, else 0.35 below quality 70, 0.7 below 85 and 1.0 from 85 (a lower distortion weight pays at
 * low qualities and costs at high ones; measured on seeded synthetic image sets). */
double rcg_perceptual_strength(const rcg_perceptual_options* opts, int quality);

/* d SSIMULACRA2(reference, decoded) / d coefficient for the coefficient layout `layout` (64 zigzag entries per block,
 * components in order; dequantized units: multiply by the quantization step for d score / d quantized value). Both
 * images are 8-bit with `channels` (1 or 3, matching layout->ncomp); the gradient is taken at the decoded samples as
 * f32 (FP64 adjoint), then pulled back linearly (roundings and clamps of the decoder dropped). Host buffers. */
int rcg_coef_gradient(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* decoded, uint32_t width, uint32_t height,
                      int channels, const rcg_coef_layout* layout, double* score, double* grad, size_t grad_len);

/* The perceptual trellis weights (f32, the coefficient layout of `layout`) from the gradient at `decoded`. */
int rcg_perceptual_weights(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* decoded, uint32_t width,
                           uint32_t height, int channels, const rcg_coef_layout* layout,
                           const rcg_perceptual_options* popts, double* score, float* weights, size_t weights_len);

/* rcg_build_coefs with the trellis pass in the perceptual mode (`weights`: the layout's ncoefs entries). */
int rcg_build_coefs_weighted(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                             const rcg_encode_options* opts, const float* weights, size_t weights_len, int16_t* coefs,
                             size_t coefs_len, uint8_t* qtables);

/* rcg_search with every candidate's trellis in the perceptual mode. The layout must not depend on the quality:
 * an explicit subsampling (or Gray), trellis on. */
int rcg_search_weighted(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                        double target, int max_quality, const rcg_encode_options* opts, const float* weights,
                        size_t weights_len, rcg_found* found, int16_t* coefs, size_t coefs_len, uint8_t* qtables);

/* The perceptual search: the plain search (`plain` receives its result), the weights from the gradient at the plain
 * result's decoded image, then the weighted search. Both results are sized with write_best's plan (rcg_plan;
 * `sizes` (nullable) receives {plain, perceptual} as min(progressive, baseline) bytes); `found`, `coefs` and
 * `qtables` receive the weighted search's result, or the plain one when popts->keep_smaller is set and it is smaller
 * (`*chose_perceptual`, nullable, says which). `weights` (nullable) receives the weights used. */
int rcg_search_perceptual(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                          double target, int max_quality, const rcg_encode_options* opts,
                          const rcg_perceptual_options* popts, rcg_found* plain, rcg_found* found, uint64_t* sizes,
                          int* chose_perceptual, int16_t* coefs, size_t coefs_len, uint8_t* qtables, float* weights,
                          size_t weights_len);

/* The perceptual search in one full search: the plain bisection's first four candidates only (the maximum quality,
 * then three bisection steps; `probe`, nullable, receives their trace and, as quality and score, the one scoring closest
 * to the target), the weights from the gradient at that candidate's decoded image (strength by its quality when
 * popts->strength_by_quality), then the weighted search, whose result `found`, `coefs` and `qtables` receive. No plain search to compare with and no
 * plans: the result is the weighted search's whatever its size (popts->keep_smaller does not apply). 12 candidates
 * against rcg_search_perceptual's 16. */
int rcg_search_perceptual_fast(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                               double target, int max_quality, const rcg_encode_options* opts,
                               const rcg_perceptual_options* popts, rcg_found* probe, rcg_found* found,
                               int16_t* coefs, size_t coefs_len, uint8_t* qtables, float* weights,
                               size_t weights_len);

#ifdef __cplusplus
}
#endif

#endif /* RCG_H */
