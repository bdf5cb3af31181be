// Internal declarations shared by the rcg translation units (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/rcg.h"

namespace rcg {

// ------------------------------------------------------------------------------------------------ constants

constexpr int kMaxScales = 6;     // core/src/ssimulacra2.rs:27 (NUM_SCALES)
constexpr int kMinSide = 8;       // core/src/ssimulacra2.rs:25 (MIN_SIDE)
constexpr int kMaxSteps = 16;     // candidates per search (8 suffice for max_quality <= 100)
constexpr int kScoreSums = 18;    // 3 channels x 6 sums (core/src/ssimulacra2.rs:323-326)

// Scorer tile: TW x TH output pixels per CTA, with a 5-pixel halo (11-tap blur, core/src/ssimulacra2.rs:31).
constexpr int kRadius = 5;
constexpr int kTileW = 32;
constexpr int kTileH = 32;
constexpr int kTileThreads = 256;

// ------------------------------------------------------------------------------------------------ descriptors

// One scale of the scorer's pyramid: planes are channel-planar f32, [3][h][w], at `off` (floats) in a pyramid buffer.
struct ScaleDesc {
  int w, h;
  int tiles_x, tiles_y;  // CTAs across and down (32-column bands of nch chunks of 32 rows; nch = 1: 32x32 tiles)
  int tile0;        // first CTA of this scale in the multi-scale launch
  int nch;          // 32-row chunks per CTA (ssim2.cu, ssim2_band)
  int chunk0;       // first 32x32 chunk of this scale (CTA-major, nch per CTA) in chunk-indexed buffers
  long long off;    // float offset of channel 0 of this scale
};

struct PyramidDesc {
  int nscales;
  int total_tiles;
  ScaleDesc s[kMaxScales];
  long long floats;  // total floats of one image's pyramid
  int total_chunks;  // chunks of every CTA of every scale (total_tiles x nch, per scale)
};

// One JPEG component of the current candidate, as the device kernels see it.
struct CompDesc {
  int bw, bh;            // block grid (blocks_w, blocks_h)
  int h, v;              // sampling factors
  int cls;               // quantization / Huffman class: 0 luma, 1 chroma (component index min 1)
  int cache;             // which FDCT cache plane set holds this component (index into StepDesc-independent caches)
  long long blk0;        // first block of this component in the concatenated block space
  long long plane_off;   // byte offset of the decoded component plane (stride bw*8) in the plane buffer
};

// Everything the per-candidate kernels need; lives in device memory. Written by the host for single calls and by
// the device-side search for each bisection step.
struct StepDesc {
  int active;            // 0: nothing to do (the search has finished)
  int quality;
  int use_trellis;       // trellis && quality < 100 (jpeg/src/encode.rs:527)
  int ncomp;
  int hmax, vmax;
  long long nblocks;     // total blocks of all components
  CompDesc comp[3];
  // Per-component tables (index = component). The encoder gives components 1 and 2 the same chroma table
  // (jpeg/src/quality.rs:37-43); a requantization gives each component its own (jpeg/src/encode.rs:120-126).
  uint8_t qt[3][64];     // quantization table of each component, natural order
  float divz[3][64];     // fdct divisors per zigzag position: div[ZZ_T[k]] (jpeg/src/encode.rs:174-183, :202)
  float mult[3][64];     // dequantization multipliers, natural order (jpeg/src/decode.rs:1316-1321)
  // Trellis (jpeg/src/rdo.rs:14-52), per component
  float rq[3][64];       // step per zigzag position
  float rw[3][64];       // distortion weight per zigzag position
  float lambda[3];
  float eob[3];          // lambda * len[0x00]
  float lr[3][64 * 16];  // lambda * rate(run, v) for run 0..63, size 0..15 (index run*16 + size)
  unsigned int hist[2][256];  // AC symbol histogram of the plain pass, per class (jpeg/src/encode.rs:223-227)
  // Requantization of existing coefficients (jpeg/src/encode.rs:107-172)
  int requant;           // 1: the candidate requantizes coef_src instead of quantizing the FDCT cache
  int changed;           // some component's table changed (gates the trellis pass, encode.rs:152)
  int mcus_x, mcus_y;    // MCU grid: the rate model counts only blocks inside it (encode.rs:376-398)
  const int16_t* coef_src;
  uint8_t src_qt[3][64]; // the source table of each component (old; all ones where its slot is empty)
  float ratio[3][64];    // old / new per zigzag position
  int16_t* coefs;        // where this candidate's coefficients go
  // Perceptual trellis (opt-in): per-coefficient distortion weights in the coefficient layout ([block][64], zigzag),
  // read only by the weighted trellis instantiation.
  const float* pweights;
};

// The device-side bisection (jpeg/src/target.rs:29-56).
struct SearchState {
  int lo, hi;
  int step;              // index of the candidate being evaluated
  int done;
  int best_q;
  int best_step;
  double best_score;
  double target;
  int max_q;
  int subsampling;
  int trellis;
  int channels;
  int qs[kMaxSteps];
  double scores[kMaxSteps];
  int status;            // nonzero: a device-side check failed
  // Near ties: a candidate whose score lies within tie_band of the target pauses the search (done = 2) so that the
  // host can decide it on the reference-order FP64 score (exact.cu); 0 disables the pause.
  double tie_band;
};

// One bisection step of jpeg/src/target.rs:35-53 on the device, after candidate `ss->step` scored `sv`: the first
// candidate (max quality) ends the search when it misses the target; later ones move hi (accepted, s >= target) or
// lo; the next quality is lo + (hi - lo) / 2 until lo == hi.
// A candidate scored within tie_band of the target (by the fast f32 scorer) pauses instead: done = 2, the step and
// its score kept, nothing decided; search_resume later records the candidate's exact score with the pause disabled.
__device__ __forceinline__ void search_record(SearchState* ss, double sv, bool may_pause = true) {
  if (ss->done) return;
  const int step = ss->step;
  const int q = ss->qs[step];
  ss->scores[step] = sv;
  if (may_pause && ss->tie_band > 0.0 && fabs(sv - ss->target) <= ss->tie_band) {
    ss->done = 2;
    return;
  }
  if (step == 0) {
    ss->best_q = q;
    ss->best_score = sv;
    ss->best_step = 0;
    if (sv < ss->target) ss->done = 1;
  } else if (sv >= ss->target) {
    ss->hi = q;
    ss->best_q = q;
    ss->best_score = sv;
    ss->best_step = step;
  } else {
    ss->lo = q + 1;
  }
  if (!ss->done) {
    if (ss->lo < ss->hi && step + 1 < kMaxSteps) {
      ss->step = step + 1;
      ss->qs[step + 1] = ss->lo + (ss->hi - ss->lo) / 2;
    } else {
      ss->done = 1;
    }
  }
}

// One image of a lockstep batch of searches (capi.cu, rcg_search_batch_lockstep): every bisection step of every
// image runs as one work-list launch per stage, each CTA finding its image by the first-CTA offsets below.
struct LockItem {
  SearchState* ss;
  StepDesc* st;
  const float* caches[9];  // FDCT caches of the sampling layouts (as CacheSet)
  int16_t* slots;          // coefficient slots, one per step
  long long slot_stride;
  uint8_t* planes;         // decoded component planes
  int w, h;
  float* ref_pyr;          // the reference's linear pyramid
  float* dist_pyr;         // the candidate's (scale 0 written by the upsampling)
  double* partials;        // scorer scratch: per-CTA sums, per-scale sums, completion counter, score
  double* scale_sums;
  unsigned* counter;
  double* score;
  PyramidDesc pd;          // the scorer's CTA layout (bands)
  float2* refm;            // the reference moments (null: the store is off)
  long long q0;            // first CTA in the block grids (quantize, trellis, dequantize: 128 blocks a CTA)
  long long u0;            // first CTA in the upsampling grid (ux x uy CTAs)
  int ux, uy;
  long long p0;            // first CTA in the pyramid grid
  long long t0;            // first CTA in the scorer's grid (pd.total_tiles)
};

// Last item whose first CTA (field `f` of LockItem) is <= x (n >= 1, the first item's offset 0).
template <long long LockItem::*f>
__device__ __forceinline__ int lock_find(const LockItem* __restrict__ items, int n, long long x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].*f <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------------------------------------------ context

struct KernelTimes {
  uint64_t launches = 0;
  double ms = 0.0;
};

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace rcg

struct rcg_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t switch_event = nullptr;  // orders a stream switch after the old stream's queued work
  std::string last_error;
  uint64_t launches = 0;
  bool profiling = false;
  std::map<std::string, rcg::KernelTimes> ktimes;
  struct PendingEvent {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<PendingEvent> pending;
  std::vector<cudaEvent_t> event_pool;
  std::map<std::string, rcg::DeviceBuffer> bufs;
  float* lut16 = nullptr;  // 65536-entry sRGB->linear table for 16-bit samples (allocated on first use)
  std::vector<rcg_ctx*> workers;  // sub-contexts of rcg_search_batch (own streams and workspaces)
  std::vector<rcg_ctx*> lock_subs;  // per-image sub-contexts of rcg_search_batch_lockstep (buffers, set-up streams)
  // Pinned host staging for host-buffer calls (grow-only): pageable copies go through the driver's own staging and
  // serialize across threads; these let a worker thread do its memcpy in parallel with other workers' GPU work.
  bool stage_copies = false;  // set on batch worker contexts
  void* pinned_in = nullptr;
  size_t pinned_in_bytes = 0;
  void* pinned_out = nullptr;
  size_t pinned_out_bytes = 0;
  // Step loops of the device searches captured as CUDA graphs (capi.cu, run_step_loop). A loop's launches and their
  // arguments follow from the image shape, the options and the workspace pointers, so the key holds the first two
  // and ws_gen stands for the third: every workspace (re)allocation bumps it and makes older graphs stale.
  struct StepGraph {
    std::vector<long long> key;
    uint64_t gen = 0;
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;  // kernels per replay
    uint64_t last_use = 0;
  };
  std::vector<StepGraph> graphs;
  bool use_graphs = true;
  uint64_t ws_gen = 0;
  // Loops run as plain launches lately (key, ws_gen): captured when one comes again with the same ws_gen.
  std::vector<std::pair<std::vector<long long>, uint64_t>> warm;
  uint64_t graph_tick = 0, graph_captures = 0, graph_replays = 0;
  // Near-tie rescoring of the SSIMULACRA2 searches (exact.cu): band around the target, and how many candidates were
  // decided on the reference-order FP64 score so far.
  double tie_band = 1e-3;
  uint64_t tie_rescores = 0;
  // Scorer bands: 0 autotunes the chunks per band per size class (ssim2.cu, band_chunks); >= 1 fixes them.
  int band_chunks = 0;
  // The searches' reference moments (kRefWrite at the first candidate, kRefRead after): on by default.
  bool ref_cache = true;
};

namespace rcg {

// Error helpers: every entry point returns a status and stores a message; nothing aborts.
int fail(rcg_ctx* ctx, int status, const std::string& msg);
int cuda_fail(rcg_ctx* ctx, cudaError_t e, const char* what);

// Grow-only named device workspace. Returns nullptr (and sets the error) on allocation failure. A (re)allocation
// retires the context's stored graphs unless `in_graphs` is false: buffers that no captured step loop uses (the exact
// scorer's) move without making the graphs stale.
void* workspace(rcg_ctx* ctx, const char* name, size_t bytes, bool in_graphs = true);

// Host<->device copies of caller buffers: the driver's path for single calls; on batch worker contexts direct DMA when
// the caller's memory is pinned, else through the context's pinned staging buffer. copy_to_device is asynchronous on the context stream (the source may be reused as soon as it
// returns); copy_to_host synchronizes the stream.
int copy_to_device(rcg_ctx* ctx, void* dst, const void* src, size_t bytes);
int copy_to_host(rcg_ctx* ctx, void* dst, const void* src, size_t bytes);

// Kernel launch bookkeeping: counts launches and, when profiling, brackets them with events.
void launch_begin(rcg_ctx* ctx, const char* name, cudaEvent_t* a, cudaEvent_t* b);
void launch_end(rcg_ctx* ctx, const char* name, cudaEvent_t a, cudaEvent_t b);
void collect_times(rcg_ctx* ctx);

// Issue a device search's step loop (`issue` launches every step's kernels on ctx->stream). With graphs on, the
// first loop of a key runs as plain launches (it may allocate workspace), the next one with the same key is
// captured and replayed, and later ones replay the stored graph: one graph launch per search instead of ~10
// kernel launches per step. Plain launches whenever profiling is on, the stream is the legacy default stream, or
// the caller is capturing the stream itself.
int run_step_loop(rcg_ctx* ctx, const std::vector<long long>& key, const std::function<void()>& issue);
// Release the context's stored graphs.
void drop_graphs(rcg_ctx* ctx);

#define RCG_LAUNCH(ctx, name, kernel, grid, block, smem, ...)                     \
  do {                                                                            \
    cudaEvent_t _ea = nullptr, _eb = nullptr;                                     \
    ::rcg::launch_begin((ctx), (name), &_ea, &_eb);                               \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);              \
    ::rcg::launch_end((ctx), (name), _ea, _eb);                                   \
  } while (0)

// Host-side sRGB -> linear tables (core/src/ssimulacra2.rs:172-175, :192, :207).
void srgb_lut8(float out[256]);
const float* srgb_lut16_device(rcg_ctx* ctx);

// Pyramid geometry of the scorer for a w x h image (core/src/ssimulacra2.rs:480-490).
PyramidDesc make_pyramid(int w, int h);

// ---- scorer (ssim2.cu)
// Upload the 8-bit LUT to constant memory once per device.
int scorer_init(rcg_ctx* ctx);
// Interleaved 8-bit Gray/Rgb (or GrayAlpha/Rgba, or 16-bit) image -> linear planes at scale 0 of `pyr`.
int to_linear(rcg_ctx* ctx, const uint8_t* d_img, int w, int h, int channels, int depth, float* d_pyr);
// Fill scales 1.. of a pyramid from scale 0 (core/src/ssimulacra2.rs:225-247).
int build_pyramid(rcg_ctx* ctx, const PyramidDesc& pd, float* d_pyr);
// The same, skipped on the device when the search step is inactive.
int build_pyramid_gated(rcg_ctx* ctx, const PyramidDesc& pd, float* d_pyr, const StepDesc* st);
// CTAs of one pyramid launch (k_pyramid and the work-list forms): one per scale-1 tile, 0 for a single scale.
int pyramid_ctas(const PyramidDesc& pd);
// upsample_color's linear planes and build_pyramid_gated in one launch, for a step whose layout is the 4:2:0 case of
// upsample420.cuh (the caller's promise: 3 components, luma 2x2 and chroma 1x1 sampling, w % 4 == 0).
int upsample_pyramid(rcg_ctx* ctx, StepDesc* d_step, const uint8_t* d_planes, int w, int h, const PyramidDesc& pd,
                     float* d_pyr);
// Reference moments of the tile kernel: kRefNone computes every blurred moment; kRefWrite also stores the
// reference-only ones (blur a', blur a'^2) for later candidates against the same reference; kRefRead reads them
// instead of blurring them. Same scores in every mode. The store is chunk-major: per 32x32 chunk of the banded
// layout the scorer runs (plan_bands), kRefChunk float2 as [channel][row][column], ref_moment_bytes() in all.
constexpr int kRefChunk = 3 * kTileH * kTileW;
constexpr int kRefNone = 0, kRefWrite = 1, kRefRead = 2;
// Score: per-tile sums of every scale, then the final mapping. `d_score` receives the score (f64); when
// `search` is non-null the final kernel also advances the device-side bisection. `refm`/`ref_mode`: the reference
// moments (nullptr / kRefNone: none).
int score_pyramids(rcg_ctx* ctx, const PyramidDesc& pd, const float* d_ref, const float* d_dist, double* d_score,
                   SearchState* search, StepDesc* step, float2* refm = nullptr, int ref_mode = kRefNone);
// The reference-order FP64 score (exact.cu) of two images given as scale-0 linear planes ([3][h][w] f32, as
// to_linear writes them): to d_score (NaN for the reference's non-finite Err), queued on the context stream.
int exact_score(rcg_ctx* ctx, const float* d_ref0, const float* d_dist0, int w, int h, double* d_score);
// Record the exact score of a paused search's candidate (search_record without the pause) and let it go on.
int search_resume(rcg_ctx* ctx, SearchState* d_ss, const double* d_score);
// The scorer's CTA layout for a pyramid: 32-column bands of `nch0` chunks of 32 rows at the scales with at least
// `min_tiles` tiles, 32x32 tiles elsewhere (nch0 = 1: tiles everywhere).
PyramidDesc banded(const PyramidDesc& pd, int nch0, int min_tiles);
// The layout a context scores this pyramid with (its fixed chunks at every scale, or the tuned ones).
PyramidDesc plan_bands(rcg_ctx* ctx, const PyramidDesc& pd);
// Chunks per band for a pyramid of this geometry: the context's fixed choice, or the process-wide autotuned one for
// its size class (tuned on first use by timing the candidates; small images always take 1).
int band_chunks(rcg_ctx* ctx, const PyramidDesc& pd);
// Bytes of the reference-moment store for a banded layout.
inline size_t ref_moment_bytes(const PyramidDesc& banded_pd) {
  return (size_t)banded_pd.total_chunks * kRefChunk * 8;
}
// Allocate (or find) the scratch score_pyramids uses for a pyramid of this geometry.
int score_workspace(rcg_ctx* ctx, const PyramidDesc& pd);
// Score n device-resident pairs (checked sizes and formats; depths nullable = 8) with the work-list kernels;
// *d_scores receives the device array of the n scores (NaN where a score is not finite), ready once the stream is.
int score_batch(rcg_ctx* ctx, int n, const uint8_t* const* d_refs, const uint8_t* const* d_dists,
                const uint32_t* widths, const uint32_t* heights, const int* channels, const int* depths,
                double** d_scores);

// ---- lockstep batch (work-list launches over the LockItems of a batch; totals are the grids' CTA counts)
void lock_step_codec(rcg_ctx* ctx, const LockItem* d_items, int n, long long q_total, long long u_total);
void lock_step_score(rcg_ctx* ctx, const LockItem* d_items, int n, long long p_total, long long t_total,
                     int max_scales, int ref_mode = kRefNone);

// ---- codec (codec.cu)
// Colour conversion + edge padding (jpeg/src/encode.rs:463-477): full-resolution padded Y/Cb/Cr planes.
int color_pad(rcg_ctx* ctx, const uint8_t* d_src, int w, int h, int channels, int pw, int ph, uint8_t* d_y,
              uint8_t* d_cb, uint8_t* d_cr);
// 2-D box downsample of a padded chroma plane (jpeg/src/encode.rs:478-499).
int chroma_down(rcg_ctx* ctx, const uint8_t* d_src, int src_stride, int pw, int ph, int fx, int fy, uint8_t* d_dst);
// FDCT of every block of a plane into the zigzag [k][block] cache (quality-independent; jpeg/src/encode.rs:189-196).
int fdct_cache(rcg_ctx* ctx, const uint8_t* d_plane, int stride, int bw, int bh, float* d_cache);
// Per-candidate pipeline pieces, all driven by a device StepDesc.
int quantize(rcg_ctx* ctx, StepDesc* d_step, const float* const* d_caches, long long max_blocks);
// Plain requantization of st->coef_src into st->coefs, with the AC histogram when the trellis pass follows.
int requantize_plain(rcg_ctx* ctx, StepDesc* d_step, long long max_blocks);
int rate_tables(rcg_ctx* ctx, StepDesc* d_step);
// weighted: the perceptual mode (d_step->pweights); otherwise the reference's plain trellis.
int trellis(rcg_ctx* ctx, StepDesc* d_step, const float* const* d_caches, long long max_blocks, bool weighted = false);
// d_coefs null: decode the candidate's own coefficients (d_step->coefs).
int dequant_idct(rcg_ctx* ctx, StepDesc* d_step, const int16_t* d_coefs, uint8_t* d_planes, long long max_blocks);
// Upsample + YCbCr->RGB (jpeg/src/decode.rs:1404-1444). Writes interleaved 8-bit pixels to d_rgb (nullable)
// and/or linear planes to d_lin (nullable).
int upsample_color(rcg_ctx* ctx, StepDesc* d_step, const uint8_t* d_planes, int w, int h, uint8_t* d_rgb,
                   float* d_lin);
// Host-side table setup of one quality into a host StepDesc (no device work).
void host_step_tables(StepDesc* st, int quality, int subsampling, int channels, int trellis, int w, int h);
// core/src/metrics.rs on device images: ssim (score to d_score; with ss, one bisection step; gated by st), the
// squared-error sum of psnr, luma and downsample2 of ms_ssim.
int ssim_score(rcg_ctx* ctx, const uint8_t* d_a, const uint8_t* d_b, int w, int h, int ch, double* d_score,
               SearchState* ss, const StepDesc* st);
int squared_error(rcg_ctx* ctx, const uint8_t* d_a, const uint8_t* d_b, size_t n, unsigned long long* d_out);
int luma8(rcg_ctx* ctx, const uint8_t* d_a, size_t npx, int ch, uint8_t* d_out);
int downsample2(rcg_ctx* ctx, const uint8_t* d_in, int w, int h, uint8_t* d_out);

// parse(data)?.into_coefs() for sequential Huffman JPEGs; coefs NULL: header only.
int jpeg_decode(rcg_ctx* ctx, const uint8_t* data, size_t len, rcg_jpeg_info* info, rcg_coef_layout* layout,
                rcg_qtables* tables, int16_t* coefs, size_t coefs_len, bool coefs_on_device);

// The scorer's 108 weights (core/src/ssimulacra2.rs:54-163), host side.
const double* scorer_weights();
// d SSIMULACRA2 / d distorted RGB samples (continuous, f32 in [0, 255]); the reference image is 8-bit RGB. FP64
// throughout (the checked gradient) or, with fp32, the same pass in f32 (the perceptual weights); both write f64.
int ssim2_grad_device(rcg_ctx* ctx, const uint8_t* d_ref, const float* d_dist, int w, int h, double* score,
                      double* d_grad, bool fp32 = false);

// write_best's plan (progressive candidates + baseline estimate) of coefficients on the device; `lay` carries the
// component layout (ncomp, hmax, vmax, comp[]).
int plan_scans(rcg_ctx* ctx, const StepDesc* lay, int w, int h, const int16_t* d_coefs, rcg_plan_result* res);

// Natural (row * 8 + column) index of zigzag position k (jpeg/src/lib.rs:14-19), host side.
int zigzag_natural(int k);
// Dequantization multiplier of one entry (jpeg/src/decode.rs:1316-1321), host side.
float mult_entry_host(const uint8_t* q, int n);
// Dequantization multipliers from caller-given tables (ntables 1 or 2; natural order).
void fill_mult(StepDesc* st, const uint8_t* qtables, int ntables);
// Quantization tables of a quality, slot 0 then slot 1 (jpeg/src/quality.rs:37-43).
void qtables_for(int quality, uint8_t* out128);
// Copy the 8-bit sRGB table to the codec's constant memory (current device).
int codec_upload_lut(const float* lut8);
// Requantization tables of one quality (new tables, ratios, Rdo parameters, slot assignment) from the source
// tables in st->src_qt, on the host (single calls) and on the device (search steps): identical bits.
void host_requant_tables(StepDesc* st, int quality, int trellis, int tq_out[3], uint8_t slot_qt_out[4][64],
                         int present_out[4]);
int step_tables_requant(rcg_ctx* ctx, SearchState* d_search, StepDesc* d_step, int16_t* d_coef_slots,
                        long long slot_stride);
// Device-side: fill the step tables from the quality the search state holds.
int step_tables(rcg_ctx* ctx, SearchState* d_search, StepDesc* d_step, int w, int h, int16_t* d_coef_slots,
                long long slot_stride, const float* d_pweights = nullptr);

// ---- perceptual trellis weights (perceptual.cu)
struct PerceptualParams {
  double strength, gamma, w_min, w_max;
  int radius;
  bool gradient_fp64;  // the FP64 adjoint (else the FP32 instantiation)
};
// d SSIMULACRA2 / d coefficient of a decoded candidate: the pixel gradient (f64, [h][w][3]) pulled back through the
// YCbCr->RGB conversion, the chroma upsampling and the orthonormal 8x8 IDCT, per coefficient in the coefficient
// layout (zigzag, dequantized units; d_coef_grad nullable), plus the perceptual weights (d_weights nullable) for the
// layout of `lay` (ncomp, hmax, vmax, comp[].bw/bh/h/v/blk0).
int perceptual_pullback(rcg_ctx* ctx, const double* d_grad, int w, int h, const StepDesc* lay,
                        const PerceptualParams& p, double* d_coef_grad, float* d_weights);
// 8-bit Gray/RGB -> 8-bit RGB (d_rgb8) and/or f32 RGB (d_rgbf); either output nullable.
int expand_rgb(rcg_ctx* ctx, const uint8_t* d_src, int channels, size_t npx, uint8_t* d_rgb8, float* d_rgbf);

}  // namespace rcg
