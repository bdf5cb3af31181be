// C ABI of rcg (include/rcg.h): contexts, workspace, the host-driven single calls (build_coefs, reconstruct,
// ssimulacra2) and the device-driven quality search.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>
#include <atomic>
#include <numeric>

#include "rcg_internal.cuh"

namespace rcg {

// ------------------------------------------------------------------------------------------------ errors, workspace

int fail(rcg_ctx* ctx, int status, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return status;
}

int cuda_fail(rcg_ctx* ctx, cudaError_t e, const char* what) {
  if (ctx) ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? RCG_NO_MEMORY : RCG_CUDA_ERROR;
}

void* workspace(rcg_ctx* ctx, const char* name, size_t bytes, bool in_graphs) {
  DeviceBuffer& b = ctx->bufs[name];
  if (b.ptr && b.bytes >= bytes) return b.ptr;
  if (b.ptr) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
  }
  size_t sz = std::max<size_t>(bytes, 256);
  if (cudaMalloc(&b.ptr, sz) != cudaSuccess) {
    cudaGetLastError();
    b.ptr = nullptr;
    fail(ctx, RCG_NO_MEMORY, std::string("device allocation of ") + std::to_string(sz) + " bytes for " + name);
    return nullptr;
  }
  cudaMemsetAsync(b.ptr, 0, sz, ctx->stream);
  b.bytes = sz;
  if (in_graphs) ctx->ws_gen++;
  return b.ptr;
}

// ------------------------------------------------------------------------------------------------ step-loop graphs

constexpr size_t kMaxGraphs = 4;  // per context; the least recently used one goes first

void drop_graphs(rcg_ctx* ctx) {
  for (auto& g : ctx->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  ctx->graphs.clear();
  ctx->warm.clear();
}

int run_step_loop(rcg_ctx* ctx, const std::vector<long long>& key, const std::function<void()>& issue) {
  bool can = ctx->use_graphs && !ctx->profiling && ctx->stream != nullptr && ctx->stream != cudaStreamLegacy &&
             ctx->stream != cudaStreamPerThread;
  if (can) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess) {
      cudaGetLastError();
      can = false;
    } else if (cs != cudaStreamCaptureStatusNone) {
      can = false;  // the caller is capturing our launches into its own graph
    }
  }
  if (!can) {
    issue();
    return RCG_OK;
  }
  for (size_t i = 0; i < ctx->graphs.size();) {  // graphs of reallocated workspace point at freed memory
    if (ctx->graphs[i].gen != ctx->ws_gen) {
      cudaGraphExecDestroy(ctx->graphs[i].exec);
      ctx->graphs.erase(ctx->graphs.begin() + (long)i);
    } else {
      i++;
    }
  }
  for (auto& g : ctx->graphs) {
    if (g.key != key) continue;
    cudaError_t e = cudaGraphLaunch(g.exec, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph launch of a search loop");
    g.last_use = ++ctx->graph_tick;
    ctx->launches += g.launches;
    ctx->graph_replays++;
    return RCG_OK;
  }
  auto seen = std::find_if(ctx->warm.begin(), ctx->warm.end(), [&](const auto& w) { return w.first == key; });
  if (seen == ctx->warm.end() || seen->second != ctx->ws_gen) {
    // First sight of this key with these buffers: plain launches. A one-off shape (a batch of many sizes) never
    // pays for a capture.
    if (seen != ctx->warm.end()) ctx->warm.erase(seen);
    issue();
    if (ctx->warm.size() >= 2 * kMaxGraphs) ctx->warm.erase(ctx->warm.begin());
    ctx->warm.emplace_back(key, ctx->ws_gen);
    return RCG_OK;
  }
  ctx->warm.erase(seen);
  const uint64_t gen0 = ctx->ws_gen, l0 = ctx->launches;
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaGetLastError();
    issue();
    return RCG_OK;
  }
  issue();
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &graph);
  const uint64_t n = ctx->launches - l0;
  ctx->launches = l0;
  cudaGraphExec_t exec = nullptr;
  if (e == cudaSuccess && ctx->ws_gen != gen0) e = cudaErrorStreamCaptureInvalidated;  // workspace moved meanwhile
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    issue();  // a capture runs nothing: issue the loop as plain launches instead
    return RCG_OK;
  }
  if (ctx->graphs.size() >= kMaxGraphs) {
    auto lru = std::min_element(ctx->graphs.begin(), ctx->graphs.end(),
                                [](const rcg_ctx::StepGraph& a, const rcg_ctx::StepGraph& b) {
                                  return a.last_use < b.last_use;
                                });
    cudaGraphExecDestroy(lru->exec);
    ctx->graphs.erase(lru);
  }
  rcg_ctx::StepGraph g;
  g.key = key;
  g.gen = gen0;
  g.exec = exec;
  g.launches = n;
  g.last_use = ++ctx->graph_tick;
  ctx->graphs.push_back(g);
  ctx->graph_captures++;
  e = cudaGraphLaunch(exec, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "graph launch of a search loop");
  ctx->launches += n;
  ctx->graph_replays++;
  return RCG_OK;
}

void launch_begin(rcg_ctx* ctx, const char* name, cudaEvent_t* a, cudaEvent_t* b) {
  (void)name;
  ctx->launches++;
  if (!ctx->profiling) return;
  auto take = [&]() {
    cudaEvent_t e;
    if (!ctx->event_pool.empty()) {
      e = ctx->event_pool.back();
      ctx->event_pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  };
  *a = take();
  *b = take();
  cudaEventRecord(*a, ctx->stream);
}

void launch_end(rcg_ctx* ctx, const char* name, cudaEvent_t a, cudaEvent_t b) {
  if (!ctx->profiling || !a) return;
  cudaEventRecord(b, ctx->stream);
  ctx->pending.push_back({name, a, b});
}

void collect_times(rcg_ctx* ctx) {
  if (ctx->pending.empty()) return;
  cudaStreamSynchronize(ctx->stream);
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      KernelTimes& kt = ctx->ktimes[p.name];
      kt.launches++;
      kt.ms += ms;
    }
    ctx->event_pool.push_back(p.a);
    ctx->event_pool.push_back(p.b);
  }
  ctx->pending.clear();
}

// ------------------------------------------------------------------------------------------------ host copies

static bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

static void* grow_pinned(void** buf, size_t* cap, size_t bytes) {
  if (*buf && *cap >= bytes) return *buf;
  if (*buf) cudaFreeHost(*buf);
  *buf = nullptr;
  *cap = 0;
  if (cudaHostAlloc(buf, bytes, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    *buf = nullptr;
    return nullptr;
  }
  *cap = bytes;
  return *buf;
}

int copy_to_device(rcg_ctx* ctx, void* dst, const void* src, size_t bytes) {
  cudaError_t e;
  if (!ctx->stage_copies || is_pinned(src)) {
    e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  } else {
    // the staging buffer may still feed the previous call's copy: wait for the stream before overwriting it
    cudaStreamSynchronize(ctx->stream);
    void* st = grow_pinned(&ctx->pinned_in, &ctx->pinned_in_bytes, bytes);
    if (!st) {
      e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream);  // pageable fallback
    } else {
      std::memcpy(st, src, bytes);
      e = cudaMemcpyAsync(dst, st, bytes, cudaMemcpyHostToDevice, ctx->stream);
    }
  }
  return e == cudaSuccess ? RCG_OK : cuda_fail(ctx, e, "host to device copy");
}

int copy_to_host(rcg_ctx* ctx, void* dst, const void* src, size_t bytes) {
  cudaError_t e;
  if (!ctx->stage_copies || is_pinned(dst)) {
    e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  } else {
    void* st = grow_pinned(&ctx->pinned_out, &ctx->pinned_out_bytes, bytes);
    if (!st) {
      e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    } else {
      e = cudaMemcpyAsync(st, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
      if (e == cudaSuccess) std::memcpy(dst, st, bytes);
    }
  }
  return e == cudaSuccess ? RCG_OK : cuda_fail(ctx, e, "device to host copy");
}

// ------------------------------------------------------------------------------------------------ sRGB tables

// core/src/ssimulacra2.rs:172-175 in f64, rounded to f32 as :192 does.
static double srgb_to_linear(double v) { return v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4); }

void srgb_lut8(float out[256]) {
  for (int v = 0; v < 256; v++) out[v] = (float)srgb_to_linear((double)v / 255.0);
}

const float* srgb_lut16_device(rcg_ctx* ctx) {
  if (ctx->lut16) return ctx->lut16;
  std::vector<float> lut(65536);
  for (int v = 0; v < 65536; v++) lut[v] = (float)srgb_to_linear((double)v / 65535.0);
  float* d = nullptr;
  if (cudaMalloc(&d, 65536 * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    fail(ctx, RCG_NO_MEMORY, "device allocation of the 16-bit sRGB table");
    return nullptr;
  }
  cudaMemcpy(d, lut.data(), 65536 * sizeof(float), cudaMemcpyHostToDevice);
  ctx->lut16 = d;
  return d;
}

// ------------------------------------------------------------------------------------------------ helpers

static std::mutex g_init_mu;

static int ensure_init(rcg_ctx* ctx) {
  std::lock_guard<std::mutex> lk(g_init_mu);
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  return scorer_init(ctx);
}

static int finish(rcg_ctx* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, what);
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, what);
  if (ctx->profiling) collect_times(ctx);
  ctx->last_error.clear();
  return RCG_OK;
}

static void layout_of(int w, int h, int channels, int quality, int subsampling, rcg_coef_layout* out) {
  StepDesc* st = new StepDesc;
  host_step_tables(st, quality, subsampling, channels, 0, w, h);
  std::memset(out, 0, sizeof *out);
  out->ncomp = st->ncomp;
  for (int c = 0; c < st->ncomp; c++) {
    out->h[c] = st->comp[c].h;
    out->v[c] = st->comp[c].v;
    out->blocks_w[c] = st->comp[c].bw;
    out->blocks_h[c] = st->comp[c].bh;
  }
  out->ncoefs = st->nblocks * 64;
  delete st;
}

// Encoder front half shared by build_coefs and the search: colour planes and the FDCT caches of every sampling
// layout the options can produce (two for Subsampling::Auto, whose layout depends on the quality).
struct EncoderSetup {
  const float* caches[9] = {nullptr};
  long long max_blocks = 0;
  long long max_coefs = 0;
  long long max_plane_bytes = 0;
};

static int setup_encoder(rcg_ctx* ctx, const uint8_t* d_src, int w, int h, int channels, int subsampling,
                         EncoderSetup* es) {
  bool kinds[3] = {false, false, false};
  if (channels == 1) {
    kinds[2] = true;
  } else {
    switch (subsampling) {
      case RCG_SUB_420: kinds[0] = true; break;
      case RCG_SUB_422: kinds[1] = true; break;
      case RCG_SUB_444: kinds[2] = true; break;
      default: kinds[0] = kinds[2] = true;
    }
  }
  const int hv[3][2] = {{2, 2}, {2, 1}, {1, 1}};
  int pw_max = 0, ph_max = 0;
  for (int k = 0; k < 3; k++) {
    if (!kinds[k]) continue;
    int hm = channels == 1 ? 1 : hv[k][0], vm = channels == 1 ? 1 : hv[k][1];
    pw_max = std::max(pw_max, (w + 8 * hm - 1) / (8 * hm) * 8 * hm);
    ph_max = std::max(ph_max, (h + 8 * vm - 1) / (8 * vm) * 8 * vm);
  }
  size_t plane = (size_t)pw_max * ph_max;
  uint8_t* yp = (uint8_t*)workspace(ctx, "plane_y", plane);
  uint8_t* cbp = channels == 1 ? nullptr : (uint8_t*)workspace(ctx, "plane_cb", plane);
  uint8_t* crp = channels == 1 ? nullptr : (uint8_t*)workspace(ctx, "plane_cr", plane);
  if (!yp || (channels == 3 && (!cbp || !crp))) return RCG_NO_MEMORY;
  color_pad(ctx, d_src, w, h, channels, pw_max, ph_max, yp, cbp, crp);
  for (int k = 0; k < 3; k++) {
    if (!kinds[k]) continue;
    int hm = channels == 1 ? 1 : hv[k][0], vm = channels == 1 ? 1 : hv[k][1];
    int pw = (w + 8 * hm - 1) / (8 * hm) * 8 * hm, ph = (h + 8 * vm - 1) / (8 * vm) * 8 * vm;
    long long blocks = 0, pbytes = 0;
    for (int c = 0; c < (channels == 1 ? 1 : 3); c++) {
      int cw = c == 0 ? pw : pw / hm, chh = c == 0 ? ph : ph / vm;
      int bw = cw / 8, bh = chh / 8;
      std::string name = "fdct_cache_" + std::to_string(k * 3 + c);
      float* cache = (float*)workspace(ctx, name.c_str(), (size_t)bw * bh * 64 * sizeof(float));
      if (!cache) return RCG_NO_MEMORY;
      const uint8_t* src = c == 0 ? yp : (c == 1 ? cbp : crp);
      int stride = pw_max;
      if (c > 0 && hm * vm > 1) {
        std::string dn = "plane_sub_" + std::to_string(k * 3 + c);
        uint8_t* sub = (uint8_t*)workspace(ctx, dn.c_str(), (size_t)cw * chh);
        if (!sub) return RCG_NO_MEMORY;
        chroma_down(ctx, src, pw_max, pw, ph, hm, vm, sub);
        src = sub;
        stride = cw;
      }
      fdct_cache(ctx, src, stride, bw, bh, cache);
      es->caches[k * 3 + c] = cache;
      blocks += (long long)bw * bh;
      pbytes += (long long)cw * chh;
    }
    es->max_blocks = std::max(es->max_blocks, blocks);
    es->max_coefs = std::max(es->max_coefs, blocks * 64);
    es->max_plane_bytes = std::max(es->max_plane_bytes, pbytes);
  }
  return RCG_OK;
}

static int check_image(rcg_ctx* ctx, uint32_t w, uint32_t h, int channels) {
  if (w == 0 || h == 0) return fail(ctx, RCG_INVALID, "empty image");
  if (channels != 1 && channels != 3) return fail(ctx, RCG_INVALID, "the JPEG path takes 8-bit Gray or Rgb pixels");
  if (w > 65535 || h > 65535) return fail(ctx, RCG_UNSUPPORTED, "JPEG dimensions are limited to 65535 pixels");
  return RCG_OK;
}

static int check_opts(rcg_ctx* ctx, const rcg_encode_options* o, bool need_quality) {
  if (!o) return fail(ctx, RCG_INVALID, "null options");
  if (need_quality && (o->quality < 1 || o->quality > 100)) return fail(ctx, RCG_INVALID, "quality must be 1..=100");
  if (o->subsampling < RCG_SUB_AUTO || o->subsampling > RCG_SUB_420)
    return fail(ctx, RCG_INVALID, "unknown subsampling");
  return RCG_OK;
}

// Block layout of a caller-given CoefImage (jpeg/src/decode.rs:334-357, :1345-1358): integral sampling ratios, block
// grids at least as large as the MCU grid.
static int layout_step(rcg_ctx* ctx, StepDesc* st, int w, int h, const rcg_coef_layout* layout) {
  std::memset(st, 0, sizeof *st);
  st->active = 1;
  const int nc = layout->ncomp;
  st->ncomp = nc;
  int hmax = 1, vmax = 1;
  for (int c = 0; c < nc; c++) {
    hmax = std::max(hmax, (int)layout->h[c]);
    vmax = std::max(vmax, (int)layout->v[c]);
  }
  st->hmax = hmax;
  st->vmax = vmax;
  long long blk = 0, poff = 0;
  int mcus_x = (w + 8 * hmax - 1) / (8 * hmax), mcus_y = (h + 8 * vmax - 1) / (8 * vmax);
  st->mcus_x = mcus_x;
  st->mcus_y = mcus_y;
  for (int c = 0; c < nc; c++) {
    CompDesc& cd = st->comp[c];
    cd.h = layout->h[c];
    cd.v = layout->v[c];
    cd.bw = layout->blocks_w[c];
    cd.bh = layout->blocks_h[c];
    cd.cls = c == 0 ? 0 : 1;
    if (cd.h < 1 || cd.v < 1 || hmax % cd.h || vmax % cd.v)
      return fail(ctx, RCG_UNSUPPORTED, "non-integral chroma subsampling ratio");
    if (cd.bw < mcus_x * cd.h || cd.bh < mcus_y * cd.v)
      return fail(ctx, RCG_INVALID, "block grid smaller than the MCU grid");
    cd.blk0 = blk;
    cd.plane_off = poff;
    blk += (long long)cd.bw * cd.bh;
    poff += (long long)cd.bw * 8 * cd.bh * 8;
  }
  st->nblocks = blk;
  if (layout->ncoefs != blk * 64) return fail(ctx, RCG_INVALID, "layout.ncoefs does not match the block grids");
  return RCG_OK;
}

static long long plane_bytes(const StepDesc* st) {
  long long b = 0;
  for (int c = 0; c < st->ncomp; c++) b += (long long)st->comp[c].bw * 8 * st->comp[c].bh * 8;
  return b;
}

// ---- requantization

// Source tables per component (jpeg/src/encode.rs:121): the slot the component names, all ones where it is empty.
static int requant_inputs(rcg_ctx* ctx, const rcg_qtables* in, StepDesc* st) {
  if (!in) return fail(ctx, RCG_INVALID, "null tables");
  for (int c = 0; c < st->ncomp; c++) {
    int slot = in->tq[c];
    if (slot < 0 || slot > 3) return fail(ctx, RCG_INVALID, "table slot out of range");
    if (in->present[slot])
      std::memcpy(st->src_qt[c], in->qtables[slot], 64);
    else
      std::memset(st->src_qt[c], 1, 64);  // jpeg/src/encode.rs:121: unwrap_or([1; 64])
  }
  return RCG_OK;
}

static void qtables_out(const int tq[3], const uint8_t slot_qt[4][64], const int present[4], int ncomp,
                        rcg_qtables* out) {
  if (!out) return;
  std::memset(out, 0, sizeof *out);
  for (int c = 0; c < ncomp; c++) out->tq[c] = tq[c];
  for (int sl = 0; sl < 4; sl++) {
    out->present[sl] = present[sl];
    if (present[sl]) std::memcpy(out->qtables[sl], slot_qt[sl], 64);
  }
}

}  // namespace rcg

using namespace rcg;

extern "C" {

int rcg_ctx_create(int device, rcg_ctx** out) {
  if (!out) return RCG_INVALID;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return RCG_CUDA_ERROR;
  }
  rcg_ctx* ctx = new (std::nothrow) rcg_ctx;
  if (!ctx) return RCG_NO_MEMORY;
  ctx->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&ctx->own_stream,
                                                                                   cudaStreamNonBlocking)) !=
                                                        cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return RCG_CUDA_ERROR;
  }
  ctx->stream = ctx->own_stream;
  int rc = ensure_init(ctx);
  if (rc != RCG_OK) {
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return rc;
  }
  *out = ctx;
  return RCG_OK;
}

void rcg_ctx_destroy(rcg_ctx* ctx) {
  if (!ctx) return;
  for (rcg_ctx* wk : ctx->workers) rcg_ctx_destroy(wk);
  ctx->workers.clear();
  for (rcg_ctx* sub : ctx->lock_subs) rcg_ctx_destroy(sub);
  ctx->lock_subs.clear();
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  drop_graphs(ctx);
  for (auto& kv : ctx->bufs)
    if (kv.second.ptr) cudaFree(kv.second.ptr);
  if (ctx->lut16) cudaFree(ctx->lut16);
  if (ctx->pinned_in) cudaFreeHost(ctx->pinned_in);
  if (ctx->pinned_out) cudaFreeHost(ctx->pinned_out);
  for (auto& p : ctx->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->switch_event) cudaEventDestroy(ctx->switch_event);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

const char* rcg_last_error(const rcg_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int rcg_ctx_set_stream(rcg_ctx* ctx, void* stream) {
  if (!ctx) return RCG_INVALID;
  cudaStream_t next = stream ? (cudaStream_t)stream : ctx->own_stream;
  if (next == ctx->stream) return RCG_OK;
  // The context's workspace and stored graphs move to the new stream with it: work still queued on the old stream
  // must finish before the new stream touches the same buffers. An event recorded on the old stream and waited on
  // by the new one orders them without blocking the host. A stream under capture is left to the capturing caller
  // (an event of a capture cannot be waited on outside it).
  cudaSetDevice(ctx->device);
  cudaStreamCaptureStatus a = cudaStreamCaptureStatusNone, b = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(ctx->stream, &a) != cudaSuccess || cudaStreamIsCapturing(next, &b) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, RCG_CUDA_ERROR, "stream switch: cannot query the streams");
  }
  if (a == cudaStreamCaptureStatusNone && b == cudaStreamCaptureStatusNone) {
    if (!ctx->switch_event) {
      cudaError_t e = cudaEventCreateWithFlags(&ctx->switch_event, cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "stream switch event");
    }
    cudaError_t e = cudaEventRecord(ctx->switch_event, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(next, ctx->switch_event, 0);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stream switch ordering");
  }
  ctx->stream = next;
  return RCG_OK;
}

void* rcg_ctx_stream(const rcg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int rcg_ctx_synchronize(rcg_ctx* ctx) {
  if (!ctx) return RCG_INVALID;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
  return RCG_OK;
}

uint64_t rcg_ctx_launch_count(const rcg_ctx* ctx) { return ctx ? ctx->launches : 0; }

int rcg_ctx_set_profiling(rcg_ctx* ctx, int on) {
  if (!ctx) return RCG_INVALID;
  collect_times(ctx);
  ctx->profiling = on != 0;
  if (on) ctx->ktimes.clear();
  return RCG_OK;
}

int rcg_ctx_set_graphs(rcg_ctx* ctx, int on) {
  if (!ctx) return RCG_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->use_graphs = on != 0;
  if (!on) drop_graphs(ctx);
  return RCG_OK;
}

int rcg_ctx_graph_stats(const rcg_ctx* ctx, uint64_t* captures, uint64_t* replays) {
  if (!ctx) return RCG_INVALID;
  if (captures) *captures = ctx->graph_captures;
  if (replays) *replays = ctx->graph_replays;
  return RCG_OK;
}

int rcg_ctx_kernel_time(rcg_ctx* ctx, const char* name, uint64_t* launches, double* total_ms) {
  if (!ctx || !name) return RCG_INVALID;
  collect_times(ctx);
  auto it = ctx->ktimes.find(name);
  if (launches) *launches = it == ctx->ktimes.end() ? 0 : it->second.launches;
  if (total_ms) *total_ms = it == ctx->ktimes.end() ? 0.0 : it->second.ms;
  return RCG_OK;
}

int rcg_coef_layout_for(uint32_t width, uint32_t height, int channels, const rcg_encode_options* opts,
                        rcg_coef_layout* out) {
  if (!opts || !out || width == 0 || height == 0 || (channels != 1 && channels != 3)) return RCG_INVALID;
  int q = opts->quality < 1 ? 1 : (opts->quality > 100 ? 100 : opts->quality);
  layout_of((int)width, (int)height, channels, q, opts->subsampling, out);
  return RCG_OK;
}

int rcg_ctx_set_tie_band(rcg_ctx* ctx, double band) {
  if (!ctx) return RCG_INVALID;
  if (!(band >= 0.0)) return fail(ctx, RCG_INVALID, "the tie band must be >= 0");
  ctx->tie_band = band;
  return RCG_OK;
}

uint64_t rcg_ctx_tie_rescores(const rcg_ctx* ctx) { return ctx ? ctx->tie_rescores : 0; }

int rcg_ctx_set_band_chunks(rcg_ctx* ctx, int chunks) {
  if (!ctx) return RCG_INVALID;
  if (chunks < 0 || chunks > 64) return fail(ctx, RCG_INVALID, "band chunks must be 0 (autotune) or 1..64");
  if (chunks != ctx->band_chunks) drop_graphs(ctx);  // captured step loops hold the old band layout
  ctx->band_chunks = chunks;
  return RCG_OK;
}

int rcg_ctx_set_ref_cache(rcg_ctx* ctx, int on) {
  if (!ctx) return RCG_INVALID;
  if ((on != 0) != ctx->ref_cache) drop_graphs(ctx);  // captured step loops hold the old scorer launches
  ctx->ref_cache = on != 0;
  return RCG_OK;
}

int rcg_ctx_band_chunks(rcg_ctx* ctx, uint32_t width, uint32_t height) {
  if (!ctx || width < (uint32_t)kMinSide || height < (uint32_t)kMinSide) return 0;
  cudaSetDevice(ctx->device);
  return band_chunks(ctx, make_pyramid((int)width, (int)height));
}

// ---- scorer

static int score_device_images(rcg_ctx* ctx, const uint8_t* d_ref, const uint8_t* d_dist, int w, int h, int channels,
                               int depth, double* score) {
  PyramidDesc pd = make_pyramid(w, h);
  float* ref_pyr = (float*)workspace(ctx, "ref_pyr", (size_t)pd.floats * sizeof(float));
  float* dist_pyr = (float*)workspace(ctx, "dist_pyr", (size_t)pd.floats * sizeof(float));
  double* d_score = (double*)workspace(ctx, "score", sizeof(double));
  if (!ref_pyr || !dist_pyr || !d_score) return RCG_NO_MEMORY;
  int rc;
  if ((rc = to_linear(ctx, d_ref, w, h, channels, depth, ref_pyr)) != RCG_OK) return rc;
  if ((rc = to_linear(ctx, d_dist, w, h, channels, depth, dist_pyr)) != RCG_OK) return rc;
  build_pyramid(ctx, pd, ref_pyr);
  build_pyramid(ctx, pd, dist_pyr);
  score_pyramids(ctx, pd, ref_pyr, dist_pyr, d_score, nullptr, nullptr);
  double s = 0.0;
  cudaMemcpyAsync(&s, d_score, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if ((rc = finish(ctx, "ssimulacra2")) != RCG_OK) return rc;
  if (!std::isfinite(s)) return fail(ctx, RCG_INVALID, "SSIMULACRA 2 produced a non-finite score");
  *score = s;
  return RCG_OK;
}

int rcg_ssimulacra2(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* distorted, uint32_t width,
                    uint32_t height, int channels, int depth, double* score) {
  if (!ctx) return RCG_INVALID;
  if (!reference || !distorted || !score) return fail(ctx, RCG_INVALID, "null pointer");
  if (channels < 1 || channels > 4 || (depth != 8 && depth != 16))
    return fail(ctx, RCG_INVALID, "channels must be 1..4 and depth 8 or 16");
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
    return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
  cudaSetDevice(ctx->device);
  size_t bytes = (size_t)width * height * channels * (depth / 8);
  uint8_t* d_a = (uint8_t*)workspace(ctx, "img_a", bytes);
  uint8_t* d_b = (uint8_t*)workspace(ctx, "img_b", bytes);
  if (!d_a || !d_b) return RCG_NO_MEMORY;
  int rc;
  if ((rc = copy_to_device(ctx, d_a, reference, bytes)) != RCG_OK) return rc;
  if ((rc = copy_to_device(ctx, d_b, distorted, bytes)) != RCG_OK) return rc;
  return score_device_images(ctx, d_a, d_b, (int)width, (int)height, channels, depth, score);
}

int rcg_ssimulacra2_exact(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* distorted, uint32_t width,
                          uint32_t height, int channels, int depth, double* score) {
  if (!ctx) return RCG_INVALID;
  if (!reference || !distorted || !score) return fail(ctx, RCG_INVALID, "null pointer");
  if (channels < 1 || channels > 4 || (depth != 8 && depth != 16))
    return fail(ctx, RCG_INVALID, "channels must be 1..4 and depth 8 or 16");
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
    return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
  cudaSetDevice(ctx->device);
  const int w = (int)width, h = (int)height;
  const size_t bytes = (size_t)width * height * channels * (depth / 8), np = (size_t)3 * width * height;
  uint8_t* d_a = (uint8_t*)workspace(ctx, "img_a", bytes);
  uint8_t* d_b = (uint8_t*)workspace(ctx, "img_b", bytes);
  float* lin = (float*)workspace(ctx, "x_lin", 2 * np * sizeof(float), false);
  double* d_score = (double*)workspace(ctx, "x_score", sizeof(double), false);
  if (!d_a || !d_b || !lin || !d_score) return RCG_NO_MEMORY;
  int rc;
  if ((rc = copy_to_device(ctx, d_a, reference, bytes)) != RCG_OK) return rc;
  if ((rc = copy_to_device(ctx, d_b, distorted, bytes)) != RCG_OK) return rc;
  if ((rc = to_linear(ctx, d_a, w, h, channels, depth, lin)) != RCG_OK) return rc;
  if ((rc = to_linear(ctx, d_b, w, h, channels, depth, lin + np)) != RCG_OK) return rc;
  if ((rc = exact_score(ctx, lin, lin + np, w, h, d_score)) != RCG_OK) return rc;
  double s = 0.0;
  cudaMemcpyAsync(&s, d_score, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if ((rc = finish(ctx, "ssimulacra2_exact")) != RCG_OK) return rc;
  if (!std::isfinite(s)) return fail(ctx, RCG_INVALID, "SSIMULACRA 2 produced a non-finite score");
  *score = s;
  return RCG_OK;
}

int rcg_ssimulacra2_device(rcg_ctx* ctx, const uint8_t* d_reference, const uint8_t* d_distorted, uint32_t width,
                           uint32_t height, int channels, double* score) {
  if (!ctx) return RCG_INVALID;
  if (!d_reference || !d_distorted || !score) return fail(ctx, RCG_INVALID, "null pointer");
  if (channels != 1 && channels != 3) return fail(ctx, RCG_INVALID, "device scorer takes 8-bit Gray or Rgb");
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
    return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
  cudaSetDevice(ctx->device);
  return score_device_images(ctx, d_reference, d_distorted, (int)width, (int)height, channels, 8, score);
}

// ---- many pairs at once

static int check_pairs(rcg_ctx* ctx, int n, const void* a, const void* b, const uint32_t* widths,
                       const uint32_t* heights, const int* channels, const int* depths, const double* scores) {
  if (n < 0 || n > 65535) return fail(ctx, RCG_INVALID, "a batch holds 0..=65535 pairs");
  if (n > 0 && (!a || !b || !widths || !heights || !channels || !scores)) return fail(ctx, RCG_INVALID, "null pointer");
  for (int i = 0; i < n; i++) {
    const int depth = depths ? depths[i] : 8;
    if (channels[i] < 1 || channels[i] > 4 || (depth != 8 && depth != 16))
      return fail(ctx, RCG_INVALID, "pair " + std::to_string(i) + ": channels must be 1..4 and depth 8 or 16");
    if (widths[i] < (uint32_t)kMinSide || heights[i] < (uint32_t)kMinSide)
      return fail(ctx, RCG_INVALID, "pair " + std::to_string(i) + ": SSIMULACRA 2 needs at least 8x8 pixels");
  }
  return RCG_OK;
}

static int batch_scores_out(rcg_ctx* ctx, int n, const double* d_scores, double* scores) {
  int rc = copy_to_host(ctx, scores, d_scores, (size_t)n * sizeof(double));
  if (rc != RCG_OK) return rc;
  if ((rc = finish(ctx, "ssimulacra2 batch")) != RCG_OK) return rc;
  for (int i = 0; i < n; i++)
    if (!std::isfinite(scores[i]))
      return fail(ctx, RCG_INVALID, "pair " + std::to_string(i) + ": SSIMULACRA 2 produced a non-finite score");
  return RCG_OK;
}

int rcg_ssimulacra2_batch_device(rcg_ctx* ctx, int n, const uint8_t* const* d_references,
                                 const uint8_t* const* d_distorted, const uint32_t* widths, const uint32_t* heights,
                                 const int* channels, const int* depths, double* scores) {
  if (!ctx) return RCG_INVALID;
  int rc = check_pairs(ctx, n, d_references, d_distorted, widths, heights, channels, depths, scores);
  if (rc != RCG_OK || n == 0) return rc;
  for (int i = 0; i < n; i++)
    if (!d_references[i] || !d_distorted[i]) return fail(ctx, RCG_INVALID, "null pointer");
  cudaSetDevice(ctx->device);
  double* d_scores = nullptr;
  if ((rc = score_batch(ctx, n, d_references, d_distorted, widths, heights, channels, depths, &d_scores)) != RCG_OK)
    return rc;
  return batch_scores_out(ctx, n, d_scores, scores);
}

int rcg_ssimulacra2_batch(rcg_ctx* ctx, int n, const uint8_t* const* references, const uint8_t* const* distorted,
                          const uint32_t* widths, const uint32_t* heights, const int* channels, const int* depths,
                          double* scores) {
  if (!ctx) return RCG_INVALID;
  int rc = check_pairs(ctx, n, references, distorted, widths, heights, channels, depths, scores);
  if (rc != RCG_OK || n == 0) return rc;
  for (int i = 0; i < n; i++)
    if (!references[i] || !distorted[i]) return fail(ctx, RCG_INVALID, "null pointer");
  cudaSetDevice(ctx->device);
  // One device copy per distinct host image: pairs that pass the same reference buffer (several candidates of one
  // image) upload it once and share its planes in the scorer.
  auto bytes_of = [&](int i) {
    return (size_t)widths[i] * heights[i] * channels[i] * ((depths ? depths[i] : 8) / 8);
  };
  std::map<std::tuple<const uint8_t*, uint32_t, uint32_t, int, int>, size_t> ref_off;
  std::vector<size_t> roff((size_t)n), doff((size_t)n);
  size_t total = 0;
  auto take = [&](size_t b) {
    size_t o = total;
    total += (b + 255) / 256 * 256;
    return o;
  };
  for (int i = 0; i < n; i++) {
    auto key = std::make_tuple(references[i], widths[i], heights[i], channels[i], depths ? depths[i] : 8);
    auto it = ref_off.find(key);
    if (it == ref_off.end()) it = ref_off.emplace(key, take(bytes_of(i))).first;
    roff[(size_t)i] = it->second;
    doff[(size_t)i] = take(bytes_of(i));
  }
  uint8_t* d_imgs = (uint8_t*)workspace(ctx, "batch_imgs", total);
  if (!d_imgs) return RCG_NO_MEMORY;
  std::vector<const uint8_t*> d_ref((size_t)n), d_dist((size_t)n);
  std::vector<char> sent(total / 256 + 1, 0);
  for (int i = 0; i < n; i++) {
    d_ref[(size_t)i] = d_imgs + roff[(size_t)i];
    d_dist[(size_t)i] = d_imgs + doff[(size_t)i];
    if (!sent[roff[(size_t)i] / 256]) {
      sent[roff[(size_t)i] / 256] = 1;
      if ((rc = copy_to_device(ctx, d_imgs + roff[(size_t)i], references[i], bytes_of(i))) != RCG_OK) return rc;
    }
    if ((rc = copy_to_device(ctx, d_imgs + doff[(size_t)i], distorted[i], bytes_of(i))) != RCG_OK) return rc;
  }
  double* d_scores = nullptr;
  if ((rc = score_batch(ctx, n, d_ref.data(), d_dist.data(), widths, heights, channels, depths, &d_scores)) !=
      RCG_OK)
    return rc;
  return batch_scores_out(ctx, n, d_scores, scores);
}

// ---- rate-quality sweep

// Device bytes one image of a sweep holds until its group is scored: the image and its candidates (8-bit), and both
// sides' linear pyramids in the scorer (3 channels, 4/3 for the coarser scales, 4-byte floats: 16 B per pixel).
static size_t sweep_bytes(uint32_t w, uint32_t h, int channels, int nq) {
  const size_t px = (size_t)w * h;
  return (px * channels + 16 * px) * (size_t)(nq + 1);
}
constexpr size_t kSweepGroupBytes = 8ull << 30;  // images per group: as many as fit this estimate

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// A group of images of rcg_sweep_qualities: every image's candidates at every quality encoded and decoded to 8-bit
// pixels on the device, then all of the group's pairs scored by one work-list scorer call (each image converted once
// as the reference of its candidates).
static int sweep_group(rcg_ctx* ctx, int n, const uint8_t* const* images, const uint32_t* widths,
                       const uint32_t* heights, const int* channels, int nq, const int* qualities,
                       const rcg_encode_options* opts, double* scores) {
  int rc;
  std::vector<size_t> img_off((size_t)n), cand_off((size_t)n), img_bytes((size_t)n);
  size_t tot_img = 0, tot_cand = 0;
  for (int i = 0; i < n; i++) {
    img_bytes[(size_t)i] = (size_t)widths[i] * heights[i] * channels[i];
    img_off[(size_t)i] = tot_img;
    tot_img += align256(img_bytes[(size_t)i]);
    cand_off[(size_t)i] = tot_cand;
    tot_cand += align256(img_bytes[(size_t)i]) * (size_t)nq;
  }
  // build_coefs' tables per (image, quality) (jpeg/src/encode.rs:426-539), one descriptor per candidate.
  std::vector<StepDesc> st((size_t)n * nq);
  long long max_coefs = 0, max_planes = 0;
  for (int i = 0; i < n; i++)
    for (int k = 0; k < nq; k++) {
      StepDesc& d = st[(size_t)i * nq + k];
      host_step_tables(&d, qualities[k], opts->subsampling, channels[i], opts->trellis, (int)widths[i],
                       (int)heights[i]);
      max_coefs = std::max(max_coefs, d.nblocks * 64);
      max_planes = std::max(max_planes, plane_bytes(&d));
    }
  uint8_t* d_imgs = (uint8_t*)workspace(ctx, "sweep_imgs", tot_img);
  uint8_t* d_cand = (uint8_t*)workspace(ctx, "sweep_cands", tot_cand);
  int16_t* d_coefs = (int16_t*)workspace(ctx, "sweep_coefs", (size_t)max_coefs * 2);
  uint8_t* d_planes = (uint8_t*)workspace(ctx, "sweep_planes", (size_t)max_planes);
  StepDesc* d_sts = (StepDesc*)workspace(ctx, "sweep_steps", sizeof(StepDesc) * st.size());
  if (!d_imgs || !d_cand || !d_coefs || !d_planes || !d_sts) return RCG_NO_MEMORY;
  for (StepDesc& d : st) d.coefs = d_coefs;  // one candidate at a time, in stream order
  // Host copies first: a pageable copy waits for the stream, so they go before any kernel of the group.
  for (int i = 0; i < n; i++)
    if ((rc = copy_to_device(ctx, d_imgs + img_off[(size_t)i], images[i], img_bytes[(size_t)i])) != RCG_OK) return rc;
  cudaError_t e = cudaMemcpyAsync(d_sts, st.data(), sizeof(StepDesc) * st.size(), cudaMemcpyHostToDevice,
                                  ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "sweep tables upload");
  std::vector<const uint8_t*> refs(st.size()), dists(st.size());
  std::vector<uint32_t> ws(st.size()), hs(st.size());
  std::vector<int> cs(st.size());
  for (int i = 0; i < n; i++) {
    const uint8_t* d_src = d_imgs + img_off[(size_t)i];
    EncoderSetup es;
    if ((rc = setup_encoder(ctx, d_src, (int)widths[i], (int)heights[i], channels[i], opts->subsampling, &es)) !=
        RCG_OK)
      return rc;
    for (int k = 0; k < nq; k++) {
      const size_t j = (size_t)i * nq + k;
      StepDesc* d_st = d_sts + j;
      quantize(ctx, d_st, es.caches, es.max_blocks);
      rate_tables(ctx, d_st);
      trellis(ctx, d_st, es.caches, es.max_blocks);
      dequant_idct(ctx, d_st, nullptr, d_planes, es.max_blocks);  // reconstruct (jpeg/src/decode.rs:334-389)
      uint8_t* out = d_cand + cand_off[(size_t)i] + align256(img_bytes[(size_t)i]) * (size_t)k;
      upsample_color(ctx, d_st, d_planes, (int)widths[i], (int)heights[i], out, nullptr);
      refs[j] = d_src;
      dists[j] = out;
      ws[j] = widths[i];
      hs[j] = heights[i];
      cs[j] = channels[i];
    }
  }
  double* d_scores = nullptr;
  if ((rc = score_batch(ctx, (int)st.size(), refs.data(), dists.data(), ws.data(), hs.data(), cs.data(), nullptr,
                        &d_scores)) != RCG_OK)
    return rc;
  if ((rc = copy_to_host(ctx, scores, d_scores, sizeof(double) * st.size())) != RCG_OK) return rc;
  return finish(ctx, "sweep");
}

int rcg_sweep_qualities(rcg_ctx* ctx, int n, const uint8_t* const* images, const uint32_t* widths,
                        const uint32_t* heights, const int* channels, int nq, const int* qualities,
                        const rcg_encode_options* opts, double* scores) {
  if (!ctx) return RCG_INVALID;
  if (n < 0 || nq < 1 || nq > 100) return fail(ctx, RCG_INVALID, "a sweep takes n >= 0 images and 1..=100 qualities");
  if (n == 0) return RCG_OK;
  if (!images || !widths || !heights || !channels || !qualities || !scores) return fail(ctx, RCG_INVALID, "null pointer");
  int rc = check_opts(ctx, opts, false);
  if (rc != RCG_OK) return rc;
  for (int k = 0; k < nq; k++)
    if (qualities[k] < 1 || qualities[k] > 100) return fail(ctx, RCG_INVALID, "qualities are 1..=100");
  for (int i = 0; i < n; i++) {
    if (!images[i]) return fail(ctx, RCG_INVALID, "null pointer");
    if ((rc = check_image(ctx, widths[i], heights[i], channels[i])) != RCG_OK) return rc;
    if (widths[i] < (uint32_t)kMinSide || heights[i] < (uint32_t)kMinSide)
      return fail(ctx, RCG_INVALID, "image " + std::to_string(i) + ": SSIMULACRA 2 needs at least 8x8 pixels");
  }
  cudaSetDevice(ctx->device);
  for (int i0 = 0; i0 < n;) {
    int i1 = i0 + 1;
    size_t bytes = sweep_bytes(widths[i0], heights[i0], channels[i0], nq);
    while (i1 < n && (size_t)(i1 - i0 + 1) * nq <= 65535 &&
           bytes + sweep_bytes(widths[i1], heights[i1], channels[i1], nq) <= kSweepGroupBytes)
      bytes += sweep_bytes(widths[i1], heights[i1], channels[i1], nq), i1++;
    if ((rc = sweep_group(ctx, i1 - i0, images + i0, widths + i0, heights + i0, channels + i0, nq, qualities, opts,
                          scores + (size_t)i0 * nq)) != RCG_OK)
      return rc;
    i0 = i1;
  }
  for (int i = 0; i < n; i++)
    for (int k = 0; k < nq; k++)
      if (!std::isfinite(scores[(size_t)i * nq + k]))
        return fail(ctx, RCG_INVALID, "image " + std::to_string(i) + ": SSIMULACRA 2 produced a non-finite score");
  return RCG_OK;
}

// ---- other metrics

static int metric_on_device(rcg_ctx* ctx, int metric, const uint8_t* d_a, const uint8_t* d_b, int w, int h, int ch,
                            double* score) {
  int rc;
  if (metric == RCG_METRIC_SSIMULACRA2) {
    if (w < kMinSide || h < kMinSide) return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
    return score_device_images(ctx, d_a, d_b, w, h, ch, 8, score);
  }
  if (metric == RCG_METRIC_SSIM) {
    double* d = (double*)workspace(ctx, "metric_score", sizeof(double) * 8);
    if (!d) return RCG_NO_MEMORY;
    if ((rc = ssim_score(ctx, d_a, d_b, w, h, ch, d, nullptr, nullptr)) != RCG_OK) return rc;
    cudaMemcpyAsync(score, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    return finish(ctx, "ssim");
  }
  if (metric == RCG_METRIC_PSNR) {
    // core/src/metrics.rs:67-73: mean squared error over every sample, +infinity for identical images
    unsigned long long* d = (unsigned long long*)workspace(ctx, "metric_sq", sizeof(unsigned long long));
    if (!d) return RCG_NO_MEMORY;
    const size_t n = (size_t)w * h * ch;
    squared_error(ctx, d_a, d_b, n, d);
    unsigned long long se = 0;
    cudaMemcpyAsync(&se, d, sizeof se, cudaMemcpyDeviceToHost, ctx->stream);
    if ((rc = finish(ctx, "psnr")) != RCG_OK) return rc;
    const double mse = (double)se / (double)std::max<size_t>(n, 1);
    *score = mse == 0.0 ? INFINITY : 10.0 * std::log10(255.0 * 255.0 / mse);
    return RCG_OK;
  }
  if (metric == RCG_METRIC_MS_SSIM) {
    // core/src/metrics.rs:111-127: luma SSIM at five dyadic scales, clamped at 1e-9, combined with the weights.
    static const double kW[5] = {0.0448, 0.2856, 0.3001, 0.2363, 0.1333};
    const size_t npx = (size_t)w * h;
    uint8_t* x = (uint8_t*)workspace(ctx, "msssim_x", npx);
    uint8_t* y = (uint8_t*)workspace(ctx, "msssim_y", npx);
    uint8_t* x2 = (uint8_t*)workspace(ctx, "msssim_x2", npx / 4 + 1);
    uint8_t* y2 = (uint8_t*)workspace(ctx, "msssim_y2", npx / 4 + 1);
    double* d = (double*)workspace(ctx, "metric_score", sizeof(double) * 8);
    if (!x || !y || !x2 || !y2 || !d) return RCG_NO_MEMORY;
    luma8(ctx, d_a, npx, ch, x);
    luma8(ctx, d_b, npx, ch, y);
    int cw = w, chh = h;
    for (int i = 0; i < 5; i++) {
      if ((rc = ssim_score(ctx, x, y, cw, chh, 1, d + i, nullptr, nullptr)) != RCG_OK) return rc;
      if (i + 1 < 5 && cw / 2 > 0 && chh / 2 > 0) {
        downsample2(ctx, x, cw, chh, x2);
        downsample2(ctx, y, cw, chh, y2);
        std::swap(x, x2);
        std::swap(y, y2);
        cw /= 2;
        chh /= 2;
      }
    }
    double s[5];
    cudaMemcpyAsync(s, d, sizeof s, cudaMemcpyDeviceToHost, ctx->stream);
    if ((rc = finish(ctx, "ms_ssim")) != RCG_OK) return rc;
    double out = 1.0;
    for (int i = 0; i < 5; i++) out *= std::pow(std::max(s[i], 1e-9), kW[i]);
    *score = out;
    return RCG_OK;
  }
  return fail(ctx, RCG_INVALID, "unknown metric");
}

int rcg_metric_score(rcg_ctx* ctx, int metric, const uint8_t* reference, const uint8_t* candidate, uint32_t width,
                     uint32_t height, int channels, double* score) {
  if (!ctx) return RCG_INVALID;
  if (!reference || !candidate || !score) return fail(ctx, RCG_INVALID, "null pointer");
  if (channels < 1 || channels > 4) return fail(ctx, RCG_INVALID, "channels must be 1..4");
  if (width == 0 || height == 0) return fail(ctx, RCG_INVALID, "empty image");
  cudaSetDevice(ctx->device);
  const size_t bytes = (size_t)width * height * channels;
  uint8_t* d_a = (uint8_t*)workspace(ctx, "img_a", bytes);
  uint8_t* d_b = (uint8_t*)workspace(ctx, "img_b", bytes);
  if (!d_a || !d_b) return RCG_NO_MEMORY;
  int rc;
  if ((rc = copy_to_device(ctx, d_a, reference, bytes)) != RCG_OK) return rc;
  if ((rc = copy_to_device(ctx, d_b, candidate, bytes)) != RCG_OK) return rc;
  return metric_on_device(ctx, metric, d_a, d_b, (int)width, (int)height, channels, score);
}

int rcg_metric_score_device(rcg_ctx* ctx, int metric, const uint8_t* d_reference, const uint8_t* d_candidate,
                            uint32_t width, uint32_t height, int channels, double* score) {
  if (!ctx) return RCG_INVALID;
  if (!d_reference || !d_candidate || !score) return fail(ctx, RCG_INVALID, "null pointer");
  if (channels < 1 || channels > 4) return fail(ctx, RCG_INVALID, "channels must be 1..4");
  if (width == 0 || height == 0) return fail(ctx, RCG_INVALID, "empty image");
  cudaSetDevice(ctx->device);
  return metric_on_device(ctx, metric, d_reference, d_candidate, (int)width, (int)height, channels, score);
}

// ---- encoder

// build_coefs (jpeg/src/encode.rs:426-539); `weights` (host, nullable, ncoefs entries) runs the trellis pass in the
// perceptual mode.
static int build_coefs_impl(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                            const rcg_encode_options* opts, const float* weights, size_t weights_len, int16_t* coefs,
                            size_t coefs_len, uint8_t* qtables) {
  if (!ctx) return RCG_INVALID;
  int rc;
  if ((rc = check_image(ctx, width, height, channels)) != RCG_OK) return rc;
  if ((rc = check_opts(ctx, opts, true)) != RCG_OK) return rc;
  if (!src || !coefs) return fail(ctx, RCG_INVALID, "null pointer");
  int w = (int)width, h = (int)height;
  StepDesc* st = new StepDesc;
  host_step_tables(st, opts->quality, opts->subsampling, channels, opts->trellis, w, h);
  long long ncoefs = st->nblocks * 64;
  if ((long long)coefs_len < ncoefs) {
    delete st;
    return fail(ctx, RCG_INVALID, "coefficient buffer too short");
  }
  if (weights && (long long)weights_len != ncoefs) {
    delete st;
    return fail(ctx, RCG_INVALID, "weights do not match the coefficient layout");
  }
  cudaSetDevice(ctx->device);
  size_t bytes = (size_t)w * h * channels;
  uint8_t* d_src = (uint8_t*)workspace(ctx, "img_a", bytes);
  int16_t* d_coefs = (int16_t*)workspace(ctx, "coefs_single", (size_t)ncoefs * 2);
  StepDesc* d_st = (StepDesc*)workspace(ctx, "step_single", sizeof(StepDesc));
  float* d_w = weights ? (float*)workspace(ctx, "weights_single", (size_t)ncoefs * sizeof(float)) : nullptr;
  if (!d_src || !d_coefs || !d_st || (weights && !d_w)) {
    delete st;
    return RCG_NO_MEMORY;
  }
  st->coefs = d_coefs;
  st->pweights = d_w;
  if (weights) cudaMemcpyAsync(d_w, weights, (size_t)ncoefs * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(d_src, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(d_st, st, sizeof(StepDesc), cudaMemcpyHostToDevice, ctx->stream);
  EncoderSetup es;
  // Only this quality's layout is needed: pin Auto to what it resolves to.
  int sub = opts->subsampling;
  if (channels == 3 && sub == RCG_SUB_AUTO) sub = opts->quality < 90 ? RCG_SUB_420 : RCG_SUB_444;
  if ((rc = setup_encoder(ctx, d_src, w, h, channels, sub, &es)) != RCG_OK) {
    delete st;
    return rc;
  }
  quantize(ctx, d_st, es.caches, st->nblocks);
  rate_tables(ctx, d_st);
  trellis(ctx, d_st, es.caches, st->nblocks, weights != nullptr);
  cudaMemcpyAsync(coefs, d_coefs, (size_t)ncoefs * 2, cudaMemcpyDeviceToHost, ctx->stream);
  if (qtables) {
    std::memcpy(qtables, st->qt[0], 64);
    std::memcpy(qtables + 64, st->qt[1], 64);
  }
  cudaStreamSynchronize(ctx->stream);  // the host StepDesc must outlive the async upload
  delete st;
  return finish(ctx, "build_coefs");
}

int rcg_build_coefs(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                    const rcg_encode_options* opts, int16_t* coefs, size_t coefs_len, uint8_t* qtables) {
  return build_coefs_impl(ctx, src, width, height, channels, opts, nullptr, 0, coefs, coefs_len, qtables);
}

int rcg_build_coefs_weighted(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                             const rcg_encode_options* opts, const float* weights, size_t weights_len, int16_t* coefs,
                             size_t coefs_len, uint8_t* qtables) {
  if (!ctx) return RCG_INVALID;
  if (!weights) return fail(ctx, RCG_INVALID, "null weights");
  return build_coefs_impl(ctx, src, width, height, channels, opts, weights, weights_len, coefs, coefs_len, qtables);
}

// ---- decoder

// reconstruct (jpeg/src/decode.rs:334-389) with the multipliers already in `st` (owned; deleted here).
static int reconstruct_with(rcg_ctx* ctx, StepDesc* st, int w, int h, const int16_t* coefs, uint8_t* out,
                            size_t out_len) {
  const int nc = st->ncomp;
  long long blk = st->nblocks, poff = plane_bytes(st);
  if (out_len < (size_t)w * h * nc) {
    delete st;
    return fail(ctx, RCG_INVALID, "output buffer too short");
  }
  cudaSetDevice(ctx->device);
  int16_t* d_coefs = (int16_t*)workspace(ctx, "coefs_single", (size_t)blk * 64 * 2);
  uint8_t* d_planes = (uint8_t*)workspace(ctx, "dec_planes_single", (size_t)poff);
  uint8_t* d_out = (uint8_t*)workspace(ctx, "img_b", (size_t)w * h * nc);
  StepDesc* d_st = (StepDesc*)workspace(ctx, "step_single", sizeof(StepDesc));
  if (!d_coefs || !d_planes || !d_out || !d_st) {
    delete st;
    return RCG_NO_MEMORY;
  }
  cudaMemcpyAsync(d_coefs, coefs, (size_t)blk * 64 * 2, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(d_st, st, sizeof(StepDesc), cudaMemcpyHostToDevice, ctx->stream);
  dequant_idct(ctx, d_st, d_coefs, d_planes, blk);
  upsample_color(ctx, d_st, d_planes, w, h, d_out, nullptr);
  cudaMemcpyAsync(out, d_out, (size_t)w * h * nc, cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  delete st;
  return finish(ctx, "reconstruct");
}

static int reconstruct_checks(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                              const void* tables, const int16_t* coefs, uint8_t* out, StepDesc** st_out) {
  if (!layout || !tables || !coefs || !out) return fail(ctx, RCG_INVALID, "null pointer");
  if (width == 0 || height == 0) return fail(ctx, RCG_INVALID, "empty image");
  if (layout->ncomp != 1 && layout->ncomp != 3) return fail(ctx, RCG_UNSUPPORTED, "reconstruct takes 1 or 3 components");
  StepDesc* st = new StepDesc;
  int rc = layout_step(ctx, st, (int)width, (int)height, layout);
  if (rc != RCG_OK) {
    delete st;
    return rc;
  }
  *st_out = st;
  return RCG_OK;
}

int rcg_reconstruct(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                    const uint8_t* qtables, const int16_t* coefs, uint8_t* out, size_t out_len) {
  if (!ctx) return RCG_INVALID;
  StepDesc* st = nullptr;
  int rc = reconstruct_checks(ctx, width, height, layout, qtables, coefs, out, &st);
  if (rc != RCG_OK) return rc;
  // idct_planes multipliers from the given tables (jpeg/src/decode.rs:1316-1321)
  fill_mult(st, qtables, st->ncomp == 1 ? 1 : 2);
  return reconstruct_with(ctx, st, (int)width, (int)height, coefs, out, out_len);
}

int rcg_reconstruct_tables(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                           const rcg_qtables* tables, const int16_t* coefs, uint8_t* out, size_t out_len) {
  if (!ctx) return RCG_INVALID;
  StepDesc* st = nullptr;
  int rc = reconstruct_checks(ctx, width, height, layout, tables, coefs, out, &st);
  if (rc == RCG_OK) rc = requant_inputs(ctx, tables, st);
  if (rc != RCG_OK) {
    delete st;
    return rc;
  }
  for (int c = 0; c < st->ncomp; c++)
    for (int n = 0; n < 64; n++) st->mult[c][n] = mult_entry_host(st->src_qt[c], n);
  return reconstruct_with(ctx, st, (int)width, (int)height, coefs, out, out_len);
}

// ---- search

// Per-candidate scorer of the device searches: SSIMULACRA2 from the candidate's linear pyramid against the
// reference's, or SSIM from the candidate's 8-bit pixels against the reference's.
struct SearchScorer {
  int metric;
  PyramidDesc pd;
  float* ref_pyr = nullptr;
  float* dist_pyr = nullptr;
  float2* ref_moments = nullptr;  // the reference's blurred a', a'^2 per pyramid pixel (null: the cache is off)
  const uint8_t* ref_px = nullptr;
  uint8_t* cand_px = nullptr;
  double* d_score = nullptr;
  bool fuse420 = false;  // every candidate has the 4:2:0 layout of upsample_pyramid (set by the search's setup)
};

// Whether a host-side layout is the 4:2:0 case of upsample_pyramid.
static bool layout_fast420(const StepDesc* st, int w) {
  const CompDesc& c0 = st->comp[0];
  return st->ncomp == 3 && st->hmax == 2 && st->vmax == 2 && c0.h == 2 && c0.v == 2 && st->comp[1].h == 1 &&
         st->comp[1].v == 1 && st->comp[2].h == 1 && st->comp[2].v == 1 && w % 4 == 0;
}

// Every buffer the per-candidate scoring uses is allocated here, before the step loop: the loop itself never
// allocates (it may be captured as a graph, and a failed allocation inside it would go unnoticed).
static int scorer_setup(rcg_ctx* ctx, int metric, int w, int h, int channels, SearchScorer* sc) {
  sc->metric = metric;
  sc->d_score = (double*)workspace(ctx, "score", sizeof(double));
  if (!sc->d_score) return RCG_NO_MEMORY;
  if (metric == RCG_METRIC_SSIM) {
    sc->cand_px = (uint8_t*)workspace(ctx, "cand_px", (size_t)w * h * channels);
    if (!sc->cand_px) return RCG_NO_MEMORY;
    if (w >= 8 && h >= 8 && !workspace(ctx, "ssim_rows", sizeof(double) * (size_t)((h - 8) / 4 + 1)))
      return RCG_NO_MEMORY;
    return RCG_OK;
  }
  sc->pd = make_pyramid(w, h);
  sc->ref_pyr = (float*)workspace(ctx, "ref_pyr", (size_t)sc->pd.floats * sizeof(float));
  sc->dist_pyr = (float*)workspace(ctx, "dist_pyr", (size_t)sc->pd.floats * sizeof(float));
  if (!sc->ref_pyr || !sc->dist_pyr) return RCG_NO_MEMORY;
  if (ctx->ref_cache) {
    // Sized for the band layout the scorer will run (the same plan_bands call score_pyramids makes).
    sc->ref_moments = (float2*)workspace(ctx, "ref_moments", ref_moment_bytes(plan_bands(ctx, sc->pd)));
    if (!sc->ref_moments) return RCG_NO_MEMORY;
  }
  return score_workspace(ctx, sc->pd);
}

// Decoded planes of one candidate -> score -> one bisection step (all gated by the step's `active`). Step `s` of the
// loop: the first candidate of a search (s = 0, always active) stores the reference moments, later ones read them.
static void score_candidate(rcg_ctx* ctx, const SearchScorer& sc, StepDesc* d_st, const uint8_t* planes, int w,
                            int h, int channels, SearchState* d_ss, int s) {
  if (sc.metric == RCG_METRIC_SSIM) {
    upsample_color(ctx, d_st, planes, w, h, sc.cand_px, nullptr);
    ssim_score(ctx, sc.ref_px, sc.cand_px, w, h, channels, sc.d_score, d_ss, d_st);
    return;
  }
  if (sc.fuse420) {
    upsample_pyramid(ctx, d_st, planes, w, h, sc.pd, sc.dist_pyr);
  } else {
    upsample_color(ctx, d_st, planes, w, h, nullptr, sc.dist_pyr);
    build_pyramid_gated(ctx, sc.pd, sc.dist_pyr, d_st);
  }
  score_pyramids(ctx, sc.pd, sc.ref_pyr, sc.dist_pyr, sc.d_score, d_ss, d_st, sc.ref_moments,
                 s == 0 ? kRefWrite : kRefRead);
}

// Near ties. jpeg/src/target.rs:48 accepts a candidate on s >= target; the fast scorer is within about 1e-6 of the
// reference, so a candidate scored within ctx->tie_band of the target paused the device bisection (search_record,
// done = 2) with its decoded linear planes still at scale 0 of the candidate pyramid (every later step was
// inactive). Here it is rescored in the reference's f64 arithmetic and order on the GPU (exact_score), the bisection
// records that score and goes on, and the remaining steps run as plain launches; repeated while a later candidate
// pauses again. `issue_step(s)` issues step s's kernels.
static int settle_ties(rcg_ctx* ctx, const SearchScorer& sc, SearchState* d_ss, SearchState* hs, int max_steps,
                       int w, int h, const std::function<void(int)>& issue_step) {
  while (hs->done == 2) {
    if (sc.metric != RCG_METRIC_SSIMULACRA2) return fail(ctx, RCG_INVALID, "paused search without a rescorer");
    double* d_exact = (double*)workspace(ctx, "x_score", sizeof(double), false);
    if (!d_exact) return RCG_NO_MEMORY;
    int rc = exact_score(ctx, sc.ref_pyr, sc.dist_pyr, w, h, d_exact);
    if (rc != RCG_OK) return rc;
    search_resume(ctx, d_ss, d_exact);
    ctx->tie_rescores++;
    for (int s = hs->step + 1; s < max_steps; s++) issue_step(s);
    cudaMemcpyAsync(hs, d_ss, sizeof *hs, cudaMemcpyDeviceToHost, ctx->stream);
    if ((rc = finish(ctx, "search after a near tie")) != RCG_OK) return rc;
  }
  return RCG_OK;
}

// One device search from set-up to collection: its buffers (in the context's workspace), the encoder's set-up and
// the scorer.
struct SearchRun {
  int w = 0, h = 0, channels = 0, metric = 0, subsampling = 0, max_steps = 0;
  SearchScorer sc;
  EncoderSetup es;
  SearchState* d_ss = nullptr;
  StepDesc* d_st = nullptr;
  int16_t* slots = nullptr;
  uint8_t* planes = nullptr;
};

// Everything before the step loop, queued on the context's stream: the buffers, the quality-independent work (the
// reference image's linear pyramid for SSIMULACRA2, colour planes, FDCTs) and the initial bisection state.
static int search_prepare(rcg_ctx* ctx, const uint8_t* d_src, int w, int h, int channels, int metric, double target,
                          int max_q, int subsampling, int trellis_on, SearchRun* run) {
  int rc;
  run->w = w;
  run->h = h;
  run->channels = channels;
  run->metric = metric;
  run->subsampling = subsampling;
  SearchScorer& sc = run->sc;
  run->d_ss = (SearchState*)workspace(ctx, "search_state", sizeof(SearchState));
  run->d_st = (StepDesc*)workspace(ctx, "step_search", sizeof(StepDesc));
  if (!run->d_ss || !run->d_st) return RCG_NO_MEMORY;
  if ((rc = scorer_setup(ctx, metric, w, h, channels, &sc)) != RCG_OK) return rc;
  if (metric == RCG_METRIC_SSIM) {
    sc.ref_px = d_src;
  } else {
    if ((rc = to_linear(ctx, d_src, w, h, channels, 8, sc.ref_pyr)) != RCG_OK) return rc;
    build_pyramid(ctx, sc.pd, sc.ref_pyr);
  }
  // Every candidate of an explicit 4:2:0 colour search has the fused layout (the sampling factors of
  // jpeg/src/encode.rs:428-439 do not depend on the quality then).
  sc.fuse420 = metric == RCG_METRIC_SSIMULACRA2 && channels != 1 && subsampling == RCG_SUB_420 && w % 4 == 0;
  if ((rc = setup_encoder(ctx, d_src, w, h, channels, subsampling, &run->es)) != RCG_OK) return rc;
  int max_steps = 1;
  for (int span = max_q; span > 1; span = (span + 1) / 2) max_steps++;
  run->max_steps = std::min(max_steps, kMaxSteps);
  run->slots = (int16_t*)workspace(ctx, "coef_slots", (size_t)run->es.max_coefs * 2 * run->max_steps);
  run->planes = (uint8_t*)workspace(ctx, "dec_planes", (size_t)run->es.max_plane_bytes);
  if (!run->slots || !run->planes) return RCG_NO_MEMORY;
  SearchState hs;
  std::memset(&hs, 0, sizeof hs);
  hs.lo = 1;
  hs.hi = max_q;
  hs.step = 0;
  hs.qs[0] = max_q;
  hs.target = target;
  hs.max_q = max_q;
  hs.subsampling = subsampling;
  hs.trellis = trellis_on;
  hs.channels = channels;
  hs.best_q = max_q;
  hs.tie_band = metric == RCG_METRIC_SSIMULACRA2 ? ctx->tie_band : 0.0;
  // A copy from pageable memory returns once the source is staged, so `hs` may go out of scope.
  cudaError_t e = cudaMemcpyAsync(run->d_ss, &hs, sizeof hs, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "search state upload");
  return RCG_OK;
}

// The result of a finished search: Found, and the chosen coefficients and tables to device or host buffers.
static int search_collect(rcg_ctx* ctx, const SearchRun& run, const SearchState& hs, rcg_found* found,
                          int16_t* d_coefs_out, size_t coefs_len, uint8_t* d_qt_out, int16_t* h_coefs_out,
                          uint8_t* h_qt_out, bool partial = false) {
  int rc;
  if (!hs.done && !partial) return fail(ctx, RCG_TIMEOUT, "bisection did not finish within the step budget");
  found->quality = hs.best_q;
  found->score = hs.best_score;
  found->nsteps = 0;
  for (int s = 0; s < kMaxSteps && s <= hs.step; s++) {
    found->trace_q[s] = hs.qs[s];
    found->trace_score[s] = hs.scores[s];
    found->nsteps = s + 1;
  }
  rcg_coef_layout lay;
  layout_of(run.w, run.h, run.channels, hs.best_q, run.subsampling, &lay);
  const int16_t* best = run.slots + (size_t)hs.best_step * run.es.max_coefs;
  if (d_coefs_out || h_coefs_out) {
    if ((long long)coefs_len < lay.ncoefs) return fail(ctx, RCG_INVALID, "coefficient buffer too short");
    if (d_coefs_out) {
      cudaMemcpyAsync(d_coefs_out, best, (size_t)lay.ncoefs * 2, cudaMemcpyDeviceToDevice, ctx->stream);
    } else if ((rc = copy_to_host(ctx, h_coefs_out, best, (size_t)lay.ncoefs * 2)) != RCG_OK) {
      return rc;
    }
  }
  uint8_t qt[128];
  qtables_for(hs.best_q, qt);
  if (h_qt_out) std::memcpy(h_qt_out, qt, 128);
  if (d_qt_out) cudaMemcpyAsync(d_qt_out, qt, 128, cudaMemcpyHostToDevice, ctx->stream);
  return finish(ctx, "search output");
}

// d_weights (nullable): the perceptual trellis's weights in the coefficient layout of the (quality-independent)
// subsampling; every candidate's trellis then runs in the weighted mode.
static int search_impl(rcg_ctx* ctx, const uint8_t* d_src, int w, int h, int channels, int metric, double target,
                       int max_q, int subsampling, int trellis_on, rcg_found* found, int16_t* d_coefs_out,
                       size_t coefs_len, uint8_t* d_qt_out, int16_t* h_coefs_out, uint8_t* h_qt_out,
                       const float* d_weights = nullptr, int step_limit = 0) {
  SearchRun run;
  int rc = search_prepare(ctx, d_src, w, h, channels, metric, target, max_q, subsampling, trellis_on, &run);
  if (rc != RCG_OK) return rc;
  const EncoderSetup& es = run.es;
  const SearchScorer& sc = run.sc;
  SearchState* d_ss = run.d_ss;
  StepDesc* d_st = run.d_st;
  // Every launch below takes pointers into this context's workspace and sizes that follow from the key.
  // step_limit > 0: only the first steps of the bisection (a probe); the result is the best candidate so far.
  const int nsteps = step_limit > 0 ? std::min(step_limit, run.max_steps) : run.max_steps;
  const std::vector<long long> key = {1, (long long)(uintptr_t)d_src, w, h, channels, metric, subsampling, trellis_on,
                                      nsteps, (long long)(uintptr_t)d_weights};
  auto issue_step = [&](int s) {
    step_tables(ctx, d_ss, d_st, w, h, run.slots, es.max_coefs, d_weights);
    quantize(ctx, d_st, es.caches, es.max_blocks);
    rate_tables(ctx, d_st);
    trellis(ctx, d_st, es.caches, es.max_blocks, d_weights != nullptr);
    dequant_idct(ctx, d_st, nullptr, run.planes, es.max_blocks);
    score_candidate(ctx, sc, d_st, run.planes, w, h, channels, d_ss, s);
  };
  rc = run_step_loop(ctx, key, [&]() {
    for (int s = 0; s < nsteps; s++) issue_step(s);
  });
  if (rc != RCG_OK) return rc;
  SearchState hs;
  cudaMemcpyAsync(&hs, d_ss, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream);
  if ((rc = finish(ctx, "search")) != RCG_OK) return rc;
  if ((rc = settle_ties(ctx, sc, d_ss, &hs, nsteps, w, h, issue_step)) != RCG_OK) return rc;
  if (nsteps < run.max_steps && !hs.done) {
    // A probe: the evaluated candidates only (not the next one the bisection has chosen), and as its result the
    // candidate whose score is closest to the target, from either side.
    SearchState pr = hs;
    pr.step = hs.step - 1;
    int pick = 0;
    for (int s = 1; s <= pr.step; s++)
      if (std::fabs(hs.scores[s] - target) < std::fabs(hs.scores[pick] - target)) pick = s;
    pr.best_step = pick;
    pr.best_q = hs.qs[pick];
    pr.best_score = hs.scores[pick];
    return search_collect(ctx, run, pr, found, d_coefs_out, coefs_len, d_qt_out, h_coefs_out, h_qt_out, true);
  }
  return search_collect(ctx, run, hs, found, d_coefs_out, coefs_len, d_qt_out, h_coefs_out, h_qt_out);
}

// The goal checks of find_jpeg_quality (cli/src/pipeline.rs:211-218).
static int check_goal(rcg_ctx* ctx, int metric, uint32_t width, uint32_t height, double target) {
  if (metric != RCG_METRIC_SSIMULACRA2 && metric != RCG_METRIC_SSIM)
    return fail(ctx, RCG_INVALID, "the JPEG search goal is SSIMULACRA2 or SSIM");
  if (metric == RCG_METRIC_SSIMULACRA2 && (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide))
    return fail(ctx, RCG_UNSUPPORTED, "--target-ssimulacra2 needs an image of at least 8x8 pixels");
  if (!(target == target)) return fail(ctx, RCG_INVALID, "target is NaN");
  return RCG_OK;
}

int rcg_search_metric(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels, int metric,
                      double target, int max_quality, const rcg_encode_options* opts, rcg_found* found,
                      int16_t* coefs, size_t coefs_len, uint8_t* qtables) {
  if (!ctx) return RCG_INVALID;
  int rc;
  if ((rc = check_image(ctx, width, height, channels)) != RCG_OK) return rc;
  if ((rc = check_opts(ctx, opts, false)) != RCG_OK) return rc;
  if (!src || !found) return fail(ctx, RCG_INVALID, "null pointer");
  if ((rc = check_goal(ctx, metric, width, height, target)) != RCG_OK) return rc;
  int max_q = std::max(1, std::min(max_quality, 100));
  cudaSetDevice(ctx->device);
  size_t bytes = (size_t)width * height * channels;
  uint8_t* d_src = (uint8_t*)workspace(ctx, "img_src", bytes);
  if (!d_src) return RCG_NO_MEMORY;
  if ((rc = copy_to_device(ctx, d_src, src, bytes)) != RCG_OK) return rc;
  return search_impl(ctx, d_src, (int)width, (int)height, channels, metric, target, max_q, opts->subsampling,
                     opts->trellis, found, nullptr, coefs_len, nullptr, coefs, qtables);
}

int rcg_search(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels, double target,
               int max_quality, const rcg_encode_options* opts, rcg_found* found, int16_t* coefs, size_t coefs_len,
               uint8_t* qtables) {
  return rcg_search_metric(ctx, src, width, height, channels, RCG_METRIC_SSIMULACRA2, target, max_quality, opts,
                           found, coefs, coefs_len, qtables);
}

int rcg_search_device(rcg_ctx* ctx, const uint8_t* d_src, uint32_t width, uint32_t height, int channels,
                      double target, int max_quality, const rcg_encode_options* opts, rcg_found* found,
                      int16_t* d_coefs, size_t coefs_len, uint8_t* d_qtables) {
  if (!ctx) return RCG_INVALID;
  int rc;
  if ((rc = check_image(ctx, width, height, channels)) != RCG_OK) return rc;
  if ((rc = check_opts(ctx, opts, false)) != RCG_OK) return rc;
  if (!d_src || !found) return fail(ctx, RCG_INVALID, "null pointer");
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
    return fail(ctx, RCG_UNSUPPORTED, "--target-ssimulacra2 needs an image of at least 8x8 pixels");
  if (!(target == target)) return fail(ctx, RCG_INVALID, "target is NaN");
  int max_q = std::max(1, std::min(max_quality, 100));
  cudaSetDevice(ctx->device);
  return search_impl(ctx, d_src, (int)width, (int)height, channels, RCG_METRIC_SSIMULACRA2, target, max_q,
                     opts->subsampling, opts->trellis, found, d_coefs, coefs_len, d_qtables, nullptr, nullptr);
}

int rcg_search_batch(rcg_ctx* ctx, int n, const uint8_t* const* srcs, const uint32_t* widths,
                     const uint32_t* heights, const int* channels, const double* targets, int max_quality,
                     const rcg_encode_options* opts, int parallel, rcg_found* found, int16_t* const* coefs,
                     const size_t* coefs_len, uint8_t* const* qtables) {
  if (!ctx) return RCG_INVALID;
  if (n < 0 || (n > 0 && (!srcs || !widths || !heights || !channels || !targets || !found)))
    return fail(ctx, RCG_INVALID, "null pointer");
  if (n == 0) return RCG_OK;
  int rc = check_opts(ctx, opts, false);
  if (rc != RCG_OK) return rc;
  const int p = std::max(1, std::min(parallel > 0 ? parallel : 4, n));
  while ((int)ctx->workers.size() < p) {
    rcg_ctx* wk = nullptr;
    int crc = rcg_ctx_create(ctx->device, &wk);
    if (crc != RCG_OK) return fail(ctx, crc, "cannot create a batch worker context");
    wk->stage_copies = true;  // several threads copy at once: keep them off the driver's shared pageable path
    ctx->workers.push_back(wk);
  }
  // Largest images first, handed out one at a time: the workers finish at about the same time.
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (uint64_t)widths[a] * heights[a] > (uint64_t)widths[b] * heights[b];
  });
  // The workers decide near ties like the caller's context, and their rescores count toward it.
  std::vector<uint64_t> ties0;
  for (int t = 0; t < p; t++) {
    ctx->workers[t]->tie_band = ctx->tie_band;
    ties0.push_back(ctx->workers[t]->tie_rescores);
  }
  std::atomic<int> next(0);
  std::vector<int> status(n, RCG_OK);
  std::vector<std::string> messages(n);
  auto work = [&](rcg_ctx* wk) {
    cudaSetDevice(wk->device);
    for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
      const int i = order[k];
      int r = rcg_search(wk, srcs[i], widths[i], heights[i], channels[i], targets[i], max_quality, opts, &found[i],
                         coefs ? coefs[i] : nullptr, coefs_len ? coefs_len[i] : 0, qtables ? qtables[i] : nullptr);
      status[i] = r;
      if (r != RCG_OK) messages[i] = wk->last_error;
    }
  };
  std::vector<std::thread> threads;
  for (int t = 1; t < p; t++) threads.emplace_back(work, ctx->workers[t]);
  work(ctx->workers[0]);
  for (auto& th : threads) th.join();
  for (int t = 0; t < p; t++) ctx->tie_rescores += ctx->workers[t]->tie_rescores - ties0[t];
  for (int i = 0; i < n; i++)
    if (status[i] != RCG_OK) return fail(ctx, status[i], "image " + std::to_string(i) + ": " + messages[i]);
  ctx->last_error.clear();
  return RCG_OK;
}

constexpr int kLockThreads = 8;  // host threads of a lockstep batch's per-image set-up and collection

int rcg_search_batch_lockstep(rcg_ctx* ctx, int n, const uint8_t* const* srcs, const uint32_t* widths,
                              const uint32_t* heights, const int* channels, const double* targets, int max_quality,
                              const rcg_encode_options* opts, rcg_found* found, int16_t* const* coefs,
                              const size_t* coefs_len, uint8_t* const* qtables) {
  if (!ctx) return RCG_INVALID;
  if (n < 0 || (n > 0 && (!srcs || !widths || !heights || !channels || !targets || !found)))
    return fail(ctx, RCG_INVALID, "null pointer");
  if (n == 0) return RCG_OK;
  int rc = check_opts(ctx, opts, false);
  if (rc != RCG_OK) return rc;
  for (int i = 0; i < n; i++) {
    if (!srcs[i]) return fail(ctx, RCG_INVALID, "image " + std::to_string(i) + ": null pointer");
    if ((rc = check_image(ctx, widths[i], heights[i], channels[i])) != RCG_OK ||
        (rc = check_goal(ctx, RCG_METRIC_SSIMULACRA2, widths[i], heights[i], targets[i])) != RCG_OK)
      return fail(ctx, rc, "image " + std::to_string(i) + ": " + ctx->last_error);
  }
  const int max_q = std::max(1, std::min(max_quality, 100));
  cudaSetDevice(ctx->device);
  while ((int)ctx->lock_subs.size() < n) {
    rcg_ctx* sub = nullptr;
    int crc = rcg_ctx_create(ctx->device, &sub);
    if (crc != RCG_OK) return fail(ctx, crc, "cannot create a batch image context");
    sub->stage_copies = true;
    ctx->lock_subs.push_back(sub);
  }
  // Per image, on its own context's stream (the images' set-ups overlap one another): upload, colour planes, FDCTs,
  // the reference's pyramid, the initial bisection state. Host threads share the images, so the staging copies of
  // the uploads run in parallel. Then the caller's stream waits for all of them.
  std::vector<SearchRun> runs((size_t)n);
  std::vector<int> status((size_t)n, RCG_OK);
  const int nthreads = std::max(1, std::min(n, kLockThreads));
  auto for_images = [&](const std::function<void(int)>& fn) {
    std::atomic<int> next(0);
    auto work = [&]() {
      cudaSetDevice(ctx->device);
      for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) fn(i);
    };
    std::vector<std::thread> threads;
    for (int t = 1; t < nthreads; t++) threads.emplace_back(work);
    work();
    for (auto& th : threads) th.join();
  };
  for_images([&](int i) {
    rcg_ctx* sub = ctx->lock_subs[(size_t)i];
    sub->tie_band = ctx->tie_band;
    sub->band_chunks = ctx->band_chunks;
    sub->ref_cache = ctx->ref_cache;
    const size_t bytes = (size_t)widths[i] * heights[i] * channels[i];
    uint8_t* d_src = (uint8_t*)workspace(sub, "img_src", bytes);
    int r = d_src ? RCG_OK : RCG_NO_MEMORY;
    if (r == RCG_OK) r = copy_to_device(sub, d_src, srcs[i], bytes);
    if (r == RCG_OK)
      r = search_prepare(sub, d_src, (int)widths[i], (int)heights[i], channels[i], RCG_METRIC_SSIMULACRA2,
                         targets[i], max_q, opts->subsampling, opts->trellis, &runs[(size_t)i]);
    if (r == RCG_OK && !sub->switch_event &&
        cudaEventCreateWithFlags(&sub->switch_event, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      r = fail(sub, RCG_CUDA_ERROR, "batch event");
    }
    if (r == RCG_OK) cudaEventRecord(sub->switch_event, sub->stream);
    status[(size_t)i] = r;
  });
  for (int i = 0; i < n; i++) {
    if (status[(size_t)i] != RCG_OK)
      return fail(ctx, status[(size_t)i], "image " + std::to_string(i) + ": " + ctx->lock_subs[(size_t)i]->last_error);
    cudaStreamWaitEvent(ctx->stream, ctx->lock_subs[(size_t)i]->switch_event, 0);
  }
  // The work-lists: per image its StepDesc, search state, buffers and first CTA in each stage's grid.
  std::vector<LockItem> items((size_t)n);
  long long q_total = 0, u_total = 0, p_total = 0, t_total = 0;
  int max_scales = 1, max_steps = 1;
  for (int i = 0; i < n; i++) {
    const SearchRun& r = runs[(size_t)i];
    rcg_ctx* sub = ctx->lock_subs[(size_t)i];
    LockItem& it = items[(size_t)i];
    std::memset(&it, 0, sizeof it);
    it.ss = r.d_ss;
    it.st = r.d_st;
    for (int k = 0; k < 9; k++) it.caches[k] = r.es.caches[k];
    it.slots = r.slots;
    it.slot_stride = r.es.max_coefs;
    it.planes = r.planes;
    it.w = r.w;
    it.h = r.h;
    it.ref_pyr = r.sc.ref_pyr;
    it.refm = r.sc.ref_moments;
    it.dist_pyr = r.sc.dist_pyr;
    it.partials = (double*)sub->bufs["score_partials"].ptr;
    it.scale_sums = (double*)sub->bufs["score_scale_sums"].ptr;
    it.counter = (unsigned*)sub->bufs["score_counter"].ptr;
    it.score = r.sc.d_score;
    it.pd = plan_bands(ctx, r.sc.pd);
    it.q0 = q_total;
    q_total += (r.es.max_blocks + 127) / 128;
    it.ux = ((r.w + 3) / 4 + 127) / 128;
    it.uy = std::min(((r.h + 1) / 2 + 3) / 4, 65535);  // four chroma rows per CTA, as upsample_color
    it.u0 = u_total;
    u_total += (long long)it.ux * it.uy;
    it.p0 = p_total;
    p_total += pyramid_ctas(it.pd);
    it.t0 = t_total;
    t_total += it.pd.total_tiles;
    max_scales = std::max(max_scales, it.pd.nscales);
    max_steps = std::max(max_steps, r.max_steps);
  }
  if (q_total > INT32_MAX || u_total > INT32_MAX || p_total > INT32_MAX || t_total > INT32_MAX)
    return fail(ctx, RCG_INVALID, "batch too large for one launch");
  LockItem* d_items = (LockItem*)workspace(ctx, "lock_items", sizeof(LockItem) * (size_t)n);
  double* d_exact = (double*)workspace(ctx, "x_score", sizeof(double), false);
  if (!d_items || !d_exact) return RCG_NO_MEMORY;
  cudaMemcpyAsync(d_items, items.data(), sizeof(LockItem) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
  auto issue_step = [&](int s) {
    lock_step_codec(ctx, d_items, n, q_total, u_total);
    lock_step_score(ctx, d_items, n, p_total, t_total, max_scales,
                    ctx->ref_cache ? (s == 0 ? kRefWrite : kRefRead) : kRefNone);
  };
  // The grids follow from the totals; the images' buffers come in through the work-list uploaded above.
  const std::vector<long long> key = {5, n, max_steps, q_total, u_total, p_total, t_total, max_scales};
  rc = run_step_loop(ctx, key, [&]() {
    for (int s = 0; s < max_steps; s++) issue_step(s);
  });
  if (rc != RCG_OK) return rc;
  std::vector<SearchState> hs((size_t)n);
  auto read_states = [&]() -> int {
    for (int i = 0; i < n; i++)
      cudaMemcpyAsync(&hs[(size_t)i], runs[(size_t)i].d_ss, sizeof(SearchState), cudaMemcpyDeviceToHost, ctx->stream);
    return finish(ctx, "lockstep batch");
  };
  if ((rc = read_states()) != RCG_OK) return rc;
  // Near ties (settle_ties): every paused image's candidate is rescored in the reference's arithmetic and resumed,
  // then the remaining steps run for all images (the finished ones skip).
  for (;;) {
    int from = max_steps;
    for (int i = 0; i < n; i++) {
      if (hs[(size_t)i].done != 2) continue;
      const SearchRun& r = runs[(size_t)i];
      if ((rc = exact_score(ctx, r.sc.ref_pyr, r.sc.dist_pyr, r.w, r.h, d_exact)) != RCG_OK) return rc;
      search_resume(ctx, r.d_ss, d_exact);
      ctx->tie_rescores++;
      from = std::min(from, hs[(size_t)i].step + 1);
    }
    if (from == max_steps) break;
    for (int s = from; s < max_steps; s++) issue_step(s);
    if ((rc = read_states()) != RCG_OK) return rc;
  }
  // Results, each through its image's context (the step loop is complete: the states were read after it), in
  // parallel like the set-up.
  for_images([&](int i) {
    rcg_ctx* sub = ctx->lock_subs[(size_t)i];
    status[(size_t)i] = search_collect(sub, runs[(size_t)i], hs[(size_t)i], &found[i], nullptr,
                                       coefs_len ? coefs_len[i] : 0, nullptr, coefs ? coefs[i] : nullptr,
                                       qtables ? qtables[i] : nullptr);
  });
  for (int i = 0; i < n; i++)
    if (status[(size_t)i] != RCG_OK)
      return fail(ctx, status[(size_t)i], "image " + std::to_string(i) + ": " + ctx->lock_subs[(size_t)i]->last_error);
  ctx->last_error.clear();
  return RCG_OK;
}

int rcg_requantize(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                   const rcg_qtables* in, const int16_t* coefs_in, int quality, int trellis, int16_t* coefs_out,
                   size_t coefs_len, rcg_qtables* out) {
  if (!ctx) return RCG_INVALID;
  if (!layout || !coefs_in || !coefs_out) return fail(ctx, RCG_INVALID, "null pointer");
  if (width == 0 || height == 0) return fail(ctx, RCG_INVALID, "empty image");
  if (layout->ncomp != 1 && layout->ncomp != 3)
    return fail(ctx, RCG_UNSUPPORTED, "requantization takes 1 or 3 components");
  if (quality < 1 || quality > 100) return fail(ctx, RCG_INVALID, "quality must be 1..=100");
  StepDesc* st = new StepDesc;
  int rc = layout_step(ctx, st, (int)width, (int)height, layout);
  if (rc == RCG_OK) rc = requant_inputs(ctx, in, st);
  if (rc == RCG_OK && (long long)coefs_len < st->nblocks * 64) rc = fail(ctx, RCG_INVALID, "coefficient buffer too short");
  if (rc != RCG_OK) {
    delete st;
    return rc;
  }
  cudaSetDevice(ctx->device);
  const size_t cbytes = (size_t)st->nblocks * 64 * 2;
  int16_t* d_src = (int16_t*)workspace(ctx, "rq_src", cbytes);
  int16_t* d_out = (int16_t*)workspace(ctx, "coefs_single", cbytes);
  StepDesc* d_st = (StepDesc*)workspace(ctx, "step_single", sizeof(StepDesc));
  if (!d_src || !d_out || !d_st) {
    delete st;
    return RCG_NO_MEMORY;
  }
  int tq[3];
  uint8_t slot_qt[4][64];
  int present[4];
  host_requant_tables(st, quality, trellis, tq, slot_qt, present);
  st->coef_src = d_src;
  st->coefs = d_out;
  copy_to_device(ctx, d_src, coefs_in, cbytes);
  cudaMemcpyAsync(d_st, st, sizeof(StepDesc), cudaMemcpyHostToDevice, ctx->stream);
  const float* no_caches[9] = {nullptr};
  requantize_plain(ctx, d_st, st->nblocks);
  rate_tables(ctx, d_st);
  rcg::trellis(ctx, d_st, no_caches, st->nblocks);
  rc = copy_to_host(ctx, coefs_out, d_out, cbytes);
  cudaStreamSynchronize(ctx->stream);
  qtables_out(tq, slot_qt, present, st->ncomp, out);
  delete st;
  if (rc != RCG_OK) return rc;
  return finish(ctx, "requantize");
}

static int search_requantize_impl(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                                  const rcg_qtables* in, const int16_t* coefs_in, int metric, double target,
                                  int max_quality, int trellis, rcg_found* found, int16_t* coefs_out,
                                  size_t coefs_len, rcg_qtables* out, bool on_device) {
  if (!ctx) return RCG_INVALID;
  if (!layout || !coefs_in || !found) return fail(ctx, RCG_INVALID, "null pointer");
  if (on_device && ((reinterpret_cast<uintptr_t>(coefs_in) | reinterpret_cast<uintptr_t>(coefs_out)) & 15))
    return fail(ctx, RCG_INVALID, "device coefficients must be 16-byte aligned");
  if (width == 0 || height == 0 || width > 65535 || height > 65535)
    return fail(ctx, RCG_INVALID, "JPEG dimensions must be 1..=65535");
  int grc = check_goal(ctx, metric, width, height, target);
  if (grc != RCG_OK) return grc;
  if (layout->ncomp != 1 && layout->ncomp != 3)
    return fail(ctx, RCG_UNSUPPORTED, "requantization takes 1 or 3 components");
  const int w = (int)width, h = (int)height;
  const int max_q = std::max(1, std::min(max_quality, 100));
  StepDesc* st = new StepDesc;
  int rc = layout_step(ctx, st, w, h, layout);
  if (rc == RCG_OK) rc = requant_inputs(ctx, in, st);
  if (rc != RCG_OK) {
    delete st;
    return rc;
  }
  cudaSetDevice(ctx->device);
  const long long nblocks = st->nblocks;
  const size_t cbytes = (size_t)nblocks * 64 * 2;
  int max_steps = 1;
  for (int span = max_q; span > 1; span = (span + 1) / 2) max_steps++;
  max_steps = std::min(max_steps, kMaxSteps);
  const int channels = st->ncomp;
  SearchScorer sc;
  int16_t* d_src = on_device ? const_cast<int16_t*>(coefs_in) : (int16_t*)workspace(ctx, "rq_src", cbytes);
  int16_t* slots = (int16_t*)workspace(ctx, "coef_slots", cbytes * max_steps);
  uint8_t* planes = (uint8_t*)workspace(ctx, "dec_planes", (size_t)plane_bytes(st));
  uint8_t* ref_px = metric == RCG_METRIC_SSIM ? (uint8_t*)workspace(ctx, "ref_px", (size_t)w * h * channels) : nullptr;
  SearchState* d_ss = (SearchState*)workspace(ctx, "search_state", sizeof(SearchState));
  StepDesc* d_st = (StepDesc*)workspace(ctx, "step_search", sizeof(StepDesc));
  if (!d_src || !slots || !planes || !d_ss || !d_st || (metric == RCG_METRIC_SSIM && !ref_px) ||
      scorer_setup(ctx, metric, w, h, channels, &sc) != RCG_OK) {
    delete st;
    return RCG_NO_MEMORY;
  }
  sc.ref_px = ref_px;
  if (!on_device && (rc = copy_to_device(ctx, d_src, coefs_in, cbytes)) != RCG_OK) {
    delete st;
    return rc;
  }
  // The reference image: the source reconstructed with its own tables (cli/src/pipeline.rs:372).
  for (int c = 0; c < st->ncomp; c++)
    for (int n = 0; n < 64; n++) st->mult[c][n] = mult_entry_host(st->src_qt[c], n);
  st->coef_src = d_src;
  st->coefs = d_src;
  st->requant = 1;
  cudaMemcpyAsync(d_st, st, sizeof(StepDesc), cudaMemcpyHostToDevice, ctx->stream);
  dequant_idct(ctx, d_st, d_src, planes, nblocks);
  // A requantized candidate keeps the source's block layout.
  sc.fuse420 = metric == RCG_METRIC_SSIMULACRA2 && layout_fast420(st, w);
  if (metric == RCG_METRIC_SSIM) {
    upsample_color(ctx, d_st, planes, w, h, ref_px, nullptr);
  } else if (sc.fuse420) {
    upsample_pyramid(ctx, d_st, planes, w, h, sc.pd, sc.ref_pyr);
  } else {
    upsample_color(ctx, d_st, planes, w, h, nullptr, sc.ref_pyr);
    build_pyramid(ctx, sc.pd, sc.ref_pyr);
  }
  SearchState hs;
  std::memset(&hs, 0, sizeof hs);
  hs.lo = 1;
  hs.hi = max_q;
  hs.qs[0] = max_q;
  hs.target = target;
  hs.max_q = max_q;
  hs.trellis = trellis;
  hs.channels = channels;
  hs.best_q = max_q;
  hs.tie_band = metric == RCG_METRIC_SSIMULACRA2 ? ctx->tie_band : 0.0;
  cudaMemcpyAsync(d_ss, &hs, sizeof hs, cudaMemcpyHostToDevice, ctx->stream);
  const float* no_caches[9] = {nullptr};
  std::vector<long long> key = {2, (long long)(uintptr_t)d_src, w, h, st->ncomp, metric, trellis, max_steps,
                                st->hmax, st->vmax, nblocks};
  for (int c = 0; c < st->ncomp; c++) {
    const CompDesc& cd = st->comp[c];
    key.insert(key.end(), {cd.bw, cd.bh, cd.h, cd.v, cd.blk0, cd.plane_off});
  }
  auto issue_step = [&](int s) {
    step_tables_requant(ctx, d_ss, d_st, slots, nblocks * 64);
    requantize_plain(ctx, d_st, nblocks);
    rate_tables(ctx, d_st);
    rcg::trellis(ctx, d_st, no_caches, nblocks);
    dequant_idct(ctx, d_st, nullptr, planes, nblocks);
    score_candidate(ctx, sc, d_st, planes, w, h, channels, d_ss, s);
  };
  rc = run_step_loop(ctx, key, [&]() {
    for (int s = 0; s < max_steps; s++) issue_step(s);
  });
  if (rc != RCG_OK) {
    delete st;
    return rc;
  }
  cudaMemcpyAsync(&hs, d_ss, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream);
  if ((rc = finish(ctx, "search_requantize")) != RCG_OK ||
      (rc = settle_ties(ctx, sc, d_ss, &hs, max_steps, w, h, issue_step)) != RCG_OK) {
    delete st;
    return rc;
  }
  if (!hs.done) {
    delete st;
    return fail(ctx, RCG_TIMEOUT, "bisection did not finish within the step budget");
  }
  found->quality = hs.best_q;
  found->score = hs.best_score;
  found->nsteps = 0;
  for (int s = 0; s < kMaxSteps && s <= hs.step; s++) {
    found->trace_q[s] = hs.qs[s];
    found->trace_score[s] = hs.scores[s];
    found->nsteps = s + 1;
  }
  if (coefs_out) {
    if (coefs_len < (size_t)nblocks * 64) {
      delete st;
      return fail(ctx, RCG_INVALID, "coefficient buffer too short");
    }
    const int16_t* best = slots + (size_t)hs.best_step * nblocks * 64;
    if (on_device) {
      cudaMemcpyAsync(coefs_out, best, cbytes, cudaMemcpyDeviceToDevice, ctx->stream);
    } else if ((rc = copy_to_host(ctx, coefs_out, best, cbytes)) != RCG_OK) {
      delete st;
      return rc;
    }
  }
  int tq[3];
  uint8_t slot_qt[4][64];
  int present[4];
  host_requant_tables(st, hs.best_q, trellis, tq, slot_qt, present);
  qtables_out(tq, slot_qt, present, st->ncomp, out);
  delete st;
  return finish(ctx, "search_requantize output");
}

int rcg_search_requantize(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                          const rcg_qtables* in, const int16_t* coefs_in, int metric, double target, int max_quality,
                          int trellis, rcg_found* found, int16_t* coefs_out, size_t coefs_len, rcg_qtables* out) {
  return search_requantize_impl(ctx, width, height, layout, in, coefs_in, metric, target, max_quality, trellis, found,
                                coefs_out, coefs_len, out, false);
}

int rcg_search_requantize_device(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                                 const rcg_qtables* in, const int16_t* d_coefs_in, int metric, double target,
                                 int max_quality, int trellis, rcg_found* found, int16_t* d_coefs_out,
                                 size_t coefs_len, rcg_qtables* out) {
  return search_requantize_impl(ctx, width, height, layout, in, d_coefs_in, metric, target, max_quality, trellis,
                                found, d_coefs_out, coefs_len, out, true);
}

static int plan_common(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                       const int16_t* coefs, size_t coefs_len, bool on_device, rcg_plan_result* result) {
  if (!ctx) return RCG_INVALID;
  if (!layout || !coefs || !result) return fail(ctx, RCG_INVALID, "null pointer");
  if (width == 0 || height == 0 || width > 65535 || height > 65535)
    return fail(ctx, RCG_INVALID, "JPEG dimensions must be 1..=65535");
  if (layout->ncomp != 1 && layout->ncomp != 3)
    return fail(ctx, RCG_UNSUPPORTED, "scan planning takes 1 or 3 components");
  StepDesc* st = new StepDesc;
  int rc = layout_step(ctx, st, (int)width, (int)height, layout);
  if (rc == RCG_OK && !on_device && coefs_len < (size_t)st->nblocks * 64)
    rc = fail(ctx, RCG_INVALID, "coefficient buffer too short");
  if (rc != RCG_OK) {
    delete st;
    return rc;
  }
  cudaSetDevice(ctx->device);
  const int16_t* d = coefs;
  if (!on_device) {
    int16_t* buf = (int16_t*)workspace(ctx, "plan_coefs", (size_t)st->nblocks * 128);
    if (!buf) {
      delete st;
      return RCG_NO_MEMORY;
    }
    if ((rc = copy_to_device(ctx, buf, coefs, (size_t)st->nblocks * 128)) != RCG_OK) {
      delete st;
      return rc;
    }
    d = buf;
  }
  rc = plan_scans(ctx, st, (int)width, (int)height, d, result);
  delete st;
  if (rc != RCG_OK) return rc;
  return finish(ctx, "plan");
}

int rcg_plan(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout, const int16_t* coefs,
             size_t coefs_len, rcg_plan_result* result) {
  return plan_common(ctx, width, height, layout, coefs, coefs_len, false, result);
}

int rcg_plan_device(rcg_ctx* ctx, uint32_t width, uint32_t height, const rcg_coef_layout* layout,
                    const int16_t* d_coefs, rcg_plan_result* result) {
  return plan_common(ctx, width, height, layout, d_coefs, 0, true, result);
}

int rcg_decode_coefs(rcg_ctx* ctx, const uint8_t* jpeg, size_t len, rcg_jpeg_info* info, rcg_coef_layout* layout,
                     rcg_qtables* tables, int16_t* coefs, size_t coefs_len) {
  if (!ctx) return RCG_INVALID;
  if (!jpeg || !layout) return fail(ctx, RCG_INVALID, "null pointer");
  int rc = jpeg_decode(ctx, jpeg, len, info, layout, tables, coefs, coefs_len, false);
  if (rc != RCG_OK) return rc;
  return coefs ? finish(ctx, "decode") : RCG_OK;
}

int rcg_decode_coefs_device(rcg_ctx* ctx, const uint8_t* jpeg, size_t len, rcg_jpeg_info* info,
                            rcg_coef_layout* layout, rcg_qtables* tables, int16_t* d_coefs, size_t coefs_len) {
  if (!ctx) return RCG_INVALID;
  if (!jpeg || !layout) return fail(ctx, RCG_INVALID, "null pointer");
  int rc = jpeg_decode(ctx, jpeg, len, info, layout, tables, d_coefs, coefs_len, true);
  if (rc != RCG_OK) return rc;
  return d_coefs ? finish(ctx, "decode") : RCG_OK;
}

int rcg_ssimulacra2_grad_device(rcg_ctx* ctx, const uint8_t* d_reference, const float* d_distorted, uint32_t width,
                                uint32_t height, double* score, double* d_grad) {
  if (!ctx) return RCG_INVALID;
  if (!d_reference || !d_distorted || !score) return fail(ctx, RCG_INVALID, "null pointer");
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
    return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
  cudaSetDevice(ctx->device);
  int rc = ssim2_grad_device(ctx, d_reference, d_distorted, (int)width, (int)height, score, d_grad);
  if (rc != RCG_OK) return rc;
  return finish(ctx, "ssimulacra2 gradient");
}

int rcg_ssimulacra2_grad(rcg_ctx* ctx, const uint8_t* reference, const float* distorted, uint32_t width,
                         uint32_t height, double* score, double* grad) {
  if (!ctx) return RCG_INVALID;
  if (!reference || !distorted || !score) return fail(ctx, RCG_INVALID, "null pointer");
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
    return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
  cudaSetDevice(ctx->device);
  const size_t n = (size_t)width * height * 3;
  uint8_t* d_ref = (uint8_t*)workspace(ctx, "img_a", n);
  float* d_dist = (float*)workspace(ctx, "grad_dist", n * sizeof(float));
  double* d_grad = (double*)workspace(ctx, "grad_out", n * sizeof(double));
  if (!d_ref || !d_dist || !d_grad) return RCG_NO_MEMORY;
  int rc;
  if ((rc = copy_to_device(ctx, d_ref, reference, n)) != RCG_OK) return rc;
  if ((rc = copy_to_device(ctx, d_dist, distorted, n * sizeof(float))) != RCG_OK) return rc;
  if ((rc = ssim2_grad_device(ctx, d_ref, d_dist, (int)width, (int)height, score, grad ? d_grad : nullptr)) !=
      RCG_OK)
    return rc;
  if (grad && (rc = copy_to_host(ctx, grad, d_grad, n * sizeof(double))) != RCG_OK) return rc;
  return finish(ctx, "ssimulacra2 gradient");
}

// ---- perceptual trellis

void rcg_perceptual_defaults(rcg_perceptual_options* o) {
  if (!o) return;
  o->strength = 0.35;
  o->gamma = 0.5;
  o->w_min = 0.25;
  o->w_max = 4.0;
  o->radius = 1;
  o->keep_smaller = 1;
  o->gradient_fp64 = 0;
  o->strength_by_quality = 1;
}

double rcg_perceptual_strength(const rcg_perceptual_options* o, int quality) {
  if (!o) return 0.0;
  if (!o->strength_by_quality) return o->strength;
  return quality < 70 ? 0.35 : (quality < 85 ? 0.7 : 1.0);
}

static int check_popts(rcg_ctx* ctx, const rcg_perceptual_options* o, PerceptualParams* p) {
  if (!o) return fail(ctx, RCG_INVALID, "null perceptual options");
  const bool ok = std::isfinite(o->strength) && o->strength > 0.0 && std::isfinite(o->gamma) && o->gamma >= 0.0 &&
                  std::isfinite(o->w_max) && o->w_min > 0.0 && o->w_max >= o->w_min && o->radius >= 0 &&
                  o->radius <= 16;
  if (!ok) return fail(ctx, RCG_INVALID, "perceptual options out of range");
  *p = PerceptualParams{o->strength, o->gamma, o->w_min, o->w_max, o->radius, o->gradient_fp64 != 0};
  return RCG_OK;
}

// The SSIMULACRA2 gradient at the decoded image d_dec against d_ref (both 8-bit with `channels`), pulled back to the
// coefficient layout `lay`: coefficient gradient and/or weights (each nullable).
static int perceptual_impl(rcg_ctx* ctx, const uint8_t* d_ref, const uint8_t* d_dec, int w, int h, int channels,
                           const StepDesc* lay, const PerceptualParams& p, double* score, double* d_coef_grad,
                           float* d_weights) {
  const size_t npx = (size_t)w * h;
  float* d_dist = (float*)workspace(ctx, "perc_dist", npx * 3 * sizeof(float));
  double* d_grad = (double*)workspace(ctx, "perc_grad", npx * 3 * sizeof(double));
  if (!d_dist || !d_grad) return RCG_NO_MEMORY;
  const uint8_t* ref3 = d_ref;
  if (channels == 1) {
    uint8_t* r3 = (uint8_t*)workspace(ctx, "perc_ref3", npx * 3);
    if (!r3) return RCG_NO_MEMORY;
    expand_rgb(ctx, d_ref, 1, npx, r3, nullptr);
    ref3 = r3;
  }
  expand_rgb(ctx, d_dec, channels, npx, nullptr, d_dist);
  int rc = ssim2_grad_device(ctx, ref3, d_dist, w, h, score, d_grad, !p.gradient_fp64);
  if (rc != RCG_OK) return rc;
  return perceptual_pullback(ctx, d_grad, w, h, lay, p, d_coef_grad, d_weights);
}

// Shared checks and uploads of rcg_coef_gradient / rcg_perceptual_weights; `*st` owned by the caller on success.
static int pullback_inputs(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* decoded, uint32_t width,
                           uint32_t height, int channels, const rcg_coef_layout* layout, const void* out,
                           size_t out_len, StepDesc** st_out, const uint8_t** d_ref, const uint8_t** d_dec) {
  if (!reference || !decoded || !layout || !out) return fail(ctx, RCG_INVALID, "null pointer");
  int rc;
  if ((rc = check_image(ctx, width, height, channels)) != RCG_OK) return rc;
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide)
    return fail(ctx, RCG_UNSUPPORTED, "SSIMULACRA 2 needs at least 8x8 pixels");
  if (layout->ncomp != channels) return fail(ctx, RCG_INVALID, "layout.ncomp does not match the channel count");
  StepDesc* st = new StepDesc;
  if ((rc = layout_step(ctx, st, (int)width, (int)height, layout)) != RCG_OK) {
    delete st;
    return rc;
  }
  if ((long long)out_len < st->nblocks * 64) {
    delete st;
    return fail(ctx, RCG_INVALID, "output buffer too short");
  }
  cudaSetDevice(ctx->device);
  const size_t bytes = (size_t)width * height * channels;
  uint8_t* a = (uint8_t*)workspace(ctx, "img_a", bytes);
  uint8_t* b = (uint8_t*)workspace(ctx, "img_b", bytes);
  if (!a || !b) {
    delete st;
    return RCG_NO_MEMORY;
  }
  if ((rc = copy_to_device(ctx, a, reference, bytes)) == RCG_OK) rc = copy_to_device(ctx, b, decoded, bytes);
  if (rc != RCG_OK) {
    delete st;
    return rc;
  }
  *st_out = st;
  *d_ref = a;
  *d_dec = b;
  return RCG_OK;
}

int rcg_coef_gradient(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* decoded, uint32_t width, uint32_t height,
                      int channels, const rcg_coef_layout* layout, double* score, double* grad, size_t grad_len) {
  if (!ctx) return RCG_INVALID;
  if (!score) return fail(ctx, RCG_INVALID, "null pointer");
  StepDesc* st = nullptr;
  const uint8_t *d_ref = nullptr, *d_dec = nullptr;
  int rc = pullback_inputs(ctx, reference, decoded, width, height, channels, layout, grad, grad_len, &st, &d_ref,
                           &d_dec);
  if (rc != RCG_OK) return rc;
  const size_t n = (size_t)st->nblocks * 64;
  double* d_cg = (double*)workspace(ctx, "perc_coef_grad", n * sizeof(double));
  if (!d_cg) rc = RCG_NO_MEMORY;
  PerceptualParams p{1.0, 0.0, 1.0, 1.0, 0, true};  // the checked FP64 gradient
  if (rc == RCG_OK) rc = perceptual_impl(ctx, d_ref, d_dec, (int)width, (int)height, channels, st, p, score, d_cg,
                                         nullptr);
  delete st;
  if (rc == RCG_OK) rc = copy_to_host(ctx, grad, d_cg, n * sizeof(double));
  return rc == RCG_OK ? finish(ctx, "coefficient gradient") : rc;
}

int rcg_perceptual_weights(rcg_ctx* ctx, const uint8_t* reference, const uint8_t* decoded, uint32_t width,
                           uint32_t height, int channels, const rcg_coef_layout* layout,
                           const rcg_perceptual_options* popts, double* score, float* weights, size_t weights_len) {
  if (!ctx) return RCG_INVALID;
  if (!score) return fail(ctx, RCG_INVALID, "null pointer");
  PerceptualParams p;
  int rc = check_popts(ctx, popts, &p);
  if (rc != RCG_OK) return rc;
  StepDesc* st = nullptr;
  const uint8_t *d_ref = nullptr, *d_dec = nullptr;
  rc = pullback_inputs(ctx, reference, decoded, width, height, channels, layout, weights, weights_len, &st, &d_ref,
                       &d_dec);
  if (rc != RCG_OK) return rc;
  const size_t n = (size_t)st->nblocks * 64;
  float* d_w = (float*)workspace(ctx, "perc_weights", n * sizeof(float));
  if (!d_w) rc = RCG_NO_MEMORY;
  if (rc == RCG_OK) rc = perceptual_impl(ctx, d_ref, d_dec, (int)width, (int)height, channels, st, p, score, nullptr,
                                         d_w);
  delete st;
  if (rc == RCG_OK) rc = copy_to_host(ctx, weights, d_w, n * sizeof(float));
  return rc == RCG_OK ? finish(ctx, "perceptual weights") : rc;
}

// Checks of the weighted searches: SSIMULACRA2 goal, quality-independent layout, trellis on. `ncoefs` receives the
// layout's coefficient count.
static int weighted_search_checks(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                                  double target, const rcg_encode_options* opts, const rcg_found* found,
                                  long long* ncoefs) {
  int rc;
  if ((rc = check_image(ctx, width, height, channels)) != RCG_OK) return rc;
  if ((rc = check_opts(ctx, opts, false)) != RCG_OK) return rc;
  if (!src || !found) return fail(ctx, RCG_INVALID, "null pointer");
  if ((rc = check_goal(ctx, RCG_METRIC_SSIMULACRA2, width, height, target)) != RCG_OK) return rc;
  if (channels == 3 && opts->subsampling == RCG_SUB_AUTO)
    return fail(ctx, RCG_UNSUPPORTED, "the perceptual trellis needs an explicit subsampling");
  if (!opts->trellis) return fail(ctx, RCG_INVALID, "the perceptual mode weights the trellis: enable it");
  rcg_coef_layout lay;
  layout_of((int)width, (int)height, channels, 50, opts->subsampling, &lay);
  *ncoefs = lay.ncoefs;
  return RCG_OK;
}

int rcg_search_weighted(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                        double target, int max_quality, const rcg_encode_options* opts, const float* weights,
                        size_t weights_len, rcg_found* found, int16_t* coefs, size_t coefs_len, uint8_t* qtables) {
  if (!ctx) return RCG_INVALID;
  long long ncoefs = 0;
  int rc = weighted_search_checks(ctx, src, width, height, channels, target, opts, found, &ncoefs);
  if (rc != RCG_OK) return rc;
  if (!weights || (long long)weights_len != ncoefs)
    return fail(ctx, RCG_INVALID, "weights do not match the coefficient layout");
  const int max_q = std::max(1, std::min(max_quality, 100));
  cudaSetDevice(ctx->device);
  const size_t bytes = (size_t)width * height * channels;
  uint8_t* d_src = (uint8_t*)workspace(ctx, "img_src", bytes);
  float* d_w = (float*)workspace(ctx, "perc_weights", (size_t)ncoefs * sizeof(float));
  if (!d_src || !d_w) return RCG_NO_MEMORY;
  if ((rc = copy_to_device(ctx, d_src, src, bytes)) != RCG_OK) return rc;
  if ((rc = copy_to_device(ctx, d_w, weights, (size_t)ncoefs * sizeof(float))) != RCG_OK) return rc;
  return search_impl(ctx, d_src, (int)width, (int)height, channels, RCG_METRIC_SSIMULACRA2, target, max_q,
                     opts->subsampling, opts->trellis, found, nullptr, coefs_len, nullptr, coefs, qtables, d_w);
}

// write_best's size of a search result (the smaller of the planned progressive script and baseline).
static int planned_bytes(rcg_ctx* ctx, const StepDesc* lay, int w, int h, const int16_t* d_coefs, uint64_t* bytes) {
  rcg_plan_result r;
  int rc = plan_scans(ctx, lay, w, h, d_coefs, &r);
  if (rc != RCG_OK) return rc;
  *bytes = std::min(r.progressive_bytes, r.baseline_bytes);
  return RCG_OK;
}

// Candidates of the fast form's probe: the maximum quality and three bisection steps. Measured on the 64-image set
// (planned bytes of the weighted result against the plain search's): 3 -> -0.20%, 4 -> -0.74%, 5 -> -0.82%, the full
// plain search -1.32%.
constexpr int kPerceptualProbeSteps = 4;

int rcg_search_perceptual(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                          double target, int max_quality, const rcg_encode_options* opts,
                          const rcg_perceptual_options* popts, rcg_found* plain, rcg_found* found, uint64_t* sizes,
                          int* chose_perceptual, int16_t* coefs, size_t coefs_len, uint8_t* qtables, float* weights,
                          size_t weights_len) {
  if (!ctx) return RCG_INVALID;
  long long ncoefs = 0;
  int rc = weighted_search_checks(ctx, src, width, height, channels, target, opts, found, &ncoefs);
  if (rc != RCG_OK) return rc;
  PerceptualParams p;
  if ((rc = check_popts(ctx, popts, &p)) != RCG_OK) return rc;
  if (!plain) return fail(ctx, RCG_INVALID, "null pointer");
  if (weights && (long long)weights_len < ncoefs) return fail(ctx, RCG_INVALID, "weights buffer too short");
  if (coefs && (long long)coefs_len < ncoefs) return fail(ctx, RCG_INVALID, "coefficient buffer too short");
  const int w = (int)width, h = (int)height;
  const int max_q = std::max(1, std::min(max_quality, 100));
  cudaSetDevice(ctx->device);
  const size_t npx = (size_t)w * h;
  uint8_t* d_src = (uint8_t*)workspace(ctx, "img_src", npx * channels);
  int16_t* d_plain = (int16_t*)workspace(ctx, "perc_plain_coefs", (size_t)ncoefs * 2);
  int16_t* d_perc = (int16_t*)workspace(ctx, "perc_coefs", (size_t)ncoefs * 2);
  float* d_w = (float*)workspace(ctx, "perc_weights", (size_t)ncoefs * sizeof(float));
  uint8_t* d_dec = (uint8_t*)workspace(ctx, "perc_dec", npx * channels);
  StepDesc* d_st = (StepDesc*)workspace(ctx, "perc_step", sizeof(StepDesc));
  if (!d_src || !d_plain || !d_perc || !d_w || !d_dec || !d_st) return RCG_NO_MEMORY;
  if ((rc = copy_to_device(ctx, d_src, src, npx * channels)) != RCG_OK) return rc;
  // 1. the plain search
  rc = search_impl(ctx, d_src, w, h, channels, RCG_METRIC_SSIMULACRA2, target, max_q, opts->subsampling,
                   opts->trellis, plain, d_plain, (size_t)ncoefs, nullptr, nullptr, nullptr);
  if (rc != RCG_OK) return rc;
  // 2. its decoded image, and the weights from the gradient there
  p.strength = rcg_perceptual_strength(popts, plain->quality);
  StepDesc* st = new StepDesc;
  host_step_tables(st, plain->quality, opts->subsampling, channels, opts->trellis, w, h);
  uint8_t* planes = (uint8_t*)workspace(ctx, "perc_planes", (size_t)plane_bytes(st));
  if (!planes) {
    delete st;
    return RCG_NO_MEMORY;
  }
  cudaMemcpyAsync(d_st, st, sizeof(StepDesc), cudaMemcpyHostToDevice, ctx->stream);
  dequant_idct(ctx, d_st, d_plain, planes, st->nblocks);
  upsample_color(ctx, d_st, planes, w, h, d_dec, nullptr);
  double gscore = 0.0;
  rc = perceptual_impl(ctx, d_src, d_dec, w, h, channels, st, p, &gscore, nullptr, d_w);
  cudaStreamSynchronize(ctx->stream);  // the host StepDesc must outlive its upload
  // 3. the weighted search
  rcg_found perc;
  if (rc == RCG_OK)
    rc = search_impl(ctx, d_src, w, h, channels, RCG_METRIC_SSIMULACRA2, target, max_q, opts->subsampling,
                     opts->trellis, &perc, d_perc, (size_t)ncoefs, nullptr, nullptr, nullptr, d_w);
  // 4. sizes; keep the smaller
  uint64_t sz[2] = {0, 0};
  if (rc == RCG_OK) rc = planned_bytes(ctx, st, w, h, d_plain, &sz[0]);
  if (rc == RCG_OK) rc = planned_bytes(ctx, st, w, h, d_perc, &sz[1]);
  delete st;
  if (rc != RCG_OK) return rc;
  const bool use_perc = !popts->keep_smaller || sz[1] <= sz[0];
  *found = use_perc ? perc : *plain;
  if (sizes) {
    sizes[0] = sz[0];
    sizes[1] = sz[1];
  }
  if (chose_perceptual) *chose_perceptual = use_perc ? 1 : 0;
  if (coefs && (rc = copy_to_host(ctx, coefs, use_perc ? d_perc : d_plain, (size_t)ncoefs * 2)) != RCG_OK) return rc;
  if (qtables) qtables_for(found->quality, qtables);
  if (weights && (rc = copy_to_host(ctx, weights, d_w, (size_t)ncoefs * sizeof(float))) != RCG_OK) return rc;
  return finish(ctx, "perceptual search");
}

int rcg_search_perceptual_fast(rcg_ctx* ctx, const uint8_t* src, uint32_t width, uint32_t height, int channels,
                               double target, int max_quality, const rcg_encode_options* opts,
                               const rcg_perceptual_options* popts, rcg_found* probe, rcg_found* found,
                               int16_t* coefs, size_t coefs_len, uint8_t* qtables, float* weights,
                               size_t weights_len) {
  if (!ctx) return RCG_INVALID;
  long long ncoefs = 0;
  int rc = weighted_search_checks(ctx, src, width, height, channels, target, opts, found, &ncoefs);
  if (rc != RCG_OK) return rc;
  PerceptualParams p;
  if ((rc = check_popts(ctx, popts, &p)) != RCG_OK) return rc;
  if (weights && (long long)weights_len < ncoefs) return fail(ctx, RCG_INVALID, "weights buffer too short");
  if (coefs && (long long)coefs_len < ncoefs) return fail(ctx, RCG_INVALID, "coefficient buffer too short");
  const int w = (int)width, h = (int)height;
  const int max_q = std::max(1, std::min(max_quality, 100));
  cudaSetDevice(ctx->device);
  const size_t npx = (size_t)w * h;
  uint8_t* d_src = (uint8_t*)workspace(ctx, "img_src", npx * channels);
  int16_t* d_probe = (int16_t*)workspace(ctx, "perc_plain_coefs", (size_t)ncoefs * 2);
  int16_t* d_perc = (int16_t*)workspace(ctx, "perc_coefs", (size_t)ncoefs * 2);
  float* d_w = (float*)workspace(ctx, "perc_weights", (size_t)ncoefs * sizeof(float));
  uint8_t* d_dec = (uint8_t*)workspace(ctx, "perc_dec", npx * channels);
  StepDesc* d_st = (StepDesc*)workspace(ctx, "perc_step", sizeof(StepDesc));
  if (!d_src || !d_probe || !d_perc || !d_w || !d_dec || !d_st) return RCG_NO_MEMORY;
  if ((rc = copy_to_device(ctx, d_src, src, npx * channels)) != RCG_OK) return rc;
  // 1. the plain bisection's first kPerceptualProbeSteps candidates; the one scoring closest to the target stands in
  //    for the result (which lies within the 6 qualities the bisection has left after four steps from 1..100)
  rcg_found pr;
  rc = search_impl(ctx, d_src, w, h, channels, RCG_METRIC_SSIMULACRA2, target, max_q, opts->subsampling,
                   opts->trellis, &pr, d_probe, (size_t)ncoefs, nullptr, nullptr, nullptr, nullptr,
                   kPerceptualProbeSteps);
  if (rc != RCG_OK) return rc;
  if (probe) *probe = pr;
  // 2. the gradient at that candidate's decode, the weights with the strength its quality selects
  p.strength = rcg_perceptual_strength(popts, pr.quality);
  StepDesc* st = new StepDesc;
  host_step_tables(st, pr.quality, opts->subsampling, channels, opts->trellis, w, h);
  uint8_t* planes = (uint8_t*)workspace(ctx, "perc_planes", (size_t)plane_bytes(st));
  if (!planes) {
    delete st;
    return RCG_NO_MEMORY;
  }
  cudaMemcpyAsync(d_st, st, sizeof(StepDesc), cudaMemcpyHostToDevice, ctx->stream);
  dequant_idct(ctx, d_st, d_probe, planes, st->nblocks);
  upsample_color(ctx, d_st, planes, w, h, d_dec, nullptr);
  double gscore = 0.0;
  rc = perceptual_impl(ctx, d_src, d_dec, w, h, channels, st, p, &gscore, nullptr, d_w);
  cudaStreamSynchronize(ctx->stream);  // the host StepDesc must outlive its upload
  delete st;
  if (rc != RCG_OK) return rc;
  // 3. one weighted search
  rc = search_impl(ctx, d_src, w, h, channels, RCG_METRIC_SSIMULACRA2, target, max_q, opts->subsampling,
                   opts->trellis, found, d_perc, (size_t)ncoefs, nullptr, nullptr, nullptr, d_w);
  if (rc != RCG_OK) return rc;
  if (coefs && (rc = copy_to_host(ctx, coefs, d_perc, (size_t)ncoefs * 2)) != RCG_OK) return rc;
  if (qtables) qtables_for(found->quality, qtables);
  if (weights && (rc = copy_to_host(ctx, weights, d_w, (size_t)ncoefs * sizeof(float))) != RCG_OK) return rc;
  return finish(ctx, "fast perceptual search");
}

}  // extern "C"

