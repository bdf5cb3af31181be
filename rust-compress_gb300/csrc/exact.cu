// SSIMULACRA2 in the reference's own f64 arithmetic and order (core/src/ssimulacra2.rs:171-512), on the GPU.
//
// The fast scorer (ssim2.cu) computes in f32 and lands within about 1e-6 of the reference. A quality search decides
// on s >= target (jpeg/src/target.rs:48), so a candidate whose fast score falls that close to the target could be
// decided the other way from the reference. Such candidates are rescored here, with every operation the
// reference's, in f64, in its order:
//   * f32 linear planes (the caller's scale 0), then 2x2 means summed in f64 and rounded once to f32 (:223-247);
//   * XYB per pixel (:249-258), the cube root of the bias taken on the host with the platform libm, as the reference;
//   * the 11-tap blur of each row: interior samples as centre * s plus the symmetric tap pairs t = 1..5 in turn,
//     samples within 5 of the left/right edge (and every sample of a row of <= 10) tap by tap from zero (:273-319);
//   * the vertical blur with mirrored rows (:378-410), then the SSIM and edge maps (:411-431);
//   * per 96-row stripe (:33, :446-452) and channel, the six sums in row-major pixel order from zero (:432-441),
//     then the stripes added in stripe order (:453-456), the means and 4th roots (:457-465), the 108 weighted terms
//     and the final mapping (:491-511).
// This file is compiled with -fmad=false: no a * b + c is contracted into an FMA, as in the reference (Rust does not
// contract). What may still differ are the last bits of cbrt and pow (the reference calls the platform's libm, this
// file the CUDA math library), which moves a score by about 1e-15.
//
// GB300's FP64 rate is a small fraction of its FP32 rate and each stripe sum is one serial chain, so a 12 MP rescore
// takes tens of milliseconds; the searches call it only for near ties (capi.cu, settle_ties), and
// rcg_ssimulacra2_exact exposes it for callers that want the reference's score itself.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "rcg_internal.cuh"

namespace rcg {

__constant__ double c_xk[2 * kRadius + 1];  // the reference's f64 taps (:260-271)
__constant__ double c_xw[108];              // WEIGHTS (:54-163)
__constant__ double c_cbrt_bias;            // BIAS.cbrt() (:252-254)

constexpr int kStripe = 96;  // core/src/ssimulacra2.rs:33 (STRIPE)

// core/src/ssimulacra2.rs:42-52
constexpr double kXM02 = 0.078, kXM00 = 0.30, kXM01 = 1.0 - kXM02 - kXM00;
constexpr double kXM12 = 0.078, kXM10 = 0.23, kXM11 = 1.0 - kXM12 - kXM10;
constexpr double kXM20 = 0.243422689245478200, kXM21 = 0.204767444244968200, kXM22 = 1.0 - kXM20 - kXM21;
constexpr double kXBias = 0.0037930732552754493;
constexpr double kXC2 = 0.0009;

// downsample (:223-247): one output sample of channel blockIdx.y.
__global__ void __launch_bounds__(256) k_x_down(const float* __restrict__ src, int w, int h,
                                                float* __restrict__ dst, int ow, int oh) {
  const long long n = (long long)ow * oh;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = blockIdx.y;
  const int oy = (int)(i / ow), ox = (int)(i - (long long)oy * ow);
  const float* p = src + (size_t)c * w * h;
  const int y0 = oy * 2, y1 = min(oy * 2 + 2, h), x0 = ox * 2, x1 = min(ox * 2 + 2, w);
  double sum = 0.0;
  for (int y = y0; y < y1; y++)
    for (int x = x0; x < x1; x++) sum += (double)p[(size_t)y * w + x];
  dst[(size_t)c * n + i] = (float)(sum / (double)((y1 - y0) * (x1 - x0)));
}

// xyb (:249-258)
__device__ __forceinline__ void xyb_ref(double r, double g, double b, double out[3]) {
  const double cb = c_cbrt_bias;
  const double m0 = cbrt(fmax(kXM00 * r + kXM01 * g + kXM02 * b + kXBias, 0.0)) - cb;
  const double m1 = cbrt(fmax(kXM10 * r + kXM11 * g + kXM12 * b + kXBias, 0.0)) - cb;
  const double m2 = cbrt(fmax(kXM20 * r + kXM21 * g + kXM22 * b + kXBias, 0.0)) - cb;
  const double x = 0.5 * (m0 - m1);
  const double y = 0.5 * (m0 + m1);
  out[0] = x * 14.0 + 0.42;
  out[1] = y + 0.01;
  out[2] = (m2 - y) + 0.55;
}

// XYB of rows [lo, lo + rows) of both images (:353-367): planes [3][rows][w] each.
__global__ void __launch_bounds__(256) k_x_xyb(const float* __restrict__ a, const float* __restrict__ b, int w, int h,
                                               int lo, int rows, double* __restrict__ xa, double* __restrict__ xb) {
  const long long n = (long long)rows * w;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t np = (size_t)w * h, g = (size_t)lo * w + (size_t)i;
  double pa[3], pb[3];
  xyb_ref((double)a[g], (double)a[np + g], (double)a[2 * np + g], pa);
  xyb_ref((double)b[g], (double)b[np + g], (double)b[2 * np + g], pb);
#pragma unroll
  for (int c = 0; c < 3; c++) {
    xa[(size_t)c * n + i] = pa[c];
    xb[(size_t)c * n + i] = pb[c];
  }
}

// The five quantities of :373-383 at one sample: a, b, a*a, b*b, a*b.
__device__ __forceinline__ double quantity(int q, const double* ra, const double* rb, int x) {
  const double va = ra[x], vb = rb[x];
  switch (q) {
    case 0: return va;
    case 1: return vb;
    case 2: return va * va;
    case 3: return vb * vb;
    default: return va * vb;
  }
}

// blur_row (:273-319) of the five quantities of one channel at one sample: h5 [5][rows][w].
__global__ void __launch_bounds__(256) k_x_hblur(const double* __restrict__ xa, const double* __restrict__ xb, int w,
                                                 int rows, double* __restrict__ h5) {
  const long long n = (long long)rows * w;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = (int)(i / w), x = (int)(i - (long long)r * w);
  const double* ra = xa + (size_t)r * w;
  const double* rb = xb + (size_t)r * w;
  const bool interior = w > 2 * kRadius && x >= kRadius && x < w - kRadius;
#pragma unroll 1
  for (int q = 0; q < 5; q++) {
    double d;
    if (interior) {
      d = c_xk[kRadius] * quantity(q, ra, rb, x);
#pragma unroll
      for (int t = 1; t <= kRadius; t++) d += c_xk[kRadius + t] * (quantity(q, ra, rb, x - t) + quantity(q, ra, rb, x + t));
    } else {
      d = 0.0;
#pragma unroll
      for (int t = 0; t < 2 * kRadius + 1; t++) {
        const int xx = x + t - kRadius;
        const double v = (xx < 0 || xx > w - 1) ? 0.0 : quantity(q, ra, rb, xx);
        d += c_xk[t] * v;
      }
    }
    h5[(size_t)q * n + i] = d;
  }
}

// Vertical blur (:385-410) and maps (:411-431) at output rows [y0, y1) of one channel: maps [6][y1 - y0][w] hold
// d, d^4, art, art^4, det, det^4 per sample, the values the stripe sums add.
__global__ void __launch_bounds__(256) k_x_vmaps(const double* __restrict__ h5, const double* __restrict__ xa,
                                                 const double* __restrict__ xb, int w, int h, int lo, int rows,
                                                 int y0, int y1, double* __restrict__ maps) {
  const long long no = (long long)(y1 - y0) * w;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= no) return;
  const long long n = (long long)rows * w;
  const int yo = (int)(i / w), x = (int)(i - (long long)yo * w);
  const int y = y0 + yo;
  auto row = [&](int yy) -> size_t {
    if (yy < 0 || yy >= h) yy = yy < 0 ? -yy - 1 : 2 * h - 1 - yy;
    return (size_t)(yy - lo) * w + x;
  };
  double acc[5];
#pragma unroll
  for (int q = 0; q < 5; q++) {
    const double* p = h5 + (size_t)q * n;
    double v = c_xk[kRadius] * p[row(y)];
#pragma unroll
    for (int t = 1; t <= kRadius; t++) v += c_xk[kRadius + t] * (p[row(y - t)] + p[row(y + t)]);
    acc[q] = v;
  }
  const size_t self = (size_t)(y - lo) * w + x;
  const double m1 = acc[0], m2 = acc[1];
  const double s11 = acc[2], s22 = acc[3], s12 = acc[4];
  const double num_m = 1.0 - (m1 - m2) * (m1 - m2);
  const double num_s = 2.0 * (s12 - m1 * m2) + kXC2;
  const double denom_s = (s11 - m1 * m1) + (s22 - m2 * m2) + kXC2;
  const double d = fmax(1.0 - num_m * num_s / denom_s, 0.0);
  const double d1 = (1.0 + fabs(xb[self] - m2)) / (1.0 + fabs(xa[self] - m1)) - 1.0;
  const double art = fmax(d1, 0.0);
  const double det = fmax(-d1, 0.0);
  maps[0 * no + i] = d;
  maps[1 * no + i] = (d * d) * (d * d);
  maps[2 * no + i] = art;
  maps[3 * no + i] = (art * art) * (art * art);
  maps[4 * no + i] = det;
  maps[5 * no + i] = (det * det) * (det * det);
}

// The stripe sums (:432-441): thread (stripe j of the group, channel c, sum k) adds its stripe's values in row-major
// order from zero, one serial chain. maps: [3][6][orows][w] of the group; parts: [stripe][18] (c * 6 + k).
__global__ void __launch_bounds__(32) k_x_sums(const double* __restrict__ maps, int w, int orows, int nstripes,
                                               int stripe0, double* __restrict__ parts) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nstripes * kScoreSums) return;
  const int j = t / kScoreSums, ck = t - j * kScoreSums;
  const int r0 = j * kStripe, r1 = min(r0 + kStripe, orows);
  const long long no = (long long)orows * w;
  const double* p = maps + (size_t)ck * no + (size_t)r0 * w;
  const long long n = (long long)(r1 - r0) * w;
  double s = 0.0;
  long long k = 0;
  // Loads run 16 values ahead of the additions; the additions stay in order.
  if (n >= 16) {
    double cur[16];
#pragma unroll
    for (int u = 0; u < 16; u++) cur[u] = p[u];
    for (k = 16; k + 16 <= n; k += 16) {
      double nxt[16];
#pragma unroll
      for (int u = 0; u < 16; u++) nxt[u] = p[k + u];
#pragma unroll
      for (int u = 0; u < 16; u++) s += cur[u];
#pragma unroll
      for (int u = 0; u < 16; u++) cur[u] = nxt[u];
    }
#pragma unroll
    for (int u = 0; u < 16; u++) s += cur[u];
  }
  for (; k < n; k++) s += p[k];
  parts[(size_t)(stripe0 + j) * kScoreSums + ck] = s;
}

// scale_stats (:446-466): the stripes added in order, then means and 4th roots; stats [3][6] of this scale.
__global__ void k_x_stats(const double* __restrict__ parts, int nstripes, int w, int h, double* __restrict__ stats) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double count = (double)((long long)w * h);
  for (int c = 0; c < 3; c++)
    for (int k = 0; k < 6; k++) {
      double tot = 0.0;
      for (int j = 0; j < nstripes; j++) tot += parts[(size_t)j * kScoreSums + c * 6 + k];
      stats[c * 6 + k] = (k & 1) ? pow(tot / count, 0.25) : tot / count;
    }
}

// ssimulacra2 (:491-511): 108 weighted terms in the reference's order, then the mapping. NaN for the reference's
// non-finite Err.
__global__ void k_x_final(const double* __restrict__ stats, int nscales, double* __restrict__ score) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double ssim = 0.0;
  int i = 0;
  for (int c = 0; c < 3; c++)
    for (int sc = 0; sc < nscales; sc++) {
      const double* st = stats + sc * kScoreSums + c * 6;
      for (int n = 0; n < 2; n++) {
        ssim += c_xw[i] * fabs(st[n]);
        i++;
        ssim += c_xw[i] * fabs(st[2 + n]);
        i++;
        ssim += c_xw[i] * fabs(st[4 + n]);
        i++;
      }
    }
  ssim *= 0.9562382616834844;
  ssim = 2.326765642916932 * ssim - 0.020884521182843837 * ssim * ssim + 6.248496625763138e-05 * ssim * ssim * ssim;
  const double s = ssim > 0.0 ? 100.0 - 10.0 * pow(ssim, 0.6276336467831387) : 100.0;
  *score = isfinite(s) ? s : NAN;
}

// A paused search (search_record, near tie) takes its candidate's exact score and goes on.
__global__ void k_search_resume(SearchState* ss, const double* __restrict__ score) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || ss->done != 2) return;
  const double s = *score;
  ss->done = 0;
  // A non-finite score is the reference's Err, which the search maps to f64::MIN (cli/src/pipeline.rs:218).
  search_record(ss, isfinite(s) ? s : -1.7976931348623157e308, false);
}

// ------------------------------------------------------------------------------------------------ host side

int search_resume(rcg_ctx* ctx, SearchState* d_ss, const double* d_score) {
  RCG_LAUNCH(ctx, "search_resume", k_search_resume, 1, 32, 0, d_ss, d_score);
  return RCG_OK;
}

static std::mutex g_exact_mu;
static bool g_exact_ready[64];

static cudaError_t exact_constants(int device) {
  std::lock_guard<std::mutex> lk(g_exact_mu);
  if (device >= 0 && device < 64 && g_exact_ready[device]) return cudaSuccess;
  // kernel() (:260-271) with the platform libm's exp, as the reference computes it
  double k[2 * kRadius + 1], sum = 0.0;
  for (int i = 0; i < 2 * kRadius + 1; i++) {
    const double x = (double)i - (double)kRadius;
    k[i] = std::exp(-0.5 / (1.5 * 1.5) * x * x);
    sum += k[i];
  }
  for (int i = 0; i < 2 * kRadius + 1; i++) k[i] /= sum;
  const double cb = std::cbrt(kXBias);
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(c_xk, k, sizeof k)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_xw, scorer_weights(), sizeof c_xw)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_cbrt_bias, &cb, sizeof cb)) != cudaSuccess) return e;
  if (device >= 0 && device < 64) g_exact_ready[device] = true;
  return cudaSuccess;
}

// Bytes of working memory per group of stripes: XYB of both images (6 planes) and the five blurred quantities of one
// channel over the group's input rows, and the 18 map planes over its output rows.
static size_t group_bytes(int w, int orows, int rows) {
  return ((size_t)11 * rows + (size_t)18 * orows) * (size_t)w * sizeof(double);
}

constexpr size_t kExactGroupBudget = (size_t)4 << 30;

int exact_score(rcg_ctx* ctx, const float* d_ref0, const float* d_dist0, int w, int h, double* d_score) {
  cudaError_t e = exact_constants(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "exact scorer constant tables");
  // Scales (:480-490): at most 6, while both sides are >= 8.
  int sw[kMaxScales], shh[kMaxScales], ns = 0;
  size_t pyr_floats = 0;
  for (int s = 0, ww = w, hh = h; s < kMaxScales && ww >= kMinSide && hh >= kMinSide; s++) {
    sw[s] = ww;
    shh[s] = hh;
    if (s > 0) pyr_floats += (size_t)3 * ww * hh;
    ns++;
    ww = (ww + 1) / 2;
    hh = (hh + 1) / 2;
  }
  if (ns == 0) return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
  // Stripes per group: as many as fit the working-memory budget (at least one).
  const size_t per_stripe = group_bytes(w, kStripe, kStripe);
  const int gstripes = (int)std::max<size_t>(1, kExactGroupBudget / std::max<size_t>(per_stripe, 1));
  size_t gmax = 0;
  int max_stripes = 0;
  for (int s = 0; s < ns; s++) {
    const int nst = (shh[s] + kStripe - 1) / kStripe;
    max_stripes = std::max(max_stripes, nst);
    const int g = std::min(nst, gstripes);
    const int orows = std::min(g * kStripe, shh[s]);
    gmax = std::max(gmax, group_bytes(sw[s], orows, std::min(orows + 2 * kRadius, shh[s])));
  }
  float* pyr = (float*)workspace(ctx, "x_pyr", std::max<size_t>(2 * pyr_floats * sizeof(float), 256), false);
  double* work = (double*)workspace(ctx, "x_work", gmax, false);
  double* parts = (double*)workspace(ctx, "x_parts", (size_t)max_stripes * kScoreSums * sizeof(double), false);
  double* stats = (double*)workspace(ctx, "x_stats", (size_t)kMaxScales * kScoreSums * sizeof(double), false);
  if (!pyr || !work || !parts || !stats) return RCG_NO_MEMORY;
  const float* a = d_ref0;
  const float* b = d_dist0;
  float* next = pyr;
  for (int s = 0; s < ns; s++) {
    const int W = sw[s], H = shh[s];
    const int nst = (H + kStripe - 1) / kStripe;
    for (int j0 = 0; j0 < nst; j0 += gstripes) {
      const int j1 = std::min(nst, j0 + gstripes);
      const int y0 = j0 * kStripe, y1 = std::min(j1 * kStripe, H);
      const int lo = std::max(y0 - kRadius, 0), hi = std::min(y1 + kRadius, H);
      const int rows = hi - lo, orows = y1 - y0;
      const long long n = (long long)rows * W, no = (long long)orows * W;
      double* xa = work;
      double* xb = xa + 3 * n;
      double* h5 = xb + 3 * n;
      double* maps = h5 + 5 * n;
      const unsigned gi = (unsigned)((n + 255) / 256), go = (unsigned)((no + 255) / 256);
      RCG_LAUNCH(ctx, "x_xyb", k_x_xyb, gi, 256, 0, a, b, W, H, lo, rows, xa, xb);
      for (int c = 0; c < 3; c++) {
        RCG_LAUNCH(ctx, "x_hblur", k_x_hblur, gi, 256, 0, xa + c * n, xb + c * n, W, rows, h5);
        RCG_LAUNCH(ctx, "x_vmaps", k_x_vmaps, go, 256, 0, h5, xa + c * n, xb + c * n, W, H, lo, rows, y0, y1,
                   maps + (size_t)c * 6 * no);
      }
      const int nthreads = (j1 - j0) * kScoreSums;
      RCG_LAUNCH(ctx, "x_sums", k_x_sums, (nthreads + 31) / 32, 32, 0, maps, W, orows, j1 - j0, j0, parts);
    }
    RCG_LAUNCH(ctx, "x_stats", k_x_stats, 1, 32, 0, parts, nst, W, H, stats + s * kScoreSums);
    if (s + 1 < ns) {
      const int ow = sw[s + 1], oh = shh[s + 1];
      const size_t np = (size_t)3 * ow * oh;
      float* na = next;
      float* nb = next + np;
      next += 2 * np;
      const dim3 g((unsigned)(((long long)ow * oh + 255) / 256), 3);
      RCG_LAUNCH(ctx, "x_down", k_x_down, g, 256, 0, a, W, H, na, ow, oh);
      RCG_LAUNCH(ctx, "x_down", k_x_down, g, 256, 0, b, W, H, nb, ow, oh);
      a = na;
      b = nb;
    }
  }
  RCG_LAUNCH(ctx, "x_final", k_x_final, 1, 32, 0, stats, ns, d_score);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "exact scorer launch");
  return RCG_OK;
}

}  // namespace rcg
