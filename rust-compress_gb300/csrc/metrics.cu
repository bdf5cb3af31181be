// The other image metrics of core/src/metrics.rs on the GPU: ssim (:13-62), psnr (:64-73) and ms_ssim (:75-127),
// for the scorer callers that use them (cli/src/pipeline.rs:130-138) and for the `--target-ssim` JPEG search
// (jpeg/src/target.rs:24, cli/src/pipeline.rs:213).
//
// SSIM: every window sum is an integer (8x8 pixels of 8-bit samples), so the sums are exact in int32 and the
// per-window f64 formula is evaluated with the reference's operations in the reference's order (explicit
// round-to-nearest intrinsics, no contraction), giving the reference's window values bit for bit. One CTA per row of
// windows: 4-column group sums (a window is two adjacent groups), the window values, then the row's sum from left to
// right. The rows are added in order by one thread (the reference adds them with rayon's reduce, whose association
// is unspecified; the two agree to rounding).

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "rcg_internal.cuh"

namespace rcg {

namespace {

constexpr double kC1 = 6.5025;   // (0.01 * 255)^2, core/src/metrics.rs:6
constexpr double kC2 = 58.5225;  // (0.03 * 255)^2, core/src/metrics.rs:7
constexpr int kWinTile = 256;    // windows per tile of a row

// window_ssim's per-channel term (core/src/metrics.rs:54-59) from exact sums over n pixels.
__device__ __forceinline__ double ssim_term(double sx, double sy, double sxx, double syy, double sxy, double n) {
  const double mx = __ddiv_rn(sx, n), my = __ddiv_rn(sy, n);
  const double vx = __dsub_rn(__ddiv_rn(sxx, n), __dmul_rn(mx, mx));
  const double vy = __dsub_rn(__ddiv_rn(syy, n), __dmul_rn(my, my));
  const double cov = __dsub_rn(__ddiv_rn(sxy, n), __dmul_rn(mx, my));
  const double num = __dmul_rn(__dadd_rn(__dmul_rn(__dmul_rn(2.0, mx), my), kC1), __dadd_rn(__dmul_rn(2.0, cov), kC2));
  const double den =
      __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(mx, mx), __dmul_rn(my, my)), kC1), __dadd_rn(__dadd_rn(vx, vy), kC2));
  return __ddiv_rn(num, den);
}

template <int CH>
__global__ void __launch_bounds__(256) k_ssim_rows(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                                   int w, int nx, int ny, double* __restrict__ rowsums,
                                                   const StepDesc* __restrict__ st) {
  if (st && !st->active) return;
  __shared__ int gs[kWinTile + 1][CH][5];
  __shared__ double vals[kWinTile];
  for (int j = blockIdx.x; j < ny; j += gridDim.x) {
    const size_t y0 = 4 * (size_t)j;
    double rowsum = 0.0;
    for (int t0 = 0; t0 < nx; t0 += kWinTile) {
      const int nwin = min(kWinTile, nx - t0);
      for (int g = threadIdx.x; g <= nwin; g += blockDim.x) {
        const size_t x0 = 4 * (size_t)(t0 + g);
        int acc[CH][5];
#pragma unroll
        for (int c = 0; c < CH; c++)
#pragma unroll
          for (int k = 0; k < 5; k++) acc[c][k] = 0;
        for (int r = 0; r < 8; r++) {
          const uint8_t* pa = a + ((y0 + r) * w + x0) * CH;
          const uint8_t* pb = b + ((y0 + r) * w + x0) * CH;
#pragma unroll
          for (int i = 0; i < 4 * CH; i++) {
            const int p = pa[i], q = pb[i], c = i % CH;
            acc[c][0] += p;
            acc[c][1] += q;
            acc[c][2] += p * p;
            acc[c][3] += q * q;
            acc[c][4] += p * q;
          }
        }
#pragma unroll
        for (int c = 0; c < CH; c++)
#pragma unroll
          for (int k = 0; k < 5; k++) gs[g][c][k] = acc[c][k];
      }
      __syncthreads();
      for (int i = threadIdx.x; i < nwin; i += blockDim.x) {
        double total = 0.0;
#pragma unroll
        for (int c = 0; c < CH; c++) {
          double s[5];
#pragma unroll
          for (int k = 0; k < 5; k++) s[k] = (double)(gs[i][c][k] + gs[i + 1][c][k]);
          total = __dadd_rn(total, ssim_term(s[0], s[1], s[2], s[3], s[4], 64.0));
        }
        vals[i] = __ddiv_rn(total, (double)CH);
      }
      __syncthreads();
      if (threadIdx.x == 0)
        for (int i = 0; i < nwin; i++) rowsum = __dadd_rn(rowsum, vals[i]);
      __syncthreads();
    }
    if (threadIdx.x == 0) rowsums[j] = rowsum;
  }
}

__global__ void k_ssim_final(const double* __restrict__ rowsums, int nx, int ny, double* __restrict__ score,
                             SearchState* __restrict__ ss, const StepDesc* __restrict__ st) {
  if (st && !st->active) return;
  if (threadIdx.x != 0) return;
  double sum = 0.0;
  for (int j = 0; j < ny; j++) sum = __dadd_rn(sum, rowsums[j]);
  const double v = __ddiv_rn(sum, (double)((long long)nx * ny));
  *score = v;
  if (ss) search_record(ss, v);
}

// Below 8 pixels in either direction: one window over the whole image (core/src/metrics.rs:18-21).
template <int CH>
__global__ void __launch_bounds__(256) k_ssim_global(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                                     int w, int h, double* __restrict__ score,
                                                     SearchState* __restrict__ ss, const StepDesc* __restrict__ st) {
  if (st && !st->active) return;
  __shared__ unsigned long long sums[CH][5];
  if (threadIdx.x < CH * 5) (&sums[0][0])[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long acc[CH][5];
#pragma unroll
  for (int c = 0; c < CH; c++)
#pragma unroll
    for (int k = 0; k < 5; k++) acc[c][k] = 0;
  const size_t npx = (size_t)w * h;
  for (size_t i = threadIdx.x; i < npx; i += blockDim.x) {
#pragma unroll
    for (int c = 0; c < CH; c++) {
      const unsigned long long p = a[i * CH + c], q = b[i * CH + c];
      acc[c][0] += p;
      acc[c][1] += q;
      acc[c][2] += p * p;
      acc[c][3] += q * q;
      acc[c][4] += p * q;
    }
  }
#pragma unroll
  for (int c = 0; c < CH; c++)
#pragma unroll
    for (int k = 0; k < 5; k++) atomicAdd(&sums[c][k], acc[c][k]);
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double n = __dmul_rn((double)w, (double)h);
  double total = 0.0;
  for (int c = 0; c < CH; c++)
    total = __dadd_rn(total, ssim_term((double)sums[c][0], (double)sums[c][1], (double)sums[c][2],
                                       (double)sums[c][3], (double)sums[c][4], n));
  const double v = __ddiv_rn(total, (double)CH);
  *score = v;
  if (ss) search_record(ss, v);
}

// Sum of squared sample differences (psnr, core/src/metrics.rs:70): exact in 64-bit integers.
__global__ void __launch_bounds__(256) k_sq_err(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                                size_t n, unsigned long long* __restrict__ out) {
  unsigned long long acc = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int d = (int)a[i] - (int)b[i];
    acc += (unsigned long long)(d * d);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// luma (core/src/metrics.rs:75-87): Gray as is, GrayAlpha's gray, else (299R + 587G + 114B + 500) / 1000.
__global__ void k_luma(const uint8_t* __restrict__ a, size_t npx, int ch, uint8_t* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += (size_t)gridDim.x * blockDim.x) {
    const uint8_t* p = a + i * ch;
    out[i] = ch <= 2 ? p[0] : (uint8_t)((299u * p[0] + 587u * p[1] + 114u * p[2] + 500u) / 1000u);
  }
}

// downsample2 (core/src/metrics.rs:89-106): floor of the 2x2 mean, odd edges dropped.
__global__ void k_down2(const uint8_t* __restrict__ in, int w, int nw, int nh, uint8_t* __restrict__ out) {
  const size_t n = (size_t)nw * nh;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / nw), x = (int)(i % nw);
    const uint8_t* p = in + (size_t)(2 * y) * w + 2 * x;
    out[i] = (uint8_t)(((unsigned)p[0] + p[1] + p[w] + p[w + 1]) / 4u);
  }
}

int grid_for(size_t n, int threads) {
  return (int)std::min<size_t>((n + threads - 1) / threads, (size_t)152 * 16);
}

}  // namespace

int ssim_score(rcg_ctx* ctx, const uint8_t* d_a, const uint8_t* d_b, int w, int h, int ch, double* d_score,
               SearchState* ss, const StepDesc* st) {
  if (ch < 1 || ch > 4) return fail(ctx, RCG_INVALID, "ssim takes 1..=4 channels");
  if (w < 8 || h < 8) {
    switch (ch) {
      case 1: RCG_LAUNCH(ctx, "ssim_global", k_ssim_global<1>, 1, 256, 0, d_a, d_b, w, h, d_score, ss, st); break;
      case 2: RCG_LAUNCH(ctx, "ssim_global", k_ssim_global<2>, 1, 256, 0, d_a, d_b, w, h, d_score, ss, st); break;
      case 3: RCG_LAUNCH(ctx, "ssim_global", k_ssim_global<3>, 1, 256, 0, d_a, d_b, w, h, d_score, ss, st); break;
      default: RCG_LAUNCH(ctx, "ssim_global", k_ssim_global<4>, 1, 256, 0, d_a, d_b, w, h, d_score, ss, st); break;
    }
    return RCG_OK;
  }
  const int nx = (w - 8) / 4 + 1, ny = (h - 8) / 4 + 1;
  double* rows = (double*)workspace(ctx, "ssim_rows", sizeof(double) * (size_t)ny);
  if (!rows) return RCG_NO_MEMORY;
  const int grid = std::min(ny, 65535);
  switch (ch) {
    case 1: RCG_LAUNCH(ctx, "ssim_rows", k_ssim_rows<1>, grid, 256, 0, d_a, d_b, w, nx, ny, rows, st); break;
    case 2: RCG_LAUNCH(ctx, "ssim_rows", k_ssim_rows<2>, grid, 256, 0, d_a, d_b, w, nx, ny, rows, st); break;
    case 3: RCG_LAUNCH(ctx, "ssim_rows", k_ssim_rows<3>, grid, 256, 0, d_a, d_b, w, nx, ny, rows, st); break;
    default: RCG_LAUNCH(ctx, "ssim_rows", k_ssim_rows<4>, grid, 256, 0, d_a, d_b, w, nx, ny, rows, st); break;
  }
  RCG_LAUNCH(ctx, "ssim_final", k_ssim_final, 1, 32, 0, rows, nx, ny, d_score, ss, st);
  return RCG_OK;
}

int squared_error(rcg_ctx* ctx, const uint8_t* d_a, const uint8_t* d_b, size_t n, unsigned long long* d_out) {
  cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), ctx->stream);
  RCG_LAUNCH(ctx, "sq_err", k_sq_err, grid_for(n, 256), 256, 0, d_a, d_b, n, d_out);
  return RCG_OK;
}

int luma8(rcg_ctx* ctx, const uint8_t* d_a, size_t npx, int ch, uint8_t* d_out) {
  RCG_LAUNCH(ctx, "luma", k_luma, grid_for(npx, 256), 256, 0, d_a, npx, ch, d_out);
  return RCG_OK;
}

int downsample2(rcg_ctx* ctx, const uint8_t* d_in, int w, int h, uint8_t* d_out) {
  const int nw = w / 2, nh = h / 2;
  RCG_LAUNCH(ctx, "down2", k_down2, grid_for((size_t)nw * nh, 256), 256, 0, d_in, w, nw, nh, d_out);
  return RCG_OK;
}

}  // namespace rcg
