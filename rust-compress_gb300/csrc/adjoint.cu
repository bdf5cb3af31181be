// Reverse-mode derivative of SSIMULACRA2 (core/src/ssimulacra2.rs:171-512) with respect to the distorted image's
// RGB samples, taken as continuous values in [0, 255], on the GPU.
//
// Forward: linear light by the sRGB curve itself (:172-175; the reference's 8-bit table samples it), the 2x2
// pyramid, and per scale the XYB planes, the five blurred moments per channel and the six map sums. Backward, from
// the coarsest scale to the finest: d score / d map from the 108-term sum, the final mapping and the L1/L4 norms;
// through the SSIM and edge maps to the moments and the XYB samples (one-sided derivatives at the max(., 0) and |.|
// kinks); through the blurs (the zero-padded row blur is its own transpose, the mirrored column blur scatters
// back); through XYB to linear light; plus the coarser scales' gradients spread back over their 2x2 blocks; and
// finally through the sRGB curve. The blur intermediates are recomputed per scale in the backward pass, not kept
// from the forward one. Plane kernels, one thread per sample, templated on the real type: FP64 (the checked
// gradient: it matches the FP64 CPU gradient to rounding) and FP32 (the perceptual weights, where a few significant
// digits suffice: the variances' cancellation error, ~1e-8, is small against the SSIM constant 9e-4 that bounds
// every denominator, and GB300's FP32 rate is many times its FP64 rate). Sums of the maps are f64 across threads in
// both; the final mapping runs on the host in f64.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "rcg_internal.cuh"

namespace rcg {

namespace {

constexpr int kR = 5;  // kernel radius (:16)
constexpr double kBiasD = 0.0037930732552754493;
constexpr double kM00 = 0.30, kM02 = 0.078, kM01 = 1.0 - kM02 - kM00;
constexpr double kM10 = 0.23, kM12 = 0.078, kM11 = 1.0 - kM12 - kM10;
constexpr double kM20 = 0.2434226892454782, kM21 = 0.2047674442449682, kM22 = 1.0 - kM20 - kM21;
constexpr double kC2 = 0.0009;

// normalized Gaussian taps (sigma 1.5) in both types
__constant__ double c_k64[2 * kR + 1];
__constant__ float c_k32[2 * kR + 1];
// The curve and its derivative at the 256 integer samples, computed on the host with the same expressions (an
// 8-bit reference, and decoded candidates passed as whole-number samples, skip the pow).
__constant__ double c_lin8[256];
__constant__ double c_dlin8[256];

template <typename T> __device__ __forceinline__ T tap(int t);
template <> __device__ __forceinline__ double tap<double>(int t) { return c_k64[t]; }
template <> __device__ __forceinline__ float tap<float>(int t) { return c_k32[t]; }
__device__ __forceinline__ double cbrt_t(double x) { return cbrt(x); }
__device__ __forceinline__ float cbrt_t(float x) { return cbrtf(x); }

__device__ __forceinline__ double srgb64(double v) {
  return v <= 0.04045 ? v / 12.92 : pow((v + 0.055) / 1.055, 2.4);
}
__device__ __forceinline__ double srgb64_deriv(double v255) {
  const double v = v255 / 255.0;
  return v <= 0.04045 ? 1.0 / (12.92 * 255.0) : 2.4 * pow((v + 0.055) / 1.055, 1.4) / (1.055 * 255.0);
}

__device__ __forceinline__ long long tid1() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }

// Index of a whole-number sample in [0, 255], else -1.
__device__ __forceinline__ int sample8(float v) {
  return (v >= 0.0f && v <= 255.0f && v == rintf(v)) ? (int)v : -1;
}

// Linear planes [3][n] of the reference (8-bit samples) and of the distorted image (f32 samples), by the curve.
template <typename T>
__global__ void k_lin(const uint8_t* __restrict__ ref, const float* __restrict__ dist, long long n,
                      T* __restrict__ la, T* __restrict__ lb) {
  __shared__ T lut[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = (T)c_lin8[i];
  __syncthreads();
  for (long long i = tid1(); i < n; i += (long long)gridDim.x * blockDim.x)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      // both images through the same curve: identical inputs give identical planes (and the score 100)
      la[c * n + i] = lut[ref[i * 3 + c]];
      const float v = dist[i * 3 + c];
      const int k = sample8(v);
      lb[c * n + i] = k >= 0 ? lut[k] : (T)srgb64((double)v / 255.0);
    }
}

// 2x2 means (:225-247), fewer samples at odd edges; 3 channels.
// Grid (output columns, rows, channels): see grid_rows.
template <typename T>
__global__ void k_down(const T* __restrict__ src, int w, int h, T* __restrict__ dst, int ow, int oh) {
  const int ox = blockIdx.x * blockDim.x + threadIdx.x;
  if (ox >= ow) return;
  const long long n = (long long)ow * oh;
  const int c = blockIdx.z;
  const T* p = src + (long long)c * w * h;
  const int x1 = min(2 * ox + 2, w);
  for (int oy = blockIdx.y; oy < oh; oy += gridDim.y) {
    const int y1 = min(2 * oy + 2, h);
    T s = 0;
    for (int y = 2 * oy; y < y1; y++)
      for (int x = 2 * ox; x < x1; x++) s += p[(long long)y * w + x];
    dst[c * n + (long long)oy * ow + ox] = s / (T)((y1 - 2 * oy) * (x1 - 2 * ox));
  }
}

// XYB (:249-258) of 3 linear planes.
template <typename T>
__global__ void k_xyb(const T* __restrict__ lin, long long n, T* __restrict__ xyb) {
  const T M00 = (T)kM00, M01 = (T)kM01, M02 = (T)kM02, M10 = (T)kM10, M11 = (T)kM11, M12 = (T)kM12;
  const T M20 = (T)kM20, M21 = (T)kM21, M22 = (T)kM22, bias = (T)kBiasD;
  const T cb = cbrt_t(bias);
  for (long long i = tid1(); i < n; i += (long long)gridDim.x * blockDim.x) {
    const T r = lin[i], g = lin[n + i], b = lin[2 * n + i];
    const T m0 = cbrt_t(fmax(M00 * r + M01 * g + M02 * b + bias, (T)0)) - cb;
    const T m1 = cbrt_t(fmax(M10 * r + M11 * g + M12 * b + bias, (T)0)) - cb;
    const T m2 = cbrt_t(fmax(M20 * r + M21 * g + M22 * b + bias, (T)0)) - cb;
    const T x = (T)0.5 * (m0 - m1), y = (T)0.5 * (m0 + m1);
    xyb[i] = x * (T)14.0 + (T)0.42;
    xyb[n + i] = y + (T)0.01;
    xyb[2 * n + i] = (m2 - y) + (T)0.55;
  }
}

// The plane kernels below run on a (columns / 256, rows, planes) grid: a thread owns one column of one plane and
// strides over the rows, so no sample index is divided back into (plane, row, column).
dim3 grid_rows(int w, int h, int planes) {
  return dim3((unsigned)((w + 255) / 256), (unsigned)std::min(h, 65535), (unsigned)planes);
}

// Outputs per thread of the row blurs: a run of kHRun consecutive outputs reads its kHRun + 10 source samples once
// (in registers) instead of 11 per output; every output still sums its in-range taps in the same order.
constexpr int kHRun = 4;

// The row blurs' grid: (column runs / 256, rows, planes).
dim3 grid_row_runs(int w, int h, int planes) {
  return dim3((unsigned)(((w + kHRun - 1) / kHRun + 255) / 256), (unsigned)std::min(h, 65535), (unsigned)planes);
}

// Row blur (zero outside) of one plane: the backward pass's rows (the zero-padded row blur is its own transpose).
// One plane per grid z.
template <typename T>
__global__ void k_hblur(const T* __restrict__ src, int w, int h, T* __restrict__ dst) {
  const int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * kHRun;
  if (x0 >= w) return;
  const long long n = (long long)w * h;
  const T* sp = src + blockIdx.z * n;
  T* dp = dst + blockIdx.z * n;
  for (int y = blockIdx.y; y < h; y += gridDim.y) {
    const T* row = sp + (long long)y * w;
    T v[kHRun + 2 * kR];
#pragma unroll
    for (int k = 0; k < kHRun + 2 * kR; k++) {
      const int xx = x0 + k - kR;
      v[k] = xx >= 0 && xx < w ? row[xx] : (T)0;
    }
#pragma unroll
    for (int o = 0; o < kHRun; o++) {
      const int x = x0 + o;
      if (x >= w) break;
      T s = 0;
#pragma unroll
      for (int t = 0; t <= 2 * kR; t++) {
        const int xx = x + t - kR;
        if (xx < 0 || xx >= w) continue;
        s += tap<T>(t) * v[o + t];
      }
      dp[(long long)y * w + x] = s;
    }
  }
}

// A thread's run of kHRun outputs in each of the five planes: one 16-byte store per plane (two for double) when the
// run lies in the row and the planes are 4-sample aligned, else one store per output.
template <typename T>
__device__ __forceinline__ void store_run5(T* __restrict__ dst, long long n, long long rowi, int x0, int w,
                                           const T (&out)[5][kHRun]) {
  static_assert(kHRun == 4, "vector stores of four samples");
  const long long i = rowi + x0;
  if (x0 + kHRun <= w && (w & 3) == 0 && ((uintptr_t)dst & 31) == 0) {
#pragma unroll
    for (int q = 0; q < 5; q++) {
      if constexpr (sizeof(T) == 4) {
        *reinterpret_cast<float4*>(dst + q * n + i) = make_float4(out[q][0], out[q][1], out[q][2], out[q][3]);
      } else {
        reinterpret_cast<double2*>(dst + q * n + i)[0] = make_double2(out[q][0], out[q][1]);
        reinterpret_cast<double2*>(dst + q * n + i)[1] = make_double2(out[q][2], out[q][3]);
      }
    }
    return;
  }
#pragma unroll
  for (int o = 0; o < kHRun; o++)
    if (x0 + o < w)
#pragma unroll
      for (int q = 0; q < 5; q++) dst[q * n + i + o] = out[q][o];
}

// The five products of the forward pass blurred along rows in one sweep: dst + q * n for q = 0 xa, 1 xb, 2 xa^2,
// 3 xb^2, 4 xa xb (each output summed over the taps in the same order as k_hblur).
template <typename T>
__global__ void k_hblur5(const T* __restrict__ xa, const T* __restrict__ xb, int w, int h, T* __restrict__ dst) {
  const int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * kHRun;
  if (x0 >= w) return;
  const long long n = (long long)w * h;
  for (int y = blockIdx.y; y < h; y += gridDim.y) {
    const long long rowi = (long long)y * w;
    T va[kHRun + 2 * kR], vb[kHRun + 2 * kR];
#pragma unroll
    for (int k = 0; k < kHRun + 2 * kR; k++) {
      const int xx = x0 + k - kR;
      const bool in = xx >= 0 && xx < w;
      va[k] = in ? xa[rowi + xx] : (T)0;
      vb[k] = in ? xb[rowi + xx] : (T)0;
    }
    T out[5][kHRun];
#pragma unroll
    for (int o = 0; o < kHRun; o++) {
      const int x = x0 + o;
      T s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
#pragma unroll
      for (int t = 0; t <= 2 * kR; t++) {
        const int xx = x + t - kR;
        if (xx < 0 || xx >= w) continue;
        const T a = va[o + t], b = vb[o + t], k = tap<T>(t);
        s0 += k * a;
        s1 += k * b;
        s2 += k * (a * a);
        s3 += k * (b * b);
        s4 += k * (a * b);
      }
      out[0][o] = s0;
      out[1][o] = s1;
      out[2][o] = s2;
      out[3][o] = s3;
      out[4][o] = s4;
    }
    store_run5(dst, n, rowi, x0, w, out);
  }
}

__device__ __forceinline__ int mirror64(int yy, int h) { return yy < 0 ? -yy - 1 : (yy >= h ? 2 * h - 1 - yy : yy); }

// Rows per thread of the column blurs: a run of kRun outputs reads its kRun + 10 source rows once (in registers)
// instead of 11 rows per output; every output still sums its taps in the same order. The forward blur takes runs of
// 16 (0.94 against 1.18 ms per perceptual search at 12 MP with 8), its transpose runs of 8 (0.39 against 0.47 with 16).
constexpr int kRunN = 16, kRun = 8;

// Column blur with mirrored rows (:385-397), one plane per grid z, grid y over runs of kRunN rows.
template <typename T>
__global__ void k_vblur_n(const T* __restrict__ src, int w, int h, T* __restrict__ dst) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= w) return;
  const long long n = (long long)w * h;
  const T* sp = src + blockIdx.z * n + x;
  T* dp = dst + blockIdx.z * n + x;
  const int runs = (h + kRunN - 1) / kRunN;
  for (int r = blockIdx.y; r < runs; r += gridDim.y) {
    const int y0 = r * kRunN;
    T v[kRunN + 2 * kR];
#pragma unroll
    for (int k = 0; k < kRunN + 2 * kR; k++) {
      const int yy = y0 + k - kR;
      v[k] = yy <= h - 1 + kR ? sp[(long long)mirror64(yy, h) * w] : (T)0;  // rows past a short last run: unused
    }
#pragma unroll
    for (int o = 0; o < kRunN; o++) {
      if (y0 + o >= h) break;
      T s = 0;
#pragma unroll
      for (int t = 0; t <= 2 * kR; t++) s += tap<T>(t) * v[o + t];
      dp[(long long)(y0 + o) * w] = s;
    }
  }
}

// Transpose of the column blur as a gather: row y' receives tap t from the rows y whose mirrored source row is y', i.e.
// from source index y' (y = y' - t + R), -y' - 1 (mirrored at the top) and 2h - 1 - y' (at the bottom).
// One plane per grid z, grid y over runs of kRun rows; a run inside the interior reads its rows once.
template <typename T>
__global__ void k_vblur_t(const T* __restrict__ gsrc, int w, int h, T* __restrict__ dst) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= w) return;
  const long long n = (long long)w * h;
  const T* g = gsrc + blockIdx.z * n;
  T* dp = dst + blockIdx.z * n;
  const int runs = (h + kRun - 1) / kRun;
  for (int r = blockIdx.y; r < runs; r += gridDim.y) {
    const int y0 = r * kRun;
    if (y0 >= kR && y0 + kRun - 1 < h - kR) {
      // every output row of the run is interior: row yp takes tap t from source row yp - t + kR
      T v[kRun + 2 * kR];
#pragma unroll
      for (int k = 0; k < kRun + 2 * kR; k++) v[k] = g[(long long)(y0 - kR + k) * w + x];
#pragma unroll
      for (int o = 0; o < kRun; o++) {
        T s = 0;
#pragma unroll
        for (int t = 0; t <= 2 * kR; t++) s += tap<T>(t) * v[o + 2 * kR - t];
        dp[(long long)(y0 + o) * w + x] = s;
      }
      continue;
    }
    for (int yp = y0; yp < min(y0 + kRun, h); yp++) {
      T s = 0;
      if (yp >= kR && yp < h - kR) {
        // interior: only the direct source row is in range (the mirrored ones are not)
#pragma unroll
        for (int t = 0; t <= 2 * kR; t++) s += tap<T>(t) * g[(long long)(yp - t + kR) * w + x];
      } else {
#pragma unroll
        for (int t = 0; t <= 2 * kR; t++) {
          const int ys[3] = {yp - t + kR, -yp - 1 - t + kR, 2 * h - 1 - yp - t + kR};
#pragma unroll
          for (int e = 0; e < 3; e++)
            if (ys[e] >= 0 && ys[e] < h) s += tap<T>(t) * g[(long long)ys[e] * w + x];
        }
      }
      dp[(long long)yp * w + x] = s;
    }
  }
}

// The six map sums of one channel (:421-440): per-thread sums in T, then f64 per-CTA partials (parts[block][6]);
// k_sum_parts adds them in a fixed order, so the score and the gradient are the same bits on every run.
template <typename T>
__global__ void __launch_bounds__(256) k_maps(const T* __restrict__ mom, const T* __restrict__ xa,
                                              const T* __restrict__ xb, long long n, double* __restrict__ parts) {
  __shared__ double red[6][8];
  const T one = 1, c2 = (T)kC2;
  T acc[6] = {0, 0, 0, 0, 0, 0};
  for (long long i = tid1(); i < n; i += (long long)gridDim.x * blockDim.x) {
    const T m1 = mom[i], m2 = mom[n + i], s11 = mom[2 * n + i], s22 = mom[3 * n + i], s12 = mom[4 * n + i];
    const T num_m = one - (m1 - m2) * (m1 - m2);
    const T num_s = (T)2 * (s12 - m1 * m2) + c2;
    const T den_s = (s11 - m1 * m1) + (s22 - m2 * m2) + c2;
    const T d = fmax(one - num_m * num_s / den_s, (T)0);
    const T d1 = (one + fabs(xb[i] - m2)) / (one + fabs(xa[i] - m1)) - one;
    const T art = fmax(d1, (T)0), det = fmax(-d1, (T)0);
    acc[0] += d;
    acc[1] += (d * d) * (d * d);
    acc[2] += art;
    acc[3] += (art * art) * (art * art);
    acc[4] += det;
    acc[5] += (det * det) * (det * det);
  }
  // Warp sums in T (the FP32 pass keeps its shuffles off this part's narrow FP64 pipe, which otherwise took half
  // of each launch), then f64 across the warps and CTAs in a fixed order.
#pragma unroll
  for (int k = 0; k < 6; k++) {
    T v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = (double)v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int wi = 0; wi < 8; wi++) v += red[threadIdx.x][wi];
    parts[(size_t)blockIdx.x * 6 + threadIdx.x] = v;
  }
}

// sums[k] = the nparts partials of column k, one warp per column, lanes strided then a shuffle tree.
__global__ void __launch_bounds__(192) k_sum_parts(const double* __restrict__ parts, int nparts,
                                                   double* __restrict__ sums) {
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double v = 0.0;
  for (int i = lane; i < nparts; i += 32) v += parts[(size_t)i * 6 + k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sums[k] = v;
}

// Per sample of one channel: d score / d (m2, s22, s12) and the direct d score / d xb of the edge maps, given the
// norms' coefficients g1 (L1: weight / count) and g4 (L4: weight (S/count)^-3/4 / count) of (ssim, artifact,
// detail).
struct NormCoef {
  double g1[3], g4[3];
};

template <typename T>
__global__ void k_mapgrad(const T* __restrict__ mom, const T* __restrict__ xa, const T* __restrict__ xb, long long n,
                          NormCoef ncd, T* __restrict__ g_m2, T* __restrict__ g_s22, T* __restrict__ g_s12,
                          T* __restrict__ g_xb) {
  const T one = 1, two = 2, zero = 0, c2 = (T)kC2;
  T g1[3], g4[3];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    g1[m] = (T)ncd.g1[m];
    g4[m] = (T)ncd.g4[m];
  }
  for (long long i = tid1(); i < n; i += (long long)gridDim.x * blockDim.x) {
    const T m1 = mom[i], m2 = mom[n + i], s11 = mom[2 * n + i], s22 = mom[3 * n + i], s12 = mom[4 * n + i];
    const T num_m = one - (m1 - m2) * (m1 - m2);
    const T num_s = two * (s12 - m1 * m2) + c2;
    const T den_s = (s11 - m1 * m1) + (s22 - m2 * m2) + c2;
    const T dv = one - num_m * num_s / den_s;
    T gm2 = zero, gs22 = zero, gs12 = zero;
    if (dv > zero) {
      const T gd = g1[0] + g4[0] * dv * dv * dv;
      const T g_num_m = -gd * num_s / den_s, g_num_s = -gd * num_m / den_s;
      const T g_den = gd * num_m * num_s / (den_s * den_s);
      gm2 = g_num_m * (two * (m1 - m2)) + g_num_s * (-two * m1) + g_den * (-two * m2);
      gs22 = g_den;
      gs12 = two * g_num_s;
    }
    const T a = xa[i], b = xb[i];
    const T Nn = one + fabs(b - m2), Dn = one + fabs(a - m1);
    const T d1 = Nn / Dn - one;
    const T gd1 = (d1 > zero ? g1[1] + g4[1] * d1 * d1 * d1 : zero) -
                  (d1 < zero ? g1[2] + g4[2] * (-d1) * (-d1) * (-d1) : zero);
    const T sb = b - m2 > zero ? one : (b - m2 < zero ? -one : zero);
    g_xb[i] = gd1 * sb / Dn;
    g_m2[i] = gm2 - gd1 * sb / Dn;
    g_s22[i] = gs22;
    g_s12[i] = gs12;
  }
}

// d score / d xb = direct + G^T(g_m2) + 2 xb G^T(g_s22) + xa G^T(g_s12) for one channel.
template <typename T>
__global__ void k_combine(const T* __restrict__ t_m2, const T* __restrict__ t_s22, const T* __restrict__ t_s12,
                          const T* __restrict__ xa, const T* __restrict__ xb, long long n, T* __restrict__ g_xb) {
  for (long long i = tid1(); i < n; i += (long long)gridDim.x * blockDim.x)
    g_xb[i] += t_m2[i] + (T)2 * xb[i] * t_s22[i] + xa[i] * t_s12[i];
}

// XYB adjoint to the linear planes of this scale, plus the coarser scale's gradient spread over its 2x2 blocks.
template <typename T>
__global__ void k_xyb_adj(const T* __restrict__ lin, const T* __restrict__ g_xyb, int w, int h,
                          const T* __restrict__ g_coarse, int cw, T* __restrict__ g_lin) {
  const T M00 = (T)kM00, M01 = (T)kM01, M02 = (T)kM02, M10 = (T)kM10, M11 = (T)kM11, M12 = (T)kM12;
  const T M20 = (T)kM20, M21 = (T)kM21, M22 = (T)kM22, bias = (T)kBiasD;
  const T zero = 0, one = 1, three = 3, half = (T)0.5, seven = 7;
  const long long n = (long long)w * h, cn = (long long)cw * ((h + 1) / 2);
  for (long long i = tid1(); i < n; i += (long long)gridDim.x * blockDim.x) {
    const T r = lin[i], g = lin[n + i], b = lin[2 * n + i];
    const T u0 = M00 * r + M01 * g + M02 * b + bias, u1 = M10 * r + M11 * g + M12 * b + bias,
            u2 = M20 * r + M21 * g + M22 * b + bias;
    const T d0 = u0 > zero ? one / (three * cbrt_t(u0) * cbrt_t(u0)) : zero;
    const T d1 = u1 > zero ? one / (three * cbrt_t(u1) * cbrt_t(u1)) : zero;
    const T d2 = u2 > zero ? one / (three * cbrt_t(u2) * cbrt_t(u2)) : zero;
    const T gX = g_xyb[i], gY = g_xyb[n + i], gB = g_xyb[2 * n + i];
    const T gu0 = (seven * gX + half * gY - half * gB) * d0, gu1 = (-seven * gX + half * gY - half * gB) * d1,
            gu2 = gB * d2;
    T o[3] = {gu0 * M00 + gu1 * M10 + gu2 * M20, gu0 * M01 + gu1 * M11 + gu2 * M21,
              gu0 * M02 + gu1 * M12 + gu2 * M22};
    if (g_coarse) {
      const unsigned ui = (unsigned)i;  // within one plane: fewer than 2^32 samples
      const int y = (int)(ui / (unsigned)w), x = (int)(ui - (unsigned)y * (unsigned)w), ox = x / 2, oy = y / 2;
      const int nx = min(2 * ox + 2, w) - 2 * ox, ny = min(2 * oy + 2, h) - 2 * oy;
      const T inv = one / (T)(nx * ny);
#pragma unroll
      for (int c = 0; c < 3; c++) o[c] += g_coarse[c * cn + (long long)oy * cw + ox] * inv;
    }
#pragma unroll
    for (int c = 0; c < 3; c++) g_lin[c * n + i] = o[c];
  }
}

// Through the sRGB curve to the samples (interleaved RGB), written as f64.
template <typename T>
__global__ void k_grad_out(const T* __restrict__ g_lin, const float* __restrict__ dist, long long n,
                           double* __restrict__ grad) {
  __shared__ double dlut[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) dlut[i] = c_dlin8[i];
  __syncthreads();
  for (long long i = tid1(); i < n; i += (long long)gridDim.x * blockDim.x)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float v = dist[i * 3 + c];
      const int k = sample8(v);
      grad[i * 3 + c] = (double)g_lin[c * n + i] * (k >= 0 ? dlut[k] : srgb64_deriv((double)v));
    }
}

unsigned grid_of(long long n) {
  return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32));
}

// The whole pass in real type T; workspace buffers are named per type.
template <typename T>
int grad_impl(rcg_ctx* ctx, const uint8_t* d_ref, const float* d_dist, int w, int h, double* score, double* d_grad) {
  const std::string pfx = sizeof(T) == 8 ? "adj64_" : "adj32_";
  auto ws = [&](const char* name, size_t count) { return (T*)workspace(ctx, (pfx + name).c_str(), count * sizeof(T)); };
  // constants
  double k[2 * kR + 1], sum = 0.0;
  for (int i = 0; i <= 2 * kR; i++) {
    const double x = (double)(i - kR);
    k[i] = std::exp(-0.5 / (1.5 * 1.5) * x * x);
    sum += k[i];
  }
  float k32[2 * kR + 1];
  for (int i = 0; i <= 2 * kR; i++) {
    k[i] /= sum;
    k32[i] = (float)k[i];
  }
  // pageable sources: each upload has read its source when the call returns
  cudaMemcpyToSymbolAsync(c_k64, k, sizeof k, 0, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyToSymbolAsync(c_k32, k32, sizeof k32, 0, cudaMemcpyHostToDevice, ctx->stream);
  double lin8[256], dlin8[256];
  for (int i = 0; i < 256; i++) {
    const double v = (double)i / 255.0;
    lin8[i] = v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4);
    dlin8[i] = v <= 0.04045 ? 1.0 / (12.92 * 255.0) : 2.4 * std::pow((v + 0.055) / 1.055, 1.4) / (1.055 * 255.0);
  }
  cudaMemcpyToSymbolAsync(c_lin8, lin8, sizeof lin8, 0, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyToSymbolAsync(c_dlin8, dlin8, sizeof dlin8, 0, cudaMemcpyHostToDevice, ctx->stream);
  // pyramid of both images (linear)
  struct Sc {
    int w, h;
    long long n, off;
  };
  std::vector<Sc> sc;
  long long total = 0;
  for (int s = 0, sw = w, sh = h; s < kMaxScales && sw >= kMinSide && sh >= kMinSide; s++) {
    sc.push_back({sw, sh, (long long)sw * sh, total});
    total += 3LL * sw * sh;
    sw = (sw + 1) / 2;
    sh = (sh + 1) / 2;
  }
  const int ns = (int)sc.size();
  if (ns == 0) return fail(ctx, RCG_INVALID, "SSIMULACRA 2 needs at least 8x8 pixels");
  const long long n0 = sc[0].n;
  T* pa = ws("pa", total);
  T* pb = ws("pb", total);
  T* xa = ws("xa", 3 * n0);
  T* xb = ws("xb", 3 * n0);
  T* hb5 = ws("hb5", 5 * n0);  // row-blurred products (forward), column-blurred gradients (backward)
  T* mom = ws("mom", 5 * n0);
  T* gq = ws("gq", 3 * n0);  // g_m2, g_s22, g_s12
  T* tq = ws("tq", 3 * n0);  // their blur adjoints
  T* gx = ws("gx", 3 * n0);  // d score / d xb
  T* gl = ws("gl", total);   // d score / d linear, per scale
  double* sums = (double*)workspace(ctx, (pfx + "sums").c_str(), sizeof(double) * kMaxScales * 18);
  double* parts = (double*)workspace(ctx, (pfx + "parts").c_str(), sizeof(double) * 6 * grid_of(n0));
  if (!pa || !pb || !xa || !xb || !hb5 || !mom || !gq || !tq || !gx || !gl || !sums || !parts)
    return RCG_NO_MEMORY;
  RCG_LAUNCH(ctx, "adj_lin", k_lin<T>, grid_of(n0), 256, 0, d_ref, d_dist, n0, pa, pb);
  for (int s = 1; s < ns; s++) {
    RCG_LAUNCH(ctx, "adj_down", k_down<T>, grid_rows(sc[s].w, sc[s].h, 3), 256, 0, pa + sc[s - 1].off, sc[s - 1].w,
               sc[s - 1].h, pa + sc[s].off, sc[s].w, sc[s].h);
    RCG_LAUNCH(ctx, "adj_down", k_down<T>, grid_rows(sc[s].w, sc[s].h, 3), 256, 0, pb + sc[s - 1].off, sc[s - 1].w,
               sc[s - 1].h, pb + sc[s].off, sc[s].w, sc[s].h);
  }
  // forward: the moments and map sums of every scale
  auto moments = [&](int s, int c) {
    const long long n = sc[s].n;
    RCG_LAUNCH(ctx, "adj_hblur5", k_hblur5<T>, grid_row_runs(sc[s].w, sc[s].h, 1), 256, 0, xa + c * n, xb + c * n,
               sc[s].w, sc[s].h, hb5);
    RCG_LAUNCH(ctx, "adj_vblur", k_vblur_n<T>, grid_rows(sc[s].w, (sc[s].h + kRunN - 1) / kRunN, 5), 256, 0, hb5,
               sc[s].w, sc[s].h, mom);
  };
  for (int s = 0; s < ns; s++) {
    const long long n = sc[s].n;
    RCG_LAUNCH(ctx, "adj_xyb", k_xyb<T>, grid_of(n), 256, 0, pa + sc[s].off, n, xa);
    RCG_LAUNCH(ctx, "adj_xyb", k_xyb<T>, grid_of(n), 256, 0, pb + sc[s].off, n, xb);
    for (int c = 0; c < 3; c++) {
      moments(s, c);
      RCG_LAUNCH(ctx, "adj_maps", k_maps<T>, grid_of(n), 256, 0, mom, xa + c * n, xb + c * n, n, parts);
      RCG_LAUNCH(ctx, "adj_sum_parts", k_sum_parts, 1, 192, 0, parts, (int)grid_of(n), sums + s * 18 + c * 6);
    }
  }
  double hs[kMaxScales * 18];
  cudaMemcpyAsync(hs, sums, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "ssimulacra2 gradient");
  // final mapping (:491-511) and d score / d stat
  double st[kMaxScales][3][6], wst[kMaxScales][3][6];
  for (int s = 0; s < ns; s++) {
    const double count = (double)sc[s].n;
    for (int c = 0; c < 3; c++)
      for (int m = 0; m < 3; m++) {
        st[s][c][2 * m] = hs[s * 18 + c * 6 + 2 * m] / count;
        st[s][c][2 * m + 1] = std::pow(hs[s * 18 + c * 6 + 2 * m + 1] / count, 0.25);
      }
  }
  const double* W = scorer_weights();
  double wsum = 0.0;
  int i = 0;
  for (int c = 0; c < 3; c++)
    for (int s = 0; s < ns; s++)
      for (int nrm = 0; nrm < 2; nrm++)
        for (int m = 0; m < 3; m++) {
          wst[s][c][2 * m + nrm] = W[i];
          wsum += W[i] * std::fabs(st[s][c][2 * m + nrm]);
          i++;
        }
  const double kq = 0.9562382616834844, q = wsum * kq;
  const double P = 2.326765642916932 * q - 0.020884521182843837 * q * q + 6.248496625763138e-05 * q * q * q;
  const double ex = 0.6276336467831387;
  *score = P > 0.0 ? 100.0 - 10.0 * std::pow(P, ex) : 100.0;
  const long long npx = (long long)w * h;
  if (!d_grad) return RCG_OK;  // the score alone
  if (!(P > 0.0)) {
    cudaMemsetAsync(d_grad, 0, sizeof(double) * 3 * npx, ctx->stream);
    return RCG_OK;
  }
  const double dsum = -10.0 * ex * std::pow(P, ex - 1.0) *
                      (2.326765642916932 - 2.0 * 0.020884521182843837 * q + 3.0 * 6.248496625763138e-05 * q * q) *
                      kq;
  // backward, coarsest scale first
  for (int s = ns - 1; s >= 0; s--) {
    const long long n = sc[s].n;
    const double count = (double)n;
    RCG_LAUNCH(ctx, "adj_xyb", k_xyb<T>, grid_of(n), 256, 0, pa + sc[s].off, n, xa);
    RCG_LAUNCH(ctx, "adj_xyb", k_xyb<T>, grid_of(n), 256, 0, pb + sc[s].off, n, xb);
    for (int c = 0; c < 3; c++) {
      NormCoef nc;
      for (int m = 0; m < 3; m++) {
        nc.g1[m] = dsum * wst[s][c][2 * m] / count;
        const double mean4 = hs[s * 18 + c * 6 + 2 * m + 1] / count;
        nc.g4[m] = mean4 > 0.0 ? dsum * wst[s][c][2 * m + 1] * std::pow(mean4, -0.75) / count : 0.0;
      }
      moments(s, c);  // recomputed, not stored
      RCG_LAUNCH(ctx, "adj_mapgrad", k_mapgrad<T>, grid_of(n), 256, 0, mom, xa + c * n, xb + c * n, n, nc, gq,
                 gq + n, gq + 2 * n, gx + c * n);
      // the three gradient planes through the transposed column blur, then the row blur (its own transpose)
      RCG_LAUNCH(ctx, "adj_vblur_t", k_vblur_t<T>, grid_rows(sc[s].w, (sc[s].h + kRun - 1) / kRun, 3), 256, 0, gq,
                 sc[s].w, sc[s].h, hb5);
      RCG_LAUNCH(ctx, "adj_hblur", k_hblur<T>, grid_row_runs(sc[s].w, sc[s].h, 3), 256, 0, hb5, sc[s].w, sc[s].h, tq);
      RCG_LAUNCH(ctx, "adj_combine", k_combine<T>, grid_of(n), 256, 0, tq, tq + n, tq + 2 * n, xa + c * n,
                 xb + c * n, n, gx + c * n);
    }
    RCG_LAUNCH(ctx, "adj_xyb_adj", k_xyb_adj<T>, grid_of(n), 256, 0, pb + sc[s].off, gx, sc[s].w, sc[s].h,
               s + 1 < ns ? gl + sc[s + 1].off : nullptr, s + 1 < ns ? sc[s + 1].w : 0, gl + sc[s].off);
  }
  RCG_LAUNCH(ctx, "adj_out", k_grad_out<T>, grid_of(npx), 256, 0, gl + sc[0].off, d_dist, npx, d_grad);
  return RCG_OK;
}

}  // namespace

int ssim2_grad_device(rcg_ctx* ctx, const uint8_t* d_ref, const float* d_dist, int w, int h, double* score,
                      double* d_grad, bool fp32) {
  return fp32 ? grad_impl<float>(ctx, d_ref, d_dist, w, h, score, d_grad)
              : grad_impl<double>(ctx, d_ref, d_dist, w, h, score, d_grad);
}

}  // namespace rcg
