// JPEG encoder and decoder kernels of the quality search (K1-K7).
//
// Bit-exactness: every f32 operation the reference performs is written as an explicit round-to-nearest intrinsic
// (__fadd_rn, __fsub_rn, __fmul_rn, __fdiv_rn) in the reference's order, so no FMA contraction can change a result
// (rustc never contracts). The translation unit is also compiled with -fmad=false as a second guard. Integer steps
// (colour conversion, subsampling, upsampling, histograms) are exact by construction.
//
// Layouts in HBM:
//   padded planes      u8, row-major, stride = padded width (the MCU-padded grid of jpeg/src/encode.rs:440-443)
//   FDCT cache         f32, [64][nblocks] per component: zigzag coefficient k of block b at k*nblocks + b, so a
//                      thread-per-block kernel reads one coalesced row per coefficient. Quality-independent: the
//                      reference recomputes it for every candidate (jpeg/src/encode.rs:189-196).
//   coefficients       i16, the flat CoefImage: components back to back, 64 zigzag values per block.
//   decoded planes     u8, one per component, stride blocks_w*8 (jpeg/src/decode.rs:1322-1323).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>

#include "rcg_internal.cuh"
#include "huffman.cuh"
#include "upsample420.cuh"

namespace rcg {

// ------------------------------------------------------------------------------------------------ tables

// jpeg/src/lib.rs:14-19
__host__ __device__ inline int zigzag(int k) {
  constexpr int Z[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                         41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                         30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
  return Z[k];
}

// jpeg/src/dct.rs:8 (AAN scale factors)
__host__ __device__ inline float aan(int i) {
  constexpr float A[8] = {1.0f, 1.3870398f, 1.306563f, 1.1758756f, 1.0f, 0.78569495f, 0.5411961f, 0.27589938f};
  return A[i];
}

// jpeg/src/quality.rs:26-35
__host__ __device__ inline uint8_t perceptual_q(int i) {
  constexpr uint8_t P[64] = {16, 16, 16,  18,  25,  37,  56,  85,  16, 17, 20,  27,  34,  40,  53,  75,
                             16, 20, 24,  31,  43,  62,  91,  135, 18, 27, 31,  40,  53,  74,  106, 156,
                             25, 34, 43,  53,  69,  94,  131, 189, 37, 40, 62,  74,  94,  124, 169, 238,
                             56, 53, 91,  106, 131, 169, 226, 255, 85, 75, 135, 156, 189, 238, 255, 255};
  return P[i];
}

// Exact f32 arithmetic on host and device: round-to-nearest, never contracted.
__host__ __device__ inline float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  volatile float r = a + b;
  return r;
#endif
}
__host__ __device__ inline float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}
__host__ __device__ inline float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  volatile float r = a * b;
  return r;
#endif
}
__host__ __device__ inline float fdiv(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdiv_rn(a, b);
#else
  volatile float r = a / b;
  return r;
#endif
}

// jpeg/src/dct.rs:125-129: round half to even for |x| < 2^22; wrapping integer arithmetic beyond, as the reference.
__device__ __forceinline__ int round_f32(float x) {
  return (int)((unsigned)__float_as_int(__fadd_rn(x, 12582912.0f)) - 0x4B400000u);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

// Sampling factors build_coefs chooses (jpeg/src/encode.rs:428-439).
__host__ __device__ inline void sampling(int channels, int subsampling, int quality, int* hmax, int* vmax) {
  if (channels == 1) {
    *hmax = 1;
    *vmax = 1;
    return;
  }
  switch (subsampling) {
    case RCG_SUB_420: *hmax = 2; *vmax = 2; break;
    case RCG_SUB_422: *hmax = 2; *vmax = 1; break;
    case RCG_SUB_444: *hmax = 1; *vmax = 1; break;
    default:
      if (quality < 90) { *hmax = 2; *vmax = 2; } else { *hmax = 1; *vmax = 1; }
  }
}

// FDCT cache slot of a component for a sampling layout: 3 caches (Y, Cb, Cr) per layout kind.
__host__ __device__ inline int layout_kind(int hmax, int vmax) { return hmax == 2 ? (vmax == 2 ? 0 : 1) : 2; }

// One entry of the per-quality tables, shared by the host (fill_step) and the device (k_step_tables) so both give
// identical bits. `q` is the quantization table (natural order).
//   quant value at natural index n (jpeg/src/quality.rs:6-15)
__host__ __device__ inline uint8_t qtable_entry(int quality, int n) {
  unsigned q = (unsigned)(quality < 1 ? 1 : (quality > 100 ? 100 : quality));
  unsigned scale = q < 50 ? 5000 / q : 200 - 2 * q;
  unsigned v = ((unsigned)perceptual_q(n) * scale + 50) / 100;
  return (uint8_t)(v < 1 ? 1 : (v > 255 ? 255 : v));
}
//   fdct divisor for zigzag position k: fdct_divisors stores 1 / (q[v*8+u] * AAN[u] * AAN[v] * 8) at [u*8+v]
//   (jpeg/src/encode.rs:174-183) and quantize_plane reads it at ZZ_T[k] = (n%8)*8 + n/8 (:202), i.e. u = n%8,
//   v = n/8, q[v*8+u] = q[n]
__host__ __device__ inline float divz_entry(const uint8_t* q, int k) {
  int n = zigzag(k);
  return fdiv(1.0f, fmul(fmul(fmul((float)q[n], aan(n % 8)), aan(n / 8)), 8.0f));
}
//   dequantization multiplier at natural index n = v*8+u: q[v*8+u] * AAN[u] * AAN[v] (jpeg/src/decode.rs:1316-1321)
__host__ __device__ inline float mult_entry(const uint8_t* q, int n) {
  return fmul(fmul((float)q[n], aan(n % 8)), aan(n / 8));
}

// Block layout of a candidate (jpeg/src/encode.rs:428-443, :511-517).
__host__ __device__ inline void fill_layout(StepDesc* st, int quality, int subsampling, int channels, int trellis,
                                            int w, int h) {
  st->quality = quality;
  st->use_trellis = (trellis && quality < 100) ? 1 : 0;
  int hmax, vmax;
  sampling(channels, subsampling, quality, &hmax, &vmax);
  st->hmax = hmax;
  st->vmax = vmax;
  int pw = (w + 8 * hmax - 1) / (8 * hmax) * 8 * hmax;
  int ph = (h + 8 * vmax - 1) / (8 * vmax) * 8 * vmax;
  st->ncomp = channels == 1 ? 1 : 3;
  long long blk = 0, poff = 0;
  int kind = layout_kind(hmax, vmax);
  for (int c = 0; c < st->ncomp; c++) {
    CompDesc& cd = st->comp[c];
    cd.h = c == 0 ? hmax : 1;
    cd.v = c == 0 ? vmax : 1;
    cd.bw = c == 0 ? pw / 8 : pw / hmax / 8;
    cd.bh = c == 0 ? ph / 8 : ph / vmax / 8;
    cd.cls = c == 0 ? 0 : 1;
    cd.cache = kind * 3 + c;
    cd.blk0 = blk;
    cd.plane_off = poff;
    blk += (long long)cd.bw * cd.bh;
    poff += (long long)cd.bw * 8 * cd.bh * 8;
  }
  st->nblocks = blk;
}

// The per-quality tables of one candidate: quantization tables (jpeg/src/quality.rs), fdct divisors
// (jpeg/src/encode.rs:174-183), dequantization multipliers (jpeg/src/decode.rs:1316-1321), the Rdo parameters that
// do not depend on the rate model (jpeg/src/rdo.rs:28-45), and the block layout (jpeg/src/encode.rs:440-517).
// Host version (single calls); k_step_tables computes the same entries in parallel on the device.
inline void fill_step(StepDesc* st, int quality, int subsampling, int channels, int trellis, int w, int h) {
  const float kappa = 0.02f;  // TRELLIS_KAPPA, jpeg/src/encode.rs:42
  fill_layout(st, quality, subsampling, channels, trellis, w, h);
  // luma_table == chroma_table (jpeg/src/quality.rs:37-43): every component gets the same entries
  for (int c = 0; c < 3; c++) {
    uint8_t* qt = st->qt[c];
    for (int n = 0; n < 64; n++) qt[n] = qtable_entry(quality, n);
    for (int k = 0; k < 64; k++) st->divz[c][k] = divz_entry(qt, k);
    for (int n = 0; n < 64; n++) st->mult[c][n] = mult_entry(qt, n);
    // Rdo::new: q per zigzag position, median of q[1..] (sorted, index 31), w = (median/q)^1, lambda.
    float sorted[63];
    for (int k = 0; k < 64; k++) st->rq[c][k] = (float)qt[zigzag(k)];
    for (int k = 1; k < 64; k++) sorted[k - 1] = st->rq[c][k];
    std::sort(sorted, sorted + 63);
    float median = sorted[31];
    st->rw[c][0] = 1.0f;
    // FREQ_WEIGHT_GAMMA is 1.0 (jpeg/src/rdo.rs:12) and pow(x, 1) == x, so w = median / q exactly.
    for (int k = 1; k < 64; k++) st->rw[c][k] = fdiv(median, st->rq[c][k]);
    st->lambda[c] = fmul(fmul(kappa, median), median);
  }
}

void fill_mult(StepDesc* st, const uint8_t* qtables, int ntables) {
  for (int c = 0; c < 3; c++) {
    const uint8_t* qt = qtables + 64 * (c == 0 || ntables < 2 ? 0 : 1);
    std::memcpy(st->qt[c], qt, 64);
    for (int n = 0; n < 64; n++) st->mult[c][n] = mult_entry(qt, n);
  }
}

float mult_entry_host(const uint8_t* q, int n) { return mult_entry(q, n); }

int zigzag_natural(int k) { return zigzag(k); }

void qtables_for(int quality, uint8_t* out128) {
  for (int n = 0; n < 64; n++) out128[n] = out128[64 + n] = qtable_entry(quality, n);
}

void host_step_tables(StepDesc* st, int quality, int subsampling, int channels, int trellis, int w, int h) {
  std::memset(st, 0, sizeof *st);
  st->active = 1;
  fill_step(st, quality, subsampling, channels, trellis, w, h);
}

struct CacheSet {
  const float* p[9];
};

// Locate the component of a global block index.
__device__ __forceinline__ int comp_of(const StepDesc* st, long long gb) {
  int c = 0;
  if (st->ncomp > 1 && gb >= st->comp[1].blk0) c = gb >= st->comp[2].blk0 ? 2 : 1;
  return c;
}

// ------------------------------------------------------------------------------------------------ K1 colour + pad

// jpeg/src/encode.rs:451-477: edge-replicated Y/Cb/Cr planes over the padded grid (Gray: Y only).
__global__ void k_color_pad(const uint8_t* __restrict__ src, int w, int h, int channels, int pw, int ph,
                            uint8_t* __restrict__ yp, uint8_t* __restrict__ cbp, uint8_t* __restrict__ crp) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= pw) return;
  for (int r = blockIdx.y; r < ph; r += gridDim.y) {
    int sr = min(r, h - 1), sx = min(x, w - 1);
    size_t o = (size_t)r * pw + x;
    if (channels == 1) {
      yp[o] = src[(size_t)sr * w + sx];
      continue;
    }
    size_t i = ((size_t)sr * w + sx) * 3;
    int rr = src[i], gg = src[i + 1], bb = src[i + 2];
    yp[o] = (uint8_t)((19595 * rr + 38470 * gg + 7471 * bb + 32768) >> 16);
    cbp[o] = (uint8_t)((-11059 * rr - 21709 * gg + 32768 * bb + (128 << 16) + 32767) >> 16);
    crp[o] = (uint8_t)((32768 * rr - 27439 * gg - 5329 * bb + (128 << 16) + 32767) >> 16);
  }
}

int color_pad(rcg_ctx* ctx, const uint8_t* d_src, int w, int h, int channels, int pw, int ph, uint8_t* d_y,
              uint8_t* d_cb, uint8_t* d_cr) {
  dim3 grid((pw + 255) / 256, std::min(ph, 65535));
  RCG_LAUNCH(ctx, "color_pad", k_color_pad, grid, 256, 0, d_src, w, h, channels, pw, ph, d_y, d_cb, d_cr);
  return RCG_OK;
}

// jpeg/src/encode.rs:478-499 (down): (sum + n/2) / n over fx*fy samples. Source stride pw, output (pw/fx)x(ph/fy).
__global__ void k_chroma_down(const uint8_t* __restrict__ p, int stride, int pw, int ph, int fx, int fy,
                              uint8_t* __restrict__ o) {
  int cw = pw / fx, ch = ph / fy;
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= cw) return;
  for (int r = blockIdx.y; r < ch; r += gridDim.y) {
    unsigned s = 0;
    for (int dy = 0; dy < fy; dy++)
      for (int dx = 0; dx < fx; dx++) s += p[(size_t)(fy * r + dy) * stride + fx * x + dx];
    unsigned n = (unsigned)(fx * fy);
    o[(size_t)r * cw + x] = (uint8_t)((s + n / 2) / n);
  }
}

int chroma_down(rcg_ctx* ctx, const uint8_t* d_src, int src_stride, int pw, int ph, int fx, int fy, uint8_t* d_dst) {
  dim3 grid((pw / fx + 255) / 256, std::min(ph / fy, 65535));
  RCG_LAUNCH(ctx, "chroma_down", k_chroma_down, grid, 256, 0, d_src, src_stride, pw, ph, fx, fy, d_dst);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ K2 FDCT cache

// jpeg/src/dct.rs:20-57 (fdct_pass) on column j of a row-major 8x8 block held in registers.
__device__ __forceinline__ void fdct_pass(float (&d)[64]) {
#pragma unroll
  for (int j = 0; j < 8; j++) {
    float d0 = d[0 * 8 + j], d1 = d[1 * 8 + j], d2 = d[2 * 8 + j], d3 = d[3 * 8 + j];
    float d4 = d[4 * 8 + j], d5 = d[5 * 8 + j], d6 = d[6 * 8 + j], d7 = d[7 * 8 + j];
    float tmp0 = fadd(d0, d7), tmp7 = fsub(d0, d7), tmp1 = fadd(d1, d6), tmp6 = fsub(d1, d6);
    float tmp2 = fadd(d2, d5), tmp5 = fsub(d2, d5), tmp3 = fadd(d3, d4), tmp4 = fsub(d3, d4);
    float tmp10 = fadd(tmp0, tmp3), tmp13 = fsub(tmp0, tmp3), tmp11 = fadd(tmp1, tmp2), tmp12 = fsub(tmp1, tmp2);
    d[0 * 8 + j] = fadd(tmp10, tmp11);
    d[4 * 8 + j] = fsub(tmp10, tmp11);
    float z1 = fmul(fadd(tmp12, tmp13), 0.70710677f);
    d[2 * 8 + j] = fadd(tmp13, z1);
    d[6 * 8 + j] = fsub(tmp13, z1);
    float t10 = fadd(tmp4, tmp5), t11 = fadd(tmp5, tmp6), t12 = fadd(tmp6, tmp7);
    float z5 = fmul(fsub(t10, t12), 0.38268343f);
    float z2 = fadd(fmul(0.5411961f, t10), z5);
    float z4 = fadd(fmul(1.306563f, t12), z5);
    float z3 = fmul(t11, 0.70710677f);
    float z11 = fadd(tmp7, z3), z13 = fsub(tmp7, z3);
    d[5 * 8 + j] = fadd(z13, z2);
    d[3 * 8 + j] = fsub(z13, z2);
    d[1 * 8 + j] = fadd(z11, z4);
    d[7 * 8 + j] = fsub(z11, z4);
  }
}

__device__ __forceinline__ void transpose8(float (&b)[64]) {
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = i + 1; j < 8; j++) {
      float t = b[i * 8 + j];
      b[i * 8 + j] = b[j * 8 + i];
      b[j * 8 + i] = t;
    }
}

// One thread per block: level shift (x - 128), FDCT (jpeg/src/dct.rs:59-65), store in zigzag order
// (flat[ZZ_T[k]], jpeg/src/encode.rs:201-211) as cache[k*nb + b].
__global__ void k_fdct_cache(const uint8_t* __restrict__ plane, int stride, int bw, int bh, float* __restrict__ cache) {
  long long nb = (long long)bw * bh;
  long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  int by = (int)(b / bw), bx = (int)(b % bw);
  float blk[64];
#pragma unroll
  for (int y = 0; y < 8; y++) {
    const uint8_t* src = plane + (size_t)(by * 8 + y) * stride + bx * 8;
    uint2 v = *reinterpret_cast<const uint2*>(src);
#pragma unroll
    for (int x = 0; x < 8; x++) {
      unsigned word = x < 4 ? v.x : v.y;
      unsigned byte = (word >> (8 * (x & 3))) & 0xFF;
      blk[y * 8 + x] = fsub((float)byte, 128.0f);
    }
  }
  fdct_pass(blk);
  transpose8(blk);
  fdct_pass(blk);
#pragma unroll
  for (int k = 0; k < 64; k++) {
    constexpr int ZT[64] = {0,  8,  1,  2,  9,  16, 24, 17, 10, 3,  4,  11, 18, 25, 32, 40, 33, 26, 19, 12, 5,  6,
                            13, 20, 27, 34, 41, 48, 56, 49, 42, 35, 28, 21, 14, 7,  15, 22, 29, 36, 43, 50, 57, 58,
                            51, 44, 37, 30, 23, 31, 38, 45, 52, 59, 60, 53, 46, 39, 47, 54, 61, 62, 55, 63};
    cache[(long long)k * nb + b] = blk[ZT[k]];
  }
}

int fdct_cache(rcg_ctx* ctx, const uint8_t* d_plane, int stride, int bw, int bh, float* d_cache) {
  long long nb = (long long)bw * bh;
  int grid = (int)((nb + 127) / 128);
  RCG_LAUNCH(ctx, "fdct_cache", k_fdct_cache, grid, 128, 0, d_plane, stride, bw, bh, d_cache);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ K3 quantize

__device__ __forceinline__ int bitlen(unsigned v) { return 32 - __clz(v); }

// Plain quantization (jpeg/src/encode.rs:200-205): round_f32(flat*div) clamped to +-2047. When the candidate uses
// the trellis, the plain coefficients only feed the AC symbol histogram of the rate model (jpeg/src/encode.rs:
// 221-228, :343-374: (run<<4)|size symbols, ZRL 0xF0, EOB 0x00; luma = component 0, chroma = components 1-2);
// otherwise they are the candidate's output.
// At most 128 registers: 4 CTAs per SM instead of 3 (34 -> 30 us per 12 MP candidate, small spill).
__device__ __forceinline__ void quantize_body(StepDesc* __restrict__ st, const CacheSet& cs, long long bx) {
  __shared__ unsigned int sh[2][256];
  if (!st->active) return;
  const bool hist = st->use_trellis != 0;
  if (hist) {
    for (int i = threadIdx.x; i < 512; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
  }
  const long long gb = bx * blockDim.x + threadIdx.x;
  if (gb < st->nblocks) {
    int c = comp_of(st, gb);
    const CompDesc& cd = st->comp[c];
    const long long nb = (long long)cd.bw * cd.bh;
    const float* cache = cs.p[cd.cache] + (gb - cd.blk0);
    const float* divz = st->divz[c];
    // All 64 loads are issued before any is used (fully unrolled into registers).
    int v[64];
#pragma unroll
    for (int k = 0; k < 64; k++) v[k] = clampi(round_f32(fmul(__ldg(cache + (long long)k * nb), divz[k])), -2047, 2047);
    if (!hist) {
      int16_t* out = st->coefs + gb * 64;
#pragma unroll
      for (int g = 0; g < 8; g++) {
        int4 pk;
        pk.x = (v[g * 8 + 0] & 0xFFFF) | (v[g * 8 + 1] << 16);
        pk.y = (v[g * 8 + 2] & 0xFFFF) | (v[g * 8 + 3] << 16);
        pk.z = (v[g * 8 + 4] & 0xFFFF) | (v[g * 8 + 5] << 16);
        pk.w = (v[g * 8 + 6] & 0xFFFF) | (v[g * 8 + 7] << 16);
        reinterpret_cast<int4*>(out)[g] = pk;
      }
    } else {
      unsigned* hs = sh[cd.cls];
      unsigned run = 0;
#pragma unroll
      for (int k = 1; k < 64; k++) {
        if (v[k] == 0) {
          run++;
          continue;
        }
        while (run >= 16) {
          atomicAdd(&hs[0xF0], 1u);
          run -= 16;
        }
        unsigned size = (unsigned)bitlen((unsigned)abs(v[k]));
        atomicAdd(&hs[(run << 4) | size], 1u);
        run = 0;
      }
      if (run > 0) atomicAdd(&hs[0], 1u);
    }
  }
  if (hist) {
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x) {
      unsigned v = (&sh[0][0])[i];
      if (v) atomicAdd(&(&st->hist[0][0])[i], v);
    }
  }
}

__global__ void __launch_bounds__(128, 4) k_quantize(StepDesc* __restrict__ st, CacheSet cs) {
  quantize_body(st, cs, blockIdx.x);
}

int quantize(rcg_ctx* ctx, StepDesc* d_step, const float* const* d_caches, long long max_blocks) {
  CacheSet cs;
  for (int i = 0; i < 9; i++) cs.p[i] = d_caches[i];
  int grid = (int)((max_blocks + 127) / 128);
  RCG_LAUNCH(ctx, "quantize", k_quantize, grid, 128, 0, d_step, cs);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ K4 rate model

// Code lengths of the measured AC statistics (huff_lengths: build_lengths over the 256 symbols plus optimal_table's
// dummy), then optimal_table's sizes (jpeg/src/encode.rs:245-262), Rdo's code-length table (jpeg/src/rdo.rs:36-39)
// and the lambda*rate table (jpeg/src/rdo.rs:47-52). One CTA per component.
__device__ __forceinline__ void rate_tables_body(StepDesc* __restrict__ st, const int comp) {
  __shared__ unsigned freq[kHuffSyms];
  __shared__ unsigned char lens[kHuffSyms];
  __shared__ HuffScratch scratch;
  __shared__ float len[256];
  if (!st->active || !st->use_trellis) return;
  // the rate model is per class, lambda per component
  if (comp >= st->ncomp) return;
  const int cls = comp < 1 ? comp : 1;
  const int t = threadIdx.x;
  if (t < kHuffSyms) freq[t] = t < 256 ? st->hist[cls][t] : 1u;
  huff_lengths(freq, lens, scratch);
  // optimal_table sizes of the 256 real symbols; an empty table gets symbol 0 at length 1. Rdo: 0 -> 18 bits.
  if (t < 256) {
    bool any = false;
    for (int s = 0; s < 256; s++) any |= lens[s] > 0;
    unsigned size = lens[t];
    if (!any && t == 0) size = 1;
    len[t] = size == 0 ? 18.0f : (float)size;
  }
  __syncthreads();
  const float lambda = st->lambda[comp];
  // rate(run, v) = zrl * len[0xF0] + len[((run % 16) << 4) | size] + size, for size = bit length of v.
  for (int i = t; i < 64 * 16; i += blockDim.x) {
    int run = i / 16, size = i % 16;
    float rate = fadd(fadd(fmul((float)(run / 16), len[0xF0]), len[((run % 16) << 4) | size]), (float)size);
    st->lr[comp][i] = fmul(lambda, rate);
  }
  if (t == 0) st->eob[comp] = fmul(lambda, len[0]);
}

__global__ void __launch_bounds__(288) k_rate_tables(StepDesc* __restrict__ st) { rate_tables_body(st, blockIdx.x); }

int rate_tables(rcg_ctx* ctx, StepDesc* d_step) {
  RCG_LAUNCH(ctx, "rate_tables", k_rate_tables, 3, 288, 0, d_step);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ K5 trellis

// Rdo::quantize_ac (jpeg/src/rdo.rs:54-119) for one block per thread, plus the DC rounding of the trellis pass
// (jpeg/src/encode.rs:206-214). Same candidates, costs, evaluation order and strict `<` tie rule as the reference;
// both candidate values of a position scan the earlier nodes in one pass (neither sees the other: the reference
// skips nodes at the same position, :86-88). zd[i-1] is carried as a running sum, and each node keeps zd at its
// own position, so no 64-entry zd table is needed.
// kWeighted: the perceptual mode. Each coefficient's distortion weight becomes rw[k] * pweights[block][k] (one f32
// product, then the same squared-error product as the plain weight); the plain instantiation reads no weights.
// 8 CTAs per SM (64 registers; the weighted instantiation spills 8 bytes and is still faster, 20.9 against 24.1 us
// per candidate of a 3 MP perceptual search). The DP is latency-bound (one block's positions are serial); measured per
// 12 MP candidate: 16-coefficient chunks at 6 CTAs per SM 75.6 us, 8-coefficient chunks at 8 CTAs 72.1 us. A rolled
// DP loop over cp.async-staged shared-memory coefficients, (cost, zd) node pairs and an unrolled node scan were all
// slower or no faster (80-92, 74.2 and 72.3-76.6 us). So was a work-list: at the qualities a search visits most
// blocks have no position with a candidate (72% at q74, 96% at q62, yet only 3% of 32-block warps are all such
// blocks), so the quantize kernel wrote those blocks' results (DC only) and listed the rest for the trellis: the
// trellis went 70 -> 61 us but the quantize kernel 29 -> 40 us (the extra test per coefficient and the writes it
// took over); listing the blocks in buckets by their count of candidates, heaviest first, scattered each warp's
// blocks and cost 78 + 41 us. Sorting each CTA's blocks by that count, heaviest first, after a counting pass (the
// DC-only blocks written there) gave the same 70.6 us: the cost is the per-position work every lane runs, not the
// lanes that wait for a heavy neighbour. Cutting that work did help: each position's scale, step and weight are one
// 16-byte shared-memory entry, and a node keeps its value with its sign instead of a 64-bit sign mask updated at
// every position: 70.7 -> 66.8 us, the same coefficients. The pass then waits on its coefficient loads, yet deeper
// prefetches measured slower: two chunks ahead 68.5 us, 16-position chunks 71.2 us (7 CTAs per SM), two or three
// chunks staged ahead in shared memory by 4-byte cp.async copies 79-81 us.
template <bool kWeighted>
__device__ __forceinline__ void trellis_body(StepDesc* __restrict__ st, const CacheSet& cs, long long bx) {
  // The per-position tables of every component and the lambda*rate tables of the components this CTA's blocks
  // belong to (usually one), staged in shared memory: the DP reads them at every position.
  __shared__ float lr[3][64 * 16];
  __shared__ float4 s_tab[3][64];  // per position: (scale, step, weight, -)
  if (!st->active || !st->use_trellis) return;
  const bool requant = st->requant != 0;
  const long long blk0 = bx * blockDim.x;
  const int c_lo = comp_of(st, blk0), c_hi = comp_of(st, min(blk0 + (long long)blockDim.x, st->nblocks) - 1);
  for (int i = threadIdx.x; i < (c_hi - c_lo + 1) * 64 * 16; i += blockDim.x)
    (&lr[c_lo][0])[i] = (&st->lr[c_lo][0])[i];
  for (int i = threadIdx.x; i < 3 * 64; i += blockDim.x) {
    const int c = i / 64, k = i % 64;
    s_tab[c][k] = make_float4(requant ? st->ratio[c][k] : st->divz[c][k], st->rq[c][k], st->rw[c][k], 0.0f);
  }
  __syncthreads();
  const long long gb = blk0 + threadIdx.x;
  if (gb >= st->nblocks) return;
  const int c = comp_of(st, gb);
  const CompDesc& cd = st->comp[c];
  const long long nb = (long long)cd.bw * cd.bh;
  // Encoding: a[k] = flat[ZZ_T[k]] * div[ZZ_T[k]] from the FDCT cache (jpeg/src/encode.rs:207-211).
  // Requantization: a[k] = source[k] * ratio[k] (jpeg/src/encode.rs:162-166); the DC stays the plain value.
  const float* cache = requant ? nullptr : cs.p[cd.cache] + (gb - cd.blk0);
  const int16_t* src = requant ? st->coef_src + gb * 64 : nullptr;
  const float4* tab = s_tab[c];
  const float* lrc = lr[c];
  const float* pw = kWeighted ? st->pweights + gb * 64 : nullptr;  // 16-byte aligned rows of 64 floats

  float ncost[128], nzd[128];
  unsigned char npos[128];
  short nv[128];
  signed char nprev[128];
  int nn = 0;
  int dc = 0;
  float zprev = 0.0f;  // zd[i-1]

  // The coefficients arrive 8 at a time: the next chunk's loads are in flight while this chunk's DP steps run.
  constexpr int kChunk = 8;
  auto load = [&](int k) -> float {
    return requant ? (float)__ldg(src + k) : __ldg(cache + (long long)k * nb);
  };
  float cur[kChunk], nxt[kChunk];
#pragma unroll
  for (int j = 0; j < kChunk; j++) cur[j] = load(j);
#pragma unroll 1
  for (int c0 = 0; c0 < 64; c0 += kChunk) {
    if (c0 + kChunk < 64) {
#pragma unroll
      for (int j = 0; j < kChunk; j++) nxt[j] = load(c0 + kChunk + j);
    }
    float wv[kChunk];
    if constexpr (kWeighted) {
      const float4* p4 = reinterpret_cast<const float4*>(pw + c0);
#pragma unroll
      for (int g = 0; g < kChunk / 4; g++) {
        const float4 v = __ldg(p4 + g);
        wv[4 * g] = v.x;
        wv[4 * g + 1] = v.y;
        wv[4 * g + 2] = v.z;
        wv[4 * g + 3] = v.w;
      }
    }
#pragma unroll
    for (int j = 0; j < kChunk; j++) {
      const int i = c0 + j;
      const float4 tb = tab[i];
      float a = fmul(cur[j], tb.x);
      if (i == 0) {
        dc = clampi(round_f32(a), -2047, 2047);
        continue;
      }
      float q = tb.y, w = kWeighted ? fmul(tb.z, wv[j]) : tb.z;
      const bool neg = a < 0.0f;  // a node keeps its value with this sign
      float m = fabsf(a);
      unsigned v0 = (unsigned)fadd(m, 0.5f);
      int pushed = 0;
      if (v0 != 0) {
        unsigned lo = v0 > 1 ? v0 - 1 : v0;
        bool two = lo != v0;
        // candidate lo (first) and v0 (second, if distinct)
        float e_lo = fmul(fsub(m, (float)lo), q);
        float dnz_lo = fmul(fmul(e_lo, e_lo), w);
        float e_hi = fmul(fsub(m, (float)v0), q);
        float dnz_hi = fmul(fmul(e_hi, e_hi), w);
        int s_lo = bitlen(lo), s_hi = bitlen(v0);
        float best_lo = fadd(fadd(zprev, lrc[(i - 1) * 16 + s_lo]), dnz_lo);
        float best_hi = fadd(fadd(zprev, lrc[(i - 1) * 16 + s_hi]), dnz_hi);
        int prev_lo = -1, prev_hi = -1;
        for (int ni = 0; ni < nn; ni++) {
          float base = fadd(ncost[ni], fsub(zprev, nzd[ni]));
          int ridx = (i - npos[ni] - 1) * 16;
          float c_lo = fadd(fadd(base, lrc[ridx + s_lo]), dnz_lo);
          float c_hi = fadd(fadd(base, lrc[ridx + s_hi]), dnz_hi);
          if (c_lo < best_lo) {
            best_lo = c_lo;
            prev_lo = ni;
          }
          if (c_hi < best_hi) {
            best_hi = c_hi;
            prev_hi = ni;
          }
        }
        ncost[nn] = best_lo;
        npos[nn] = (unsigned char)i;
        nv[nn] = (short)(neg ? -(int)lo : (int)lo);
        nprev[nn] = (signed char)prev_lo;
        nn++;
        pushed = 1;
        if (two) {
          ncost[nn] = best_hi;
          npos[nn] = (unsigned char)i;
          nv[nn] = (short)(neg ? -(int)v0 : (int)v0);
          nprev[nn] = (signed char)prev_hi;
          nn++;
          pushed = 2;
        }
      }
      // zd[i] = zd[i-1] + (a*q)^2 * w; a node at position i keeps zd[i] (the reference reads zd[n.pos]).
      float e = fmul(a, q);
      float zcur = fadd(zprev, fmul(fmul(e, e), w));
      if (pushed >= 1) nzd[nn - 1] = zcur;
      if (pushed == 2) nzd[nn - 2] = zcur;
      zprev = zcur;
    }
#pragma unroll
    for (int j = 0; j < kChunk; j++) cur[j] = nxt[j];
  }
  // End of block (jpeg/src/rdo.rs:98-108): zprev is zd[63].
  const float eob = st->eob[c];
  float best_cost = fadd(zprev, eob);
  int best_end = -1;
  for (int ni = 0; ni < nn; ni++) {
    float cst = fadd(fadd(ncost[ni], fsub(zprev, nzd[ni])), npos[ni] < 63 ? eob : 0.0f);
    if (cst < best_cost) {
      best_cost = cst;
      best_end = ni;
    }
  }
  int16_t* out = st->coefs + gb * 64;
  int4 z = make_int4(0, 0, 0, 0);
  int4 first = z;
  // quantize_ac clears positions 1..63 (jpeg/src/rdo.rs:109-111); the DC is the rounded a[0] when encoding and the
  // plain requantized value (already in place) when requantizing.
  first.x = requant ? (reinterpret_cast<const int4*>(out)[0].x & 0xFFFF) : (dc & 0xFFFF);
  reinterpret_cast<int4*>(out)[0] = first;
#pragma unroll
  for (int g = 1; g < 8; g++) reinterpret_cast<int4*>(out)[g] = z;
  int node = best_end;
  while (node >= 0) {
    int p = npos[node];
    short v = nv[node];
    out[p] = (int16_t)v;
    node = nprev[node];
  }
}

template <bool kWeighted>
__global__ void __launch_bounds__(128, 8) k_trellis(StepDesc* __restrict__ st, CacheSet cs) {
  trellis_body<kWeighted>(st, cs, blockIdx.x);
}

int trellis(rcg_ctx* ctx, StepDesc* d_step, const float* const* d_caches, long long max_blocks, bool weighted) {
  CacheSet cs;
  for (int i = 0; i < 9; i++) cs.p[i] = d_caches ? d_caches[i] : nullptr;
  int grid = (int)((max_blocks + 127) / 128);
  if (weighted)
    RCG_LAUNCH(ctx, "trellis_weighted", k_trellis<true>, grid, 128, 0, d_step, cs);
  else
    RCG_LAUNCH(ctx, "trellis", k_trellis<false>, grid, 128, 0, d_step, cs);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ K6 IDCT

// jpeg/src/dct.rs:67-109 (idct_pass)
__device__ __forceinline__ void idct_pass(float (&d)[64]) {
  const float SQRT_2 = 1.41421356237309504880f;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    float tmp0 = d[0 * 8 + j], tmp1 = d[2 * 8 + j], tmp2 = d[4 * 8 + j], tmp3 = d[6 * 8 + j];
    float tmp10 = fadd(tmp0, tmp2), tmp11 = fsub(tmp0, tmp2), tmp13 = fadd(tmp1, tmp3);
    float tmp12 = fsub(fmul(fsub(tmp1, tmp3), SQRT_2), tmp13);
    float e0 = fadd(tmp10, tmp13), e3 = fsub(tmp10, tmp13), e1 = fadd(tmp11, tmp12), e2 = fsub(tmp11, tmp12);
    float tmp4 = d[1 * 8 + j], tmp5 = d[3 * 8 + j], tmp6 = d[5 * 8 + j], tmp7 = d[7 * 8 + j];
    float z13 = fadd(tmp6, tmp5), z10 = fsub(tmp6, tmp5), z11 = fadd(tmp4, tmp7), z12 = fsub(tmp4, tmp7);
    float o7 = fadd(z11, z13);
    float o11 = fmul(fsub(z11, z13), SQRT_2);
    float z5 = fmul(fadd(z10, z12), 1.8477591f);
    float o10 = fsub(fmul(1.0823922f, z12), z5);
    float o12 = fadd(fmul(-2.613126f, z10), z5);
    float o6 = fsub(o12, o7);
    float o5 = fsub(o11, o6);
    float o4 = fadd(o10, o5);
    d[0 * 8 + j] = fadd(e0, o7);
    d[7 * 8 + j] = fsub(e0, o7);
    d[1 * 8 + j] = fadd(e1, o6);
    d[6 * 8 + j] = fsub(e1, o6);
    d[2 * 8 + j] = fadd(e2, o5);
    d[5 * 8 + j] = fsub(e2, o5);
    d[4 * 8 + j] = fadd(e3, o4);
    d[3 * 8 + j] = fsub(e3, o4);
  }
}

// idct_planes (jpeg/src/decode.rs:1310-1343): dequantize into natural order, IDCT (jpeg/src/dct.rs:111-123),
// round_f32 + 128 clamped to 0..255. One thread per block.
__device__ __forceinline__ void dequant_idct_body(const StepDesc* __restrict__ st, const int16_t* __restrict__ coefs,
                                                  uint8_t* __restrict__ planes, long long cta) {
  if (!st->active) return;
  long long gb = cta * blockDim.x + threadIdx.x;
  if (gb >= st->nblocks) return;
  int c = comp_of(st, gb);
  const CompDesc& cd = st->comp[c];
  long long lb = gb - cd.blk0;
  int by = (int)(lb / cd.bw), bx = (int)(lb % cd.bw);
  const float* mult = st->mult[c];
  float blk[64];
  const int16_t* base = coefs ? coefs : st->coefs;
  const int4* src = reinterpret_cast<const int4*>(base + gb * 64);
#pragma unroll
  for (int g = 0; g < 8; g++) {
    int4 pk = src[g];
    int w4[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
    for (int j = 0; j < 8; j++) {
      int k = g * 8 + j;
      int v = (int)(short)((w4[j >> 1] >> (16 * (j & 1))) & 0xFFFF);
      int n = zigzag(k);
      blk[n] = fmul((float)v, mult[n]);
    }
  }
  idct_pass(blk);
  transpose8(blk);
  idct_pass(blk);
  transpose8(blk);
  int stride = cd.bw * 8;
  uint8_t* dst = planes + cd.plane_off + (size_t)(by * 8) * stride + bx * 8;
#pragma unroll
  for (int y = 0; y < 8; y++) {
    unsigned lo = 0, hi = 0;
#pragma unroll
    for (int x = 0; x < 8; x++) {
      unsigned p = (unsigned)clampi(round_f32(fmul(blk[y * 8 + x], 0.125f)) + 128, 0, 255);
      if (x < 4)
        lo |= p << (8 * x);
      else
        hi |= p << (8 * (x - 4));
    }
    *reinterpret_cast<uint2*>(dst + (size_t)y * stride) = make_uint2(lo, hi);
  }
}

__global__ void __launch_bounds__(128) k_dequant_idct(const StepDesc* __restrict__ st,
                                                     const int16_t* __restrict__ coefs, uint8_t* __restrict__ planes) {
  dequant_idct_body(st, coefs, planes, blockIdx.x);
}

int dequant_idct(rcg_ctx* ctx, StepDesc* d_step, const int16_t* d_coefs, uint8_t* d_planes, long long max_blocks) {
  int grid = (int)((max_blocks + 127) / 128);
  RCG_LAUNCH(ctx, "dequant_idct", k_dequant_idct, grid, 128, 0, d_step, d_coefs, d_planes);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ K7 upsample+colour

__constant__ float c_lut8[256];

// upsample (jpeg/src/decode.rs:1768-1828) of one component sample at full-resolution (x, y).
__device__ __forceinline__ int up_sample(const uint8_t* p, int stride, int cw, int ch, int fx, int fy, int x, int y) {
  auto px = [&](int xx, int yy) -> int { return p[(size_t)yy * stride + xx]; };
  if (fx == 1 && fy == 1) return px(x, y);
  if (fx == 2 && fy == 1) {
    int i = x / 2;
    int nr = px(i, y);
    int fr = (x % 2 == 0) ? px(max(i - 1, 0), y) : px(min(i + 1, cw - 1), y);
    return (3 * nr + fr + ((x % 2 == 0) ? 1 : 2)) >> 2;
  }
  if (fx == 1 && fy == 2) {
    int j = y / 2;
    int fy_ = (y % 2 == 0) ? max(j - 1, 0) : min(j + 1, ch - 1);
    return (3 * px(x, j) + px(x, fy_) + ((y % 2 == 0) ? 1 : 2)) >> 2;
  }
  if (fx == 2 && fy == 2) {
    int j = y / 2;
    int fy_ = (y % 2 == 0) ? max(j - 1, 0) : min(j + 1, ch - 1);
    int i = x / 2;
    int fi = (x % 2 == 0) ? max(i - 1, 0) : min(i + 1, cw - 1);
    int nr = 3 * px(i, j) + px(i, fy_);
    int fr = 3 * px(fi, j) + px(fi, fy_);
    return (3 * nr + fr + ((x % 2 == 0) ? 8 : 7)) >> 4;
  }
  return px(x / fx, y / fy);
}

// The search's common case (upsample420.cuh): one thread = 4 columns x 2 rows (output rows 2j, 2j+1 of chroma row
// j), stored as one 16-byte write per row and plane. Same arithmetic as the general path below
// (jpeg/src/decode.rs:1806-1818, :1438-1441).
__device__ __forceinline__ void upsample_420(const StepDesc* __restrict__ st, const uint8_t* __restrict__ planes,
                                             int w, int h, float* __restrict__ lin, const float* lut, int x0,
                                             int j) {
  float l[2][3][4];
  upsample_420_rows(st, planes, w, h, lut, x0, j, l);
  const size_t np = (size_t)w * h;
#pragma unroll
  for (int par = 0; par < 2; par++) {
    const int y = 2 * j + par;
    if (y >= h) break;
    const size_t o = (size_t)y * w + x0;
#pragma unroll
    for (int c = 0; c < 3; c++)
      *reinterpret_cast<float4*>(lin + c * np + o) = make_float4(l[par][c][0], l[par][c][1], l[par][c][2],
                                                                 l[par][c][3]);
  }
}

// Decoder::finish for an 8-bit YCbCr or Gray CoefImage (jpeg/src/decode.rs:1404-1444): upsample every component to
// full resolution, then the fixed-point YCbCr->RGB of :1438-1441. Writes interleaved pixels and/or the linear-light
// planes the scorer starts from (core/src/ssimulacra2.rs:192-203: Gray is replicated to three channels).
// 10 CTAs per SM (48 registers) instead of 7: the kernel waits on loads, so more warps hide more of it
// (51 -> 47 us per 12 MP candidate).
__device__ __forceinline__ void upsample_color_body(const StepDesc* __restrict__ st,
                                                    const uint8_t* __restrict__ planes, int w, int h,
                                                    uint8_t* __restrict__ rgb, float* __restrict__ lin,
                                                    const unsigned bx, const unsigned by, const unsigned gy) {
  if (!st->active) return;
  const int ncomp = st->ncomp, hmax = st->hmax, vmax = st->vmax;
  const CompDesc c0 = st->comp[0];
  // 4:2:0 linear planes for the scorer: the two-row path, over chroma rows (half the grid's rows)
  const bool fast420 = !rgb && lin && layout_is_fast420(st, w);
  if (fast420 && (int)by >= (h + 1) / 2) return;
  // The sRGB table lives in shared memory: per-thread indices differ, which would serialize constant-memory reads.
  __shared__ float lut[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = c_lut8[i];
  __syncthreads();
  // Four consecutive pixels of one row per thread, so each thread moves enough bytes per request.
  const int x0 = 4 * (bx * blockDim.x + threadIdx.x);
  if (x0 >= w) return;
  if (fast420) {
    for (int j = by; j < (h + 1) / 2; j += gy) upsample_420(st, planes, w, h, lin, lut, x0, j);
    return;
  }
  const size_t np = (size_t)w * h;
  const bool vec_out = (w % 4 == 0) && (np % 4 == 0) && (x0 + 4 <= w);
  for (int y = by; y < h; y += gy) {
    int yv[4], cbv[4], crv[4];
    // Luma: full resolution when it carries the maximum sampling factors (always, for this encoder's layouts).
    if (c0.h == hmax && c0.v == vmax) {
      const uint8_t* yr = planes + c0.plane_off + (size_t)y * (c0.bw * 8);
      uint32_t q = *reinterpret_cast<const uint32_t*>(yr + x0);  // x0 % 4 == 0, row stride % 8 == 0
#pragma unroll
      for (int k = 0; k < 4; k++) yv[k] = (q >> (8 * k)) & 0xFF;
    } else {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        int x = min(x0 + k, w - 1);
        yv[k] = up_sample(planes + c0.plane_off, c0.bw * 8, (w * c0.h + hmax - 1) / hmax,
                          (h * c0.v + vmax - 1) / vmax, hmax / c0.h, vmax / c0.v, x, y);
      }
    }
    if (ncomp == 3) {
#pragma unroll
      for (int c = 1; c < 3; c++) {
        const CompDesc cd = st->comp[c];
        const uint8_t* p = planes + cd.plane_off;
        const int stride = cd.bw * 8;
        const int cw = (w * cd.h + hmax - 1) / hmax, ch = (h * cd.v + vmax - 1) / vmax;
        const int fx = hmax / cd.h, fy = vmax / cd.v;
        int* out = c == 1 ? cbv : crv;
        if (fx == 2 && fy == 2) {
          // Triangle filter of jpeg/src/decode.rs:1806-1818 for x0..x0+3 (x0 even): chroma columns i-1..i+2.
          const int j = y / 2;
          const int far_y = (y % 2 == 0) ? max(j - 1, 0) : min(j + 1, ch - 1);
          const uint8_t* rn = p + (size_t)j * stride;
          const uint8_t* rf = p + (size_t)far_y * stride;
          const int i = x0 / 2;
          int vert[4];
#pragma unroll
          for (int d = 0; d < 4; d++) {
            int col = min(max(i - 1 + d, 0), cw - 1);
            vert[d] = 3 * rn[col] + rf[col];
          }
          out[0] = (3 * vert[1] + vert[0] + 8) >> 4;  // x0 even: far = i-1
          out[1] = (3 * vert[1] + vert[2] + 7) >> 4;  // x0+1 odd: far = i+1
          out[2] = (3 * vert[2] + vert[1] + 8) >> 4;  // x0+2 even: near i+1, far i
          out[3] = (3 * vert[2] + vert[3] + 7) >> 4;  // x0+3 odd: near i+1, far i+2
          // Clamping every column to [0, cw-1] is the reference's rule (saturating i-1, min(i+1, cw-1)); a near
          // column never needs it for a pixel inside the image (x < w implies x/2 < cw).
        } else {
#pragma unroll
          for (int k = 0; k < 4; k++) out[k] = up_sample(p, stride, cw, ch, fx, fy, min(x0 + k, w - 1), y);
        }
      }
    }
    float l[3][4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (ncomp == 1) {
        l[0][k] = l[1][k] = l[2][k] = lut[yv[k]];
        if (rgb && x0 + k < w) rgb[(size_t)y * w + x0 + k] = (uint8_t)yv[k];
      } else {
        int cb = cbv[k] - 128, cr = crv[k] - 128;
        int r = clampi(yv[k] + ((91881 * cr + 32768) >> 16), 0, 255);
        int g = clampi(yv[k] - ((22554 * cb + 46802 * cr + 32768) >> 16), 0, 255);
        int b = clampi(yv[k] + ((116130 * cb + 32768) >> 16), 0, 255);
        l[0][k] = lut[r];
        l[1][k] = lut[g];
        l[2][k] = lut[b];
        if (rgb && x0 + k < w) {
          size_t i = ((size_t)y * w + x0 + k) * 3;
          rgb[i] = (uint8_t)r;
          rgb[i + 1] = (uint8_t)g;
          rgb[i + 2] = (uint8_t)b;
        }
      }
    }
    if (lin) {
      size_t i = (size_t)y * w + x0;
      if (vec_out) {
#pragma unroll
        for (int c = 0; c < 3; c++)
          *reinterpret_cast<float4*>(lin + c * np + i) = make_float4(l[c][0], l[c][1], l[c][2], l[c][3]);
      } else {
        for (int k = 0; k < 4 && x0 + k < w; k++)
#pragma unroll
          for (int c = 0; c < 3; c++) lin[c * np + i + k] = l[c][k];
      }
    }
  }
}

__global__ void __launch_bounds__(128, 10) k_upsample_color(const StepDesc* __restrict__ st,
                                                             const uint8_t* __restrict__ planes, int w, int h,
                                                             uint8_t* __restrict__ rgb, float* __restrict__ lin) {
  upsample_color_body(st, planes, w, h, rgb, lin, blockIdx.x, blockIdx.y, gridDim.y);
}

int upsample_color(rcg_ctx* ctx, StepDesc* d_step, const uint8_t* d_planes, int w, int h, uint8_t* d_rgb,
                   float* d_lin) {
  // (h + 1) / 8 rows of CTAs: the 4:2:0 path writes two rows per chroma row and each CTA takes four chroma rows (its
  // shared-memory table filled once for 8 output rows: 46.5 -> 40.7 us per 12 MP candidate against one chroma row
  // per CTA); the general path strides over the rows by the grid height, so every layout is covered.
  dim3 grid(((w + 3) / 4 + 127) / 128, std::min(((h + 1) / 2 + 3) / 4, 65535));
  RCG_LAUNCH(ctx, "upsample_color", k_upsample_color, grid, 128, 0, d_step, d_planes, w, h, d_rgb, d_lin);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ step tables

// First kernel of every search step: the bisection state names the quality; fill the candidate's tables. 192
// threads: one per (component, coefficient) entry; the Rdo median is the element of rank 31 among q[1..63] (ties
// broken by index, which leaves the value unchanged), the same value the reference's sort yields.
__device__ __forceinline__ void step_tables_body(const SearchState* __restrict__ ss, StepDesc* __restrict__ st,
                                                 int w, int h, int16_t* slots, long long slot_stride,
                                                 const float* pweights) {
  __shared__ uint8_t qt[64];
  __shared__ float rq[64];
  __shared__ float median;
  const int t = threadIdx.x;
  if (ss->done) {
    if (t == 0) st->active = 0;
    return;
  }
  const int step = ss->step;
  const int q = ss->qs[step];
  if (t == 0) {
    st->active = 1;
    st->requant = 0;
    fill_layout(st, q, ss->subsampling, ss->channels, ss->trellis, w, h);
    st->coefs = slots + (long long)step * slot_stride;
    st->pweights = pweights;
  }
  if (t < 64) qt[t] = qtable_entry(q, t);
  __syncthreads();
  // luma_table == chroma_table (jpeg/src/quality.rs:37-43): every component gets the same entries
  const int c = t / 64, k = t % 64;
  st->qt[c][k] = qt[k];
  st->divz[c][k] = divz_entry(qt, k);
  st->mult[c][k] = mult_entry(qt, k);
  float rk = (float)qt[zigzag(k)];
  st->rq[c][k] = rk;
  if (c == 0) rq[k] = rk;
  for (int i = t; i < 512; i += blockDim.x) (&st->hist[0][0])[i] = 0;
  __syncthreads();
  if (c == 0 && k >= 1) {
    int rank = 0;
    for (int j = 1; j < 64; j++) rank += (rq[j] < rk || (rq[j] == rk && j < k)) ? 1 : 0;
    if (rank == 31) median = rk;
  }
  __syncthreads();
  st->rw[c][k] = k == 0 ? 1.0f : fdiv(median, rk);
  if (k == 0) st->lambda[c] = fmul(fmul(0.02f, median), median);  // TRELLIS_KAPPA (jpeg/src/encode.rs:42)
}

__global__ void __launch_bounds__(192) k_step_tables(const SearchState* __restrict__ ss, StepDesc* __restrict__ st,
                                                     int w, int h, int16_t* slots, long long slot_stride,
                                                     const float* pweights) {
  step_tables_body(ss, st, w, h, slots, slot_stride, pweights);
}

int step_tables(rcg_ctx* ctx, SearchState* d_search, StepDesc* d_step, int w, int h, int16_t* d_coef_slots,
                long long slot_stride, const float* d_pweights) {
  RCG_LAUNCH(ctx, "step_tables", k_step_tables, 1, 192, 0, d_search, d_step, w, h, d_coef_slots, slot_stride,
             d_pweights);
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ lockstep batch

// One bisection step of every image of a lockstep batch: the same kernel bodies as one search, each launch over a
// work-list of every image's CTAs (an image whose search has finished skips through its StepDesc's `active`).
__global__ void __launch_bounds__(192) k_step_tables_lock(const LockItem* __restrict__ items) {
  const LockItem& it = items[blockIdx.x];
  step_tables_body(it.ss, it.st, it.w, it.h, it.slots, it.slot_stride, nullptr);
}

__device__ __forceinline__ CacheSet lock_caches(const LockItem& it) {
  CacheSet cs;
#pragma unroll
  for (int i = 0; i < 9; i++) cs.p[i] = it.caches[i];
  return cs;
}

__global__ void __launch_bounds__(128, 4) k_quantize_lock(const LockItem* __restrict__ items, int n) {
  const int i = lock_find<&LockItem::q0>(items, n, blockIdx.x);
  const LockItem& it = items[i];
  quantize_body(it.st, lock_caches(it), (long long)blockIdx.x - it.q0);
}

__global__ void __launch_bounds__(288) k_rate_tables_lock(const LockItem* __restrict__ items) {
  rate_tables_body(items[blockIdx.y].st, blockIdx.x);
}

__global__ void __launch_bounds__(128, 8) k_trellis_lock(const LockItem* __restrict__ items, int n) {
  const int i = lock_find<&LockItem::q0>(items, n, blockIdx.x);
  const LockItem& it = items[i];
  trellis_body<false>(it.st, lock_caches(it), (long long)blockIdx.x - it.q0);
}

__global__ void __launch_bounds__(128) k_dequant_idct_lock(const LockItem* __restrict__ items, int n) {
  const int i = lock_find<&LockItem::q0>(items, n, blockIdx.x);
  const LockItem& it = items[i];
  dequant_idct_body(it.st, nullptr, it.planes, (long long)blockIdx.x - it.q0);
}

__global__ void __launch_bounds__(128, 10) k_upsample_color_lock(const LockItem* __restrict__ items, int n) {
  const int i = lock_find<&LockItem::u0>(items, n, blockIdx.x);
  const LockItem& it = items[i];
  const long long local = (long long)blockIdx.x - it.u0;
  const unsigned bx = (unsigned)(local % it.ux), by = (unsigned)(local / it.ux);
  upsample_color_body(it.st, it.planes, it.w, it.h, nullptr, it.dist_pyr, bx, by, (unsigned)it.uy);
}

void lock_step_codec(rcg_ctx* ctx, const LockItem* d_items, int n, long long q_total, long long u_total) {
  RCG_LAUNCH(ctx, "step_tables_lock", k_step_tables_lock, n, 192, 0, d_items);
  RCG_LAUNCH(ctx, "quantize_lock", k_quantize_lock, (unsigned)q_total, 128, 0, d_items, n);
  RCG_LAUNCH(ctx, "rate_tables_lock", k_rate_tables_lock, dim3(3, n), 288, 0, d_items);
  RCG_LAUNCH(ctx, "trellis_lock", k_trellis_lock, (unsigned)q_total, 128, 0, d_items, n);
  RCG_LAUNCH(ctx, "dequant_idct_lock", k_dequant_idct_lock, (unsigned)q_total, 128, 0, d_items, n);
  RCG_LAUNCH(ctx, "upsample_color_lock", k_upsample_color_lock, (unsigned)u_total, 128, 0, d_items, n);
}

int codec_upload_lut(const float* lut8) {
  cudaError_t e = cudaMemcpyToSymbol(c_lut8, lut8, 256 * sizeof(float));
  return e == cudaSuccess ? 0 : (int)e;
}

// ------------------------------------------------------------------------------------------------ requantization

// Table of one component for a requantization to `quality` (jpeg/src/encode.rs:121-126): the quality's table,
// never finer than the source's.
__host__ __device__ inline uint8_t requant_entry(const uint8_t* old, int quality, int n) {
  uint8_t t = qtable_entry(quality, n);
  return t > old[n] ? t : old[n];
}

// Slot assignment of jpeg/src/encode.rs:139-148: components with equal tables share a slot, a new table takes the
// first free one. Also reports whether any table changed (:127) and the slot tables.
__host__ __device__ inline int requant_slots(const StepDesc* st, int* tq, uint8_t (*slot_qt)[64], int* present) {
  int changed = 0;
  for (int sl = 0; sl < 4; sl++) present[sl] = 0;
  for (int c = 0; c < st->ncomp; c++) {
    bool same_as_old = true;
    for (int n = 0; n < 64; n++) same_as_old &= st->qt[c][n] == st->src_qt[c][n];
    changed |= same_as_old ? 0 : 1;
    int slot = -1;
    for (int sl = 0; sl < 4 && slot < 0; sl++) {
      if (!present[sl]) continue;
      bool eq = true;
      for (int n = 0; n < 64; n++) eq &= slot_qt[sl][n] == st->qt[c][n];
      if (eq) slot = sl;
    }
    if (slot < 0) {
      for (int sl = 0; sl < 4 && slot < 0; sl++)
        if (!present[sl]) slot = sl;
      for (int n = 0; n < 64; n++) slot_qt[slot][n] = st->qt[c][n];
      present[slot] = 1;
    }
    tq[c] = slot;
  }
  return changed;
}

void host_requant_tables(StepDesc* st, int quality, int trellis, int tq_out[3], uint8_t slot_qt_out[4][64],
                         int present_out[4]) {
  const float kappa = 0.02f;  // TRELLIS_KAPPA, jpeg/src/encode.rs:42
  st->quality = quality;
  st->requant = 1;
  for (int c = 0; c < st->ncomp; c++) {
    uint8_t* nt = st->qt[c];
    for (int n = 0; n < 64; n++) nt[n] = requant_entry(st->src_qt[c], quality, n);
    for (int k = 0; k < 64; k++) {
      int n = zigzag(k);
      st->ratio[c][k] = fdiv((float)st->src_qt[c][n], (float)nt[n]);
      st->rq[c][k] = (float)nt[n];
    }
    for (int n = 0; n < 64; n++) st->mult[c][n] = mult_entry(nt, n);
    float sorted[63];
    for (int k = 1; k < 64; k++) sorted[k - 1] = st->rq[c][k];
    std::sort(sorted, sorted + 63);
    float median = sorted[31];
    st->rw[c][0] = 1.0f;
    for (int k = 1; k < 64; k++) st->rw[c][k] = fdiv(median, st->rq[c][k]);
    st->lambda[c] = fmul(fmul(kappa, median), median);
  }
  st->changed = requant_slots(st, tq_out, slot_qt_out, present_out);
  st->use_trellis = (trellis && st->changed) ? 1 : 0;
  std::memset(st->hist, 0, sizeof st->hist);
}

// Search step of the JPEG->JPEG search: the same tables as host_requant_tables, 192 threads (component,
// coefficient); each component's Rdo median is the element of rank 31 among its q[1..63].
__global__ void __launch_bounds__(192) k_step_tables_rq(const SearchState* __restrict__ ss, StepDesc* __restrict__ st,
                                                        int16_t* slots, long long slot_stride) {
  __shared__ float rq[3][64];
  __shared__ float median[3];
  const int t = threadIdx.x;
  if (ss->done) {
    if (t == 0) st->active = 0;
    return;
  }
  const int step = ss->step;
  const int q = ss->qs[step];
  const int c = t / 64, k = t % 64;
  const bool live = c < st->ncomp;
  if (live) {
    int n = zigzag(k);
    uint8_t nn = requant_entry(st->src_qt[c], q, n);
    st->qt[c][n] = nn;
    st->ratio[c][k] = fdiv((float)st->src_qt[c][n], (float)nn);
    st->rq[c][k] = (float)nn;
    rq[c][k] = (float)nn;
  }
  for (int i = t; i < 512; i += blockDim.x) (&st->hist[0][0])[i] = 0;
  __syncthreads();
  if (live) {
    st->mult[c][k] = mult_entry(st->qt[c], k);
    if (k >= 1) {
      float rk = rq[c][k];
      int rank = 0;
      for (int j = 1; j < 64; j++) rank += (rq[c][j] < rk || (rq[c][j] == rk && j < k)) ? 1 : 0;
      if (rank == 31) median[c] = rk;
    }
  }
  __syncthreads();
  if (live) {
    st->rw[c][k] = k == 0 ? 1.0f : fdiv(median[c], rq[c][k]);
    if (k == 0) st->lambda[c] = fmul(fmul(0.02f, median[c]), median[c]);
  }
  if (t == 0) {
    int tq[3];
    uint8_t slot_qt[4][64];
    int present[4];
    st->active = 1;
    st->requant = 1;
    st->quality = q;
    st->changed = requant_slots(st, tq, slot_qt, present);
    st->use_trellis = (ss->trellis && st->changed) ? 1 : 0;
    st->coefs = slots + (long long)step * slot_stride;
  }
}

int step_tables_requant(rcg_ctx* ctx, SearchState* d_search, StepDesc* d_step, int16_t* d_coef_slots,
                        long long slot_stride) {
  RCG_LAUNCH(ctx, "step_tables", k_step_tables_rq, 1, 192, 0, d_search, d_step, d_coef_slots, slot_stride);
  return RCG_OK;
}

// Plain requantization (jpeg/src/encode.rs:132-138): round_f32(coef * old/new) clamped to +-2047, every position.
// When the trellis pass follows, also the AC symbol histogram of the result over the blocks of the MCU grid
// (ac_code_lengths, :155 -> :223-227, :376-398).
__global__ void __launch_bounds__(128) k_requant_plain(StepDesc* __restrict__ st) {
  __shared__ unsigned int sh[2][256];
  if (!st->active) return;
  const bool hist = st->use_trellis != 0;
  if (hist) {
    for (int i = threadIdx.x; i < 512; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
  }
  const long long gb = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gb < st->nblocks) {
    const int c = comp_of(st, gb);
    const CompDesc& cd = st->comp[c];
    const float* ratio = st->ratio[c];
    const int4* src = reinterpret_cast<const int4*>(st->coef_src + gb * 64);
    int v[64];
#pragma unroll
    for (int g = 0; g < 8; g++) {
      int4 pk = __ldg(src + g);
      int w4[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
      for (int j = 0; j < 8; j++) {
        int k = g * 8 + j;
        int x = (int)(short)((w4[j >> 1] >> (16 * (j & 1))) & 0xFFFF);
        v[k] = clampi(round_f32(fmul((float)x, ratio[k])), -2047, 2047);
      }
    }
    int16_t* out = st->coefs + gb * 64;
#pragma unroll
    for (int g = 0; g < 8; g++) {
      int4 pk;
      pk.x = (v[g * 8 + 0] & 0xFFFF) | (v[g * 8 + 1] << 16);
      pk.y = (v[g * 8 + 2] & 0xFFFF) | (v[g * 8 + 3] << 16);
      pk.z = (v[g * 8 + 4] & 0xFFFF) | (v[g * 8 + 5] << 16);
      pk.w = (v[g * 8 + 6] & 0xFFFF) | (v[g * 8 + 7] << 16);
      reinterpret_cast<int4*>(out)[g] = pk;
    }
    const long long lb = gb - cd.blk0;
    const int by = (int)(lb / cd.bw), bx = (int)(lb % cd.bw);
    if (hist && bx < st->mcus_x * cd.h && by < st->mcus_y * cd.v) {
      unsigned* hs = sh[cd.cls];
      unsigned run = 0;
#pragma unroll
      for (int k = 1; k < 64; k++) {
        if (v[k] == 0) {
          run++;
          continue;
        }
        while (run >= 16) {
          atomicAdd(&hs[0xF0], 1u);
          run -= 16;
        }
        unsigned size = (unsigned)bitlen((unsigned)abs(v[k]));
        atomicAdd(&hs[(run << 4) | size], 1u);
        run = 0;
      }
      if (run > 0) atomicAdd(&hs[0], 1u);
    }
  }
  if (hist) {
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x) {
      unsigned x = (&sh[0][0])[i];
      if (x) atomicAdd(&(&st->hist[0][0])[i], x);
    }
  }
}

int requantize_plain(rcg_ctx* ctx, StepDesc* d_step, long long max_blocks) {
  int grid = (int)((max_blocks + 127) / 128);
  RCG_LAUNCH(ctx, "requant_plain", k_requant_plain, grid, 128, 0, d_step);
  return RCG_OK;
}

}  // namespace rcg
