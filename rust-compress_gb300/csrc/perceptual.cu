// Perceptual trellis weights: the SSIMULACRA2 pixel gradient pulled back to the DCT coefficients.
//
// The decoder's pixels are a function of the dequantized coefficients: orthonormal 8x8 IDCT per component block
// (jpeg/src/dct.rs:67-119 computes exactly that transform, with the AAN scale folded into the multipliers of
// jpeg/src/decode.rs:1316-1321), the triangle-filter chroma upsampling of jpeg/src/decode.rs:1768-1828 (weights 3/4
// near, 1/4 far per axis, edge-clamped) and the fixed-point YCbCr->RGB of jpeg/src/decode.rs:1438-1441. Dropping the
// roundings and clamps, the adjoint of that linear map takes d score / d RGB sample to d score / d coefficient:
//   colour:    gY = gR + gG + gB,  gCb = (-22554 gG + 116130 gB) / 65536,  gCr = (91881 gR - 46802 gG) / 65536
//              (Gray: gY = gR + gG + gB, the decoder replicates Y to three channels)
//   upsample:  each chroma sample gathers 3/4 or 1/4 (or both, at a clamped edge) of the full-resolution samples it
//              feeds, per axis
//   IDCT:      G = C g C^T per block (C the orthonormal DCT-II matrix), stored in zigzag order.
// The weights: a block's sensitivity is the RMS, over its (2r+1)^2 neighbourhood of blocks (edge-replicated), of the
// coefficient-gradient energy sum_k G_k^2 (= sum of the block's squared pixel-domain gradient, Parseval); normalised
// by the component's mean sensitivity, raised to `gamma`, clamped to [w_min, w_max] and scaled by `strength`:
//   W[b][k] = strength * clamp((s_b / mean_c s)^gamma, w_min, w_max)   (all k of the block)
// The trellis multiplies its distortion weight by W (the perceptual mode); everything here runs in f64.

#include <algorithm>
#include <cmath>

#include "rcg_internal.cuh"

namespace rcg {

namespace {

struct PullComp {
  int bw, bh;    // block grid
  int fx, fy;    // upsampling factors (1 or 2)
  int cw, ch;    // component samples covering the image (jpeg/src/decode.rs:1411-1412)
  long long blk0;
};

struct PullDesc {
  int ncomp, w, h;
  long long nblocks;
  PullComp c[3];
};

__constant__ double c_dct[64];   // C[u][x] = c(u) cos((2x + 1) u pi / 16), c(0) = sqrt(1/8), c(u > 0) = 1/2
__constant__ int c_izz[64];      // natural index -> zigzag position

__device__ __forceinline__ int comp_of_block(const PullDesc& d, long long gb) {
  if (d.ncomp == 1) return 0;
  return gb >= d.c[2].blk0 ? 2 : (gb >= d.c[1].blk0 ? 1 : 0);
}

// Full-resolution samples feeding component sample `i` along one axis, with their weights: near = X / 2 (3/4),
// far = X - 1 / X + 1 in component samples, clamped to [0, n_c - 1] (1/4). Candidates X in [2i - 1, 2i + 2].
template <typename T>
__device__ __forceinline__ int up_taps(int i, int f, int n_full, int n_c, int* xs, T* ws) {
  if (f == 1) {
    xs[0] = i;
    ws[0] = T(1);
    return 1;
  }
  int n = 0;
  for (int X = 2 * i - 1; X <= 2 * i + 2; X++) {
    if (X < 0 || X >= n_full) continue;
    const int near = X >> 1;
    const int far = (X & 1) == 0 ? max(near - 1, 0) : min(near + 1, n_c - 1);
    const T wt = (near == i ? T(0.75) : T(0)) + (far == i ? T(0.25) : T(0));
    if (wt != 0.0) {
      xs[n] = X;
      ws[n] = wt;
      n++;
    }
  }
  return n;
}

// Four blocks per CTA, one thread per sample: component gradient -> smem -> row and column DCT -> coefficient
// gradient (zigzag) and the block's gradient energy. T is the arithmetic of the gather (the upsampling and colour
// transposes): double for the checked coefficient gradient and for weights from the FP64 adjoint; float for the
// weights from the FP32 adjoint, whose gradient is already a few 1e-4 from the FP64 one (the FP64 gather took
// 1.2 ms at 12 MP on this part's FP64 rate). Only the energy is kept with float (coef_grad must be null).
template <typename T>
__global__ void __launch_bounds__(256) k_coef_grad(const double* __restrict__ g, PullDesc d,
                                                   double* __restrict__ coef_grad, double* __restrict__ energy) {
  __shared__ double gs[4][64];
  __shared__ double tmp[4][64];
  __shared__ double wsum[8];
  const int grp = threadIdx.x >> 6, t = threadIdx.x & 63;
  const int ty = t >> 3, tx = t & 7;
  const long long gb = (long long)blockIdx.x * 4 + grp;
  const bool live = gb < d.nblocks;
  double gc = 0.0;
  if (live) {
    const int c = comp_of_block(d, gb);
    const PullComp& pc = d.c[c];
    const long long b = gb - pc.blk0;
    const int cy = (int)(b / pc.bw) * 8 + ty, cx = (int)(b % pc.bw) * 8 + tx;
    if (cx < pc.cw && cy < pc.ch) {
      T aR, aG, aB;
      if (d.ncomp == 1 || c == 0) {
        aR = aG = aB = T(1);
      } else if (c == 1) {
        aR = T(0);
        aG = T(-22554.0 / 65536.0);
        aB = T(116130.0 / 65536.0);
      } else {
        aR = T(91881.0 / 65536.0);
        aG = T(-46802.0 / 65536.0);
        aB = T(0);
      }
      int xs[4], ys[4];
      T wx[4], wy[4];
      const int nx = up_taps<T>(cx, pc.fx, d.w, pc.cw, xs, wx);
      const int ny = up_taps<T>(cy, pc.fy, d.h, pc.ch, ys, wy);
      T acc = T(0);
      for (int j = 0; j < ny; j++) {
        T row = T(0);
        for (int i = 0; i < nx; i++) {
          const double* p = g + ((size_t)ys[j] * d.w + xs[i]) * 3;
          row += wx[i] * (aR * T(p[0]) + aG * T(p[1]) + aB * T(p[2]));
        }
        acc += wy[j] * row;
      }
      gc = (double)acc;
    }
  }
  gs[grp][t] = gc;
  // block energy: two warps per block, shuffle sums, then warp 0 + warp 1
  double e = gc * gc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = e;
  __syncthreads();
  if (!coef_grad) {  // the weights need the energy alone (Parseval)
    if (live && t == 0) energy[gb] = wsum[2 * grp] + wsum[2 * grp + 1];
    return;
  }
  // rows: tmp[y][u] = sum_x g[y][x] C[u][x]
  double r = 0.0;
#pragma unroll
  for (int x = 0; x < 8; x++) r += gs[grp][ty * 8 + x] * c_dct[tx * 8 + x];
  tmp[grp][t] = r;
  __syncthreads();
  if (!live) return;
  // columns: G[v][u] = sum_y C[v][y] tmp[y][u]
  double G = 0.0;
#pragma unroll
  for (int y = 0; y < 8; y++) G += c_dct[ty * 8 + y] * tmp[grp][y * 8 + tx];
  coef_grad[gb * 64 + c_izz[t]] = G;
  if (t == 0) energy[gb] = wsum[2 * grp] + wsum[2 * grp + 1];
}

// Neighbourhood RMS of the block energies (edge-replicated window, rows then columns in order).
__global__ void k_block_sensitivity(PullDesc d, const double* __restrict__ energy, int radius,
                                    double* __restrict__ sens) {
  const long long gb = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gb >= d.nblocks) return;
  const PullComp& pc = d.c[comp_of_block(d, gb)];
  const long long b = gb - pc.blk0;
  const int by = (int)(b / pc.bw), bx = (int)(b % pc.bw);
  double acc = 0.0;
  for (int dy = -radius; dy <= radius; dy++) {
    const int yy = min(max(by + dy, 0), pc.bh - 1);
    for (int dx = -radius; dx <= radius; dx++) {
      const int xx = min(max(bx + dx, 0), pc.bw - 1);
      acc += energy[pc.blk0 + (long long)yy * pc.bw + xx];
    }
  }
  const int n = (2 * radius + 1) * (2 * radius + 1);
  sens[gb] = sqrt(acc / (double)n);
}

// Mean sensitivity of each component: one CTA per component, fixed summation order (deterministic).
__global__ void __launch_bounds__(1024) k_component_mean(PullDesc d, const double* __restrict__ sens,
                                                         double* __restrict__ mean) {
  __shared__ double part[1024];
  const PullComp& pc = d.c[blockIdx.x];
  const long long nb = (long long)pc.bw * pc.bh;
  double s = 0.0;
  for (long long i = threadIdx.x; i < nb; i += blockDim.x) s += sens[pc.blk0 + i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) mean[blockIdx.x] = part[0] / (double)nb;
}

// W[b][k] for all 64 k of a block. One warp per 32 blocks: each lane evaluates its block's weight once, then the
// warp writes the 32 blocks' 2048 floats as coalesced float4 rows (each value taken from its block's lane).
__global__ void k_weights(PullDesc d, const double* __restrict__ sens, const double* __restrict__ mean,
                          PerceptualParams p, float* __restrict__ weights) {
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5 << 5;  // first block of the warp
  const int lane = threadIdx.x & 31;
  if (warp0 >= d.nblocks) return;
  const long long gb = warp0 + lane;
  float f = 0.0f;
  if (gb < d.nblocks) {
    const double m = mean[comp_of_block(d, gb)];
    const double r = m > 0.0 ? sens[gb] / m : 1.0;  // an all-zero gradient leaves every weight at clamp(1)
    f = (float)(fmin(fmax(pow(r, p.gamma), p.w_min), p.w_max) * p.strength);
  }
  float4* out = reinterpret_cast<float4*>(weights) + warp0 * 16;
  const long long n4 = (d.nblocks - warp0) * 16;  // float4 entries left from this warp's first block
#pragma unroll 4
  for (int j = 0; j < 16; j++) {
    const int q = j * 32 + lane;  // float4 index within the warp's 32 blocks
    const float v = __shfl_sync(0xffffffffu, f, q >> 4);
    if (q < n4) out[q] = make_float4(v, v, v, v);
  }
}

// 8-bit Gray or RGB -> 8-bit RGB and/or f32 RGB (Gray replicated, as the scorer does: core/src/ssimulacra2.rs:192-203).
__global__ void k_expand_rgb(const uint8_t* __restrict__ src, int channels, size_t npx, uint8_t* __restrict__ rgb8,
                             float* __restrict__ rgbf) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += (size_t)gridDim.x * blockDim.x) {
    uint8_t v[3];
    if (channels == 1) {
      v[0] = v[1] = v[2] = src[i];
    } else {
      v[0] = src[3 * i];
      v[1] = src[3 * i + 1];
      v[2] = src[3 * i + 2];
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (rgb8) rgb8[3 * i + c] = v[c];
      if (rgbf) rgbf[3 * i + c] = (float)v[c];
    }
  }
}

bool g_tables_ready[64] = {false};

int upload_tables(rcg_ctx* ctx) {
  if (ctx->device >= 0 && ctx->device < 64 && g_tables_ready[ctx->device]) return RCG_OK;
  double C[64];
  for (int u = 0; u < 8; u++)
    for (int x = 0; x < 8; x++)
      C[u * 8 + x] = (u == 0 ? std::sqrt(1.0 / 8.0) : 0.5) * std::cos((2 * x + 1) * u * M_PI / 16.0);
  int izz[64];
  for (int k = 0; k < 64; k++) izz[zigzag_natural(k)] = k;
  cudaError_t e = cudaMemcpyToSymbol(c_dct, C, sizeof C);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_izz, izz, sizeof izz);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "perceptual tables");
  if (ctx->device >= 0 && ctx->device < 64) g_tables_ready[ctx->device] = true;
  return RCG_OK;
}

}  // namespace

int expand_rgb(rcg_ctx* ctx, const uint8_t* d_src, int channels, size_t npx, uint8_t* d_rgb8, float* d_rgbf) {
  const unsigned grid = (unsigned)std::min<size_t>((npx + 255) / 256, 152 * 16);
  RCG_LAUNCH(ctx, "expand_rgb", k_expand_rgb, grid, 256, 0, d_src, channels, npx, d_rgb8, d_rgbf);
  return RCG_OK;
}

int perceptual_pullback(rcg_ctx* ctx, const double* d_grad, int w, int h, const StepDesc* lay,
                        const PerceptualParams& p, double* d_coef_grad, float* d_weights) {
  int rc = upload_tables(ctx);
  if (rc != RCG_OK) return rc;
  PullDesc d;
  d.ncomp = lay->ncomp;
  d.w = w;
  d.h = h;
  d.nblocks = lay->nblocks;
  for (int c = 0; c < 3; c++) {
    PullComp& pc = d.c[c];
    if (c >= lay->ncomp) {
      pc = PullComp{1, 1, 1, 1, 1, 1, lay->nblocks};
      continue;
    }
    const CompDesc& cd = lay->comp[c];
    pc.bw = cd.bw;
    pc.bh = cd.bh;
    pc.fx = lay->hmax / cd.h;
    pc.fy = lay->vmax / cd.v;
    if (pc.fx > 2 || pc.fy > 2) return fail(ctx, RCG_UNSUPPORTED, "perceptual weights take 1x or 2x chroma sampling");
    pc.cw = (w * cd.h + lay->hmax - 1) / lay->hmax;
    pc.ch = (h * cd.v + lay->vmax - 1) / lay->vmax;
    pc.blk0 = cd.blk0;
  }
  const long long nb = lay->nblocks;
  double* energy = (double*)workspace(ctx, "perc_energy", (size_t)nb * sizeof(double));
  double* sens = (double*)workspace(ctx, "perc_sens", (size_t)nb * sizeof(double));
  double* mean = (double*)workspace(ctx, "perc_mean", 3 * sizeof(double));
  if (!energy || !sens || !mean) return RCG_NO_MEMORY;
  if (!d_coef_grad && !p.gradient_fp64)
    RCG_LAUNCH(ctx, "coef_grad", k_coef_grad<float>, (unsigned)((nb + 3) / 4), 256, 0, d_grad, d, d_coef_grad, energy);
  else
    RCG_LAUNCH(ctx, "coef_grad", k_coef_grad<double>, (unsigned)((nb + 3) / 4), 256, 0, d_grad, d, d_coef_grad,
               energy);
  if (!d_weights) return RCG_OK;
  RCG_LAUNCH(ctx, "block_sensitivity", k_block_sensitivity, (unsigned)((nb + 255) / 256), 256, 0, d, energy,
             p.radius, sens);
  RCG_LAUNCH(ctx, "component_mean", k_component_mean, d.ncomp, 1024, 0, d, sens, mean);
  RCG_LAUNCH(ctx, "weights", k_weights, (unsigned)((nb + 255) / 256), 256, 0, d, sens, mean, p, d_weights);
  return RCG_OK;
}

}  // namespace rcg
