// SSIMULACRA2 scorer kernels (K8-K10): the reference's core/src/ssimulacra2.rs on one GPU.
//
// Pipeline per score: linear-light planes (f32, channel-planar) -> 2x2 pyramid (scales 1..5) -> one launch that
// covers every tile of every scale (XYB, five moments, 11-tap blur, error maps, six partial sums per channel) ->
// a deterministic f64 reduction and the final 108-weight mapping.
//
// Arithmetic. The reference holds the planes in f32 and computes XYB, the blur, the maps and the sums in f64
// (:18, :345-346, :361). GB300's FP64 rate is a small fraction of its FP32 rate, so here:
//   * planes: f32 exactly as the reference (LUT values; the 2x2 average is a compensated sum that rounds like the
//     reference's f64 sum nearly always);
//   * XYB, blur and maps: f32, arranged so that nothing cancels catastrophically. Each pixel carries the reference
//     image's XYB and the XYB *difference* of the two images, both computed from cube-root difference identities
//     (see pix()); both are offset by their value at the tile centre, so the five blurred moments (mu_a, mu_(a-b),
//     E[a^2], E[b^2], E[(a-b)^2]) are small where the image is smooth. The variances and mu1 - mu2 are recovered
//     exactly from them (the offsets cancel wherever the blur taps sum to 1 and are corrected with the in-image tap
//     sum within 5 columns of the zero left/right border, :34-40). The SSIM term is evaluated as
//     (sigma_(a-b)^2 + (mu1-mu2)^2 num_s) / denom_s and the edge term from r1 = a - mu1 and its difference, forms
//     that equal the reference's expressions algebraically but keep full relative precision for similar images;
//   * cube roots: 2^(log2(x) / 3) from the hardware's approximate log2 and exp2 (relative error a few 1e-7; the
//     differences between the two images never go through them, only through the identity below);
//   * sums: f32 over the 4 pixels of a thread (in registers, then added to the thread's running sums of its band),
//     f32 across a warp, f64 from there on, in a fixed order (bit-reproducible from run to run, as the reference's
//     test :630 requires).
// Identical images give exactly 100: every difference term is exactly 0, so every map value is exactly 0.
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "rcg_internal.cuh"
#include "upsample420.cuh"

namespace rcg {

__constant__ float c_gauss[2 * kRadius + 1];
__constant__ float c_lut8s[256];
__constant__ double c_weights[108];

// core/src/ssimulacra2.rs:42-52 (opsin absorbance matrix and bias), as f32
constexpr double kM02 = 0.078, kM00 = 0.30, kM01 = 1.0 - kM02 - kM00;
constexpr double kM12 = 0.078, kM10 = 0.23, kM11 = 1.0 - kM12 - kM10;
constexpr double kM20 = 0.2434226892454782, kM21 = 0.2047674442449682, kM22 = 1.0 - kM20 - kM21;
constexpr double kBias = 0.0037930732552754493;

// Cube root of x > 0 as 2^(log2(x) / 3) with the hardware's approximate log2 and exp2 (a few ulp). The flush-to-zero
// forms: every argument here is at least the opsin bias (0.0038) and every result at least its cube root, so no
// subnormal can occur, and the forms without .ftz only add a range check and rescaling around each operation
// (measured: the tile kernel 608 -> 556 us per 12 MP score with these and the division below).
__device__ __forceinline__ float cbrt_fast(float x) {
  float l, y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l) : "f"(x));
  l *= (1.0f / 3.0f);
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(l));
  return y;
}

// a / b as a * approximate(1 / b) (2 ulp), flush-to-zero form; the divisors below are normal and well inside the
// range where the reciprocal is defined.
__device__ __forceinline__ float fdiv_ftz(float a, float b) {
  float r;
  asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// x^2 + x*y + y^2: cbrt(u) - cbrt(v) = (u - v) / D(cbrt(u), cbrt(v)).
__device__ __forceinline__ float dsq(float x, float y) { return fmaf(x, x, fmaf(x, y, y * y)); }

// q_a/D_a - q_b/D_b without cancellation: (dq*D_b - q_b*dD) / (D_a*D_b), dq = q_a - q_b and dD = D_a - D_b given.
__device__ __forceinline__ float qdiff(float qb, float dq, float Da, float Db, float dD) {
  return fdiv_ftz(fmaf(dq, Db, -qb * dD), Da * Db);
}

// One pixel of the tile: the reference image's XYB minus the tile offsets (`a`, core/src/ssimulacra2.rs:249-258)
// and XYB(reference) - XYB(distorted) minus the tile's difference offsets (`d`). Every quantity that is a small
// difference of nearly equal cube roots is formed from the identity above, so it keeps its relative precision in
// f32: X - 0.42 = 7 (c0 - c1), B - 0.55 = ((c2 - c0) + (c2 - c1)) / 2, each c_i - c_j from the difference of two
// opsin-matrix rows applied to (r, g, b); and the per-pixel differences between the two images from the linear
// differences (r_a - r_b, ...).
struct Pix {
  float a[3], d[3];
};

__device__ __forceinline__ Pix pix(float ra, float ga, float ba, float rb, float gb, float bb, const float* oa,
                                   const float* od, float cbrt_bias) {
  const float bias = (float)kBias;
  // opsin rows (f32) and the exact differences of rows, rounded once
  const float M00 = (float)kM00, M01 = (float)kM01, M02 = (float)kM02;
  const float M10 = (float)kM10, M11 = (float)kM11, M12 = (float)kM12;
  const float M20 = (float)kM20, M21 = (float)kM21, M22 = (float)kM22;
  const float L20r = (float)(kM20 - kM00), L20g = (float)(kM21 - kM01), L20b = (float)(kM22 - kM02);
  const float L21r = (float)(kM20 - kM10), L21g = (float)(kM21 - kM11), L21b = (float)(kM22 - kM12);
  float ca[3], cb[3];
  ca[0] = cbrt_fast(fmaxf(fmaf(M00, ra, fmaf(M01, ga, fmaf(M02, ba, bias))), 0.0f));
  ca[1] = cbrt_fast(fmaxf(fmaf(M10, ra, fmaf(M11, ga, fmaf(M12, ba, bias))), 0.0f));
  ca[2] = cbrt_fast(fmaxf(fmaf(M20, ra, fmaf(M21, ga, fmaf(M22, ba, bias))), 0.0f));
  cb[0] = cbrt_fast(fmaxf(fmaf(M00, rb, fmaf(M01, gb, fmaf(M02, bb, bias))), 0.0f));
  cb[1] = cbrt_fast(fmaxf(fmaf(M10, rb, fmaf(M11, gb, fmaf(M12, bb, bias))), 0.0f));
  cb[2] = cbrt_fast(fmaxf(fmaf(M20, rb, fmaf(M21, gb, fmaf(M22, bb, bias))), 0.0f));
  float q01a = 0.07f * (ra - ga), q01b = 0.07f * (rb - gb);
  float q20a = fmaf(L20r, ra, fmaf(L20g, ga, L20b * ba)), q20b = fmaf(L20r, rb, fmaf(L20g, gb, L20b * bb));
  float q21a = fmaf(L21r, ra, fmaf(L21g, ga, L21b * ba)), q21b = fmaf(L21r, rb, fmaf(L21g, gb, L21b * bb));
  float D01a = dsq(ca[0], ca[1]), D20a = dsq(ca[2], ca[0]), D21a = dsq(ca[2], ca[1]);
  float D01b = dsq(cb[0], cb[1]), D20b = dsq(cb[2], cb[0]), D21b = dsq(cb[2], cb[1]);
  Pix o;
  float ya = 0.5f * (ca[0] + ca[1]);
  o.a[0] = fmaf(7.0f, fdiv_ftz(q01a, D01a), 0.42f - oa[0]);
  o.a[1] = (ya - cbrt_bias) + (0.01f - oa[1]);
  o.a[2] = 0.5f * (fdiv_ftz(q20a, D20a) + fdiv_ftz(q21a, D21a)) + (0.55f - oa[2]);
  float dr = ra - rb, dg = ga - gb, db = ba - bb;
  float dc0 = fdiv_ftz(fmaf(M00, dr, fmaf(M01, dg, M02 * db)), dsq(ca[0], cb[0]));
  float dc1 = fdiv_ftz(fmaf(M10, dr, fmaf(M11, dg, M12 * db)), dsq(ca[1], cb[1]));
  float dc2 = fdiv_ftz(fmaf(M20, dr, fmaf(M21, dg, M22 * db)), dsq(ca[2], cb[2]));
  // D(x, y) of image a minus of image b: dx (xa + xb) + dx ya + xb dy + dy (ya + yb)
  float dD01 = fmaf(dc0, ca[0] + cb[0], fmaf(dc0, ca[1], fmaf(cb[0], dc1, dc1 * (ca[1] + cb[1]))));
  float dD20 = fmaf(dc2, ca[2] + cb[2], fmaf(dc2, ca[0], fmaf(cb[2], dc0, dc0 * (ca[0] + cb[0]))));
  float dD21 = fmaf(dc2, ca[2] + cb[2], fmaf(dc2, ca[1], fmaf(cb[2], dc1, dc1 * (ca[1] + cb[1]))));
  float dq01 = 0.07f * (dr - dg);
  float dq20 = fmaf(L20r, dr, fmaf(L20g, dg, L20b * db));
  float dq21 = fmaf(L21r, dr, fmaf(L21g, dg, L21b * db));
  o.d[0] = 7.0f * qdiff(q01b, dq01, D01a, D01b, dD01) - od[0];
  o.d[1] = 0.5f * (dc0 + dc1) - od[1];
  o.d[2] = 0.5f * (qdiff(q20b, dq20, D20a, D20b, dD20) + qdiff(q21b, dq21, D21a, D21b, dD21)) - od[2];
  return o;
}

// Row index under the top/bottom mirror rule (core/src/ssimulacra2.rs:385-397); -1 for rows no valid output reads.
__device__ __forceinline__ int mirror_row(int yy, int h) {
  if (yy < -kRadius || yy > h - 1 + kRadius) return -1;
  if (yy < 0) return -yy - 1;
  if (yy >= h) return 2 * h - 1 - yy;
  return yy;
}

// Row pitch 45 pairs (>= 42 columns): a horizontal-pass item reads 8-byte (a', d') pairs at a stride of 4 pairs,
// and 2 * 45 = 26 mod 32 shifts each of the 4 rows a half-warp covers to its own bank class, so its 16 loads hit
// 32 distinct banks.
constexpr int kIW = 45;
constexpr int kIH = kTileH + 2 * kRadius;  // 42
constexpr int kHx = 4;                     // horizontal-pass outputs per item
constexpr size_t kTileSmem = (size_t)(6 * kIH * kIW + 5 * kIH * kTileW) * sizeof(float);

// One CTA = one band of 32 output columns and nch chunks of 32 output rows of one scale, walked top to bottom.
// Shared memory: per channel the (a', d') pairs of the chunk plus its 5-pixel halo (42 x 42); then per channel the
// horizontally blurred five moments of the 42 halo rows. Between chunks the 10 halo rows that the next chunk shares
// with this one (its top halo and first output rows) move to the top of the buffer instead of being converted to XYB
// again, so a band pays the vertical halo's XYB once: 42 x (32 nch + 10) conversions for 32 x 32 nch outputs where
// nch separate tiles pay 42 x 42 x nch. The blurs run the moment pairs that share a tap weight ((a', d'),
// (a'^2, d'^2)) as packed two-lane f32 FMAs, each lane exactly fmaf, so the results are those of scalar FMAs in the
// same order.
// Offsets: every chunk takes the XYB and XYB difference at its own centre, as a 32 x 32 tile does; the carried rows
// are re-offset by the change (one f32 subtraction each). With nch = 1 the band is exactly the single tile.
// Band `local` of scale `sd` (sd.tiles_x bands across; sd.nch chunks each) of a pyramid pair; the band's 18 sums go to
// out[i * stride], i < 18.
// Reference moments (kRef). The offsets a chunk subtracts come from the reference alone (its XYB at the chunk
// centre), so the blurred a' and a'^2 of every output pixel depend on the reference and the band layout only. A
// search scores every candidate against one reference: its first candidate runs kRef = kRefWrite, which also stores
// (blur a', blur a'^2) per output pixel and channel; the later ones run kRef = kRefRead, which blur only (b'^2, d'^2)
// as a packed pair and d', and read the other two. Each blurred moment is the same chain of per-lane fmaf in every
// mode, so the scores are bit-identical to kRefNone. The store keeps each chunk's 3 x 32 x 32 pairs contiguous
// (24 KB, [channel][row][column]); a reading CTA asks for the whole block in L2 with one bulk prefetch per channel
// as the chunk starts and reads it in its vertical pass. Measured per 12 MP score: 584.7 us without the store,
// 612.7 us writing it, 547.0 us reading it (before the flush-to-zero forms and packed squares: 651.5 / 680.0 /
// 608.9, and 603 us with the two moments left out altogether); with the store indexed like the pyramid planes and
// no bulk prefetch the read mode took 645 us, and staging each channel's block in shared memory with cp.async 629.

template <int kRef>
__device__ __forceinline__ void ssim2_band(const ScaleDesc sd, const int local, const float* __restrict__ ref,
                                           const float* __restrict__ dist, double* __restrict__ out,
                                           const size_t stride, float2* __restrict__ refm) {
  extern __shared__ float smem[];
  float2* xs = reinterpret_cast<float2*>(smem);  // [3][kIH][kIW] pairs (a', d') per channel
  float* hb = smem + 6 * kIH * kIW;              // pair planes (m0, m1), (m2, m3) then m4, [kIH][kTileW] each
  __shared__ float s_red[kTileThreads / 32][kScoreSums];
  __shared__ float s_oa[3], s_od[3], s_noa[3], s_nod[3];

  const int tx = local % sd.tiles_x, ty = local / sd.tiles_x;
  const int nch = sd.nch;
  const int x0 = tx * kTileW, ybeg = ty * kTileH * nch;
  const int w = sd.w, h = sd.h;
  const size_t np = (size_t)w * h;
  const float* ra = ref + sd.off;
  const float* rb = dist + sd.off;
  const float cb_bias = cbrt_fast((float)kBias);
  const int tid = threadIdx.x;
  constexpr int kCols = kTileW + 2 * kRadius;  // 42 real columns of the kIW-pitched rows
  constexpr int kCarry = 2 * kRadius;          // rows a chunk hands to the next

  // The six plane values of halo pixel e of the chunk at y0 (rows from r0 on), with the mirror rule for rows.
  auto load6 = [&](int e, int y0, int r0, float* v) -> bool {
    int r = r0 + e / kCols, c = e - (r - r0) * kCols;
    int gy = mirror_row(y0 - kRadius + r, h);
    int gx = x0 - kRadius + c;
    if (r < kIH && gy >= 0 && gx >= 0 && gx < w) {
      size_t i = (size_t)gy * w + gx;
      v[0] = __ldg(ra + i);
      v[1] = __ldg(ra + np + i);
      v[2] = __ldg(ra + 2 * np + i);
      v[3] = __ldg(rb + i);
      v[4] = __ldg(rb + np + i);
      v[5] = __ldg(rb + 2 * np + i);
      return true;
    }
    return false;
  };
  // Per-chunk offsets: the reference's XYB and the XYB difference at the centre of the chunk at y0. Stored values
  // are a' = a - oa and d' = (a - b) - od inside the image and 0 outside (the zero border). Every moment the maps
  // need is recovered exactly from the blurred primed values and the in-image tap sum K of the column (K = 1 away
  // from the left/right edges, where the offsets cancel outright).
  auto centre = [&](int y0, float* oa_out, float* od_out) {
    int cx = min(x0 + kTileW / 2, w - 1), cy = min(y0 + kTileH / 2, h - 1);
    size_t i = (size_t)cy * w + cx;
    const float z[3] = {0.f, 0.f, 0.f};
    Pix c = pix(ra[i], ra[np + i], ra[2 * np + i], rb[i], rb[np + i], rb[2 * np + i], z, z, cb_bias);
    for (int k = 0; k < 3; k++) {
      oa_out[k] = c.a[k];
      od_out[k] = c.d[k];
    }
  };

  float sums[kScoreSums];
#pragma unroll
  for (int i = 0; i < kScoreSums; i++) sums[i] = 0.0f;
  // The blur's six distinct taps as (k, k) pairs, held in registers for the packed FMAs (the taps are symmetric:
  // tap t and tap 2 kRadius - t are the same f32 value).
  float2 g2[kRadius + 1];
#pragma unroll
  for (int t = 0; t <= kRadius; t++) g2[t] = make_float2(c_gauss[t], c_gauss[t]);

  const int col = tid & 31, rg = tid >> 5;  // vertical pass: column, group of 4 output rows
  const int gx = x0 + col;
  // In-image tap sum of this column (1 except within kRadius of the left/right edge).
  const bool edge = gx < kRadius || gx >= w - kRadius;
  float K = 1.0f;
  if (edge) {
    K = 0.0f;
#pragma unroll
    for (int t = 0; t < 2 * kRadius + 1; t++) {
      int xx = gx + t - kRadius;
      if (xx >= 0 && xx < w) K += c_gauss[t];
    }
  }
  const float omk = 1.0f - K;

#pragma unroll 1
  for (int chunk = 0; chunk < nch; chunk++) {
    const int y0 = ybeg + chunk * kTileH;
    if (y0 >= h) break;
    // Rows of the halo buffer converted in this chunk: all 42 in the first, the 32 below the carried ones after.
    const int r0 = chunk == 0 ? 0 : kCarry;
    float cur[6], nxt[6];
    bool cur_ok;
    if (chunk == 0) {
      // The first pixel's loads go out before the offsets are settled (they do not depend on them).
      cur_ok = load6(tid, y0, r0, cur);
      if (tid == 0) centre(y0, s_oa, s_od);
      __syncthreads();
    } else {
      __syncthreads();  // the previous chunk's passes are done with xs and hb; s_noa/s_nod are visible
      cur_ok = load6(tid, y0, r0, cur);
      // Carried rows: rows 32..41 of the previous chunk become rows 0..9, re-offset from the previous chunk's
      // offsets to this one's (s_noa/s_nod, computed during the previous chunk).
      float da[3], dd[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        da[k] = s_noa[k] - s_oa[k];
        dd[k] = s_nod[k] - s_od[k];
      }
      constexpr int kCarried = kCarry * kCols * 3, kPer = (kCarried + kTileThreads - 1) / kTileThreads;
      float2 keep[kPer];
#pragma unroll
      for (int j = 0; j < kPer; j++) {
        const int e = tid + j * kTileThreads;
        if (e < kCarried) {
          const int k = e / (kCarry * kCols), rem = e - k * (kCarry * kCols);
          const int r = rem / kCols, c = rem - r * kCols;
          float2 v = xs[k * kIH * kIW + (r + kTileH) * kIW + c];
          // inside the image the stored values move with the offsets; outside they stay 0 (the zero border)
          const int gy = mirror_row(y0 - kRadius + r, h), gxx = x0 - kRadius + c;
          if (gy >= 0 && gxx >= 0 && gxx < w) {
            const float dak = k == 0 ? da[0] : (k == 1 ? da[1] : da[2]);
            const float ddk = k == 0 ? dd[0] : (k == 1 ? dd[1] : dd[2]);
            v = make_float2(v.x - dak, v.y - ddk);
          }
          keep[j] = v;
        }
      }
      __syncthreads();  // every carried value is read before rows 32..41 are overwritten
#pragma unroll
      for (int j = 0; j < kPer; j++) {
        const int e = tid + j * kTileThreads;
        if (e < kCarried) {
          const int k = e / (kCarry * kCols), rem = e - k * (kCarry * kCols);
          const int r = rem / kCols, c = rem - r * kCols;
          xs[k * kIH * kIW + r * kIW + c] = keep[j];
        }
      }
      if (tid < 3) {
        s_oa[tid] = s_noa[tid];
        s_od[tid] = s_nod[tid];
      }
      __syncthreads();
    }
    float oa[3] = {s_oa[0], s_oa[1], s_oa[2]}, od[3] = {s_od[0], s_od[1], s_od[2]};
    // This chunk's block of reference moments (kRefChunk float2).
    float2* rchunk = nullptr;
    if constexpr (kRef != kRefNone) rchunk = refm + (size_t)(sd.chunk0 + local * nch + chunk) * kRefChunk;
    if constexpr (kRef == kRefRead) {
      // Into L2 while this chunk's XYB and horizontal passes run: 8 KB per channel (16-byte aligned, as the bulk
      // prefetch requires: blocks are 24 KB apart from an aligned base).
      if (tid < 3) {
        const float2* p = rchunk + tid * kTileH * kTileW;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(kTileH * kTileW * 8) : "memory");
      }
    }

    // XYB of the chunk's new rows; the six plane values of the next pixel are loaded before the current one is
    // converted, so the global loads overlap the arithmetic. Two halo pixels per trip: the measured best unroll.
    const int nconv = (kIH - r0) * kCols;
#pragma unroll 2
    for (int e = tid; e < nconv; e += kTileThreads) {
      bool nxt_ok = load6(e + kTileThreads, y0, r0, nxt);
      float v[6] = {0, 0, 0, 0, 0, 0};
      if (cur_ok) {
        Pix p = pix(cur[0], cur[1], cur[2], cur[3], cur[4], cur[5], oa, od, cb_bias);
        v[0] = p.a[0]; v[1] = p.a[1]; v[2] = p.a[2];
        v[3] = p.d[0]; v[4] = p.d[1]; v[5] = p.d[2];
      }
      const int r = r0 + e / kCols, idx = r * kIW + (e - (r - r0) * kCols);
#pragma unroll
      for (int k = 0; k < 3; k++) xs[k * kIH * kIW + idx] = make_float2(v[k], v[3 + k]);
#pragma unroll
      for (int k = 0; k < 6; k++) cur[k] = nxt[k];
      cur_ok = nxt_ok;
    }
    // The next chunk's offsets, while the other threads finish their conversions.
    if (tid == 0 && chunk + 1 < nch && y0 + kTileH < h) centre(y0 + kTileH, s_noa, s_nod);

#pragma unroll 1
    for (int ch = 0; ch < 3; ch++) {
      __syncthreads();  // xs complete (ch 0) / previous channel's vertical pass done with hb
      const float2* X = xs + ch * kIH * kIW;
      // Horizontal pass: kHx adjacent outputs per item; moments a', d', a'^2, b'^2 (b' = a' - d'), d'^2. The pairs
      // (a', d') and (a'^2, d'^2) share every tap weight and run as packed two-lane FMAs (per lane exactly fmaf);
      // the squares of a loaded (a', d') pair are one packed multiply.
      // Items: each half-warp takes 4 rows x 4 items, so its 64-bit loads (row pitch 45 pairs = 26 banks mod 32)
      // fall in distinct banks.
      static_assert(kTileThreads == 256 && kTileH == 32 && kTileW == 32 && kIH - kTileH == 10, "item layout");
      // One item: NX adjacent outputs of row r from column c0 on.
      auto hitem = [&](auto nx, const int r, const int c0) {
        constexpr int NX = decltype(nx)::value;
        const float2* xr = X + r * kIW + c0;
        if constexpr (kRef == kRefRead) {
          // (b'^2, d'^2) pairs and d'; the first plane of hb holds (blur b'^2, blur d'^2). b' replaces a' in its
          // pair, so one packed multiply squares both.
          float2 vsq[NX + 2 * kRadius];
          float vd[NX + 2 * kRadius];
#pragma unroll
          for (int t = 0; t < NX + 2 * kRadius; t++) {
            float2 bd = xr[t];
            vd[t] = bd.y;
            bd.x = __fsub_rn(bd.x, bd.y);
            vsq[t] = __fmul2_rn(bd, bd);
          }
          float2 m13[NX];
          float m4[NX];
#pragma unroll
          for (int o = 0; o < NX; o++) {
            float2 s13 = make_float2(0.f, 0.f);
            float sd = 0.f;
#pragma unroll
            for (int t = 0; t < 2 * kRadius + 1; t++) {
              const float2 kk = g2[t <= kRadius ? t : 2 * kRadius - t];
              s13 = __ffma2_rn(kk, vsq[o + t], s13);
              sd = fmaf(kk.x, vd[o + t], sd);
            }
            m13[o] = s13;
            m4[o] = sd;
          }
          float* h13 = hb + (r * kTileW + c0) * 2;
          float* h4 = hb + 4 * kIH * kTileW + r * kTileW + c0;
#pragma unroll
          for (int o = 0; o < NX; o += 2)
            reinterpret_cast<float4*>(h13)[o / 2] = make_float4(m13[o].x, m13[o].y, m13[o + 1].x, m13[o + 1].y);
          if constexpr (NX == 4) *reinterpret_cast<float4*>(h4) = make_float4(m4[0], m4[1], m4[2], m4[3]);
          else *reinterpret_cast<float2*>(h4) = make_float2(m4[0], m4[1]);
        } else {
          // Pairs (a', d') and (a'^2, d'^2) (one packed multiply of the loaded pair), b'^2 alone.
          float2 vad[NX + 2 * kRadius], vsq[NX + 2 * kRadius];
          float vbb[NX + 2 * kRadius];
#pragma unroll
          for (int t = 0; t < NX + 2 * kRadius; t++) {
            const float2 ad = xr[t];
            const float bb = __fsub_rn(ad.x, ad.y);
            vad[t] = ad;
            vsq[t] = __fmul2_rn(ad, ad);
            vbb[t] = __fmul_rn(bb, bb);
          }
          float2 m01[NX], m23[NX];
          float m4[NX];
#pragma unroll
          for (int o = 0; o < NX; o++) {
            float2 s01 = make_float2(0.f, 0.f), s24 = make_float2(0.f, 0.f);
            float sbb = 0.f;
#pragma unroll
            for (int t = 0; t < 2 * kRadius + 1; t++) {
              const float2 kk = g2[t <= kRadius ? t : 2 * kRadius - t];
              s01 = __ffma2_rn(kk, vad[o + t], s01);
              s24 = __ffma2_rn(kk, vsq[o + t], s24);
              sbb = fmaf(kk.x, vbb[o + t], sbb);
            }
            m01[o] = s01;
            m23[o] = s24;
            m4[o] = sbb;
          }
          // hb: two planes of (moment 0, moment 1) and (moment 2, moment 4) pairs, then moment 3
          float* h01 = hb + (r * kTileW + c0) * 2;
          float* h23 = hb + (kIH * kTileW + r * kTileW + c0) * 2;
          float* h4 = hb + 4 * kIH * kTileW + r * kTileW + c0;
#pragma unroll
          for (int o = 0; o < NX; o += 2) {
            reinterpret_cast<float4*>(h01)[o / 2] = make_float4(m01[o].x, m01[o].y, m01[o + 1].x, m01[o + 1].y);
            reinterpret_cast<float4*>(h23)[o / 2] = make_float4(m23[o].x, m23[o].y, m23[o + 1].x, m23[o + 1].y);
          }
          if constexpr (NX == 4) *reinterpret_cast<float4*>(h4) = make_float4(m4[0], m4[1], m4[2], m4[3]);
          else *reinterpret_cast<float2*>(h4) = make_float2(m4[0], m4[1]);
        }
      };
      // Rows 0..31: one item of kHx = 4 outputs per thread; each half-warp takes 4 rows x 4 items, so its 64-bit
      // loads (row pitch 45 pairs = 26 banks mod 32) fall in distinct banks.
      {
        const int hw = tid >> 4, j = tid & 15;
        hitem(std::integral_constant<int, kHx>(), (hw >> 1) * 4 + (j >> 2), kHx * ((j & 3) + 4 * (hw & 1)));
      }
      // The 10 halo rows below: 160 items of 2 outputs (a half-warp takes 2 rows x 8 items, again distinct banks),
      // so this round costs about half an item of 4 and runs on 5 warps instead of 2.5 (measured per 12 MP launch:
      // reading form 547 -> 537 us, storing form 615 -> 596 us, same bits).
      if (tid < (kIH - kTileH) * (kTileW / 2)) {
        const int hw = tid >> 4, j = tid & 15;
        hitem(std::integral_constant<int, 2>(), kTileH + (hw >> 1) * 2 + (j >> 3), 2 * ((j & 7) + 8 * (hw & 1)));
      }
      __syncthreads();
      // Vertical pass + error maps: 4 output rows of one column per thread, the same pairs packed.
      float mu[5][4];
      float2* rrow = nullptr;  // this thread's row 0 in the chunk's block
      if constexpr (kRef != kRefNone) rrow = rchunk + (ch * kTileH + rg * 4) * kTileW + col;
      if constexpr (kRef == kRefRead) {
        // The reference moments first (their loads overlap the blur), then (blur b'^2, blur d'^2) and blur d'.
#pragma unroll
        for (int o = 0; o < 4; o++) {
          float2 rm = make_float2(0.f, 0.f);
          if (gx < w && y0 + rg * 4 + o < h) rm = __ldg(rrow + o * kTileW);
          mu[0][o] = rm.x;
          mu[2][o] = rm.y;
        }
        const float2* h13 = reinterpret_cast<const float2*>(hb);
        const float* h4 = hb + 4 * kIH * kTileW;
        float2 v13[4 + 2 * kRadius];
        float v4[4 + 2 * kRadius];
#pragma unroll
        for (int t = 0; t < 4 + 2 * kRadius; t++) {
          const int i = (rg * 4 + t) * kTileW + col;
          v13[t] = h13[i];
          v4[t] = h4[i];
        }
#pragma unroll
        for (int o = 0; o < 4; o++) {
          float2 a13 = make_float2(0.f, 0.f);
          float a4 = 0.f;
#pragma unroll
          for (int t = 0; t < 2 * kRadius + 1; t++) {
            const float2 kk = g2[t <= kRadius ? t : 2 * kRadius - t];
            a13 = __ffma2_rn(kk, v13[o + t], a13);
            a4 = fmaf(kk.x, v4[o + t], a4);
          }
          mu[3][o] = a13.x;
          mu[4][o] = a13.y;
          mu[1][o] = a4;
        }
      } else {
        const float2* h01 = reinterpret_cast<const float2*>(hb);
        const float2* h23 = reinterpret_cast<const float2*>(hb) + kIH * kTileW;
        const float* h4 = hb + 4 * kIH * kTileW;
        float2 v01[4 + 2 * kRadius], v23[4 + 2 * kRadius];
        float v4[4 + 2 * kRadius];
#pragma unroll
        for (int t = 0; t < 4 + 2 * kRadius; t++) {
          const int i = (rg * 4 + t) * kTileW + col;
          v01[t] = h01[i];
          v23[t] = h23[i];
          v4[t] = h4[i];
        }
#pragma unroll
        for (int o = 0; o < 4; o++) {
          float2 a01 = make_float2(0.f, 0.f), a23 = make_float2(0.f, 0.f);
          float a4 = 0.f;
#pragma unroll
          for (int t = 0; t < 2 * kRadius + 1; t++) {
            const float2 kk = g2[t <= kRadius ? t : 2 * kRadius - t];
            a01 = __ffma2_rn(kk, v01[o + t], a01);
            a23 = __ffma2_rn(kk, v23[o + t], a23);
            a4 = fmaf(kk.x, v4[o + t], a4);
          }
          mu[0][o] = a01.x;
          mu[1][o] = a01.y;
          mu[2][o] = a23.x;
          mu[4][o] = a23.y;
          mu[3][o] = a4;
          if constexpr (kRef == kRefWrite) {
            if (gx < w && y0 + rg * 4 + o < h) rrow[o * kTileW] = make_float2(a01.x, a23.x);
          }
        }
      }
      const float ca = s_oa[ch], cd = s_od[ch], cbv = ca - cd;
      float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int o = 0; o < 4; o++) {
        int ry = rg * 4 + o;
        int gy = y0 + ry;
        if (gx < w && gy < h) {
          // Blurred primed moments -> sigma_1^2, sigma_2^2, sigma_(a-b)^2, mu1 - mu2 (exactly, given K).
          float m1 = mu[0][o], dmp = mu[1][o], m2 = m1 - dmp;
          float v1 = fmaf(-m1, m1, mu[2][o]);
          float v2 = fmaf(-m2, m2, mu[3][o]);
          float vd = fmaf(-dmp, dmp, mu[4][o]);
          float dmu;
          if (edge) {
            v1 = fmaf(omk * ca, fmaf(ca, K, 2.0f * m1), v1);
            v2 = fmaf(omk * cbv, fmaf(cbv, K, 2.0f * m2), v2);
            vd = fmaf(omk * cd, fmaf(cd, K, 2.0f * dmp), vd);
            dmu = fmaf(cd, K, dmp);
          } else {
            dmu = dmp + cd;
          }
          // SSIM error (core/src/ssimulacra2.rs:427-430) as (sigma_(a-b)^2 + dmu^2 num_s) / denom_s, which equals
          // 1 - (1 - dmu^2) num_s / denom_s since num_s = denom_s - sigma_(a-b)^2.
          float den = (v1 + v2) + 0.0009f;
          float num_s = den - vd;
          float d = fmaxf(fdiv_ftz(fmaf(dmu * dmu, num_s, vd), den), 0.0f);
          // Edge maps (:431-433): d1 = (|r2| - |r1|) / (1 + |r1|) with r1 = a - mu1, r2 = b - mu2 = r1 - rd.
          const float2 c0 = X[(ry + kRadius) * kIW + col + kRadius];
          float a0 = c0.x, d0 = c0.y;
          float r1 = a0 - m1, rd = d0 - dmp;
          if (edge) {
            r1 = fmaf(ca, omk, r1);
            rd = fmaf(cd, omk, rd);
          }
          // t is 0 (then so is the numerator) or far above the subnormal range: the residuals are differences of
          // f32 values of order 1e-3..1 and their blurs, so the flush-to-zero division sees a normal divisor.
          float t = fabsf(r1 - rd) + fabsf(r1);
          float d1 = t > 0.0f ? fdiv_ftz(-rd * (2.0f * r1 - rd), t * (1.0f + fabsf(r1))) : 0.0f;
          float art = fmaxf(d1, 0.0f), det = fmaxf(-d1, 0.0f);
          float d2 = d * d, a2 = art * art, e2 = det * det;
          acc[0] += d;
          acc[1] += d2 * d2;
          acc[2] += art;
          acc[3] += a2 * a2;
          acc[4] += det;
          acc[5] += e2 * e2;
        }
      }
#pragma unroll
      for (int i = 0; i < 6; i++) sums[ch * 6 + i] += acc[i];
    }
  }
  // Warp sums (f32, 32 threads x 4 pixels), then the 8 warps in f64 in a fixed order. Sums 0..15 by a reduce-scatter
  // butterfly: at each exchange (lane distance 16, 8, 4, 2) a lane keeps half of the values it carries and adds its
  // partner's copy of that half, then distance 1 adds the pair; lane l ends with sum l >> 1. The additions are those
  // of a full butterfly per sum, so every sum has the same bits, in 16 shuffles instead of 80. Sums 16 and 17 by full
  // butterflies.
  const int lane = tid & 31, warp = tid >> 5;
  {
    float a[16];
#pragma unroll
    for (int i = 0; i < 16; i++) a[i] = sums[i];
#pragma unroll
    for (int m = 8, off = 16; m >= 1; m >>= 1, off >>= 1) {
      const bool upper = (lane & off) != 0;
#pragma unroll
      for (int i = 0; i < m; i++) {
        const float keep = upper ? a[i + m] : a[i];
        const float send = upper ? a[i] : a[i + m];
        a[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
      }
    }
    a[0] += __shfl_xor_sync(0xffffffffu, a[0], 1);
    if ((lane & 1) == 0) s_red[warp][lane >> 1] = a[0];
  }
#pragma unroll
  for (int i = 16; i < kScoreSums; i++) {
    float v = sums[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) s_red[warp][i] = v;
  }
  __syncthreads();
  if (tid < kScoreSums) {
    double acc = 0.0;
    for (int wi = 0; wi < kTileThreads / 32; wi++) acc += (double)s_red[wi][tid];
    out[(size_t)tid * stride] = acc;  // sum-major: the reduction reads each sum contiguously
  }
}

template <int kRef>
__global__ void __launch_bounds__(kTileThreads, 3)
    k_ssim2_tiles(PyramidDesc pd, const float* __restrict__ ref, const float* __restrict__ dist,
                  double* __restrict__ partials, const StepDesc* __restrict__ st, float2* __restrict__ refm) {
  if (st && !st->active) return;
  const int blk = blockIdx.x;
  int s = 0;
  while (s + 1 < pd.nscales && blk >= pd.s[s + 1].tile0) s++;
  const ScaleDesc sd = pd.s[s];
  ssim2_band<kRef>(sd, blk - sd.tile0, ref, dist, partials + blk, (size_t)pd.total_tiles, refm);
}

// Deterministic reduction of the per-tile sums: CTA (scale, sum index); the last CTA to finish computes the score
// (core/src/ssimulacra2.rs:457-511) and, in a search, advances the bisection (jpeg/src/target.rs:29-56).
// CTA (scale blockIdx.x, sum blockIdx.y) of one score; the last of its nscales x 18 CTAs maps the sums.
__device__ __forceinline__ void reduce_scale_sum(const PyramidDesc& pd, const double* __restrict__ partials,
                                                 double* __restrict__ scale_sums, unsigned* __restrict__ counter,
                                                 double* __restrict__ score_out, SearchState* __restrict__ ss) {
  __shared__ double red[8];
  __shared__ bool last;
  const int s = blockIdx.x, i = blockIdx.y;
  const ScaleDesc sd = pd.s[s];
  const int n = sd.tiles_x * sd.tiles_y;
  double acc = 0.0;
  const double* col = partials + (size_t)i * pd.total_tiles + sd.tile0;
  for (int t = threadIdx.x; t < n; t += 256) acc += col[t];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int wi = 0; wi < 8; wi++) tot += red[wi];
    scale_sums[s * kScoreSums + i] = tot;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    last = prev == (unsigned)(pd.nscales * kScoreSums) - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // The last CTA maps the per-scale sums to the score. Term t follows the reference's weight order: channel, scale,
  // norm (mean, 4-norm), then (ssim, artifact, detail) (core/src/ssimulacra2.rs:491-506); one thread per term, then
  // the terms summed by a fixed pairwise tree (18.4 against 20.5 us per launch for the serial sum).
  __shared__ double terms[3 * kMaxScales * 6];
  const volatile double* vs = scale_sums;
  const int ns = pd.nscales, nterms = 3 * ns * 6, t = threadIdx.x;
  if (t < nterms) {
    int c = t / (ns * 6), rem = t % (ns * 6), sc = rem / 6, r2 = rem % 6, nrm = r2 / 3, k = r2 % 3;
    double count = (double)pd.s[sc].w * (double)pd.s[sc].h;
    double v = vs[sc * kScoreSums + c * 6 + 2 * k + nrm] / count;
    if (nrm == 1) v = sqrt(sqrt(v));  // (sum of 4th powers / count)^0.25 (:462)
    terms[t] = c_weights[t] * fabs(v);
  }
  __syncthreads();
  // Fixed-order pairwise sum of the terms (deterministic; the same tree on every call).
  for (int span = 1; span < nterms; span *= 2) {
    if (t % (2 * span) == 0 && t + span < nterms) terms[t] += terms[t + span];
    __syncthreads();
  }
  if (t != 0) return;
  *counter = 0;
  double ssim = terms[0];
  ssim *= 0.9562382616834844;
  ssim = 2.326765642916932 * ssim - 0.020884521182843837 * ssim * ssim + 6.248496625763138e-05 * ssim * ssim * ssim;
  double score = ssim > 0.0 ? 100.0 - 10.0 * pow(ssim, 0.6276336467831387) : 100.0;
  // A non-finite score is the reference's Err, which the search maps to f64::MIN (cli/src/pipeline.rs:218).
  bool finite = isfinite(score);
  *score_out = finite ? score : NAN;
  if (ss) search_record(ss, finite ? score : -1.7976931348623157e308);
}

__global__ void __launch_bounds__(256) k_ssim2_reduce(PyramidDesc pd, const double* __restrict__ partials,
                                                      double* __restrict__ scale_sums, unsigned* __restrict__ counter,
                                                      double* __restrict__ score_out, SearchState* __restrict__ ss,
                                                      const StepDesc* __restrict__ st) {
  if (st && !st->active) return;
  reduce_scale_sum(pd, partials, scale_sums, counter, score_out, ss);
}

// ------------------------------------------------------------------------------------------------ planes, pyramid

// Linear planes of an interleaved image (core/src/ssimulacra2.rs:177-221, with core/src/image.rs:143-190 for alpha:
// 16-bit samples rounded to 8 bits, then composited onto mid-grey 128). Four consecutive pixels per thread (in
// row-major order; the planes are contiguous [3][h][w]) so each thread moves enough bytes per request.
// CTA `cta` of an image's 4-pixel groups; lut8: the 8-bit table in shared memory.
__device__ __forceinline__ void to_linear_groups(const uint8_t* __restrict__ img, int w, int h, int channels, int depth,
                                                 const float* __restrict__ lut16, float* __restrict__ out,
                                                 size_t cta, const float* lut8) {
  const size_t np = (size_t)w * h;
  const size_t i0 = 4 * (cta * blockDim.x + threadIdx.x);
  if (i0 >= np) return;
  const int n = (int)min((size_t)4, np - i0);
  float v[3][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
  const bool alpha = channels == 2 || channels == 4;
  if (depth == 8 && channels == 3 && n == 4 && ((uintptr_t)img & 3) == 0) {
    // 12 bytes at 12 * (i0/4): 4-byte aligned when the image is (callers may pass any device pointer)
    const uint32_t* p = reinterpret_cast<const uint32_t*>(img + i0 * 3);
    uint32_t q0 = p[0], q1 = p[1], q2 = p[2];
    uint32_t b[12] = {q0 & 0xFF, (q0 >> 8) & 0xFF, (q0 >> 16) & 0xFF, q0 >> 24, q1 & 0xFF, (q1 >> 8) & 0xFF,
                      (q1 >> 16) & 0xFF, q1 >> 24, q2 & 0xFF, (q2 >> 8) & 0xFF, (q2 >> 16) & 0xFF, q2 >> 24};
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int c = 0; c < 3; c++) v[c][k] = lut8[b[3 * k + c]];
  } else {
    for (int k = 0; k < n; k++) {
      size_t i = i0 + k;
      if (depth == 8 && !alpha) {
        if (channels == 1) {
          v[0][k] = v[1][k] = v[2][k] = lut8[img[i]];
        } else {
          v[0][k] = lut8[img[i * 3]];
          v[1][k] = lut8[img[i * 3 + 1]];
          v[2][k] = lut8[img[i * 3 + 2]];
        }
      } else if (!alpha) {
        auto s16 = [&](int c) -> unsigned {
          const uint8_t* p = img + (i * channels + c) * 2;
          return ((unsigned)p[0] << 8) | p[1];
        };
        if (channels == 1) {
          v[0][k] = v[1][k] = v[2][k] = lut16[s16(0)];
        } else {
          v[0][k] = lut16[s16(0)];
          v[1][k] = lut16[s16(1)];
          v[2][k] = lut16[s16(2)];
        }
      } else {
        unsigned sm[4];
        for (int c = 0; c < channels; c++) {
          if (depth == 8) {
            sm[c] = img[i * channels + c];
          } else {
            const uint8_t* p = img + (i * channels + c) * 2;
            unsigned u = ((unsigned)p[0] << 8) | p[1];
            sm[c] = (u * 255 + 32767) / 65535;
          }
        }
        unsigned a = sm[channels - 1];
        auto blend = [&](unsigned c) -> unsigned { return (c * a + 128u * (255 - a) + 127) / 255; };
        if (channels == 2) {
          v[0][k] = v[1][k] = v[2][k] = lut8[blend(sm[0])];
        } else {
          v[0][k] = lut8[blend(sm[0])];
          v[1][k] = lut8[blend(sm[1])];
          v[2][k] = lut8[blend(sm[2])];
        }
      }
    }
  }
  if (n == 4 && np % 4 == 0 && ((uintptr_t)out & 15) == 0) {
#pragma unroll
    for (int c = 0; c < 3; c++)
      *reinterpret_cast<float4*>(out + c * np + i0) = make_float4(v[c][0], v[c][1], v[c][2], v[c][3]);
  } else {
    for (int k = 0; k < n; k++)
#pragma unroll
      for (int c = 0; c < 3; c++) out[c * np + i0 + k] = v[c][k];
  }
}

__global__ void k_to_linear(const uint8_t* __restrict__ img, int w, int h, int channels, int depth,
                            const float* __restrict__ lut16, float* __restrict__ out) {
  // The table lives in shared memory: per-thread indices differ, which would serialize constant-memory reads.
  __shared__ float lut8[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lut8[i] = c_lut8s[i];
  __syncthreads();
  to_linear_groups(img, w, h, channels, depth, lut16, out, blockIdx.x, lut8);
}

// Error-free transform: s + e == a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}

// Mean of the 2x2 block at output (ox, oy) of a plane of w x h (fewer samples at odd edges), as downsample
// (core/src/ssimulacra2.rs:223-247) computes it: the reference sums in f64, which is exact for these inputs, then
// rounds once to f32; the compensated sum here (TwoSum) rounds the same exact sum once, so the planes agree with the
// reference's except in rare double-rounding cases.
// kFresh: the plane was written earlier in the same kernel (the fused upsample + pyramid), so loads go through L2
// (ld.global.cg) and never through the read-only data path, which need not see this kernel's own writes.
template <bool kFresh>
__device__ __forceinline__ float ldp(const float* p) {
  if constexpr (kFresh) return __ldcg(p);
  else return *p;
}
template <bool kFresh>
__device__ __forceinline__ float4 ldp4(const float4* p) {
  if constexpr (kFresh) return __ldcg(p);
  else return *p;
}

template <bool kFresh = false>
__device__ __forceinline__ float mean2x2(const float* p, int stride, int w, int h, int ox, int oy) {
  int x0 = ox * 2, x1 = min(ox * 2 + 2, w), y0 = oy * 2, y1 = min(oy * 2 + 2, h);
  float s = 0.0f, err = 0.0f;
  for (int y = y0; y < y1; y++)
    for (int x = x0; x < x1; x++) {
      float e;
      s = two_sum(s, ldp<kFresh>(p + (size_t)y * stride + x), e);
      err += e;
    }
  // count is 1, 2 or 4: the scaling is exact.
  return __fadd_rn(s, err) * (1.0f / (float)((y1 - y0) * (x1 - x0)));
}

// Every coarser scale of a pyramid from scale 0 in one launch. One CTA owns a kPyrTW x kPyrTH tile of scale 1 (a
// block of scale 0 twice as wide and tall) and the tiles of scales 2-5 below it, each half the one above, kept in
// shared memory between levels: tiles nest exactly because each level halves the previous one, and odd edges occur
// only in the last tile of a row or column, where mean2x2 clips to the level's size. The scale-5 tile is
// kPyrTW/16 x kPyrTH/16.
constexpr int kPyrTW = 32, kPyrTH = 32;
constexpr int kPyrThreads = 256;  // every pyramid launch
static_assert(kPyrTH % 16 == 0 && kPyrTW % 32 == 0 && kPyrTW * kPyrTH % (2 * kPyrThreads) == 0, "pyramid tile");

int pyramid_ctas(const PyramidDesc& pd) {
  if (pd.nscales < 2) return 0;
  return ((pd.s[1].w + kPyrTW - 1) / kPyrTW) * ((pd.s[1].h + kPyrTH - 1) / kPyrTH);
}

// Scale-1 tile (tx, ty) from scale 0 into `out` (shared) and dst1 (global). Each thread takes pairs of adjacent
// outputs, whose 2x4 source samples per channel are two aligned 16-byte loads when the scale-0 rows are (width a
// multiple of 4, planes 16-byte aligned; the usual case); each output sums its four samples in mean2x2's order.
// Partial blocks (the last odd column or row) and unaligned planes take the general path. Source and destination
// are separate restricted pointers, so the loads of later outputs may be issued before the stores of earlier ones.
__device__ __forceinline__ float quad_mean(float q0, float q1, float q2, float q3) {
  float e0, e1, e2;
  float t = two_sum(q0, q1, e0);  // 0 + q0 is exact, so this matches mean2x2's first steps
  t = two_sum(t, q2, e1);
  t = two_sum(t, q3, e2);
  return __fadd_rn(t, (e0 + e1) + e2) * 0.25f;
}

template <bool kFresh>
__device__ __forceinline__ void scale1_tile(const float* __restrict__ src0, float* __restrict__ dst1,
                                            const ScaleDesc& s0, const ScaleDesc& s1, int tx, int ty,
                                            float (*out)[kPyrTH][kPyrTW + 1]) {
  const size_t np0 = (size_t)s0.w * s0.h, np1 = (size_t)s1.w * s1.h;
  const bool vec = (s0.w & 3) == 0 && ((uintptr_t)src0 & 15) == 0;
#pragma unroll
  for (int k = 0; k < kPyrTW * kPyrTH / (2 * kPyrThreads); k++) {
    const int i = threadIdx.x + k * kPyrThreads;
    const int lx = 2 * (i % (kPyrTW / 2)), ly = i / (kPyrTW / 2);
    const int ox = tx * kPyrTW + lx, oy = ty * kPyrTH + ly;
    if (ox >= s1.w || oy >= s1.h) continue;
    float v[2][3];
    const bool two = ox + 1 < s1.w;
    if (vec && 2 * ox + 3 < s0.w && 2 * oy + 1 < s0.h) {
      float4 r0[3], r1[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float4* p = reinterpret_cast<const float4*>(src0 + c * np0 + (size_t)(2 * oy) * s0.w + 2 * ox);
        r0[c] = ldp4<kFresh>(p);
        r1[c] = ldp4<kFresh>(p + s0.w / 4);
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        v[0][c] = quad_mean(r0[c].x, r0[c].y, r1[c].x, r1[c].y);
        v[1][c] = quad_mean(r0[c].z, r0[c].w, r1[c].z, r1[c].w);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int x = ox + j;
        if (j == 1 && !two) break;
        const bool full = 2 * x + 1 < s0.w && 2 * oy + 1 < s0.h;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          if (full) {
            const float* p = src0 + c * np0 + (size_t)(2 * oy) * s0.w + 2 * x;
            v[j][c] = quad_mean(ldp<kFresh>(p), ldp<kFresh>(p + 1), ldp<kFresh>(p + s0.w), ldp<kFresh>(p + s0.w + 1));
          } else {
            v[j][c] = mean2x2<kFresh>(src0 + c * np0, s0.w, s0.w, s0.h, x, oy);
          }
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      out[c][ly][lx] = v[0][c];
      float* d = dst1 + c * np1 + (size_t)oy * s1.w + ox;
      d[0] = v[0][c];
      if (two) {
        out[c][ly][lx + 1] = v[1][c];
        d[1] = v[1][c];
      }
    }
  }
}

// Every output of every level of tile (tx, ty) is a full 2x2 mean (no clipped block at an odd edge).
__device__ __forceinline__ bool pyramid_interior(const PyramidDesc& pd, int tx, int ty) {
  int tw = kPyrTW, th = kPyrTH;
  for (int L = 1; L < pd.nscales; L++) {
    if (2 * (tx + 1) * tw > pd.s[L - 1].w || 2 * (ty + 1) * th > pd.s[L - 1].h) return false;
    tw /= 2;
    th /= 2;
  }
  return true;
}

// Tile (tx, ty) when it is interior and scale 0 takes 16-byte row loads: each thread owns a 2x2 block of scale 1 (its
// 4x4 scale-0 source as 16-byte loads) and so one scale-2 sample, computed in registers; the four scale-2 samples of
// a scale-3 sample sit in one warp (a warp holds two scale-2 rows) and meet by shuffles; scales 4 and 5 (16 and 4
// samples) go through shared memory. Every sample is quad_mean of its four sources in mean2x2's order, as the general
// path computes it for full blocks, so the planes are the same bits.
// Scales 1-5 of interior tile (tx, ty) from the thread's 2x2 block of scale 1 (v1[row][column][channel], at
// scale-1 origin (tx * 32 + 2 (t % 16), ty * 32 + 2 (t / 16))).
__device__ __forceinline__ void pyramid_levels_interior(const PyramidDesc& pd, float* __restrict__ pyr, int tx,
                                                        int ty, const float (&v1)[2][2][3]) {
  static_assert(kPyrTW == 32 && kPyrTH == 32 && kPyrThreads == 256, "thread layout of the interior path");
  __shared__ float l3[3][8][8], l4[3][4][4];
  const ScaleDesc s1 = pd.s[1];
  const size_t np1 = (size_t)s1.w * s1.h;
  const int t = threadIdx.x, bx = t % 16, by = t / 16;
  const int ox = tx * 32 + 2 * bx, oy = ty * 32 + 2 * by;  // scale-1 origin of the thread's 2x2 block
  float* dst1 = pyr + s1.off;
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float* d = dst1 + c * np1 + (size_t)(oy + r) * s1.w + ox;
      d[0] = v1[r][0][c];
      d[1] = v1[r][1][c];
    }
  if (pd.nscales < 3) return;
  const ScaleDesc s2 = pd.s[2];
  const size_t np2 = (size_t)s2.w * s2.h;
  float v2[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    v2[c] = quad_mean(v1[0][0][c], v1[0][1][c], v1[1][0][c], v1[1][1][c]);
    pyr[s2.off + c * np2 + (size_t)(ty * 16 + by) * s2.w + tx * 16 + bx] = v2[c];
  }
  if (pd.nscales < 4) return;
  // Scale 3: lane = 16 * (row parity) + column; the sample at (column pair, warp) takes lanes l, l+1, l+16, l+17.
  const ScaleDesc s3 = pd.s[3];
  const size_t np3 = (size_t)s3.w * s3.h;
  const int lane = t & 31, warp = t >> 5;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float q1 = __shfl_down_sync(0xffffffffu, v2[c], 1);
    const float q2 = __shfl_down_sync(0xffffffffu, v2[c], 16);
    const float q3 = __shfl_down_sync(0xffffffffu, v2[c], 17);
    if (lane < 16 && (lane & 1) == 0) {
      const float v3 = quad_mean(v2[c], q1, q2, q3);
      const int X = lane / 2, Y = warp;
      pyr[s3.off + c * np3 + (size_t)(ty * 8 + Y) * s3.w + tx * 8 + X] = v3;
      l3[c][Y][X] = v3;
    }
  }
  if (pd.nscales < 5) return;
  __syncthreads();
  const ScaleDesc s4 = pd.s[4];
  const size_t np4 = (size_t)s4.w * s4.h;
  if (t < 16) {
    const int X = t % 4, Y = t / 4;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float v4 = quad_mean(l3[c][2 * Y][2 * X], l3[c][2 * Y][2 * X + 1], l3[c][2 * Y + 1][2 * X],
                                 l3[c][2 * Y + 1][2 * X + 1]);
      pyr[s4.off + c * np4 + (size_t)(ty * 4 + Y) * s4.w + tx * 4 + X] = v4;
      l4[c][Y][X] = v4;
    }
  }
  if (pd.nscales < 6 || t >= 32) return;
  __syncwarp();
  const ScaleDesc s5 = pd.s[5];
  const size_t np5 = (size_t)s5.w * s5.h;
  if (t < 4) {
    const int X = t % 2, Y = t / 2;
#pragma unroll
    for (int c = 0; c < 3; c++)
      pyr[s5.off + c * np5 + (size_t)(ty * 2 + Y) * s5.w + tx * 2 + X] =
          quad_mean(l4[c][2 * Y][2 * X], l4[c][2 * Y][2 * X + 1], l4[c][2 * Y + 1][2 * X], l4[c][2 * Y + 1][2 * X + 1]);
  }
}

// Interior tile (tx, ty) from scale 0 in memory: each thread's 4x4 source block as 16-byte row loads.
__device__ __forceinline__ void pyramid_tile_interior(const PyramidDesc& pd, float* __restrict__ pyr, int tx, int ty) {
  const ScaleDesc s0 = pd.s[0];
  const size_t np0 = (size_t)s0.w * s0.h;
  const float* src0 = pyr + s0.off;
  const int t = threadIdx.x, bx = t % 16, by = t / 16;
  const int ox = tx * 32 + 2 * bx, oy = ty * 32 + 2 * by;
  float v1[2][2][3];  // [row][column][channel]
#pragma unroll
  for (int r = 0; r < 2; r++) {
    float4 a0[3], a1[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float4* p = reinterpret_cast<const float4*>(src0 + c * np0 + (size_t)(2 * (oy + r)) * s0.w + 2 * ox);
      a0[c] = p[0];
      a1[c] = p[s0.w / 4];
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      v1[r][0][c] = quad_mean(a0[c].x, a0[c].y, a1[c].x, a1[c].y);
      v1[r][1][c] = quad_mean(a0[c].z, a0[c].w, a1[c].z, a1[c].w);
    }
  }
  pyramid_levels_interior(pd, pyr, tx, ty, v1);
}

__device__ __forceinline__ bool pyramid_fast_tile(const PyramidDesc& pd, const float* pyr, int tx, int ty) {
  return (pd.s[0].w & 3) == 0 && ((uintptr_t)(pyr + pd.s[0].off) & 15) == 0 && pyramid_interior(pd, tx, ty);
}

// Tile (tx, ty) by the general path: scale 1 from scale 0 in memory, then each coarser level from the one above in
// shared memory.
template <bool kFresh>
__device__ __forceinline__ void pyramid_tile_general(const PyramidDesc& pd, float* __restrict__ pyr, int tx, int ty) {
  __shared__ float buf[2][3][kPyrTH][kPyrTW + 1];
  const ScaleDesc s0 = pd.s[0], s1 = pd.s[1];
  scale1_tile<kFresh>(pyr + s0.off, pyr + s1.off, s0, s1, tx, ty, buf[0]);
  int cur = 0, tw = kPyrTW, th = kPyrTH;
  for (int L = 2; L < pd.nscales; L++) {
    __syncthreads();
    const ScaleDesc a = pd.s[L - 1], b = pd.s[L];
    const size_t npb = (size_t)b.w * b.h;
    const int hw = tw / 2, hh = th / 2;
    const int ax0 = tx * tw, ay0 = ty * th;  // tile origin at level L-1
    for (int i = threadIdx.x; i < hw * hh; i += blockDim.x) {
      int lx = i % hw, ly = i / hw;
      int ox = tx * hw + lx, oy = ty * hh + ly;
      if (ox < b.w && oy < b.h) {
        // the 2x2 source block lies in this CTA's level L-1 tile; clip to level L-1's size like mean2x2
        int x1 = min(ox * 2 + 2, a.w) - ax0, y1 = min(oy * 2 + 2, a.h) - ay0;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          float sum = 0.0f, err = 0.0f;
          for (int y = 2 * ly; y < y1; y++)
            for (int x = 2 * lx; x < x1; x++) {
              float e;
              sum = two_sum(sum, buf[cur][c][y][x], e);
              err += e;
            }
          float v = __fadd_rn(sum, err) * (1.0f / (float)((y1 - 2 * ly) * (x1 - 2 * lx)));
          buf[cur ^ 1][c][ly][lx] = v;
          pyr[b.off + c * npb + (size_t)oy * b.w + ox] = v;
        }
      }
    }
    cur ^= 1;
    tw = hw;
    th = hh;
  }
}

// Scale-1 tile `blk` of a pyramid and every coarser tile below it.
__device__ __forceinline__ void pyramid_tile(const PyramidDesc& pd, float* __restrict__ pyr, const int blk) {
  const int tiles_x = (pd.s[1].w + kPyrTW - 1) / kPyrTW;
  const int tx = blk % tiles_x, ty = blk / tiles_x;
  if (pyramid_fast_tile(pd, pyr, tx, ty)) pyramid_tile_interior(pd, pyr, tx, ty);
  else pyramid_tile_general<false>(pd, pyr, tx, ty);
}

__global__ void __launch_bounds__(256, 5) k_pyramid(const __grid_constant__ PyramidDesc pd, float* __restrict__ pyr,
                                                 const StepDesc* __restrict__ st) {
  if (st && !st->active) return;
  pyramid_tile(pd, pyr, blockIdx.x);
}

// A search candidate's linear planes and pyramid in one pass, for the 4:2:0 layouts of upsample420.cuh. CTA = pyramid
// tile (tx, ty): its threads upsample the tile's 64 x 64 block of scale 0 (thread t the 4 x 4 block at columns
// tx * 64 + 4 (t % 16), rows ty * 64 + 4 (t / 16)), write it as scale 0 for the scorer, and, on an interior tile,
// build scale 1 from the same registers: that 4 x 4 block is exactly the source of the thread's 2 x 2 block of scale
// 1 in the pyramid's interior path, so scale 0 is never read back (the separate kernels wrote 144 MB at 12 MP and read
// it back from DRAM). Edge tiles read their block back through L2 after a barrier and take the general path. The
// planes are the same bits as the decoder's upsampling kernel followed by k_pyramid. Measured per 12 MP candidate:
// 63.6 us converting the block as two 2-row halves, 61.0 us with all of its loads issued first (upsample_420_quad),
// against 40.7 + 41.9 us for the two kernels; 72 us at 3 or 5 CTAs per SM.
__global__ void __launch_bounds__(kPyrThreads, 4) k_upsample_pyramid(const StepDesc* __restrict__ st,
                                                                    const uint8_t* __restrict__ planes, int w, int h,
                                                                    const __grid_constant__ PyramidDesc pd,
                                                                    float* __restrict__ pyr) {
  if (!st->active) return;
  __shared__ float lut[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = c_lut8s[i];
  __syncthreads();
  const int tiles_x = (pd.s[1].w + kPyrTW - 1) / kPyrTW;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int t = threadIdx.x, bx = t % 16, by = t / 16;
  const int x0 = tx * 2 * kPyrTW + 4 * bx, j0 = ty * kPyrTH + 2 * by;  // columns x0.., chroma rows j0, j0 + 1
  const size_t np0 = (size_t)w * h;
  float* lin = pyr + pd.s[0].off;
  const bool fast = pyramid_fast_tile(pd, pyr, tx, ty);
  float v1[2][2][3];  // the interior path's scale-1 block: [row][column][channel]
  if (x0 < w && 2 * j0 < h) {
    float l[4][3][4];  // [row][channel][column]
    upsample_420_quad(st, planes, w, h, lut, x0, j0, l);
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int y = 2 * j0 + r;
      if (y >= h) break;
#pragma unroll
      for (int c = 0; c < 3; c++)
        *reinterpret_cast<float4*>(lin + c * np0 + (size_t)y * w + x0) =
            make_float4(l[r][c][0], l[r][c][1], l[r][c][2], l[r][c][3]);
    }
    if (fast) {
#pragma unroll
      for (int r = 0; r < 2; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          v1[r][0][c] = quad_mean(l[2 * r][c][0], l[2 * r][c][1], l[2 * r + 1][c][0], l[2 * r + 1][c][1]);
          v1[r][1][c] = quad_mean(l[2 * r][c][2], l[2 * r][c][3], l[2 * r + 1][c][2], l[2 * r + 1][c][3]);
        }
    }
  }
  if (fast) {
    pyramid_levels_interior(pd, pyr, tx, ty, v1);
    return;
  }
  __syncthreads();  // the tile's scale 0 is written; a block's global writes are visible to it after the barrier
  pyramid_tile_general<true>(pd, pyr, tx, ty);
}

// ------------------------------------------------------------------------------------------------ work-list scorer

// Many (reference, distorted) pairs of any sizes scored together: one launch per stage over a work-list of every
// pair's CTAs (linear planes, pyramid tiles, scorer tiles, reductions). Each stage's CTA finds its pair by a binary
// search over the pairs' first-CTA indices; a pair with no CTAs in a stage has the same first index as the next
// pair, and the search returns the last pair whose first index is <= the CTA's, so it is never chosen. Pairs that
// name the same reference (same device pointer, size and format) share the first such pair's reference planes,
// which are converted once.
struct ScoreItem {
  PyramidDesc pd;
  const uint8_t* img[2];  // reference, distorted (interleaved samples)
  float* pyr[2];          // their pyramids (pyr[0] may be an earlier pair's)
  int channels, depth;
  int own_ref;            // 1: this pair converts its reference; 0: it reuses an earlier pair's planes
  int lin_ctas;           // to_linear CTAs per image
  int pyr_ctas;           // pyramid CTAs per image
  long long lin0, pyr0, tile0;  // first CTA / tile of this pair in each stage (own reference first, then distorted)
  long long part;         // first double of this pair's [18][total_tiles] partial sums
};

// One scale of one pair in the tile work-list, with everything a tile needs resolved on the host.
struct TileSeg {
  const float* ref;   // channel 0 of this scale's planes
  const float* dist;
  double* out;        // partial sums of the segment's first band; band k, sum i at out[i * stride + k]
  int w, h, tiles_x;
  int nch;            // chunks per band
  int stride;         // bands of the pair (the sum-major stride of its partials)
};

// Last index whose first entry is <= x in an ascending array of first indices (n >= 1, first[0] = 0).
__device__ __forceinline__ int find_first(const long long* __restrict__ first, int n, long long x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(first + mid) <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Which image of the pair (0 reference, 1 distorted) and which CTA of it a stage's pair-local CTA index names.
__device__ __forceinline__ int split_image(const ScoreItem& it, long long& local, int per_image) {
  if (it.own_ref && local < per_image) return 0;
  if (it.own_ref) local -= per_image;
  return 1;
}

__global__ void __launch_bounds__(256) k_to_linear_batch(const ScoreItem* __restrict__ items,
                                                         const long long* __restrict__ lin0, int n,
                                                         const float* __restrict__ lut16) {
  __shared__ float lut8[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lut8[i] = c_lut8s[i];
  __syncthreads();
  const int i = find_first(lin0, n, blockIdx.x);
  const ScoreItem& it = items[i];
  long long local = (long long)blockIdx.x - it.lin0;
  const int which = split_image(it, local, it.lin_ctas);
  to_linear_groups(it.img[which], it.pd.s[0].w, it.pd.s[0].h, it.channels, it.depth, lut16, it.pyr[which],
                   (size_t)local, lut8);
}

__global__ void __launch_bounds__(256, 5) k_pyramid_batch(const ScoreItem* __restrict__ items,
                                                          const long long* __restrict__ pyr0, int n) {
  const int i = find_first(pyr0, n, blockIdx.x);
  const ScoreItem& it = items[i];
  long long local = (long long)blockIdx.x - it.pyr0;
  const int which = split_image(it, local, it.pyr_ctas);
  pyramid_tile(it.pd, it.pyr[which], (int)local);
}

// One CTA per tile of the work-list. A persistent form (a fixed grid of k CTAs per SM striding over the list, each
// CTA reusing its shared memory tile after tile) measured slower on 64 pairs of mixed sizes: 22.7 / 25.4 / 38.9 ms
// at k = 3 / 2 / 1 against 21.1 ms here, because the block scheduler hands tiles to whichever CTA slot frees first.
__global__ void __launch_bounds__(kTileThreads, 3)
    k_ssim2_tiles_batch(const TileSeg* __restrict__ segs, const long long* __restrict__ seg0, int nseg) {
  const long long t = blockIdx.x;
  const int g = find_first(seg0, nseg, t);
  const TileSeg sg = segs[g];
  ScaleDesc sd;
  sd.w = sg.w;
  sd.h = sg.h;
  sd.tiles_x = sg.tiles_x;
  sd.tiles_y = 0;
  sd.tile0 = 0;
  sd.nch = sg.nch;
  sd.off = 0;
  const int local = (int)(t - __ldg(seg0 + g));
  ssim2_band<kRefNone>(sd, local, sg.ref, sg.dist, sg.out + local, (size_t)sg.stride, nullptr);
}

// CTA (scale, sum, pair); scale_sums [n][kMaxScales][18], counters and scores [n].
__global__ void __launch_bounds__(256) k_ssim2_reduce_batch(const ScoreItem* __restrict__ items,
                                                            const double* __restrict__ partials,
                                                            double* __restrict__ scale_sums,
                                                            unsigned* __restrict__ counters,
                                                            double* __restrict__ scores) {
  const int p = blockIdx.z;
  const ScoreItem& it = items[p];
  if ((int)blockIdx.x >= it.pd.nscales) return;
  reduce_scale_sum(it.pd, partials + it.part, scale_sums + (size_t)p * kMaxScales * kScoreSums, counters + p,
                   scores + p, nullptr);
}

// ------------------------------------------------------------------------------------------------ lockstep batch

// The scoring half of one bisection step of every image of a lockstep batch (capi.cu): the candidate pyramids, the
// tiles and the reductions, each one launch over a work-list of every image's CTAs; an image whose search has
// finished skips through its StepDesc's `active`.
__global__ void __launch_bounds__(256, 4) k_pyramid_lock(const LockItem* __restrict__ items, int n) {
  const int i = lock_find<&LockItem::p0>(items, n, blockIdx.x);
  const LockItem& it = items[i];
  if (!it.st->active) return;
  pyramid_tile(it.pd, it.dist_pyr, (int)((long long)blockIdx.x - it.p0));
}

template <int kRef>
__global__ void __launch_bounds__(kTileThreads, 3) k_ssim2_tiles_lock(const LockItem* __restrict__ items, int n) {
  const int i = lock_find<&LockItem::t0>(items, n, blockIdx.x);
  const LockItem& it = items[i];
  if (!it.st->active) return;
  const int blk = (int)((long long)blockIdx.x - it.t0);
  int s = 0;
  while (s + 1 < it.pd.nscales && blk >= it.pd.s[s + 1].tile0) s++;
  const ScaleDesc sd = it.pd.s[s];
  ssim2_band<kRef>(sd, blk - sd.tile0, it.ref_pyr, it.dist_pyr, it.partials + blk, (size_t)it.pd.total_tiles,
                   it.refm);
}

__global__ void __launch_bounds__(256) k_ssim2_reduce_lock(const LockItem* __restrict__ items) {
  const LockItem& it = items[blockIdx.z];
  if (!it.st->active || (int)blockIdx.x >= it.pd.nscales) return;
  reduce_scale_sum(it.pd, it.partials, it.scale_sums, it.counter, it.score, it.ss);
}

void lock_step_score(rcg_ctx* ctx, const LockItem* d_items, int n, long long p_total, long long t_total,
                     int max_scales, int ref_mode) {
  if (p_total > 0) RCG_LAUNCH(ctx, "pyramid_lock", k_pyramid_lock, (unsigned)p_total, 256, 0, d_items, n);
  // Every image of the batch is at the same step: the first stores its reference moments, the later ones read them.
  if (ref_mode == kRefWrite)
    RCG_LAUNCH(ctx, "ssim2_tiles_lock", k_ssim2_tiles_lock<kRefWrite>, (unsigned)t_total, kTileThreads, kTileSmem,
               d_items, n);
  else if (ref_mode == kRefRead)
    RCG_LAUNCH(ctx, "ssim2_tiles_lock", k_ssim2_tiles_lock<kRefRead>, (unsigned)t_total, kTileThreads, kTileSmem,
               d_items, n);
  else
    RCG_LAUNCH(ctx, "ssim2_tiles_lock", k_ssim2_tiles_lock<kRefNone>, (unsigned)t_total, kTileThreads, kTileSmem,
               d_items, n);
  RCG_LAUNCH(ctx, "ssim2_reduce_lock", k_ssim2_reduce_lock, dim3(max_scales, kScoreSums, n), 256, 0, d_items);
}

int to_linear(rcg_ctx* ctx, const uint8_t* d_img, int w, int h, int channels, int depth, float* d_pyr) {
  const float* lut16 = nullptr;
  if (depth == 16 && channels != 2 && channels != 4) {
    lut16 = srgb_lut16_device(ctx);
    if (!lut16) return RCG_NO_MEMORY;
  }
  const long long groups = ((long long)w * h + 3) / 4;
  RCG_LAUNCH(ctx, "to_linear", k_to_linear, (unsigned)((groups + 255) / 256), 256, 0, d_img, w, h, channels, depth,
             lut16, d_pyr);
  return RCG_OK;
}

int build_pyramid_gated(rcg_ctx* ctx, const PyramidDesc& pd, float* d_pyr, const StepDesc* st) {
  if (pd.nscales < 2) return RCG_OK;
  RCG_LAUNCH(ctx, "pyramid", k_pyramid, pyramid_ctas(pd), kPyrThreads, 0, pd, d_pyr, st);
  return RCG_OK;
}

int build_pyramid(rcg_ctx* ctx, const PyramidDesc& pd, float* d_pyr) {
  return build_pyramid_gated(ctx, pd, d_pyr, nullptr);
}

int upsample_pyramid(rcg_ctx* ctx, StepDesc* d_step, const uint8_t* d_planes, int w, int h, const PyramidDesc& pd,
                     float* d_pyr) {
  if (pd.nscales < 2) return upsample_color(ctx, d_step, d_planes, w, h, nullptr, d_pyr + pd.s[0].off);
  RCG_LAUNCH(ctx, "upsample_pyramid", k_upsample_pyramid, pyramid_ctas(pd), kPyrThreads, 0, d_step, d_planes, w, h,
             pd, d_pyr);
  return RCG_OK;
}

PyramidDesc make_pyramid(int w, int h) {
  PyramidDesc pd;
  std::memset(&pd, 0, sizeof pd);
  long long off = 0;
  int tiles = 0;
  for (int s = 0; s < kMaxScales; s++) {
    if (w < kMinSide || h < kMinSide) break;
    ScaleDesc& sd = pd.s[s];
    sd.w = w;
    sd.h = h;
    sd.tiles_x = (w + kTileW - 1) / kTileW;
    sd.tiles_y = (h + kTileH - 1) / kTileH;
    sd.tile0 = tiles;
    sd.nch = 1;
    sd.chunk0 = tiles;
    sd.off = off;
    tiles += sd.tiles_x * sd.tiles_y;
    off += 3LL * w * h;
    pd.nscales = s + 1;
    w = (w + 1) / 2;
    h = (h + 1) / 2;
  }
  pd.total_tiles = tiles;
  pd.total_chunks = tiles;
  pd.floats = off;
  return pd;
}

static std::mutex g_scorer_mu;
static bool g_scorer_ready[64];

// Upload the scorer's constant tables to the current device once (cudaMemcpyToSymbol only; nothing is allocated).
// core/src/ssimulacra2.rs:54-163 (WEIGHTS)
static const double kScorerWeights[108] = {
    0.0, 0.0007376606707406586, 0.0, 0.0, 0.0007793481682867309, 0.0,
    0.0, 0.0004371155730107379, 0.0, 1.1041726426657346, 0.00066284834129271, 0.00015231632783718752,
    0.0, 0.0016406437456599754, 0.0, 1.8422455520539298, 11.441172603757666, 0.0,
    0.0007989109436015163, 0.000176816438078653, 0.0, 1.8787594979546387, 10.94906990605142, 0.0,
    0.0007289346991508072, 0.9677937080626833, 0.0, 0.00014003424285435884, 0.9981766977854967, 0.00031949755934435053,
    0.0004550992113792063, 0.0, 0.0, 0.0013648766163243398, 0.0, 0.0,
    0.0, 0.0, 0.0, 7.466890328078848, 0.0, 17.445833984131262,
    0.0006235601634041466, 0.0, 0.0, 6.683678146179332, 0.00037724407979611296, 1.027889937768264,
    225.20515300849274, 0.0, 0.0, 19.213238186143016, 0.0011401524586618361, 0.001237755635509985,
    176.39317598450694, 0.0, 0.0, 24.43300999870476, 0.28520802612117757, 0.0004485436923833408,
    0.0, 0.0, 0.0, 34.77906344483772, 44.835625328877896, 0.0,
    0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
    0.0, 0.0008680556573291698, 0.0, 0.0, 0.0, 0.0,
    0.0, 0.0005313191874358747, 0.0, 0.00016533814161379112, 0.0, 0.0,
    0.0, 0.0, 0.0, 0.0004179171803251336, 0.0017290828234722833, 0.0,
    0.0020827005846636437, 0.0, 0.0, 8.826982764996862, 23.19243343998926, 0.0,
    95.1080498811086, 0.9863978034400682, 0.9834382792465353, 0.0012286405048278493, 171.2667255897307, 0.9807858872435379,
    0.0, 0.0, 0.0, 0.0005130064588990679, 0.0, 0.00010854057858411537};

const double* scorer_weights() { return kScorerWeights; }

static cudaError_t scorer_constants(int device) {
  std::lock_guard<std::mutex> lk(g_scorer_mu);
  if (device >= 0 && device < 64 && g_scorer_ready[device]) return cudaSuccess;
  // core/src/ssimulacra2.rs:260-271 (kernel): f64 taps, rounded to f32 here.
  double k[2 * kRadius + 1], sum = 0.0;
  for (int i = 0; i < 2 * kRadius + 1; i++) {
    double x = (double)i - (double)kRadius;
    k[i] = std::exp(-0.5 / (1.5 * 1.5) * x * x);
    sum += k[i];
  }
  // Taps i and 2 kRadius - i have the same x * x, hence the same f32 value: the tile kernel holds six distinct taps.
  float kf[2 * kRadius + 1];
  for (int i = 0; i < 2 * kRadius + 1; i++) kf[i] = (float)(k[i] / sum);
  float lut[256];
  srgb_lut8(lut);
  const double* W = scorer_weights();
  cudaError_t e;
  if ((e = cudaMemcpyToSymbol(c_gauss, kf, sizeof kf)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_lut8s, lut, sizeof lut)) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_weights, W, sizeof c_weights)) != cudaSuccess) return e;
  if (int ce = codec_upload_lut(lut)) return (cudaError_t)ce;
  if ((e = cudaFuncSetAttribute(k_ssim2_tiles<kRefNone>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_ssim2_tiles<kRefWrite>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_ssim2_tiles<kRefRead>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_ssim2_tiles_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_ssim2_tiles_lock<kRefNone>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_ssim2_tiles_lock<kRefWrite>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_ssim2_tiles_lock<kRefRead>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmem)) != cudaSuccess)
    return e;
  if (device >= 0 && device < 64) g_scorer_ready[device] = true;
  return cudaSuccess;
}

int scorer_init(rcg_ctx* ctx) {
  cudaError_t e = scorer_constants(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "scorer constant tables");
  return RCG_OK;
}

// ------------------------------------------------------------------------------------------------ band autotuner

// Bands pay off where a scale has enough tiles to keep every SM busy with long CTAs; smaller scales (and whole
// images below kBandMinTiles0 scale-0 tiles, which are never tuned) keep 32x32 tiles.
constexpr int kBandMinTiles = 3 * 152;
constexpr int kBandMinTiles0 = 1024;
constexpr int kBandCandidates[] = {1, 2, 4, 8};

PyramidDesc banded(const PyramidDesc& pd, int nch0, int min_tiles) {
  PyramidDesc b = pd;
  int total = 0, chunks = 0;
  for (int s = 0; s < pd.nscales; s++) {
    ScaleDesc& sd = b.s[s];
    const int tiles = pd.s[s].tiles_x * pd.s[s].tiles_y;
    const int n = (nch0 > 1 && tiles >= min_tiles) ? std::min(nch0, pd.s[s].tiles_y) : 1;
    sd.nch = n;
    sd.tiles_y = (pd.s[s].tiles_y + n - 1) / n;
    sd.tile0 = total;
    sd.chunk0 = chunks;
    total += sd.tiles_x * sd.tiles_y;
    chunks += sd.tiles_x * sd.tiles_y * n;
  }
  b.total_tiles = total;
  b.total_chunks = chunks;
  return b;
}

// Deterministic stand-in content for the tuning runs (linear values in [0, 1), the second image a perturbed copy);
// the kernel's time does not depend on the values.
__global__ void k_tune_fill(float* __restrict__ p, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    uint32_t x = (uint32_t)(i % (n / 2)) * 2654435761u;
    x ^= x >> 15;
    float v = (float)(x & 0xFFFFFF) * (1.0f / 16777216.0f);
    p[i] = i < n / 2 ? v : fminf(1.0f, v * 0.98f + 0.01f);
  }
}

static std::mutex g_band_mu;
static std::map<std::pair<int, int>, int> g_band_choice;  // (device, size class) -> chunks per band

// Size class: scale-0 tiles in half-octave steps.
static int band_class(const PyramidDesc& pd) {
  const double t = (double)pd.s[0].tiles_x * pd.s[0].tiles_y;
  return (int)std::floor(2.0 * std::log2(std::max(1.0, t)));
}

// Time k_ssim2_tiles for each candidate on a stand-in pair of this geometry (own allocation, freed after); the
// fastest by the best of three launches wins.
static int tune_bands(rcg_ctx* ctx, const PyramidDesc& pd) {
  float* pyr = nullptr;
  double* part = nullptr;
  const long long n = 2 * pd.floats;
  if (cudaMalloc(&pyr, (size_t)n * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&part, (size_t)pd.total_tiles * kScoreSums * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    if (pyr) cudaFree(pyr);
    return 1;  // no room to tune: tiles
  }
  k_tune_fill<<<4 * 152, 256, 0, ctx->stream>>>(pyr, n);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int best = 1;
  float best_ms = 1e30f;
  for (int nch0 : kBandCandidates) {
    const PyramidDesc pb = banded(pd, nch0, kBandMinTiles);
    float t = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
      cudaEventRecord(a, ctx->stream);
      k_ssim2_tiles<kRefNone><<<pb.total_tiles, kTileThreads, kTileSmem, ctx->stream>>>(pb, pyr, pyr + pd.floats,
                                                                                        part, nullptr, nullptr);
      cudaEventRecord(b, ctx->stream);
      cudaEventSynchronize(b);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, a, b);
      if (rep > 0) t = std::min(t, ms);  // the first launch warms up
    }
    if (t < best_ms * 0.99f) {  // a longer band must win by more than noise
      best_ms = t;
      best = nch0;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(pyr);
  cudaFree(part);
  cudaGetLastError();
  return best;
}

PyramidDesc plan_bands(rcg_ctx* ctx, const PyramidDesc& pd) {
  // A fixed choice applies at every scale; a tuned one only where a scale has tiles enough to fill the GPU.
  return banded(pd, band_chunks(ctx, pd), ctx->band_chunks > 0 ? 0 : kBandMinTiles);
}

int band_chunks(rcg_ctx* ctx, const PyramidDesc& pd) {
  if (ctx->band_chunks > 0) return ctx->band_chunks;
  if (pd.nscales == 0 || pd.s[0].tiles_x * pd.s[0].tiles_y < kBandMinTiles0) return 1;
  const auto key = std::make_pair(ctx->device, band_class(pd));
  std::lock_guard<std::mutex> lk(g_band_mu);
  auto it = g_band_choice.find(key);
  if (it != g_band_choice.end()) return it->second;
  const int best = tune_bands(ctx, pd);
  g_band_choice[key] = best;
  return best;
}

int score_workspace(rcg_ctx* ctx, const PyramidDesc& pd) {
  double* partials = (double*)workspace(ctx, "score_partials", (size_t)pd.total_tiles * kScoreSums * sizeof(double));
  double* scale_sums = (double*)workspace(ctx, "score_scale_sums", kMaxScales * kScoreSums * sizeof(double));
  unsigned* counter = (unsigned*)workspace(ctx, "score_counter", 256);
  return partials && scale_sums && counter ? RCG_OK : RCG_NO_MEMORY;
}

int score_pyramids(rcg_ctx* ctx, const PyramidDesc& pd, const float* d_ref, const float* d_dist, double* d_score,
                   SearchState* search, StepDesc* step, float2* refm, int ref_mode) {
  if (score_workspace(ctx, pd) != RCG_OK) return RCG_NO_MEMORY;
  double* partials = (double*)ctx->bufs["score_partials"].ptr;
  double* scale_sums = (double*)ctx->bufs["score_scale_sums"].ptr;
  unsigned* counter = (unsigned*)ctx->bufs["score_counter"].ptr;
  const PyramidDesc pb = plan_bands(ctx, pd);
  if (!refm || ref_mode == kRefNone)
    RCG_LAUNCH(ctx, "ssim2_tiles", k_ssim2_tiles<kRefNone>, pb.total_tiles, kTileThreads, kTileSmem, pb, d_ref, d_dist,
               partials, step, nullptr);
  else if (ref_mode == kRefWrite)
    RCG_LAUNCH(ctx, "ssim2_tiles_store", k_ssim2_tiles<kRefWrite>, pb.total_tiles, kTileThreads, kTileSmem, pb, d_ref,
               d_dist, partials, step, refm);
  else
    RCG_LAUNCH(ctx, "ssim2_tiles_cached", k_ssim2_tiles<kRefRead>, pb.total_tiles, kTileThreads, kTileSmem, pb, d_ref,
               d_dist, partials, step, refm);
  dim3 rg(pb.nscales, kScoreSums);
  RCG_LAUNCH(ctx, "ssim2_reduce", k_ssim2_reduce, rg, 256, 0, pb, partials, scale_sums, counter, d_score, search,
             step);
  return RCG_OK;
}

int score_batch(rcg_ctx* ctx, int n, const uint8_t* const* d_refs, const uint8_t* const* d_dists,
                const uint32_t* widths, const uint32_t* heights, const int* channels, const int* depths,
                double** d_scores) {
  std::vector<ScoreItem> items((size_t)n);
  std::vector<long long> off_ref((size_t)n, -1), off_dist((size_t)n);
  std::vector<int> ref_of((size_t)n);
  std::map<std::tuple<const uint8_t*, uint32_t, uint32_t, int, int>, int> first_ref;
  long long lin = 0, pyr = 0, tiles = 0, parts = 0, floats = 0;
  int max_scales = 1;
  bool need16 = false;
  auto align64 = [](long long f) { return (f + 63) / 64 * 64; };  // 256-byte plane starts (vector stores)
  for (int i = 0; i < n; i++) {
    ScoreItem& it = items[(size_t)i];
    std::memset(&it, 0, sizeof it);
    const int w = (int)widths[i], h = (int)heights[i];
    it.pd = make_pyramid(w, h);
    it.pd = plan_bands(ctx, it.pd);
    it.img[0] = d_refs[i];
    it.img[1] = d_dists[i];
    it.channels = channels[i];
    it.depth = depths ? depths[i] : 8;
    auto key = std::make_tuple(d_refs[i], widths[i], heights[i], it.channels, it.depth);
    auto found = first_ref.find(key);
    it.own_ref = found == first_ref.end();
    if (it.own_ref) {
      first_ref.emplace(key, i);
      ref_of[(size_t)i] = i;
      off_ref[(size_t)i] = floats;
      floats = align64(floats + it.pd.floats);
    } else {
      ref_of[(size_t)i] = found->second;
    }
    off_dist[(size_t)i] = floats;
    floats = align64(floats + it.pd.floats);
    const int copies = it.own_ref ? 2 : 1;
    it.lin_ctas = (int)((((long long)w * h + 3) / 4 + 255) / 256);
    it.pyr_ctas = pyramid_ctas(it.pd);
    it.lin0 = lin;
    lin += (long long)copies * it.lin_ctas;
    it.pyr0 = pyr;
    pyr += (long long)copies * it.pyr_ctas;
    it.tile0 = tiles;
    tiles += it.pd.total_tiles;
    it.part = parts;
    parts += (long long)kScoreSums * it.pd.total_tiles;
    max_scales = std::max(max_scales, it.pd.nscales);
    need16 |= it.depth == 16 && it.channels != 2 && it.channels != 4;
  }
  if (lin > INT32_MAX || pyr > INT32_MAX || tiles > INT32_MAX)
    return fail(ctx, RCG_INVALID, "batch too large for one launch");
  float* pyr_base = (float*)workspace(ctx, "batch_pyr", (size_t)floats * sizeof(float));
  double* partials = (double*)workspace(ctx, "batch_partials", (size_t)parts * sizeof(double));
  double* sums = (double*)workspace(ctx, "batch_sums", (size_t)n * kMaxScales * kScoreSums * sizeof(double));
  unsigned* counters = (unsigned*)workspace(ctx, "batch_counters", (size_t)n * sizeof(unsigned));
  double* scores = (double*)workspace(ctx, "batch_scores", (size_t)n * sizeof(double));
  // The work-list in one upload: pairs, their first to_linear / pyramid CTAs, then the tile segments (one per
  // pair and scale) and their first tiles.
  int nseg = 0;
  for (const ScoreItem& it : items) nseg += it.pd.nscales;
  const size_t o_lin = (size_t)n * sizeof(ScoreItem), o_pyr = o_lin + (size_t)n * 8,
               o_seg = o_pyr + (size_t)n * 8, o_seg0 = o_seg + (size_t)nseg * sizeof(TileSeg),
               list_bytes = o_seg0 + (size_t)nseg * 8;
  unsigned char* d_list = (unsigned char*)workspace(ctx, "batch_items", list_bytes);
  const float* lut16 = need16 ? srgb_lut16_device(ctx) : nullptr;
  if (!pyr_base || !partials || !sums || !counters || !scores || !d_list || (need16 && !lut16)) return RCG_NO_MEMORY;
  std::vector<unsigned char> list(list_bytes);
  long long* lin0 = (long long*)(list.data() + o_lin);
  long long* pyr0 = (long long*)(list.data() + o_pyr);
  TileSeg* segs = (TileSeg*)(list.data() + o_seg);
  long long* seg0 = (long long*)(list.data() + o_seg0);
  int g = 0;
  for (int i = 0; i < n; i++) {
    ScoreItem& it = items[(size_t)i];
    it.pyr[0] = pyr_base + off_ref[(size_t)ref_of[(size_t)i]];
    it.pyr[1] = pyr_base + off_dist[(size_t)i];
    lin0[i] = it.lin0;
    pyr0[i] = it.pyr0;
    for (int sc = 0; sc < it.pd.nscales; sc++, g++) {
      const ScaleDesc& sd = it.pd.s[sc];
      segs[g].ref = it.pyr[0] + sd.off;
      segs[g].dist = it.pyr[1] + sd.off;
      segs[g].out = partials + it.part + sd.tile0;
      segs[g].w = sd.w;
      segs[g].h = sd.h;
      segs[g].tiles_x = sd.tiles_x;
      segs[g].nch = sd.nch;
      segs[g].stride = it.pd.total_tiles;
      seg0[g] = it.tile0 + sd.tile0;
    }
  }
  std::memcpy(list.data(), items.data(), o_lin);
  cudaError_t e = cudaMemcpyAsync(d_list, list.data(), list_bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch work-list upload");
  const ScoreItem* d_items = (const ScoreItem*)d_list;
  const long long* d_lin0 = (const long long*)(d_list + o_lin);
  const long long* d_pyr0 = (const long long*)(d_list + o_pyr);
  const TileSeg* d_segs = (const TileSeg*)(d_list + o_seg);
  const long long* d_seg0 = (const long long*)(d_list + o_seg0);
  // The launches take only the work-list's totals and this context's buffers: a later batch with the same totals
  // replays them (its own pairs come in through the work-list uploaded above).
  const std::vector<long long> key = {3, n, nseg, lin, pyr, tiles, max_scales, (long long)(uintptr_t)lut16};
  int rc = run_step_loop(ctx, key, [&]() {
    RCG_LAUNCH(ctx, "to_linear_batch", k_to_linear_batch, (unsigned)lin, 256, 0, d_items, d_lin0, n, lut16);
    if (pyr > 0) RCG_LAUNCH(ctx, "pyramid_batch", k_pyramid_batch, (unsigned)pyr, 256, 0, d_items, d_pyr0, n);
    RCG_LAUNCH(ctx, "ssim2_tiles_batch", k_ssim2_tiles_batch, (unsigned)tiles, kTileThreads, kTileSmem, d_segs,
               d_seg0, nseg);
    RCG_LAUNCH(ctx, "ssim2_reduce_batch", k_ssim2_reduce_batch, dim3(max_scales, kScoreSums, n), 256, 0, d_items,
               partials, sums, counters, scores);
  });
  if (rc != RCG_OK) return rc;
  *d_scores = scores;
  return RCG_OK;
}

}  // namespace rcg

// ------------------------------------------------------------------------------------------------ no-alloc scorer

namespace rcg {

// Fixed scratch of rcg_ssimulacra2_device_noalloc: both images' linear pyramids, the per-tile partial sums, the
// per-scale sums and the reduction's completion counter. Sized for images of at most kNoAllocMaxPixels pixels. CUDA
// places a module's device arrays on a device when the module is first used there, so every device where any scorer
// call has run holds it (about 10 MB) until the process exits. The per-device set-up below is cached for the life of
// the process; a cudaDeviceReset invalidates it and is not supported.
constexpr long long kNoAllocMaxPixels = 512LL * 512LL;
constexpr long long kNoAllocPyrFloats = 1200000;  // one image: 3 channels x every scale, with margin
constexpr int kNoAllocMaxTiles = 4096;
constexpr size_t kNoAllocPyrBytes = (size_t)kNoAllocPyrFloats * sizeof(float);
constexpr size_t kNoAllocPartialOff = 2 * kNoAllocPyrBytes;
constexpr size_t kNoAllocSumsOff = kNoAllocPartialOff + (size_t)kNoAllocMaxTiles * kScoreSums * sizeof(double);
constexpr size_t kNoAllocCounterOff = kNoAllocSumsOff + (size_t)kMaxScales * kScoreSums * sizeof(double);
constexpr size_t kNoAllocBytes = kNoAllocCounterOff + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

static std::mutex g_noalloc_mu;
static unsigned char* g_noalloc_addr[64];

// Once per device, with that device current: the device address of the scratch (host code cannot use the symbol
// itself, which names a host-side shadow) and the scorer's constant tables.
static int noalloc_setup(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return RCG_CUDA_ERROR;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return RCG_CUDA_ERROR;
    }
    if (scorer_constants(dev) != cudaSuccess) {
      cudaGetLastError();
      return RCG_CUDA_ERROR;
    }
    g_noalloc_addr[dev] = (unsigned char*)p;
  }
  *out = g_noalloc_addr[dev];
  return RCG_OK;
}

}  // namespace rcg

extern "C" int rcg_ssimulacra2_device_noalloc(const uint8_t* d_reference, const uint8_t* d_distorted,
                                              uint32_t width, uint32_t height, int channels, double* d_score,
                                              void* stream) {
  using namespace rcg;
  if (!d_reference || !d_distorted || !d_score) return RCG_INVALID;
  if (channels != 1 && channels != 3) return RCG_INVALID;
  if (width < (uint32_t)kMinSide || height < (uint32_t)kMinSide) return RCG_INVALID;
  if ((long long)width * (long long)height > kNoAllocMaxPixels) return RCG_INVALID;
  const int w = (int)width, h = (int)height;
  PyramidDesc pd = make_pyramid(w, h);
  if (pd.floats > kNoAllocPyrFloats || pd.total_tiles > kNoAllocMaxTiles) return RCG_INVALID;
  unsigned char* base = nullptr;
  int rc = noalloc_setup(&base);
  if (rc != RCG_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  float* pyr_ref = (float*)base;
  float* pyr_dist = (float*)(base + kNoAllocPyrBytes);
  double* partials = (double*)(base + kNoAllocPartialOff);
  double* sums = (double*)(base + kNoAllocSumsOff);
  unsigned* counter = (unsigned*)(base + kNoAllocCounterOff);
  // The scratch keeps whatever the previous call left: the completion counter must start at zero.
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned), s) != cudaSuccess) {
    cudaGetLastError();
    return RCG_CUDA_ERROR;
  }
  const unsigned lg = (unsigned)((((long long)w * h + 3) / 4 + 255) / 256);
  k_to_linear<<<lg, 256, 0, s>>>(d_reference, w, h, channels, 8, nullptr, pyr_ref);
  k_to_linear<<<lg, 256, 0, s>>>(d_distorted, w, h, channels, 8, nullptr, pyr_dist);
  if (pd.nscales > 1) {
    const int pg = pyramid_ctas(pd);
    k_pyramid<<<pg, kPyrThreads, 0, s>>>(pd, pyr_ref, nullptr);
    k_pyramid<<<pg, kPyrThreads, 0, s>>>(pd, pyr_dist, nullptr);
  }
  k_ssim2_tiles<kRefNone><<<pd.total_tiles, kTileThreads, kTileSmem, s>>>(pd, pyr_ref, pyr_dist, partials, nullptr,
                                                                        nullptr);
  k_ssim2_reduce<<<dim3(pd.nscales, kScoreSums), 256, 0, s>>>(pd, partials, sums, counter, d_score, nullptr,
                                                              nullptr);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RCG_OK : RCG_CUDA_ERROR;
}
