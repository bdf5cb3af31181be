// The search's common decode case, shared by the decoder's upsampling kernel (codec.cu) and the fused
// upsample + pyramid kernel of the scorer (ssim2.cu): 3 components at 4:2:0 with luma at full resolution, linear
// planes only, w % 4 == 0. Integer arithmetic and a table lookup only, so both translation units give the same bits.
#pragma once

#include <stdint.h>

#include "rcg_internal.cuh"

namespace rcg {

// Four chroma samples of row r, columns i-1 .. i+2 clamped to [0, cw-1], packed little-endian: two aligned 32-bit
// loads and a funnel shift wherever no clamping applies and both words lie inside the row (rows start 8-byte
// aligned), the clamped byte path at the edges.
__device__ __forceinline__ uint32_t chroma4(const uint8_t* __restrict__ r, int i, int cw, int cstride) {
  const int a = (i - 1) & ~3;
  if (i >= 1 && i + 2 <= cw - 1 && a + 8 <= cstride) {
    const uint32_t* q = reinterpret_cast<const uint32_t*>(r + a);
    return __funnelshift_r(q[0], q[1], 8 * ((i - 1) & 3));
  }
  uint32_t v = 0;
#pragma unroll
  for (int d = 0; d < 4; d++) v |= (uint32_t)r[min(max(i - 1 + d, 0), cw - 1)] << (8 * d);
  return v;
}

// The triangle filter of jpeg/src/decode.rs:1806-1818 at columns x0 .. x0+3 (x0 even) of one output row, from its
// near chroma row rn and far chroma row rf (chroma4 words at i = x0/2).
__device__ __forceinline__ void chroma_up(uint32_t rn, uint32_t rf, int (&out)[4]) {
  int vert[4];
#pragma unroll
  for (int d = 0; d < 4; d++) vert[d] = 3 * (int)((rn >> (8 * d)) & 0xFF) + (int)((rf >> (8 * d)) & 0xFF);
  out[0] = (3 * vert[1] + vert[0] + 8) >> 4;
  out[1] = (3 * vert[1] + vert[2] + 7) >> 4;
  out[2] = (3 * vert[2] + vert[1] + 8) >> 4;
  out[3] = (3 * vert[2] + vert[3] + 7) >> 4;
}

// Fixed-point YCbCr -> RGB (jpeg/src/decode.rs:1438-1441) of 4 pixels (luma bytes in q) and the sRGB table.
__device__ __forceinline__ void ycc_linear(uint32_t q, const int (&cb4)[4], const int (&cr4)[4], const float* lut,
                                           float (&l)[3][4]) {
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int yv = (q >> (8 * k)) & 0xFF;
    const int cb = cb4[k] - 128, cr = cr4[k] - 128;
    l[0][k] = lut[min(max(yv + ((91881 * cr + 32768) >> 16), 0), 255)];
    l[1][k] = lut[min(max(yv - ((22554 * cb + 46802 * cr + 32768) >> 16), 0), 255)];
    l[2][k] = lut[min(max(yv + ((116130 * cb + 32768) >> 16), 0), 255)];
  }
}

// Linear-light values of 4 columns (x0 .. x0+3, x0 % 4 == 0) x 2 rows (2j, 2j+1) of the candidate. Both output rows
// share the near chroma row j, so three chroma rows per component feed 8 pixels. l[par] is left untouched for a row
// 2j + par >= h.
__device__ __forceinline__ void upsample_420_rows(const StepDesc* __restrict__ st, const uint8_t* __restrict__ planes,
                                                  int w, int h, const float* lut, int x0, int j,
                                                  float (&l)[2][3][4]) {
  const CompDesc c0 = st->comp[0];
  const int cstride = st->comp[1].bw * 8;
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  const int i = x0 / 2;
  const int jm = max(j - 1, 0), jp = min(j + 1, ch - 1);
  int up[2][2][4];  // [component][row parity][column]
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const uint8_t* p = planes + st->comp[1 + c].plane_off;
    const uint32_t rn = chroma4(p + (size_t)j * cstride, i, cw, cstride),
                   rm = chroma4(p + (size_t)jm * cstride, i, cw, cstride),
                   rp = chroma4(p + (size_t)jp * cstride, i, cw, cstride);
    chroma_up(rn, rm, up[c][0]);  // far row: j-1 for the even output row
    chroma_up(rn, rp, up[c][1]);  // j+1 for the odd one
  }
#pragma unroll
  for (int par = 0; par < 2; par++) {
    const int y = 2 * j + par;
    if (y >= h) break;
    const uint32_t q = *reinterpret_cast<const uint32_t*>(planes + c0.plane_off + (size_t)y * (c0.bw * 8) + x0);
    ycc_linear(q, up[0][par], up[1][par], lut, l[par]);
  }
}

// The same for 4 x 4 pixels: columns x0 .. x0+3, rows 2 j0 .. 2 j0 + 3 (chroma rows j0 and j0 + 1, which share two
// of their four source rows j0-1 .. j0+2). Every load is issued before any pixel is converted: 8 chroma words and
// 4 luma words per thread. l[r] is left untouched for a row 2 j0 + r >= h.
__device__ __forceinline__ void upsample_420_quad(const StepDesc* __restrict__ st, const uint8_t* __restrict__ planes,
                                                  int w, int h, const float* lut, int x0, int j0,
                                                  float (&l)[4][3][4]) {
  const CompDesc c0 = st->comp[0];
  const int cstride = st->comp[1].bw * 8;
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  const int i = x0 / 2;
  uint32_t rows[2][4];  // [component][chroma row j0-1+d, clamped to [0, ch-1]]
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const uint8_t* p = planes + st->comp[1 + c].plane_off;
#pragma unroll
    for (int d = 0; d < 4; d++) rows[c][d] = chroma4(p + (size_t)min(max(j0 - 1 + d, 0), ch - 1) * cstride, i, cw, cstride);
  }
  uint32_t q[4];
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int y = 2 * j0 + r;
    q[r] = y < h ? *reinterpret_cast<const uint32_t*>(planes + c0.plane_off + (size_t)y * (c0.bw * 8) + x0) : 0u;
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    if (2 * j0 + r >= h) break;
    // output row 2 j0 + r: near chroma row j0 + r/2 (rows[.][1 + r/2]); far row j0 + r/2 - 1 for an even row, + 1
    // for an odd one (rows[.][r/2] or rows[.][2 + r/2]), both clamped as jpeg/src/decode.rs:1806-1818 clamps them
    const int nd = 1 + r / 2, fd = (r & 1) ? 2 + r / 2 : r / 2;
    int cb[4], cr[4];
    chroma_up(rows[0][nd], rows[0][fd], cb);
    chroma_up(rows[1][nd], rows[1][fd], cr);
    ycc_linear(q[r], cb, cr, lut, l[r]);
  }
}

// Whether a candidate's layout is that case (the decoder's and the fused kernel's test, evaluated on the device).
__device__ __forceinline__ bool layout_is_fast420(const StepDesc* __restrict__ st, int w) {
  const CompDesc& c0 = st->comp[0];
  return st->ncomp == 3 && st->hmax == 2 && st->vmax == 2 && c0.h == 2 && c0.v == 2 && st->comp[1].h == 1 &&
         st->comp[1].v == 1 && st->comp[2].h == 1 && st->comp[2].v == 1 && w % 4 == 0;
}

}  // namespace rcg
