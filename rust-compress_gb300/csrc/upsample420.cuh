// The search's common decode case, shared by the decoder's upsampling kernel (codec.cu) and the fused
// upsample + pyramid kernel of the scorer (ssim2.cu): 3 components at 4:2:0 with luma at full resolution, linear
// planes only, w % 4 == 0. Integer arithmetic and a table lookup only, so both translation units give the same bits.
#pragma once

#include <stdint.h>

#include "rcg_internal.cuh"

namespace rcg {

// Linear-light values of 4 columns (x0 .. x0+3, x0 % 4 == 0) x 2 rows (2j, 2j+1) of the candidate: the triangle
// filter of jpeg/src/decode.rs:1806-1818 for both chroma components, then the fixed-point YCbCr->RGB of :1438-1441
// and the sRGB table `lut`. Both output rows share the near chroma row j, so three chroma rows per component feed 8
// pixels. Each chroma row's 4 columns (i-1 .. i+2, i = x0/2) come from two aligned 32-bit loads and a funnel shift
// wherever no clamping applies and both words lie inside the row; the edges take the clamped byte path. l[par] is
// left untouched for a row 2j + par >= h.
__device__ __forceinline__ void upsample_420_rows(const StepDesc* __restrict__ st, const uint8_t* __restrict__ planes,
                                                  int w, int h, const float* lut, int x0, int j,
                                                  float (&l)[2][3][4]) {
  const CompDesc c0 = st->comp[0];
  const int cstride = st->comp[1].bw * 8;
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  const int i = x0 / 2;
  // four chroma samples of one row, columns i-1 .. i+2 clamped to [0, cw-1], packed little-endian
  auto row4 = [&](const uint8_t* r) -> uint32_t {
    const int a = (i - 1) & ~3;
    if (i >= 1 && i + 2 <= cw - 1 && a + 8 <= cstride) {
      const uint32_t* q = reinterpret_cast<const uint32_t*>(r + a);  // rows start 8-byte aligned
      return __funnelshift_r(q[0], q[1], 8 * ((i - 1) & 3));
    }
    uint32_t v = 0;
#pragma unroll
    for (int d = 0; d < 4; d++) v |= (uint32_t)r[min(max(i - 1 + d, 0), cw - 1)] << (8 * d);
    return v;
  };
  const int jm = max(j - 1, 0), jp = min(j + 1, ch - 1);
  int up[2][2][4];  // [component][row parity][column]
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const uint8_t* p = planes + st->comp[1 + c].plane_off;
    const uint32_t rn = row4(p + (size_t)j * cstride), rm = row4(p + (size_t)jm * cstride),
                   rp = row4(p + (size_t)jp * cstride);
#pragma unroll
    for (int par = 0; par < 2; par++) {
      const uint32_t rf = par == 0 ? rm : rp;  // far row: j-1 for the even output row, j+1 for the odd one
      int vert[4];
#pragma unroll
      for (int d = 0; d < 4; d++) vert[d] = 3 * (int)((rn >> (8 * d)) & 0xFF) + (int)((rf >> (8 * d)) & 0xFF);
      up[c][par][0] = (3 * vert[1] + vert[0] + 8) >> 4;
      up[c][par][1] = (3 * vert[1] + vert[2] + 7) >> 4;
      up[c][par][2] = (3 * vert[2] + vert[1] + 8) >> 4;
      up[c][par][3] = (3 * vert[2] + vert[3] + 7) >> 4;
    }
  }
#pragma unroll
  for (int par = 0; par < 2; par++) {
    const int y = 2 * j + par;
    if (y >= h) break;
    const uint32_t q = *reinterpret_cast<const uint32_t*>(planes + c0.plane_off + (size_t)y * (c0.bw * 8) + x0);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int yv = (q >> (8 * k)) & 0xFF;
      const int cb = up[0][par][k] - 128, cr = up[1][par][k] - 128;
      l[par][0][k] = lut[min(max(yv + ((91881 * cr + 32768) >> 16), 0), 255)];
      l[par][1][k] = lut[min(max(yv - ((22554 * cb + 46802 * cr + 32768) >> 16), 0), 255)];
      l[par][2][k] = lut[min(max(yv + ((116130 * cb + 32768) >> 16), 0), 255)];
    }
  }
}

// Whether a candidate's layout is that case (the decoder's and the fused kernel's test, evaluated on the device).
__device__ __forceinline__ bool layout_is_fast420(const StepDesc* __restrict__ st, int w) {
  const CompDesc& c0 = st->comp[0];
  return st->ncomp == 3 && st->hmax == 2 && st->vmax == 2 && c0.h == 2 && c0.v == 2 && st->comp[1].h == 1 &&
         st->comp[1].v == 1 && st->comp[2].h == 1 && st->comp[2].v == 1 && w % 4 == 0;
}

}  // namespace rcg
