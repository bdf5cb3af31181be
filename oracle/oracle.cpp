// CPU oracle for the JPEG `--target-ssimulacra2` search path of rust-compress.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: the parity tests, the smoke check and the bench's
// `cpu_baseline` / `--impl reference` legs load it. The product (librcg.so) never links, loads or calls it.
//
// It restates, function by function, the reference's Rust code for the path (the reference cannot be compiled
// here: there is no Rust toolchain). Every function cites the Rust file:line it follows. Arithmetic is kept in
// the reference's order and types: f32 where Rust uses f32, f64 where it uses f64, no FMA contraction (the
// build uses -ffp-contract=off, matching rustc which never contracts), libm's pow/cbrt/exp as Rust's std does.
// Parallel loops follow the reference's rayon shapes (block rows, rows, 96-row scorer stripes) with OpenMP;
// every reduction is summed in the reference's order, so results do not depend on the thread count.
//
// Pinning: the SSIMULACRA2 restatement is checked against the reference's golden vectors
// (fixtures/ssim2/expected.csv, 54 pairs, tolerance 1e-4 as in cli/tests/ssimulacra2.rs:8). The DCT, rounding
// and trellis restatements are checked against the reference's own unit-test known answers
// (jpeg/src/dct.rs:131-211, jpeg/src/rdo.rs:122-162). No reference test pins encoder coefficients, decoder
// pixels or bitstream bytes, so those rest on this line-by-line restatement alone.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <tuple>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ------------------------------------------------------------------------------------------------ tables

// jpeg/src/lib.rs:14-19
static const int ZIGZAG[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                               12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                               35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                               58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// jpeg/src/quality.rs:26-35
static const uint8_t PERCEPTUAL_Q[64] = {16, 16, 16,  18,  25,  37,  56,  85,  16, 17, 20,  27,  34,  40,  53,  75,
                                         16, 20, 24,  31,  43,  62,  91,  135, 18, 27, 31,  40,  53,  74,  106, 156,
                                         25, 34, 43,  53,  69,  94,  131, 189, 37, 40, 62,  74,  94,  124, 169, 238,
                                         56, 53, 91,  106, 131, 169, 226, 255, 85, 75, 135, 156, 189, 238, 255, 255};

// jpeg/src/quality.rs:6-15 (scale_table)
static void scale_table(const uint8_t* base, int quality, uint8_t* out) {
  uint32_t q = (uint32_t)std::min(std::max(quality, 1), 100);
  uint32_t scale = q < 50 ? 5000 / q : 200 - 2 * q;
  for (int i = 0; i < 64; i++) {
    uint32_t v = ((uint32_t)base[i] * scale + 50) / 100;
    out[i] = (uint8_t)std::min<uint32_t>(std::max<uint32_t>(v, 1), 255);
  }
}

// jpeg/src/quality.rs:37-43: luma and chroma both scale PERCEPTUAL_Q.
static void luma_table(int q, uint8_t* out) { scale_table(PERCEPTUAL_Q, q, out); }
static void chroma_table(int q, uint8_t* out) { scale_table(PERCEPTUAL_Q, q, out); }

// jpeg/src/dct.rs:8
static const float AAN[8] = {1.0f, 1.3870398f, 1.306563f, 1.1758756f, 1.0f, 0.78569495f, 0.5411961f, 0.27589938f};

// jpeg/src/encode.rs:45-54 (ZZ_T)
static int ZZ_T[64];
static struct ZztInit {
  ZztInit() {
    for (int k = 0; k < 64; k++) {
      int n = ZIGZAG[k];
      ZZ_T[k] = (n % 8) * 8 + n / 8;
    }
  }
} zzt_init;

// ------------------------------------------------------------------------------------------------ DCT

typedef float Block[8][8];

// jpeg/src/dct.rs:10-18
static void transpose(Block b) {
  for (int i = 0; i < 8; i++)
    for (int j = i + 1; j < 8; j++) {
      float t = b[i][j];
      b[i][j] = b[j][i];
      b[j][i] = t;
    }
}

// jpeg/src/dct.rs:20-57
static void fdct_pass(Block d) {
  for (int j = 0; j < 8; j++) {
    float d0 = d[0][j], d1 = d[1][j], d2 = d[2][j], d3 = d[3][j], d4 = d[4][j], d5 = d[5][j], d6 = d[6][j],
          d7 = d[7][j];
    float tmp0 = d0 + d7, tmp7 = d0 - d7, tmp1 = d1 + d6, tmp6 = d1 - d6;
    float tmp2 = d2 + d5, tmp5 = d2 - d5, tmp3 = d3 + d4, tmp4 = d3 - d4;
    float tmp10 = tmp0 + tmp3, tmp13 = tmp0 - tmp3, tmp11 = tmp1 + tmp2, tmp12 = tmp1 - tmp2;
    d[0][j] = tmp10 + tmp11;
    d[4][j] = tmp10 - tmp11;
    float z1 = (tmp12 + tmp13) * 0.70710677f;
    d[2][j] = tmp13 + z1;
    d[6][j] = tmp13 - z1;
    float t10 = tmp4 + tmp5, t11 = tmp5 + tmp6, t12 = tmp6 + tmp7;
    float z5 = (t10 - t12) * 0.38268343f;
    float z2 = 0.5411961f * t10 + z5;
    float z4 = 1.306563f * t12 + z5;
    float z3 = t11 * 0.70710677f;
    float z11 = tmp7 + z3, z13 = tmp7 - z3;
    d[5][j] = z13 + z2;
    d[3][j] = z13 - z2;
    d[1][j] = z11 + z4;
    d[7][j] = z11 - z4;
  }
}

// jpeg/src/dct.rs:59-65: input b[y][x], output b[u][v] scaled by 8*AAN[u]*AAN[v].
static void fdct(Block b) {
  fdct_pass(b);
  transpose(b);
  fdct_pass(b);
}

// jpeg/src/dct.rs:67-109
static void idct_pass(Block d) {
  const float SQRT_2 = 1.41421356237309504880f;
  for (int j = 0; j < 8; j++) {
    float tmp0 = d[0][j], tmp1 = d[2][j], tmp2 = d[4][j], tmp3 = d[6][j];
    float tmp10 = tmp0 + tmp2, tmp11 = tmp0 - tmp2, tmp13 = tmp1 + tmp3;
    float tmp12 = (tmp1 - tmp3) * SQRT_2 - tmp13;
    float e0 = tmp10 + tmp13, e3 = tmp10 - tmp13, e1 = tmp11 + tmp12, e2 = tmp11 - tmp12;
    float tmp4 = d[1][j], tmp5 = d[3][j], tmp6 = d[5][j], tmp7 = d[7][j];
    float z13 = tmp6 + tmp5, z10 = tmp6 - tmp5, z11 = tmp4 + tmp7, z12 = tmp4 - tmp7;
    float o7 = z11 + z13;
    float o11 = (z11 - z13) * SQRT_2;
    float z5 = (z10 + z12) * 1.8477591f;
    float o10 = 1.0823922f * z12 - z5;
    float o12 = -2.613126f * z10 + z5;
    float o6 = o12 - o7;
    float o5 = o11 - o6;
    float o4 = o10 + o5;
    d[0][j] = e0 + o7;
    d[7][j] = e0 - o7;
    d[1][j] = e1 + o6;
    d[6][j] = e1 - o6;
    d[2][j] = e2 + o5;
    d[5][j] = e2 - o5;
    d[4][j] = e3 + o4;
    d[3][j] = e3 - o4;
  }
}

// jpeg/src/dct.rs:111-123
static void idct(Block b) {
  idct_pass(b);
  transpose(b);
  idct_pass(b);
  transpose(b);
  for (int y = 0; y < 8; y++)
    for (int x = 0; x < 8; x++) b[y][x] *= 0.125f;
}

// jpeg/src/dct.rs:125-129: round half to even for |x| < 2^22 (wrapping integer arithmetic beyond).
static inline int32_t round_f32(float x) {
  float t = x + 12582912.0f;
  uint32_t bits;
  std::memcpy(&bits, &t, 4);
  return (int32_t)(bits - 0x4B400000u);
}

static inline int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ------------------------------------------------------------------------------------------------ Huffman

// core/src/util/huffman.rs:10-86 (build_lengths)
static std::vector<uint8_t> build_lengths(const std::vector<uint32_t>& freqs, int max_len) {
  std::vector<uint8_t> lengths(freqs.size(), 0);
  std::vector<std::pair<uint32_t, size_t>> syms;
  for (size_t i = 0; i < freqs.size(); i++)
    if (freqs[i] > 0) syms.push_back({freqs[i], i});
  if (syms.empty()) return lengths;
  if (syms.size() == 1) {
    lengths[syms[0].second] = 1;
    return lengths;
  }
  // Sort by (freq, Reverse(symbol)): keys are unique.
  std::sort(syms.begin(), syms.end(), [](const std::pair<uint32_t, size_t>& a, const std::pair<uint32_t, size_t>& b) {
    if (a.first != b.first) return a.first < b.first;
    return a.second > b.second;
  });
  size_t n = syms.size();
  std::vector<uint64_t> weight(2 * n - 1, 0);
  for (size_t i = 0; i < n; i++) weight[i] = syms[i].first;
  std::vector<size_t> parent(2 * n - 1, 0);
  size_t leaf = 0, node = n, next = n;
  while (next < 2 * n - 1) {
    size_t ab[2];
    for (int p = 0; p < 2; p++) {
      if (leaf < n && (node >= next || weight[leaf] <= weight[node])) {
        ab[p] = leaf++;
      } else {
        ab[p] = node++;
      }
    }
    weight[next] = weight[ab[0]] + weight[ab[1]];
    parent[ab[0]] = next;
    parent[ab[1]] = next;
    next++;
  }
  std::vector<uint32_t> depth(2 * n - 1, 0);
  for (size_t i = 2 * n - 2; i-- > 0;) depth[i] = depth[parent[i]] + 1;
  size_t max = (size_t)max_len;
  std::vector<uint32_t> count(max + 1, 0);
  for (size_t i = 0; i < n; i++) count[std::min<size_t>(depth[i], max)] += 1;
  uint64_t total = 0;
  for (size_t l = 1; l <= max; l++) total += (uint64_t)count[l] << (max - l);
  while (total > (1ull << max)) {
    count[max] -= 1;
    for (size_t l = max - 1; l >= 1; l--) {
      if (count[l] > 0) {
        count[l] -= 1;
        count[l + 1] += 2;
        break;
      }
    }
    total -= 1;
  }
  size_t idx = 0;
  for (size_t l = max; l >= 1; l--)
    for (uint32_t c = 0; c < count[l]; c++) lengths[syms[idx++].second] = (uint8_t)l;
  return lengths;
}

// jpeg/src/encode.rs:232-238 (HuffTable)
struct HuffTable {
  uint8_t bits[17];
  std::vector<uint8_t> vals;
  uint16_t code[256];
  uint8_t size[256];
};

// jpeg/src/encode.rs:240-263 (optimal_table)
static HuffTable optimal_table(const uint32_t* freq) {
  std::vector<uint32_t> f(freq, freq + 256);
  f.push_back(1);
  std::vector<uint8_t> lens = build_lengths(f, 16);
  std::vector<std::pair<uint8_t, uint8_t>> syms;
  for (int s = 0; s < 256; s++)
    if (lens[s] > 0) syms.push_back({lens[s], (uint8_t)s});
  if (syms.empty()) syms.push_back({1, 0});
  std::sort(syms.begin(), syms.end());
  HuffTable t;
  std::memset(t.bits, 0, sizeof t.bits);
  std::memset(t.code, 0, sizeof t.code);
  std::memset(t.size, 0, sizeof t.size);
  uint32_t code = 0;
  uint8_t prev_len = syms[0].first;
  for (auto& ls : syms) {
    code <<= (ls.first - prev_len);
    prev_len = ls.first;
    t.bits[ls.first] += 1;
    t.vals.push_back(ls.second);
    t.code[ls.second] = (uint16_t)code;
    t.size[ls.second] = ls.first;
    code += 1;
  }
  return t;
}

// ------------------------------------------------------------------------------------------------ trellis

// jpeg/src/rdo.rs:12
static const float FREQ_WEIGHT_GAMMA = 1.0f;
// jpeg/src/encode.rs:42
static const float TRELLIS_KAPPA = 0.02f;

// jpeg/src/rdo.rs:14-45 (Rdo, Rdo::new)
struct Rdo {
  float q[64];
  float lambda;
  float w[64];
  float len[256];
  Rdo(const uint8_t* table, float kappa, const uint8_t* sizes) {
    for (int k = 0; k < 64; k++) q[k] = (float)table[ZIGZAG[k]];
    std::vector<float> sorted(q + 1, q + 64);
    std::sort(sorted.begin(), sorted.end());
    float median = sorted[sorted.size() / 2];
    for (int s = 0; s < 256; s++) len[s] = sizes[s] == 0 ? 18.0f : (float)sizes[s];
    for (int k = 0; k < 64; k++) w[k] = 1.0f;
    for (int k = 1; k < 64; k++) w[k] = std::pow(median / q[k], FREQ_WEIGHT_GAMMA);
    lambda = kappa * median * median;
  }

  // jpeg/src/rdo.rs:47-52
  float rate(uint32_t run, uint32_t v) const {
    uint32_t size = 32 - (uint32_t)__builtin_clz(v);
    uint32_t zrl = run / 16;
    return (float)zrl * len[0xF0] + len[((run % 16) << 4) | size] + (float)size;
  }

  // jpeg/src/rdo.rs:54-119 (quantize_ac). `pw` (nullable, 64 entries in zigzag order) is the perceptual mode's
  // per-coefficient weight: the distortion weight of position k becomes w[k] * pw[k] (rounded to f32 first). With
  // pw == nullptr this is the reference's plain MSE trellis.
  void quantize_ac(const float* a, int16_t* out, const float* pw = nullptr) const {
    float wk[64];
    for (int k = 0; k < 64; k++) wk[k] = pw ? w[k] * pw[k] : w[k];
    struct Node {
      int pos;
      uint32_t v;
      float cost;
      int prev;
    };
    const int START = -1;
    float zd[64];
    zd[0] = 0.0f;
    for (int k = 1; k < 64; k++) {
      float e = a[k] * q[k];
      zd[k] = zd[k - 1] + e * e * wk[k];
    }
    Node nodes[128];
    int nn = 0;
    for (int i = 1; i < 64; i++) {
      float m = std::fabs(a[i]);
      uint32_t v0 = (uint32_t)(m + 0.5f);
      if (v0 == 0) continue;
      uint32_t lo = v0 > 1 ? v0 - 1 : v0;
      for (uint32_t v = lo; v <= v0; v++) {
        float e = (m - (float)v) * q[i];
        float dnz = e * e * wk[i];
        float best = zd[i - 1] + lambda * rate((uint32_t)(i - 1), v) + dnz;
        int prev = START;
        for (int ni = 0; ni < nn; ni++) {
          const Node& n = nodes[ni];
          if (n.pos >= i) continue;
          float c = n.cost + (zd[i - 1] - zd[n.pos]) + lambda * rate((uint32_t)(i - n.pos - 1), v) + dnz;
          if (c < best) {
            best = c;
            prev = ni;
          }
        }
        nodes[nn++] = Node{i, v, best, prev};
      }
    }
    float eob = lambda * len[0];
    float best_cost = zd[63] + eob;
    int best_end = START;
    for (int ni = 0; ni < nn; ni++) {
      const Node& n = nodes[ni];
      float c = n.cost + (zd[63] - zd[n.pos]) + (n.pos < 63 ? eob : 0.0f);
      if (c < best_cost) {
        best_cost = c;
        best_end = ni;
      }
    }
    for (int k = 1; k < 64; k++) out[k] = 0;
    int cur = best_end;
    while (cur != START) {
      const Node& n = nodes[cur];
      int16_t v = (int16_t)n.v;
      out[n.pos] = a[n.pos] < 0.0f ? (int16_t)-v : v;
      cur = n.prev;
    }
  }
};

// ------------------------------------------------------------------------------------------------ encoder

// jpeg/src/encode.rs:56-83 (CoefComponent, CoefImage), restricted to what the pixel path builds.
struct CoefComponent {
  uint8_t id;
  int h, v, tq;
  int blocks_w, blocks_h;
  std::vector<int16_t> coefs;
};

struct CoefImage {
  int width, height;
  std::vector<CoefComponent> comps;
  uint8_t qtables[4][64];
  bool has_q[4];
  int hv_max_h() const {
    int m = 1;
    for (auto& c : comps) m = std::max(m, c.h);
    return m;
  }
  int hv_max_v() const {
    int m = 1;
    for (auto& c : comps) m = std::max(m, c.v);
    return m;
  }
  // jpeg/src/encode.rs:90-93
  void mcus(int& mx, int& my) const {
    int hm = hv_max_h(), vm = hv_max_v();
    mx = (width + 8 * hm - 1) / (8 * hm);
    my = (height + 8 * vm - 1) / (8 * vm);
  }
};

// jpeg/src/encode.rs:174-183 (fdct_divisors)
static void fdct_divisors(const uint8_t* q, float* d) {
  for (int v = 0; v < 8; v++)
    for (int u = 0; u < 8; u++) d[u * 8 + v] = 1.0f / ((float)q[v * 8 + u] * AAN[u] * AAN[v] * 8.0f);
}

// jpeg/src/encode.rs:185-219 (quantize_plane)
static std::vector<int16_t> quantize_plane(const uint8_t* plane, int stride, int bw, int bh, const float* div,
                                           const Rdo* rdo, const float* weights = nullptr) {
  std::vector<int16_t> out((size_t)bw * bh * 64, 0);
#pragma omp parallel for schedule(dynamic)
  for (int by = 0; by < bh; by++) {
    for (int bx = 0; bx < bw; bx++) {
      Block blk;
      for (int y = 0; y < 8; y++) {
        const uint8_t* src = plane + (size_t)(by * 8 + y) * stride + bx * 8;
        for (int x = 0; x < 8; x++) blk[y][x] = (float)src[x] - 128.0f;
      }
      fdct(blk);
      const float* flat = &blk[0][0];
      int16_t* dst = out.data() + ((size_t)by * bw + bx) * 64;
      if (!rdo) {
        for (int k = 0; k < 64; k++) {
          int f = ZZ_T[k];
          dst[k] = (int16_t)clampi(round_f32(flat[f] * div[f]), -2047, 2047);
        }
      } else {
        float a[64];
        for (int k = 0; k < 64; k++) {
          int f = ZZ_T[k];
          a[k] = flat[f] * div[f];
        }
        dst[0] = (int16_t)clampi(round_f32(a[0]), -2047, 2047);
        rdo->quantize_ac(a, dst, weights ? weights + ((size_t)by * bw + bx) * 64 : nullptr);
      }
    }
  }
  return out;
}

// jpeg/src/encode.rs:265-288 (Sink, Stats)
struct Stats {
  uint32_t dc[2][256];
  uint32_t ac[2][256];
  uint64_t raw_bits;
  Stats() { std::memset(this, 0, sizeof *this); }
  void on_dc(int tbl, uint32_t cat, uint32_t) {
    dc[tbl][cat] += 1;
    raw_bits += cat;
  }
  void on_ac(int tbl, uint8_t sym, uint32_t, uint32_t nbits) {
    ac[tbl][sym] += 1;
    raw_bits += nbits;
  }
};

// jpeg/src/encode.rs:290-320 (MsbWriter)
struct MsbWriter {
  std::vector<uint8_t> out;
  uint64_t acc = 0;
  uint32_t n = 0;
  void put(uint32_t v, uint32_t len) {
    if (len == 0) return;
    acc = (acc << len) | ((uint64_t)v & ((1ull << len) - 1));
    n += len;
    while (n >= 8) {
      uint8_t byte = (uint8_t)(acc >> (n - 8));
      out.push_back(byte);
      if (byte == 0xFF) out.push_back(0);
      n -= 8;
    }
  }
  void finish() {
    if (n > 0) {
      uint32_t pad = 8 - n;
      put((1u << pad) - 1, pad);
    }
  }
};

// jpeg/src/encode.rs:322-341 (Writer)
struct Writer {
  MsbWriter w;
  const HuffTable* dct;  // [2]
  const HuffTable* act;  // [2]
  void on_dc(int tbl, uint32_t cat, uint32_t extra) {
    w.put(dct[tbl].code[cat], dct[tbl].size[cat]);
    w.put(extra, cat);
  }
  void on_ac(int tbl, uint8_t sym, uint32_t extra, uint32_t nbits) {
    w.put(act[tbl].code[sym], act[tbl].size[sym]);
    w.put(extra, nbits);
  }
};

// jpeg/src/encode.rs:343-349 (category)
static inline void category(int32_t v, uint32_t& cat, uint32_t& extra) {
  uint32_t a = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
  cat = a == 0 ? 0 : 32 - (uint32_t)__builtin_clz(a);
  uint32_t e = v < 0 ? (uint32_t)(v - 1) : (uint32_t)v;
  extra = e & (uint32_t)((1ull << cat) - 1);
}

// jpeg/src/encode.rs:351-374 (code_block)
template <class S>
static void code_block(S& s, const int16_t* blk, int16_t* pred, int tbl) {
  int32_t diff = (int32_t)blk[0] - (int32_t)*pred;
  *pred = blk[0];
  uint32_t cat, extra;
  category(diff, cat, extra);
  s.on_dc(tbl, cat, extra);
  uint32_t run = 0;
  for (int k = 1; k < 64; k++) {
    int16_t c = blk[k];
    if (c == 0) {
      run++;
      continue;
    }
    while (run >= 16) {
      s.on_ac(tbl, 0xF0, 0, 0);
      run -= 16;
    }
    category(c, cat, extra);
    s.on_ac(tbl, (uint8_t)((run << 4) | cat), extra, cat);
    run = 0;
  }
  if (run > 0) s.on_ac(tbl, 0x00, 0, 0);
}

// jpeg/src/encode.rs:376-398 (scan, scan_with; non-differential)
template <class S>
static void scan(const std::vector<CoefComponent>& comps, int mcus_x, int mcus_y, S& sink) {
  int16_t pred[4] = {0, 0, 0, 0};
  for (int my = 0; my < mcus_y; my++)
    for (int mx = 0; mx < mcus_x; mx++)
      for (size_t ci = 0; ci < comps.size(); ci++) {
        const CoefComponent& c = comps[ci];
        for (int by = 0; by < c.v; by++)
          for (int bx = 0; bx < c.h; bx++) {
            size_t b = (size_t)(my * c.v + by) * c.blocks_w + mx * c.h + bx;
            code_block(sink, &c.coefs[b * 64], &pred[ci], (int)std::min<size_t>(ci, 1));
          }
      }
}

// jpeg/src/encode.rs:221-228 (ac_code_lengths)
static void ac_code_lengths(const CoefImage& ci, uint8_t out[2][256]) {
  int mx, my;
  ci.mcus(mx, my);
  Stats st;
  scan(ci.comps, mx, my, st);
  for (int t = 0; t < 2; t++) {
    HuffTable h = optimal_table(st.ac[t]);
    std::memcpy(out[t], h.size, 256);
  }
}

enum Subsampling { SUB_AUTO = 0, SUB_444 = 1, SUB_422 = 2, SUB_420 = 3 };

// jpeg/src/encode.rs:426-539 (build_coefs). `channels` is 1 (Gray) or 3 (Rgb), 8-bit.
// `weights` (nullable): the perceptual trellis's per-coefficient weights in the coefficient layout (components in
// order, blocks row-major, 64 zigzag entries each); only the trellis pass reads them.
static CoefImage build_coefs(const uint8_t* data, int w, int h, int channels, int quality, int subsampling,
                             bool trellis, const float* weights = nullptr) {
  bool gray = channels == 1;
  int hmax, vmax;
  if (gray) {
    hmax = vmax = 1;
  } else {
    switch (subsampling) {
      case SUB_420: hmax = 2; vmax = 2; break;
      case SUB_422: hmax = 2; vmax = 1; break;
      case SUB_444: hmax = 1; vmax = 1; break;
      default:
        if (quality < 90) { hmax = 2; vmax = 2; } else { hmax = 1; vmax = 1; }
    }
  }
  int mcu_w = 8 * hmax, mcu_h = 8 * vmax;
  int mcus_x = (w + mcu_w - 1) / mcu_w, mcus_y = (h + mcu_h - 1) / mcu_h;
  int pw = mcus_x * mcu_w, ph = mcus_y * mcu_h;
  uint8_t qy[64], qc[64];
  luma_table(quality, qy);
  chroma_table(quality, qc);

  CoefImage ci;
  ci.width = w;
  ci.height = h;
  std::memset(ci.has_q, 0, sizeof ci.has_q);
  std::memcpy(ci.qtables[0], qy, 64);
  ci.has_q[0] = true;
  if (!gray) {
    std::memcpy(ci.qtables[1], qc, 64);
    ci.has_q[1] = true;
  }
  struct PlaneRef {
    std::vector<uint8_t> p;
    int stride, bw, bh, cls;
  };
  std::vector<PlaneRef> planes;
  if (gray) {
    std::vector<uint8_t> y((size_t)pw * ph);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < ph; r++) {
      int sr = std::min(r, h - 1);
      for (int x = 0; x < pw; x++) y[(size_t)r * pw + x] = data[(size_t)sr * w + std::min(x, w - 1)];
    }
    float dy[64];
    fdct_divisors(qy, dy);
    CoefComponent c{1, 1, 1, 0, pw / 8, ph / 8, quantize_plane(y.data(), pw, pw / 8, ph / 8, dy, nullptr)};
    ci.comps.push_back(std::move(c));
    planes.push_back({std::move(y), pw, pw / 8, ph / 8, 0});
  } else {
    std::vector<uint8_t> yp((size_t)pw * ph), cbp((size_t)pw * ph), crp((size_t)pw * ph);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < ph; r++) {
      int sr = std::min(r, h - 1);
      for (int x = 0; x < pw; x++) {
        size_t i = ((size_t)sr * w + std::min(x, w - 1)) * 3;
        int32_t rr = data[i], gg = data[i + 1], bb = data[i + 2];
        size_t o = (size_t)r * pw + x;
        yp[o] = (uint8_t)((19595 * rr + 38470 * gg + 7471 * bb + 32768) >> 16);
        cbp[o] = (uint8_t)((-11059 * rr - 21709 * gg + 32768 * bb + (128 << 16) + 32767) >> 16);
        crp[o] = (uint8_t)((32768 * rr - 27439 * gg - 5329 * bb + (128 << 16) + 32767) >> 16);
      }
    }
    std::vector<uint8_t> cb, cr;
    int cw, chh;
    if (hmax * vmax > 1) {
      cw = pw / hmax;
      chh = ph / vmax;
      auto down = [&](const std::vector<uint8_t>& p) {
        std::vector<uint8_t> o((size_t)cw * chh);
#pragma omp parallel for schedule(static)
        for (int r = 0; r < chh; r++)
          for (int x = 0; x < cw; x++) {
            uint32_t s = 0;
            for (int dy = 0; dy < vmax; dy++)
              for (int dx = 0; dx < hmax; dx++) s += p[(size_t)(vmax * r + dy) * pw + hmax * x + dx];
            uint32_t n = (uint32_t)(hmax * vmax);
            o[(size_t)r * cw + x] = (uint8_t)((s + n / 2) / n);
          }
        return o;
      };
      cb = down(cbp);
      cr = down(crp);
    } else {
      cb = std::move(cbp);
      cr = std::move(crp);
      cw = pw;
      chh = ph;
    }
    float dy[64], dc[64];
    fdct_divisors(qy, dy);
    fdct_divisors(qc, dc);
    CoefComponent cy{1, hmax, vmax, 0, pw / 8, ph / 8, quantize_plane(yp.data(), pw, pw / 8, ph / 8, dy, nullptr)};
    CoefComponent ccb{2, 1, 1, 1, cw / 8, chh / 8, quantize_plane(cb.data(), cw, cw / 8, chh / 8, dc, nullptr)};
    CoefComponent ccr{3, 1, 1, 1, cw / 8, chh / 8, quantize_plane(cr.data(), cw, cw / 8, chh / 8, dc, nullptr)};
    ci.comps.push_back(std::move(cy));
    ci.comps.push_back(std::move(ccb));
    ci.comps.push_back(std::move(ccr));
    planes.push_back({std::move(yp), pw, pw / 8, ph / 8, 0});
    planes.push_back({std::move(cb), cw, cw / 8, chh / 8, 1});
    planes.push_back({std::move(cr), cw, cw / 8, chh / 8, 1});
  }
  if (trellis && quality < 100) {
    uint8_t lens[2][256];
    ac_code_lengths(ci, lens);
    const uint8_t* tables[2] = {qy, qc};
    Rdo r0(tables[0], TRELLIS_KAPPA, lens[0]);
    Rdo r1(tables[1], TRELLIS_KAPPA, lens[1]);
    const Rdo* rdos[2] = {&r0, &r1};
    float divs[2][64];
    fdct_divisors(tables[0], divs[0]);
    fdct_divisors(tables[1], divs[1]);
    size_t blk0 = 0;
    for (size_t i = 0; i < ci.comps.size(); i++) {
      PlaneRef& p = planes[i];
      const float* pw = weights ? weights + blk0 * 64 : nullptr;
      ci.comps[i].coefs = quantize_plane(p.p.data(), p.stride, p.bw, p.bh, divs[p.cls], rdos[p.cls], pw);
      blk0 += (size_t)p.bw * p.bh;
    }
  }
  return ci;
}

// ------------------------------------------------------------------------------------------------ decoder

// jpeg/src/decode.rs:1310-1343 (idct_planes, 8-bit case: center 128, clamp 0..255)
static std::vector<uint8_t> idct_plane(const CoefComponent& c, const uint8_t* q) {
  float mult[8][8];
  for (int v = 0; v < 8; v++)
    for (int u = 0; u < 8; u++) mult[v][u] = (float)q[v * 8 + u] * AAN[u] * AAN[v];
  int stride = c.blocks_w * 8;
  std::vector<uint8_t> plane((size_t)stride * c.blocks_h * 8);
#pragma omp parallel for schedule(dynamic)
  for (int by = 0; by < c.blocks_h; by++) {
    for (int bx = 0; bx < c.blocks_w; bx++) {
      const int16_t* src = &c.coefs[((size_t)by * c.blocks_w + bx) * 64];
      Block blk;
      for (int k = 0; k < 64; k++) {
        int n = ZIGZAG[k];
        blk[n / 8][n % 8] = (float)src[k] * mult[n / 8][n % 8];
      }
      idct(blk);
      for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++)
          plane[(size_t)(by * 8 + y) * stride + bx * 8 + x] = (uint8_t)clampi(round_f32(blk[y][x]) + 128, 0, 255);
    }
  }
  return plane;
}

// jpeg/src/decode.rs:1768-1828 (upsample)
static std::vector<uint8_t> upsample(const std::vector<uint8_t>& p, int stride, int cw, int ch, int fx, int fy, int w,
                                     int h) {
  std::vector<uint8_t> out((size_t)w * h);
  auto px = [&](int x, int y) -> int32_t { return p[(size_t)y * stride + x]; };
  if (fx == 1 && fy == 1) {
    for (int y = 0; y < h; y++) std::memcpy(&out[(size_t)y * w], &p[(size_t)y * stride], w);
  } else if (fx == 2 && fy == 1) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++)
      for (int x = 0; x < w; x++) {
        int i = x / 2;
        int32_t near_ = px(i, y);
        int32_t far_ = x % 2 == 0 ? px(i > 0 ? i - 1 : 0, y) : px(std::min(i + 1, cw - 1), y);
        out[(size_t)y * w + x] = (uint8_t)((3 * near_ + far_ + (x % 2 == 0 ? 1 : 2)) >> 2);
      }
  } else if (fx == 1 && fy == 2) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
      int j = y / 2;
      int far_y = y % 2 == 0 ? (j > 0 ? j - 1 : 0) : std::min(j + 1, ch - 1);
      for (int x = 0; x < w; x++)
        out[(size_t)y * w + x] = (uint8_t)((3 * px(x, j) + px(x, far_y) + (y % 2 == 0 ? 1 : 2)) >> 2);
    }
  } else if (fx == 2 && fy == 2) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
      int j = y / 2;
      int far_y = y % 2 == 0 ? (j > 0 ? j - 1 : 0) : std::min(j + 1, ch - 1);
      auto vert = [&](int x) { return 3 * px(x, j) + px(x, far_y); };
      for (int x = 0; x < w; x++) {
        int i = x / 2;
        int32_t near_ = vert(i);
        int32_t far_ = x % 2 == 0 ? vert(i > 0 ? i - 1 : 0) : vert(std::min(i + 1, cw - 1));
        out[(size_t)y * w + x] = (uint8_t)((3 * near_ + far_ + (x % 2 == 0 ? 8 : 7)) >> 4);
      }
    }
  } else {
    for (int y = 0; y < h; y++)
      for (int x = 0; x < w; x++) out[(size_t)y * w + x] = p[(size_t)(y / fy) * stride + x / fx];
  }
  return out;
}

// jpeg/src/decode.rs:334-389 -> Decoder::finish (:1390-1448) for an 8-bit CoefImage built by the encoder (component
// ids 1,2,3, no Adobe marker: the YCbCr -> RGB branch). Output: Gray (1 channel) or RGB (3 channels) interleaved.
static std::vector<uint8_t> reconstruct(const CoefImage& ci, int* out_channels) {
  int hmax = ci.hv_max_h(), vmax = ci.hv_max_v();
  int w = ci.width, h = ci.height;
  std::vector<std::vector<uint8_t>> full;
  for (auto& c : ci.comps) {
    std::vector<uint8_t> plane = idct_plane(c, ci.qtables[c.tq]);
    int cw = (w * c.h + hmax - 1) / hmax;
    int chh = (h * c.v + vmax - 1) / vmax;
    full.push_back(upsample(plane, c.blocks_w * 8, cw, chh, hmax / c.h, vmax / c.v, w, h));
  }
  if (full.size() == 1) {
    *out_channels = 1;
    return full[0];
  }
  *out_channels = 3;
  std::vector<uint8_t> data((size_t)w * h * 3);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      size_t i = (size_t)y * w + x;
      int32_t a = full[0][i], b = full[1][i], c = full[2][i];
      int32_t cb = b - 128, cr = c - 128;
      data[i * 3 + 0] = (uint8_t)clampi(a + ((91881 * cr + 32768) >> 16), 0, 255);
      data[i * 3 + 1] = (uint8_t)clampi(a - ((22554 * cb + 46802 * cr + 32768) >> 16), 0, 255);
      data[i * 3 + 2] = (uint8_t)clampi(a + ((116130 * cb + 32768) >> 16), 0, 255);
    }
  return data;
}

// ------------------------------------------------------------------------------------------------ SSIMULACRA2

// core/src/ssimulacra2.rs:25-52
static const int NUM_SCALES = 6;
static const double C2 = 0.0009;
static const double SIGMA = 1.5;
static const int RADIUS = 5;
static const int STRIPE = 96;
static const double M02 = 0.078, M00 = 0.30, M01 = 1.0 - M02 - M00;
static const double M12 = 0.078, M10 = 0.23, M11 = 1.0 - M12 - M10;
static const double M20 = 0.2434226892454782, M21 = 0.2047674442449682, M22 = 1.0 - M20 - M21;
static const double BIAS = 0.0037930732552754493;

// core/src/ssimulacra2.rs:54-163
static const double WEIGHTS[108] = {
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
    0.0, 0.0, 0.0, 0.0005130064588990679, 0.0, 0.00010854057858411537
};

// core/src/ssimulacra2.rs:165-170. `P` is f32 in the reference; the FP64 oracle instantiates it with double.
template <class P>
struct Planes {
  int w, h;
  std::vector<P> ch[3];
};

// core/src/ssimulacra2.rs:172-175
static double srgb_to_linear(double v) { return v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4); }

// core/src/image.rs:186-190 (blend)
static inline uint8_t blend(uint8_t c, uint8_t a, uint8_t bg) {
  uint32_t aa = a;
  return (uint8_t)(((uint32_t)c * aa + (uint32_t)bg * (255 - aa) + 127) / 255);
}

// core/src/ssimulacra2.rs:177-221 (linear_planes) together with core/src/image.rs:143-178 (to_depth8, flatten) for
// images with alpha. `channels`: 1 Gray, 2 GrayAlpha, 3 Rgb, 4 Rgba; `depth` 8 or 16 (16-bit samples big-endian).
template <class P>
static Planes<P> linear_planes(const uint8_t* data, int w, int h, int channels, int depth) {
  Planes<P> out;
  out.w = w;
  out.h = h;
  size_t n = (size_t)w * h;
  for (int c = 0; c < 3; c++) out.ch[c].assign(n, (P)0);
  std::vector<uint8_t> flat;
  bool has_alpha = channels == 2 || channels == 4;
  if (has_alpha) {
    // flatten([128,128,128]) goes through to_depth8 first (core/src/image.rs:160-178)
    int oc = channels == 2 ? 1 : 3;
    flat.resize(n * oc);
    for (size_t i = 0; i < n; i++) {
      uint8_t s[4];
      for (int k = 0; k < channels; k++) {
        if (depth == 8) {
          s[k] = data[i * channels + k];
        } else {
          uint32_t v = ((uint32_t)data[(i * channels + k) * 2] << 8) | data[(i * channels + k) * 2 + 1];
          s[k] = (uint8_t)((v * 255 + 32767) / 65535);
        }
      }
      if (channels == 2) {
        flat[i] = blend(s[0], s[1], 128);
      } else {
        for (int k = 0; k < 3; k++) flat[i * 3 + k] = blend(s[k], s[3], 128);
      }
    }
    data = flat.data();
    channels = oc;
    depth = 8;
  }
  if (depth == 8) {
    P lut[256];
    for (int v = 0; v < 256; v++) lut[v] = (P)srgb_to_linear((double)v / 255.0);
    for (size_t i = 0; i < n; i++) {
      if (channels == 1) {
        P l = lut[data[i]];
        out.ch[0][i] = l;
        out.ch[1][i] = l;
        out.ch[2][i] = l;
      } else {
        out.ch[0][i] = lut[data[i * 3]];
        out.ch[1][i] = lut[data[i * 3 + 1]];
        out.ch[2][i] = lut[data[i * 3 + 2]];
      }
    }
  } else {
    auto s = [&](size_t i, int k) -> P {
      const uint8_t* px = data + (i * channels + k) * 2;
      uint32_t v = ((uint32_t)px[0] << 8) | px[1];
      return (P)srgb_to_linear((double)v / 65535.0);
    };
    for (size_t i = 0; i < n; i++) {
      if (channels == 1) {
        P l = s(i, 0);
        out.ch[0][i] = l;
        out.ch[1][i] = l;
        out.ch[2][i] = l;
      } else {
        out.ch[0][i] = s(i, 0);
        out.ch[1][i] = s(i, 1);
        out.ch[2][i] = s(i, 2);
      }
    }
  }
  return out;
}

// core/src/ssimulacra2.rs:223-247 (downsample)
template <class P>
static Planes<P> downsample(const Planes<P>& p) {
  int w = p.w, h = p.h;
  int ow = (w + 1) / 2, oh = (h + 1) / 2;
  Planes<P> out;
  out.w = ow;
  out.h = oh;
  for (int c = 0; c < 3; c++) {
    const std::vector<P>& src = p.ch[c];
    std::vector<P>& o = out.ch[c];
    o.assign((size_t)ow * oh, (P)0);
#pragma omp parallel for schedule(static)
    for (int oy = 0; oy < oh; oy++) {
      int y0 = oy * 2, y1 = std::min(oy * 2 + 2, h);
      for (int ox = 0; ox < ow; ox++) {
        int x0 = ox * 2, x1 = std::min(ox * 2 + 2, w);
        double sum = 0.0;
        for (int y = y0; y < y1; y++)
          for (int x = x0; x < x1; x++) sum += (double)src[(size_t)y * w + x];
        o[(size_t)oy * ow + ox] = (P)(sum / (double)((y1 - y0) * (x1 - x0)));
      }
    }
  }
  return out;
}

// core/src/ssimulacra2.rs:249-258 (xyb)
static inline void xyb(double r, double g, double b, double out[3]) {
  double cb = std::cbrt(BIAS);
  double m0 = std::cbrt(std::max(M00 * r + M01 * g + M02 * b + BIAS, 0.0)) - cb;
  double m1 = std::cbrt(std::max(M10 * r + M11 * g + M12 * b + BIAS, 0.0)) - cb;
  double m2 = std::cbrt(std::max(M20 * r + M21 * g + M22 * b + BIAS, 0.0)) - cb;
  double x = 0.5 * (m0 - m1);
  double y = 0.5 * (m0 + m1);
  out[0] = x * 14.0 + 0.42;
  out[1] = y + 0.01;
  out[2] = (m2 - y) + 0.55;
}

// core/src/ssimulacra2.rs:260-271 (kernel)
static void gauss_kernel(double k[2 * RADIUS + 1]) {
  double sum = 0.0;
  for (int i = 0; i < 2 * RADIUS + 1; i++) {
    double x = (double)i - (double)RADIUS;
    k[i] = std::exp(-0.5 / (SIGMA * SIGMA) * x * x);
    sum += k[i];
  }
  for (int i = 0; i < 2 * RADIUS + 1; i++) k[i] /= sum;
}

// core/src/ssimulacra2.rs:273-319 (blur_row), ZERO_LEFT_RIGHT = true.
static void blur_row(const double* src, double* dst, int w, const double* k) {
  auto at = [&](long i) -> double { return (i < 0 || i > (long)w - 1) ? 0.0 : src[i]; };
  auto edge = [&](int x) -> double {
    double s = 0.0;
    for (int t = 0; t < 2 * RADIUS + 1; t++) s += k[t] * at((long)x + t - RADIUS);
    return s;
  };
  if (w > 2 * RADIUS) {
    int lo = RADIUS, hi = w - RADIUS;
    double centre = k[RADIUS];
    for (int x = lo; x < hi; x++) dst[x] = centre * src[x];
    for (int t = 1; t <= RADIUS; t++) {
      double kt = k[RADIUS + t];
      for (int x = lo; x < hi; x++) dst[x] += kt * (src[x - t] + src[x + t]);
    }
    for (int x = 0; x < lo; x++) dst[x] = edge(x);
    for (int x = hi; x < w; x++) dst[x] = edge(x);
  } else {
    for (int x = 0; x < w; x++) dst[x] = edge(x);
  }
}

struct Sums {
  double v[3][6];
};

// core/src/ssimulacra2.rs:338-444 (stripe_sums)
template <class P>
static Sums stripe_sums(const Planes<P>& a, const Planes<P>& b, int y0, int y1, const double* k) {
  int w = a.w, h = a.h;
  int lo = std::max(y0 - RADIUS, 0);
  int hi = std::min(y1 + RADIUS, h);
  int rows = hi - lo;
  std::vector<double> xa[3], xb[3];
  for (int c = 0; c < 3; c++) {
    xa[c].assign((size_t)rows * w, 0.0);
    xb[c].assign((size_t)rows * w, 0.0);
  }
  for (int r = 0; r < rows; r++) {
    size_t base = (size_t)(lo + r) * w;
    for (int x = 0; x < w; x++) {
      size_t i = base + x;
      double pa[3], pb[3];
      xyb((double)a.ch[0][i], (double)a.ch[1][i], (double)a.ch[2][i], pa);
      xyb((double)b.ch[0][i], (double)b.ch[1][i], (double)b.ch[2][i], pb);
      for (int c = 0; c < 3; c++) {
        xa[c][(size_t)r * w + x] = pa[c];
        xb[c][(size_t)r * w + x] = pb[c];
      }
    }
  }
  Sums sums;
  std::memset(&sums, 0, sizeof sums);
  std::vector<double> h5[5];
  for (int q = 0; q < 5; q++) h5[q].assign((size_t)rows * w, 0.0);
  std::vector<double> tmp(w), acc[5];
  for (int q = 0; q < 5; q++) acc[q].assign(w, 0.0);
  for (int c = 0; c < 3; c++) {
    for (int r = 0; r < rows; r++) {
      const double* ra = &xa[c][(size_t)r * w];
      const double* rb = &xb[c][(size_t)r * w];
      blur_row(ra, &h5[0][(size_t)r * w], w, k);
      blur_row(rb, &h5[1][(size_t)r * w], w, k);
      for (int x = 0; x < w; x++) tmp[x] = ra[x] * ra[x];
      blur_row(tmp.data(), &h5[2][(size_t)r * w], w, k);
      for (int x = 0; x < w; x++) tmp[x] = rb[x] * rb[x];
      blur_row(tmp.data(), &h5[3][(size_t)r * w], w, k);
      for (int x = 0; x < w; x++) tmp[x] = ra[x] * rb[x];
      blur_row(tmp.data(), &h5[4][(size_t)r * w], w, k);
    }
    double* s = sums.v[c];
    auto row_of = [&](int q, long yy) -> const double* {
      long hh = h;
      if (yy < 0 || yy >= hh) yy = yy < 0 ? -yy - 1 : 2 * hh - 1 - yy;
      size_t r = (size_t)(yy - lo);
      return &h5[q][r * w];
    };
    for (int y = y0; y < y1; y++) {
      for (int q = 0; q < 5; q++) {
        const double* centre = row_of(q, y);
        for (int x = 0; x < w; x++) acc[q][x] = k[RADIUS] * centre[x];
        for (int t = 1; t <= RADIUS; t++) {
          double kt = k[RADIUS + t];
          const double* up = row_of(q, (long)y - t);
          const double* down = row_of(q, (long)y + t);
          for (int x = 0; x < w; x++) acc[q][x] += kt * (up[x] + down[x]);
        }
      }
      const double* ra = &xa[c][(size_t)(y - lo) * w];
      const double* rb = &xb[c][(size_t)(y - lo) * w];
      for (int x = 0; x < w; x++) {
        double m1 = acc[0][x], m2 = acc[1][x];
        double s11 = acc[2][x], s22 = acc[3][x], s12 = acc[4][x];
        double num_m = 1.0 - (m1 - m2) * (m1 - m2);
        double num_s = 2.0 * (s12 - m1 * m2) + C2;
        double denom_s = (s11 - m1 * m1) + (s22 - m2 * m2) + C2;
        double d = std::max(1.0 - num_m * num_s / denom_s, 0.0);
        double d1 = (1.0 + std::fabs(rb[x] - m2)) / (1.0 + std::fabs(ra[x] - m1)) - 1.0;
        double art = std::max(d1, 0.0);
        double det = std::max(-d1, 0.0);
        s[0] += d;
        s[1] += (d * d) * (d * d);
        s[2] += art;
        s[3] += (art * art) * (art * art);
        s[4] += det;
        s[5] += (det * det) * (det * det);
      }
    }
  }
  return sums;
}

// core/src/ssimulacra2.rs:446-466 (scale_stats)
template <class P>
static void scale_stats(const Planes<P>& a, const Planes<P>& b, double out[3][6]) {
  double k[2 * RADIUS + 1];
  gauss_kernel(k);
  int n = (a.h + STRIPE - 1) / STRIPE;
  std::vector<Sums> parts(n);
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < n; i++) parts[i] = stripe_sums(a, b, i * STRIPE, std::min((i + 1) * STRIPE, a.h), k);
  Sums total;
  std::memset(&total, 0, sizeof total);
  for (int i = 0; i < n; i++)
    for (int c = 0; c < 3; c++)
      for (int j = 0; j < 6; j++) total.v[c][j] += parts[i].v[c][j];
  double count = (double)a.w * (double)a.h;
  for (int c = 0; c < 3; c++)
    for (int m = 0; m < 3; m++) {
      out[c][2 * m] = total.v[c][2 * m] / count;
      out[c][2 * m + 1] = std::pow(total.v[c][2 * m + 1] / count, 0.25);
    }
}

// core/src/ssimulacra2.rs:491-511: 108-term weighted sum and final mapping from per-scale stats.
static double final_score(const std::vector<std::array<std::array<double, 6>, 3>>& scales) {
  double ssim = 0.0;
  int i = 0;
  for (int c = 0; c < 3; c++)
    for (auto& sc : scales)
      for (int n = 0; n < 2; n++) {
        ssim += WEIGHTS[i] * std::fabs(sc[c][n]);
        i++;
        ssim += WEIGHTS[i] * std::fabs(sc[c][2 + n]);
        i++;
        ssim += WEIGHTS[i] * std::fabs(sc[c][4 + n]);
        i++;
      }
  ssim *= 0.9562382616834844;
  ssim = 2.326765642916932 * ssim - 0.020884521182843837 * ssim * ssim + 6.248496625763138e-05 * ssim * ssim * ssim;
  return ssim > 0.0 ? 100.0 - 10.0 * std::pow(ssim, 0.6276336467831387) : 100.0;
}

// core/src/ssimulacra2.rs:471-512 (ssimulacra2). Returns 0 on success, 1 for the reference's Error::Invalid cases.
template <class P>
static int ssimulacra2_t(const uint8_t* ra, const uint8_t* da, int w, int h, int channels, int depth, double* score,
                         double* per_scale /* nullable: [6][3][6] */, int* nscales) {
  if (w < 8 || h < 8) return 1;
  Planes<P> a = linear_planes<P>(ra, w, h, channels, depth);
  Planes<P> b = linear_planes<P>(da, w, h, channels, depth);
  std::vector<std::array<std::array<double, 6>, 3>> scales;
  for (int s = 0; s < NUM_SCALES; s++) {
    if (a.w < 8 || a.h < 8) break;
    double st[3][6];
    scale_stats(a, b, st);
    std::array<std::array<double, 6>, 3> arr;
    for (int c = 0; c < 3; c++)
      for (int j = 0; j < 6; j++) arr[c][j] = st[c][j];
    scales.push_back(arr);
    if (s + 1 < NUM_SCALES) {
      a = downsample(a);
      b = downsample(b);
    }
  }
  if (per_scale) {
    for (size_t s = 0; s < scales.size(); s++)
      for (int c = 0; c < 3; c++)
        for (int j = 0; j < 6; j++) per_scale[(s * 3 + c) * 6 + j] = scales[s][c][j];
  }
  if (nscales) *nscales = (int)scales.size();
  double sc = final_score(scales);
  if (!std::isfinite(sc)) return 1;
  *score = sc;
  return 0;
}

// ------------------------------------------------------------------------------------------------ SSIMULACRA2 adjoint

// The score as a differentiable function of the distorted image's RGB samples taken as continuous values in
// [0, 255] (FP64 throughout): linear light by the sRGB curve itself (core/src/ssimulacra2.rs:172-175, of which the
// reference's 8-bit table is a sampling), then exactly the scorer's steps (:471-512). For integer samples it equals
// the FP64 scorer. grad64 is its reverse-mode derivative, every step's adjoint taken in turn: the 108-term sum and
// the final mapping, the L1/L4 norms, the SSIM and edge maps (one-sided derivatives at the max(., 0) and |.|
// kinks), the separable blurs (the horizontal pass with zero padding is its own transpose; the vertical pass's
// mirrored taps scatter back), the XYB transform, the 2x2 pyramid and the sRGB curve.

struct Img64 {
  int w = 0, h = 0;
  std::vector<double> ch[3];
};

static double srgb_deriv(double v255) {  // d srgb_to_linear(v / 255) / dv
  const double v = v255 / 255.0;
  if (v <= 0.04045) return 1.0 / (12.92 * 255.0);
  return 2.4 * std::pow((v + 0.055) / 1.055, 1.4) / (1.055 * 255.0);
}

static Img64 down64(const Img64& p) {
  Img64 o;
  o.w = (p.w + 1) / 2;
  o.h = (p.h + 1) / 2;
  for (int c = 0; c < 3; c++) {
    o.ch[c].assign((size_t)o.w * o.h, 0.0);
    for (int oy = 0; oy < o.h; oy++)
      for (int ox = 0; ox < o.w; ox++) {
        int x1 = std::min(2 * ox + 2, p.w), y1 = std::min(2 * oy + 2, p.h);
        double sum = 0.0;
        for (int y = 2 * oy; y < y1; y++)
          for (int x = 2 * ox; x < x1; x++) sum += p.ch[c][(size_t)y * p.w + x];
        o.ch[c][(size_t)oy * o.w + ox] = sum / (double)((y1 - 2 * oy) * (x1 - 2 * ox));
      }
  }
  return o;
}

// Row blur with zero padding (blur_row, :273-319) and column blur with mirrored rows (:385-397).
static void hblur64(const std::vector<double>& src, std::vector<double>& dst, int w, int h, const double* k) {
  dst.assign((size_t)w * h, 0.0);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      double s = 0.0;
      for (int t = 0; t <= 2 * RADIUS; t++) {
        int xx = x + t - RADIUS;
        if (xx >= 0 && xx < w) s += k[t] * src[(size_t)y * w + xx];
      }
      dst[(size_t)y * w + x] = s;
    }
}
static inline int mirror64(int yy, int h) { return yy < 0 ? -yy - 1 : (yy >= h ? 2 * h - 1 - yy : yy); }
static void vblur64(const std::vector<double>& src, std::vector<double>& dst, int w, int h, const double* k) {
  dst.assign((size_t)w * h, 0.0);
  for (int y = 0; y < h; y++)
    for (int t = 0; t <= 2 * RADIUS; t++) {
      const double* r = &src[(size_t)mirror64(y + t - RADIUS, h) * w];
      for (int x = 0; x < w; x++) dst[(size_t)y * w + x] += k[t] * r[x];
    }
}
static void vblur64_t(const std::vector<double>& g, std::vector<double>& out, int w, int h, const double* k) {
  out.assign((size_t)w * h, 0.0);
  for (int y = 0; y < h; y++)
    for (int t = 0; t <= 2 * RADIUS; t++) {
      double* r = &out[(size_t)mirror64(y + t - RADIUS, h) * w];
      for (int x = 0; x < w; x++) r[x] += k[t] * g[(size_t)y * w + x];
    }
}

struct ScaleFwd {
  int w, h;
  std::vector<double> xa[3], xb[3];   // XYB of both images
  std::vector<double> mom[3][5];      // blurred m1, m2, s11, s22, s12 per channel
  double sums[3][6];
};

static void xyb_planes(const Img64& p, std::vector<double> out[3]) {
  const size_t n = (size_t)p.w * p.h;
  for (int c = 0; c < 3; c++) out[c].assign(n, 0.0);
  for (size_t i = 0; i < n; i++) {
    double v[3];
    xyb(p.ch[0][i], p.ch[1][i], p.ch[2][i], v);
    for (int c = 0; c < 3; c++) out[c][i] = v[c];
  }
}

static void scale_forward(const Img64& a, const Img64& b, const double* k, ScaleFwd& f) {
  f.w = a.w;
  f.h = a.h;
  const int w = a.w, h = a.h;
  const size_t n = (size_t)w * h;
  xyb_planes(a, f.xa);
  xyb_planes(b, f.xb);
  std::vector<double> tmp(n), hb;
  for (int c = 0; c < 3; c++) {
    for (int q = 0; q < 5; q++) {
      for (size_t i = 0; i < n; i++) {
        const double xa = f.xa[c][i], xb = f.xb[c][i];
        tmp[i] = q == 0 ? xa : q == 1 ? xb : q == 2 ? xa * xa : q == 3 ? xb * xb : xa * xb;
      }
      hblur64(tmp, hb, w, h, k);
      vblur64(hb, f.mom[c][q], w, h, k);
    }
    for (int j = 0; j < 6; j++) f.sums[c][j] = 0.0;
    for (size_t i = 0; i < n; i++) {
      const double m1 = f.mom[c][0][i], m2 = f.mom[c][1][i];
      const double num_m = 1.0 - (m1 - m2) * (m1 - m2);
      const double num_s = 2.0 * (f.mom[c][4][i] - m1 * m2) + C2;
      const double den_s = (f.mom[c][2][i] - m1 * m1) + (f.mom[c][3][i] - m2 * m2) + C2;
      const double d = std::max(1.0 - num_m * num_s / den_s, 0.0);
      const double d1 = (1.0 + std::fabs(f.xb[c][i] - m2)) / (1.0 + std::fabs(f.xa[c][i] - m1)) - 1.0;
      const double art = std::max(d1, 0.0), det = std::max(-d1, 0.0);
      f.sums[c][0] += d;
      f.sums[c][1] += (d * d) * (d * d);
      f.sums[c][2] += art;
      f.sums[c][3] += (art * art) * (art * art);
      f.sums[c][4] += det;
      f.sums[c][5] += (det * det) * (det * det);
    }
  }
}

static Img64 linear64(const double* rgb, int w, int h) {
  Img64 o;
  o.w = w;
  o.h = h;
  for (int c = 0; c < 3; c++) o.ch[c].assign((size_t)w * h, 0.0);
  for (size_t i = 0; i < (size_t)w * h; i++)
    for (int c = 0; c < 3; c++) o.ch[c][i] = srgb_to_linear(rgb[i * 3 + c] / 255.0);
  return o;
}

// Forward pass at every scale; returns the score (100 when the weighted sum is not positive).
static double score64(const double* ref, const double* dist, int w, int h, std::vector<ScaleFwd>* keep,
                      std::vector<Img64>* pyr_b) {
  double k[2 * RADIUS + 1];
  gauss_kernel(k);
  Img64 a = linear64(ref, w, h), b = linear64(dist, w, h);
  std::vector<std::array<std::array<double, 6>, 3>> scales;
  for (int s = 0; s < NUM_SCALES; s++) {
    if (a.w < 8 || a.h < 8) break;
    ScaleFwd f;
    scale_forward(a, b, k, f);
    const double count = (double)a.w * (double)a.h;
    std::array<std::array<double, 6>, 3> arr;
    for (int c = 0; c < 3; c++)
      for (int m = 0; m < 3; m++) {
        arr[c][2 * m] = f.sums[c][2 * m] / count;
        arr[c][2 * m + 1] = std::pow(f.sums[c][2 * m + 1] / count, 0.25);
      }
    scales.push_back(arr);
    if (pyr_b) pyr_b->push_back(b);
    if (keep) keep->push_back(std::move(f));
    if (s + 1 < NUM_SCALES) {
      a = down64(a);
      b = down64(b);
    }
  }
  return final_score(scales);
}

// d score / d dist (RGB, w x h x 3). Returns the score.
static double grad64(const double* ref, const double* dist, int w, int h, double* grad) {
  double k[2 * RADIUS + 1];
  gauss_kernel(k);
  std::vector<ScaleFwd> F;
  std::vector<Img64> B;
  const double score = score64(ref, dist, w, h, &F, &B);
  const int ns = (int)F.size();
  std::memset(grad, 0, sizeof(double) * (size_t)w * h * 3);
  // final mapping and the weighted sum (:491-511): d score / d stat
  double sum = 0.0;
  std::vector<std::array<std::array<double, 6>, 3>> st(ns);
  for (int s = 0; s < ns; s++) {
    const double count = (double)F[s].w * F[s].h;
    for (int c = 0; c < 3; c++)
      for (int m = 0; m < 3; m++) {
        st[s][c][2 * m] = F[s].sums[c][2 * m] / count;
        st[s][c][2 * m + 1] = std::pow(F[s].sums[c][2 * m + 1] / count, 0.25);
      }
  }
  std::vector<std::array<std::array<double, 6>, 3>> wst(ns);  // weight of each stat in the sum
  int i = 0;
  for (int c = 0; c < 3; c++)
    for (int s = 0; s < ns; s++)
      for (int n = 0; n < 2; n++)
        for (int m = 0; m < 3; m++) {
          wst[s][c][2 * m + n] = WEIGHTS[i];
          sum += WEIGHTS[i] * std::fabs(st[s][c][2 * m + n]);
          i++;
        }
  const double kq = 0.9562382616834844;
  const double q = sum * kq;
  const double P = 2.326765642916932 * q - 0.020884521182843837 * q * q + 6.248496625763138e-05 * q * q * q;
  if (!(P > 0.0)) return score;
  const double e = 0.6276336467831387;
  const double dscore_dsum =
      -10.0 * e * std::pow(P, e - 1.0) *
      (2.326765642916932 - 2.0 * 0.020884521182843837 * q + 3.0 * 6.248496625763138e-05 * q * q) * kq;
  std::vector<double> gB[3];  // gradient w.r.t. the linear dist planes of the current scale (coarsest first)
  for (int s = ns - 1; s >= 0; s--) {
    const ScaleFwd& f = F[s];
    const int sw = f.w, sh = f.h;
    const size_t n = (size_t)sw * sh;
    const double count = (double)n;
    std::vector<double> gLin[3];
    for (int c = 0; c < 3; c++) gLin[c].assign(n, 0.0);
    std::vector<double> gxb[3];
    for (int c = 0; c < 3; c++) {
      // d score / d map(x) for the six norms: L1 -> 1/count, L4 -> map^3 (S/count)^-3/4 / count
      double g1[3], g4[3];
      for (int m = 0; m < 3; m++) {
        // stats are >= 0: |.| has derivative 1
        g1[m] = dscore_dsum * wst[s][c][2 * m] / count;
        const double mean4 = f.sums[c][2 * m + 1] / count;
        g4[m] = mean4 > 0.0 ? dscore_dsum * wst[s][c][2 * m + 1] * std::pow(mean4, -0.75) / count : 0.0;
      }
      std::vector<double> gm[5];
      for (int qq = 0; qq < 5; qq++) gm[qq].assign(n, 0.0);
      gxb[c].assign(n, 0.0);
      for (size_t p = 0; p < n; p++) {
        const double m1 = f.mom[c][0][p], m2 = f.mom[c][1][p];
        const double s11 = f.mom[c][2][p], s22 = f.mom[c][3][p], s12 = f.mom[c][4][p];
        const double num_m = 1.0 - (m1 - m2) * (m1 - m2);
        const double num_s = 2.0 * (s12 - m1 * m2) + C2;
        const double den_s = (s11 - m1 * m1) + (s22 - m2 * m2) + C2;
        const double dv = 1.0 - num_m * num_s / den_s;
        const double d = std::max(dv, 0.0);
        const double gd = g1[0] + g4[0] * d * d * d;
        if (dv > 0.0) {
          const double g_num_m = -gd * num_s / den_s, g_num_s = -gd * num_m / den_s;
          const double g_den = gd * num_m * num_s / (den_s * den_s);
          gm[0][p] += g_num_m * (-2.0 * (m1 - m2)) + g_num_s * (-2.0 * m2) + g_den * (-2.0 * m1);
          gm[1][p] += g_num_m * (2.0 * (m1 - m2)) + g_num_s * (-2.0 * m1) + g_den * (-2.0 * m2);
          gm[2][p] += g_den;
          gm[3][p] += g_den;
          gm[4][p] += 2.0 * g_num_s;
        }
        const double xa = f.xa[c][p], xb = f.xb[c][p];
        const double Nn = 1.0 + std::fabs(xb - m2), Dn = 1.0 + std::fabs(xa - m1);
        const double d1 = Nn / Dn - 1.0;
        const double art = std::max(d1, 0.0), det = std::max(-d1, 0.0);
        const double gd1 = (d1 > 0.0 ? g1[1] + g4[1] * art * art * art : 0.0) -
                           (d1 < 0.0 ? g1[2] + g4[2] * det * det * det : 0.0);
        const double sb = xb - m2 > 0.0 ? 1.0 : (xb - m2 < 0.0 ? -1.0 : 0.0);
        const double sa = xa - m1 > 0.0 ? 1.0 : (xa - m1 < 0.0 ? -1.0 : 0.0);
        gxb[c][p] += gd1 * sb / Dn;
        gm[1][p] += -gd1 * sb / Dn;
        gm[0][p] += gd1 * Nn / (Dn * Dn) * sa;
      }
      // blur adjoints for the moments that depend on the dist image: m2 = G(xb), s22 = G(xb^2), s12 = G(xa xb)
      std::vector<double> t1, t2;
      for (int qq : {1, 3, 4}) {
        vblur64_t(gm[qq], t1, sw, sh, k);
        hblur64(t1, t2, sw, sh, k);  // zero-padded symmetric row blur is its own transpose
        for (size_t p = 0; p < n; p++) {
          const double fac = qq == 1 ? 1.0 : qq == 3 ? 2.0 * f.xb[c][p] : f.xa[c][p];
          gxb[c][p] += fac * t2[p];
        }
      }
    }
    // XYB adjoint (:249-258) to the linear dist planes of this scale
    const double cbb = std::cbrt(BIAS);
    (void)cbb;
    const Img64& lb = B[s];
    for (size_t p = 0; p < n; p++) {
      const double r = lb.ch[0][p], g = lb.ch[1][p], bl = lb.ch[2][p];
      const double u[3] = {M00 * r + M01 * g + M02 * bl + BIAS, M10 * r + M11 * g + M12 * bl + BIAS,
                           M20 * r + M21 * g + M22 * bl + BIAS};
      double dm[3];
      for (int j = 0; j < 3; j++) dm[j] = u[j] > 0.0 ? 1.0 / (3.0 * std::cbrt(u[j]) * std::cbrt(u[j])) : 0.0;
      // X = 7 (m0 - m1) + 0.42, Y = (m0 + m1) / 2 + 0.01, B = m2 - (m0 + m1) / 2 + 0.55
      const double gX = gxb[0][p], gY = gxb[1][p], gBb = gxb[2][p];
      const double g_m0 = 7.0 * gX + 0.5 * gY - 0.5 * gBb, g_m1 = -7.0 * gX + 0.5 * gY - 0.5 * gBb, g_m2 = gBb;
      const double gu[3] = {g_m0 * dm[0], g_m1 * dm[1], g_m2 * dm[2]};
      gLin[0][p] += gu[0] * M00 + gu[1] * M10 + gu[2] * M20;
      gLin[1][p] += gu[0] * M01 + gu[1] * M11 + gu[2] * M21;
      gLin[2][p] += gu[0] * M02 + gu[1] * M12 + gu[2] * M22;
    }
    // plus the coarser scales' gradients, spread back over each 2x2 block
    if (s + 1 < ns) {
      const int cw = F[s + 1].w;
      for (int c = 0; c < 3; c++)
        for (int y = 0; y < sh; y++)
          for (int x = 0; x < sw; x++) {
            const int ox = x / 2, oy = y / 2;
            const int nx = std::min(2 * ox + 2, sw) - 2 * ox, ny = std::min(2 * oy + 2, sh) - 2 * oy;
            gLin[c][(size_t)y * sw + x] += gB[c][(size_t)oy * cw + ox] / (double)(nx * ny);
          }
    }
    for (int c = 0; c < 3; c++) gB[c] = std::move(gLin[c]);
  }
  for (size_t p = 0; p < (size_t)w * h; p++)
    for (int c = 0; c < 3; c++) grad[p * 3 + c] = gB[c][p] * srgb_deriv(dist[p * 3 + c]);
  return score;
}

// ------------------------------------------------------------------------------------------------ search

// jpeg/src/target.rs:12-56 (find_quality_with) with the metric of cli/src/pipeline.rs:214-219
// (ssimulacra2(..).unwrap_or(f64::MIN)) and `make` = build_coefs at quality q (cli/src/pipeline.rs:238).
struct Found {
  int quality;
  double score;
  CoefImage coefs;
};

// ------------------------------------------------------------------------------------------------ metrics

static const double SSIM_C1 = 6.5025;   // (0.01 * 255)^2, core/src/metrics.rs:6
static const double SSIM_C2 = 58.5225;  // (0.03 * 255)^2, core/src/metrics.rs:7

// core/src/metrics.rs:39-62 (window_ssim): per channel f64 sums over the window, then the SSIM formula.
static double window_ssim(const uint8_t* a, const uint8_t* b, int w, int x0, int y0, int ww, int wh, int ch) {
  double total = 0.0;
  for (int c = 0; c < ch; c++) {
    double sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
    for (int y = y0; y < y0 + wh; y++) {
      size_t row = ((size_t)y * w + x0) * ch + c;
      for (int i = 0; i < ww; i++) {
        double p = a[row + (size_t)i * ch], q = b[row + (size_t)i * ch];
        sx += p;
        sy += q;
        sxx += p * p;
        syy += q * q;
        sxy += p * q;
      }
    }
    double n = (double)ww * (double)wh;
    double mx = sx / n, my = sy / n;
    double vx = sxx / n - mx * mx, vy = syy / n - my * my, cov = sxy / n - mx * my;
    total += ((2.0 * mx * my + SSIM_C1) * (2.0 * cov + SSIM_C2)) / ((mx * mx + my * my + SSIM_C1) * (vx + vy + SSIM_C2));
  }
  return total / ch;
}

// core/src/metrics.rs:13-37 (ssim): 8x8 windows every 4 pixels, or one global window below 8 pixels. Each row of
// windows is summed left to right; the rows are added in order (the reference adds them with rayon's reduce, whose
// association is unspecified: the two agree to rounding).
static double ssim(const uint8_t* a, const uint8_t* b, int w, int h, int ch) {
  if (w < 8 || h < 8) return window_ssim(a, b, w, 0, 0, w, h, ch);
  int ny = (h - 8) / 4 + 1, nx = (w - 8) / 4 + 1;
  std::vector<double> rows(ny);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; j++) {
    double sum = 0.0;
    for (int i = 0; i < nx; i++) sum += window_ssim(a, b, w, 4 * i, 4 * j, 8, 8, ch);
    rows[j] = sum;
  }
  double sum = 0.0;
  for (int j = 0; j < ny; j++) sum += rows[j];
  return sum / (double)((size_t)ny * nx);
}

// core/src/metrics.rs:64-73 (psnr)
static double psnr(const uint8_t* a, const uint8_t* b, size_t n) {
  double se = 0.0;
  for (size_t i = 0; i < n; i++) {
    double d = (double)a[i] - (double)b[i];
    se += d * d;
  }
  double mse = se / (double)std::max<size_t>(n, 1);
  return mse == 0.0 ? INFINITY : 10.0 * std::log10(255.0 * 255.0 / mse);
}

// core/src/metrics.rs:75-87 (luma): Gray as is, GrayAlpha's gray, Rgb/Rgba -> (299R + 587G + 114B + 500) / 1000.
static std::vector<uint8_t> luma(const uint8_t* a, size_t npx, int ch) {
  std::vector<uint8_t> out(npx);
  for (size_t i = 0; i < npx; i++) {
    const uint8_t* p = a + i * ch;
    out[i] = ch <= 2 ? p[0] : (uint8_t)((299u * p[0] + 587u * p[1] + 114u * p[2] + 500u) / 1000u);
  }
  return out;
}

// core/src/metrics.rs:89-106 (downsample2)
static std::vector<uint8_t> downsample2(const std::vector<uint8_t>& img, int& w, int& h) {
  int nw = w / 2, nh = h / 2;
  if (nw == 0 || nh == 0) return img;
  std::vector<uint8_t> out((size_t)nw * nh);
  for (int y = 0; y < nh; y++)
    for (int x = 0; x < nw; x++) {
      unsigned s = 0;
      for (int dy = 0; dy < 2; dy++)
        for (int dx = 0; dx < 2; dx++) s += img[(size_t)(2 * y + dy) * w + 2 * x + dx];
      out[(size_t)y * nw + x] = (uint8_t)(s / 4);
    }
  w = nw;
  h = nh;
  return out;
}

// core/src/metrics.rs:108-127 (ms_ssim)
static double ms_ssim(const uint8_t* a, const uint8_t* b, int w, int h, int ch, double* per_scale) {
  static const double W[5] = {0.0448, 0.2856, 0.3001, 0.2363, 0.1333};
  std::vector<uint8_t> x = luma(a, (size_t)w * h, ch), y = luma(b, (size_t)w * h, ch);
  double out = 1.0;
  int cw = w, chh = h;
  for (int i = 0; i < 5; i++) {
    double s = std::max(ssim(x.data(), y.data(), cw, chh, 1), 1e-9);
    if (per_scale) per_scale[i] = s;
    out *= std::pow(s, W[i]);
    if (i + 1 < 5) {
      int w2 = cw, h2 = chh;
      x = downsample2(x, w2, h2);
      w2 = cw;
      h2 = chh;
      y = downsample2(y, w2, h2);
      cw = w2;
      chh = h2;
    }
  }
  return out;
}

enum { METRIC_SSIMULACRA2 = 0, METRIC_SSIM = 1 };

// The search's metric on a candidate (jpeg/src/target.rs:38): ssimulacra2 maps a failure to f64::MIN
// (cli/src/pipeline.rs:218); ssim always scores.
static double score_coefs(const uint8_t* ref, int w, int h, int channels, const CoefImage& ci,
                          int metric = METRIC_SSIMULACRA2) {
  (void)channels;
  int oc = 0;
  std::vector<uint8_t> img = reconstruct(ci, &oc);
  if (metric == METRIC_SSIM) return ssim(ref, img.data(), w, h, oc);
  double s = 0.0;
  if (ssimulacra2_t<float>(ref, img.data(), w, h, oc, 8, &s, nullptr, nullptr) != 0) return -1.7976931348623157e308;
  return s;
}

static Found find_quality(const uint8_t* ref, int w, int h, int channels, double target, int max_quality,
                          int subsampling, bool trellis, std::vector<std::pair<int, double>>* trace,
                          int metric = METRIC_SSIMULACRA2, const float* weights = nullptr) {
  int lo = 1, hi = std::max(max_quality, 1);
  CoefImage top = build_coefs(ref, w, h, channels, hi, subsampling, trellis, weights);
  double top_score = score_coefs(ref, w, h, channels, top, metric);
  if (trace) trace->push_back({hi, top_score});
  Found best{hi, top_score, std::move(top)};
  if (top_score < target) return best;
  while (lo < hi) {
    int mid = lo + (hi - lo) / 2;
    CoefImage ci = build_coefs(ref, w, h, channels, mid, subsampling, trellis, weights);
    double s = score_coefs(ref, w, h, channels, ci, metric);
    if (trace) trace->push_back({mid, s});
    if (s >= target) {
      hi = mid;
      best = Found{mid, s, std::move(ci)};
    } else {
      lo = mid + 1;
    }
  }
  return best;
}

// ------------------------------------------------------------------------------------------------ requantize

// jpeg/src/encode.rs:107-172 (CoefImage::requantize) for 1- and 3-component images (table class = component index
// min 1, jpeg/src/encode.rs:99-105).
static void requantize(CoefImage& ci, int quality, bool trellis) {
  uint8_t tables[2][64];
  luma_table(quality, tables[0]);
  chroma_table(quality, tables[1]);
  uint8_t new_slots[4][64];
  bool has_new[4] = {false, false, false, false};
  bool changed = false;
  struct Plan {
    int slot;
    float ratio[64];
    uint8_t nt[64];
  };
  std::vector<Plan> plan;
  std::vector<std::vector<int16_t>> originals;
  if (trellis)
    for (auto& c : ci.comps) originals.push_back(c.coefs);
  for (size_t k = 0; k < ci.comps.size(); k++) {
    CoefComponent& c = ci.comps[k];
    uint8_t old[64];
    if (ci.has_q[c.tq])
      std::memcpy(old, ci.qtables[c.tq], 64);
    else
      std::memset(old, 1, 64);
    const uint8_t* base = tables[std::min<size_t>(k, 1)];
    Plan pl;
    for (int n = 0; n < 64; n++) pl.nt[n] = std::max(base[n], old[n]);
    changed |= std::memcmp(pl.nt, old, 64) != 0;
    for (int z = 0; z < 64; z++) pl.ratio[z] = (float)old[ZIGZAG[z]] / (float)pl.nt[ZIGZAG[z]];
    size_t nb = c.coefs.size() / 64;
#pragma omp parallel for schedule(static)
    for (long b = 0; b < (long)nb; b++) {
      int16_t* blk = &c.coefs[(size_t)b * 64];
      for (int z = 0; z < 64; z++) blk[z] = (int16_t)clampi(round_f32((float)blk[z] * pl.ratio[z]), -2047, 2047);
    }
    int slot = -1;
    for (int sl = 0; sl < 4; sl++)
      if (has_new[sl] && std::memcmp(new_slots[sl], pl.nt, 64) == 0) {
        slot = sl;
        break;
      }
    if (slot < 0) {
      for (int sl = 0; sl < 4; sl++)
        if (!has_new[sl]) {
          slot = sl;
          break;
        }
      std::memcpy(new_slots[slot], pl.nt, 64);
      has_new[slot] = true;
    }
    c.tq = slot;
    pl.slot = slot;
    plan.push_back(pl);
  }
  for (int sl = 0; sl < 4; sl++) {
    ci.has_q[sl] = has_new[sl];
    if (has_new[sl]) std::memcpy(ci.qtables[sl], new_slots[sl], 64);
  }
  if (trellis && changed) {
    uint8_t lens[2][256];
    ac_code_lengths(ci, lens);
    for (size_t k = 0; k < ci.comps.size(); k++) {
      Rdo rdo(plan[k].nt, TRELLIS_KAPPA, lens[std::min<size_t>(k, 1)]);
      CoefComponent& c = ci.comps[k];
      size_t nb = c.coefs.size() / 64;
#pragma omp parallel for schedule(dynamic, 64)
      for (long b = 0; b < (long)nb; b++) {
        float a[64];
        const int16_t* in = &originals[k][(size_t)b * 64];
        for (int z = 0; z < 64; z++) a[z] = (float)in[z] * plan[k].ratio[z];
        rdo.quantize_ac(a, &c.coefs[(size_t)b * 64]);
      }
    }
  }
}

// cli/src/pipeline.rs:369-386: the JPEG->JPEG search. The reference image is the source reconstructed; each
// candidate is the source requantized (jpeg/src/target.rs:29-56 drives it).
static Found find_quality_requantize(const CoefImage& src, double target, int max_quality, bool trellis,
                                     std::vector<std::pair<int, double>>* trace, int metric = METRIC_SSIMULACRA2) {
  int oc = 0;
  std::vector<uint8_t> ref = reconstruct(src, &oc);
  auto make = [&](int q) {
    CoefImage c = src;
    requantize(c, q, trellis);
    return c;
  };
  int lo = 1, hi = std::max(max_quality, 1);
  CoefImage top = make(hi);
  double top_score = score_coefs(ref.data(), src.width, src.height, oc, top, metric);
  if (trace) trace->push_back({hi, top_score});
  Found best{hi, top_score, std::move(top)};
  if (top_score < target) return best;
  while (lo < hi) {
    int mid = lo + (hi - lo) / 2;
    CoefImage ci = make(mid);
    double s = score_coefs(ref.data(), src.width, src.height, oc, ci, metric);
    if (trace) trace->push_back({mid, s});
    if (s >= target) {
      hi = mid;
      best = Found{mid, s, std::move(ci)};
    } else {
      lo = mid + 1;
    }
  }
  return best;
}

// ------------------------------------------------------------------------------------------------ write_best

// jpeg/src/encode.rs:400-413 (segment, write_dht)
static void segment(std::vector<uint8_t>& out, uint8_t marker, const std::vector<uint8_t>& body) {
  out.push_back(0xFF);
  out.push_back(marker);
  uint16_t len = (uint16_t)(body.size() + 2);
  out.push_back((uint8_t)(len >> 8));
  out.push_back((uint8_t)(len & 0xFF));
  out.insert(out.end(), body.begin(), body.end());
}

static void write_dht(std::vector<uint8_t>& out, uint8_t class_id, const HuffTable& t) {
  std::vector<uint8_t> body{class_id};
  body.insert(body.end(), t.bits + 1, t.bits + 17);
  body.insert(body.end(), t.vals.begin(), t.vals.end());
  segment(out, 0xC4, body);
}

// jpeg/src/encode.rs:644-673 (write_headers) for a CoefImage without metadata or Adobe marker.
static std::vector<uint8_t> write_headers(const CoefImage& ci, uint8_t sof_marker) {
  std::vector<uint8_t> out{0xFF, 0xD8};
  segment(out, 0xE0, {'J', 'F', 'I', 'F', 0, 1, 1, 0, 0, 1, 0, 1, 0, 0});
  std::vector<uint8_t> dqt;
  for (int slot = 0; slot < 4; slot++)
    if (ci.has_q[slot]) {
      dqt.push_back((uint8_t)slot);
      for (int k = 0; k < 64; k++) dqt.push_back(ci.qtables[slot][ZIGZAG[k]]);
    }
  segment(out, 0xDB, dqt);
  std::vector<uint8_t> sof{8, (uint8_t)(ci.height >> 8), (uint8_t)(ci.height & 0xFF), (uint8_t)(ci.width >> 8),
                           (uint8_t)(ci.width & 0xFF), (uint8_t)ci.comps.size()};
  for (auto& c : ci.comps) {
    sof.push_back(c.id);
    sof.push_back((uint8_t)(c.h << 4 | c.v));
    sof.push_back((uint8_t)c.tq);
  }
  segment(out, sof_marker, sof);
  return out;
}

// jpeg/src/encode.rs:548-565 (baseline_estimate)
static uint64_t baseline_estimate(const CoefImage& ci) {
  int mx, my;
  ci.mcus(mx, my);
  Stats st;
  scan(ci.comps, mx, my, st);
  uint64_t bits = st.raw_bits, total = 0;
  int ntab = ci.comps.size() == 1 ? 1 : 2;
  for (int cls = 0; cls < 2; cls++)
    for (int t = 0; t < ntab; t++) {
      const uint32_t* freq = cls == 0 ? st.dc[t] : st.ac[t];
      HuffTable ht = optimal_table(freq);
      for (int s = 0; s < 256; s++) bits += (uint64_t)freq[s] * ht.size[s];
      total += 5 + 16 + ht.vals.size();
    }
  return total + (bits + 7) / 8 + 20;
}

// jpeg/src/encode.rs:567-608 (write_jpeg / write_jpeg_with, non-differential)
static std::vector<uint8_t> write_jpeg(const CoefImage& ci) {
  int mx, my;
  ci.mcus(mx, my);
  int ntables = ci.comps.size() == 1 ? 1 : 2;
  Stats st;
  scan(ci.comps, mx, my, st);
  HuffTable dct[2] = {optimal_table(st.dc[0]), optimal_table(st.dc[1])};
  HuffTable act[2] = {optimal_table(st.ac[0]), optimal_table(st.ac[1])};
  Writer wr{MsbWriter{}, dct, act};
  scan(ci.comps, mx, my, wr);
  wr.w.finish();
  std::vector<uint8_t> out = write_headers(ci, 0xC0);
  for (int t = 0; t < ntables; t++) {
    write_dht(out, (uint8_t)t, dct[t]);
    write_dht(out, (uint8_t)(0x10 | t), act[t]);
  }
  std::vector<uint8_t> sos{(uint8_t)ci.comps.size()};
  for (size_t i = 0; i < ci.comps.size(); i++) {
    uint8_t s = (uint8_t)std::min<size_t>(i, 1);
    sos.push_back(ci.comps[i].id);
    sos.push_back((uint8_t)(s << 4 | s));
  }
  sos.push_back(0);
  sos.push_back(63);
  sos.push_back(0);
  segment(out, 0xDA, sos);
  out.insert(out.end(), wr.w.out.begin(), wr.w.out.end());
  out.push_back(0xFF);
  out.push_back(0xD9);
  return out;
}

// jpeg/src/progressive.rs:14-21 (Scan)
struct Scan {
  std::vector<int> comps;
  int ss, se;
  uint32_t ah, al;
  bool operator<(const Scan& o) const {
    return std::tie(comps, ss, se, ah, al) < std::tie(o.comps, o.ss, o.se, o.ah, o.al);
  }
};

// jpeg/src/progressive.rs:7-51 (ScanSink, Stats, Emit)
struct PStats {
  uint32_t freq[2][2][256];
  uint64_t raw_bits;
  PStats() { std::memset(this, 0, sizeof *this); }
  void sym(int cls, int slot, uint8_t s) { freq[cls][slot][s] += 1; }
  void bits(uint32_t, uint32_t n) { raw_bits += n; }
};

struct PTables {
  HuffTable t[2][2];
  bool has[2][2];
};

struct PEmit {
  MsbWriter w;
  const PTables* tables;
  void sym(int cls, int slot, uint8_t s) {
    const HuffTable& t = tables->t[cls][slot];
    w.put(t.code[s], t.size[s]);
  }
  void bits(uint32_t v, uint32_t n) { w.put(v, n); }
};

// jpeg/src/progressive.rs:53-63 (State)
struct PState {
  int32_t last_dc[4] = {0, 0, 0, 0};
  uint32_t eobrun = 0;
  std::vector<uint8_t> pending, br;
};

static const size_t MAX_CORR_BITS = 1000;
static inline uint32_t nbits(uint32_t v) { return v == 0 ? 0 : 32 - (uint32_t)__builtin_clz(v); }

// jpeg/src/progressive.rs:71-83
template <class S>
static void emit_eobrun(PState& st, S& sink) {
  if (st.eobrun > 0) {
    uint32_t nb = nbits(st.eobrun) - 1;
    sink.sym(1, 0, (uint8_t)(nb << 4));
    if (nb > 0) sink.bits(st.eobrun & ((1u << nb) - 1), nb);
    st.eobrun = 0;
    for (uint8_t b : st.pending) sink.bits(b, 1);
    st.pending.clear();
  }
}

// jpeg/src/progressive.rs:85-98
template <class S>
static void dc_first(PState& st, S& sink, const int16_t* blk, int comp, int slot, uint32_t al) {
  int32_t v = (int32_t)(blk[0] >> al);
  int32_t diff = v - st.last_dc[comp];
  st.last_dc[comp] = v;
  uint32_t nb = nbits(diff < 0 ? (uint32_t)(-(int64_t)diff) : (uint32_t)diff);
  sink.sym(0, slot, (uint8_t)nb);
  if (nb > 0) {
    uint32_t extra = (diff < 0 ? (uint32_t)(diff - 1) : (uint32_t)diff) & ((1u << nb) - 1);
    sink.bits(extra, nb);
  }
}

// jpeg/src/progressive.rs:100-102
template <class S>
static void dc_refine(S& sink, const int16_t* blk, uint32_t al) {
  sink.bits((uint32_t)((blk[0] >> al) & 1), 1);
}

// jpeg/src/progressive.rs:104-139
template <class S>
static void ac_first(PState& st, S& sink, const int16_t* blk, const Scan& sc) {
  uint32_t r = 0;
  for (int k = sc.ss; k <= sc.se; k++) {
    int32_t v = blk[k];
    if (v == 0) {
      r++;
      continue;
    }
    int32_t mag, ext;
    if (v < 0) {
      mag = (-v) >> sc.al;
      ext = ~mag;
    } else {
      mag = v >> sc.al;
      ext = mag;
    }
    if (mag == 0) {
      r++;
      continue;
    }
    emit_eobrun(st, sink);
    while (r > 15) {
      sink.sym(1, 0, 0xF0);
      r -= 16;
    }
    uint32_t nb = nbits((uint32_t)mag);
    sink.sym(1, 0, (uint8_t)((r << 4) + nb));
    sink.bits((uint32_t)ext & ((1u << nb) - 1), nb);
    r = 0;
  }
  if (r > 0) {
    st.eobrun += 1;
    if (st.eobrun == 0x7FFF) emit_eobrun(st, sink);
  }
}

// jpeg/src/progressive.rs:141-189
template <class S>
static void ac_refine(PState& st, S& sink, const int16_t* blk, const Scan& sc) {
  int32_t absv[64] = {0};
  int eob = 0;
  for (int k = sc.ss; k <= sc.se; k++) {
    int32_t t = std::abs((int32_t)blk[k]) >> sc.al;
    absv[k] = t;
    if (t == 1) eob = k;
  }
  uint32_t r = 0;
  st.br.clear();
  for (int k = sc.ss; k <= sc.se; k++) {
    int32_t t = absv[k];
    if (t == 0) {
      r++;
      continue;
    }
    while (r > 15 && k <= eob) {
      emit_eobrun(st, sink);
      sink.sym(1, 0, 0xF0);
      r -= 16;
      for (uint8_t b : st.br) sink.bits(b, 1);
      st.br.clear();
    }
    if (t > 1) {
      st.br.push_back((uint8_t)(t & 1));
      continue;
    }
    emit_eobrun(st, sink);
    sink.sym(1, 0, (uint8_t)((r << 4) + 1));
    sink.bits(blk[k] < 0 ? 0 : 1, 1);
    for (uint8_t b : st.br) sink.bits(b, 1);
    st.br.clear();
    r = 0;
  }
  if (r > 0 || !st.br.empty()) {
    st.eobrun += 1;
    st.pending.insert(st.pending.end(), st.br.begin(), st.br.end());
    st.br.clear();
    if (st.eobrun == 0x7FFF || st.pending.size() > MAX_CORR_BITS - 63) emit_eobrun(st, sink);
  }
}

// jpeg/src/progressive.rs:191-240 (run_scan, non-differential)
template <class S>
static void run_scan(const CoefImage& ci, const Scan& sc, S& sink) {
  PState st;
  int hmax = ci.hv_max_h(), vmax = ci.hv_max_v();
  bool dc_scan = sc.ss == 0;
  auto visit = [&](int ci_idx, const int16_t* blk) {
    int slot = std::min(ci_idx, 1);
    if (dc_scan) {
      if (sc.ah == 0)
        dc_first(st, sink, blk, ci_idx, slot, sc.al);
      else
        dc_refine(sink, blk, sc.al);
    } else if (sc.ah == 0) {
      ac_first(st, sink, blk, sc);
    } else {
      ac_refine(st, sink, blk, sc);
    }
  };
  if (sc.comps.size() > 1) {
    int mx, my;
    ci.mcus(mx, my);
    for (int y = 0; y < my; y++)
      for (int x = 0; x < mx; x++)
        for (int k : sc.comps) {
          const CoefComponent& c = ci.comps[k];
          for (int by = 0; by < c.v; by++)
            for (int bx = 0; bx < c.h; bx++) {
              size_t b = (size_t)(y * c.v + by) * c.blocks_w + x * c.h + bx;
              visit(k, &c.coefs[b * 64]);
            }
        }
  } else {
    int k = sc.comps[0];
    const CoefComponent& c = ci.comps[k];
    int real_w = ((ci.width * c.h + hmax - 1) / hmax + 7) / 8;
    int real_h = ((ci.height * c.v + vmax - 1) / vmax + 7) / 8;
    for (int by = 0; by < real_h; by++)
      for (int bx = 0; bx < real_w; bx++) visit(k, &c.coefs[((size_t)by * c.blocks_w + bx) * 64]);
  }
  if (!dc_scan) emit_eobrun(st, sink);
}

// jpeg/src/progressive.rs:242-295 (scripts)
static std::vector<std::vector<Scan>> scripts(int ncomp) {
  auto s = [](std::vector<int> comps, int ss, int se, uint32_t ah, uint32_t al) { return Scan{comps, ss, se, ah, al}; };
  std::vector<int> all;
  for (int i = 0; i < ncomp; i++) all.push_back(i);
  std::vector<uint32_t> chroma_als = ncomp >= 3 ? std::vector<uint32_t>{0, 1} : std::vector<uint32_t>{0};
  std::vector<int> chroma_splits = ncomp >= 3 ? std::vector<int>{-1, 2, 5} : std::vector<int>{-1};
  std::vector<std::vector<Scan>> out;
  for (uint32_t dc_al : {0u, 1u})
    for (int split : {-1, 2, 5, 8})
      for (uint32_t luma_al : {0u, 1u, 2u})
        for (uint32_t chroma_al : chroma_als)
          for (int chroma_split : chroma_splits) {
            std::vector<Scan> v{s(all, 0, 0, 0, dc_al)};
            if (split < 0) {
              v.push_back(s({0}, 1, 63, 0, luma_al));
            } else {
              v.push_back(s({0}, 1, split, 0, luma_al));
              v.push_back(s({0}, split + 1, 63, 0, luma_al));
            }
            if (ncomp >= 3)
              for (int c = 1; c < ncomp; c++) {
                if (chroma_split < 0) {
                  v.push_back(s({c}, 1, 63, 0, chroma_al));
                } else {
                  v.push_back(s({c}, 1, chroma_split, 0, chroma_al));
                  v.push_back(s({c}, chroma_split + 1, 63, 0, chroma_al));
                }
              }
            if (dc_al > 0) v.push_back(s(all, 0, 0, 1, 0));
            for (uint32_t ah = luma_al; ah >= 1; ah--) v.push_back(s({0}, 1, 63, ah, ah - 1));
            for (uint32_t ah = chroma_al; ah >= 1; ah--)
              for (int c = 1; c < ncomp; c++) v.push_back(s({c}, 1, 63, ah, ah - 1));
            out.push_back(v);
          }
  return out;
}

// jpeg/src/progressive.rs:297-307
static PTables build_tables(const PStats& st) {
  PTables t;
  for (int cls = 0; cls < 2; cls++)
    for (int slot = 0; slot < 2; slot++) {
      bool any = false;
      for (int s = 0; s < 256; s++) any |= st.freq[cls][slot][s] > 0;
      t.has[cls][slot] = any;
      if (any) t.t[cls][slot] = optimal_table(st.freq[cls][slot]);
    }
  return t;
}

// jpeg/src/progressive.rs:309-327 (scan_cost)
static uint64_t scan_cost(const CoefImage& ci, const Scan& sc) {
  PStats st;
  run_scan(ci, sc, st);
  PTables t = build_tables(st);
  uint64_t bits = st.raw_bits, total = 0;
  for (int cls = 0; cls < 2; cls++)
    for (int slot = 0; slot < 2; slot++)
      if (t.has[cls][slot]) {
        for (int s = 0; s < 256; s++) bits += (uint64_t)st.freq[cls][slot][s] * t.t[cls][slot].size[s];
        total += 5 + 16 + t.t[cls][slot].vals.size();
      }
  return total + (bits + 7) / 8 + 14;
}

// jpeg/src/progressive.rs:335-351 (plan). min_by_key keeps the first minimum.
static uint64_t plan(const CoefImage& ci, std::vector<Scan>& best_script, std::vector<Scan>* distinct_out = nullptr,
                     std::vector<uint64_t>* cost_out = nullptr) {
  std::vector<std::vector<Scan>> cands = scripts((int)ci.comps.size());
  std::vector<Scan> distinct;
  std::set<Scan> seen;
  for (auto& sc_list : cands)
    for (auto& sc : sc_list)
      if (seen.insert(sc).second) distinct.push_back(sc);
  std::vector<uint64_t> cost(distinct.size());
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < (int)distinct.size(); i++) cost[i] = scan_cost(ci, distinct[i]);
  std::map<Scan, uint64_t> costs;
  for (size_t i = 0; i < distinct.size(); i++) costs[distinct[i]] = cost[i];
  uint64_t best_total = UINT64_MAX;
  size_t best_i = 0;
  for (size_t i = 0; i < cands.size(); i++) {
    uint64_t t = 0;
    for (auto& sc : cands[i]) t += costs[sc];
    if (t < best_total) {
      best_total = t;
      best_i = i;
    }
  }
  best_script = cands[best_i];
  if (distinct_out) *distinct_out = distinct;
  if (cost_out) *cost_out = cost;
  return best_total;
}

// jpeg/src/progressive.rs:353-403 (encode_script, emit; non-differential)
static std::vector<uint8_t> emit_progressive(const CoefImage& ci, const std::vector<Scan>& script) {
  std::vector<uint8_t> body;
  for (auto& sc : script) {
    PStats st;
    run_scan(ci, sc, st);
    PTables t = build_tables(st);
    for (int cls = 0; cls < 2; cls++)
      for (int slot = 0; slot < 2; slot++)
        if (t.has[cls][slot]) write_dht(body, (uint8_t)((cls << 4) | slot), t.t[cls][slot]);
    std::vector<uint8_t> sos{(uint8_t)sc.comps.size()};
    for (int k : sc.comps) {
      uint8_t slot = (uint8_t)std::min(k, 1);
      uint8_t td = sc.ss == 0 ? slot : 0, ta = 0;
      sos.push_back(ci.comps[k].id);
      sos.push_back((uint8_t)((td << 4) | ta));
    }
    sos.push_back((uint8_t)sc.ss);
    sos.push_back((uint8_t)sc.se);
    sos.push_back((uint8_t)((sc.ah << 4) | sc.al));
    segment(body, 0xDA, sos);
    PEmit em{MsbWriter{}, &t};
    run_scan(ci, sc, em);
    em.w.finish();
    body.insert(body.end(), em.w.out.begin(), em.w.out.end());
  }
  std::vector<uint8_t> out = write_headers(ci, 0xC2);
  out.insert(out.end(), body.begin(), body.end());
  out.push_back(0xFF);
  out.push_back(0xD9);
  return out;
}

// jpeg/src/encode.rs:541-546 (write_best)
static std::vector<uint8_t> write_best(const CoefImage& ci) {
  std::vector<Scan> script;
  uint64_t prog_est = plan(ci, script);
  if (baseline_estimate(ci) <= prog_est) return write_jpeg(ci);
  return emit_progressive(ci, script);
}

// ------------------------------------------------------------------------------------------------ C ABI glue

// Flat coefficient layout shared with the product's C ABI: components back to back, each blocks_w*blocks_h blocks
// of 64 zigzag-ordered i16 coefficients in raster block order.
static CoefImage coef_from_flat(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                                const uint8_t* qtables /* [2][64] natural order */, const int16_t* coefs) {
  CoefImage ci;
  ci.width = w;
  ci.height = h;
  std::memset(ci.has_q, 0, sizeof ci.has_q);
  std::memcpy(ci.qtables[0], qtables, 64);
  ci.has_q[0] = true;
  if (ncomp > 1) {
    std::memcpy(ci.qtables[1], qtables + 64, 64);
    ci.has_q[1] = true;
  }
  size_t off = 0;
  for (int i = 0; i < ncomp; i++) {
    CoefComponent c;
    c.id = (uint8_t)(i + 1);
    c.h = hs[i];
    c.v = vs[i];
    c.tq = std::min(i, 1);
    c.blocks_w = bws[i];
    c.blocks_h = bhs[i];
    size_t n = (size_t)bws[i] * bhs[i] * 64;
    c.coefs.assign(coefs + off, coefs + off + n);
    off += n;
    ci.comps.push_back(std::move(c));
  }
  return ci;
}

// General flat form: per-component table slot `tq`, four table slots (has_q marks the present ones).
static CoefImage coef_from_flat_tq(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws,
                                   const int* bhs, const int* tq, const uint8_t* qtables4, const uint8_t* has_q,
                                   const int16_t* coefs) {
  CoefImage ci;
  ci.width = w;
  ci.height = h;
  for (int sl = 0; sl < 4; sl++) {
    ci.has_q[sl] = has_q[sl] != 0;
    std::memcpy(ci.qtables[sl], qtables4 + 64 * sl, 64);
  }
  size_t off = 0;
  for (int i = 0; i < ncomp; i++) {
    CoefComponent c;
    c.id = (uint8_t)(i + 1);
    c.h = hs[i];
    c.v = vs[i];
    c.tq = tq[i];
    c.blocks_w = bws[i];
    c.blocks_h = bhs[i];
    size_t n = (size_t)bws[i] * bhs[i] * 64;
    c.coefs.assign(coefs + off, coefs + off + n);
    off += n;
    ci.comps.push_back(std::move(c));
  }
  return ci;
}

static void coef_to_flat_tq(const CoefImage& ci, int16_t* out, int* tq, uint8_t* qtables4, uint8_t* has_q) {
  size_t off = 0;
  for (size_t i = 0; i < ci.comps.size(); i++) {
    std::memcpy(out + off, ci.comps[i].coefs.data(), ci.comps[i].coefs.size() * 2);
    off += ci.comps[i].coefs.size();
    if (tq) tq[i] = ci.comps[i].tq;
  }
  for (int sl = 0; sl < 4; sl++) {
    if (has_q) has_q[sl] = ci.has_q[sl] ? 1 : 0;
    if (qtables4) std::memcpy(qtables4 + 64 * sl, ci.qtables[sl], 64);
  }
}

static void coef_to_flat(const CoefImage& ci, int16_t* out, uint8_t* qtables) {
  size_t off = 0;
  for (auto& c : ci.comps) {
    std::memcpy(out + off, c.coefs.data(), c.coefs.size() * 2);
    off += c.coefs.size();
  }
  if (qtables) {
    std::memcpy(qtables, ci.qtables[0], 64);
    std::memcpy(qtables + 64, ci.has_q[1] ? ci.qtables[1] : ci.qtables[0], 64);
  }
}

// ------------------------------------------------------------------------------------------------ sequential decode

// jpeg/src/decode.rs:16-114 (BitReader): bytes with 0xFF00 stuffing; at a marker (0xFF not followed by 0) or the end
// of the data it feeds zero bits; restart() drops the buffer and skips to just past the next RSTn.
struct BitReader {
  const uint8_t* d;
  size_t len, pos;
  uint64_t acc = 0;
  uint32_t n = 0;
  bool marker = false;
  void fill() {
    while (n <= 56) {
      uint8_t byte = 0;
      if (!marker) {
        if (pos >= len) {
          marker = true;
        } else if (d[pos] == 0xFF) {
          if (pos + 1 < len && d[pos + 1] == 0) {
            pos += 2;
            byte = 0xFF;
          } else {
            marker = true;
          }
        } else {
          byte = d[pos++];
        }
      }
      acc = (acc << 8) | byte;
      n += 8;
    }
  }
  uint32_t peek(uint32_t k) {
    if (n < k) fill();
    return (uint32_t)((acc >> (n - k)) & ((1ull << k) - 1));
  }
  void skip(uint32_t k) { n -= k; }
  uint32_t bits(uint32_t k) {
    if (k == 0) return 0;
    uint32_t v = peek(k);
    skip(k);
    return v;
  }
  void restart() {
    acc = 0;
    n = 0;
    marker = false;
    while (pos + 1 < len) {
      if (d[pos] != 0xFF) {
        pos++;
        continue;
      }
      uint8_t m = d[pos + 1];
      if (m == 0) {
        pos += 2;
      } else if (m >= 0xD0 && m <= 0xD7) {
        pos += 2;
        return;
      } else {
        return;
      }
    }
  }
};

// jpeg/src/decode.rs:117-188 (HuffDec): 9-bit lookup, canonical search for longer codes.
struct HuffDec {
  uint16_t fast[512];
  int mincode[17], maxcode[18], valptr[17];
  std::vector<uint8_t> vals;
};

static int huffdec_build(const uint8_t bits[16], const uint8_t* vals, size_t nvals, HuffDec& h) {
  size_t total = 0;
  for (int i = 0; i < 16; i++) total += bits[i];
  if (total > 256 || total > nvals) return 1;
  std::memset(h.fast, 0, sizeof h.fast);
  for (int i = 0; i < 17; i++) h.mincode[i] = h.valptr[i] = 0;
  for (int i = 0; i < 18; i++) h.maxcode[i] = -1;
  h.vals.assign(vals, vals + total);
  int code = 0;
  size_t k = 0;
  for (int len = 1; len <= 16; len++) {
    int n = bits[len - 1];
    h.valptr[len] = (int)k;
    h.mincode[len] = code;
    if (n > 0) {
      if (code + n > (1 << len)) return 1;
      if (len <= 9)
        for (int i = 0; i < n; i++) {
          int c = code + i;
          uint8_t sym = h.vals[k + i];
          int shift = 9 - len;
          for (int f = 0; f < (1 << shift); f++) h.fast[(c << shift) | f] = (uint16_t)((len << 8) | sym);
        }
      code += n;
      k += n;
      h.maxcode[len] = code - 1;
    }
    code <<= 1;
  }
  return 0;
}

static int huff_decode(const HuffDec& h, BitReader& br, int* sym) {
  uint16_t e = h.fast[br.peek(9)];
  if (e != 0) {
    br.skip(e >> 8);
    *sym = e & 0xFF;
    return 0;
  }
  for (int len = 1; len <= 16; len++) {
    int code = (int)br.peek(len);
    if (h.maxcode[len] >= 0 && code <= h.maxcode[len] && code >= h.mincode[len]) {
      br.skip(len);
      *sym = h.vals[h.valptr[len] + code - h.mincode[len]];
      return 0;
    }
  }
  return 1;
}

static int32_t extend_bits(uint32_t v, uint32_t t) {
  if (t == 0) return 0;
  if (v < (1u << (t - 1))) return (int32_t)v - (int32_t)(1u << t) + 1;
  return (int32_t)v;
}

// jpeg/src/decode.rs:1480-1507 (decode_sequential)
static int decode_sequential(BitReader& br, const HuffDec& dc, const HuffDec& ac, int16_t* blk, int32_t* pred) {
  int t;
  if (huff_decode(dc, br, &t)) return 1;
  if (t > 16) return 1;
  int32_t diff = extend_bits(br.bits((uint32_t)t), (uint32_t)t);
  *pred = (int32_t)((uint32_t)*pred + (uint32_t)diff);
  blk[0] = (int16_t)*pred;
  int k = 1;
  while (k < 64) {
    int rs;
    if (huff_decode(ac, br, &rs)) return 1;
    int r = rs >> 4, sz = rs & 15;
    if (sz == 0) {
      if (r == 15) {
        k += 16;
        continue;
      }
      break;
    }
    k += r;
    if (k > 63) return 1;
    blk[k] = (int16_t)extend_bits(br.bits((uint32_t)sz), (uint32_t)sz);
    k++;
  }
  return 0;
}

// jpeg/src/decode.rs:1509-1517 (decode_dc_first)
static int decode_dc_first(BitReader& br, const HuffDec& dc, int16_t* blk, int32_t* pred, uint32_t al) {
  int t;
  if (huff_decode(dc, br, &t)) return 1;
  if (t > 16) return 1;
  *pred = (int32_t)((uint32_t)*pred + (uint32_t)extend_bits(br.bits((uint32_t)t), (uint32_t)t));
  blk[0] = (int16_t)(int32_t)((uint32_t)*pred << al);
  return 0;
}

struct ProgParams {
  int ss, se;
  uint32_t ah, al;
};

// jpeg/src/decode.rs:1519-1547 (decode_ac_first)
static int decode_ac_first(BitReader& br, const HuffDec& ac, int16_t* blk, uint32_t* eobrun, const ProgParams& p) {
  if (*eobrun > 0) {
    (*eobrun)--;
    return 0;
  }
  int k = p.ss;
  while (k <= p.se) {
    int rs;
    if (huff_decode(ac, br, &rs)) return 1;
    int r = rs >> 4, sz = rs & 15;
    if (sz == 0) {
      if (r < 15) {
        *eobrun = (1u << r) - 1;
        if (r > 0) *eobrun += br.bits((uint32_t)r);
        break;
      }
      k += 16;
      continue;
    }
    k += r;
    if (k > 63) return 1;
    blk[k] = (int16_t)(int32_t)((uint32_t)extend_bits(br.bits((uint32_t)sz), (uint32_t)sz) << p.al);
    k++;
  }
  return 0;
}

// jpeg/src/decode.rs:1549-1601 (decode_ac_refine)
static int decode_ac_refine(BitReader& br, const HuffDec& ac, int16_t* blk, uint32_t* eobrun, const ProgParams& p) {
  const int16_t p1 = (int16_t)(1 << p.al), m1 = (int16_t)(-1 * (1 << p.al));
  int k = p.ss;
  if (*eobrun == 0) {
    while (k <= p.se) {
      int rs;
      if (huff_decode(ac, br, &rs)) return 1;
      int r = rs >> 4, sz = rs & 15;
      int16_t value = 0;
      if (sz != 0) {
        value = br.bits(1) ? p1 : m1;
      } else if (r != 15) {
        *eobrun = 1u << r;
        if (r > 0) *eobrun += br.bits((uint32_t)r);
        break;
      }
      while (k <= p.se) {
        int16_t& c = blk[k];
        if (c != 0) {
          if (br.bits(1) && (c & p1) == 0) c = (int16_t)(c + (c >= 0 ? p1 : m1));
        } else {
          r--;
          if (r < 0) break;
        }
        k++;
      }
      if (value != 0) {
        if (k > 63) return 1;
        blk[k] = value;
      }
      k++;
    }
  }
  if (*eobrun > 0) {
    while (k <= p.se) {
      int16_t& c = blk[k];
      if (c != 0 && br.bits(1) && (c & p1) == 0) c = (int16_t)(c + (c >= 0 ? p1 : m1));
      k++;
    }
    (*eobrun)--;
  }
  return 0;
}

struct ParsedComp {
  uint8_t id = 0;
  int h = 1, v = 1, tq = 0, blocks_w = 0, blocks_h = 0, real_bw = 0, real_bh = 0;
  std::vector<int16_t> coefs;
  bool has_snap = false;
  uint16_t snap[64] = {0};
};

// jpeg::decode::parse(data)?.into_coefs() (jpeg/src/decode.rs:397-445, :540-570, :622-697, :906-1103, :1230-1309)
// for sequential and progressive Huffman frames (SOF0, SOF1, SOF2). Returns 0, 1 (invalid) or 2 (unsupported: other
// frame kinds, 12-bit, RGB-coded, 16-bit tables, four components).
static int parse_huffman(const uint8_t* d, size_t len, CoefImage& out) {
  if (len < 4 || d[0] != 0xFF || d[1] != 0xD8) return 1;
  size_t pos = 2;
  bool has_qt[4] = {false, false, false, false};
  uint16_t qt[4][64];
  bool has_dc[4] = {false, false, false, false}, has_ac[4] = {false, false, false, false};
  HuffDec dct[4], act[4];
  std::vector<ParsedComp> comps;
  int width = 0, height = 0, hmax = 1, vmax = 1, mcus_x = 0, mcus_y = 0;
  size_t ri = 0;
  int scans = 0;
  int adobe = -1;
  bool progressive = false;
  auto be16 = [&](size_t at, size_t* v) -> bool {
    if (at + 2 > len) return false;
    *v = ((size_t)d[at] << 8) | d[at + 1];
    return true;
  };
  for (;;) {
    // next_marker (:623-640)
    while (pos < len && d[pos] != 0xFF) pos++;
    while (pos < len && d[pos] == 0xFF) pos++;
    if (pos >= len) return 1;
    uint8_t m = d[pos++];
    if (m == 0 || (m >= 0xD0 && m <= 0xD7)) continue;
    if (m == 0xD9) break;
    if (m == 0x01) continue;
    size_t slen;
    if (!be16(pos, &slen)) return 1;
    if (slen < 2 || pos + slen > len) {
      if (scans > 0) break;
      return 1;
    }
    const uint8_t* b = d + pos + 2;
    size_t bl = slen - 2;
    pos += slen;
    if (m == 0xDB) {
      while (bl > 0) {
        int pq = b[0] >> 4, tq = b[0] & 15;
        if (tq > 3 || pq > 1) return 1;
        size_t need = 1 + 64 * (size_t)(pq + 1);
        if (bl < need) return 1;
        for (int k = 0; k < 64; k++)
          qt[tq][ZIGZAG[k]] = pq == 0 ? b[1 + k] : (uint16_t)((b[1 + 2 * k] << 8) | b[2 + 2 * k]);
        has_qt[tq] = true;
        b += need;
        bl -= need;
      }
    } else if (m == 0xC4) {
      while (bl > 0) {
        if (bl < 17) return 1;
        int tc = b[0] >> 4, th = b[0] & 15;
        if (tc > 1 || th > 3) return 1;
        size_t total = 0;
        for (int i = 0; i < 16; i++) total += b[1 + i];
        if (bl < 17 + total) return 1;
        HuffDec& hd = tc == 0 ? dct[th] : act[th];
        if (huffdec_build(b + 1, b + 17, total, hd)) return 1;
        (tc == 0 ? has_dc : has_ac)[th] = true;
        b += 17 + total;
        bl -= 17 + total;
      }
    } else if (m == 0xC0 || m == 0xC1 || m == 0xC2) {
      if (!comps.empty()) return 2;  // a second frame: hierarchical
      progressive = m == 0xC2;
      if (bl < 6) return 1;
      if (b[0] != 8) return b[0] == 12 ? 2 : 2;
      height = (b[1] << 8) | b[2];
      width = (b[3] << 8) | b[4];
      int nc = b[5];
      if (width == 0 || height == 0) return 1;
      if (nc == 4) return 2;
      if (nc != 1 && nc != 3) return 2;
      if (bl < 6 + 3 * (size_t)nc) return 1;
      for (int i = 0; i < nc; i++) {
        const uint8_t* c = b + 6 + 3 * i;
        int hs = c[1] >> 4, vs = c[1] & 15;
        if (hs < 1 || hs > 4 || vs < 1 || vs > 4 || c[2] > 3) return 1;
        ParsedComp pc;
        pc.id = c[0];
        pc.h = nc == 1 ? 1 : hs;
        pc.v = nc == 1 ? 1 : vs;
        pc.tq = c[2];
        comps.push_back(pc);
      }
      for (auto& c : comps) {
        hmax = std::max(hmax, c.h);
        vmax = std::max(vmax, c.v);
      }
      mcus_x = (width + 8 * hmax - 1) / (8 * hmax);
      mcus_y = (height + 8 * vmax - 1) / (8 * vmax);
      for (auto& c : comps) {
        c.blocks_w = mcus_x * c.h;
        c.blocks_h = mcus_y * c.v;
        int cw = (width * c.h + hmax - 1) / hmax, chh = (height * c.v + vmax - 1) / vmax;
        c.real_bw = (cw + 7) / 8;
        c.real_bh = (chh + 7) / 8;
        c.coefs.assign((size_t)c.blocks_w * c.blocks_h * 64, 0);
      }
    } else if ((m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) || m == 0xDE || m == 0xDF) {
      return 2;  // lossless, hierarchical or arithmetic frames
    } else if (m == 0xDD) {
      if (bl < 2) return 1;
      ri = ((size_t)b[0] << 8) | b[1];
    } else if (m == 0xEE && bl >= 12 && std::memcmp(b, "Adobe", 5) == 0) {
      adobe = b[11];
    } else if (m == 0xDA) {
      if (comps.empty()) return 1;
      if (bl < 1) return 1;
      int ns = b[0];
      if (ns == 0 || ns > (int)comps.size() || bl < 1 + 2 * (size_t)ns + 3) return 1;
      int idx[4], dci[4], aci[4];
      for (int i = 0; i < ns; i++) {
        uint8_t cid = b[1 + 2 * i], t = b[2 + 2 * i];
        int k = -1;
        for (size_t j = 0; j < comps.size(); j++)
          if (comps[j].id == cid) {
            k = (int)j;
            break;
          }
        if (k < 0) return 1;
        for (int j = 0; j < i; j++)
          if (idx[j] == k) return 1;
        idx[i] = k;
        dci[i] = (t >> 4) & 3;
        aci[i] = (t & 15) & 3;
      }
      // scan parameters (:1084-1096)
      const uint8_t* tp = b + 1 + 2 * ns;
      ProgParams pp{0, 63, 0, 0};
      if (progressive) {
        pp = ProgParams{tp[0], tp[1], (uint32_t)(tp[2] >> 4), (uint32_t)(tp[2] & 15)};
        if (pp.ss > pp.se || pp.se > 63 || pp.al > 13 || (pp.ss == 0 && pp.se != 0) || (pp.ss > 0 && ns != 1))
          return 1;
      }
      // tables the scan needs (:1240-1248)
      const bool need_dc = !progressive || (pp.ss == 0 && pp.ah == 0);
      const bool need_ac = !progressive || pp.ss > 0;
      for (int i = 0; i < ns; i++) {
        ParsedComp& c = comps[idx[i]];
        if (!c.has_snap && has_qt[c.tq]) {
          std::memcpy(c.snap, qt[c.tq], sizeof c.snap);
          c.has_snap = true;
        }
        if ((need_dc && !has_dc[dci[i]]) || (need_ac && !has_ac[aci[i]])) return 1;
      }
      // decode_scan (:1230-1309), Huffman
      BitReader br{d, len, pos};
      int32_t pred[4] = {0, 0, 0, 0};
      uint32_t eobrun = 0;
      bool inter = ns > 1;
      size_t mx_n = inter ? (size_t)mcus_x : (size_t)comps[idx[0]].real_bw;
      size_t my_n = inter ? (size_t)mcus_y : (size_t)comps[idx[0]].real_bh;
      size_t total = mx_n * my_n;
      for (size_t mcu = 0; mcu < total; mcu++) {
        if (ri > 0 && mcu > 0 && mcu % ri == 0) {
          br.restart();
          for (int i = 0; i < 4; i++) pred[i] = 0;
          eobrun = 0;
        }
        size_t mx = mcu % mx_n, my = mcu / mx_n;
        for (int si = 0; si < ns; si++) {
          ParsedComp& c = comps[idx[si]];
          int bh = inter ? c.h : 1, bv = inter ? c.v : 1;
          for (int by = 0; by < bv; by++)
            for (int bx = 0; bx < bh; bx++) {
              size_t col = mx * bh + bx, row = my * bv + by;
              int16_t* blk = &c.coefs[(row * c.blocks_w + col) * 64];
              int bad;
              if (!progressive)
                bad = decode_sequential(br, dct[dci[si]], act[aci[si]], blk, &pred[si]);
              else if (pp.ss == 0 && pp.ah == 0)
                bad = decode_dc_first(br, dct[dci[si]], blk, &pred[si], pp.al);
              else if (pp.ss == 0) {
                blk[0] = (int16_t)(blk[0] | (int16_t)(br.bits(1) << pp.al));
                bad = 0;
              } else if (pp.ah == 0)
                bad = decode_ac_first(br, act[aci[si]], blk, &eobrun, pp);
              else
                bad = decode_ac_refine(br, act[aci[si]], blk, &eobrun, pp);
              if (bad) return 1;
            }
        }
      }
      pos = br.pos;
      scans++;
    }
  }
  if (scans == 0 || comps.empty()) return 1;
  // into_coefs (:540-570)
  std::vector<uint8_t> ids;
  for (auto& c : comps) ids.push_back(c.id);
  bool coded_rgb = comps.size() == 3 && (adobe == 0 || (adobe < 0 && ids[0] == 'R' && ids[1] == 'G' && ids[2] == 'B'));
  if (coded_rgb) return 2;
  out.width = width;
  out.height = height;
  out.comps.clear();
  for (int sl = 0; sl < 4; sl++) out.has_q[sl] = false;
  for (auto& c : comps) {
    const uint16_t* t = c.has_snap ? c.snap : (has_qt[c.tq] ? qt[c.tq] : nullptr);
    if (!t) return 1;
    for (int i = 0; i < 64; i++)
      if (t[i] > 255 || t[i] == 0) return 2;
    for (int i = 0; i < 64; i++) out.qtables[c.tq][i] = (uint8_t)t[i];
    out.has_q[c.tq] = true;
  }
  for (auto& c : comps) out.comps.push_back(CoefComponent{c.id, c.h, c.v, c.tq, c.blocks_w, c.blocks_h, c.coefs});
  return 0;
}

// A baseline writer with options the reference's writer never uses, for decoder tests only (T.81 restart intervals
// and one scan per component): the tables and entropy coding of write_jpeg, then DRI/RSTn or per-component SOS.
static std::vector<uint8_t> write_jpeg_variant(const CoefImage& ci, int restart_interval, bool per_component) {
  int mx, my;
  ci.mcus(mx, my);
  const int nc = (int)ci.comps.size();
  const int hmax = ci.hv_max_h(), vmax = ci.hv_max_v();
  std::vector<std::vector<int>> scans;
  if (per_component) {
    for (int k = 0; k < nc; k++) scans.push_back({k});
  } else {
    std::vector<int> all;
    for (int k = 0; k < nc; k++) all.push_back(k);
    scans.push_back(all);
  }
  // Visit the blocks of one scan as a decoder would, with the DC predictions reset at every restart.
  auto visit = [&](const std::vector<int>& sc, auto&& on_restart, auto&& on_block) {
    int16_t pred[4] = {0, 0, 0, 0};
    const bool inter = sc.size() > 1;
    const int nx = inter ? mx : ((ci.width * ci.comps[sc[0]].h + hmax - 1) / hmax + 7) / 8;
    const int ny = inter ? my : ((ci.height * ci.comps[sc[0]].v + vmax - 1) / vmax + 7) / 8;
    int rst = 0;
    for (int m = 0; m < nx * ny; m++) {
      if (restart_interval > 0 && m > 0 && m % restart_interval == 0) {
        on_restart(rst++);
        for (int i = 0; i < 4; i++) pred[i] = 0;
      }
      const int x = m % nx, y = m / nx;
      for (int k : sc) {
        const CoefComponent& c = ci.comps[k];
        const int bh = inter ? c.h : 1, bv = inter ? c.v : 1;
        for (int by = 0; by < bv; by++)
          for (int bx = 0; bx < bh; bx++) {
            const size_t bi = (size_t)(y * bv + by) * c.blocks_w + x * bh + bx;
            on_block(&c.coefs[bi * 64], &pred[k], std::min(k, 1));
          }
      }
    }
  };
  // Tables from the statistics of exactly what is written (restart resets change the DC differences).
  Stats st;
  for (auto& sc : scans)
    visit(sc, [](int) {}, [&](const int16_t* blk, int16_t* pred, int tbl) { code_block(st, blk, pred, tbl); });
  HuffTable dct2[2] = {optimal_table(st.dc[0]), optimal_table(st.dc[1])};
  HuffTable act2[2] = {optimal_table(st.ac[0]), optimal_table(st.ac[1])};
  std::vector<uint8_t> out = write_headers(ci, 0xC0);
  const int ntables = nc == 1 ? 1 : 2;
  for (int t = 0; t < ntables; t++) {
    write_dht(out, (uint8_t)t, dct2[t]);
    write_dht(out, (uint8_t)(0x10 | t), act2[t]);
  }
  if (restart_interval > 0) segment(out, 0xDD, {(uint8_t)(restart_interval >> 8), (uint8_t)restart_interval});
  for (auto& sc : scans) {
    std::vector<uint8_t> sos{(uint8_t)sc.size()};
    for (int k : sc) {
      const uint8_t s = (uint8_t)std::min(k, 1);
      sos.push_back(ci.comps[k].id);
      sos.push_back((uint8_t)(s << 4 | s));
    }
    sos.push_back(0);
    sos.push_back(63);
    sos.push_back(0);
    segment(out, 0xDA, sos);
    Writer wr{MsbWriter{}, dct2, act2};
    visit(
        sc,
        [&](int rst) {
          wr.w.finish();
          wr.w.out.push_back(0xFF);
          wr.w.out.push_back((uint8_t)(0xD0 + (rst & 7)));
          wr.w.acc = 0;
          wr.w.n = 0;
        },
        [&](const int16_t* blk, int16_t* pred, int tbl) { code_block(wr, blk, pred, tbl); });
    wr.w.finish();
    out.insert(out.end(), wr.w.out.begin(), wr.w.out.end());
  }
  out.push_back(0xFF);
  out.push_back(0xD9);
  return out;
}

}  // namespace orc

extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int32_t orc_round_f32(float x) { return orc::round_f32(x); }

void orc_fdct(float* b) { orc::fdct(*(orc::Block*)b); }
void orc_idct(float* b) { orc::idct(*(orc::Block*)b); }
const float* orc_aan(void) { return orc::AAN; }

void orc_scale_table(int quality, uint8_t* out) { orc::luma_table(quality, out); }

void orc_fdct_divisors(const uint8_t* q, float* d) { orc::fdct_divisors(q, d); }

// Rdo::new + quantize_ac on one block: `a` are 64 values in units of quantization steps (zigzag order).
void orc_rdo_quantize_ac(const uint8_t* table, float kappa, const uint8_t* sizes, const float* a, int16_t* out) {
  orc::Rdo r(table, kappa, sizes);
  r.quantize_ac(a, out);
}

// Rdo::new parameters: q (zigzag), w, lambda, len.
void orc_rdo_params(const uint8_t* table, float kappa, const uint8_t* sizes, float* q, float* w, float* lambda,
                    float* len) {
  orc::Rdo r(table, kappa, sizes);
  std::memcpy(q, r.q, sizeof r.q);
  std::memcpy(w, r.w, sizeof r.w);
  *lambda = r.lambda;
  std::memcpy(len, r.len, sizeof r.len);
}

void orc_build_lengths(const uint32_t* freqs, int n, int max_len, uint8_t* out) {
  std::vector<uint32_t> f(freqs, freqs + n);
  std::vector<uint8_t> l = orc::build_lengths(f, max_len);
  std::memcpy(out, l.data(), n);
}

// optimal_table(freq).size for a 256-entry frequency table.
void orc_optimal_sizes(const uint32_t* freq, uint8_t* sizes) {
  orc::HuffTable t = orc::optimal_table(freq);
  std::memcpy(sizes, t.size, 256);
}

// Layout of the CoefImage build_coefs makes (jpeg/src/encode.rs:426-517).
int orc_coef_layout(int w, int h, int channels, int quality, int subsampling, int* ncomp, int* hs, int* vs, int* bws,
                    int* bhs) {
  if (w < 1 || h < 1 || (channels != 1 && channels != 3)) return 1;
  bool gray = channels == 1;
  int hmax = 1, vmax = 1;
  if (!gray) {
    if (subsampling == orc::SUB_420 || (subsampling == orc::SUB_AUTO && quality < 90)) {
      hmax = 2;
      vmax = 2;
    } else if (subsampling == orc::SUB_422) {
      hmax = 2;
      vmax = 1;
    }
  }
  int pw = (w + 8 * hmax - 1) / (8 * hmax) * 8 * hmax, ph = (h + 8 * vmax - 1) / (8 * vmax) * 8 * vmax;
  *ncomp = gray ? 1 : 3;
  hs[0] = hmax;
  vs[0] = vmax;
  bws[0] = pw / 8;
  bhs[0] = ph / 8;
  for (int i = 1; i < *ncomp; i++) {
    hs[i] = 1;
    vs[i] = 1;
    bws[i] = pw / hmax / 8;
    bhs[i] = ph / vmax / 8;
  }
  return 0;
}

int orc_build_coefs(const uint8_t* data, int w, int h, int channels, int quality, int subsampling, int trellis,
                    int16_t* coefs_out, uint8_t* qtables_out, const float* weights) {
  if (w < 1 || h < 1 || (channels != 1 && channels != 3)) return 1;
  orc::CoefImage ci = orc::build_coefs(data, w, h, channels, quality, subsampling, trellis != 0, weights);
  orc::coef_to_flat(ci, coefs_out, qtables_out);
  return 0;
}

// AC code lengths (rate model of the trellis) measured on a flat CoefImage.
int orc_ac_code_lengths(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                        const uint8_t* qtables, const int16_t* coefs, uint8_t* out /* [2][256] */) {
  orc::CoefImage ci = orc::coef_from_flat(w, h, ncomp, hs, vs, bws, bhs, qtables, coefs);
  uint8_t l[2][256];
  orc::ac_code_lengths(ci, l);
  std::memcpy(out, l, 512);
  return 0;
}

int orc_reconstruct(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                    const uint8_t* qtables, const int16_t* coefs, uint8_t* out, int* out_channels) {
  orc::CoefImage ci = orc::coef_from_flat(w, h, ncomp, hs, vs, bws, bhs, qtables, coefs);
  std::vector<uint8_t> img = orc::reconstruct(ci, out_channels);
  std::memcpy(out, img.data(), img.size());
  return 0;
}

// Reference-exact scorer (f32 planes, f64 arithmetic). per_scale (nullable) receives [6][3][6] pooled stats.
int orc_ssimulacra2(const uint8_t* ref, const uint8_t* dist, int w, int h, int channels, int depth, double* score,
                    double* per_scale, int* nscales) {
  return orc::ssimulacra2_t<float>(ref, dist, w, h, channels, depth, score, per_scale, nscales);
}

// FP64 oracle: the same algorithm with f64 planes throughout (no f32 rounding of the LUT or the pyramid).
int orc_ssimulacra2_fp64(const uint8_t* ref, const uint8_t* dist, int w, int h, int channels, int depth,
                         double* score, double* per_scale, int* nscales) {
  return orc::ssimulacra2_t<double>(ref, dist, w, h, channels, depth, score, per_scale, nscales);
}

// find_quality_with over build_coefs + reconstruct + ssimulacra2. trace_q/trace_s (nullable, >= 8 entries) receive
// every evaluated (quality, score) in order; *ntrace their count.
int orc_search(const uint8_t* data, int w, int h, int channels, double target, int max_quality, int subsampling,
               int trellis, int* found_q, double* found_score, int16_t* coefs_out, uint8_t* qtables_out, int* trace_q,
               double* trace_s, int* ntrace, int metric, const float* weights) {
  if (channels != 1 && channels != 3) return 1;
  if (metric == orc::METRIC_SSIMULACRA2 && (w < 8 || h < 8)) return 1;
  std::vector<std::pair<int, double>> tr;
  orc::Found f = orc::find_quality(data, w, h, channels, target, max_quality, subsampling, trellis != 0, &tr, metric,
                                   weights);
  *found_q = f.quality;
  *found_score = f.score;
  if (coefs_out) orc::coef_to_flat(f.coefs, coefs_out, qtables_out);
  if (ntrace) *ntrace = (int)tr.size();
  for (size_t i = 0; i < tr.size() && i < 16; i++) {
    if (trace_q) trace_q[i] = tr[i].first;
    if (trace_s) trace_s[i] = tr[i].second;
  }
  return 0;
}

// core/src/metrics.rs:13 (ssim), :67 (psnr), :111 (ms_ssim) of two 8-bit interleaved images with `ch` channels.
double orc_ssim(const uint8_t* a, const uint8_t* b, int w, int h, int ch) { return orc::ssim(a, b, w, h, ch); }
double orc_psnr(const uint8_t* a, const uint8_t* b, int w, int h, int ch) {
  return orc::psnr(a, b, (size_t)w * h * ch);
}
double orc_ms_ssim(const uint8_t* a, const uint8_t* b, int w, int h, int ch, double* per_scale) {
  return orc::ms_ssim(a, b, w, h, ch, per_scale);
}

// CoefImage::requantize (jpeg/src/encode.rs:111) of a general flat CoefImage (1 or 3 components).
int orc_requantize(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                   const int* tq, const uint8_t* qtables4, const uint8_t* has_q, const int16_t* coefs, int quality,
                   int trellis, int16_t* coefs_out, int* tq_out, uint8_t* qtables4_out, uint8_t* has_q_out) {
  if (ncomp != 1 && ncomp != 3) return 1;
  orc::CoefImage ci = orc::coef_from_flat_tq(w, h, ncomp, hs, vs, bws, bhs, tq, qtables4, has_q, coefs);
  orc::requantize(ci, quality, trellis != 0);
  orc::coef_to_flat_tq(ci, coefs_out, tq_out, qtables4_out, has_q_out);
  return 0;
}

// reconstruct of a general flat CoefImage.
int orc_reconstruct_tq(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                       const int* tq, const uint8_t* qtables4, const uint8_t* has_q, const int16_t* coefs,
                       uint8_t* out, int* out_channels) {
  orc::CoefImage ci = orc::coef_from_flat_tq(w, h, ncomp, hs, vs, bws, bhs, tq, qtables4, has_q, coefs);
  std::vector<uint8_t> img = orc::reconstruct(ci, out_channels);
  std::memcpy(out, img.data(), img.size());
  return 0;
}

// The JPEG->JPEG search (cli/src/pipeline.rs:369-386) over a general flat CoefImage.
int orc_search_requantize(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                          const int* tq, const uint8_t* qtables4, const uint8_t* has_q, const int16_t* coefs,
                          double target, int max_quality, int trellis, int* found_q, double* found_score,
                          int16_t* coefs_out, int* tq_out, uint8_t* qtables4_out, uint8_t* has_q_out, int* trace_q,
                          double* trace_s, int* ntrace, int metric) {
  if (ncomp != 1 && ncomp != 3) return 1;
  orc::CoefImage ci = orc::coef_from_flat_tq(w, h, ncomp, hs, vs, bws, bhs, tq, qtables4, has_q, coefs);
  std::vector<std::pair<int, double>> tr;
  orc::Found f = orc::find_quality_requantize(ci, target, max_quality, trellis != 0, &tr, metric);
  *found_q = f.quality;
  *found_score = f.score;
  orc::coef_to_flat_tq(f.coefs, coefs_out, tq_out, qtables4_out, has_q_out);
  if (ntrace) *ntrace = (int)tr.size();
  for (size_t i = 0; i < tr.size() && i < 16; i++) {
    if (trace_q) trace_q[i] = tr[i].first;
    if (trace_s) trace_s[i] = tr[i].second;
  }
  return 0;
}

// write_best of a general flat CoefImage (per-component table slots).
long orc_write_best_tq(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                       const int* tq, const uint8_t* qtables4, const uint8_t* has_q, const int16_t* coefs,
                       uint8_t* out, long cap, int* progressive) {
  orc::CoefImage ci = orc::coef_from_flat_tq(w, h, ncomp, hs, vs, bws, bhs, tq, qtables4, has_q, coefs);
  std::vector<orc::Scan> script;
  uint64_t prog_est = orc::plan(ci, script);
  uint64_t base_est = orc::baseline_estimate(ci);
  std::vector<uint8_t> bytes = base_est <= prog_est ? orc::write_jpeg(ci) : orc::emit_progressive(ci, script);
  if (progressive) *progressive = base_est <= prog_est ? 0 : 1;
  if (out) std::memcpy(out, bytes.data(), std::min<size_t>(bytes.size(), (size_t)cap));
  return (long)bytes.size();
}

// write_best's plan (jpeg/src/encode.rs:543-565, jpeg/src/progressive.rs:335-351) of a flat CoefImage: estimated
// sizes, the chosen script and every distinct candidate scan with its cost. Scans are 8 ints each: ncomps,
// comps[4], ss, se, ah*16+al.
int orc_plan(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
             const int16_t* coefs, uint64_t* prog_est, uint64_t* base_est, int* nscans, int* scans, int* ndistinct,
             int* distinct, uint64_t* costs) {
  uint8_t ones[128];
  std::memset(ones, 1, sizeof ones);
  orc::CoefImage ci = orc::coef_from_flat(w, h, ncomp, hs, vs, bws, bhs, ones, coefs);
  std::vector<orc::Scan> best, dist;
  std::vector<uint64_t> cost;
  *prog_est = orc::plan(ci, best, &dist, &cost);
  *base_est = orc::baseline_estimate(ci);
  auto put = [](const orc::Scan& sc, int* o) {
    o[0] = (int)sc.comps.size();
    for (int i = 0; i < 4; i++) o[1 + i] = i < (int)sc.comps.size() ? sc.comps[i] : 0;
    o[5] = sc.ss;
    o[6] = sc.se;
    o[7] = (int)(sc.ah * 16 + sc.al);
  };
  *nscans = (int)best.size();
  for (size_t i = 0; i < best.size(); i++) put(best[i], scans + 8 * i);
  *ndistinct = (int)dist.size();
  for (size_t i = 0; i < dist.size(); i++) {
    put(dist[i], distinct + 8 * i);
    costs[i] = cost[i];
  }
  return 0;
}

// write_best (jpeg/src/encode.rs:543-546) of a flat CoefImage. Returns the byte count; writes at most `cap` bytes.
long orc_write_best(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                    const uint8_t* qtables, const int16_t* coefs, uint8_t* out, long cap, int* progressive) {
  orc::CoefImage ci = orc::coef_from_flat(w, h, ncomp, hs, vs, bws, bhs, qtables, coefs);
  std::vector<orc::Scan> script;
  uint64_t prog_est = orc::plan(ci, script);
  uint64_t base_est = orc::baseline_estimate(ci);
  std::vector<uint8_t> bytes = base_est <= prog_est ? orc::write_jpeg(ci) : orc::emit_progressive(ci, script);
  if (progressive) *progressive = base_est <= prog_est ? 0 : 1;
  if (out) std::memcpy(out, bytes.data(), std::min<size_t>(bytes.size(), (size_t)cap));
  return (long)bytes.size();
}

// progressive::emit (jpeg/src/progressive.rs:397-403) of candidate script `index` of scripts(ncomp)
// (jpeg/src/progressive.rs:242-295) for a flat CoefImage; returns the byte count (out may be NULL), -1 for a bad
// index. Test input for the progressive decoders.
long orc_emit_script(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                     const uint8_t* qtables, const int16_t* coefs, int index, uint8_t* out, long cap) {
  orc::CoefImage ci = orc::coef_from_flat(w, h, ncomp, hs, vs, bws, bhs, qtables, coefs);
  std::vector<std::vector<orc::Scan>> cands = orc::scripts(ncomp);
  if (index < 0 || index >= (int)cands.size()) return -1;
  std::vector<uint8_t> bytes = orc::emit_progressive(ci, cands[(size_t)index]);
  if (out) std::memcpy(out, bytes.data(), std::min<size_t>(bytes.size(), (size_t)cap));
  return (long)bytes.size();
}

int orc_script_count(int ncomp) { return (int)orc::scripts(ncomp).size(); }

// parse(data)?.into_coefs() for sequential and progressive Huffman JPEGs. Query with coefs_out == NULL: fills w, h,
// ncomp, layout, ids. Returns 0, 1 (invalid), 2 (unsupported).
int orc_decode_sequential(const uint8_t* data, long len, int* w, int* h, int* ncomp, int* hs, int* vs, int* bws,
                          int* bhs, uint8_t* ids, int16_t* coefs_out, int* tq, uint8_t* qtables4, uint8_t* has_q) {
  orc::CoefImage ci;
  int rc = orc::parse_huffman(data, (size_t)len, ci);
  if (rc) return rc;
  *w = ci.width;
  *h = ci.height;
  *ncomp = (int)ci.comps.size();
  for (size_t i = 0; i < ci.comps.size(); i++) {
    hs[i] = ci.comps[i].h;
    vs[i] = ci.comps[i].v;
    bws[i] = ci.comps[i].blocks_w;
    bhs[i] = ci.comps[i].blocks_h;
    ids[i] = ci.comps[i].id;
  }
  if (coefs_out) orc::coef_to_flat_tq(ci, coefs_out, tq, qtables4, has_q);
  return 0;
}

// Baseline JPEG bytes of a general flat CoefImage, with an optional restart interval and one scan per component
// (decoder tests). Returns the size; writes at most cap bytes.
long orc_write_jpeg_variant(int w, int h, int ncomp, const int* hs, const int* vs, const int* bws, const int* bhs,
                            const int* tq, const uint8_t* qtables4, const uint8_t* has_q, const int16_t* coefs,
                            int restart_interval, int per_component, uint8_t* out, long cap) {
  orc::CoefImage ci = orc::coef_from_flat_tq(w, h, ncomp, hs, vs, bws, bhs, tq, qtables4, has_q, coefs);
  std::vector<uint8_t> bytes = orc::write_jpeg_variant(ci, restart_interval, per_component != 0);
  if (out) std::memcpy(out, bytes.data(), std::min<size_t>(bytes.size(), (size_t)cap));
  return (long)bytes.size();
}

// The FP64 score of a continuous-valued distorted image (RGB, w x h x 3 doubles in [0, 255]) against ref, and its
// gradient (grad may be NULL).
double orc_score64(const double* ref, const double* dist, int w, int h) {
  return orc::score64(ref, dist, w, h, nullptr, nullptr);
}
double orc_grad64(const double* ref, const double* dist, int w, int h, double* grad) {
  return orc::grad64(ref, dist, w, h, grad);
}

}  // extern "C"

