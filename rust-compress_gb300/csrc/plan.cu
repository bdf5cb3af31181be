// write_best's size estimates on the GPU (jpeg/src/encode.rs:543-565 with jpeg/src/progressive.rs:191-351):
// symbol statistics of every distinct scan of the 144 (3 components) or 24 (gray) candidate progressive scripts and
// of the baseline scan, their optimal Huffman code lengths, the scan costs, and the script with the smallest total.
// Emission stays with the caller: it writes baseline or the chosen script, as write_best would.
//
// Work layout. Every scan visits its blocks in the reference's order ("positions"): MCU order over all components
// for interleaved scans (the DC scans of colour images and the baseline scan), raster order over the blocks that
// overlap the image for single-component scans. Positions are cut into chunks of 1024; one CTA per (scan, chunk).
//  k_plan_blocks    everything a block contributes on its own: DC differences (the predecessor is re-read), AC
//                   symbols, raw bits; for AC scans a 16-bit flag per position (emits a symbol / ends inside an
//                   end-of-band run / correction bits left pending) and per-chunk aggregates.
//  k_plan_chunks    per AC scan, exclusive scans of the chunk aggregates (last symbol position, pending-bit sum).
//  k_plan_prefix    per AC position, the previous symbol position and the prefix sum of pending bits.
//  k_plan_eobruns   the end-of-band runs: each symbol position (and the end of the scan) closes the run since the
//                   previous one; a run is cut at 0x7FFF blocks and, in refinement scans, where the pending
//                   correction bits pass 937 (progressive.rs:136, :184). Each cut emits one EOBn symbol.
//  k_plan_tables    Huffman code lengths per (scan, class, slot) and the coded bits.
//  k_plan_choose    scan costs (progressive.rs:310-327, encode.rs:550-565) and the first cheapest script.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "huffman.cuh"
#include "rcg_internal.cuh"

namespace rcg {

namespace {

enum : int { kDcFirst = 0, kDcRefine = 1, kAcFirst = 2, kAcRefine = 3, kBaseline = 4 };

constexpr int kChunk = 1024;
constexpr int kThreads = 256;
constexpr int kMaxScans = 49;  // 48 distinct progressive scans of a 3-component image, then the baseline scan
constexpr int kMaxScripts = 144;
constexpr int kMaxScriptLen = 16;
constexpr int kMaxEobRun = 0x7FFF;         // jpeg/src/progressive.rs:136
constexpr unsigned kMaxPending = 1000 - 63;  // MAX_CORR_BITS - 63, jpeg/src/progressive.rs:65, :184

struct ScanDesc {
  int kind;
  int comp;         // single-component scans
  int interleaved;  // MCU order over all components
  int ss, se, al;
  int real_w;       // single-component visiting grid width (blocks)
  long long npos;
  long long chunk0;  // first chunk of this scan
  long long aux0;    // AC scans: offset of the per-position flag / predecessor arrays
  long long p0;      // refinement scans: offset of the pending-bit prefix array (npos + 1 entries)
};

struct PlanDesc {
  int nscans;  // distinct progressive scans, then the baseline scan
  int nscripts;
  int ncomp;
  int mcus_x, mcus_y, mcu_blocks;
  int mcu_off[3];
  CompDesc comp[3];
  long long nchunks;
  ScanDesc scan[kMaxScans];
  int script_len[kMaxScripts];
  unsigned char script[kMaxScripts][kMaxScriptLen];
};

struct ScanStats {
  unsigned freq[2][2][256];  // [class: 0 DC, 1 AC][table slot][symbol]
  unsigned long long raw_bits;
};

struct PlanOut {
  unsigned long long cost[kMaxScans];
  unsigned long long prog;
  int best;
};

__device__ __forceinline__ int nbits(unsigned v) { return v == 0 ? 0 : 32 - __clz(v); }

__device__ __forceinline__ int find_scan(const PlanDesc* pd, long long chunk) {
  int s = 0;
  for (int i = 1; i < pd->nscans; i++)
    if (pd->scan[i].chunk0 <= chunk) s = i;
  return s;
}

// Block index of a position and of the previous block of the same component in visiting order (-1: none).
__device__ __forceinline__ long long visit_block(const PlanDesc* pd, const ScanDesc& sc, long long pos, int* comp,
                                                 long long* pred) {
  if (sc.interleaved) {
    const long long m = pos / pd->mcu_blocks;
    const int u = (int)(pos - m * pd->mcu_blocks);
    int k = 0;
    while (k + 1 < pd->ncomp && u >= pd->mcu_off[k + 1]) k++;
    const CompDesc& c = pd->comp[k];
    const int local = u - pd->mcu_off[k];
    auto at = [&](long long mm, int l) {
      const int my = (int)(mm / pd->mcus_x), mx = (int)(mm % pd->mcus_x);
      return c.blk0 + (long long)(my * c.v + l / c.h) * c.bw + mx * c.h + l % c.h;
    };
    *comp = k;
    *pred = local > 0 ? at(m, local - 1) : (m > 0 ? at(m - 1, c.h * c.v - 1) : -1);
    return at(m, local);
  }
  const CompDesc& c = pd->comp[sc.comp];
  auto at = [&](long long p) { return c.blk0 + (p / sc.real_w) * c.bw + p % sc.real_w; };
  *comp = sc.comp;
  *pred = pos > 0 ? at(pos - 1) : -1;
  return at(pos);
}

__device__ __forceinline__ void load_block(const int16_t* blk, int (&v)[64]) {
  const int4* q = reinterpret_cast<const int4*>(blk);
#pragma unroll
  for (int g = 0; g < 8; g++) {
    int4 pk = __ldg(q + g);
    int w4[4] = {pk.x, pk.y, pk.z, pk.w};
#pragma unroll
    for (int j = 0; j < 8; j++) v[g * 8 + j] = (int)(short)((w4[j >> 1] >> (16 * (j & 1))) & 0xFFFF);
  }
}

// Flag bits of an AC position.
constexpr uint16_t kFlagSym = 0x8000;  // the block emits a Huffman symbol (closes the pending run first)
constexpr uint16_t kFlagEob = 0x4000;  // the block ends inside an end-of-band run (eobrun += 1)
constexpr uint16_t kFlagPend = 0x007F;  // correction bits the block adds to the pending list

__global__ void __launch_bounds__(kThreads) k_plan_blocks(const PlanDesc* __restrict__ pd,
                                                          const int16_t* __restrict__ coefs, ScanStats* stats,
                                                          uint16_t* __restrict__ flags, int* __restrict__ chunk_last,
                                                          unsigned long long* __restrict__ chunk_pend) {
  __shared__ unsigned hist[2][2][256];
  __shared__ int s_scan, last_sym;
  __shared__ unsigned long long pend_sum;
  const int t = threadIdx.x;
  const long long chunk = blockIdx.x;
  if (t == 0) {
    s_scan = find_scan(pd, chunk);
    last_sym = -1;
    pend_sum = 0;
  }
  for (int i = t; i < 1024; i += kThreads) (&hist[0][0][0])[i] = 0;
  __syncthreads();
  const int s = s_scan;
  const ScanDesc sc = pd->scan[s];
  const long long base = (chunk - sc.chunk0) * kChunk;
  unsigned raw = 0;
  for (int j = 0; j < kChunk / kThreads; j++) {
    const long long pos = base + j * kThreads + t;
    if (pos >= sc.npos) break;
    int k;
    long long pred;
    const long long b = visit_block(pd, sc, pos, &k, &pred);
    const int16_t* blk = coefs + b * 64;
    const int slot = k < 1 ? k : 1;
    if (sc.kind == kDcFirst) {
      // dc_first (progressive.rs:85-98)
      const int v = (int)(blk[0] >> sc.al);
      const int pv = pred >= 0 ? (int)(coefs[pred * 64] >> sc.al) : 0;
      const int nb = nbits((unsigned)abs(v - pv));
      atomicAdd(&hist[0][slot][nb], 1u);
      raw += nb;
    } else if (sc.kind == kDcRefine) {
      raw += 1;  // dc_refine (progressive.rs:100-102)
    } else if (sc.kind == kBaseline) {
      // code_block (encode.rs:351-374)
      int v[64];
      load_block(blk, v);
      const int pv = pred >= 0 ? (int)coefs[pred * 64] : 0;
      const int cat = nbits((unsigned)abs(v[0] - pv));
      atomicAdd(&hist[0][slot][cat], 1u);
      raw += cat;
      int run = 0;
#pragma unroll
      for (int q = 1; q < 64; q++) {
        if (v[q] == 0) {
          run++;
        } else {
          if (run >= 16) atomicAdd(&hist[1][slot][0xF0], (unsigned)(run >> 4));
          const int c = nbits((unsigned)abs(v[q]));
          atomicAdd(&hist[1][slot][((run & 15) << 4) | c], 1u);
          raw += c;
          run = 0;
        }
      }
      if (run > 0) atomicAdd(&hist[1][slot][0], 1u);
    } else if (sc.kind == kAcFirst) {
      // ac_first (progressive.rs:104-139) without the end-of-band runs
      int v[64];
      load_block(blk, v);
      int r = 0;
      bool sym = false;
#pragma unroll
      for (int q = 1; q < 64; q++) {
        if (q >= sc.ss && q <= sc.se) {
          const int mag = abs(v[q]) >> sc.al;
          if (mag == 0) {
            r++;
          } else {
            sym = true;
            if (r > 15) atomicAdd(&hist[1][0][0xF0], (unsigned)(r >> 4));
            const int nb = nbits((unsigned)mag);
            atomicAdd(&hist[1][0][((r & 15) << 4) + nb], 1u);
            raw += nb;
            r = 0;
          }
        }
      }
      flags[sc.aux0 + pos] = (uint16_t)((sym ? kFlagSym : 0) | (r > 0 ? kFlagEob : 0));
      if (sym) atomicMax(&last_sym, (int)pos);
    } else {
      // ac_refine (progressive.rs:141-189) without the end-of-band runs. Every correction bit is emitted exactly
      // once (inline, or with the run that holds it), so raw bits count them where they arise.
      int v[64];
      load_block(blk, v);
      int eob = 0;
#pragma unroll
      for (int q = 1; q < 64; q++)
        if (q >= sc.ss && q <= sc.se && (abs(v[q]) >> sc.al) == 1) eob = q;
      int r = 0, br = 0;
#pragma unroll
      for (int q = 1; q < 64; q++) {
        if (q >= sc.ss && q <= sc.se) {
          const int tq = abs(v[q]) >> sc.al;
          if (tq == 0) {
            r++;
          } else {
            if (r > 15 && q <= eob) {
              atomicAdd(&hist[1][0][0xF0], (unsigned)(r >> 4));
              r &= 15;
              br = 0;
            }
            if (tq > 1) {
              br++;
              raw += 1;
            } else {
              atomicAdd(&hist[1][0][(r << 4) + 1], 1u);
              raw += 1;
              br = 0;
              r = 0;
            }
          }
        }
      }
      const bool sym = eob > 0;
      const bool ends = r > 0 || br > 0;
      flags[sc.aux0 + pos] = (uint16_t)((sym ? kFlagSym : 0) | (ends ? kFlagEob : 0) | (ends ? br : 0));
      if (sym) atomicMax(&last_sym, (int)pos);
      if (ends && br) atomicAdd(&pend_sum, (unsigned long long)br);
    }
  }
  raw = __reduce_add_sync(0xffffffffu, raw);
  if ((t & 31) == 0 && raw) atomicAdd(&stats[s].raw_bits, (unsigned long long)raw);
  __syncthreads();
  for (int i = t; i < 1024; i += kThreads) {
    unsigned x = (&hist[0][0][0])[i];
    if (x) atomicAdd(&(&stats[s].freq[0][0][0])[i], x);
  }
  if (t == 0) {
    chunk_last[chunk] = last_sym;
    chunk_pend[chunk] = pend_sum;
  }
}

// Block-wide exclusive scans (max of int, sum of u64) over one value per thread; returns the totals too.
template <int N>
__device__ __forceinline__ void block_scan(int m, unsigned long long p, int* m_ex, unsigned long long* p_ex,
                                           int* m_tot, unsigned long long* p_tot) {
  __shared__ int wm[N / 32];
  __shared__ unsigned long long wp[N / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int mi = m;
  unsigned long long pi = p;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int mo = __shfl_up_sync(0xffffffffu, mi, o);
    unsigned long long po = __shfl_up_sync(0xffffffffu, pi, o);
    if (lane >= o) {
      mi = max(mi, mo);
      pi += po;
    }
  }
  if (lane == 31) {
    wm[w] = mi;
    wp[w] = pi;
  }
  __syncthreads();
  if (w == 0) {
    int a = lane < N / 32 ? wm[lane] : -1;
    unsigned long long b = lane < N / 32 ? wp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int ao = __shfl_up_sync(0xffffffffu, a, o);
      unsigned long long bo = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a = max(a, ao);
        b += bo;
      }
    }
    if (lane < N / 32) {
      wm[lane] = a;
      wp[lane] = b;
    }
  }
  __syncthreads();
  const int before_m = w > 0 ? wm[w - 1] : -1;
  const unsigned long long before_p = w > 0 ? wp[w - 1] : 0;
  int mex = __shfl_up_sync(0xffffffffu, mi, 1);
  unsigned long long pex = __shfl_up_sync(0xffffffffu, pi, 1);
  if (lane == 0) {
    mex = -1;
    pex = 0;
  }
  *m_ex = max(before_m, mex);
  *p_ex = before_p + pex;
  *m_tot = wm[N / 32 - 1];
  *p_tot = wp[N / 32 - 1];
  __syncthreads();
}

// One CTA per AC scan: exclusive scans of the chunk aggregates.
__global__ void __launch_bounds__(1024) k_plan_chunks(const PlanDesc* __restrict__ pd, const int* chunk_last,
                                                      const unsigned long long* chunk_pend, int* chunk_prev,
                                                      unsigned long long* chunk_pbase) {
  const ScanDesc sc = pd->scan[blockIdx.x];
  if (sc.kind != kAcFirst && sc.kind != kAcRefine) return;
  const long long nch = (sc.npos + kChunk - 1) / kChunk;
  int carry_m = -1;
  unsigned long long carry_p = 0;
  for (long long off = 0; off < nch; off += 1024) {
    const long long i = off + threadIdx.x;
    const int m = i < nch ? chunk_last[sc.chunk0 + i] : -1;
    const unsigned long long p = i < nch ? chunk_pend[sc.chunk0 + i] : 0;
    int mex, mtot;
    unsigned long long pex, ptot;
    block_scan<1024>(m, p, &mex, &pex, &mtot, &ptot);
    if (i < nch) {
      chunk_prev[sc.chunk0 + i] = max(carry_m, mex);
      chunk_pbase[sc.chunk0 + i] = carry_p + pex;
    }
    carry_m = max(carry_m, mtot);
    carry_p += ptot;
  }
}

// Per AC position: previous symbol position (-1: none) and, for refinement scans, the prefix sum of pending bits
// (P[pos] = bits of positions < pos; P[npos] = total). Each thread takes 4 consecutive positions.
__global__ void __launch_bounds__(kThreads) k_plan_prefix(const PlanDesc* __restrict__ pd,
                                                          const uint16_t* __restrict__ flags,
                                                          const int* __restrict__ chunk_prev,
                                                          const unsigned long long* __restrict__ chunk_pbase,
                                                          int* __restrict__ prev, unsigned long long* __restrict__ P,
                                                          int* __restrict__ prev_end) {
  __shared__ int s_scan;
  const long long chunk = blockIdx.x;
  if (threadIdx.x == 0) s_scan = find_scan(pd, chunk);
  __syncthreads();
  const int s = s_scan;
  const ScanDesc sc = pd->scan[s];
  if (sc.kind != kAcFirst && sc.kind != kAcRefine) return;
  const long long pos0 = (chunk - sc.chunk0) * kChunk + 4 * threadIdx.x;
  uint16_t f[4];
  int m = -1;
  unsigned long long p = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const long long pos = pos0 + j;
    f[j] = pos < sc.npos ? flags[sc.aux0 + pos] : 0;
    if (f[j] & kFlagSym) m = (int)pos;
    p += f[j] & kFlagPend;
  }
  int mex, mtot;
  unsigned long long pex, ptot;
  block_scan<kThreads>(m, p, &mex, &pex, &mtot, &ptot);
  int run_m = max(chunk_prev[chunk], mex);
  unsigned long long run_p = chunk_pbase[chunk] + pex;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const long long pos = pos0 + j;
    if (pos >= sc.npos) break;
    prev[sc.aux0 + pos] = run_m;
    if (sc.kind == kAcRefine) P[sc.p0 + pos] = run_p;
    if (f[j] & kFlagSym) run_m = (int)pos;
    run_p += f[j] & kFlagPend;
    if (pos == sc.npos - 1) {
      prev_end[s] = run_m;
      if (sc.kind == kAcRefine) P[sc.p0 + sc.npos] = run_p;
    }
  }
}

// The end-of-band runs closed at symbol positions (and at the end of each AC scan).
__global__ void __launch_bounds__(kThreads) k_plan_eobruns(const PlanDesc* __restrict__ pd,
                                                           const uint16_t* __restrict__ flags,
                                                           const int* __restrict__ prev,
                                                           const unsigned long long* __restrict__ P,
                                                           const int* __restrict__ prev_end, ScanStats* stats) {
  __shared__ int s_scan;
  __shared__ unsigned cnt[16];
  __shared__ unsigned long long raw_sh;
  const long long chunk = blockIdx.x;
  if (threadIdx.x == 0) {
    s_scan = find_scan(pd, chunk);
    raw_sh = 0;
  }
  if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int s = s_scan;
  const ScanDesc sc = pd->scan[s];
  if (sc.kind != kAcFirst && sc.kind != kAcRefine) return;
  const long long base = (chunk - sc.chunk0) * kChunk;
  unsigned long long raw = 0;
  auto flush = [&](long long n) {
    const int nb = nbits((unsigned)n) - 1;
    atomicAdd(&cnt[nb], 1u);
    raw += nb;
  };
  // The run closed at position i (a symbol position, or npos): elements [a, i-1], where the previous symbol
  // position counts when it ended inside a run itself.
  auto close_run = [&](long long i, int prv) {
    long long a = 0;
    if (prv >= 0) a = (flags[sc.aux0 + prv] & kFlagEob) ? prv : prv + 1;
    if (a >= i) return;
    if (sc.kind == kAcFirst) {
      const long long n = i - a;
      const long long full = n / kMaxEobRun, rem = n % kMaxEobRun;
      if (full) {
        atomicAdd(&cnt[14], (unsigned)full);
        raw += 14ull * full;
      }
      if (rem) flush(rem);
      return;
    }
    const unsigned long long* Ps = P + sc.p0;
    long long st = a;
    while (st <= i - 1) {
      // first element t >= st after which the pending bits pass the limit: smallest t1 in [st+1, i] with
      // P[t1] > P[st] + limit, t = t1 - 1
      const unsigned long long lim = Ps[st] + kMaxPending;
      long long lo = st + 1, hi = i + 1;  // search in [lo, hi)
      while (lo < hi) {
        long long mid = lo + (hi - lo) / 2;
        if (Ps[mid] > lim)
          hi = mid;
        else
          lo = mid + 1;
      }
      long long t_cut = lo <= i ? lo - 1 : (long long)1 << 62;
      t_cut = min(t_cut, st + kMaxEobRun - 1);
      if (t_cut <= i - 1) {
        flush(t_cut - st + 1);
        st = t_cut + 1;
      } else {
        flush(i - st);
        break;
      }
    }
  };
  for (int j = 0; j < kChunk / kThreads; j++) {
    const long long pos = base + j * kThreads + threadIdx.x;
    if (pos >= sc.npos) break;
    if (flags[sc.aux0 + pos] & kFlagSym) close_run(pos, prev[sc.aux0 + pos]);
  }
  if (threadIdx.x == 0 && base + kChunk >= sc.npos) close_run(sc.npos, prev_end[s]);
  if (raw) atomicAdd(&raw_sh, raw);
  __syncthreads();
  if (threadIdx.x < 16 && cnt[threadIdx.x]) atomicAdd(&stats[s].freq[1][0][threadIdx.x << 4], cnt[threadIdx.x]);
  if (threadIdx.x == 0 && raw_sh) atomicAdd(&stats[s].raw_bits, raw_sh);
}

// Code lengths and coded bits per (scan, class, slot). Progressive scans build a table only for a non-empty
// histogram (progressive.rs:297-307); the baseline estimate builds one per class for each table slot in use
// (encode.rs:552-560), empty or not.
__global__ void __launch_bounds__(288) k_plan_tables(const PlanDesc* __restrict__ pd, const ScanStats* stats,
                                                     unsigned long long* table_bits, int* dht_bytes) {
  __shared__ unsigned freq[kHuffSyms];
  __shared__ unsigned char lens[kHuffSyms];
  __shared__ HuffScratch scratch;
  __shared__ int any, nvals;
  __shared__ unsigned long long bits;
  const int s = blockIdx.x, cs = blockIdx.y, cls = cs >> 1, slot = cs & 1;
  const int t = threadIdx.x;
  const bool baseline = pd->scan[s].kind == kBaseline;
  if (t == 0) {
    any = 0;
    nvals = 0;
    bits = 0;
  }
  __syncthreads();
  if (t < kHuffSyms) {
    freq[t] = t < 256 ? stats[s].freq[cls][slot][t] : 1u;
    if (t < 256 && freq[t]) atomicOr(&any, 1);
  }
  __syncthreads();
  const bool build = baseline ? slot < (pd->ncomp == 1 ? 1 : 2) : any != 0;
  if (!build) {
    if (t == 0) {
      table_bits[s * 4 + cs] = 0;
      dht_bytes[s * 4 + cs] = 0;
    }
    return;
  }
  huff_lengths(freq, lens, scratch);
  if (t < 256) {
    if (lens[t]) {
      atomicAdd(&nvals, 1);
      if (freq[t]) atomicAdd(&bits, (unsigned long long)freq[t] * lens[t]);
    }
  }
  __syncthreads();
  if (t == 0) {
    table_bits[s * 4 + cs] = bits;
    dht_bytes[s * 4 + cs] = 5 + 16 + (nvals > 0 ? nvals : 1);  // an empty table holds symbol 0 (encode.rs:246-248)
  }
}

__global__ void __launch_bounds__(256) k_plan_choose(const PlanDesc* __restrict__ pd, const ScanStats* stats,
                                                     const unsigned long long* table_bits, const int* dht_bytes,
                                                     PlanOut* out) {
  __shared__ unsigned long long cost[kMaxScans];
  __shared__ unsigned long long best_v[256];
  __shared__ int best_i[256];
  const int t = threadIdx.x;
  if (t < pd->nscans) {
    unsigned long long bits = stats[t].raw_bits, total = 0;
    for (int cs = 0; cs < 4; cs++) {
      bits += table_bits[t * 4 + cs];
      total += (unsigned long long)dht_bytes[t * 4 + cs];
    }
    const bool baseline = pd->scan[t].kind == kBaseline;
    cost[t] = total + (bits + 7) / 8 + (baseline ? 20 : 14);
    out->cost[t] = cost[t];
  }
  __syncthreads();
  unsigned long long bv = ~0ull;
  int bi = 0x7fffffff;
  for (int i = t; i < pd->nscripts; i += blockDim.x) {
    unsigned long long sum = 0;
    for (int j = 0; j < pd->script_len[i]; j++) sum += cost[pd->script[i][j]];
    if (sum < bv) {
      bv = sum;
      bi = i;
    }
  }
  best_v[t] = bv;
  best_i[t] = bi;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (t < o) {
      const unsigned long long v2 = best_v[t + o];
      const int i2 = best_i[t + o];
      if (v2 < best_v[t] || (v2 == best_v[t] && i2 < best_i[t])) {
        best_v[t] = v2;
        best_i[t] = i2;
      }
    }
    __syncthreads();
  }
  if (t == 0) {
    out->prog = best_v[0];
    out->best = best_i[0];
  }
}

struct HostScan {
  std::vector<int> comps;
  int ss, se, ah, al;
  bool operator==(const HostScan& o) const {
    return comps == o.comps && ss == o.ss && se == o.se && ah == o.ah && al == o.al;
  }
};

// The candidate scripts of jpeg/src/progressive.rs:246-295 (the family must be the reference's: its members and
// their order decide which script wins a tie). DC precision x luma band split x luma successive-approximation depth
// x (colour only) chroma depth x chroma band split.
std::vector<std::vector<HostScan>> candidate_scripts(int ncomp) {
  std::vector<int> all;
  for (int i = 0; i < ncomp; i++) all.push_back(i);
  const bool colour = ncomp >= 3;
  const int chroma_depths = colour ? 2 : 1;
  const int chroma_splits[3] = {-1, 2, 5};
  const int n_chroma_splits = colour ? 3 : 1;
  const int luma_splits[4] = {-1, 2, 5, 8};
  std::vector<std::vector<HostScan>> out;
  for (int dc_al = 0; dc_al <= 1; dc_al++)
    for (int ls : luma_splits)
      for (int luma_al = 0; luma_al <= 2; luma_al++)
        for (int chroma_al = 0; chroma_al < chroma_depths; chroma_al++)
          for (int cs_i = 0; cs_i < n_chroma_splits; cs_i++) {
            const int cs = chroma_splits[cs_i];
            std::vector<HostScan> v;
            v.push_back({all, 0, 0, 0, dc_al});
            if (ls < 0) {
              v.push_back({{0}, 1, 63, 0, luma_al});
            } else {
              v.push_back({{0}, 1, ls, 0, luma_al});
              v.push_back({{0}, ls + 1, 63, 0, luma_al});
            }
            if (colour)
              for (int c = 1; c < ncomp; c++) {
                if (cs < 0) {
                  v.push_back({{c}, 1, 63, 0, chroma_al});
                } else {
                  v.push_back({{c}, 1, cs, 0, chroma_al});
                  v.push_back({{c}, cs + 1, 63, 0, chroma_al});
                }
              }
            if (dc_al > 0) v.push_back({all, 0, 0, 1, 0});
            for (int ah = luma_al; ah >= 1; ah--) v.push_back({{0}, 1, 63, ah, ah - 1});
            for (int ah = chroma_al; ah >= 1; ah--)
              for (int c = 1; c < ncomp; c++) v.push_back({{c}, 1, 63, ah, ah - 1});
            out.push_back(v);
          }
  return out;
}

void to_abi(const HostScan& h, rcg_scan* o) {
  std::memset(o, 0, sizeof *o);
  o->ncomps = (int)h.comps.size();
  for (size_t i = 0; i < h.comps.size() && i < 4; i++) o->comps[i] = h.comps[i];
  o->ss = h.ss;
  o->se = h.se;
  o->ah = h.ah;
  o->al = h.al;
}

}  // namespace

int plan_scans(rcg_ctx* ctx, const StepDesc* lay, int w, int h, const int16_t* d_coefs, rcg_plan_result* res) {
  const int nc = lay->ncomp;
  if (nc != 1 && nc != 3) return fail(ctx, RCG_UNSUPPORTED, "scan planning takes 1 or 3 components");
  if ((reinterpret_cast<uintptr_t>(d_coefs) & 15) != 0)
    return fail(ctx, RCG_INVALID, "device coefficients must be 16-byte aligned");
  std::vector<std::vector<HostScan>> scripts = candidate_scripts(nc);
  std::vector<HostScan> distinct;
  PlanDesc* pd = new PlanDesc;
  std::memset(pd, 0, sizeof *pd);
  pd->ncomp = nc;
  pd->nscripts = (int)scripts.size();
  for (size_t i = 0; i < scripts.size(); i++) {
    pd->script_len[i] = (int)scripts[i].size();
    for (size_t j = 0; j < scripts[i].size(); j++) {
      size_t d = 0;
      while (d < distinct.size() && !(distinct[d] == scripts[i][j])) d++;
      if (d == distinct.size()) distinct.push_back(scripts[i][j]);
      pd->script[i][j] = (unsigned char)d;
    }
  }
  const int hmax = lay->hmax, vmax = lay->vmax;
  pd->mcus_x = (w + 8 * hmax - 1) / (8 * hmax);
  pd->mcus_y = (h + 8 * vmax - 1) / (8 * vmax);
  int mb = 0;
  for (int c = 0; c < nc; c++) {
    pd->comp[c] = lay->comp[c];
    pd->mcu_off[c] = mb;
    mb += lay->comp[c].h * lay->comp[c].v;
  }
  pd->mcu_blocks = mb;
  pd->nscans = (int)distinct.size() + 1;
  long long chunks = 0, aux = 0, pre = 0;
  const long long mcu_pos = (long long)pd->mcus_x * pd->mcus_y * mb;
  for (int s = 0; s < pd->nscans; s++) {
    ScanDesc& sd = pd->scan[s];
    if (s == pd->nscans - 1) {
      sd.kind = kBaseline;
      sd.interleaved = 1;
      sd.npos = mcu_pos;
    } else {
      const HostScan& hs = distinct[s];
      sd.kind = hs.ss == 0 ? (hs.ah == 0 ? kDcFirst : kDcRefine) : (hs.ah == 0 ? kAcFirst : kAcRefine);
      sd.ss = hs.ss;
      sd.se = hs.se;
      sd.al = hs.al;
      if (hs.comps.size() > 1) {
        sd.interleaved = 1;
        sd.npos = mcu_pos;
      } else {
        // Non-interleaved scans cover the blocks that overlap the image (progressive.rs:226-229).
        const int k = hs.comps[0];
        const CompDesc& c = lay->comp[k];
        sd.comp = k;
        sd.real_w = ((w * c.h + hmax - 1) / hmax + 7) / 8;
        const int real_h = ((h * c.v + vmax - 1) / vmax + 7) / 8;
        sd.npos = (long long)sd.real_w * real_h;
      }
    }
    sd.chunk0 = chunks;
    chunks += (sd.npos + kChunk - 1) / kChunk;
    sd.aux0 = sd.p0 = -1;
    if (sd.kind == kAcFirst || sd.kind == kAcRefine) {
      sd.aux0 = aux;
      aux += sd.npos;
    }
    if (sd.kind == kAcRefine) {
      sd.p0 = pre;
      pre += sd.npos + 1;
    }
  }
  pd->nchunks = chunks;
  if (mcu_pos >= (1ll << 31) || chunks >= (1ll << 31)) {
    delete pd;
    return fail(ctx, RCG_UNSUPPORTED, "image too large for scan planning");
  }
  const int ns = pd->nscans;
  PlanDesc* d_pd = (PlanDesc*)workspace(ctx, "plan_desc", sizeof(PlanDesc));
  ScanStats* d_stats = (ScanStats*)workspace(ctx, "plan_stats", sizeof(ScanStats) * kMaxScans);
  uint16_t* d_flags = (uint16_t*)workspace(ctx, "plan_flags", (size_t)std::max(aux, 1ll) * 2);
  int* d_prev = (int*)workspace(ctx, "plan_prev", (size_t)std::max(aux, 1ll) * 4);
  unsigned long long* d_P = (unsigned long long*)workspace(ctx, "plan_pending", (size_t)std::max(pre, 1ll) * 8);
  int* d_chunk_last = (int*)workspace(ctx, "plan_chunk_last", (size_t)chunks * 4);
  unsigned long long* d_chunk_pend = (unsigned long long*)workspace(ctx, "plan_chunk_pend", (size_t)chunks * 8);
  int* d_chunk_prev = (int*)workspace(ctx, "plan_chunk_prev", (size_t)chunks * 4);
  unsigned long long* d_chunk_pbase = (unsigned long long*)workspace(ctx, "plan_chunk_pbase", (size_t)chunks * 8);
  int* d_prev_end = (int*)workspace(ctx, "plan_prev_end", sizeof(int) * kMaxScans);
  unsigned long long* d_tbits = (unsigned long long*)workspace(ctx, "plan_table_bits", 8 * 4 * kMaxScans);
  int* d_dht = (int*)workspace(ctx, "plan_dht", 4 * 4 * kMaxScans);
  PlanOut* d_out = (PlanOut*)workspace(ctx, "plan_out", sizeof(PlanOut));
  if (!d_pd || !d_stats || !d_flags || !d_prev || !d_P || !d_chunk_last || !d_chunk_pend || !d_chunk_prev ||
      !d_chunk_pbase || !d_prev_end || !d_tbits || !d_dht || !d_out) {
    delete pd;
    return RCG_NO_MEMORY;
  }
  cudaMemcpyAsync(d_pd, pd, sizeof(PlanDesc), cudaMemcpyHostToDevice, ctx->stream);
  cudaMemsetAsync(d_stats, 0, sizeof(ScanStats) * ns, ctx->stream);
  RCG_LAUNCH(ctx, "plan_blocks", k_plan_blocks, (unsigned)chunks, kThreads, 0, d_pd, d_coefs, d_stats, d_flags,
             d_chunk_last, d_chunk_pend);
  RCG_LAUNCH(ctx, "plan_chunks", k_plan_chunks, ns, 1024, 0, d_pd, d_chunk_last, d_chunk_pend, d_chunk_prev,
             d_chunk_pbase);
  RCG_LAUNCH(ctx, "plan_prefix", k_plan_prefix, (unsigned)chunks, kThreads, 0, d_pd, d_flags, d_chunk_prev,
             d_chunk_pbase, d_prev, d_P, d_prev_end);
  RCG_LAUNCH(ctx, "plan_eobruns", k_plan_eobruns, (unsigned)chunks, kThreads, 0, d_pd, d_flags, d_prev, d_P,
             d_prev_end, d_stats);
  RCG_LAUNCH(ctx, "plan_tables", k_plan_tables, dim3(ns, 4), 288, 0, d_pd, d_stats, d_tbits, d_dht);
  RCG_LAUNCH(ctx, "plan_choose", k_plan_choose, 1, 256, 0, d_pd, d_stats, d_tbits, d_dht, d_out);
  PlanOut host_out;
  cudaMemcpyAsync(&host_out, d_out, sizeof(PlanOut), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    delete pd;
    return cuda_fail(ctx, e, "scan planning");
  }
  std::memset(res, 0, sizeof *res);
  res->progressive_bytes = host_out.prog;
  res->baseline_bytes = host_out.cost[ns - 1];
  res->progressive = res->baseline_bytes <= res->progressive_bytes ? 0 : 1;  // encode.rs:545
  const std::vector<HostScan>& best = scripts[host_out.best];
  res->nscans = (int)best.size();
  for (size_t i = 0; i < best.size(); i++) to_abi(best[i], &res->scans[i]);
  res->ndistinct = (int)distinct.size();
  for (size_t i = 0; i < distinct.size(); i++) {
    to_abi(distinct[i], &res->distinct[i]);
    res->distinct_bytes[i] = host_out.cost[i];
  }
  delete pd;
  return RCG_OK;
}

}  // namespace rcg
