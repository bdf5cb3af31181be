// Entropy decoding of Huffman JPEGs on the GPU: jpeg::decode::parse(data)?.into_coefs()
// (jpeg/src/decode.rs:397-445, :540-570) for SOF0/SOF1 (sequential) and SOF2 (progressive) 8-bit frames with 1 or 3
// components, any sampling, restart intervals and any number of scans.
//
// The host walks the markers (decode.rs:622-697: DQT, DHT, SOF, DRI, SOS, APP14), builds each scan's Huffman tables
// as they stand when the scan starts, removes the 0xFF00 stuffing and cuts each scan into its restart segments,
// following the bit reader's rules exactly (decode.rs:16-114): a segment's bits end at the first 0xFF not followed
// by 0x00, reads past the end give zero bits, and the next segment starts just past the next RSTn (if the marker
// found there is not an RSTn, that segment and all later ones read zero bits).
//
// The device decodes each segment in parallel by self-synchronization. A decoding state at a codeword boundary is
// (bit position, block of the MCU, next coefficient index). The segment's bits are cut into spans of 2048 bits, one
// thread each, and each span into pieces of 256 bits. Round after round every thread decodes its span from its
// current start state, records the state and the block count and DC-difference sums at every piece boundary, and
// hands the state where it crosses into the next span to its successor. The first span of a segment starts from
// the exact state, so the states become exact from front to back; Huffman codes resynchronize within a few
// codewords, but the block-of-the-MCU part of the state only when a desynchronization happens to realign it, which
// takes a few MCUs, hence spans long enough to settle in a few rounds. When a round changes nothing, every piece
// start is exact; prefix sums of the counts give each piece its first block and DC predictions, and a last pass,
// one thread per piece, decodes again and writes the coefficients. If the rounds do not settle within a bound, one
// thread per segment follows the chain of states instead.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "rcg_internal.cuh"

namespace rcg {

namespace {

constexpr int kSubBits = 256;   // a piece: the unit of the writing pass
constexpr int kSpanSubs = 8;    // a span (8 pieces, 2048 bits): the unit of the synchronization rounds
constexpr int kDecThreads = 64;
constexpr int kFirstBatch = 3;  // rounds launched before the first convergence check
constexpr int kMaxRounds = 48;
constexpr int kMaxMcuBlocks = 48;
constexpr unsigned long long kMaxPixels = 150000000ull;  // core/src/image.rs:33 (MAX_PIXELS)
constexpr size_t kMaxScans = 1000;                         // jpeg/src/decode.rs:282 (MAX_SCANS)

const int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                         41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                         30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// A Huffman table for decoding (decode.rs:117-188): 9-bit lookup (length << 8 | symbol, 0 = longer code), then the
// canonical search over lengths 10..16.
struct DevHuff {
  uint16_t fast[512];
  int32_t mincode[17];
  int32_t maxcode[18];
  int32_t valptr[17];
  uint8_t vals[256];
};

// decode.rs:126-166 (HuffDec::new). Returns false for an oversubscribed or overlong table.
bool build_huff(const uint8_t bits[16], const uint8_t* vals, size_t nvals, DevHuff* h) {
  size_t total = 0;
  for (int i = 0; i < 16; i++) total += bits[i];
  if (total > 256 || total > nvals) return false;
  std::memset(h, 0, sizeof *h);
  for (int i = 0; i < 18; i++) h->maxcode[i] = -1;
  std::memcpy(h->vals, vals, total);
  int code = 0;
  int k = 0;
  for (int len = 1; len <= 16; len++) {
    const int n = bits[len - 1];
    h->valptr[len] = k;
    h->mincode[len] = code;
    if (n > 0) {
      if (code + n > (1 << len)) return false;
      if (len <= 9)
        for (int i = 0; i < n; i++) {
          const int c = code + i, shift = 9 - len;
          for (int f = 0; f < (1 << shift); f++) h->fast[(c << shift) | f] = (uint16_t)((len << 8) | h->vals[k + i]);
        }
      code += n;
      k += n;
      h->maxcode[len] = code - 1;
    }
    code <<= 1;
  }
  return true;
}

struct Segment {
  long long byte0;    // first destuffed byte of the segment in the scan's buffer
  long long nbytes;   // destuffed bytes of the segment (reads beyond give zeros)
  long long block0;   // first block of the segment in the scan's visiting order
  long long nblocks;  // blocks the segment decodes
  long long sub0;     // first piece of the segment
  int nsub;           // pieces
  long long span0;    // first span of the segment
  int nspan;          // spans
};

// Scan kinds (jpeg/src/decode.rs:1275-1300): sequential, and the four progressive ones. The first three decode by
// self-synchronization; a DC refinement scan is one raw bit per block; an AC refinement scan reads one correction
// bit per coefficient that earlier scans made nonzero, so where its bits fall depends on every block's history and
// one thread decodes each restart segment in order.
enum ScanKind { kSeq = 0, kDcFirst = 1, kDcRefine = 2, kAcFirst = 3, kAcRefine = 4 };

struct ScanDesc {
  int kind;                   // ScanKind
  int ss, se, ah, al;         // spectral band and successive approximation (sequential: 0, 63, 0, 0)
  int k0;                     // coefficient index at a block's start (ss for AC scans, else 0)
  int ns;                     // components in the scan
  int bmcu;                   // blocks per MCU (1 for a single-component scan)
  int mcus_x;                 // MCUs per row
  int mcu_si[kMaxMcuBlocks];  // scan component of each block of the MCU
  int mcu_dy[kMaxMcuBlocks], mcu_dx[kMaxMcuBlocks];
  int comp[4];                // frame component of each scan component
  int dc[4], ac[4];           // table slot of each scan component
  CompDesc fc[3];             // frame components (block grids, offsets)
  int nseg;
  long long nsub;   // pieces of the scan
  long long nspan;  // spans of the scan
};

struct SubState {
  long long bit;  // segment-relative bit position of a codeword boundary
  int u;          // block of the MCU
  int k;          // next coefficient (0: the DC)
};

struct SubCount {
  long long blocks;  // blocks completed
  uint32_t dc[4];    // sums of DC differences per scan component (wrapping, as the reference's i32 predictor)
};

// Bit reader over a segment's unstuffed bytes: reads past the segment's end give zeros (decode.rs:30-60). Bytes
// inside a shared-memory window (the CTA's slice of the buffer, loaded once, coalesced) come from there; the rest
// from global memory.
struct Reader {
  const uint8_t* p;       // segment start in global memory
  const uint8_t* win;     // shared-memory copy of global bytes [win_lo, win_hi) of the scan buffer
  long long seg_at;       // scan-buffer offset of the segment start
  long long win_lo, win_hi;
  long long len, next;
  uint64_t buf;
  int n;
  long long bit;
  __device__ void init(const uint8_t* data, long long seg_byte0, long long nbytes, long long at,
                       const uint8_t* window = nullptr, long long lo = 0, long long hi = 0) {
    p = data + seg_byte0;
    seg_at = seg_byte0;
    win = window;
    win_lo = lo;
    win_hi = hi;
    len = nbytes;
    next = at >> 3;
    buf = 0;
    n = 0;
    bit = at;
    refill();
    skip((int)(at & 7));
    bit = at;
  }
  __device__ __forceinline__ uint64_t byte_at(long long j) const {
    if (j >= len) return 0;
    const long long g = seg_at + j;
    if (g >= win_lo && g < win_hi) return win[g - win_lo];
    return p[j];
  }
  __device__ __forceinline__ void refill() {
    // Four bytes at a time (whole window hits take no per-byte checks); keeps at least 32 bits buffered.
    while (n <= 32) {
      const long long g = seg_at + next;
      uint32_t w;
      if (next + 4 <= len && g >= win_lo && g + 4 <= win_hi) {
        const uint8_t* q = win + (g - win_lo);
        w = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
      } else {
        w = (uint32_t)((byte_at(next) << 24) | (byte_at(next + 1) << 16) | (byte_at(next + 2) << 8) |
                       byte_at(next + 3));
      }
      buf |= (uint64_t)w << (32 - n);
      next += 4;
      n += 32;
    }
  }
  __device__ __forceinline__ uint32_t peek(int k) {
    if (n < k) refill();
    return (uint32_t)(buf >> (64 - k));
  }
  __device__ __forceinline__ void skip(int k) {
    buf <<= k;
    n -= k;
    bit += k;
  }
  __device__ __forceinline__ uint32_t bits(int k) {
    if (k == 0) return 0;
    const uint32_t v = peek(k);
    skip(k);
    return v;
  }
};

__device__ __forceinline__ int huff_decode(const DevHuff& h, Reader& r) {
  const uint16_t e = h.fast[r.peek(9)];
  if (e != 0) {
    r.skip(e >> 8);
    return e & 0xFF;
  }
  const uint32_t w = r.peek(16);
  for (int len = 10; len <= 16; len++) {
    const int code = (int)(w >> (16 - len));
    if (h.maxcode[len] >= 0 && code <= h.maxcode[len] && code >= h.mincode[len]) {
      r.skip(len);
      return h.vals[h.valptr[len] + code - h.mincode[len]];
    }
  }
  return -1;
}

__device__ __forceinline__ int extend_bits(uint32_t v, int t) {
  if (t == 0) return 0;
  return v < (1u << (t - 1)) ? (int)v - (1 << t) + 1 : (int)v;
}

struct Tables {
  DevHuff dc[4], ac[4];
};

// Decodes from `st` until the bit position reaches `stop_bit` or `max_blocks` blocks are complete. WRITE: also
// stores the coefficients of block `block_base + blocks` onward (zigzag order), with DC predictors `pred`.
// Returns 0, or 1 on a bad code (decode.rs:1482-1506).
template <bool WRITE>
__device__ __forceinline__ int decode_run(const Tables& tb, const ScanDesc& sd, Reader& r, SubState& st, long long stop_bit,
                          long long max_blocks, SubCount& cnt, long long block_base, uint32_t* pred,
                          int16_t* __restrict__ out) {
  int u = st.u, k = st.k;
  uint32_t d0 = cnt.dc[0], d1 = cnt.dc[1], d2 = cnt.dc[2], d3 = cnt.dc[3];
  const uint32_t p0 = WRITE ? pred[0] - d0 : 0u, p1 = WRITE ? pred[1] - d1 : 0u, p2 = WRITE ? pred[2] - d2 : 0u,
                 p3 = WRITE ? pred[3] - d3 : 0u;
  int16_t* blk = nullptr;
  auto block_ptr = [&](long long b) -> int16_t* {
    const long long mcu = b / sd.bmcu;
    const int uu = (int)(b - mcu * sd.bmcu);
    const int si = sd.mcu_si[uu];
    const CompDesc& c = sd.fc[sd.comp[si]];
    const long long my = mcu / sd.mcus_x, mx = mcu - my * sd.mcus_x;
    const long long row = my * (sd.bmcu == 1 ? 1 : c.v) + sd.mcu_dy[uu];
    const long long col = mx * (sd.bmcu == 1 ? 1 : c.h) + sd.mcu_dx[uu];
    return out + (c.blk0 + row * c.bw + col) * 64;
  };
  if (WRITE && cnt.blocks < max_blocks) blk = block_ptr(block_base + cnt.blocks);
  int err = 0;
  // One symbol per iteration with a single code path for DC and AC symbols (the lanes of a warp decode different
  // streams; branches would serialize them). decode_sequential (decode.rs:1482-1506) in select form: a DC symbol is
  // a size t <= 16 and t extra bits; an AC symbol (run, size) is EOB (size 0, run < 15), ZRL (size 0, run 15: k += 16)
  // or a coefficient at k + run (error past 63); the block ends when k reaches 64 or at EOB. The progressive first
  // scans are the same loop: decode_dc_first (:1509-1517) is a DC symbol per block, its value shifted left by al;
  // decode_ac_first (:1519-1547) runs k from ss, ends the block past se, shifts values by al, and an EOB symbol
  // there is an end-of-band run: 2^run - 1 + (run extra bits) further blocks read no bits at all.
  const bool dc_only = sd.kind == kDcFirst, ac_first = sd.kind == kAcFirst;
  const int kend = ac_first ? sd.se : 63, shift = sd.al;
  long long blocks = cnt.blocks;
  while (blocks < max_blocks && r.bit < stop_bit) {
    const int si = sd.mcu_si[u];
    const bool dc = dc_only || (!ac_first && k == 0);
    const int sym = huff_decode(dc ? tb.dc[sd.dc[si]] : tb.ac[sd.ac[si]], r);
    const int run = dc ? 0 : (sym >> 4);
    const int sz = dc ? sym : (sym & 15);
    if (sym < 0 || sz > 16 || (!dc && sz > 0 && k + run > 63)) {
      err = 1;
      break;
    }
    const int v = extend_bits(r.bits(sz), sz);
    // end-of-band run of an AC first scan (sz == 0 here, so no value bits were read)
    const long long skip = (ac_first && sz == 0 && run < 15) ? (long long)((1u << run) - 1u + r.bits(run)) : 0;
    const uint32_t ud = dc ? (uint32_t)v : 0u;  // selects instead of indexing by si: the sums stay in registers
    d0 += si == 0 ? ud : 0u;
    d1 += si == 1 ? ud : 0u;
    d2 += si == 2 ? ud : 0u;
    d3 += si == 3 ? ud : 0u;
    if (WRITE) {
      if (dc)
        blk[0] = (int16_t)((si == 0 ? p0 + d0 : si == 1 ? p1 + d1 : si == 2 ? p2 + d2 : p3 + d3) << shift);
      else if (sz > 0)
        blk[k + run] = (int16_t)((uint32_t)v << shift);
    }
    const int nk = dc ? (dc_only ? 64 : 1) : (sz == 0 ? (run == 15 ? k + 16 : 64) : k + run + 1);
    const bool end = nk > kend;
    k = end ? sd.k0 : nk;
    if (end) {
      u = u + 1 == sd.bmcu ? 0 : u + 1;
      blocks += 1 + skip;
      if (WRITE && blocks < max_blocks) blk = block_ptr(block_base + blocks);
    }
  }
  cnt.blocks = blocks;
  st.bit = r.bit;
  st.u = u;
  st.k = k;
  cnt.dc[0] = d0;
  cnt.dc[1] = d1;
  cnt.dc[2] = d2;
  cnt.dc[3] = d3;
  return err;
}

struct SubRef {
  int seg;
  int local;  // index within the segment
};

// The segment holding piece (spans == false) or span (spans == true) t.
__device__ __forceinline__ SubRef find_sub(const Segment* segs, int nseg, long long t, bool spans) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if ((spans ? segs[mid].span0 : segs[mid].sub0) <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return {lo, (int)(t - (spans ? segs[lo].span0 : segs[lo].sub0))};
}

constexpr int kTail = 64;  // bytes past a unit a decode may read (last codeword, reader look-ahead)

// Scan-buffer byte range [lo, hi) of the units (spans or pieces) [t0, t0 + count) of one CTA, rounded out to
// 16 bytes and capped at `cap` bytes. Units of consecutive segments are consecutive in the buffer.
__device__ __forceinline__ void unit_window(const Segment* segs, int nseg, long long t0, long long count,
                                            long long nunits, bool spans, long long cap, long long* lo,
                                            long long* hi) {
  const int ub = spans ? kSpanSubs * kSubBits / 8 : kSubBits / 8;
  const SubRef a = find_sub(segs, nseg, t0, spans);
  const SubRef b = find_sub(segs, nseg, min(t0 + count, nunits) - 1, spans);
  const long long l = (segs[a.seg].byte0 + (long long)a.local * ub) & ~15ll;
  const long long h = (segs[b.seg].byte0 + (long long)(b.local + 1) * ub + kTail + 15) & ~15ll;
  *lo = l;
  *hi = min(h, l + cap);
}

// Copies scan-buffer bytes [lo, hi) (16-byte aligned; the buffer is padded past its end) into shared memory.
__device__ __forceinline__ void load_window(const uint8_t* data, long long lo, long long hi, uint8_t* win) {
  const int4* src = reinterpret_cast<const int4*>(data + lo);
  int4* dst = reinterpret_cast<int4*>(win);
  for (long long i = threadIdx.x; i < (hi - lo) / 16; i += blockDim.x) dst[i] = __ldg(src + i);
}

__device__ __forceinline__ void load_tables(Tables& sh, const Tables* g) {
  const int4* src = reinterpret_cast<const int4*>(g);
  int4* dst = reinterpret_cast<int4*>(&sh);
  for (int i = threadIdx.x; i < (int)(sizeof(Tables) / 16); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

// One round, one thread per span: decode the span's pieces from the span's current start, record the state and
// the counts at every piece boundary, and propose the state at the span's end as the next span's start.
__global__ void __launch_bounds__(kDecThreads) k_seq_sync(const ScanDesc* __restrict__ sdp, const Tables* __restrict__ tg,
                                                          const Segment* __restrict__ segs,
                                                          const uint8_t* __restrict__ data,
                                                          const SubState* __restrict__ cur, SubState* __restrict__ nxt,
                                                          SubState* __restrict__ piece_state,
                                                          SubCount* __restrict__ counts, int* __restrict__ changed) {
  __shared__ __align__(16) Tables tb;
  __shared__ ScanDesc sd;
  if (threadIdx.x == 0) sd = *sdp;
  load_tables(tb, tg);
  constexpr long long kWin = (long long)kDecThreads * (kSpanSubs * kSubBits / 8 + 4) + kTail + 32;
  __shared__ __align__(16) uint8_t win[kWin];
  __shared__ long long w_lo, w_hi;
  const long long t0 = (long long)blockIdx.x * blockDim.x;
  if (threadIdx.x == 0) unit_window(segs, sd.nseg, t0, blockDim.x, sd.nspan, true, kWin & ~15ll, &w_lo, &w_hi);
  __syncthreads();
  load_window(data, w_lo, w_hi, win);
  __syncthreads();
  const long long t = t0 + threadIdx.x;
  if (t >= sd.nspan) return;
  const SubRef ref = find_sub(segs, sd.nseg, t, true);
  const Segment& sg = segs[ref.seg];
  if (ref.local == 0) nxt[t] = SubState{0, 0, sd.k0};
  const int f0 = ref.local * kSpanSubs, f1 = min(f0 + kSpanSubs, sg.nsub);
  SubState st = cur[t];
  piece_state[sg.sub0 + f0] = st;
  Reader r;
  r.init(data, sg.byte0, sg.nbytes, st.bit, win, w_lo, w_hi);
  for (int f = f0; f < f1 && f + 1 < sg.nsub; f++) {
    SubCount cnt{};
    const long long stop = (long long)(f + 1) * kSubBits;
    if (decode_run<false>(tb, sd, r, st, stop, LLONG_MAX, cnt, 0, nullptr, nullptr)) {
      st = SubState{stop, 0, sd.k0};  // desynchronized: any guess will do
      r.init(data, sg.byte0, sg.nbytes, stop, win, w_lo, w_hi);
    }
    counts[sg.sub0 + f] = cnt;
    piece_state[sg.sub0 + f + 1] = st;
  }
  if (ref.local + 1 >= sg.nspan) return;  // the segment's last span proposes nothing
  nxt[t + 1] = st;
  const SubState& old = cur[t + 1];
  if (old.bit != st.bit || old.u != st.u || old.k != st.k) atomicOr(changed, 1);
}

// Fallback when the rounds do not settle: one thread per segment follows the chain of exact piece states.
__global__ void k_seq_chain(const ScanDesc* __restrict__ sdp, const Tables* __restrict__ tg,
                            const Segment* __restrict__ segs, const uint8_t* __restrict__ data,
                            SubState* __restrict__ piece_state, SubCount* __restrict__ counts) {
  __shared__ __align__(16) Tables tb;
  __shared__ ScanDesc sd;
  if (threadIdx.x == 0) sd = *sdp;
  load_tables(tb, tg);
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < sd.nseg; s += gridDim.x * blockDim.x) {
    const Segment& sg = segs[s];
    SubState st{0, 0, sd.k0};
    Reader r;
    r.init(data, sg.byte0, sg.nbytes, 0);
    for (int i = 0; i + 1 < sg.nsub; i++) {
      piece_state[sg.sub0 + i] = st;
      SubCount cnt{};
      const long long stop = (long long)(i + 1) * kSubBits;
      if (decode_run<false>(tb, sd, r, st, stop, LLONG_MAX, cnt, 0, nullptr, nullptr)) {
        st = SubState{stop, 0, sd.k0};
        r.init(data, sg.byte0, sg.nbytes, stop);
      }
      counts[sg.sub0 + i] = cnt;
    }
    piece_state[sg.sub0 + sg.nsub - 1] = st;
  }
}

// Per segment, exclusive prefix sums of the pieces' block counts and DC sums (one CTA per segment, 1024 pieces at a
// time: warp shuffles, then the 32 warp totals).
__global__ void __launch_bounds__(1024) k_seq_prefix(const ScanDesc* __restrict__ sdp, const Segment* __restrict__ segs,
                                                     const SubCount* __restrict__ counts, SubCount* __restrict__ base) {
  __shared__ long long wb[32];
  __shared__ uint32_t wd[4][32];
  const ScanDesc& sd = *sdp;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = blockIdx.x; s < sd.nseg; s += gridDim.x) {
    const Segment& sg = segs[s];
    long long carry_b = 0;
    uint32_t carry_d[4] = {0, 0, 0, 0};
    for (int off = 0; off < sg.nsub; off += 1024) {
      const int i = off + threadIdx.x;
      // piece i starts after pieces 0..i-1 (the last piece's counts are never needed)
      SubCount c{};
      if (i >= 1 && i < sg.nsub) c = counts[sg.sub0 + i - 1];
      long long b = c.blocks;
      uint32_t d[4] = {c.dc[0], c.dc[1], c.dc[2], c.dc[3]};
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long bo = __shfl_up_sync(0xffffffffu, b, o);
        uint32_t dq[4];
#pragma unroll
        for (int q = 0; q < 4; q++) dq[q] = __shfl_up_sync(0xffffffffu, d[q], o);
        if (lane >= o) {
          b += bo;
#pragma unroll
          for (int q = 0; q < 4; q++) d[q] += dq[q];
        }
      }
      if (lane == 31) {
        wb[warp] = b;
#pragma unroll
        for (int q = 0; q < 4; q++) wd[q][warp] = d[q];
      }
      __syncthreads();
      if (warp == 0) {
        long long x = wb[lane];
        uint32_t y[4] = {wd[0][lane], wd[1][lane], wd[2][lane], wd[3][lane]};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const long long xo = __shfl_up_sync(0xffffffffu, x, o);
          uint32_t yo[4];
#pragma unroll
          for (int q = 0; q < 4; q++) yo[q] = __shfl_up_sync(0xffffffffu, y[q], o);
          if (lane >= o) {
            x += xo;
#pragma unroll
            for (int q = 0; q < 4; q++) y[q] += yo[q];
          }
        }
        wb[lane] = x;
#pragma unroll
        for (int q = 0; q < 4; q++) wd[q][lane] = y[q];
      }
      __syncthreads();
      if (warp > 0) {
        b += wb[warp - 1];
#pragma unroll
        for (int q = 0; q < 4; q++) d[q] += wd[q][warp - 1];
      }
      if (i < sg.nsub) {
        SubCount o;
        o.blocks = carry_b + b;
#pragma unroll
        for (int q = 0; q < 4; q++) o.dc[q] = carry_d[q] + d[q];
        base[sg.sub0 + i] = o;
      }
      carry_b += wb[31];
#pragma unroll
      for (int q = 0; q < 4; q++) carry_d[q] += wd[q][31];
      __syncthreads();
    }
  }
}

// Final pass: decode each subsequence from its exact start and write the coefficients.
__global__ void __launch_bounds__(kDecThreads) k_seq_write(const ScanDesc* __restrict__ sdp, const Tables* __restrict__ tg,
                                                   const Segment* __restrict__ segs, const uint8_t* __restrict__ data,
                                                   const SubState* __restrict__ states,
                                                   const SubCount* __restrict__ base, int16_t* __restrict__ out,
                                                   int* __restrict__ error) {
  __shared__ __align__(16) Tables tb;
  __shared__ ScanDesc sd;
  if (threadIdx.x == 0) sd = *sdp;
  load_tables(tb, tg);
  constexpr long long kWin = (long long)kDecThreads * (kSubBits / 8 + 4) + kTail + 32;
  __shared__ __align__(16) uint8_t win[kWin];
  __shared__ long long w_lo, w_hi;
  const long long t0 = (long long)blockIdx.x * blockDim.x;
  if (threadIdx.x == 0) unit_window(segs, sd.nseg, t0, blockDim.x, sd.nsub, false, kWin & ~15ll, &w_lo, &w_hi);
  __syncthreads();
  load_window(data, w_lo, w_hi, win);
  __syncthreads();
  const long long t = t0 + threadIdx.x;
  if (t >= sd.nsub) return;
  const SubRef ref = find_sub(segs, sd.nseg, t, false);
  const Segment& sg = segs[ref.seg];
  const SubCount b = base[t];
  if (b.blocks >= sg.nblocks) return;  // past the segment's last block: padding
  SubState st = states[t];
  if (st.u != (int)((sg.block0 + b.blocks) % sd.bmcu)) {
    atomicCAS(error, 0, 2);  // inconsistent start (cannot happen for exact states)
    return;
  }
  SubCount cnt{};
  uint32_t pred[4] = {b.dc[0], b.dc[1], b.dc[2], b.dc[3]};
  Reader r;
  r.init(data, sg.byte0, sg.nbytes, st.bit, win, w_lo, w_hi);
  const long long stop = ref.local + 1 < sg.nsub ? (long long)(ref.local + 1) * kSubBits : LLONG_MAX;
  if (decode_run<true>(tb, sd, r, st, stop, sg.nblocks - b.blocks, cnt, sg.block0 + b.blocks, pred, out))
    atomicCAS(error, 0, 1);
}

// The visiting-order block b of a scan -> its coefficients.
__device__ __forceinline__ int16_t* scan_block(const ScanDesc& sd, int16_t* out, long long b) {
  const long long mcu = b / sd.bmcu;
  const int uu = (int)(b - mcu * sd.bmcu);
  const int si = sd.mcu_si[uu];
  const CompDesc& c = sd.fc[sd.comp[si]];
  const long long my = mcu / sd.mcus_x, mx = mcu - my * sd.mcus_x;
  const long long row = my * (sd.bmcu == 1 ? 1 : c.v) + sd.mcu_dy[uu];
  const long long col = mx * (sd.bmcu == 1 ? 1 : c.h) + sd.mcu_dx[uu];
  return out + (c.blk0 + row * c.bw + col) * 64;
}

// DC refinement (decode.rs:1283-1286): block j of a segment reads bit j of the segment (zero past its end) into bit al
// of its DC. One thread per block of the scan.
__global__ void __launch_bounds__(256) k_dc_refine(const ScanDesc* __restrict__ sdp, const Segment* __restrict__ segs,
                                                   const uint8_t* __restrict__ data, long long nblocks,
                                                   int16_t* __restrict__ out) {
  const ScanDesc& sd = *sdp;
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  int lo = 0, hi = sd.nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (segs[mid].block0 <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  const Segment& sg = segs[lo];
  const long long j = b - sg.block0;
  const int bit = (j >> 3) < sg.nbytes ? (data[sg.byte0 + (j >> 3)] >> (7 - (int)(j & 7))) & 1 : 0;
  int16_t* blk = scan_block(sd, out, b);
  blk[0] = (int16_t)(blk[0] | (int16_t)(bit << sd.al));
}

// Reads n (0..64) bits MSB first into the low bits of a 64-bit value.
__device__ __forceinline__ uint64_t read_bits64(Reader& r, int n) {
  uint64_t v = 0;
  while (n > 0) {
    const int k = n > 24 ? 24 : n;
    v = (v << k) | r.bits(k);
    n -= k;
  }
  return v;
}

// Correction bits (decode.rs:1571-1575, :1590-1595) for the already-nonzero coefficients at the set positions of
// `corr`, in ascending order, one bit each: a set bit with the al bit of the magnitude still clear moves the
// coefficient away from zero by 2^al.
__device__ __forceinline__ void refine_corrections(Reader& r, int16_t* c, uint64_t corr, int16_t p1, int16_t m1) {
  int nb = __popcll(corr);
  while (nb > 0) {
    const int take = nb > 32 ? 32 : nb;
    const uint64_t bits = read_bits64(r, take);
    for (int j = take - 1; j >= 0; j--) {
      const int pos = __ffsll((long long)corr) - 1;
      corr &= corr - 1;
      const int16_t v = c[pos];
      if (((bits >> j) & 1) && (v & p1) == 0) c[pos] = (int16_t)(v + (v >= 0 ? p1 : m1));
    }
    nb -= take;
  }
}

// AC refinement (decode.rs:1549-1601, decode_ac_refine), one thread per restart segment, its blocks in order: the
// bits a block reads depend on which of its coefficients earlier scans made nonzero. Each block's 64 coefficients
// come in once (eight 16-byte loads, the next block's issued before this one is decoded) to a per-thread row of
// shared memory with a 64-bit mask of the nonzero ones; a run of zero-history coefficients and the correction bits
// of the nonzero ones inside it are then one mask operation and one multi-bit read each, instead of a step per
// coefficient. Same bits read, same values as the reference's loop.
constexpr int kRefineThreads = 32;

__global__ void __launch_bounds__(kRefineThreads) k_ac_refine(const ScanDesc* __restrict__ sdp,
                                                              const Tables* __restrict__ tg,
                                                              const Segment* __restrict__ segs,
                                                              const uint8_t* __restrict__ data,
                                                              int16_t* __restrict__ out, int* __restrict__ error) {
  __shared__ __align__(16) Tables tb;
  __shared__ ScanDesc sd;
  __shared__ __align__(16) int16_t rows[kRefineThreads][64];
  if (threadIdx.x == 0) sd = *sdp;
  load_tables(tb, tg);
  const int16_t p1 = (int16_t)(1 << sd.al), m1 = (int16_t)(-(1 << sd.al));
  const int ss = sd.ss, se = sd.se;
  const uint64_t band = (se >= 63 ? ~0ull : ((1ull << (se + 1)) - 1)) & ~((1ull << ss) - 1);
  int16_t* c = rows[threadIdx.x];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < sd.nseg; s += gridDim.x * blockDim.x) {
    const Segment& sg = segs[s];
    const DevHuff& ac = tb.ac[sd.ac[0]];
    Reader r;
    r.init(data, sg.byte0, sg.nbytes, 0);
    uint32_t eobrun = 0;
    int4 nxt[8];
    if (sg.nblocks > 0) {
      const int4* src = reinterpret_cast<const int4*>(scan_block(sd, out, sg.block0));
#pragma unroll
      for (int g = 0; g < 8; g++) nxt[g] = src[g];
    }
    for (long long b = 0; b < sg.nblocks; b++) {
      int16_t* blk = scan_block(sd, out, sg.block0 + b);
      int4* crow = reinterpret_cast<int4*>(c);
      uint64_t mask = 0;
#pragma unroll
      for (int g = 0; g < 8; g++) {
        crow[g] = nxt[g];
        const uint32_t wv[4] = {(uint32_t)nxt[g].x, (uint32_t)nxt[g].y, (uint32_t)nxt[g].z, (uint32_t)nxt[g].w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (wv[q] & 0xFFFFu) mask |= 1ull << (g * 8 + 2 * q);
          if (wv[q] >> 16) mask |= 1ull << (g * 8 + 2 * q + 1);
        }
      }
      if (b + 1 < sg.nblocks) {
        const int4* src = reinterpret_cast<const int4*>(scan_block(sd, out, sg.block0 + b + 1));
#pragma unroll
        for (int g = 0; g < 8; g++) nxt[g] = src[g];
      }
      const uint64_t hist = mask & band;  // coefficients earlier scans made nonzero, inside the band
      int k = ss;
      if (eobrun == 0) {
        while (k <= se) {
          const int rs = huff_decode(ac, r);
          if (rs < 0) {
            atomicCAS(error, 0, 1);
            return;
          }
          const int run = rs >> 4, sz = rs & 15;
          int16_t value = 0;
          if (sz != 0) {
            value = r.bits(1) ? p1 : m1;
          } else if (run != 15) {
            eobrun = (1u << run) + (run > 0 ? r.bits(run) : 0u);
            break;
          }
          // Skip `run` zero-history coefficients (and refine the nonzero ones among them): stop at the next
          // zero-history one after them, or past the band.
          uint64_t zeros = ~mask & band & (~0ull << k);
          for (int i = 0; i < run && zeros; i++) zeros &= zeros - 1;
          const int t = zeros ? __ffsll((long long)zeros) - 1 : se + 1;
          const uint64_t below = t >= 64 ? ~0ull : ((1ull << t) - 1);
          refine_corrections(r, c, hist & below & (~0ull << k), p1, m1);
          k = t;
          if (value != 0) {
            if (k > 63) {
              atomicCAS(error, 0, 1);
              return;
            }
            c[k] = value;
          }
          k++;
        }
      }
      if (eobrun > 0) {
        if (k <= se) refine_corrections(r, c, hist & (~0ull << k), p1, m1);
        eobrun--;
      }
      int4* dst = reinterpret_cast<int4*>(blk);
#pragma unroll
      for (int g = 0; g < 8; g++) dst[g] = crow[g];
    }
  }
}

struct HostComp {
  uint8_t id;
  int h, v, tq, bw, bh, real_bw, real_bh;
  bool snap = false;
  uint16_t snapq[64];
};

struct HostScan {
  ScanDesc sd;
  Tables tables;
  std::vector<Segment> segs;
  std::vector<uint8_t> bytes;  // destuffed segments
};

struct Parsed {
  int width = 0, height = 0;
  bool progressive = false;
  std::vector<HostComp> comps;
  std::vector<HostScan> scans;
  uint8_t qt8[4][64];
  int present[4] = {0, 0, 0, 0};
  int tq[3] = {0, 0, 0};
};

// Destuffed bytes of one segment starting at `pos`: until the first 0xFF not followed by 0x00 (or the end).
// Returns the position of that 0xFF (or len).
size_t destuff(const uint8_t* d, size_t len, size_t pos, std::vector<uint8_t>& out) {
  for (;;) {
    const void* f = pos < len ? std::memchr(d + pos, 0xFF, len - pos) : nullptr;
    const size_t ff = f ? (size_t)((const uint8_t*)f - d) : len;
    out.insert(out.end(), d + pos, d + ff);
    if (ff >= len) return len;
    if (ff + 1 < len && d[ff + 1] == 0) {
      out.push_back(0xFF);
      pos = ff + 2;
      continue;
    }
    return ff;
  }
}

int fail_parse(rcg_ctx* ctx, int status, const char* msg) { return fail(ctx, status, msg); }

// The host part of parse() (decode.rs:622-697, :906-1103) for sequential and progressive Huffman frames.
int parse_jpeg(rcg_ctx* ctx, const uint8_t* d, size_t len, Parsed& P) {
  if (len < 4 || d[0] != 0xFF || d[1] != 0xD8) return fail_parse(ctx, RCG_INVALID, "not a JPEG file");
  size_t pos = 2;
  bool has_qt[4] = {false, false, false, false};
  uint16_t qt[4][64];
  bool has_dc[4] = {false, false, false, false}, has_ac[4] = {false, false, false, false};
  DevHuff dct[4], act[4];
  int hmax = 1, vmax = 1, mcus_x = 0, mcus_y = 0;
  size_t ri = 0;
  int adobe = -1;
  for (;;) {
    while (pos < len && d[pos] != 0xFF) pos++;
    while (pos < len && d[pos] == 0xFF) pos++;
    if (pos >= len) return fail_parse(ctx, RCG_INVALID, "unexpected end of JPEG");
    const uint8_t m = d[pos++];
    if (m == 0 || (m >= 0xD0 && m <= 0xD7) || m == 0x01) continue;
    if (m == 0xD9) break;
    if (pos + 2 > len) return fail_parse(ctx, RCG_INVALID, "unexpected end of JPEG");
    const size_t slen = ((size_t)d[pos] << 8) | d[pos + 1];
    if (slen < 2 || pos + slen > len) {
      if (!P.scans.empty()) break;
      return fail_parse(ctx, RCG_INVALID, "truncated JPEG segment");
    }
    const uint8_t* b = d + pos + 2;
    size_t bl = slen - 2;
    pos += slen;
    if (m == 0xDB) {
      while (bl > 0) {
        const int pq = b[0] >> 4, t = b[0] & 15;
        if (t > 3 || pq > 1) return fail_parse(ctx, RCG_INVALID, "bad DQT");
        const size_t need = 1 + 64 * (size_t)(pq + 1);
        if (bl < need) return fail_parse(ctx, RCG_INVALID, "truncated DQT");
        for (int k = 0; k < 64; k++)
          qt[t][kZigzag[k]] = pq == 0 ? b[1 + k] : (uint16_t)((b[1 + 2 * k] << 8) | b[2 + 2 * k]);
        has_qt[t] = true;
        b += need;
        bl -= need;
      }
    } else if (m == 0xC4) {
      while (bl > 0) {
        if (bl < 17) return fail_parse(ctx, RCG_INVALID, "truncated DHT");
        const int tc = b[0] >> 4, th = b[0] & 15;
        if (tc > 1 || th > 3) return fail_parse(ctx, RCG_INVALID, "bad DHT");
        size_t total = 0;
        for (int i = 0; i < 16; i++) total += b[1 + i];
        if (bl < 17 + total) return fail_parse(ctx, RCG_INVALID, "truncated DHT");
        if (!build_huff(b + 1, b + 17, total, tc == 0 ? &dct[th] : &act[th]))
          return fail_parse(ctx, RCG_INVALID, "bad JPEG huffman table");
        (tc == 0 ? has_dc : has_ac)[th] = true;
        b += 17 + total;
        bl -= 17 + total;
      }
    } else if (m == 0xC0 || m == 0xC1 || m == 0xC2) {
      if (!P.comps.empty()) return fail_parse(ctx, RCG_INVALID, "multiple SOF markers");
      P.progressive = m == 0xC2;
      if (bl < 6) return fail_parse(ctx, RCG_INVALID, "bad SOF");
      if (b[0] != 8) return fail_parse(ctx, RCG_UNSUPPORTED, "only 8-bit JPEGs are decoded on the GPU");
      P.height = (b[1] << 8) | b[2];
      P.width = (b[3] << 8) | b[4];
      const int nc = b[5];
      if (P.width == 0 || P.height == 0) return fail_parse(ctx, RCG_INVALID, "zero JPEG dimension (DNL not supported)");
      if ((unsigned long long)P.width * (unsigned long long)P.height > kMaxPixels)
        return fail_parse(ctx, RCG_INVALID, "unreasonable image dimensions");
      if (nc != 1 && nc != 3) return fail_parse(ctx, RCG_UNSUPPORTED, "only 1- or 3-component JPEGs are decoded");
      if (bl < 6 + 3 * (size_t)nc) return fail_parse(ctx, RCG_INVALID, "bad SOF");
      for (int i = 0; i < nc; i++) {
        const uint8_t* c = b + 6 + 3 * i;
        const int hs = c[1] >> 4, vs = c[1] & 15;
        if (hs < 1 || hs > 4 || vs < 1 || vs > 4 || c[2] > 3)
          return fail_parse(ctx, RCG_INVALID, "bad component description");
        HostComp hc;
        hc.id = c[0];
        hc.h = nc == 1 ? 1 : hs;
        hc.v = nc == 1 ? 1 : vs;
        hc.tq = c[2];
        P.comps.push_back(hc);
      }
      for (auto& c : P.comps) {
        hmax = std::max(hmax, c.h);
        vmax = std::max(vmax, c.v);
      }
      mcus_x = (P.width + 8 * hmax - 1) / (8 * hmax);
      mcus_y = (P.height + 8 * vmax - 1) / (8 * vmax);
      for (auto& c : P.comps) {
        c.bw = mcus_x * c.h;
        c.bh = mcus_y * c.v;
        c.real_bw = ((P.width * c.h + hmax - 1) / hmax + 7) / 8;
        c.real_bh = ((P.height * c.v + vmax - 1) / vmax + 7) / 8;
      }
    } else if ((m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) || m == 0xDE || m == 0xDF) {
      return fail_parse(ctx, RCG_UNSUPPORTED, "lossless, hierarchical and arithmetic JPEGs are decoded on the host");
    } else if (m == 0xDD) {
      if (bl < 2) return fail_parse(ctx, RCG_INVALID, "bad DRI");
      ri = ((size_t)b[0] << 8) | b[1];
    } else if (m == 0xEE && bl >= 12 && std::memcmp(b, "Adobe", 5) == 0) {
      adobe = b[11];
    } else if (m == 0xDA) {
      if (P.scans.size() >= kMaxScans) return fail_parse(ctx, RCG_UNSUPPORTED, "too many scans in a JPEG frame");
      if (P.comps.empty()) return fail_parse(ctx, RCG_INVALID, "SOS before SOF");
      if (bl < 1) return fail_parse(ctx, RCG_INVALID, "bad SOS");
      const int ns = b[0];
      if (ns == 0 || ns > (int)P.comps.size() || bl < 1 + 2 * (size_t)ns + 3)
        return fail_parse(ctx, RCG_INVALID, "bad SOS");
      HostScan sc;
      std::memset(&sc.sd, 0, sizeof sc.sd);
      std::memset(&sc.tables, 0, sizeof sc.tables);
      sc.sd.ns = ns;
      for (int i = 0; i < ns; i++) {
        const uint8_t cid = b[1 + 2 * i], t = b[2 + 2 * i];
        int k = -1;
        for (size_t j = 0; j < P.comps.size(); j++)
          if (P.comps[j].id == cid) {
            k = (int)j;
            break;
          }
        if (k < 0) return fail_parse(ctx, RCG_INVALID, "SOS references unknown component");
        for (int j = 0; j < i; j++)
          if (sc.sd.comp[j] == k) return fail_parse(ctx, RCG_INVALID, "duplicate component in scan");
        sc.sd.comp[i] = k;
        sc.sd.dc[i] = (t >> 4) & 3;
        sc.sd.ac[i] = (t & 15) & 3;
      }
      // Scan parameters (decode.rs:1084-1096): the spectral band and successive approximation of a progressive scan.
      const uint8_t* tp = b + 1 + 2 * ns;
      sc.sd.ss = 0;
      sc.sd.se = 63;
      if (P.progressive) {
        sc.sd.ss = tp[0];
        sc.sd.se = tp[1];
        sc.sd.ah = tp[2] >> 4;
        sc.sd.al = tp[2] & 15;
        if (sc.sd.ss > sc.sd.se || sc.sd.se > 63 || sc.sd.al > 13 || (sc.sd.ss == 0 && sc.sd.se != 0) ||
            (sc.sd.ss > 0 && ns != 1))
          return fail_parse(ctx, RCG_INVALID, "bad progressive scan parameters");
        sc.sd.kind = sc.sd.ss == 0 ? (sc.sd.ah == 0 ? kDcFirst : kDcRefine) : (sc.sd.ah == 0 ? kAcFirst : kAcRefine);
      } else {
        sc.sd.kind = kSeq;
      }
      sc.sd.k0 = sc.sd.ss;
      // The tables the scan decodes with (decode.rs:1240-1248).
      const bool need_dc = sc.sd.kind == kSeq || sc.sd.kind == kDcFirst;
      const bool need_ac = sc.sd.kind == kSeq || sc.sd.ss > 0;
      for (int i = 0; i < ns; i++) {
        HostComp& c = P.comps[sc.sd.comp[i]];
        if (!c.snap && has_qt[c.tq]) {
          std::memcpy(c.snapq, qt[c.tq], sizeof c.snapq);
          c.snap = true;
        }
        if ((need_dc && !has_dc[sc.sd.dc[i]]) || (need_ac && !has_ac[sc.sd.ac[i]]))
          return fail_parse(ctx, RCG_INVALID, "scan uses undefined huffman table");
        if (has_dc[sc.sd.dc[i]]) sc.tables.dc[sc.sd.dc[i]] = dct[sc.sd.dc[i]];
        if (has_ac[sc.sd.ac[i]]) sc.tables.ac[sc.sd.ac[i]] = act[sc.sd.ac[i]];
      }
      // MCU pattern and geometry (decode.rs:1251-1258, :1270-1275)
      const bool inter = ns > 1;
      int bm = 0;
      for (int i = 0; i < ns; i++) {
        const HostComp& c = P.comps[sc.sd.comp[i]];
        const int bh = inter ? c.h : 1, bv = inter ? c.v : 1;
        for (int by = 0; by < bv; by++)
          for (int bx = 0; bx < bh; bx++) {
            if (bm >= kMaxMcuBlocks) return fail_parse(ctx, RCG_UNSUPPORTED, "MCU too large");
            sc.sd.mcu_si[bm] = i;
            sc.sd.mcu_dy[bm] = by;
            sc.sd.mcu_dx[bm] = bx;
            bm++;
          }
      }
      sc.sd.bmcu = bm;
      const long long nx = inter ? mcus_x : P.comps[sc.sd.comp[0]].real_bw;
      const long long ny = inter ? mcus_y : P.comps[sc.sd.comp[0]].real_bh;
      sc.sd.mcus_x = (int)nx;
      const long long total = nx * ny;
      // Restart segments as the bit reader sees them (decode.rs:90-114): each ends at the first 0xFF not followed
      // by 0x00; the next starts past an RSTn found there, else it (and every later one) reads zero bits.
      const long long seg_mcus = ri > 0 ? (long long)ri : total;
      const long long nseg = (total + seg_mcus - 1) / seg_mcus;
      size_t p = pos;
      bool dead = false;
      long long sub = 0, span = 0;
      for (long long s = 0; s < nseg; s++) {
        Segment g;
        g.byte0 = (long long)sc.bytes.size();
        g.block0 = s * seg_mcus * bm;
        g.nblocks = std::min(seg_mcus, total - s * seg_mcus) * bm;
        if (s > 0 && !dead) {
          // restart(): past an RSTn at p, else stay (a different marker: zero bits from here on)
          if (p + 1 < len && d[p] == 0xFF && d[p + 1] >= 0xD0 && d[p + 1] <= 0xD7)
            p += 2;
          else
            dead = true;
        }
        if (!dead) p = destuff(d, len, p, sc.bytes);
        g.nbytes = (long long)sc.bytes.size() - g.byte0;
        g.nsub = (int)std::max<long long>(1, (g.nbytes * 8 + kSubBits - 1) / kSubBits);
        g.sub0 = sub;
        sub += g.nsub;
        g.nspan = (g.nsub + kSpanSubs - 1) / kSpanSubs;
        g.span0 = span;
        span += g.nspan;
        sc.segs.push_back(g);
        // keep segments 4-byte aligned in the buffer
        while (sc.bytes.size() % 4) sc.bytes.push_back(0);
      }
      sc.sd.nseg = (int)nseg;
      sc.sd.nsub = sub;
      sc.sd.nspan = span;
      pos = p;  // the marker search resumes where the entropy data stopped (decode.rs:1100-1101)
      P.scans.push_back(std::move(sc));
    }
  }
  if (P.scans.empty() || P.comps.empty()) return fail_parse(ctx, RCG_INVALID, "JPEG contains no image data");
  // into_coefs (decode.rs:540-570)
  if (P.comps.size() == 3 && (adobe == 0 || (adobe < 0 && P.comps[0].id == 'R' && P.comps[1].id == 'G' &&
                                             P.comps[2].id == 'B')))
    return fail_parse(ctx, RCG_UNSUPPORTED, "RGB-coded JPEG");
  for (size_t i = 0; i < P.comps.size(); i++) {
    const HostComp& c = P.comps[i];
    const uint16_t* t = c.snap ? c.snapq : (has_qt[c.tq] ? qt[c.tq] : nullptr);
    if (!t) return fail_parse(ctx, RCG_INVALID, "missing quantization table");
    for (int n = 0; n < 64; n++)
      if (t[n] > 255 || t[n] == 0) return fail_parse(ctx, RCG_UNSUPPORTED, "16-bit quantization table");
    for (int n = 0; n < 64; n++) P.qt8[c.tq][n] = (uint8_t)t[n];
    P.present[c.tq] = 1;
    P.tq[i] = c.tq;
  }
  return RCG_OK;
}

}  // namespace

int jpeg_decode(rcg_ctx* ctx, const uint8_t* data, size_t len, rcg_jpeg_info* info, rcg_coef_layout* layout,
                rcg_qtables* tables, int16_t* coefs, size_t coefs_len, bool coefs_on_device) {
  Parsed P;
  int rc = parse_jpeg(ctx, data, len, P);
  if (rc != RCG_OK) return rc;
  const int nc = (int)P.comps.size();
  std::memset(layout, 0, sizeof *layout);
  layout->ncomp = nc;
  long long nblocks = 0;
  CompDesc fc[3];
  std::memset(fc, 0, sizeof fc);
  for (int i = 0; i < nc; i++) {
    const HostComp& c = P.comps[i];
    layout->h[i] = c.h;
    layout->v[i] = c.v;
    layout->blocks_w[i] = c.bw;
    layout->blocks_h[i] = c.bh;
    fc[i].bw = c.bw;
    fc[i].bh = c.bh;
    fc[i].h = c.h;
    fc[i].v = c.v;
    fc[i].cls = i == 0 ? 0 : 1;
    fc[i].blk0 = nblocks;
    nblocks += (long long)c.bw * c.bh;
  }
  layout->ncoefs = nblocks * 64;
  if (info) {
    std::memset(info, 0, sizeof *info);
    info->width = (uint32_t)P.width;
    info->height = (uint32_t)P.height;
    for (int i = 0; i < nc; i++) info->ids[i] = P.comps[i].id;
    info->scans = (int)P.scans.size();
  }
  if (tables) {
    std::memset(tables, 0, sizeof *tables);
    for (int i = 0; i < nc; i++) tables->tq[i] = P.tq[i];
    for (int s = 0; s < 4; s++) {
      tables->present[s] = P.present[s];
      if (P.present[s]) std::memcpy(tables->qtables[s], P.qt8[s], 64);
    }
  }
  if (!coefs) return RCG_OK;
  if ((long long)coefs_len < nblocks * 64) return fail(ctx, RCG_INVALID, "coefficient buffer too short");
  cudaSetDevice(ctx->device);
  // The kernels move whole blocks with 16-byte accesses: a caller buffer that is not 16-byte aligned gets the
  // coefficients through the context's own buffer and one device copy.
  const bool direct = coefs_on_device && ((uintptr_t)coefs & 15) == 0;
  int16_t* d_out = direct ? coefs : (int16_t*)workspace(ctx, "dec_coefs", (size_t)nblocks * 128);
  int* d_err = (int*)workspace(ctx, "dec_error", sizeof(int) * 4);
  ScanDesc* d_sd = (ScanDesc*)workspace(ctx, "dec_scan", sizeof(ScanDesc));
  Tables* d_tab = (Tables*)workspace(ctx, "dec_tables", sizeof(Tables));
  if (!d_out || !d_err || !d_sd || !d_tab) return RCG_NO_MEMORY;
  cudaMemsetAsync(d_out, 0, (size_t)nblocks * 128, ctx->stream);
  cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream);
  int h_changed = 0;
  int rounds_max = 0;
  bool fell_back = false;
  for (HostScan& sc : P.scans) {
    std::memcpy(sc.sd.fc, fc, sizeof fc);
    const long long nsub = sc.sd.nsub, nspan = sc.sd.nspan;
    // Padded: a CTA's shared-memory window covers whole units plus kTail bytes, rounded up to 16, so it may run up
    // to one span (256 B) + kTail + 15 bytes past the last segment's data.
    uint8_t* d_bytes = (uint8_t*)workspace(ctx, "dec_bytes", sc.bytes.size() + 1024);
    Segment* d_segs = (Segment*)workspace(ctx, "dec_segs", sizeof(Segment) * sc.segs.size());
    SubState* d_s0 = (SubState*)workspace(ctx, "dec_state0", sizeof(SubState) * (size_t)nspan);
    SubState* d_s1 = (SubState*)workspace(ctx, "dec_state1", sizeof(SubState) * (size_t)nspan);
    SubState* d_piece = (SubState*)workspace(ctx, "dec_pieces", sizeof(SubState) * (size_t)nsub);
    SubCount* d_cnt = (SubCount*)workspace(ctx, "dec_counts", sizeof(SubCount) * (size_t)nsub);
    SubCount* d_base = (SubCount*)workspace(ctx, "dec_base", sizeof(SubCount) * (size_t)nsub);
    int* d_changed = (int*)workspace(ctx, "dec_changed", sizeof(int));
    if (!d_bytes || !d_segs || !d_s0 || !d_s1 || !d_piece || !d_cnt || !d_base || !d_changed) return RCG_NO_MEMORY;
    if (!sc.bytes.empty() && (rc = copy_to_device(ctx, d_bytes, sc.bytes.data(), sc.bytes.size())) != RCG_OK)
      return rc;
    cudaMemcpyAsync(d_segs, sc.segs.data(), sizeof(Segment) * sc.segs.size(), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(d_sd, &sc.sd, sizeof(ScanDesc), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(d_tab, &sc.tables, sizeof(Tables), cudaMemcpyHostToDevice, ctx->stream);
    if (sc.sd.kind == kDcRefine) {
      long long nb = 0;
      for (const Segment& g : sc.segs) nb = std::max(nb, g.block0 + g.nblocks);
      if (nb > 0)
        RCG_LAUNCH(ctx, "dc_refine", k_dc_refine, (unsigned)((nb + 255) / 256), 256, 0, d_sd, d_segs, d_bytes, nb,
                   d_out);
      continue;
    }
    if (sc.sd.kind == kAcRefine) {
      RCG_LAUNCH(ctx, "ac_refine", k_ac_refine, (unsigned)((sc.sd.nseg + kRefineThreads - 1) / kRefineThreads),
                 kRefineThreads, 0, d_sd, d_tab, d_segs, d_bytes, d_out, d_err);
      continue;
    }
    // Initial guesses: every span starts at its first bit, first block of the MCU, at a block's first coefficient.
    std::vector<SubState> init((size_t)nspan);
    for (const Segment& g : sc.segs)
      for (int i = 0; i < g.nspan; i++)
        init[g.span0 + i] = SubState{(long long)i * kSpanSubs * kSubBits, 0, sc.sd.k0};
    cudaMemcpyAsync(d_s0, init.data(), sizeof(SubState) * (size_t)nspan, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(d_cnt, 0, sizeof(SubCount) * (size_t)nsub, ctx->stream);
    const unsigned grid_span = (unsigned)((nspan + kDecThreads - 1) / kDecThreads);
    const unsigned grid = (unsigned)((nsub + kDecThreads - 1) / kDecThreads);
    SubState* cur = d_s0;
    SubState* nxt = d_s1;
    bool settled = false;
    int round = 0;
    while (round < kMaxRounds) {
      // A few rounds back to back (most streams settle within them), then one round per check: the check of a
      // batch looks at its last round only, which changes nothing exactly when the states have settled.
      const int batch = round == 0 ? kFirstBatch : 1;
      for (int b = 0; b < batch; b++, round++) {
        if (b == batch - 1) cudaMemsetAsync(d_changed, 0, sizeof(int), ctx->stream);
        RCG_LAUNCH(ctx, "seq_sync", k_seq_sync, grid_span, kDecThreads, 0, d_sd, d_tab, d_segs, d_bytes, cur, nxt,
                   d_piece, d_cnt, d_changed);
        std::swap(cur, nxt);
      }
      cudaMemcpyAsync(&h_changed, d_changed, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "JPEG decode");
      if (!h_changed) {
        settled = true;
        break;
      }
    }
    if (settled)
      rounds_max = std::max(rounds_max, round);
    else
      fell_back = true;
    if (!settled) {
      RCG_LAUNCH(ctx, "seq_chain", k_seq_chain, (unsigned)std::min<long long>((sc.sd.nseg + 127) / 128, 1024), 128, 0,
                 d_sd, d_tab, d_segs, d_bytes, d_piece, d_cnt);
    }
    RCG_LAUNCH(ctx, "seq_prefix", k_seq_prefix, (unsigned)std::min(sc.sd.nseg, 1024), 1024, 0, d_sd, d_segs, d_cnt,
               d_base);
    RCG_LAUNCH(ctx, "seq_write", k_seq_write, grid, kDecThreads, 0, d_sd, d_tab, d_segs, d_bytes, d_piece, d_base,
               d_out, d_err);
  }
  int h_err = 0;
  cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "JPEG decode");
  if (h_err) return fail(ctx, RCG_INVALID, h_err == 1 ? "bad JPEG entropy-coded data" : "JPEG decode lost its place");
  if (info) info->sync_rounds = fell_back ? -1 : rounds_max;
  if (!coefs_on_device) return copy_to_host(ctx, coefs, d_out, (size_t)nblocks * 128);
  if (!direct) {
    e = cudaMemcpyAsync(coefs, d_out, (size_t)nblocks * 128, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "JPEG decode output copy");
  }
  return RCG_OK;
}

}  // namespace rcg
