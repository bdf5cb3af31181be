// Length-limited Huffman code lengths for one CTA (core/src/util/huffman.rs:10-86, build_lengths with max_len 16)
// over 257 symbols: the 256 real symbols plus the dummy symbol of frequency 1 that optimal_table adds
// (jpeg/src/encode.rs:241-244). The sort is a parallel rank sort on the unique keys (freq, reverse symbol); the
// two-queue merge and the Kraft fix-up are sequential, as in the reference; the leaf depths, the per-length counts
// and the final assignment are computed one thread per leaf, with the same results.
#pragma once

namespace rcg {

constexpr int kHuffSyms = 257;

struct HuffScratch {
  int order[kHuffSyms];  // sorted position -> symbol
  unsigned long long weight[2 * kHuffSyms];
  int parent[2 * kHuffSyms];
  int count[17];
  int n_used;
};

// freq: 257 counts in shared memory (freq[256] = 1); lens: 257 code lengths out (0 = unused), shared memory.
// Every thread of the CTA calls it; the CTA has at least 257 threads.
//
// The two-queue merge is the one sequential step: one thread, with the head of each queue and the element behind it
// held in registers so that a pick does not wait for a shared-memory load. The depth pass, the per-length counts
// and the final assignment run one thread per leaf / sorted position.
__device__ inline void huff_lengths(const unsigned* freq, unsigned char* lens, HuffScratch& s) {
  const int t = threadIdx.x;
  if (t < kHuffSyms) lens[t] = 0;
  if (t == 0) s.n_used = 0;
  if (t < 17) s.count[t] = 0;
  __syncthreads();
  if (t < kHuffSyms && freq[t] > 0) {
    unsigned f = freq[t];
    int r = 0;
    for (int j = 0; j < kHuffSyms; j++) {
      unsigned g = freq[j];
      if (g > 0 && (g < f || (g == f && j > t))) r++;
    }
    s.order[r] = t;
    s.weight[r] = f;
    atomicAdd(&s.n_used, 1);
  }
  __syncthreads();
  const int n = s.n_used;
  if (n == 1) {
    if (t == 0) lens[s.order[0]] = 1;
  } else if (n > 1) {
    if (t == 0) {
      // Leaves 0..n-1 ascending, internal nodes n.. in creation order; ties go to the leaf (huffman.rs:38-46).
      unsigned long long* W = s.weight;
      int leaf = 0, node = n, next = n;
      unsigned long long wl = W[0], wl1 = W[1], wn = 0, wn1 = 0;
      auto pick = [&](unsigned long long& w) -> int {
        if (leaf < n && (node >= next || wl <= wn)) {
          w = wl;
          wl = wl1;
          wl1 = leaf + 2 < n ? W[leaf + 2] : 0;
          return leaf++;
        }
        w = wn;
        wn = wn1;
        wn1 = node + 2 < next ? W[node + 2] : 0;
        return node++;
      };
      while (next < 2 * n - 1) {
        unsigned long long wa, wb;
        const int a = pick(wa);
        const int b = pick(wb);
        const unsigned long long sum = wa + wb;
        W[next] = sum;
        s.parent[a] = next;
        s.parent[b] = next;
        if (node == next)
          wn = sum;
        else if (node + 1 == next)
          wn1 = sum;
        next++;
      }
    }
    __syncthreads();
    // Depth of each leaf = its number of ancestors (the root is node 2n-2); counts per length, capped at 16.
    const int root = 2 * n - 2;
    if (t < n) {
      int d = 0;
      for (int j = t; j != root; j = s.parent[j]) d++;
      atomicAdd(&s.count[min(d, 16)], 1);
    }
    __syncthreads();
    if (t == 0) {
      // Kraft fix-up (huffman.rs:60-78): lengthen codes until the 16-bit limit holds.
      unsigned long long total = 0;
      for (int l = 1; l <= 16; l++) total += (unsigned long long)s.count[l] << (16 - l);
      while (total > (1ull << 16)) {
        s.count[16] -= 1;
        for (int l = 15; l >= 1; l--) {
          if (s.count[l] > 0) {
            s.count[l] -= 1;
            s.count[l + 1] += 2;
            break;
          }
        }
        total -= 1;
      }
    }
    __syncthreads();
    // Lengths 16, 15, .. 1 go to the sorted positions 0, 1, .. in turn (huffman.rs:80-85).
    if (t < n) {
      int start = 0, l = 16;
      while (l > 1 && t >= start + s.count[l]) start += s.count[l--];
      lens[s.order[t]] = (unsigned char)l;
    }
  }
  __syncthreads();
}

}  // namespace rcg
