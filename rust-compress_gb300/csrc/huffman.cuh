// Length-limited Huffman code lengths for one CTA (core/src/util/huffman.rs:10-86, build_lengths with max_len 16)
// over 257 symbols: the 256 real symbols plus the dummy symbol of frequency 1 that optimal_table adds
// (jpeg/src/encode.rs:241-244). The sort is a parallel rank sort on the unique keys (freq, reverse symbol); the
// two-queue merge, the depth pass and the Kraft fix-up are sequential, as in the reference.
#pragma once

namespace rcg {

constexpr int kHuffSyms = 257;

struct HuffScratch {
  int order[kHuffSyms];  // sorted position -> symbol
  unsigned long long weight[2 * kHuffSyms];
  int parent[2 * kHuffSyms];
  unsigned char depth[2 * kHuffSyms];
  int count[17];
  int n_used;
};

// freq: 257 counts in shared memory (freq[256] = 1); lens: 257 code lengths out (0 = unused), shared memory.
// Every thread of the CTA calls it; the CTA has at least 257 threads.
__device__ inline void huff_lengths(const unsigned* freq, unsigned char* lens, HuffScratch& s) {
  const int t = threadIdx.x;
  if (t < kHuffSyms) lens[t] = 0;
  if (t == 0) s.n_used = 0;
  __syncthreads();
  if (t < kHuffSyms && freq[t] > 0) {
    unsigned f = freq[t];
    int r = 0;
    for (int j = 0; j < kHuffSyms; j++) {
      unsigned g = freq[j];
      if (g > 0 && (g < f || (g == f && j > t))) r++;
    }
    s.order[r] = t;
    atomicAdd(&s.n_used, 1);
  }
  __syncthreads();
  const int n = s.n_used;
  if (t == 0) {
    if (n == 1) {
      lens[s.order[0]] = 1;
    } else if (n > 1) {
      for (int i = 0; i < n; i++) s.weight[i] = freq[s.order[i]];
      int leaf = 0, node = n, next = n;
      while (next < 2 * n - 1) {
        int ab[2];
        for (int p = 0; p < 2; p++) {
          if (leaf < n && (node >= next || s.weight[leaf] <= s.weight[node]))
            ab[p] = leaf++;
          else
            ab[p] = node++;
        }
        s.weight[next] = s.weight[ab[0]] + s.weight[ab[1]];
        s.parent[ab[0]] = next;
        s.parent[ab[1]] = next;
        next++;
      }
      s.depth[2 * n - 2] = 0;
      for (int i = 2 * n - 3; i >= 0; i--) s.depth[i] = (unsigned char)(s.depth[s.parent[i]] + 1);
      for (int l = 0; l <= 16; l++) s.count[l] = 0;
      for (int i = 0; i < n; i++) s.count[min((int)s.depth[i], 16)] += 1;
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
      int idx = 0;
      for (int l = 16; l >= 1; l--)
        for (int c = 0; c < s.count[l]; c++) lens[s.order[idx++]] = (unsigned char)l;
    }
  }
  __syncthreads();
}

}  // namespace rcg
