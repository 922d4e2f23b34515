// Stable LSD radix sort of (32-bit key, int value) pairs, 8 bits per pass, written
// from the published LSD scheme: per pass, a per-tile digit histogram, one exclusive
// scan over (digit, tile), and a stable scatter in which each tile ranks its keys with
// warp-level match/popc and per-warp digit counters, reorders them by digit in shared
// memory and writes each digit's run with consecutive threads on consecutive addresses
// (coalesced stores instead of one scattered store per key).  Deterministic.
#pragma once

#include "common.cuh"
#include "scan.cuh"

namespace rubix {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // keys per tile
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;

// Per-tile histogram of one digit; hist is digit-major: hist[d * n_tiles + tile].
__global__ void __launch_bounds__(kSortThreads)
radix_hist_kernel(const unsigned* __restrict__ keys, long long n, int shift,
                  unsigned digit_mask, int n_tiles, int* __restrict__ hist) {
  __shared__ int s_hist[kRadix];
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) s_hist[d] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kSortTile;
  for (int it = 0; it < kSortItems; ++it) {
    long long e = base + it * kSortThreads + threadIdx.x;
    if (e < n) atomicAdd(&s_hist[(keys[e] >> shift) & digit_mask], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d <= (int)digit_mask; d += blockDim.x)
    hist[(long long)d * n_tiles + blockIdx.x] = s_hist[d];
}

// Stable scatter of one digit pass.  Warp w of the tile owns the contiguous keys
// [base + w*512, base + (w+1)*512) and walks them in 16 rounds of 32, so
// (warp, round, lane) order equals input order.
// One block per digit: the exclusive scan of the digit's row of tile counts, in place,
// and the row total (the digits' offsets are added by the scatter).
__global__ void __launch_bounds__(kSortThreads)
radix_rowscan_kernel(int* __restrict__ hist, int n_tiles, int* __restrict__ totals) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ int s_warp[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* row = hist + (long long)blockIdx.x * n_tiles;
  int carry = 0;
  for (int base = 0; base < n_tiles; base += kSortThreads) {
    const int t = base + threadIdx.x;
    const int v = t < n_tiles ? row[t] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    int before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      const int ws = s_warp[w];
      before += w < warp ? ws : 0;
      all += ws;
    }
    if (t < n_tiles) row[t] = carry + before + x - v;
    carry += all;
    __syncthreads();  // s_warp is rewritten by the next chunk
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads)
radix_scatter_kernel(const unsigned* __restrict__ keys_in, const int* __restrict__ vals_in,
                     unsigned* __restrict__ keys_out, int* __restrict__ vals_out, long long n,
                     int shift, unsigned digit_mask, int n_tiles,
                     const int* __restrict__ hist_scanned, const int* __restrict__ totals) {
  constexpr int kWarps = kSortThreads / 32;
  static_assert(kSortThreads == kRadix, "one thread per digit for the digit offsets");
  __shared__ int s_cnt[kWarps][kRadix];
  __shared__ int s_base[kRadix];
  __shared__ int s_dw[kWarps];
  __shared__ int s_tstart[kRadix];  // start of digit d in the tile's digit-ordered copy
  __shared__ unsigned s_k[kSortTile];
  __shared__ int s_v[kSortTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kWarps * kRadix; i += kSortThreads) (&s_cnt[0][0])[i] = 0;
  const int n_digits = (int)digit_mask + 1;
  {
    // offset of digit d: the totals of the digits below it (exclusive block scan), plus
    // this tile's position in d's row (already scanned)
    const int d = threadIdx.x;
    const int v = d < n_digits ? totals[d] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_dw[warp] = x;
    __syncthreads();
    int before = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) before += w < warp ? s_dw[w] : 0;
    if (d < n_digits)
      s_base[d] = before + x - v + hist_scanned[(long long)d * n_tiles + blockIdx.x];
  }
  __syncthreads();

  const long long wbase = (long long)blockIdx.x * kSortTile + (long long)warp * (32 * kSortItems);
  const unsigned lt_mask = (1u << lane) - 1u;
  unsigned key[kSortItems];
  int val[kSortItems];
  int rank[kSortItems];
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    long long e = wbase + r * 32 + lane;
    bool valid = e < n;
    key[r] = valid ? keys_in[e] : 0u;
    val[r] = valid ? vals_in[e] : 0;
    int d = valid ? (int)((key[r] >> shift) & digit_mask) : kRadix;  // kRadix: own group
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int before = valid ? s_cnt[warp][d] : 0;
    rank[r] = before + __popc(peers & lt_mask);
    __syncwarp();
    if (valid && (peers & lt_mask) == 0) s_cnt[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // Exclusive prefix over warps, per digit (one digit per thread), and the tile's count
  // of each digit, scanned over the digits into the digit's start in the tile.
  {
    const int d = threadIdx.x;
    int run = 0;
    if (d < n_digits) {
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        int c = s_cnt[w][d];
        s_cnt[w][d] = run;
        run += c;
      }
    }
    int x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_dw[warp] = x;
    __syncthreads();
    int before = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) before += w < warp ? s_dw[w] : 0;
    s_tstart[d] = before + x - run;
  }
  __syncthreads();
  // the tile in (digit, original position) order in shared memory
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    long long e = wbase + r * 32 + lane;
    if (e < n) {
      int d = (int)((key[r] >> shift) & digit_mask);
      const int lpos = s_tstart[d] + s_cnt[warp][d] + rank[r];
      s_k[lpos] = key[r];
      s_v[lpos] = val[r];
    }
  }
  __syncthreads();
  // each digit's run to its place: consecutive threads, consecutive addresses
  const long long tile0 = (long long)blockIdx.x * kSortTile;
  const int tile_n = (int)min((long long)kSortTile, n - tile0);
  for (int i = threadIdx.x; i < tile_n; i += kSortThreads) {
    const unsigned k = s_k[i];
    const int d = (int)((k >> shift) & digit_mask);
    const long long pos = (long long)s_base[d] + (i - s_tstart[d]);
    keys_out[pos] = k;
    vals_out[pos] = s_v[i];
  }
}

inline long long radix_tiles(long long n) {
  const long long t = (n + kSortTile - 1) / kSortTile;
  return t < 1 ? 1 : t;
}

// Ints of the histogram workspace of a sort of n keys: [digit][tile] counts, then the
// kRadix digit totals.
inline long long radix_hist_ints(long long n) { return (long long)kRadix * (radix_tiles(n) + 1); }

// Sorts n pairs by bits [0, bits) of the keys, stably, ping-ponging between (k0, v0)
// and (k1, v1); `hist` holds radix_hist_ints(n) ints.  Returns 0 when the sorted
// pairs end in (k0, v0), 1 when in (k1, v1).  bits = 0 sorts nothing.
inline int radix_sort_pairs(unsigned* k0, int* v0, unsigned* k1, int* v1, long long n, int bits,
                            int* hist, cudaStream_t st) {  // hist: radix_hist_ints(n) ints
  const int n_tiles = (int)radix_tiles(n);
  unsigned* kin = k0;
  unsigned* kout = k1;
  int* vin = v0;
  int* vout = v1;
  int where = 0;
  for (int shift = 0; shift < bits; shift += kRadixBits) {
    const unsigned dmask = (unsigned)(kRadix - 1);
    int* totals = hist + (long long)kRadix * n_tiles;
    radix_hist_kernel<<<n_tiles, kSortThreads, 0, st>>>(kin, n, shift, dmask, n_tiles, hist);
    radix_rowscan_kernel<<<kRadix, kSortThreads, 0, st>>>(hist, n_tiles, totals);
    radix_scatter_kernel<<<n_tiles, kSortThreads, 0, st>>>(kin, vin, kout, vout, n, shift, dmask,
                                                           n_tiles, hist, totals);
    unsigned* tk = kin;
    kin = kout;
    kout = tk;
    int* tv = vin;
    vin = vout;
    vout = tv;
    where ^= 1;
  }
  return where;
}

}  // namespace
}  // namespace rubix
