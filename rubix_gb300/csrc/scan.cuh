// Single-block exclusive scan used by the setup passes of several kernels.
#pragma once

#include "common.cuh"

namespace rubix {
namespace {

// Exclusive scan of `count` ints in place by one block of 1024 threads, in tiles of
// 16384 (16 consecutive values per thread, warp-shuffle scans); `data` 16-byte aligned.
// The grand total is written to data[count] when `with_total` is set (data then has
// count+1 slots).
__device__ __forceinline__ void scan_exclusive_block(int* __restrict__ data, long long count,
                                                     int with_total);

__global__ void __launch_bounds__(1024)
scan_exclusive_1block(int* __restrict__ data, long long count, int with_total) {
  scan_exclusive_block(data, count, with_total);
}

// Three independent scans (with totals) in one launch: block b scans array b.
__global__ void __launch_bounds__(1024)
scan_exclusive_3(int* __restrict__ a, int* __restrict__ b, int* __restrict__ c, long long count) {
  scan_exclusive_block(blockIdx.x == 0 ? a : (blockIdx.x == 1 ? b : c), count, 1);
}

__device__ __forceinline__ void scan_exclusive_block(int* __restrict__ data, long long count,
                                                     int with_total) {
  // Tiles of 16384: thread t owns 16 consecutive values (four 16-byte loads when the
  // tile is full; data must be 16-byte aligned), warp-shuffle scans of the thread
  // sums, then of the 32 warp sums.
  constexpr int kPer = 16;
  constexpr long long kTileN = 1024LL * kPer;
  __shared__ int s_warp[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  long long carry = 0;
  for (long long base = 0; base < count; base += kTileN) {
    const long long i0 = base + (long long)kPer * t;
    int v[kPer];
    const bool full = i0 + kPer <= count;
    if (full) {
      const int4* src = reinterpret_cast<const int4*>(data + i0);
#pragma unroll
      for (int q = 0; q < kPer / 4; ++q) {
        const int4 x = src[q];
        v[4 * q] = x.x;
        v[4 * q + 1] = x.y;
        v[4 * q + 2] = x.z;
        v[4 * q + 3] = x.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < kPer; ++j) v[j] = (i0 + j < count) ? data[i0 + j] : 0;
    }
    int tsum = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) tsum += v[j];
    int x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    if (w == 0) {
      int ws = s_warp[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, ws, o);
        if (lane >= o) ws += y;
      }
      s_warp[lane] = ws;
    }
    __syncthreads();
    int run = (int)(carry + (x - tsum) + (w > 0 ? s_warp[w - 1] : 0));
    if (full) {
      int4* dst = reinterpret_cast<int4*>(data + i0);
#pragma unroll
      for (int q = 0; q < kPer / 4; ++q) {
        int4 o;
        o.x = run;
        run += v[4 * q];
        o.y = run;
        run += v[4 * q + 1];
        o.z = run;
        run += v[4 * q + 2];
        o.w = run;
        run += v[4 * q + 3];
        dst[q] = o;
      }
    } else {
#pragma unroll
      for (int j = 0; j < kPer; ++j) {
        if (i0 + j < count) data[i0 + j] = run;
        run += v[j];
      }
    }
    carry += s_warp[31];
    __syncthreads();
  }
  if (with_total && t == 0) data[count] = (int)carry;
}

}  // namespace
}  // namespace rubix
