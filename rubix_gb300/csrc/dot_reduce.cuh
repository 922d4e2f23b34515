// Deterministic cross-block reduction of a fused dot product: every block sums its
// threads' float partials in double (fixed shuffle tree, then warps in order), writes
// the block sum to the scratch, and the last block to finish adds the block sums up in
// block order.  The host zeroes the scratch's counter before each launch.
#pragma once

#include "common.cuh"

namespace rubix {

constexpr int kFusedDotMaxBlocks = 8192;

struct FusedDotScratch {
  double partial[kFusedDotMaxBlocks];
  unsigned counter;
};

// Block sum of v (blockDim.x a multiple of 32, at most 1024 threads); valid in thread 0.
__device__ __forceinline__ double fused_block_sum(double v, double* s_w) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();  // s_w free from any earlier use
  if (lane == 0) s_w[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_w[w];
  return t;
}

// Every thread of every block calls this once with its partial sum; the block index is
// the linear one of a 1-D or 2-D grid.  s_w: blockDim.x / 32 doubles of shared memory.
__device__ __forceinline__ void fused_dot_finish(float partial, FusedDotScratch* ws, double* out,
                                                 double* s_w, int* s_last) {
  const int nblk = gridDim.x * gridDim.y;
  const int b = blockIdx.y * gridDim.x + blockIdx.x;
  const double t = fused_block_sum((double)partial, s_w);
  if (threadIdx.x == 0) {
    ws->partial[b] = t;
    __threadfence();
    *s_last = atomicAdd(&ws->counter, 1u) == (unsigned)nblk - 1u;
  }
  __syncthreads();
  if (!*s_last) return;
  __threadfence();
  double v = 0.0;
  for (int k = threadIdx.x; k < nblk; k += blockDim.x) v += __ldcg(&ws->partial[k]);
  const double total = fused_block_sum(v, s_w);
  if (threadIdx.x == 0) {
    *out = total;
  }
}

}  // namespace rubix
