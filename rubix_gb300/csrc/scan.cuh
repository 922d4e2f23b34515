// Single-block exclusive scan used by the setup passes of several kernels.
#pragma once

#include "common.cuh"

namespace rubix {
namespace {

// Exclusive scan of `count` ints in place by one block of 1024 threads; the grand
// total is written to data[count] when `with_total` is set (data has count+1 slots).
__global__ void __launch_bounds__(1024)
scan_exclusive_1block(int* __restrict__ data, long long count, int with_total) {
  __shared__ long long s_part[1024];
  const int t = threadIdx.x;
  const long long per = (count + 1023) / 1024;
  const long long b = t * per;
  const long long e = b + per < count ? b + per : count;
  long long sum = 0;
  for (long long i = b; i < e; ++i) sum += data[i];
  s_part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    long long v = (t >= off) ? s_part[t - off] : 0;
    __syncthreads();
    s_part[t] += v;
    __syncthreads();
  }
  long long run = (t == 0) ? 0 : s_part[t - 1];
  for (long long i = b; i < e; ++i) {
    int v = data[i];
    data[i] = (int)run;
    run += v;
  }
  if (with_total && t == 1023) data[count] = (int)s_part[1023];
}

}  // namespace
}  // namespace rubix
