// Deterministic dot product of two float arrays: a fixed grid of blocks, per-thread
// float partial sums (four independent chains), double block sums written to the
// workspace, and the last block to finish adding them up in block order.
#include "common.cuh"

namespace rubix {
namespace {

constexpr int kDotBlocks = 1024;
constexpr int kDotThreads = 256;

struct DotScratch {
  double partial[kDotBlocks];
  unsigned counter;
};

__device__ __forceinline__ double block_sum(double v, double* s_w) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) s_w[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kDotThreads / 32; ++w) t += s_w[w];
  return t;  // valid in thread 0
}

__global__ void __launch_bounds__(kDotThreads) dot_kernel(const float* __restrict__ a,
                                                          const float* __restrict__ b,
                                                          long long n, DotScratch* ws,
                                                          double* out) {
  __shared__ double s_w[kDotThreads / 32];
  __shared__ int s_last;
  const long long stride = (long long)gridDim.x * kDotThreads;
  float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
  long long i = (long long)blockIdx.x * kDotThreads + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    c0 = fmaf(a[i], b[i], c0);
    c1 = fmaf(a[i + stride], b[i + stride], c1);
    c2 = fmaf(a[i + 2 * stride], b[i + 2 * stride], c2);
    c3 = fmaf(a[i + 3 * stride], b[i + 3 * stride], c3);
  }
  for (; i < n; i += stride) c0 = fmaf(a[i], b[i], c0);
  const double t = block_sum(((double)c0 + (double)c1) + ((double)c2 + (double)c3), s_w);
  if (threadIdx.x == 0) {
    ws->partial[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(&ws->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double v = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += kDotThreads) v += __ldcg(&ws->partial[k]);
  __syncthreads();
  const double total = block_sum(v, s_w);
  if (threadIdx.x == 0) {
    *out = total;
    ws->counter = 0u;
  }
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" size_t rubix_dot_workspace_size(void) { return sizeof(DotScratch); }

extern "C" int rubix_dot(const float* a, const float* b, int64_t n, double* out, void* workspace,
                         size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n >= 0, RUBIX_E_SHAPE, "rubix_dot: n < 0");
  RUBIX_REQUIRE(out != nullptr, RUBIX_E_INVALID, "rubix_dot: null output");
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= sizeof(DotScratch) &&
                    (reinterpret_cast<uintptr_t>(workspace) & 7) == 0,
                RUBIX_E_WORKSPACE, "rubix_dot: workspace of %zu bytes (8-byte aligned) needed",
                sizeof(DotScratch));
  RUBIX_REQUIRE(n == 0 || (a && b), RUBIX_E_INVALID, "rubix_dot: null input");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  DotScratch* ws = static_cast<DotScratch*>(workspace);
  RUBIX_CUDA_TRY(cudaMemsetAsync(&ws->counter, 0, sizeof(unsigned), st));
  dot_kernel<<<kDotBlocks, kDotThreads, 0, st>>>(a, b, n, ws, out);
  RUBIX_LAUNCH_CHECK("dot_kernel");
  return RUBIX_OK;
}
