// Diagnostic: the FP32 FMA rate of this GPU, for the compute roofline of the kernels.
// Every thread runs 8 independent FMA chains (enough to cover the FMA latency with
// 8 resident warps per scheduler); the result is stored so nothing is eliminated.
#include "common.cuh"

namespace rubix {
namespace {

__global__ void __launch_bounds__(256) fma_probe_kernel(float* __restrict__ out, int iters,
                                                        float a, float b) {
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = fmaf(v[i], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_fma_probe_blocks(void) { return sm_count() * 8; }

extern "C" int rubix_fma_probe(float* out, int32_t iters, void* stream) {
  RUBIX_REQUIRE(out != nullptr && iters > 0, RUBIX_E_INVALID, "rubix_fma_probe: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  fma_probe_kernel<<<sm_count() * 8, 256, 0, st>>>(out, iters, 0.999999f, 1e-7f);
  RUBIX_LAUNCH_CHECK("fma_probe_kernel");
  return RUBIX_OK;
}
