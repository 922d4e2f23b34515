// Bench-only measurement aid (not part of librubix_gb300): the FP32 FMA rate of this GPU,
// against which bench.py states the compute roofline of the kernels.  Every thread runs
// 8 independent FMA chains (enough to cover the FMA latency with 8 resident warps per
// scheduler); the result is stored so nothing is eliminated.  Built by
// rubix_gb300/_build.py:build_probe() into rubix_gb300/librubix_gb300_probe.so.
#include <cuda_runtime.h>

#include <cstdint>

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

int blocks_for_current_device() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  return sms * 8;
}

}  // namespace

// Blocks of 256 threads one probe launch uses on the current device (-1 on a CUDA error).
extern "C" __attribute__((visibility("default"))) int rubix_probe_fma_blocks(void) {
  return blocks_for_current_device();
}

// One launch: rubix_probe_fma_blocks() * 256 threads each run iters * 128 FMAs (8 chains)
// and store one float into out.  0 on success, -1 for bad arguments, -4 on a launch error.
extern "C" __attribute__((visibility("default"))) int rubix_probe_fma(float* out, int32_t iters,
                                                                     void* stream) {
  const int blocks = blocks_for_current_device();
  if (out == nullptr || iters <= 0 || blocks <= 0) return -1;
  fma_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(out, iters, 0.999999f,
                                                                          1e-7f);
  return cudaGetLastError() == cudaSuccess ? 0 : -4;
}
