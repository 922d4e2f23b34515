// rubix_cube_fwd_noalloc: the fused accumulate kernel without a caller workspace.
//
// Some callers cannot allocate device memory at the point where they render a cube:
// a host framework that owns every byte of GPU memory through its own pool and does not
// let plugins call cudaMalloc (for example a custom operation running inside another
// framework's compiled program), or a latency-critical loop that must never enter an
// allocator.  This entry point serves them: it takes its scratch memory from a static
// device array compiled into this library instead of from a workspace argument.  The
// caller still passes every input and the output cube.
//
// Limits and rules of use
//   * The array holds RUBIX_CUBE_NOALLOC_SCRATCH_BYTES (64 MiB).  Every GPU on which
//     this part of the library is loaded keeps that much memory until the process
//     exits.  Problems whose workspace (rubix_cube_workspace_size) is larger are
//     rejected with RUBIX_E_WORKSPACE before any GPU work.
//   * The device address of the array is looked up with cudaGetSymbolAddress during the
//     first call on each device (with that device current) and cached; make the first
//     call on a device before any stream capture.
//   * All calls share the one array.  Calls whose GPU work overlaps -- on different
//     streams, or from different host threads on the same device -- race on it and
//     corrupt each other's results; serialise them.
//   * The array keeps the contents of the last call.  That is harmless: every value the
//     kernels read before writing (work counters, per-spaxel completion counters, the
//     device error word, spacing extrema) is reset at the start of each call.
//   * No call here allocates or frees device memory.
#include "common.cuh"

#include <mutex>

namespace rubix {
namespace {

static __device__ __align__(256) unsigned char g_cube_scratch[RUBIX_CUBE_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_cube_scratch on the current device (looked up once per device).
int scratch_address(void** out) {
  int dev = -1;
  RUBIX_CUDA_TRY(cudaGetDevice(&dev));
  RUBIX_REQUIRE(dev >= 0 && dev < kMaxDevices, RUBIX_E_UNSUPPORTED,
                "rubix_cube_fwd_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_cube_scratch);
    if (e != cudaSuccess || p == nullptr)
      return set_error(RUBIX_E_CUDA,
                       "rubix_cube_fwd_noalloc: cudaGetSymbolAddress of the static scratch "
                       "failed on device %d: %s",
                       dev, cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix

extern "C" int rubix_cube_fwd_noalloc(const float* ssp_flux, const float* ssp_metallicity,
                                      const float* ssp_age, const float* ssp_wave_z,
                                      int32_t n_met, int32_t n_age, int32_t n_wave,
                                      const float* wave_t, int32_t n_wave_t, const float* mass,
                                      const float* metallicity, const float* age,
                                      const float* velocity, int64_t vel_stride,
                                      int32_t vel_component, const int32_t* perm,
                                      const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                      const float* lsf_taps, int32_t n_lsf_taps,
                                      int32_t lsf_crop, float* cube, int64_t spaxel_stride,
                                      void* stream) {
  const size_t need =
      rubix_cube_workspace_size(n, n_segments, n_wave_t, n_met, n_age, n_wave);
  RUBIX_REQUIRE(need <= (size_t)RUBIX_CUBE_NOALLOC_SCRATCH_BYTES, RUBIX_E_WORKSPACE,
                "rubix_cube_fwd_noalloc: this problem needs %zu bytes of scratch but the "
                "static array holds %zu; use rubix_cube_fwd with a caller workspace",
                need, (size_t)RUBIX_CUBE_NOALLOC_SCRATCH_BYTES);
  void* ws = nullptr;
  const int rc = rubix::scratch_address(&ws);
  if (rc != RUBIX_OK) return rc;
  return rubix_cube_fwd(ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, n_met, n_age, n_wave,
                        wave_t, n_wave_t, mass, metallicity, age, velocity, vel_stride,
                        vel_component, perm, seg_offsets, n_segments, n, lsf_taps, n_lsf_taps,
                        lsf_crop, cube, spaxel_stride, ws,
                        (size_t)RUBIX_CUBE_NOALLOC_SCRATCH_BYTES, stream);
}
