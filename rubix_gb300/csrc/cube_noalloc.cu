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
//     rejected with RUBIX_E_WORKSPACE before any GPU work, after the same argument
//     checks as rubix_cube_fwd (so a malformed call gets the same code from both).
//   * The device address of the array is looked up with cudaGetSymbolAddress, with the
//     device current, the first time a call runs in a CUDA context, and cached under
//     that context's unique id.  A call in another context (a cudaDeviceReset followed
//     by a new primary context, or a context the host framework created itself) looks
//     the address up again.  The first call in a context should come before any stream
//     capture.
//   * All calls share the one array.  Calls whose GPU work overlaps -- on different
//     streams, or from different host threads on the same device -- race on it and
//     corrupt each other's results; serialise them.
//   * The array keeps the contents of the last call.  That is harmless: every value the
//     kernels read before writing (work counters, per-spaxel completion counters, the
//     device error word, spacing extrema) is reset at the start of each call.
//   * rubix_cube_noalloc_status reads the device error word of the last call (a bounded
//     shared-memory copy wait that gave up leaves an invalid cube).
//   * No call here allocates or frees device memory.
#include "common.cuh"

#include <cuda.h>  // CUcontext / CUresult types; the functions come through the runtime

#include <mutex>

namespace rubix {

int cube_fwd_check_args(const char* who, const float* ssp_flux, const float* ssp_metallicity,
                        const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                        int32_t n_age, int32_t n_wave, const float* wave_t, int32_t n_wave_t,
                        const float* mass, const float* metallicity, const float* age,
                        const float* velocity, int64_t vel_stride, int32_t vel_component,
                        const int32_t* perm, const int32_t* seg_offsets, int32_t n_segments,
                        int64_t n, const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop,
                        const float* cube, int64_t spaxel_stride, bool* nothing_to_do);
int cube_fwd_named(const char* who, const float* ssp_flux, const float* ssp_metallicity,
                   const float* ssp_age, const float* ssp_wave_z, int32_t n_met, int32_t n_age,
                   int32_t n_wave, const float* wave_t, int32_t n_wave_t, const float* mass,
                   const float* metallicity, const float* age, const float* velocity,
                   int64_t vel_stride, int32_t vel_component, const int32_t* perm,
                   const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                   const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop, float* cube,
                   int64_t spaxel_stride, void* workspace, size_t workspace_bytes,
                   void* stream);

namespace {

static __device__ __align__(256) unsigned char g_cube_scratch[RUBIX_CUBE_NOALLOC_SCRATCH_BYTES];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct ScratchSlot {
  unsigned long long ctx_id;  // unique over the process lifetime (cuCtxGetId)
  void* addr;
};

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
ScratchSlot g_scratch[kMaxDevices] = {};
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

int driver_entry_points() {
  if (g_ctx_get_current && g_ctx_get_id) return RUBIX_OK;
  cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
  void *f1 = nullptr, *f2 = nullptr;
  const cudaError_t e1 =
      cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
  const cudaError_t e2 =
      cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
  if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
      q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
    return set_error(RUBIX_E_CUDA,
                     "rubix_cube_fwd_noalloc: driver entry points cuCtxGetCurrent/cuCtxGetId "
                     "unavailable (%s)",
                     cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
  g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
  g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  return RUBIX_OK;
}

// Unique id of the context current on this thread (0 when none is current yet).
int current_context_id(unsigned long long* id) {
  *id = 0;
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS)
    return set_error(RUBIX_E_CUDA, "rubix_cube_fwd_noalloc: cuCtxGetCurrent failed");
  if (ctx != nullptr && g_ctx_get_id(ctx, id) != CUDA_SUCCESS)
    return set_error(RUBIX_E_CUDA, "rubix_cube_fwd_noalloc: cuCtxGetId failed");
  return RUBIX_OK;
}

// Device address of g_cube_scratch in the context current on this thread: looked up
// once per context (with its device current) and cached under the context's id.
int scratch_address(void** out) {
  int dev = -1;
  RUBIX_CUDA_TRY(cudaGetDevice(&dev));
  RUBIX_REQUIRE(dev >= 0 && dev < kMaxDevices, RUBIX_E_UNSUPPORTED,
                "rubix_cube_fwd_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  int rc = driver_entry_points();
  if (rc != RUBIX_OK) return rc;
  unsigned long long id = 0;
  rc = current_context_id(&id);
  if (rc != RUBIX_OK) return rc;
  if (id != 0 && g_scratch[dev].ctx_id == id && g_scratch[dev].addr != nullptr) {
    *out = g_scratch[dev].addr;
    return RUBIX_OK;
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_cube_scratch);
  if (e != cudaSuccess || p == nullptr)
    return set_error(RUBIX_E_CUDA,
                     "rubix_cube_fwd_noalloc: cudaGetSymbolAddress of the static scratch "
                     "failed on device %d: %s",
                     dev, cudaGetErrorString(e));
  // The lookup makes the runtime's context current when none was; key on that one.
  rc = current_context_id(&id);
  if (rc != RUBIX_OK) return rc;
  g_scratch[dev] = ScratchSlot{id, p};
  *out = p;
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
  static const char* kWho = "rubix_cube_fwd_noalloc";
  bool nothing_to_do = false;
  int rc = rubix::cube_fwd_check_args(kWho, ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z,
                                      n_met, n_age, n_wave, wave_t, n_wave_t, mass,
                                      metallicity, age, velocity, vel_stride, vel_component,
                                      perm, seg_offsets, n_segments, n, lsf_taps, n_lsf_taps,
                                      lsf_crop, cube, spaxel_stride, &nothing_to_do);
  if (rc != RUBIX_OK || nothing_to_do) return rc;
  const size_t need =
      rubix_cube_workspace_size(n, n_segments, n_wave_t, n_met, n_age, n_wave);
  RUBIX_REQUIRE(need <= (size_t)RUBIX_CUBE_NOALLOC_SCRATCH_BYTES, RUBIX_E_WORKSPACE,
                "%s: this problem needs %zu bytes of scratch but the static array holds "
                "%zu; use rubix_cube_fwd with a caller workspace",
                kWho, need, (size_t)RUBIX_CUBE_NOALLOC_SCRATCH_BYTES);
  void* ws = nullptr;
  rc = rubix::scratch_address(&ws);
  if (rc != RUBIX_OK) return rc;
  return rubix::cube_fwd_named(kWho, ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, n_met,
                               n_age, n_wave, wave_t, n_wave_t, mass, metallicity, age,
                               velocity, vel_stride, vel_component, perm, seg_offsets,
                               n_segments, n, lsf_taps, n_lsf_taps, lsf_crop, cube,
                               spaxel_stride, ws, (size_t)RUBIX_CUBE_NOALLOC_SCRATCH_BYTES,
                               stream);
}

extern "C" int rubix_cube_noalloc_status(int* device_error, void* stream) {
  RUBIX_REQUIRE(device_error != nullptr, RUBIX_E_INVALID,
                "rubix_cube_noalloc_status: null pointer");
  void* ws = nullptr;
  const int rc = rubix::scratch_address(&ws);
  if (rc != RUBIX_OK) return rc;
  return rubix_cube_status(ws, device_error, stream);
}
