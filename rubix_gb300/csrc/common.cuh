// Shared helpers for the rubix_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include <stdarg.h>

#include <algorithm>

#include "../../include/rubix_gb300.h"

namespace rubix {

// Records a formatted message as this thread's last error and returns `code`.
int set_error(int code, const char* fmt, ...);
void clear_error();

// Checks a CUDA runtime call; on failure records the error and returns RUBIX_E_CUDA.
#define RUBIX_CUDA_TRY(expr)                                                        \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess) {                                                        \
      return ::rubix::set_error(RUBIX_E_CUDA, "%s failed: %s (%s:%d)", #expr,       \
                                cudaGetErrorString(_e), __FILE__, __LINE__);        \
    }                                                                               \
  } while (0)

#define RUBIX_LAUNCH_CHECK(name)                                                    \
  do {                                                                              \
    cudaError_t _e = cudaGetLastError();                                            \
    if (_e != cudaSuccess) {                                                        \
      return ::rubix::set_error(RUBIX_E_CUDA, "launch of %s failed: %s", name,      \
                                cudaGetErrorString(_e));                            \
    }                                                                               \
  } while (0)

#define RUBIX_REQUIRE(cond, code, ...)                                              \
  do {                                                                              \
    if (!(cond)) return ::rubix::set_error(code, __VA_ARGS__);                      \
  } while (0)

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Bump allocator over a caller-provided workspace; sizes are rounded to 256 bytes.
struct Carve {
  char* base;
  size_t off;
  explicit Carve(void* p) : base(static_cast<char*>(p)), off(0) {}
  template <class T>
  T* take(size_t count) {
    T* r = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += align_up(count * sizeof(T), 256);
    return r;
  }
};

int sm_count();  // cached multiprocessor count of the current device

constexpr double kSpeedOfLight = 299792.458;  // km/s, rubix_config.yml:8
constexpr float kFltMax = 3.402823466e+38f;

#ifdef __CUDACC__
// exp(v / c) rounded once to float32: the Doppler factor of rubix's
// velocity_doppler_shift (spectra/ifu.py:190).  In float64 by the Taylor series of exp
// (degree 8, Horner form) for |v| <= 10^4 km/s, where the truncated terms are below
// 2e-18 of the sum; exp() beyond.  Eight FMAs instead of a general float64 exp keeps
// the per-particle setup off the slow float64 pipe.
__device__ __forceinline__ float doppler_factor(float v) {
  const double x = (double)v * (1.0 / kSpeedOfLight);
  if (!(fabs(x) <= 1.0e4 / kSpeedOfLight)) return (float)exp(x);
  double p = 1.0 / 40320.0;
  p = fma(p, x, 1.0 / 5040.0);
  p = fma(p, x, 1.0 / 720.0);
  p = fma(p, x, 1.0 / 120.0);
  p = fma(p, x, 1.0 / 24.0);
  p = fma(p, x, 1.0 / 6.0);
  p = fma(p, x, 0.5);
  p = fma(p, x, 1.0);
  p = fma(p, x, 1.0);
  return (float)p;
}

// The dust transmission 2^(e A_V) of a resampled spectrum at one telescope wavelength
// (e = -0.4 log2(10) A(lambda)/A(V), rubix's 10^(-0.4 A_lambda),
// spectra/dust/dust_baseclasses.py:163-164): one hardware 2^x (PTX ex2.approx.ftz.f32,
// relative error about 2^-22, results below 2^-126 flushed to 0).
__device__ __forceinline__ float dust_transmission(float e, float av) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(__fmul_rn(e, av)));
  return y;
}
#endif

}  // namespace rubix
