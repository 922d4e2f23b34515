// Kernel (d): 1-D convolution of every spectrum of a datacube along wavelength,
// the full convolution cropped to [crop, n + crop) (rubix/telescope/lsf/lsf.py:29-105).
//
// A block stages one spectrum in shared memory with K-1 zeros of halo and each
// thread produces 4 consecutive outputs from float4 loads of its window, so the
// shared-memory traffic is (K+3)/4 vector loads per 4 outputs and the kernel stays
// bound by the one read and one write of the cube in HBM.
#include "common.cuh"
#include "dot_reduce.cuh"

namespace rubix {
namespace {

constexpr int kLsfThreads = 256;
constexpr int kLsfMaxTaps = 255;

struct LsfArgs {
  const float* in;
  float* out;
  long long rows;
  int n;
  long long sin, sout;
  int K, crop;
  float taps[kLsfMaxTaps + 1];
  const float* taps_dev;  // when set, the taps are read from device memory instead
};

// out[t] = sum_q w[q] * s[t + q] with s[i] = in[i - (K-1-crop)] and w[q] = taps[K-1-q].
// kDot: instead of storing out, sum wt[row][t] * out[t] over the cube (wt with the
// output's layout, row stride sout) into *dot_out, deterministically.
template <int KC, bool kDot = false>
__global__ void __launch_bounds__(kLsfThreads)
    lsf_vec_kernel(LsfArgs a, const float* __restrict__ wt = nullptr,
                   FusedDotScratch* dot_ws = nullptr, double* dot_out = nullptr) {
  extern __shared__ __align__(16) float s_row[];
  __shared__ float s_w[KC * 4];
  float dot = 0.f;
  const int tid = threadIdx.x;
  const float* tp = a.taps_dev ? a.taps_dev : a.taps;
  for (int q = tid; q < KC * 4; q += kLsfThreads) s_w[q] = (q < a.K) ? tp[a.K - 1 - q] : 0.f;
  const int lead = a.K - 1 - a.crop;           // zeros before in[0]
  const int n4 = (a.n + 3) / 4;                 // output groups of 4
  const int span = n4 * 4 + KC * 4;             // staged length (multiple of 4)
  for (long long row = blockIdx.x; row < a.rows; row += gridDim.x) {
    __syncthreads();
    const float* src = a.in + row * a.sin;
    for (int i = tid; i < span; i += kLsfThreads) {
      const int g = i - lead;
      s_row[i] = (g >= 0 && g < a.n) ? src[g] : 0.f;
    }
    __syncthreads();
    float* dst = a.out + row * a.sout;
    for (int u = tid; u < n4; u += kLsfThreads) {
      // dot mode: the four weights first, so the window loads and FMAs hide them
      float wq[4] = {0.f, 0.f, 0.f, 0.f};
      if constexpr (kDot) {
        const float* wr = wt + row * a.sout;
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (4 * u + c < a.n) wq[c] = wr[4 * u + c];
      }
      float win[KC * 4 + 4];
      const float4* p = reinterpret_cast<const float4*>(s_row + 4 * u);
#pragma unroll
      for (int c = 0; c <= KC; ++c) {
        float4 v = p[c];
        win[4 * c] = v.x;
        win[4 * c + 1] = v.y;
        win[4 * c + 2] = v.z;
        win[4 * c + 3] = v.w;
      }
      float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
#pragma unroll
      for (int q = 0; q < KC * 4; ++q) {
        const float w = s_w[q];
        o0 = fmaf(w, win[q], o0);
        o1 = fmaf(w, win[q + 1], o1);
        o2 = fmaf(w, win[q + 2], o2);
        o3 = fmaf(w, win[q + 3], o3);
      }
      const int t = 4 * u;
      if constexpr (kDot) {
        // wq is 0 past the row's end
        dot = fmaf(wq[3], o3, fmaf(wq[2], o2, fmaf(wq[1], o1, fmaf(wq[0], o0, dot))));
      } else {
        if (t < a.n) dst[t] = o0;
        if (t + 1 < a.n) dst[t + 1] = o1;
        if (t + 2 < a.n) dst[t + 2] = o2;
        if (t + 3 < a.n) dst[t + 3] = o3;
      }
    }
  }
  if constexpr (kDot) {
    __shared__ double s_red[kLsfThreads / 32];
    __shared__ int s_last;
    fused_dot_finish(dot, dot_ws, dot_out, s_red, &s_last);
  }
}

// Generic path for long kernels: one output per thread iteration.
__global__ void __launch_bounds__(kLsfThreads) lsf_scalar_kernel(LsfArgs a) {
  extern __shared__ __align__(16) float s_row[];
  __shared__ float s_w[kLsfMaxTaps + 1];
  const int tid = threadIdx.x;
  const float* tp = a.taps_dev ? a.taps_dev : a.taps;
  for (int q = tid; q < a.K; q += kLsfThreads) s_w[q] = tp[a.K - 1 - q];
  const int lead = a.K - 1 - a.crop;
  const int span = a.n + a.K - 1;
  for (long long row = blockIdx.x; row < a.rows; row += gridDim.x) {
    __syncthreads();
    const float* src = a.in + row * a.sin;
    for (int i = tid; i < span; i += kLsfThreads) {
      const int g = i - lead;
      s_row[i] = (g >= 0 && g < a.n) ? src[g] : 0.f;
    }
    __syncthreads();
    float* dst = a.out + row * a.sout;
    for (int t = tid; t < a.n; t += kLsfThreads) {
      float o = 0.f;
      for (int q = 0; q < a.K; ++q) o = fmaf(s_w[q], s_row[t + q], o);
      dst[t] = o;
    }
  }
}

template <int KC>
int launch_vec(const LsfArgs& a, cudaStream_t st) {
  const int n4 = (a.n + 3) / 4;
  const size_t smem = sizeof(float) * ((size_t)n4 * 4 + KC * 4 + 4);
  cudaError_t e = cudaFuncSetAttribute(lsf_vec_kernel<KC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess)
    return set_error(RUBIX_E_CUDA, "cudaFuncSetAttribute(lsf_vec_kernel): %s", cudaGetErrorString(e));
  long long grid = std::min<long long>(a.rows, (long long)sm_count() * 8);
  lsf_vec_kernel<KC><<<(int)grid, kLsfThreads, smem, st>>>(a);
  RUBIX_LAUNCH_CHECK("lsf_vec_kernel");
  return RUBIX_OK;
}

template <int KC>
int launch_vec_dot(const LsfArgs& a, const float* wt, FusedDotScratch* ws, double* out,
                   cudaStream_t st) {
  const int n4 = (a.n + 3) / 4;
  const size_t smem = sizeof(float) * ((size_t)n4 * 4 + KC * 4 + 4);
  cudaError_t e = cudaFuncSetAttribute(lsf_vec_kernel<KC, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess)
    return set_error(RUBIX_E_CUDA, "cudaFuncSetAttribute(lsf_vec_kernel): %s", cudaGetErrorString(e));
  const long long grid = std::min<long long>(
      std::min<long long>(a.rows, (long long)sm_count() * 8), kFusedDotMaxBlocks);
  lsf_vec_kernel<KC, true><<<(int)grid, kLsfThreads, smem, st>>>(a, wt, ws, out);
  RUBIX_LAUNCH_CHECK("lsf_vec_kernel");
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix

using namespace rubix;

namespace rubix {
namespace {

int lsf_fwd_impl(const float* in, float* out, int64_t n_rows, int32_t n_wave_t,
                 int64_t row_stride_in, int64_t row_stride_out, const float* taps,
                 int32_t n_taps, int32_t crop, bool device_taps, void* stream) {
  RUBIX_REQUIRE(n_rows >= 0 && n_wave_t >= 0, RUBIX_E_SHAPE, "rubix_lsf_fwd: negative size");
  RUBIX_REQUIRE(n_taps >= 1 && n_taps <= kLsfMaxTaps, RUBIX_E_SHAPE,
                "rubix_lsf_fwd: n_taps must be in [1, %d]", kLsfMaxTaps);
  RUBIX_REQUIRE(crop >= 0 && crop <= n_taps - 1, RUBIX_E_SHAPE,
                "rubix_lsf_fwd: crop must be in [0, n_taps-1]");
  RUBIX_REQUIRE(row_stride_in >= n_wave_t && row_stride_out >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_lsf_fwd: row stride smaller than n_wave_t");
  RUBIX_REQUIRE((long long)n_wave_t + n_taps + 8 <= 48 * 1024, RUBIX_E_SHAPE,
                "rubix_lsf_fwd: spectrum too long for one shared-memory row");
  if (n_rows == 0 || n_wave_t == 0) return RUBIX_OK;
  RUBIX_REQUIRE(in && out && taps, RUBIX_E_INVALID, "rubix_lsf_fwd: null pointer");
  RUBIX_REQUIRE(in != out, RUBIX_E_INVALID, "rubix_lsf_fwd: in and out must differ");
  LsfArgs a;
  a.in = in;
  a.out = out;
  a.rows = n_rows;
  a.n = n_wave_t;
  a.sin = row_stride_in;
  a.sout = row_stride_out;
  a.K = n_taps;
  a.crop = crop;
  a.taps_dev = device_taps ? taps : nullptr;
  for (int i = 0; i <= kLsfMaxTaps; ++i) a.taps[i] = (!device_taps && i < n_taps) ? taps[i] : 0.f;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // KC = ceil(K/4) weight chunks; each thread's window is KC+1 float4 loads.
  switch ((n_taps + 3) / 4) {
    case 0:
    case 1: return launch_vec<1>(a, st);
    case 2: return launch_vec<2>(a, st);
    case 3: return launch_vec<3>(a, st);
    case 4: return launch_vec<4>(a, st);
    case 5: return launch_vec<5>(a, st);
    case 6: return launch_vec<6>(a, st);
    case 7: return launch_vec<7>(a, st);
    default: break;
  }
  const size_t smem = sizeof(float) * ((size_t)n_wave_t + n_taps + 4);
  RUBIX_CUDA_TRY(cudaFuncSetAttribute(lsf_scalar_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  long long grid = std::min<long long>(n_rows, (long long)sm_count() * 8);
  lsf_scalar_kernel<<<(int)grid, kLsfThreads, smem, st>>>(a);
  RUBIX_LAUNCH_CHECK("lsf_scalar_kernel");
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix

extern "C" int rubix_lsf_fwd(const float* in, float* out, int64_t n_rows, int32_t n_wave_t,
                             int64_t row_stride_in, int64_t row_stride_out, const float* taps,
                             int32_t n_taps, int32_t crop, void* stream) {
  return lsf_fwd_impl(in, out, n_rows, n_wave_t, row_stride_in, row_stride_out, taps, n_taps,
                      crop, false, stream);
}

extern "C" int rubix_lsf_dot_dtaps(const float* in, int64_t n_rows, int32_t n_wave_t,
                                   int64_t row_stride_in, const float* w, int64_t row_stride_w,
                                   const float* taps, int32_t n_taps, int32_t crop, double* out,
                                   void* workspace, size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n_rows >= 0 && n_wave_t >= 0, RUBIX_E_SHAPE, "rubix_lsf_dot_dtaps: negative size");
  RUBIX_REQUIRE(n_taps >= 1 && n_taps <= 28, RUBIX_E_UNSUPPORTED,
                "rubix_lsf_dot_dtaps: n_taps must be in [1, 28], got %d", n_taps);
  RUBIX_REQUIRE(crop >= 0 && crop <= n_taps - 1, RUBIX_E_SHAPE,
                "rubix_lsf_dot_dtaps: crop must be in [0, n_taps-1]");
  RUBIX_REQUIRE(row_stride_in >= n_wave_t && row_stride_w >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_lsf_dot_dtaps: row stride smaller than n_wave_t");
  RUBIX_REQUIRE((long long)n_wave_t + n_taps + 8 <= 48 * 1024, RUBIX_E_SHAPE,
                "rubix_lsf_dot_dtaps: spectrum too long for one shared-memory row");
  RUBIX_REQUIRE(out != nullptr, RUBIX_E_INVALID, "rubix_lsf_dot_dtaps: null output");
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= sizeof(FusedDotScratch) &&
                    (reinterpret_cast<uintptr_t>(workspace) & 7) == 0,
                RUBIX_E_WORKSPACE,
                "rubix_lsf_dot_dtaps: workspace of %zu bytes (8-byte aligned) needed",
                sizeof(FusedDotScratch));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_rows == 0 || n_wave_t == 0) {
    RUBIX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double), st));
    return RUBIX_OK;
  }
  RUBIX_REQUIRE(in && w && taps, RUBIX_E_INVALID, "rubix_lsf_dot_dtaps: null pointer");
  LsfArgs a;
  a.in = in;
  a.out = nullptr;
  a.rows = n_rows;
  a.n = n_wave_t;
  a.sin = row_stride_in;
  a.sout = row_stride_w;
  a.K = n_taps;
  a.crop = crop;
  a.taps_dev = taps;
  for (int i = 0; i <= kLsfMaxTaps; ++i) a.taps[i] = 0.f;
  auto* ws = static_cast<FusedDotScratch*>(workspace);
  RUBIX_CUDA_TRY(cudaMemsetAsync(&ws->counter, 0, sizeof(unsigned), st));
  switch ((n_taps + 3) / 4) {
    case 1: return launch_vec_dot<1>(a, w, ws, out, st);
    case 2: return launch_vec_dot<2>(a, w, ws, out, st);
    case 3: return launch_vec_dot<3>(a, w, ws, out, st);
    case 4: return launch_vec_dot<4>(a, w, ws, out, st);
    case 5: return launch_vec_dot<5>(a, w, ws, out, st);
    case 6: return launch_vec_dot<6>(a, w, ws, out, st);
    default: return launch_vec_dot<7>(a, w, ws, out, st);
  }
}

extern "C" int rubix_lsf_fwd_dtaps(const float* in, float* out, int64_t n_rows,
                                   int32_t n_wave_t, int64_t row_stride_in,
                                   int64_t row_stride_out, const float* taps, int32_t n_taps,
                                   int32_t crop, void* stream) {
  return lsf_fwd_impl(in, out, n_rows, n_wave_t, row_stride_in, row_stride_out, taps, n_taps,
                      crop, true, stream);
}
