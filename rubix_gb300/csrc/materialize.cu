// Kernels that materialise the intermediate per-particle arrays of rubix's step chain,
// for callers that run the steps one by one or hand in their own spectra:
//   rubix_ssp_lookup       calculate_spectra (+ scale_spectrum_by_mass)  -> [n][n_wave]
//   rubix_resample_rows    doppler_shift_and_resampling of given spectra -> [n][n_wave_t]
//   rubix_segment_sum_rows calculate_cube of given spectra               -> [n_seg][n_wave_t]
// The fused path (rubix_cube_fwd) never writes these arrays.
#include "common.cuh"

namespace rubix {
namespace {

__device__ __forceinline__ int count_le_f(const float* __restrict__ g, int n, float x) {
  if (x != x) return n;
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (g[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// interpax.interp2d(method="linear", extrap=0) of flux[Z, age, :] at (Z_i, age_i), times
// mass_i when mass is given.
__global__ void ssp_lookup_kernel(const float* __restrict__ flux, const float* __restrict__ zg,
                                  int nZ, const float* __restrict__ ag, int nA, int nW,
                                  const float* __restrict__ Z, const float* __restrict__ A,
                                  const float* __restrict__ mass, long long n,
                                  float* __restrict__ out, long long out_stride) {
  for (long long i = blockIdx.x; i < n; i += gridDim.x) {
    const float z = Z[i], a = A[i];
    const int iz = min(max(count_le_f(zg, nZ, z), 1), nZ - 1);
    const int ia = min(max(count_le_f(ag, nA, a), 1), nA - 1);
    const float dz = zg[iz] - zg[iz - 1], da = ag[ia] - ag[ia - 1];
    const float tz = dz == 0.f ? 0.f : (z - zg[iz - 1]) / dz;
    const float ta = da == 0.f ? 0.f : (a - ag[ia - 1]) / da;
    const bool outside = (z < zg[0]) || (z > zg[nZ - 1]) || (a < ag[0]) || (a > ag[nA - 1]);
    const float m = mass ? mass[i] : 1.f;
    const float w00 = (1.f - tz) * (1.f - ta), w10 = tz * (1.f - ta);
    const float w01 = (1.f - tz) * ta, w11 = tz * ta;
    const float* f00 = flux + ((long long)(iz - 1) * nA + (ia - 1)) * nW;
    const float* f10 = f00 + (long long)nA * nW;
    float* o = out + i * out_stride;
    for (int k = threadIdx.x; k < nW; k += blockDim.x) {
      float g = 0.f;
      if (!outside) {
        g = w00 * f00[k];
        g = fmaf(w10, f10[k], g);
        g = fmaf(w01, f00[k + nW], g);
        g = fmaf(w11, f10[k + nW], g);
      }
      o[k] = g * m;
    }
  }
}

__device__ __forceinline__ float block_sum(float v, float* s_tmp) {
  // fixed-order block reduction (deterministic)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_tmp[warp] = v;
  __syncthreads();
  float t = 0.f;
  const int nw = (blockDim.x + 31) >> 5;
  for (int w = 0; w < nw; ++w) t += s_tmp[w];
  return t;
}

// resample_spectrum (spectra/ifu.py:224-266) of row i of `spec` given on the grid
// lambda'_k = fl32(wave_z_k * fl32(exp(v_i / c))).
__global__ void resample_rows_kernel(const float* __restrict__ spec, long long spec_stride,
                                     const float* __restrict__ wave_z, int nW,
                                     const float* __restrict__ vel, long long vel_stride,
                                     int vel_comp, long long n, const float* __restrict__ wave_t,
                                     int nT, float* __restrict__ out, long long out_stride) {
  extern __shared__ float s_buf[];  // lambda' [nW], F [nW]
  __shared__ float s_tmp[32];
  float* s_lp = s_buf;
  float* s_f = s_buf + nW;
  const float t_lo = wave_t[0], t_hi = wave_t[nT - 1];
  for (long long i = blockIdx.x; i < n; i += gridDim.x) {
    const float alpha = doppler_factor(vel[i * vel_stride + vel_comp]);
    const float* F = spec + i * spec_stride;
    __syncthreads();
    for (int k = threadIdx.x; k < nW; k += blockDim.x) {
      s_lp[k] = __fmul_rn(wave_z[k], alpha);
      s_f[k] = F[k];
    }
    __syncthreads();
    float tp = 0.f;
    for (int k = threadIdx.x + 1; k < nW; k += blockDim.x) {
      const float lp = s_lp[k];
      if (lp >= t_lo && lp <= t_hi) tp = fmaf(s_f[k], lp - s_lp[k - 1], tp);
    }
    const float T = block_sum(tp, s_tmp);
    float tn = 0.f;
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
      const float x = wave_t[t];
      float v;
      if (x < s_lp[0]) {
        v = s_f[0];
      } else if (x > s_lp[nW - 1]) {
        v = s_f[nW - 1];
      } else {
        const int j = min(max(count_le_f(s_lp, nW, x), 1), nW - 1);  // bracket [j-1, j]
        const float dx = s_lp[j] - s_lp[j - 1];
        v = dx == 0.f ? s_f[j - 1]
                      : fmaf(x - s_lp[j - 1], __fdiv_rn(s_f[j] - s_f[j - 1], dx), s_f[j - 1]);
      }
      out[i * out_stride + t] = v;
      if (t > 0) tn = fmaf(v, x - wave_t[t - 1], tn);
    }
    const float Tn = block_sum(tn, s_tmp);
    float sc = T / Tn;
    if (sc != sc) sc = 0.f;
    if (isinf(sc)) sc = copysignf(kFltMax, sc);
    __syncthreads();
    for (int t = threadIdx.x; t < nT; t += blockDim.x) out[i * out_stride + t] *= sc;
  }
}

// out[s][t] = sum over sorted particles j of spaxel s of rows[perm[j]][t], in order.
__global__ void segment_sum_rows_kernel(const float* __restrict__ rows, long long row_stride,
                                        const int* __restrict__ perm,
                                        const int* __restrict__ seg_off, int n_seg, int nT,
                                        float* __restrict__ out, long long out_stride) {
  for (int s = blockIdx.x; s < n_seg; s += gridDim.x) {
    const int b = seg_off[s], e = seg_off[s + 1];
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
      float acc = 0.f;
      for (int j = b; j < e; ++j) acc += rows[(long long)perm[j] * row_stride + t];
      out[(long long)s * out_stride + t] = acc;
    }
  }
}

// out[i][k] = rows[i][k] * mass[i]  (scale_spectrum_by_mass, core/ifu.py:149-157)
__global__ void scale_rows_kernel(const float* __restrict__ rows, long long row_stride,
                                  const float* __restrict__ mass, long long n, int nW,
                                  float* __restrict__ out, long long out_stride) {
  for (long long i = blockIdx.x; i < n; i += gridDim.x) {
    const float m = mass[i];
    for (int k = threadIdx.x; k < nW; k += blockDim.x)
      out[i * out_stride + k] = rows[i * row_stride + k] * m;
  }
}

// values[i][0..width) = 0 where mask[i] == 0 (filter_particles, core/telescope.py:159-172)
__global__ void mask_zero_kernel(float* __restrict__ values, long long n, int width,
                                 long long stride, const unsigned char* __restrict__ mask) {
  const long long total = n * width;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long i = q / width;
    if (mask[i] == 0) values[i * stride + (q - i * width)] = 0.f;
  }
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_mask_zero(float* values, int64_t n, int32_t width, int64_t stride,
                               const uint8_t* mask, void* stream) {
  RUBIX_REQUIRE(n >= 0 && width >= 0 && stride >= width, RUBIX_E_SHAPE,
                "rubix_mask_zero: bad sizes");
  if (n == 0 || width == 0) return RUBIX_OK;
  RUBIX_REQUIRE(values && mask, RUBIX_E_INVALID, "rubix_mask_zero: null pointer");
  const long long total = n * (long long)width;
  const int g = (int)std::min<long long>((total + 255) / 256, (long long)sm_count() * 16);
  mask_zero_kernel<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(values, n, width, stride,
                                                                      mask);
  RUBIX_LAUNCH_CHECK("mask_zero_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_scale_rows(const float* rows, int64_t row_stride, const float* mass,
                                int64_t n, int32_t n_wave, float* out, int64_t out_stride,
                                void* stream) {
  RUBIX_REQUIRE(n >= 0 && n_wave >= 0, RUBIX_E_SHAPE, "rubix_scale_rows: bad sizes");
  RUBIX_REQUIRE(row_stride >= n_wave && out_stride >= n_wave, RUBIX_E_SHAPE,
                "rubix_scale_rows: stride smaller than the row");
  if (n == 0 || n_wave == 0) return RUBIX_OK;
  RUBIX_REQUIRE(rows && mass && out, RUBIX_E_INVALID, "rubix_scale_rows: null pointer");
  const int g = (int)std::min<long long>(n, (long long)sm_count() * 16);
  scale_rows_kernel<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(rows, row_stride, mass, n,
                                                                       n_wave, out, out_stride);
  RUBIX_LAUNCH_CHECK("scale_rows_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_ssp_lookup(const float* ssp_flux, const float* ssp_metallicity,
                                const float* ssp_age, int32_t n_met, int32_t n_age,
                                int32_t n_wave, const float* metallicity, const float* age,
                                const float* mass, int64_t n, float* out, int64_t out_stride,
                                void* stream) {
  RUBIX_REQUIRE(n >= 0, RUBIX_E_SHAPE, "rubix_ssp_lookup: n < 0");
  RUBIX_REQUIRE(n_met >= 2 && n_age >= 2 && n_wave >= 1, RUBIX_E_SHAPE,
                "rubix_ssp_lookup: SSP grid needs >= 2 metallicities and >= 2 ages");
  RUBIX_REQUIRE(out_stride >= n_wave, RUBIX_E_SHAPE, "rubix_ssp_lookup: out_stride < n_wave");
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(ssp_flux && ssp_metallicity && ssp_age && metallicity && age && out,
                RUBIX_E_INVALID, "rubix_ssp_lookup: null pointer");
  const int g = (int)std::min<long long>(n, (long long)sm_count() * 16);
  ssp_lookup_kernel<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      ssp_flux, ssp_metallicity, n_met, ssp_age, n_age, n_wave, metallicity, age, mass, n, out,
      out_stride);
  RUBIX_LAUNCH_CHECK("ssp_lookup_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_resample_rows(const float* spectra, int64_t spectra_stride,
                                   const float* ssp_wave_z, int32_t n_wave,
                                   const float* velocity, int64_t vel_stride,
                                   int32_t vel_component, int64_t n, const float* wave_t,
                                   int32_t n_wave_t, float* out, int64_t out_stride,
                                   void* stream) {
  RUBIX_REQUIRE(n >= 0 && n_wave >= 2 && n_wave_t >= 1, RUBIX_E_SHAPE,
                "rubix_resample_rows: bad sizes");
  RUBIX_REQUIRE(spectra_stride >= n_wave && out_stride >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_resample_rows: stride smaller than the row");
  RUBIX_REQUIRE(vel_component >= 0 && vel_component < vel_stride, RUBIX_E_INVALID,
                "rubix_resample_rows: vel_component outside the velocity row");
  const size_t smem = sizeof(float) * 2 * (size_t)n_wave;
  RUBIX_REQUIRE(smem <= 200 * 1024, RUBIX_E_UNSUPPORTED,
                "rubix_resample_rows: %d wavelengths do not fit in shared memory", n_wave);
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(spectra && ssp_wave_z && velocity && wave_t && out, RUBIX_E_INVALID,
                "rubix_resample_rows: null pointer");
  RUBIX_CUDA_TRY(cudaFuncSetAttribute(resample_rows_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int g = (int)std::min<long long>(n, (long long)sm_count() * 8);
  resample_rows_kernel<<<g, 256, smem, static_cast<cudaStream_t>(stream)>>>(
      spectra, spectra_stride, ssp_wave_z, n_wave, velocity, vel_stride, vel_component, n,
      wave_t, n_wave_t, out, out_stride);
  RUBIX_LAUNCH_CHECK("resample_rows_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_segment_sum_rows(const float* rows, int64_t row_stride, int32_t n_wave_t,
                                      const int32_t* perm, const int32_t* seg_offsets,
                                      int32_t n_segments, float* out, int64_t out_stride,
                                      void* stream) {
  RUBIX_REQUIRE(n_segments >= 0 && n_wave_t >= 0, RUBIX_E_SHAPE,
                "rubix_segment_sum_rows: bad sizes");
  RUBIX_REQUIRE(row_stride >= n_wave_t && out_stride >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_segment_sum_rows: stride smaller than the row");
  if (n_segments == 0 || n_wave_t == 0) return RUBIX_OK;
  RUBIX_REQUIRE(seg_offsets && out, RUBIX_E_INVALID, "rubix_segment_sum_rows: null pointer");
  const int g = std::min(n_segments, sm_count() * 16);
  segment_sum_rows_kernel<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      rows, row_stride, perm, seg_offsets, n_segments, n_wave_t, out, out_stride);
  RUBIX_LAUNCH_CHECK("segment_sum_rows_kernel");
  return RUBIX_OK;
}
