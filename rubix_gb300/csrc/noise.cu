// Observation noise after PSF and LSF (rubix/core/noise.py:17-80,
// rubix/telescope/noise/noise.py:35-115):
//   flux[s]  = sum_t cube[s][t]
//   median   = median of flux over all spaxels, 0 when any flux <= 0 (rubix takes
//              jnp.median of where(flux > 0, flux, nan): one NaN makes it NaN, and
//              nan_to_num turns that into 0)
//   sigma[s] = sqrt(median) / signal_to_noise / sqrt(flux[s])  (0 where flux <= 0)
//   cube[s][t] += cube[s][t] * sigma[s] * z[s][t],   z ~ N(0, 1) or U[0, 1)
// rubix draws z from jax.random with a fixed key; here z comes from a Philox4x32-10
// counter-based generator (Salmon, Moraes, Dror and Shaw, SC'11) keyed by a caller
// seed: element (s, t) has the index e = s * L + t in the unpadded [spaxel][lambda]
// order and takes output e % 4 of the call with counter (e / 4 as two 32-bit words, 0,
// 0), so one call serves four consecutive elements (one float4 of an unpadded,
// 16-byte-aligned cube).  Results are reproducible for a seed but not equal to rubix's
// draws.  Normal draws pair outputs (0, 1) and (2, 3) by Box-Muller on the hardware
// log2 / sin / cos approximations (relative errors near 1e-6, far below anything the
// noise statistics can show).  The median is an exact radix select (four 8-bit passes
// over the float bit patterns, integer histograms), in one block for up to 2^20
// spaxels.
#include <math.h>

#include "common.cuh"

namespace rubix {
namespace {

// ---------------------------------------------------------------- Philox4x32-10
struct U4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ void mulhilo(uint32_t a, uint32_t b, uint32_t& hi,
                                                 uint32_t& lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(M0, c.x, hi0, lo0);
    mulhilo(M1, c.z, hi1, lo1);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// 32 random bits -> (0, 1]
__device__ __forceinline__ float u01_open0(uint32_t v) {
  return ((float)(v >> 8) + 1.0f) * (1.0f / 16777216.0f);
}
// 32 random bits -> [0, 1)
__device__ __forceinline__ float u01(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }

// ---------------------------------------------------------------- flux image
__global__ void flux_image_kernel(const float* __restrict__ cube, long long n_spaxels, int L,
                                  long long stride, float* __restrict__ flux) {
  const int lane = threadIdx.x & 31;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long n_warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long s = warp; s < n_spaxels; s += n_warps) {
    const float* row = cube + s * stride;
    float acc = 0.f;
    for (int t = lane; t < L; t += 32) acc += row[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) flux[s] = acc;
  }
}

// ---------------------------------------------------------------- median (radix select)
struct SelectState {
  unsigned hist[256];
  unsigned rank[2];      // ranks still sought inside the prefix (lower and upper middle)
  unsigned bits[2];      // finished bit patterns of the two middle elements
  int any_nonpositive;
};

// Pass over the values whose bits match the prefix of the current pass: histogram of
// the next 8-bit digit.  Values are non-negative floats here (any value <= 0 or NaN
// only raises the flag), so their bit patterns order like the floats.
__global__ void select_hist_kernel(const float* __restrict__ v, long long n, int shift,
                                   unsigned prefix_mask, int which,
                                   SelectState* __restrict__ st) {
  __shared__ unsigned h[256];
  const unsigned prefix = st->bits[which] & prefix_mask;  // digits picked so far
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float x = v[i];
    if (!(x > 0.f)) {
      st->any_nonpositive = 1;
      continue;
    }
    const unsigned b = __float_as_uint(x);
    if ((b & prefix_mask) == prefix) atomicAdd(&h[(b >> shift) & 255u], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&st->hist[i], h[i]);
}

// One thread: find the digit holding rank[j] for the element followed in this pass.
__global__ void select_pick_kernel(SelectState* __restrict__ st, int shift, int which) {
  unsigned r = st->rank[which];
  unsigned d = 0;
  for (; d < 256; ++d) {
    if (r < st->hist[d]) break;
    r -= st->hist[d];
  }
  st->rank[which] = r;
  st->bits[which] |= (d & 255u) << shift;
  for (int i = 0; i < 256; ++i) st->hist[i] = 0u;
}

__global__ void select_finish_kernel(const SelectState* __restrict__ st, long long n,
                                     float* __restrict__ median) {
  if (st->any_nonpositive || n == 0) {
    *median = 0.f;
    return;
  }
  const float a = __uint_as_float(st->bits[0]), b = __uint_as_float(st->bits[1]);
  *median = (n & 1) ? a : 0.5f * (a + b);
}

// The whole select in one block (n <= 2^20): the histogram passes of both middle
// elements, with the digit picks between them, in shared memory.
__global__ void __launch_bounds__(1024) select_block_kernel(const float* __restrict__ v,
                                                            long long n,
                                                            float* __restrict__ median) {
  __shared__ unsigned h[256];
  __shared__ unsigned s_rank, s_bits;
  __shared__ int s_bad;
  __shared__ unsigned s_res[2];
  const int tid = threadIdx.x;
  // rubix's median is NaN (hence 0) as soon as one value is <= 0 (or NaN): one pass
  // over the values settles that before any histogram pass
  int bad0 = 0;
  for (long long i = tid; i < n; i += blockDim.x) bad0 |= !(v[i] > 0.f);
  if (__syncthreads_or(bad0) || n == 0) {
    if (tid == 0) *median = 0.f;
    return;
  }
  if (tid == 0) s_bad = 0;
  for (int which = 0; which < 2; ++which) {
    if (tid == 0) {
      s_rank = which == 0 ? (unsigned)((n - 1) / 2) : (unsigned)(n / 2);
      s_bits = 0u;
    }
    unsigned mask = 0u;
    for (int shift = 24; shift >= 0; shift -= 8) {
      for (int i = tid; i < 256; i += blockDim.x) h[i] = 0u;
      __syncthreads();
      const unsigned prefix = s_bits & mask;
      int bad = 0;
      for (long long i = tid; i < n; i += blockDim.x) {
        const float x = v[i];
        if (!(x > 0.f)) {
          bad = 1;
          continue;
        }
        const unsigned b = __float_as_uint(x);
        if ((b & mask) == prefix) atomicAdd(&h[(b >> shift) & 255u], 1u);
      }
      if (bad) s_bad = 1;
      __syncthreads();
      if (tid == 0) {
        unsigned r = s_rank, d = 0;
        for (; d < 255; ++d) {
          if (r < h[d]) break;
          r -= h[d];
        }
        s_rank = r;
        s_bits |= d << shift;
      }
      __syncthreads();
      mask |= 255u << shift;
    }
    if (tid == 0) s_res[which] = s_bits;
    __syncthreads();
  }
  if (tid == 0) {
    if (s_bad || n == 0) {
      *median = 0.f;
    } else {
      const float a = __uint_as_float(s_res[0]), b = __uint_as_float(s_res[1]);
      *median = (n & 1) ? a : 0.5f * (a + b);
    }
  }
}

__global__ void select_init_kernel(SelectState* __restrict__ st, long long n) {
  for (int i = 0; i < 256; ++i) st->hist[i] = 0u;
  st->rank[0] = (unsigned)((n - 1) / 2);  // lower middle (the median for odd n)
  st->rank[1] = (unsigned)(n / 2);        // upper middle
  st->bits[0] = st->bits[1] = 0u;
  st->any_nonpositive = 0;
}

// ---------------------------------------------------------------- noise
// The four draws of one Philox call.
__device__ __forceinline__ void quad_draws(U4 r, int distribution, float z[4]) {
  if (distribution == 0) {  // Box-Muller on two pairs
    const float two_pi = 6.283185307179586f;
    const float u1 = u01_open0(r.x), u2 = u01(r.y), u3 = u01_open0(r.z), u4 = u01(r.w);
    const float r1 = sqrtf(-2.0f * __logf(u1)), r2 = sqrtf(-2.0f * __logf(u3));
    float s1, c1, s2, c2;
    // angles in [-pi, pi): the argument range of the hardware approximations
    __sincosf(two_pi * (u2 - 0.5f), &s1, &c1);
    __sincosf(two_pi * (u4 - 0.5f), &s2, &c2);
    z[0] = r1 * c1;
    z[1] = r1 * s1;
    z[2] = r2 * c2;
    z[3] = r2 * s2;
  } else {
    z[0] = u01(r.x);
    z[1] = u01(r.y);
    z[2] = u01(r.z);
    z[3] = u01(r.w);
  }
}

constexpr int kNoiseThreads = 256;
constexpr int kNoiseQuads = 4;  // Philox calls per thread per pass over a row

// Blocks stride over spaxel rows; a pass over a row covers kNoiseThreads * kNoiseQuads
// consecutive quads (calls), with all of a thread's float4 loads issued before its
// Philox arithmetic.  Quads that straddle the row's ends (and every quad when the
// cube is padded or not 16-byte aligned) update their elements of this row one by one.
__global__ void __launch_bounds__(kNoiseThreads) noise_kernel(
    float* __restrict__ cube, long long n_spaxels, int L, long long stride,
    const float* __restrict__ flux, const float* __restrict__ median, float inv_s2n,
    int distribution, uint32_t k0, uint32_t k1, int vec) {
  const float scale = sqrtf(*median) * inv_s2n;
  // a zero median (rubix's rule for a cube with an empty spaxel) adds no noise: every
  // finite element stays as it is, so the pass is skipped
  if (!(scale != 0.f)) return;
  for (long long s = blockIdx.x; s < n_spaxels; s += gridDim.x) {
    const float f = flux[s];
    const float sig = f > 0.f ? scale / sqrtf(f) : 0.f;
    const long long e0 = s * (long long)L;  // logical index of the row's first element
    const long long qa = e0 >> 2, qb = (e0 + L - 1) >> 2;  // quads touching the row
    float* row = cube + s * stride;
    for (long long base = qa; base <= qb; base += kNoiseThreads * kNoiseQuads) {
      float4 c[kNoiseQuads];
      bool whole[kNoiseQuads];
#pragma unroll
      for (int k = 0; k < kNoiseQuads; ++k) {
        const long long q = base + threadIdx.x + k * kNoiseThreads;
        const long long tq = 4 * q - e0;  // row position of the quad's first element
        whole[k] = vec && q <= qb && tq >= 0 && tq + 4 <= L;
        // vec: stride == L and a 16-byte aligned cube, so row + tq == cube + 4 q
        if (whole[k]) c[k] = *reinterpret_cast<const float4*>(row + tq);
      }
#pragma unroll
      for (int k = 0; k < kNoiseQuads; ++k) {
        const long long q = base + threadIdx.x + k * kNoiseThreads;
        if (q > qb) continue;
        float z[4];
        quad_draws(philox4x32_10(U4{(uint32_t)q, (uint32_t)(q >> 32), 0u, 0u}, k0, k1),
                   distribution, z);
        const long long tq = 4 * q - e0;
        if (whole[k]) {
          float4 v = c[k];
          v.x = v.x + v.x * (sig * z[0]);
          v.y = v.y + v.y * (sig * z[1]);
          v.z = v.z + v.z * (sig * z[2]);
          v.w = v.w + v.w * (sig * z[3]);
          *reinterpret_cast<float4*>(row + tq) = v;
        } else {
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const long long t = tq + j;
            if (t >= 0 && t < L) {
              const float v = row[t];
              row[t] = v + v * (sig * z[j]);
            }
          }
        }
      }
    }
  }
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_flux_image(const float* cube, int64_t n_spaxels, int32_t n_wave_t,
                                int64_t spaxel_stride, float* flux, void* stream) {
  RUBIX_REQUIRE(n_spaxels >= 0 && n_wave_t >= 0 && spaxel_stride >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_flux_image: bad sizes");
  if (n_spaxels == 0) return RUBIX_OK;
  RUBIX_REQUIRE(cube && flux, RUBIX_E_INVALID, "rubix_flux_image: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int g = (int)std::min<long long>((n_spaxels * 32 + 255) / 256, (long long)sm_count() * 16);
  flux_image_kernel<<<g, 256, 0, st>>>(cube, n_spaxels, n_wave_t, spaxel_stride, flux);
  RUBIX_LAUNCH_CHECK("flux_image_kernel");
  return RUBIX_OK;
}

extern "C" size_t rubix_noise_median_workspace_size(void) { return sizeof(SelectState); }

extern "C" int rubix_noise_median(const float* flux, int64_t n, float* median, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n >= 0 && n < (1LL << 32), RUBIX_E_SHAPE, "rubix_noise_median: bad n");
  RUBIX_REQUIRE(median && (n == 0 || flux), RUBIX_E_INVALID, "rubix_noise_median: null pointer");
  RUBIX_REQUIRE(workspace && workspace_bytes >= sizeof(SelectState) &&
                    (reinterpret_cast<uintptr_t>(workspace) & 7) == 0,
                RUBIX_E_WORKSPACE, "rubix_noise_median: workspace of %zu bytes needed",
                sizeof(SelectState));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n <= (1LL << 20)) {
    select_block_kernel<<<1, 1024, 0, st>>>(flux, n, median);
    RUBIX_LAUNCH_CHECK("select_block_kernel");
    return RUBIX_OK;
  }
  SelectState* s = static_cast<SelectState*>(workspace);
  select_init_kernel<<<1, 1, 0, st>>>(s, n);
  RUBIX_LAUNCH_CHECK("select_init_kernel");
  if (n > 0) {
    const int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 4);
    for (int which = 0; which < 2; ++which) {
      unsigned mask = 0u;
      for (int shift = 24; shift >= 0; shift -= 8) {
        // the digits picked so far for this middle element live in bits[which]
        select_hist_kernel<<<g, 256, 0, st>>>(flux, n, shift, mask, which, s);
        RUBIX_LAUNCH_CHECK("select_hist_kernel");
        select_pick_kernel<<<1, 1, 0, st>>>(s, shift, which);
        RUBIX_LAUNCH_CHECK("select_pick_kernel");
        mask |= 255u << shift;
      }
    }
  }
  select_finish_kernel<<<1, 1, 0, st>>>(s, n, median);
  RUBIX_LAUNCH_CHECK("select_finish_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_apply_noise(float* cube, int64_t n_spaxels, int32_t n_wave_t,
                                 int64_t spaxel_stride, const float* flux, const float* median,
                                 float signal_to_noise, int32_t distribution, uint64_t seed,
                                 void* stream) {
  RUBIX_REQUIRE(n_spaxels >= 0 && n_wave_t >= 0 && spaxel_stride >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_apply_noise: bad sizes");
  RUBIX_REQUIRE(distribution == 0 || distribution == 1, RUBIX_E_INVALID,
                "rubix_apply_noise: distribution must be 0 (normal) or 1 (uniform)");
  RUBIX_REQUIRE(signal_to_noise > 0.f, RUBIX_E_INVALID,
                "rubix_apply_noise: signal_to_noise must be > 0");
  if (n_spaxels == 0 || n_wave_t == 0) return RUBIX_OK;
  RUBIX_REQUIRE(cube && flux && median, RUBIX_E_INVALID, "rubix_apply_noise: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  static int blocks_per_sm = 0;
  if (blocks_per_sm == 0) {
    RUBIX_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, noise_kernel,
                                                                 kNoiseThreads, 0));
    blocks_per_sm = std::max(blocks_per_sm, 1);
  }
  const int grid = (int)std::min<long long>(n_spaxels, (long long)sm_count() * blocks_per_sm);
  const int vec = spaxel_stride == n_wave_t && (reinterpret_cast<uintptr_t>(cube) & 15) == 0;
  noise_kernel<<<grid, kNoiseThreads, 0, st>>>(cube, n_spaxels, n_wave_t, spaxel_stride, flux,
                                               median, 1.0f / signal_to_noise, distribution,
                                               (uint32_t)seed, (uint32_t)(seed >> 32), vec);
  RUBIX_LAUNCH_CHECK("noise_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_philox4x32_10(const uint32_t* counter4, const uint32_t* key2,
                                   uint32_t* out4) {
  RUBIX_REQUIRE(counter4 && key2 && out4, RUBIX_E_INVALID, "rubix_philox4x32_10: null pointer");
  const U4 r = philox4x32_10(U4{counter4[0], counter4[1], counter4[2], counter4[3]}, key2[0],
                             key2[1]);
  out4[0] = r.x;
  out4[1] = r.y;
  out4[2] = r.z;
  out4[3] = r.w;
  return RUBIX_OK;
}
