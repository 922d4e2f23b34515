// Shared parts of the datacube kernels (forward accumulation and its adjoint):
// constants, the per-particle record, the setup passes over the SSP grid and the
// telescope grid, the gather of spaxel-sorted particles into records, the work-item
// list and the workspace carve-up.  Everything lives in an anonymous namespace: each
// translation unit that includes this header gets its own copy of the kernels.
#pragma once

#include "common.cuh"
#include "scan.cuh"

namespace rubix {

// Work-item tuning of the cube kernels, per device (tuning.cu; rubix_cube_tuning_set).
struct CubeTuning {
  int chunk;     // particles per work item, 32..256, multiple of 32
  int big_item;  // single-chunk spaxels with at least this many particles go first
};
CubeTuning cube_tuning_current();  // of the current device

namespace {

constexpr int kAccThreads = 384;  // forward kernel: 2 blocks of 12 warps per SM
constexpr int kAccWarps = kAccThreads / 32;
constexpr int kPB = 2;          // staging/row pools of the forward kernel: kPB full rows
constexpr int kMaxChunk = 256;  // largest work item (particles); records staged per item
constexpr int kMinChunk = 32;
constexpr int kBuckets = 1024;  // log-wavelength bucket table entries
constexpr double kVmaxKms = 10000.0;  // bucket table and one-step-walk check sized for this
constexpr int kMaxWaveT = 4096;  // telescope wavelengths per spectrum
constexpr int kGenericFlag = 1 << 30;  // in rec.b.z: particle needs the general walk
constexpr int kMaxLsfTaps = 63;

struct CubeCtrl {
  int next_item;
  int n_items;
  int error;               // 1: a TMA wait timed out
  unsigned dz_min_bits;    // min SSP spacing near the telescope range (float bits)
  unsigned dt_max_bits;    // max telescope bin width (float bits)
  float bmax;              // |B| limit: (vmax / c) / h
  double lnq0;             // log of the lowest wavelength covered by bucket 0
  double h;                // bucket width in log wavelength
  double inv_h;            // 1 / h
};

struct ParticleRec {  // 48 bytes, three vector loads
  float4 a;  // mass, alpha, B = (v/c)/h in bucket units, tz
  int4 b;    // cell (iz*(nA-1)+ia, -1 outside the grid), kstart, kend|flags, ta bits
  float4 c;  // T = in-range flux sum of the mixed template, dT/dZ, dT/dage (gradient
             // passes only), A_V of the dust in front of the particle (0 without dust)
};

__device__ __forceinline__ int count_le_scaled(const float* __restrict__ wz, int n, float alpha,
                                               float q) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__fmul_rn(wz[mid], alpha) <= q) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int count_le(const float* __restrict__ g, int n, float x) {
  if (x != x) return n;
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (g[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void bucket_params(const float* wave_t, int n_t, double& lnq0,
                                              double& h) {
  const double c = kSpeedOfLight;
  lnq0 = log((double)wave_t[0]) - kVmaxKms / c;
  const double hi = log((double)wave_t[n_t - 1]) + kVmaxKms / c;
  h = (hi - lnq0) / (double)(kBuckets - 2);
  if (!(h > 0.0)) h = 1e-6;
}

// Bucket table over log(q), per-wavelength bucket coordinates A_t, and the spacing
// extrema that decide whether the one-step walk is exact.  Any number of blocks;
// ctrl->dz_min_bits / dt_max_bits must be preset to 0xffffffff / 0.
__global__ void cube_setup_kernel(const float* __restrict__ wave_z, int n_wave,
                                  const float* __restrict__ wave_t, int n_t,
                                  CubeCtrl* __restrict__ ctrl, float* __restrict__ At,
                                  int2* __restrict__ bucket) {
  double lnq0, h;
  bucket_params(wave_t, n_t, lnq0, h);
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gsz = gridDim.x * blockDim.x;
  if (gtid == 0) {
    ctrl->next_item = 0;
    ctrl->error = 0;
    ctrl->lnq0 = lnq0;
    ctrl->h = h;
    ctrl->inv_h = 1.0 / h;
    ctrl->bmax = (float)(kVmaxKms / kSpeedOfLight / h);
  }
  for (int t = gtid; t < n_t; t += gsz) {
    At[t] = (float)((log((double)wave_t[t]) - lnq0) / h);
    if (t > 0) {
      float d = wave_t[t] - wave_t[t - 1];
      if (!(d >= 0.f)) d = 3.0e38f;  // non-ascending grid: disable the one-step walk
      atomicMax(&ctrl->dt_max_bits, __float_as_uint(d));
    }
  }
  // SSP spacing over the wavelengths any particle with |v| <= vmax can bracket.
  const double qlo = exp(lnq0) * 0.999, qhi = exp(lnq0 + (kBuckets - 2) * h) * 1.001;
  for (int k = gtid; k + 1 < n_wave; k += gsz) {
    const double a = wave_z[k], b = wave_z[k + 1];
    if (b >= qlo && a <= qhi) {
      float d = wave_z[k + 1] - wave_z[k];
      if (!(d > 0.f)) d = 0.f;
      atomicMin(&ctrl->dz_min_bits, __float_as_uint(d));
    }
  }
  for (int b = gtid; b < kBuckets; b += gsz) {
    // Bucket b covers u in [b - 0.5, b + 0.5) (round-to-nearest lookup).
    const double q = exp(lnq0 + ((double)b - 0.5) * h);
    int lo = 0, hi = n_wave;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if ((double)wave_z[mid] <= q) lo = mid + 1; else hi = mid;
    }
    const int k0 = lo - 1;
    float thr = 3.0e38f;
    if (k0 + 1 < n_wave) thr = (float)((log((double)wave_z[k0 + 1]) - lnq0) / h);
    bucket[b] = make_int2(k0, __float_as_int(thr));
  }
}

// Corner table: ct[(iz*(nA-1) + ia)*nW + k] = (F[iz][ia][k], F[iz+1][ia][k],
// F[iz][ia+1][k], F[iz+1][ia+1][k]).
__global__ void cube_corner_table_kernel(const float* __restrict__ flux, int nZ, int nA,
                                         int nW, float4* __restrict__ ct) {
  const long long total = (long long)(nZ - 1) * (nA - 1) * nW;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long cell = i / nW;
    const int k = (int)(i - cell * nW);
    const int iz = (int)(cell / (nA - 1)), ia = (int)(cell - (long long)iz * (nA - 1));
    const long long b00 = ((long long)iz * nA + ia) * nW + k;
    const long long b10 = b00 + (long long)nA * nW;
    ct[i] = make_float4(flux[b00], flux[b10], flux[b00 + nW], flux[b10 + nW]);
  }
}

// prefix[r][k] = sum_{k'=1..k} F[r][k'] * (lambda_z,k' - lambda_z,k'-1) for every SSP row
// r (float64), prefix[r][0] = 0.  With it the in-range flux sum of a particle,
// T = sum_{k in mask} G_k (lambda'_k - lambda'_{k-1}) (rubix/spectra/ifu.py:241-245),
// is alpha * sum_c w_c (prefix[c][kb] - prefix[c][ka-1]): the float32 rounding of
// lambda'_k = fl32(lambda_z,k * alpha) enters that sum only through telescoping
// differences, ~1e-7 relative.
constexpr int kPrefixThreads = 128;

// Per SSP row r: prefix[r][k] = sum_{j=1..k} F[r][j] (lambda_z[j] - lambda_z[j-1]) in
// float64.  One block per row: each thread sums a run of consecutive entries, a block
// scan of the run totals gives each run's offset, and the run is written out.
__global__ void __launch_bounds__(kPrefixThreads) cube_prefix_kernel(
    const float* __restrict__ flux, int rows, int nW, const float* __restrict__ wave_z,
    double* __restrict__ prefix) {
  __shared__ double s_warp[kPrefixThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int per = (nW + kPrefixThreads - 1) / kPrefixThreads;
  const int k0 = threadIdx.x * per;
  const int k1 = min(k0 + per, nW);
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const float* f = flux + (long long)r * nW;
    double* o = prefix + (long long)r * nW;
    double sum = 0.0;
    for (int k = max(k0, 1); k < k1; ++k) sum += (double)f[k] * (double)(wave_z[k] - wave_z[k - 1]);
    double x = sum;  // inclusive scan over the block's runs
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    double run = x - sum;
    for (int w = 0; w < warp; ++w) run += s_warp[w];
    for (int k = k0; k < k1; ++k) {
      if (k >= 1) run += (double)f[k] * (double)(wave_z[k] - wave_z[k - 1]);
      o[k] = run;
    }
    __syncthreads();  // s_warp is reused by the next row
  }
}

__global__ void cube_gather_kernel(const float* __restrict__ mass, const float* __restrict__ met,
                                   const float* __restrict__ age, const float* __restrict__ vel,
                                   long long vel_stride, int vel_comp,
                                   const int* __restrict__ perm, const int* __restrict__ seg_off,
                                   int n_seg, long long n, const float* __restrict__ zg, int nZ,
                                   const float* __restrict__ ag, int nA,
                                   const float* __restrict__ wave_z, int n_wave,
                                   const float* __restrict__ wave_t, int n_t,
                                   const double* __restrict__ prefix,
                                   const CubeCtrl* __restrict__ ctrl,
                                   ParticleRec* __restrict__ rec, int with_grad,
                                   const float* __restrict__ av, float alo, float ahi) {
  const long long n_valid = seg_off[n_seg];
  const float t_lo = wave_t[0], t_hi = wave_t[n_t - 1];
  const double inv_h = ctrl->inv_h;
  const float bmax = ctrl->bmax;
  // lambda' spacing >= alpha*dz minus two float32 roundings of lambda' (|lambda'| < 2^14)
  const float dz = __uint_as_float(ctrl->dz_min_bits), dt = __uint_as_float(ctrl->dt_max_bits);
  const bool coarse_ok = dz * alo - 4.0e-3f > dt;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n && j < n_valid;
       j += (long long)gridDim.x * blockDim.x) {
    const long long i = perm[j];
    const float Z = met[i], A = age[i], m = mass[i];
    const float v = vel[i * vel_stride + vel_comp];
    // interpax.interp2d(method="linear"): cell from searchsorted(side='right').
    const int iz = min(max(count_le(zg, nZ, Z), 1), nZ - 1);
    const int ia = min(max(count_le(ag, nA, A), 1), nA - 1);
    const float dzg = zg[iz] - zg[iz - 1], dag = ag[ia] - ag[ia - 1];
    const float tz = dzg == 0.f ? 0.f : (Z - zg[iz - 1]) / dzg;
    const float ta = dag == 0.f ? 0.f : (A - ag[ia - 1]) / dag;
    const bool outside = (Z < zg[0]) || (Z > zg[nZ - 1]) || (A < ag[0]) || (A > ag[nA - 1]);
    const int cell = outside ? -1 : (iz - 1) * (nA - 1) + (ia - 1);
    const float alpha = doppler_factor(v);
    // B only seeds the bracket search (first_bracket corrects it exactly)
    float B = (float)((double)v * (1.0 / kSpeedOfLight) * inv_h);
    B = fminf(fmaxf(B, -bmax), bmax);
    const int ks = count_le_scaled(wave_z, n_wave, alpha, t_lo) - 1;
    const int ke_raw = count_le_scaled(wave_z, n_wave, alpha, t_hi) - 1;
    int ke = ke_raw;
    ke = max(ke, ks);  // keeps the shared-memory row non-empty for any input grid
    const bool coarse = coarse_ok && alpha >= alo && alpha <= ahi;
    // In-range flux sum T: entries ka..kb with t_lo <= lambda'_k <= t_hi, k >= 1.
    float T = 0.f;
    double TZ = 0.0, TA = 0.0;
    if (cell >= 0) {
      int ka = (ks >= 0 && __fmul_rn(wave_z[ks], alpha) >= t_lo) ? ks : ks + 1;
      ka = max(ka, 1);
      const int kb = min(ke_raw, n_wave - 1);
      if (ka <= kb) {
        const long long r00 = (long long)(iz - 1) * nA + (ia - 1);
        const long long rr[4] = {r00, r00 + nA, r00 + 1, r00 + nA + 1};  // 00, 10, 01, 11
        // float64 differences of the float64 prefix sums, mixed in float32 (rubix's
        // sum is float32 throughout)
        const float w[4] = {(1.f - tz) * (1.f - ta), tz * (1.f - ta), (1.f - tz) * ta,
                            tz * ta};
        double d[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          d[c] = prefix[rr[c] * n_wave + kb] - prefix[rr[c] * n_wave + ka - 1];
          T = fmaf(w[c], (float)d[c], T);
        }
        T *= alpha;
        if (with_grad) {
          // dT/dZ and dT/d(age): the bilinear weights' derivatives, same sums
          const double iz_w = dzg == 0.f ? 0.0 : 1.0 / (double)dzg;
          const double ia_w = dag == 0.f ? 0.0 : 1.0 / (double)dag;
          TZ = (double)alpha * iz_w *
               ((1.0 - ta) * (d[1] - d[0]) + (double)ta * (d[3] - d[2]));
          TA = (double)alpha * ia_w *
               ((1.0 - tz) * (d[2] - d[0]) + (double)tz * (d[3] - d[1]));
        }
      }
    }
    ParticleRec r;
    r.a = make_float4(m, alpha, B, tz);
    r.b = make_int4(cell, ks, ke | (coarse ? 0 : kGenericFlag), __float_as_int(ta));
    r.c = make_float4(T, (float)TZ, (float)TA, av ? av[i] : 0.f);
    rec[j] = r;
  }
}

// Per spaxel: chunk count.  Multi-chunk spaxels get one item (and partial slot) per
// chunk; single-chunk spaxels are split into a "big" and a "small" class.
__global__ void cube_count_kernel(const int* __restrict__ seg_off, int n_seg, int chunk,
                                  int big_item, int* __restrict__ slot_cnt,
                                  int* __restrict__ big_cnt, int* __restrict__ small_cnt) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_seg; s += gridDim.x * blockDim.x) {
    const int cnt = seg_off[s + 1] - seg_off[s];
    const int nch = cnt <= chunk ? 1 : (cnt + chunk - 1) / chunk;
    slot_cnt[s] = nch > 1 ? nch : 0;
    big_cnt[s] = (nch == 1 && cnt >= big_item) ? 1 : 0;
    small_cnt[s] = (nch == 1 && cnt < big_item) ? 1 : 0;
  }
}

// Item order: chunks of multi-chunk spaxels (item index = partial slot), then big
// single-chunk spaxels, then the rest.
__global__ void cube_fill_items_kernel(const int* __restrict__ seg_off, int n_seg, int chunk,
                                       int big_item, const int* __restrict__ slot_start,
                                       const int* __restrict__ big_start,
                                       const int* __restrict__ small_start,
                                       int2* __restrict__ items, CubeCtrl* __restrict__ ctrl) {
  const int total_slots = slot_start[n_seg];
  const int total_big = big_start[n_seg];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_seg; s += gridDim.x * blockDim.x) {
    const int cnt = seg_off[s + 1] - seg_off[s];
    if (cnt > chunk) {
      const int nch = (cnt + chunk - 1) / chunk;
      for (int c = 0; c < nch; ++c) items[slot_start[s] + c] = make_int2(s, c);
    } else if (cnt >= big_item) {
      items[total_slots + big_start[s]] = make_int2(s, 0);
    } else {
      items[total_slots + total_big + small_start[s]] = make_int2(s, 0);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0)
    ctrl->n_items = total_slots + total_big + small_start[n_seg];
}

struct CubeLayout {
  CubeCtrl* ctrl;
  float* At;
  int2* bucket;
  float4* ct;
  double* prefix;
  ParticleRec* rec;
  int* slot_cnt;
  int* big_cnt;
  int* small_cnt;
  int2* items;
  int* done;
  float* partials;
  size_t bytes;
};

long long max_slots(long long n, int chunk) { return 2 * ((n + chunk - 1) / chunk); }

CubeLayout carve_cube(void* ws, long long n, int n_seg, int n_t, int nZ, int nA, int nW,
                      int chunk) {
  Carve c(ws);
  CubeLayout L;
  L.ctrl = c.take<CubeCtrl>(1);
  L.At = c.take<float>((size_t)n_t);
  L.bucket = c.take<int2>(kBuckets);
  L.ct = c.take<float4>((size_t)(nZ > 1 ? nZ - 1 : 0) * (nA > 1 ? nA - 1 : 0) * nW);
  L.prefix = c.take<double>((size_t)nZ * nA * nW);
  L.rec = c.take<ParticleRec>((size_t)(n > 0 ? n : 1));
  L.slot_cnt = c.take<int>((size_t)n_seg + 1);
  L.big_cnt = c.take<int>((size_t)n_seg + 1);
  L.small_cnt = c.take<int>((size_t)n_seg + 1);
  L.items = c.take<int2>((size_t)(max_slots(n, chunk) + n_seg));
  L.done = c.take<int>((size_t)n_seg);
  L.partials = c.take<float>((size_t)max_slots(n, chunk) * n_t);
  L.bytes = c.off;
  return L;
}

// Work-item tuning of the cube kernels (set per device through rubix_cube_tuning_set;
// defined in tuning.cu).

// Everything the setup passes read: the SSP grid, the telescope grid and the
// spaxel-sorted particles.
struct CubeInputs {
  const float* ssp_flux;
  const float* ssp_met;
  const float* ssp_age;
  const float* ssp_wave_z;
  int n_met, n_age, n_wave;
  const float* wave_t;
  int n_wave_t;
  const float* mass;
  const float* met;
  const float* age;
  const float* vel;
  long long vel_stride;
  int vel_comp;
  const int* perm;
  const int* seg_off;
  int n_seg;
  long long n;
  const float* av = nullptr;  // per-particle A_V (dust), input order; nullptr: none
};

// Launches the setup passes into the carved workspace: bucket table, corner table,
// prefix sums, particle records (with dT/dZ, dT/dage when with_grad) and the work-item
// list.  Six to eight kernels plus three small memsets on stream st.
inline int cube_prepare(const CubeInputs& in, const CubeLayout& L, const CubeTuning& tune,
                        bool with_grad, cudaStream_t st) {
  RUBIX_CUDA_TRY(cudaMemsetAsync(&L.ctrl->dz_min_bits, 0xff, sizeof(unsigned), st));
  RUBIX_CUDA_TRY(cudaMemsetAsync(&L.ctrl->dt_max_bits, 0, sizeof(unsigned), st));
  {
    const int work = std::max(std::max(in.n_wave_t, in.n_wave), kBuckets);
    cube_setup_kernel<<<div_up(work, 128), 128, 0, st>>>(in.ssp_wave_z, in.n_wave, in.wave_t,
                                                         in.n_wave_t, L.ctrl, L.At, L.bucket);
    RUBIX_LAUNCH_CHECK("cube_setup_kernel");
  }
  {
    const long long total = (long long)(in.n_met - 1) * (in.n_age - 1) * in.n_wave;
    const int g = (int)std::min<long long>((total + 255) / 256, (long long)sm_count() * 8);
    cube_corner_table_kernel<<<g, 256, 0, st>>>(in.ssp_flux, in.n_met, in.n_age, in.n_wave,
                                                L.ct);
    RUBIX_LAUNCH_CHECK("cube_corner_table_kernel");
    const int rows = in.n_met * in.n_age;
    const int pg = std::min(rows, sm_count() * 16);
    cube_prefix_kernel<<<pg, kPrefixThreads, 0, st>>>(in.ssp_flux, rows, in.n_wave,
                                                      in.ssp_wave_z, L.prefix);
    RUBIX_LAUNCH_CHECK("cube_prefix_kernel");
  }
  if (in.n > 0) {
    const int g = (int)std::min<long long>((in.n + 255) / 256, (long long)sm_count() * 8);
    cube_gather_kernel<<<g, 256, 0, st>>>(in.mass, in.met, in.age, in.vel, in.vel_stride,
                                          in.vel_comp, in.perm, in.seg_off, in.n_seg, in.n,
                                          in.ssp_met, in.n_met, in.ssp_age, in.n_age,
                                          in.ssp_wave_z, in.n_wave, in.wave_t, in.n_wave_t,
                                          L.prefix, L.ctrl, L.rec, with_grad ? 1 : 0, in.av,
                                          (float)std::exp(-kVmaxKms / kSpeedOfLight),
                                          (float)std::exp(kVmaxKms / kSpeedOfLight));
    RUBIX_LAUNCH_CHECK("cube_gather_kernel");
  }
  {
    const int g = (int)std::min<long long>((in.n_seg + 255) / 256, (long long)sm_count() * 8);
    cube_count_kernel<<<g, 256, 0, st>>>(in.seg_off, in.n_seg, tune.chunk, tune.big_item,
                                         L.slot_cnt, L.big_cnt, L.small_cnt);
    RUBIX_LAUNCH_CHECK("cube_count_kernel");
    scan_exclusive_3<<<3, 1024, 0, st>>>(L.slot_cnt, L.big_cnt, L.small_cnt, in.n_seg);
    RUBIX_LAUNCH_CHECK("scan_exclusive_3");
    cube_fill_items_kernel<<<g, 256, 0, st>>>(in.seg_off, in.n_seg, tune.chunk,
                                              tune.big_item, L.slot_cnt, L.big_cnt,
                                              L.small_cnt, L.items, L.ctrl);
    RUBIX_LAUNCH_CHECK("cube_fill_items_kernel");
    RUBIX_CUDA_TRY(cudaMemsetAsync(L.done, 0, sizeof(int) * (size_t)in.n_seg, st));
  }
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix
