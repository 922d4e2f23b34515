// Kernel (b): fused SSP lookup (bilinear in metallicity and age), mass scaling,
// Doppler shift, flux-conserving resampling onto the telescope grid and the
// per-spaxel accumulation of the datacube.
//
// Work decomposition
//   * Particles arrive sorted by spaxel (kernel (a)).  A setup pass gathers each
//     particle into a 32-byte record (mass, Doppler factor, interpolation cell and
//     weights, first/last SSP bracket of the telescope range).
//   * Work items are (spaxel, chunk of <= kChunk particles).  A persistent kernel
//     pulls items from an atomic counter.  A block of 256 threads owns the whole
//     telescope grid of its spaxel: thread `tid` holds t = tid + 256*r, r < R, in
//     registers (wavelength, bin width, bucket coordinate, accumulator).
//   * Per batch of kPB particles the block builds, in shared memory, the particle's
//     mixed template row restricted to the telescope range: entry k holds
//     (lambda'_k, slope_k, G_k, lambda'_{k+1}) with lambda'_k = fl32(lambda_z,k *
//     fl32(exp(v/c))) -- the float32 grid rubix materialises -- and the in-range
//     flux sum T.  Each thread then interpolates its R wavelengths (bracket from a
//     log-wavelength bucket table, corrected by exact comparisons on lambda'),
//     keeps the values in registers and sums T' = sum_t I_t dlambda_t.  One block
//     reduction per batch gives s = nan_to_num(T/T'), and the accumulators take
//     mass * s * I.  No particle spectrum is ever written to memory.
//   * Spaxels with more than kChunk particles are split; each chunk writes a partial
//     spectrum to the workspace and the last chunk to finish sums the partials in
//     chunk order (Kahan), so the cube is bit-reproducible with no float atomics.
#include "common.cuh"
#include "scan.cuh"

namespace rubix {
namespace {

constexpr int kAccThreads = 256;
constexpr int kAccWarps = kAccThreads / 32;
constexpr int kPB = 2;          // particles per batch
constexpr int kChunk = 512;     // particles per work item
constexpr int kBuckets = 2048;  // log-wavelength bucket table entries
constexpr double kVmaxKms = 10000.0;  // bucket table sized for |v| <= 10^4 km/s
constexpr int kMaxWaveT = kAccThreads * 16;

struct CubeCtrl {
  int next_item;
  int n_items;
  int error;
  int pad0;
  double lnq0;   // log of the lowest wavelength covered by bucket 0
  double h;      // bucket width in log wavelength
  float bmax;    // |B| clamp in bucket units
  float pad1[3];
};

struct ParticleRec {  // 32 bytes, two vector loads
  float4 a;  // mass, alpha = fl32(exp(v/c)), B = (v/c)/h (bucket units), tz
  int4 b;    // cell (lower corner iz*nA+ia, -1 if outside), kstart, kend, ta bits
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

// Bucket table over log(q) and per-wavelength bucket coordinates A_t.
__global__ void cube_setup_kernel(const float* __restrict__ wave_z, int n_wave,
                                  const float* __restrict__ wave_t, int n_t,
                                  CubeCtrl* __restrict__ ctrl, float* __restrict__ At,
                                  int2* __restrict__ bucket) {
  __shared__ double s_lnq0, s_h;
  if (threadIdx.x == 0) {
    const double c = kSpeedOfLight;
    double lo = log((double)wave_t[0]) - kVmaxKms / c;
    double hi = log((double)wave_t[n_t - 1]) + kVmaxKms / c;
    double h = (hi - lo) / (double)(kBuckets - 2);
    if (!(h > 0.0)) h = 1e-6;
    s_lnq0 = lo;
    s_h = h;
    ctrl->next_item = 0;
    ctrl->error = 0;
    ctrl->lnq0 = lo;
    ctrl->h = h;
    ctrl->bmax = (float)((kVmaxKms / c) / h);
  }
  __syncthreads();
  const double lnq0 = s_lnq0, h = s_h;
  for (int t = threadIdx.x; t < n_t; t += blockDim.x)
    At[t] = (float)((log((double)wave_t[t]) - lnq0) / h);
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) {
    // Bucket b covers u in [b - 0.5, b + 0.5) (round-to-nearest lookup).
    double q = exp(lnq0 + ((double)b - 0.5) * h);
    int lo = 0, hi = n_wave;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if ((double)wave_z[mid] <= q) lo = mid + 1; else hi = mid;
    }
    int k0 = lo - 1;
    float thr = 3.0e38f;
    if (k0 + 1 < n_wave) thr = (float)((log((double)wave_z[k0 + 1]) - lnq0) / h);
    bucket[b] = make_int2(k0, __float_as_int(thr));
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
                                   const CubeCtrl* __restrict__ ctrl,
                                   ParticleRec* __restrict__ rec) {
  const long long n_valid = seg_off[n_seg];
  const float t_lo = wave_t[0], t_hi = wave_t[n_t - 1];
  const double h = ctrl->h;
  const float bmax = ctrl->bmax;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n && j < n_valid;
       j += (long long)gridDim.x * blockDim.x) {
    const long long i = perm[j];
    const float Z = met[i], A = age[i], m = mass[i];
    const float v = vel[i * vel_stride + vel_comp];
    // interpax.interp2d(method="linear"): cell from searchsorted(side='right').
    int iz = min(max(count_le(zg, nZ, Z), 1), nZ - 1);
    int ia = min(max(count_le(ag, nA, A), 1), nA - 1);
    float dz = zg[iz] - zg[iz - 1], da = ag[ia] - ag[ia - 1];
    float tz = dz == 0.f ? 0.f : (Z - zg[iz - 1]) / dz;
    float ta = da == 0.f ? 0.f : (A - ag[ia - 1]) / da;
    bool outside = (Z < zg[0]) || (Z > zg[nZ - 1]) || (A < ag[0]) || (A > ag[nA - 1]);
    int cell = outside ? -1 : (iz - 1) * nA + (ia - 1);
    const double vc = (double)v / kSpeedOfLight;
    const float alpha = (float)exp(vc);
    float B = (float)(vc / h);
    B = fminf(fmaxf(B, -bmax), bmax);
    int ks = count_le_scaled(wave_z, n_wave, alpha, t_lo) - 1;
    int ke = count_le_scaled(wave_z, n_wave, alpha, t_hi) - 1;
    ke = max(ke, ks);  // keeps the shared-memory row non-empty for any input grid
    ParticleRec r;
    r.a = make_float4(m, alpha, B, tz);
    r.b = make_int4(cell, ks, ke, __float_as_int(ta));
    rec[j] = r;
  }
}

// Per spaxel: number of chunks; multi-chunk spaxels get slots, the others a flag.
__global__ void cube_count_kernel(const int* __restrict__ seg_off, int n_seg,
                                  int* __restrict__ slot_cnt, int* __restrict__ single_cnt) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_seg; s += gridDim.x * blockDim.x) {
    int cnt = seg_off[s + 1] - seg_off[s];
    int nch = cnt <= kChunk ? 1 : (cnt + kChunk - 1) / kChunk;
    slot_cnt[s] = nch > 1 ? nch : 0;
    single_cnt[s] = nch > 1 ? 0 : 1;
  }
}

// Items [0, total_slots) are the chunks of multi-chunk spaxels (item = partial slot),
// then one item per single-chunk spaxel.
__global__ void cube_fill_items_kernel(const int* __restrict__ seg_off, int n_seg,
                                       const int* __restrict__ slot_start,
                                       const int* __restrict__ single_start,
                                       int2* __restrict__ items, CubeCtrl* __restrict__ ctrl) {
  const int total_slots = slot_start[n_seg];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_seg; s += gridDim.x * blockDim.x) {
    int cnt = seg_off[s + 1] - seg_off[s];
    if (cnt > kChunk) {
      int nch = (cnt + kChunk - 1) / kChunk;
      for (int c = 0; c < nch; ++c) items[slot_start[s] + c] = make_int2(s, c);
    } else {
      items[total_slots + single_start[s]] = make_int2(s, 0);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->n_items = total_slots + single_start[n_seg];
}

struct MainArgs {
  const float* flux;
  const float* wave_z;
  int nZ, nA, n_wave;
  const float* wave_t;
  const float* At;
  int n_t;
  const ParticleRec* rec;
  const int* seg_off;
  const int* slot_start;
  const int2* items;
  int* done;
  float* partials;
  float* cube;
  long long spaxel_stride;
  CubeCtrl* ctrl;
  const int2* bucket;
  int row_cap;
};

struct alignas(16) BatchMeta {
  int ks[kPB];
  int ke[kPB];
  float B[kPB];
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Builds the shared-memory rows of particles [j0, j0+cnt) and writes each
// particle's partial in-range flux sums T into red[.].x.
__device__ __forceinline__ void build_rows(const MainArgs& a, long long j0, int cnt,
                                           float4* __restrict__ rows, BatchMeta* meta,
                                           float2* red, float* red_m, int lane, int warp) {
  const float t_lo = a.wave_t[0], t_hi = a.wave_t[a.n_t - 1];
  const int nW = a.n_wave;
  for (int p = 0; p < cnt; ++p) {
    const ParticleRec r = a.rec[j0 + p];
    const float m = r.a.x, alpha = r.a.y, tz = r.a.w;
    const int cell = r.b.x, ks = r.b.y, ke = r.b.z;
    const float ta = __int_as_float(r.b.w);
    if (threadIdx.x == 0) {
      meta->ks[p] = ks;
      meta->ke[p] = ke;
      meta->B[p] = r.a.z;
      red_m[p] = m;
    }
    const float w00 = (1.f - tz) * (1.f - ta), w10 = tz * (1.f - ta);
    const float w01 = (1.f - tz) * ta, w11 = tz * ta;
    const float* f00 = a.flux + (long long)(cell < 0 ? 0 : cell) * nW;
    const float* f10 = f00 + (long long)a.nA * nW;
    const float* f01 = f00 + nW;
    const float* f11 = f10 + nW;
    float4* row = rows + p * a.row_cap;
    const int n_e = ke - ks + 1;
    float tsum = 0.f;
    for (int base = warp * 31; base < n_e; base += kAccWarps * 31) {
      const int e = base + lane;
      const int k = ks + e;  // in [-1, nW]
      float lp, G;
      {
        const int kk = min(max(k, 0), nW - 1);
        G = 0.f;
        if (cell >= 0) {
          G = w00 * __ldg(f00 + kk);
          G = fmaf(w10, __ldg(f10 + kk), G);
          G = fmaf(w01, __ldg(f01 + kk), G);
          G = fmaf(w11, __ldg(f11 + kk), G);
        }
        lp = (k < 0) ? -kFltMax : (k >= nW ? kFltMax : __fmul_rn(__ldg(a.wave_z + k), alpha));
      }
      const float lp_next = __shfl_down_sync(0xffffffffu, lp, 1);
      const float G_next = __shfl_down_sync(0xffffffffu, G, 1);
      float lp_prev = __shfl_up_sync(0xffffffffu, lp, 1);
      if (lane == 0)
        lp_prev = (k - 1 >= 0 && k - 1 < nW) ? __fmul_rn(__ldg(a.wave_z + k - 1), alpha) : lp;
      if (lane < 31 && e < n_e) {
        float slope = 0.f;
        if (k >= 0 && k + 1 < nW) {
          const float dl = lp_next - lp;
          slope = dl > 0.f ? __fdividef(G_next - G, dl) : 0.f;
        }
        const float lpx = lp;
        const float lpw = (k + 1 >= nW) ? kFltMax : lp_next;
        row[e] = make_float4(lpx, slope, G, lpw);
        // T term: G_k * (lambda'_k - lambda'_{k-1}) for lambda'_k inside the telescope range.
        if (k >= 1 && k < nW && lp >= t_lo && lp <= t_hi) tsum = fmaf(G, lp - lp_prev, tsum);
      }
    }
    tsum = warp_sum(tsum);
    if (lane == 0) red[warp * kPB + p].x = tsum;
  }
}

template <int R>
__global__ void __launch_bounds__(kAccThreads, 2) cube_main_kernel(MainArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  int2* s_bucket = reinterpret_cast<int2*>(smem);
  float4* s_rows = reinterpret_cast<float4*>(smem + sizeof(int2) * kBuckets);  // [2][kPB][row_cap]
  float2* s_red = reinterpret_cast<float2*>(s_rows + 2 * kPB * a.row_cap);       // [3][warps][kPB]
  float* s_redm = reinterpret_cast<float*>(s_red + 3 * kAccWarps * kPB);         // [3][kPB]
  BatchMeta* s_meta = reinterpret_cast<BatchMeta*>(s_redm + 4 * kPB);            // [2]
  __shared__ int s_item, s_last;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int b = tid; b < kBuckets; b += kAccThreads) s_bucket[b] = a.bucket[b];

  const int n_t = a.n_t;
  float A[R], lam[R], dlam[R], acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    int t = tid + r * kAccThreads;
    int tc = t < n_t ? t : n_t - 1;
    A[r] = a.At[tc];
    lam[r] = a.wave_t[tc];
    dlam[r] = (t < n_t && t > 0) ? (a.wave_t[t] - a.wave_t[t - 1]) : 0.f;
  }
  const int n_items = a.ctrl->n_items;
  __syncthreads();

  for (;;) {
    if (tid == 0) s_item = atomicAdd(&a.ctrl->next_item, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= n_items) break;
    const int2 it = a.items[item];
    const int s = it.x, chunk = it.y;
    const int seg_b = a.seg_off[s], seg_e = a.seg_off[s + 1];
    const int cnt_s = seg_e - seg_b;
    const long long jb = (long long)seg_b + (long long)chunk * kChunk;
    const long long je = min((long long)seg_e, jb + kChunk);
    const int np = (int)(je - jb);
    const int nbatch = (np + kPB - 1) / kPB;

#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = 0.f;

    if (nbatch > 0) {
      build_rows(a, jb, min(kPB, np), s_rows, &s_meta[0], s_red, s_redm, lane, warp);
      __syncthreads();
    }
    for (int bt = 0; bt < nbatch; ++bt) {
      const int buf = bt & 1, slot = bt % 3;
      const int cnt = min(kPB, np - bt * kPB);
      float I[kPB][R];
      const BatchMeta meta = s_meta[buf];
#pragma unroll
      for (int p = 0; p < kPB; ++p) {
        if (p < cnt) {
          const int ks = meta.ks[p], ke = meta.ke[p];
          const float B = meta.B[p];
          const float4* rowp = s_rows + (buf * kPB + p) * a.row_cap - ks;
          float tp = 0.f;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float u = A[r] - B;
            int b = __float_as_int(u + 12582912.0f) - 0x4B400000;
            b = min(max(b, 0), kBuckets - 1);
            const int2 te = s_bucket[b];
            int k = te.x + (u >= __int_as_float(te.y) ? 1 : 0);
            k = min(max(k, ks), ke);
            float4 e = rowp[k];
            const float x = lam[r];
            if (x < e.x) {
              while (k > ks && x < e.x) { --k; e = rowp[k]; }
            } else if (x >= e.w) {
              while (k < ke && x >= e.w) { ++k; e = rowp[k]; }
            }
            const float v = fmaf(x - e.x, e.y, e.z);
            I[p][r] = v;
            tp = fmaf(v, dlam[r], tp);
          }
          tp = warp_sum(tp);
          if (lane == 0) s_red[(slot * kAccWarps + warp) * kPB + p].y = tp;
        }
      }
      if (bt + 1 < nbatch) {
        const int nslot = (bt + 1) % 3;
        build_rows(a, jb + (long long)(bt + 1) * kPB, min(kPB, np - (bt + 1) * kPB),
                   s_rows + (buf ^ 1) * kPB * a.row_cap, &s_meta[buf ^ 1],
                   s_red + nslot * kAccWarps * kPB, s_redm + nslot * kPB, lane, warp);
      }
      __syncthreads();
      float beta[kPB];
#pragma unroll
      for (int p = 0; p < kPB; ++p) {
        beta[p] = 0.f;
        if (p < cnt) {
          float T = 0.f, Tn = 0.f;
#pragma unroll
          for (int w = 0; w < kAccWarps; ++w) {
            float2 v = s_red[(slot * kAccWarps + w) * kPB + p];
            T += v.x;
            Tn += v.y;
          }
          const float m = s_redm[slot * kPB + p];
          float sc = T / Tn;
          if (sc != sc) sc = 0.f;
          if (isinf(sc)) sc = copysignf(kFltMax, sc);
          beta[p] = (m == 0.f) ? 0.f : m * sc;
        }
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        float add = beta[0] * I[0][r];
#pragma unroll
        for (int p = 1; p < kPB; ++p)
          if (p < cnt) add = fmaf(beta[p], I[p][r], add);
        acc[r] += add;
      }
    }

    const int nch = cnt_s <= kChunk ? 1 : (cnt_s + kChunk - 1) / kChunk;
    if (nch == 1) {
      float* out = a.cube + (long long)s * a.spaxel_stride;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int t = tid + r * kAccThreads;
        if (t < n_t) out[t] = acc[r];
      }
    } else {
      float* part = a.partials + (long long)item * n_t;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int t = tid + r * kAccThreads;
        if (t < n_t) part[t] = acc[r];
      }
      __threadfence();
      __syncthreads();
      if (tid == 0) s_last = (atomicAdd(&a.done[s], 1) == nch - 1) ? 1 : 0;
      __syncthreads();
      if (s_last) {
        __threadfence();
        const long long slot0 = a.slot_start[s];
        float* out = a.cube + (long long)s * a.spaxel_stride;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          int t = tid + r * kAccThreads;
          if (t < n_t) {
            float sum = 0.f, comp = 0.f;
            for (int c = 0; c < nch; ++c) {
              float y = __ldcg(a.partials + (slot0 + c) * n_t + t) - comp;
              float tt = sum + y;
              comp = (tt - sum) - y;
              sum = tt;
            }
            out[t] = sum;
          }
        }
      }
    }
    __syncthreads();
  }
}

struct CubeLayout {
  CubeCtrl* ctrl;
  float* At;
  int2* bucket;
  ParticleRec* rec;
  int* slot_cnt;
  int* single_cnt;
  int2* items;
  int* done;
  float* partials;
  size_t bytes;
};

long long max_slots(long long n) { return 2 * ((n + kChunk - 1) / kChunk); }

CubeLayout carve_cube(void* ws, long long n, int n_seg, int n_t) {
  Carve c(ws);
  CubeLayout L;
  L.ctrl = c.take<CubeCtrl>(1);
  L.At = c.take<float>((size_t)n_t);
  L.bucket = c.take<int2>(kBuckets);
  L.rec = c.take<ParticleRec>((size_t)(n > 0 ? n : 1));
  L.slot_cnt = c.take<int>((size_t)n_seg + 1);
  L.single_cnt = c.take<int>((size_t)n_seg + 1);
  L.items = c.take<int2>((size_t)(max_slots(n) + n_seg));
  L.done = c.take<int>((size_t)n_seg);
  L.partials = c.take<float>((size_t)max_slots(n) * n_t);
  L.bytes = c.off;
  return L;
}

template <int R>
int launch_main(const MainArgs& args, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(cube_main_kernel<R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess)
    return set_error(RUBIX_E_CUDA, "cudaFuncSetAttribute(cube_main_kernel): %s",
                     cudaGetErrorString(e));
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cube_main_kernel<R>, kAccThreads,
                                                    smem);
  if (e != cudaSuccess || per_sm < 1)
    return set_error(RUBIX_E_UNSUPPORTED,
                     "cube_main_kernel does not fit on an SM with %zu bytes of shared memory",
                     smem);
  int grid = sm_count() * per_sm;
  cube_main_kernel<R><<<grid, kAccThreads, smem, st>>>(args);
  RUBIX_LAUNCH_CHECK("cube_main_kernel");
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" size_t rubix_cube_workspace_size(int64_t n, int32_t n_segments, int32_t n_wave_t,
                                            int32_t n_wave) {
  (void)n_wave;
  if (n < 0 || n_segments < 0 || n_wave_t < 0) return 0;
  return carve_cube(nullptr, n, n_segments, n_wave_t).bytes;
}

extern "C" int rubix_cube_fwd(const float* ssp_flux, const float* ssp_metallicity,
                              const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                              int32_t n_age, int32_t n_wave, const float* wave_t,
                              int32_t n_wave_t, const float* mass, const float* metallicity,
                              const float* age, const float* velocity, int64_t vel_stride,
                              int32_t vel_component, const int32_t* perm,
                              const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                              float* cube, int64_t spaxel_stride, void* workspace,
                              size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n >= 0 && n < (1LL << 31), RUBIX_E_SHAPE, "rubix_cube_fwd: bad n");
  RUBIX_REQUIRE(n_segments >= 0, RUBIX_E_SHAPE, "rubix_cube_fwd: n_segments < 0");
  RUBIX_REQUIRE(n_met >= 2 && n_age >= 2, RUBIX_E_SHAPE,
                "rubix_cube_fwd: SSP grid needs >= 2 metallicities and >= 2 ages");
  RUBIX_REQUIRE(n_wave >= 2, RUBIX_E_SHAPE, "rubix_cube_fwd: SSP grid needs >= 2 wavelengths");
  RUBIX_REQUIRE(n_wave_t >= 1 && n_wave_t <= kMaxWaveT, RUBIX_E_SHAPE,
                "rubix_cube_fwd: n_wave_t must be in [1, %d], got %d", kMaxWaveT, n_wave_t);
  RUBIX_REQUIRE(spaxel_stride >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_cube_fwd: spaxel_stride < n_wave_t");
  RUBIX_REQUIRE(vel_component >= 0 && vel_component < vel_stride, RUBIX_E_INVALID,
                "rubix_cube_fwd: vel_component outside the velocity row");
  if (n_segments == 0) return RUBIX_OK;
  RUBIX_REQUIRE(ssp_flux && ssp_metallicity && ssp_age && ssp_wave_z && wave_t && seg_offsets &&
                    cube,
                RUBIX_E_INVALID, "rubix_cube_fwd: null pointer");
  RUBIX_REQUIRE(n == 0 || (mass && metallicity && age && velocity && perm), RUBIX_E_INVALID,
                "rubix_cube_fwd: null particle pointer");
  const size_t need = rubix_cube_workspace_size(n, n_segments, n_wave_t, n_wave);
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= need, RUBIX_E_WORKSPACE,
                "rubix_cube_fwd: workspace of %zu bytes needed, %zu given", need,
                workspace_bytes);
  const int row_cap = n_wave + 2;
  const size_t smem = sizeof(int2) * kBuckets + sizeof(float4) * 2 * kPB * row_cap +
                      sizeof(float2) * 3 * kAccWarps * kPB + sizeof(float) * 4 * kPB +
                      sizeof(BatchMeta) * 2;
  RUBIX_REQUIRE(smem <= 227 * 1024, RUBIX_E_UNSUPPORTED,
                "rubix_cube_fwd: SSP grid of %d wavelengths needs %zu bytes of shared memory",
                n_wave, smem);

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CubeLayout L = carve_cube(workspace, n, n_segments, n_wave_t);
  cube_setup_kernel<<<1, 256, 0, st>>>(ssp_wave_z, n_wave, wave_t, n_wave_t, L.ctrl, L.At,
                                       L.bucket);
  RUBIX_LAUNCH_CHECK("cube_setup_kernel");
  if (n > 0) {
    int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
    cube_gather_kernel<<<g, 256, 0, st>>>(mass, metallicity, age, velocity, vel_stride,
                                          vel_component, perm, seg_offsets, n_segments, n,
                                          ssp_metallicity, n_met, ssp_age, n_age, ssp_wave_z,
                                          n_wave, wave_t, n_wave_t, L.ctrl, L.rec);
    RUBIX_LAUNCH_CHECK("cube_gather_kernel");
  }
  {
    int g = (int)std::min<long long>((n_segments + 255) / 256, (long long)sm_count() * 8);
    cube_count_kernel<<<g, 256, 0, st>>>(seg_offsets, n_segments, L.slot_cnt, L.single_cnt);
    RUBIX_LAUNCH_CHECK("cube_count_kernel");
    scan_exclusive_1block<<<1, 1024, 0, st>>>(L.slot_cnt, n_segments, 1);
    RUBIX_LAUNCH_CHECK("scan_exclusive_1block");
    scan_exclusive_1block<<<1, 1024, 0, st>>>(L.single_cnt, n_segments, 1);
    RUBIX_LAUNCH_CHECK("scan_exclusive_1block");
    cube_fill_items_kernel<<<g, 256, 0, st>>>(seg_offsets, n_segments, L.slot_cnt, L.single_cnt,
                                              L.items, L.ctrl);
    RUBIX_LAUNCH_CHECK("cube_fill_items_kernel");
    RUBIX_CUDA_TRY(cudaMemsetAsync(L.done, 0, sizeof(int) * (size_t)n_segments, st));
  }
  MainArgs args;
  args.flux = ssp_flux;
  args.wave_z = ssp_wave_z;
  args.nZ = n_met;
  args.nA = n_age;
  args.n_wave = n_wave;
  args.wave_t = wave_t;
  args.At = L.At;
  args.n_t = n_wave_t;
  args.rec = L.rec;
  args.seg_off = seg_offsets;
  args.slot_start = L.slot_cnt;
  args.items = L.items;
  args.done = L.done;
  args.partials = L.partials;
  args.cube = cube;
  args.spaxel_stride = spaxel_stride;
  args.ctrl = L.ctrl;
  args.bucket = L.bucket;
  args.row_cap = row_cap;
  const int R = (n_wave_t + kAccThreads - 1) / kAccThreads;
  if (R <= 1) return launch_main<1>(args, smem, st);
  if (R <= 2) return launch_main<2>(args, smem, st);
  if (R <= 4) return launch_main<4>(args, smem, st);
  if (R <= 8) return launch_main<8>(args, smem, st);
  return launch_main<16>(args, smem, st);
}
