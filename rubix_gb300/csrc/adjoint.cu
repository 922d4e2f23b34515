// Adjoint of kernel (b): gradients of L with respect to each particle's mass,
// metallicity, age and line-of-sight velocity, given A = dL/d(cube before PSF and LSF).
//
// A particle p in spaxel s adds c_t = beta * I_t to the cube, with I_t the
// interpolated mixed template on the telescope grid, beta = m * T / T'
// (rubix/spectra/ifu.py:224-266) and T' = sum_t I_t dlambda_t.  So
//   dL/dm     = (T / T') * gamma,                     gamma = sum_t A[s,t] I_t
//   dL/dtheta = beta * H_theta + gamma * (m / T') * (dT/dtheta - (T / T') * D_theta)
// for theta in {Z, age, v}, with H_theta = sum_t A[s,t] dI_t/dtheta and
// D_theta = sum_t dlambda_t dI_t/dtheta (= dT'/dtheta).  dI/dZ and dI/dage are the
// interpolants of the bilinear weights' derivatives applied to the four corner
// spectra; lambda'_k = lambda_z,k * exp(v/c) gives dI_t/dv = -lambda_t * slope_k / c,
// and dT/dv = T / c.  dT/dZ and dT/dage come from the prefix sums in the gather.
// These are the derivatives of the forward formulas with the float32 bracket choices
// and the in-range mask held fixed, as an automatic differentiation of them gives.
//
// Same decomposition as the forward kernel (persistent blocks pulling spaxel chunks,
// TMA-staged corner-table segments, per-particle rows built in shared memory, thread i
// owning R consecutive telescope wavelengths), one particle per step: each thread
// accumulates 8 partial sums over its wavelengths, the block reduces them in a fixed
// order, and warp 0 writes the particle's gradients.  No atomics, deterministic.
#include "cube_common.cuh"
#include "tma.cuh"

namespace rubix {
namespace {

constexpr int kAdjThreads = 384;  // 2 blocks of 12 warps per SM
constexpr int kAdjWarps = kAdjThreads / 32;
static_assert(kAdjWarps == 12, "the partial-sum finalize reads warps w, w + 4, w + 8");
constexpr int kAdjSums = 8;

struct AdjArgs {
  const float4* ct;
  const float* wave_z;
  int nZ, nA, n_wave;
  const float* zg;
  const float* ag;
  const float* wave_t;
  const float* At;
  int n_t;
  const ParticleRec* rec;
  const int* seg_off;
  const int* perm;
  const int2* items;
  const float* adj;
  long long adj_stride;
  float* g_mass;
  float* g_met;
  float* g_age;
  float* g_vlos;
  float* g_av;  // dust only: dL/dA_V per particle (optional)
  CubeCtrl* ctrl;
  const int2* bucket;
  int row_cap;
  int staged;  // corner segments and SSP wavelengths in shared memory (else via L1/L2)
  int chunk;
  const float* dust_e2;  // per telescope wavelength: -0.4 log2(10) A(lambda)/A(V)
};

struct AdjSmem {
  size_t wz, bucket, grid, stage, row_a, row_b, red, rec, perm, total;
};

__host__ __device__ inline AdjSmem adj_smem_layout(int n_wave, int n_grid, int row_cap,
                                                   bool staged) {
  AdjSmem L;
  size_t o = 0;
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  L.wz = o;     o = al(o + sizeof(float) * (staged ? n_wave : 0));
  L.bucket = o; o = al(o + sizeof(int2) * kBuckets);
  L.grid = o;   o = al(o + sizeof(float) * n_grid);
  L.stage = o;  o = al(o + sizeof(float4) * (staged ? (size_t)row_cap : 0));
  L.row_a = o;  o = al(o + sizeof(float4) * (size_t)row_cap);
  L.row_b = o;  o = al(o + sizeof(float4) * (size_t)row_cap);
  L.red = o;    o = al(o + sizeof(float) * 2 * kAdjWarps * kAdjSums);
  L.rec = o;    o = al(o + sizeof(ParticleRec) * kMaxChunk);
  L.perm = o;   o = al(o + sizeof(int) * kMaxChunk);
  L.total = o;
  return L;
}

// Thread 0: bulk copy of the particle's corner-table segment (its bracket range).
__device__ __forceinline__ void adj_issue(const AdjArgs& a, const ParticleRec& r, float4* stage,
                                          uint64_t* bar) {
  fence_proxy_async_smem();
  const int4 b = r.b;
  const int ks = b.y, ke = b.z & ~kGenericFlag;
  const int klo = max(ks, 0);
  const int nk = min(ke + 1, a.n_wave - 1) - klo + 1;
  const uint32_t bytes = b.x >= 0 ? 16u * (uint32_t)nk : 0u;
  mbar_arrive_expect_tx(bar, bytes);
  if (b.x >= 0) bulk_copy_g2s(stage, a.ct + (long long)b.x * a.n_wave + klo, bytes, bar);
}

// The particle's mixing weights: G = w00 F00 + w10 F10 + w01 F01 + w11 F11 and the
// derivative weights GZ = z0 (F10 - F00) + z1 (F11 - F01), GA = a0 (F01 - F00) +
// a1 (F11 - F10); zeros outside the grid.  One thread computes them per particle.
__device__ __forceinline__ void adj_weights(const AdjArgs& a, const ParticleRec& r,
                                            const float* __restrict__ s_grid, float4& w,
                                            float4& d) {
  w = make_float4(0.f, 0.f, 0.f, 0.f);
  d = w;
  const int cell = r.b.x;
  if (cell < 0) return;
  const float tz = r.a.w, ta = __int_as_float(r.b.w);
  const int iz = cell / (a.nA - 1), ia = cell - iz * (a.nA - 1);
  const float dz = s_grid[iz + 1] - s_grid[iz];
  const float da = s_grid[a.nZ + ia + 1] - s_grid[a.nZ + ia];
  const float izw = dz == 0.f ? 0.f : 1.f / dz, iaw = da == 0.f ? 0.f : 1.f / da;
  w = make_float4((1.f - tz) * (1.f - ta), tz * (1.f - ta), (1.f - tz) * ta, tz * ta);
  d = make_float4((1.f - ta) * izw, ta * izw, (1.f - tz) * iaw, tz * iaw);
}

// Row entry e (SSP index k = kstart + e): row_a = (lambda'_k, slope, G_k, lambda'_{k+1}),
// row_b = (GZ_k, slopeZ, GA_k, slopeA) with GZ = dG/dZ, GA = dG/dage; sentinels as in
// the forward rows (k = -1: lambda' = -FLT_MAX, value G_0, slope 0; k >= nW-1: slope 0).
__device__ __forceinline__ void adj_build(const AdjArgs& a, const ParticleRec& r,
                                          const float* __restrict__ s_wz, float4 wt, float4 dw,
                                          const float4* __restrict__ stage,
                                          float4* __restrict__ row_a, float4* __restrict__ row_b,
                                          int lane, int warp) {
  const int nW = a.n_wave;
  const float alpha = r.a.y;
  const int ks = r.b.y, ke = r.b.z & ~kGenericFlag;
  const int klo = max(ks, 0), khi = min(ke + 1, nW - 1);
  const int n_e = ke - ks + 1;
  const int cell = r.b.x;
  const bool has_cell = cell >= 0;
  const float w00 = wt.x, w10 = wt.y, w01 = wt.z, w11 = wt.w;
  const float z0 = dw.x, z1 = dw.y, a0 = dw.z, a1 = dw.w;
  // staged: the segment [klo, khi] in shared memory; else the cell's corner-table row
  const float4* st = a.staged ? stage - klo : a.ct + (long long)max(cell, 0) * nW;
  for (int base = warp * 31; base < n_e; base += kAdjWarps * 31) {
    const int e = base + lane;
    const int k = ks + e;
    const int kk = min(max(k, klo), khi);
    float G = 0.f, GZ = 0.f, GA = 0.f;
    if (has_cell) {
      const float4 c = st[kk];
      G = w00 * c.x;
      G = fmaf(w10, c.y, G);
      G = fmaf(w01, c.z, G);
      G = fmaf(w11, c.w, G);
      GZ = fmaf(z0, c.y - c.x, z1 * (c.w - c.z));
      GA = fmaf(a0, c.z - c.x, a1 * (c.w - c.y));
    }
    const float lp = (k < 0) ? -kFltMax : (k >= nW ? kFltMax : __fmul_rn(s_wz[k], alpha));
    const float lp_next = __shfl_down_sync(0xffffffffu, lp, 1);
    const float G_next = __shfl_down_sync(0xffffffffu, G, 1);
    const float GZ_next = __shfl_down_sync(0xffffffffu, GZ, 1);
    const float GA_next = __shfl_down_sync(0xffffffffu, GA, 1);
    if (lane < 31 && e < n_e) {
      float inv = 0.f;
      if (k >= 0 && k + 1 < nW) {
        const float dl = lp_next - lp;
        inv = dl > 0.f ? __fdividef(1.f, dl) : 0.f;
      }
      const float lpw = (k + 1 >= nW) ? kFltMax : lp_next;
      row_a[e] = make_float4(lp, (G_next - G) * inv, G, lpw);
      row_b[e] = make_float4(GZ, (GZ_next - GZ) * inv, GA, (GA_next - GA) * inv);
    }
  }
}

constexpr int kAdjBU = 3;
// Grouped build: thread g builds entries [g*kAdjBU, (g+1)*kAdjBU) of the particle's two
// rows from kAdjBU + 1 positions of its own (no shuffles), so an ~800-entry row takes one
// round of ~270 threads instead of two or three 31-entry warp steps per warp.  Staged rows
// touching neither grid end (kstart >= 0, kend + 1 <= nW - 1) need no clamps; the others
// take adj_build's per-entry arithmetic.  Same operations per entry as adj_build:
// identical rows.
__device__ __forceinline__ void adj_build_groups(const AdjArgs& a, const ParticleRec& r,
                                                 const float* __restrict__ s_wz, float4 wt,
                                                 float4 dw, const float4* __restrict__ stage,
                                                 float4* __restrict__ row_a,
                                                 float4* __restrict__ row_b, int tid) {
  const int nW = a.n_wave;
  const float alpha = r.a.y;
  const int ks = r.b.y, ke = r.b.z & ~kGenericFlag;
  const int klo = max(ks, 0), khi = min(ke + 1, nW - 1);
  const int n_e = ke - ks + 1;
  const int cell = r.b.x;
  const bool has_cell = cell >= 0;
  // staged only: the loads of a partial last group run up to 2 entries past the row,
  // which stays inside the staging buffer (n_wave + 2 entries) and shared memory
  const bool plain = a.staged && ks >= 0 && ke + 1 <= nW - 1;
  const float4* st = a.staged ? stage - klo : a.ct + (long long)max(cell, 0) * nW;
  for (int e0 = tid * kAdjBU; e0 < n_e; e0 += kAdjThreads * kAdjBU) {
    const int k0 = ks + e0;
    if (plain) {
      float G[kAdjBU + 1], GZ[kAdjBU + 1], GA[kAdjBU + 1], lp[kAdjBU + 1];
#pragma unroll
      for (int j = 0; j <= kAdjBU; ++j) {
        float g = 0.f, gz = 0.f, ga = 0.f;
        const float4 c = st[k0 + j];
        if (has_cell) {
          g = wt.x * c.x;
          g = fmaf(wt.y, c.y, g);
          g = fmaf(wt.z, c.z, g);
          g = fmaf(wt.w, c.w, g);
          gz = fmaf(dw.x, c.y - c.x, dw.y * (c.w - c.z));
          ga = fmaf(dw.z, c.z - c.x, dw.w * (c.w - c.y));
        }
        G[j] = g;
        GZ[j] = gz;
        GA[j] = ga;
        lp[j] = __fmul_rn(s_wz[k0 + j], alpha);
      }
#pragma unroll
      for (int j = 0; j < kAdjBU; ++j) {
        const float dl = lp[j + 1] - lp[j];
        const float inv = dl > 0.f ? __fdividef(1.f, dl) : 0.f;
        if (e0 + j < n_e) {
          row_a[e0 + j] = make_float4(lp[j], (G[j + 1] - G[j]) * inv, G[j], lp[j + 1]);
          row_b[e0 + j] = make_float4(GZ[j], (GZ[j + 1] - GZ[j]) * inv, GA[j],
                                      (GA[j + 1] - GA[j]) * inv);
        }
      }
    } else {
      for (int j = 0; j < kAdjBU; ++j) {
        const int e = e0 + j;
        if (e >= n_e) break;
        float G2[2], GZ2[2], GA2[2], lp2[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int k = ks + e + q;
          const int kk = min(max(k, klo), khi);
          float g = 0.f, gz = 0.f, ga = 0.f;
          if (has_cell) {
            const float4 c = st[kk];
            g = wt.x * c.x;
            g = fmaf(wt.y, c.y, g);
            g = fmaf(wt.z, c.z, g);
            g = fmaf(wt.w, c.w, g);
            gz = fmaf(dw.x, c.y - c.x, dw.y * (c.w - c.z));
            ga = fmaf(dw.z, c.z - c.x, dw.w * (c.w - c.y));
          }
          G2[q] = g;
          GZ2[q] = gz;
          GA2[q] = ga;
          lp2[q] = (k < 0) ? -kFltMax : (k >= nW ? kFltMax : __fmul_rn(s_wz[k], alpha));
        }
        const int k = ks + e;
        float inv = 0.f;
        if (k >= 0 && k + 1 < nW) {
          const float dl = lp2[1] - lp2[0];
          inv = dl > 0.f ? __fdividef(1.f, dl) : 0.f;
        }
        const float lpw = (k + 1 >= nW) ? kFltMax : lp2[1];
        row_a[e] = make_float4(lp2[0], (G2[1] - G2[0]) * inv, G2[0], lpw);
        row_b[e] = make_float4(GZ2[0], (GZ2[1] - GZ2[0]) * inv, GA2[0], (GA2[1] - GA2[0]) * inv);
      }
    }
  }
}

// One-step walk on the two row arrays, branch-free: if x >= e.w advance both entry
// addresses by one and load both next entries (predicated add and loads).
__device__ __forceinline__ void walk_step2(float x, unsigned& aa, unsigned& ab, float4& e,
                                           float4& f) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ge.f32 p, %10, %5;\n\t"
      "@p add.u32 %0, %0, 16;\n\t"
      "@p add.u32 %1, %1, 16;\n\t"
      "@p ld.shared.v4.f32 {%2, %3, %4, %5}, [%0];\n\t"
      "@p ld.shared.v4.f32 {%6, %7, %8, %9}, [%1];\n\t"
      "}"
      : "+r"(aa), "+r"(ab), "+f"(e.x), "+f"(e.y), "+f"(e.z), "+f"(e.w), "+f"(f.x), "+f"(f.y),
        "+f"(f.z), "+f"(f.w)
      : "f"(x)
      : "memory");
}

// The 8 partial sums of one particle over this thread's R wavelengths.  With kDust the
// cube adjoint h_t is seen through the particle's dust transmission 2^(e_t A_V): the
// particle adds beta g_t I_t to the cube, so every sum against h takes h_t g_t; `sav`
// then also takes sum_t h_t g_t e_t I_t, the A_V derivative of the particle's term up to
// beta ln 2 (d 2^(e A_V) / dA_V = ln 2 e 2^(e A_V)).
template <int R, bool kGeneric, bool kDust>
__device__ __forceinline__ void adj_eval(const float4* __restrict__ ra,
                                         const float4* __restrict__ rb, int ks, int ke, float B,
                                         float A0, const int2* __restrict__ s_bucket,
                                         const float (&lam)[R], const float (&dlam)[R],
                                         const float (&h)[R], float (&s)[kAdjSums],
                                         const float* __restrict__ e2, float av, int t0,
                                         int n_t, float& sav) {
  const float u = A0 - B;
  int b = __float_as_int(u + 12582912.0f) - 0x4B400000;
  b = min(max(b, 0), kBuckets - 1);
  const int2 te = s_bucket[b];
  int k = te.x + (u >= __int_as_float(te.y) ? 1 : 0);
  k = min(max(k, ks), ke);
  float4 e = ra[k];
  {
    const float x = lam[0];
    while (k > ks && x < e.x) { --k; e = ra[k]; }
    while (k < ke && x >= e.w) { ++k; e = ra[k]; }
  }
  float4 f = rb[k];
  unsigned aa = static_cast<unsigned>(__cvta_generic_to_shared(ra + k));
  unsigned ab = static_cast<unsigned>(__cvta_generic_to_shared(rb + k));
#pragma unroll
  for (int i = 0; i < kAdjSums; ++i) s[i] = 0.f;
  sav = 0.f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float x = lam[r];
    if (kGeneric) {
      bool moved = false;
      while (k < ke && x >= e.w) { ++k; e = ra[k]; moved = true; }
      if (moved) f = rb[k];
    } else if (r > 0) {
      walk_step2(x, aa, ab, e, f);
    }
    const float d = x - e.x;
    const float I = fmaf(d, e.y, e.z);
    const float IZ = fmaf(d, f.y, f.x);
    const float IA = fmaf(d, f.w, f.z);
    float hr = h[r];
    if constexpr (kDust) {
      const float er = __ldg(e2 + min(t0 + r, n_t - 1));
      hr = __fmul_rn(hr, dust_transmission(er, av));
      sav = fmaf(__fmul_rn(hr, er), I, sav);
    }
    s[0] = fmaf(hr, I, s[0]);
    s[1] = fmaf(dlam[r], I, s[1]);
    s[2] = fmaf(hr, IZ, s[2]);
    s[3] = fmaf(dlam[r], IZ, s[3]);
    s[4] = fmaf(hr, IA, s[4]);
    s[5] = fmaf(dlam[r], IA, s[5]);
    const float xs = x * e.y;  // lambda_t * slope
    s[6] = fmaf(hr, xs, s[6]);
    s[7] = fmaf(dlam[r], xs, s[7]);
  }
}

// Sums 8 values over the warp with 9 shuffles (transposed butterfly).  Afterwards lane
// l with (l & 3) == 0 holds the total of value ((l >> 4) & 1) * 4 + ((l >> 3) & 1) * 2 +
// ((l >> 2) & 1).
__device__ __forceinline__ float warp_reduce8(const float (&v)[8], int lane) {
  float a[4];
  const bool b4 = lane & 16;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float mine = b4 ? v[4 + i] : v[i];
    const float other = b4 ? v[i] : v[4 + i];
    a[i] = mine + __shfl_xor_sync(0xffffffffu, other, 16);
  }
  float c[2];
  const bool b3 = lane & 8;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float mine = b3 ? a[2 + i] : a[i];
    const float other = b3 ? a[i] : a[2 + i];
    c[i] = mine + __shfl_xor_sync(0xffffffffu, other, 8);
  }
  const bool b2 = lane & 4;
  float d = (b2 ? c[1] : c[0]) + __shfl_xor_sync(0xffffffffu, b2 ? c[0] : c[1], 4);
  d += __shfl_xor_sync(0xffffffffu, d, 2);
  d += __shfl_xor_sync(0xffffffffu, d, 1);
  return d;
}

template <int R, bool kDust>
__global__ void __launch_bounds__(kAdjThreads, 2) cube_adjoint_kernel(AdjArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const AdjSmem SL = adj_smem_layout(a.n_wave, a.nZ + a.nA, a.row_cap, a.staged != 0);
  float* s_wz = reinterpret_cast<float*>(smem + SL.wz);
  int2* s_bucket = reinterpret_cast<int2*>(smem + SL.bucket);
  float* s_grid = reinterpret_cast<float*>(smem + SL.grid);
  float4* s_stage = reinterpret_cast<float4*>(smem + SL.stage);
  float4* s_ra = reinterpret_cast<float4*>(smem + SL.row_a);
  float4* s_rb = reinterpret_cast<float4*>(smem + SL.row_b);
  float* s_red = reinterpret_cast<float*>(smem + SL.red);  // [2][warps][8]
  ParticleRec* s_rec = reinterpret_cast<ParticleRec*>(smem + SL.rec);
  int* s_perm = reinterpret_cast<int*>(smem + SL.perm);  // particle index of each record
  __shared__ uint64_t s_bar;
  __shared__ int s_item, s_fail;
  __shared__ float4 s_wt[2][2];  // mixing / derivative weights of the current, next particle
  __shared__ float s_red_av[2][kAdjWarps];  // dust: the A_V sum of each warp

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (a.staged)
    for (int i = tid; i < a.n_wave; i += kAdjThreads) s_wz[i] = a.wave_z[i];
  const float* wzp = a.staged ? s_wz : a.wave_z;  // SSP wavelengths: shared or L1
  const bool staged = a.staged != 0;
  for (int b = tid; b < kBuckets; b += kAdjThreads) s_bucket[b] = a.bucket[b];
  for (int i = tid; i < a.nZ; i += kAdjThreads) s_grid[i] = a.zg[i];
  for (int i = tid; i < a.nA; i += kAdjThreads) s_grid[a.nZ + i] = a.ag[i];
  if (tid == 0) {
    mbar_init(&s_bar, 1);
    fence_mbar_init();
    s_fail = 0;
  }
  const int n_t = a.n_t;
  const int t0 = tid * R;
  float lam[R], dlam[R], h[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t = t0 + r;
    const int tc = t < n_t ? t : n_t - 1;
    lam[r] = a.wave_t[tc];
    dlam[r] = (t < n_t && t > 0) ? (a.wave_t[t] - a.wave_t[t - 1]) : 0.f;
  }
  const float A0 = a.At[t0 < n_t ? t0 : n_t - 1];
  const int n_items = a.ctrl->n_items;
  uint32_t phase = 0;
  int step = 0;
  __syncthreads();

  for (;;) {
    if (tid == 0) s_item = atomicAdd(&a.ctrl->next_item, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= n_items) break;
    const int2 it = a.items[item];
    const int s = it.x, chunk = it.y;
    const int seg_b = a.seg_off[s], seg_e = a.seg_off[s + 1];
    const long long jb = (long long)seg_b + (long long)chunk * a.chunk;
    const long long je = min((long long)seg_e, jb + a.chunk);
    const int np = (int)(je - jb);
    const float* adj = a.adj + (long long)s * a.adj_stride;
#pragma unroll
    for (int r = 0; r < R; ++r) h[r] = (t0 + r < n_t) ? adj[t0 + r] : 0.f;
    for (int i = tid; i < np; i += kAdjThreads) {
      s_rec[i] = a.rec[jb + i];
      s_perm[i] = a.perm[jb + i];
    }
    __syncthreads();
    if (np > 0 && tid == 0) {
      if (staged) adj_issue(a, s_rec[0], s_stage, &s_bar);
      adj_weights(a, s_rec[0], s_grid, s_wt[step & 1][0], s_wt[step & 1][1]);
    }
    __syncthreads();  // weights of the item's first particle visible

    for (int p = 0; p < np; ++p, ++step) {
      const int buf = step & 1;
      const ParticleRec& rec = s_rec[p];
      if (staged) {
        if (!mbar_wait_bounded(&s_bar, phase)) s_fail = 1;
        phase ^= 1u;
      }
      // the dust kernels and R = 11 keep the warp-step build, which does not spill there
      if constexpr (!kDust && R <= 10)
        adj_build_groups(a, rec, wzp, s_wt[buf][0], s_wt[buf][1], s_stage, s_ra, s_rb, tid);
      else
        adj_build(a, rec, wzp, s_wt[buf][0], s_wt[buf][1], s_stage, s_ra, s_rb, lane, warp);
      __syncthreads();  // rows ready; staging consumed
      if (s_fail) {
        if (tid == 0) {
          atomicExch(&a.ctrl->error, 1);
          mbar_wait_bounded(&s_bar, phase ^ 1u);
        }
        return;
      }
      if (p + 1 < np && tid == 0) {
        // the next particle: its corner segment by TMA and its weights, read after the
        // reduction barrier below
        if (staged) adj_issue(a, s_rec[p + 1], s_stage, &s_bar);
        adj_weights(a, s_rec[p + 1], s_grid, s_wt[buf ^ 1][0], s_wt[buf ^ 1][1]);
      }
      const int4 rb = rec.b;
      const int ks = rb.y, ke = rb.z & ~kGenericFlag;
      float sums[kAdjSums];
      float sav = 0.f;
      const float av = kDust ? rec.c.w : 0.f;
      if (rb.z & kGenericFlag)
        adj_eval<R, true, kDust>(s_ra - ks, s_rb - ks, ks, ke, rec.a.z, A0, s_bucket, lam, dlam,
                                 h, sums, a.dust_e2, av, t0, n_t, sav);
      else
        adj_eval<R, false, kDust>(s_ra - ks, s_rb - ks, ks, ke, rec.a.z, A0, s_bucket, lam,
                                  dlam, h, sums, a.dust_e2, av, t0, n_t, sav);
      const float wv = warp_reduce8(sums, lane);
      if ((lane & 3) == 0) {
        const int v = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
        s_red[(buf * kAdjWarps + warp) * kAdjSums + v] = wv;
      }
      if constexpr (kDust) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sav += __shfl_xor_sync(0xffffffffu, sav, o);
        if (lane == 0) s_red_av[buf][warp] = sav;
      }
      __syncthreads();  // partial sums visible; rows free for the next particle
      // the last warp finalises: its share of the next row build is the smallest (groups
      // fill the warps in order; warp steps give the extra steps to the first warps),
      // and thread 0 issues the next particle's copy
      if (warp == kAdjWarps - 1) {
        // lane l: value l & 7 over warps (l >> 3), (l >> 3) + 4, (l >> 3) + 8 (independent
        // loads), then over the four lane groups; fixed order, so deterministic
        const float* red = s_red + buf * kAdjWarps * kAdjSums;
        const int vi = lane & 7, wg = lane >> 3;
        float tot = red[wg * kAdjSums + vi] + red[(wg + 4) * kAdjSums + vi];
        tot += red[(wg + 8) * kAdjSums + vi];
        tot += __shfl_xor_sync(0xffffffffu, tot, 8);
        tot += __shfl_xor_sync(0xffffffffu, tot, 16);
        const float gamma = __shfl_sync(0xffffffffu, tot, 0);
        const float Tp = __shfl_sync(0xffffffffu, tot, 1);
        const float HZ = __shfl_sync(0xffffffffu, tot, 2);
        const float DZ = __shfl_sync(0xffffffffu, tot, 3);
        const float HA = __shfl_sync(0xffffffffu, tot, 4);
        const float DA = __shfl_sync(0xffffffffu, tot, 5);
        const float HV = __shfl_sync(0xffffffffu, tot, 6);
        const float DV = __shfl_sync(0xffffffffu, tot, 7);
        if (lane == 0) {
          const float m = rec.a.x, T = rec.c.x, TZ = rec.c.y, TA = rec.c.z;
          const float sc = T / Tp;
          float gm = 0.f, gz = 0.f, ga = 0.f, gv = 0.f, gav = 0.f;
          if (Tp != 0.f && isfinite(sc)) {
            const float beta = m * sc;
            if constexpr (kDust) {
              if (a.g_av) {
                float t = 0.f;  // the warps' A_V sums in warp order
                for (int w = 0; w < kAdjWarps; ++w) t += s_red_av[buf][w];
                gav = beta * 0.69314718055994531f * t;
              }
            }
            const float k = m / Tp;
            const float inv_c = (float)(1.0 / kSpeedOfLight);
            gm = sc * gamma;
            gz = fmaf(beta, HZ, gamma * k * (TZ - sc * DZ));
            ga = fmaf(beta, HA, gamma * k * (TA - sc * DA));
            // dI/dv = -lambda * slope / c, dT/dv = T / c
            gv = fmaf(-beta * inv_c, HV, gamma * k * inv_c * (T + sc * DV));
          }
          // the index comes from shared memory: a global load here would hold warp 0,
          // and with it the next particle's barrier, for a memory round trip
          const long long i = s_perm[p];
          if (a.g_mass) a.g_mass[i] = gm;
          if (a.g_met) a.g_met[i] = gz;
          if (a.g_age) a.g_age[i] = ga;
          if (a.g_vlos) a.g_vlos[i] = gv;
          if (kDust && a.g_av) a.g_av[i] = gav;
        }
      }
    }
  }
}

template <int R, bool kDust>
int launch_adjoint_t(const AdjArgs& args, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(cube_adjoint_kernel<R, kDust>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess)
    return set_error(RUBIX_E_CUDA, "cudaFuncSetAttribute(cube_adjoint_kernel): %s",
                     cudaGetErrorString(e));
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cube_adjoint_kernel<R, kDust>,
                                                    kAdjThreads, smem);
  if (e != cudaSuccess || per_sm < 1)
    return set_error(RUBIX_E_UNSUPPORTED,
                     "cube_adjoint_kernel does not fit on an SM with %zu bytes of shared memory",
                     smem);
  cube_adjoint_kernel<R, kDust><<<sm_count() * per_sm, kAdjThreads, smem, st>>>(args);
  RUBIX_LAUNCH_CHECK("cube_adjoint_kernel");
  return RUBIX_OK;
}

template <int R>
int launch_adjoint(const AdjArgs& args, size_t smem, cudaStream_t st) {
  return args.dust_e2 ? launch_adjoint_t<R, true>(args, smem, st)
                      : launch_adjoint_t<R, false>(args, smem, st);
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" size_t rubix_cube_bwd_workspace_size(int64_t n, int32_t n_segments, int32_t n_wave_t,
                                                int32_t n_met, int32_t n_age, int32_t n_wave) {
  if (n < 0 || n_segments < 0 || n_wave_t < 0 || n_met < 0 || n_age < 0 || n_wave < 0) return 0;
  return carve_cube(nullptr, n, n_segments, n_wave_t, n_met, n_age, n_wave,
                    cube_tuning_current().chunk)
      .bytes;
}

namespace rubix {
namespace {

int cube_bwd_impl(const char* who, const float* ssp_flux, const float* ssp_metallicity,
                  const float* ssp_age, const float* ssp_wave_z, int32_t n_met, int32_t n_age,
                  int32_t n_wave, const float* wave_t, int32_t n_wave_t, const float* mass,
                  const float* metallicity, const float* age, const float* velocity,
                  int64_t vel_stride, int32_t vel_component, const float* av,
                  const float* dust_e2, const int32_t* perm, const int32_t* seg_offsets,
                  int32_t n_segments, int64_t n, const float* adj, int64_t adj_stride,
                  float* grad_mass, float* grad_metallicity, float* grad_age, float* grad_vlos,
                  float* grad_av, void* workspace, size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n >= 0 && n < (1LL << 31), RUBIX_E_SHAPE, "%s: bad n", who);
  RUBIX_REQUIRE(n_segments >= 0, RUBIX_E_SHAPE, "%s: n_segments < 0", who);
  RUBIX_REQUIRE(n_met >= 2 && n_age >= 2, RUBIX_E_SHAPE,
                "%s: SSP grid needs >= 2 metallicities and >= 2 ages", who);
  RUBIX_REQUIRE(n_wave >= 2, RUBIX_E_SHAPE, "%s: SSP grid needs >= 2 wavelengths", who);
  RUBIX_REQUIRE(n_wave_t >= 1 && n_wave_t <= kMaxWaveT, RUBIX_E_SHAPE,
                "%s: n_wave_t must be in [1, %d], got %d", who, kMaxWaveT, n_wave_t);
  RUBIX_REQUIRE(adj_stride >= n_wave_t, RUBIX_E_SHAPE, "%s: adj_stride < n_wave_t", who);
  RUBIX_REQUIRE(vel_component >= 0 && vel_component < vel_stride, RUBIX_E_INVALID,
                "%s: vel_component outside the velocity row", who);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // every gradient entry is written: zeros for particles outside the sorted set
  float* grads[5] = {grad_mass, grad_metallicity, grad_age, grad_vlos, grad_av};
  for (float* g : grads)
    if (g && n > 0) RUBIX_CUDA_TRY(cudaMemsetAsync(g, 0, sizeof(float) * (size_t)n, st));
  if (n_segments == 0 || n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(ssp_flux && ssp_metallicity && ssp_age && ssp_wave_z && wave_t && seg_offsets &&
                    adj && mass && metallicity && age && velocity && perm,
                RUBIX_E_INVALID, "%s: null pointer", who);
  const size_t need = rubix_cube_bwd_workspace_size(n, n_segments, n_wave_t, n_met, n_age, n_wave);
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= need, RUBIX_E_WORKSPACE,
                "%s: workspace of %zu bytes needed, %zu given", who, need, workspace_bytes);
  RUBIX_REQUIRE((reinterpret_cast<uintptr_t>(workspace) & 255) == 0, RUBIX_E_INVALID,
                "%s: workspace must be 256-byte aligned", who);
  // Grids too large for the staged layout (about 4000 SSP wavelengths) read the corners
  // and the SSP wavelengths through L1/L2 (to about 6500 wavelengths).
  const int row_cap = n_wave + 2;
  const bool staged = adj_smem_layout(n_wave, n_met + n_age, row_cap, true).total <= 227 * 1024;
  const AdjSmem SL = adj_smem_layout(n_wave, n_met + n_age, row_cap, staged);
  RUBIX_REQUIRE(SL.total <= 227 * 1024, RUBIX_E_UNSUPPORTED,
                "%s: SSP grid of %d wavelengths needs %zu bytes of shared memory "
                "(limit 232448)",
                who, n_wave, SL.total);

  const CubeTuning tune = cube_tuning_current();
  const CubeLayout L =
      carve_cube(workspace, n, n_segments, n_wave_t, n_met, n_age, n_wave, tune.chunk);
  const CubeInputs in{ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, n_met, n_age, n_wave,
                      wave_t, n_wave_t, mass, metallicity, age, velocity, vel_stride,
                      vel_component, perm, seg_offsets, n_segments, n, av};
  {
    const int rc = cube_prepare(in, L, tune, /*with_grad=*/true, st);
    if (rc != RUBIX_OK) return rc;
  }
  AdjArgs args;
  args.ct = L.ct;
  args.wave_z = ssp_wave_z;
  args.nZ = n_met;
  args.nA = n_age;
  args.n_wave = n_wave;
  args.zg = ssp_metallicity;
  args.ag = ssp_age;
  args.wave_t = wave_t;
  args.At = L.At;
  args.n_t = n_wave_t;
  args.rec = L.rec;
  args.seg_off = seg_offsets;
  args.perm = perm;
  args.items = L.items;
  args.adj = adj;
  args.adj_stride = adj_stride;
  args.g_mass = grad_mass;
  args.g_met = grad_metallicity;
  args.g_age = grad_age;
  args.g_vlos = grad_vlos;
  args.g_av = grad_av;
  args.ctrl = L.ctrl;
  args.bucket = L.bucket;
  args.row_cap = row_cap;
  args.staged = staged ? 1 : 0;
  args.chunk = tune.chunk;
  args.dust_e2 = dust_e2;
  const int need_r = (n_wave_t + kAdjThreads - 1) / kAdjThreads;
  const size_t smem = SL.total;
  if (need_r <= 1) return launch_adjoint<1>(args, smem, st);
  if (need_r <= 2) return launch_adjoint<2>(args, smem, st);
  if (need_r <= 4) return launch_adjoint<4>(args, smem, st);
  if (need_r <= 6) return launch_adjoint<6>(args, smem, st);
  if (need_r <= 8) return launch_adjoint<8>(args, smem, st);
  if (need_r <= 10) return launch_adjoint<10>(args, smem, st);
  return launch_adjoint<11>(args, smem, st);  // kAdjThreads * 11 >= kMaxWaveT
}

}  // namespace
}  // namespace rubix

extern "C" int rubix_cube_bwd(const float* ssp_flux, const float* ssp_metallicity,
                              const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                              int32_t n_age, int32_t n_wave, const float* wave_t,
                              int32_t n_wave_t, const float* mass, const float* metallicity,
                              const float* age, const float* velocity, int64_t vel_stride,
                              int32_t vel_component, const int32_t* perm,
                              const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                              const float* adj, int64_t adj_stride, float* grad_mass,
                              float* grad_metallicity, float* grad_age, float* grad_vlos,
                              void* workspace, size_t workspace_bytes, void* stream) {
  return cube_bwd_impl("rubix_cube_bwd", ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, n_met,
                       n_age, n_wave, wave_t, n_wave_t, mass, metallicity, age, velocity,
                       vel_stride, vel_component, nullptr, nullptr, perm, seg_offsets,
                       n_segments, n, adj, adj_stride, grad_mass, grad_metallicity, grad_age,
                       grad_vlos, nullptr, workspace, workspace_bytes, stream);
}

extern "C" int rubix_cube_bwd_dust(const float* ssp_flux, const float* ssp_metallicity,
                                   const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                                   int32_t n_age, int32_t n_wave, const float* wave_t,
                                   int32_t n_wave_t, const float* mass, const float* metallicity,
                                   const float* age, const float* velocity, int64_t vel_stride,
                                   int32_t vel_component, const float* av,
                                   const float* ext_exponent, const int32_t* perm,
                                   const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                   const float* adj, int64_t adj_stride, float* grad_mass,
                                   float* grad_metallicity, float* grad_age, float* grad_vlos,
                                   void* workspace, size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(ext_exponent != nullptr && (n == 0 || av != nullptr), RUBIX_E_INVALID,
                "rubix_cube_bwd_dust: null A_V or extinction exponent");
  return cube_bwd_impl("rubix_cube_bwd_dust", ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z,
                       n_met, n_age, n_wave, wave_t, n_wave_t, mass, metallicity, age, velocity,
                       vel_stride, vel_component, av, ext_exponent, perm, seg_offsets,
                       n_segments, n, adj, adj_stride, grad_mass, grad_metallicity, grad_age,
                       grad_vlos, nullptr, workspace, workspace_bytes, stream);
}

extern "C" int rubix_cube_bwd_dust_av(const float* ssp_flux, const float* ssp_metallicity,
                                      const float* ssp_age, const float* ssp_wave_z,
                                      int32_t n_met, int32_t n_age, int32_t n_wave,
                                      const float* wave_t, int32_t n_wave_t, const float* mass,
                                      const float* metallicity, const float* age,
                                      const float* velocity, int64_t vel_stride,
                                      int32_t vel_component, const float* av,
                                      const float* ext_exponent, const int32_t* perm,
                                      const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                      const float* adj, int64_t adj_stride, float* grad_mass,
                                      float* grad_metallicity, float* grad_age,
                                      float* grad_vlos, float* grad_av, void* workspace,
                                      size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(ext_exponent != nullptr && (n == 0 || av != nullptr), RUBIX_E_INVALID,
                "rubix_cube_bwd_dust_av: null A_V or extinction exponent");
  return cube_bwd_impl("rubix_cube_bwd_dust_av", ssp_flux, ssp_metallicity, ssp_age,
                       ssp_wave_z, n_met, n_age, n_wave, wave_t, n_wave_t, mass, metallicity,
                       age, velocity, vel_stride, vel_component, av, ext_exponent, perm,
                       seg_offsets, n_segments, n, adj, adj_stride, grad_mass, grad_metallicity,
                       grad_age, grad_vlos, grad_av, workspace, workspace_bytes, stream);
}
