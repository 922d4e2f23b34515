// Kernel (b): fused SSP lookup (bilinear in metallicity and age), mass scaling,
// Doppler shift, flux-conserving resampling onto the telescope grid and the
// per-spaxel accumulation of the datacube.
//
// Work decomposition
//   * Setup passes (a few microseconds): a bucket table over log wavelength, the
//     "corner table" holding, for every (metallicity, age) cell of the SSP grid and
//     every SSP wavelength, the four corner fluxes of the cell as one float4, and a
//     gather of the spaxel-sorted particles into 32-byte records (mass, Doppler factor
//     alpha = fl32(exp(v/c)), cell and bilinear weights, and the SSP brackets
//     kstart/kend of both ends of the telescope range on the particle's float32 grid
//     lambda'_k = fl32(lambda_z,k * alpha)).
//   * Work items are (spaxel, chunk of <= `chunk` particles), largest first, pulled by a
//     persistent kernel from an atomic counter.  A block of 384 threads owns the
//     telescope grid of its spaxel: thread i holds R consecutive wavelengths
//     t = i*R + r in registers (wavelength, bin width, accumulator).
//   * A batch is 1-3 particles packed by their bracket lengths into staging and row
//     pools of kPB * (nW + 2) entries.  One thread issues a 1-D TMA bulk copy of each
//     particle's corner-table segment (its bracket range only) into the staging pool; it
//     completes on an mbarrier while the block evaluates the previous batch.  The
//     threads, one group of 7 consecutive entries each, then build per particle the row
//     of entries (lambda'_k, slope_k, G_k, lambda'_{k+1}) of the mixed template
//     G = sum_c w_c F_c; the in-range flux sum T
//     (rubix/spectra/ifu.py:241-245) comes from the gather (prefix sums).
//   * Evaluation: each thread finds the exact bracket of its first wavelength (bucket
//     table + exact comparisons on lambda') and walks forward over its R wavelengths;
//     when every SSP interval is wider than every telescope bin the walk advances at
//     most once per wavelength (one predicated load); the particles of a batch are
//     evaluated interleaved for instruction-level parallelism.  Interpolated values stay in
//     registers while T' = sum_t I_t dlambda_t is reduced over the block; then
//     s = nan_to_num(T/T') and the accumulators take mass * s * I.
//   * Spaxels with more than `chunk` particles are split; each chunk writes a partial
//     spectrum to the workspace and the last chunk to finish sums the partials in chunk
//     order (Kahan).  No float atomics: results are bit-reproducible.
//   * Optional epilogue: the LSF convolution along wavelength of the finished spectrum
//     (rubix/telescope/lsf/lsf.py:29-105), which commutes with the PSF.
#include "cube_common.cuh"
#include "tma.cuh"

namespace rubix {
namespace {

struct MainArgs {
  const float4* ct;  // corner table [(nZ-1)*(nA-1)][nW]
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
  int staged;           // corner segments staged in shared memory by TMA (else read from L2)
  int pool;             // entries of the row pool (and of the staging pool when staged)
  int chunk;            // particles per work item
  int lsf_k, lsf_crop;  // lsf_k = 0: no LSF epilogue
  float lsf[kMaxLsfTaps + 1];
  const float* dust_e2;  // per telescope wavelength: -0.4 log2(10) A(lambda)/A(V)
};

// Shared-memory carve-up of the main kernel (byte offsets, 16-byte aligned): the TMA
// staging pool (`stage` entries; none when corners are read from L2) and the row pool
// (`pool` entries), shared by the up to kPBMax particles of a batch.
struct SmemLayout {
  size_t wz, bucket, stage, rows, red, rec, total;
};

__host__ __device__ inline SmemLayout smem_layout(int n_wave, int stage, int pool) {
  SmemLayout L;
  size_t o = 0;
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  L.wz = o;     o = al(o + sizeof(float) * n_wave);
  L.bucket = o; o = al(o + sizeof(int2) * kBuckets);
  L.stage = o;  o = al(o + sizeof(float4) * (size_t)stage);
  L.rows = o;   // also holds the zero-padded spectrum of the LSF epilogue
  o = al(o + std::max(sizeof(float4) * (size_t)pool,
                      sizeof(float) * (size_t)(kMaxWaveT + 2 * kMaxLsfTaps + 8)));
  L.red = o;    o = al(o + sizeof(float) * 2 * kAccWarps * 4);
  L.rec = o;    o = al(o + sizeof(ParticleRec) * kMaxChunk);
  L.total = o;
  return L;
}

// Batches of up to kPBMax particles packed into the staging and row pools of P entries
// each: particle j of a batch takes n_e + 2 entries (its row, and its staged corner
// segment of at most n_e + 1 entries) at the same offset in both pools.  Every thread
// derives the same plan from the records.
constexpr int kPBMax = 3;

struct BatchPlan {
  int cnt;
  int off[kPBMax];
};

__device__ __forceinline__ int rec_ne(const ParticleRec& r) {
  return (r.b.z & ~kGenericFlag) - r.b.y + 1;
}

__device__ __forceinline__ BatchPlan plan_batch(const ParticleRec* recs, int left, int P) {
  BatchPlan b;
  b.cnt = left > 0 ? 1 : 0;
  b.off[0] = 0;
  b.off[1] = b.off[2] = 0;
  if (left <= 0) return b;
  int used = rec_ne(recs[0]) + 2;
#pragma unroll
  for (int j = 1; j < kPBMax; ++j) {
    if (j >= left) break;
    const int need = rec_ne(recs[j]) + 2;
    if (used + need > P) break;
    b.off[j] = used;
    used += need;
    b.cnt = j + 1;
  }
  return b;
}

// Thread 0: arm the barrier and issue one bulk copy per particle of a planned batch: the
// corner-table entries k in [max(kstart,0), min(kend+1, nW-1)] of its cell.
__device__ __forceinline__ void issue_plan(const MainArgs& a, const ParticleRec* recs,
                                           const BatchPlan& bp, float4* stage, uint64_t* bar) {
  fence_proxy_async_smem();
  uint32_t bytes = 0;
#pragma unroll
  for (int p = 0; p < kPBMax; ++p) {
    if (p < bp.cnt && recs[p].b.x >= 0) {
      const int ks = recs[p].b.y, ke = recs[p].b.z & ~kGenericFlag;
      const int klo = max(ks, 0);
      bytes += 16u * (uint32_t)(min(ke + 1, a.n_wave - 1) - klo + 1);
    }
  }
  mbar_arrive_expect_tx(bar, bytes);
#pragma unroll
  for (int p = 0; p < kPBMax; ++p) {
    if (p < bp.cnt && recs[p].b.x >= 0) {
      const int ks = recs[p].b.y, ke = recs[p].b.z & ~kGenericFlag;
      const int klo = max(ks, 0);
      const int nk = min(ke + 1, a.n_wave - 1) - klo + 1;
      bulk_copy_g2s(stage + bp.off[p], a.ct + (long long)recs[p].b.x * a.n_wave + klo,
                    16u * nk, bar);
    }
  }
}

struct RowParams {
  float alpha, w00, w10, w01, w11;
  int ks, klo, khi, n_e;
  bool has_cell;
  const float4* st;  // st[k] = staged corners of SSP wavelength k
  float4* row;
};

template <bool kStaged>
__device__ __forceinline__ RowParams row_params(const ParticleRec& r, const MainArgs& a,
                                                const float4* stage, float4* row) {
  RowParams q;
  const float tz = r.a.w, ta = __int_as_float(r.b.w);
  const int ke = r.b.z & ~kGenericFlag;
  q.alpha = r.a.y;
  q.w00 = (1.f - tz) * (1.f - ta);
  q.w10 = tz * (1.f - ta);
  q.w01 = (1.f - tz) * ta;
  q.w11 = tz * ta;
  q.ks = r.b.y;
  q.klo = max(q.ks, 0);
  q.khi = min(ke + 1, a.n_wave - 1);
  q.n_e = ke - q.ks + 1;
  q.has_cell = r.b.x >= 0;
  // staged: the segment [klo, khi] in shared memory; else the cell's corner-table row
  // (row 0 stands in for particles outside the grid, whose G is forced to 0)
  if constexpr (kStaged)
    q.st = stage - q.klo;
  else
    q.st = a.ct + (long long)max(r.b.x, 0) * a.n_wave;
  q.row = row;
  return q;
}

// One warp step of a row build: entries base .. base+30 (lane 31 supplies the right
// neighbour).  Entry e (SSP index k = kstart + e) = (lambda'_k, slope_k, G_k,
// lambda'_{k+1}), with sentinels (-FLT_MAX, 0, G_0, lambda'_0) for k = -1 and
// slope 0 / FLT_MAX beyond the grid.  The corners come from the staged segment.
__device__ __forceinline__ void build_step(const RowParams& q, int base, int nW,
                                           const float* __restrict__ s_wz, int lane) {
  const int e = base + lane;
  const int k = q.ks + e;
  if (q.ks + base >= 0 && q.ks + base + 31 <= q.khi) {
    // interior step: every lane, neighbour included, is an SSP wavelength of the range
    float G = 0.f;
    if (q.has_cell) {
      const float4 c = q.st[k];
      G = q.w00 * c.x;
      G = fmaf(q.w10, c.y, G);
      G = fmaf(q.w01, c.z, G);
      G = fmaf(q.w11, c.w, G);
    }
    const float lp = __fmul_rn(s_wz[k], q.alpha);
    const float lp_next = __shfl_down_sync(0xffffffffu, lp, 1);
    const float G_next = __shfl_down_sync(0xffffffffu, G, 1);
    if (lane < 31) {
      const float dl = lp_next - lp;
      const float slope = dl > 0.f ? __fdividef(G_next - G, dl) : 0.f;
      q.row[e] = make_float4(lp, slope, G, lp_next);
    }
  } else {
    const int kk = min(max(k, q.klo), q.khi);
    float G = 0.f;
    if (q.has_cell) {
      const float4 c = q.st[kk];
      G = q.w00 * c.x;
      G = fmaf(q.w10, c.y, G);
      G = fmaf(q.w01, c.z, G);
      G = fmaf(q.w11, c.w, G);
    }
    const float lp = (k < 0) ? -kFltMax : (k >= nW ? kFltMax : __fmul_rn(s_wz[k], q.alpha));
    const float lp_next = __shfl_down_sync(0xffffffffu, lp, 1);
    const float G_next = __shfl_down_sync(0xffffffffu, G, 1);
    if (lane < 31 && e < q.n_e) {
      float slope = 0.f;
      if (k >= 0 && k + 1 < nW) {
        const float dl = lp_next - lp;
        slope = dl > 0.f ? __fdividef(G_next - G, dl) : 0.f;
      }
      const float lpw = (k + 1 >= nW) ? kFltMax : lp_next;
      q.row[e] = make_float4(lp, slope, G, lpw);
    }
  }
}

// A build step is interior when every lane, neighbour included, is an SSP wavelength of
// the particle's staged range.
__device__ __forceinline__ bool interior(const RowParams& q, int base) {
  return q.ks + base >= 0 && q.ks + base + 31 <= q.khi;
}

// Two interior steps of one particle at two bases, interleaved.
__device__ __forceinline__ void build_step_pair2(const RowParams& q, int b0, int b1,
                                                 const float* __restrict__ s_wz, int lane) {
  const int e0 = b0 + lane, e1 = b1 + lane;
  const int k0 = q.ks + e0, k1 = q.ks + e1;
  const float4 c0 = q.st[k0];
  const float4 c1 = q.st[k1];
  const float z0 = s_wz[k0], z1 = s_wz[k1];
  float G0 = q.w00 * c0.x, G1 = q.w00 * c1.x;
  G0 = fmaf(q.w10, c0.y, G0);
  G1 = fmaf(q.w10, c1.y, G1);
  G0 = fmaf(q.w01, c0.z, G0);
  G1 = fmaf(q.w01, c1.z, G1);
  G0 = fmaf(q.w11, c0.w, G0);
  G1 = fmaf(q.w11, c1.w, G1);
  if (!q.has_cell) {
    G0 = 0.f;
    G1 = 0.f;
  }
  const float lp0 = __fmul_rn(z0, q.alpha), lp1 = __fmul_rn(z1, q.alpha);
  const float lpn0 = __shfl_down_sync(0xffffffffu, lp0, 1);
  const float lpn1 = __shfl_down_sync(0xffffffffu, lp1, 1);
  const float Gn0 = __shfl_down_sync(0xffffffffu, G0, 1);
  const float Gn1 = __shfl_down_sync(0xffffffffu, G1, 1);
  if (lane < 31) {
    const float dl0 = lpn0 - lp0, dl1 = lpn1 - lp1;
    const float sl0 = dl0 > 0.f ? __fdividef(Gn0 - G0, dl0) : 0.f;
    const float sl1 = dl1 > 0.f ? __fdividef(Gn1 - G1, dl1) : 0.f;
    q.row[e0] = make_float4(lp0, sl0, G0, lpn0);
    q.row[e1] = make_float4(lp1, sl1, G1, lpn1);
  }
}

// Builds the rows of a planned batch (1..3 particles) from the staged corners.  The
// 12 warps are split evenly over the batch's particles (12, 6 or 4 warps each), so each
// warp derives one particle's row parameters; a warp interleaves two 31-entry steps of
// its particle for instruction-level parallelism.
template <bool kStaged>
__device__ __forceinline__ void build_plan(const MainArgs& a, const ParticleRec* recs,
                                           const BatchPlan& bp, const float* __restrict__ s_wz,
                                           const float4* __restrict__ stage,
                                           float4* __restrict__ rows, int lane, int warp) {
  const int cnt = bp.cnt;
  const int wpp = kAccWarps / cnt;  // kAccWarps is divisible by 1, 2 and 3
  const int p = warp / wpp;
  const int wl = warp - p * wpp;
  const int off = p == 0 ? 0 : (p == 1 ? bp.off[1] : bp.off[2]);
  const RowParams q = row_params<kStaged>(recs[p], a, stage + off, rows + off);
  const int stride = wpp * 31;
  for (int base = wl * 31; base < q.n_e; base += 2 * stride) {
    const int b2 = base + stride;
    if (b2 < q.n_e && interior(q, base) && interior(q, b2)) {
      build_step_pair2(q, base, b2, s_wz, lane);
    } else {
      build_step(q, base, a.n_wave, s_wz, lane);
      if (b2 < q.n_e) build_step(q, b2, a.n_wave, s_wz, lane);
    }
  }
}

// Row builds from staged corners by groups: the entries of a batch's rows are cut into
// groups of kBU consecutive entries of one particle, one group per thread.  A thread
// mixes the template and shifts the wavelength of its kBU entries and of the right
// neighbour itself (no shuffles, no per-warp row parameters), so an interior entry costs
// two shared loads, the four-corner mix, one multiply, the slope and one store.
// Consecutive threads are kBU entries apart; with kBU = 7 (112 bytes) the 16-byte loads
// and stores of a quarter-warp fall in distinct banks.  Every entry is computed with the
// arithmetic of build_step, so the rows equal build_plan's bit for bit.  Odd kBU keeps a
// quarter-warp's entries in distinct banks; R = 6 and R = 11 take 5-entry groups, which
// keep those kernels free of spills.
template <int R>
constexpr int build_group_len() {
  return (R > 10 || R < 8) ? 5 : 7;
}

// One particle of a planned batch, prepared once in shared memory as three 16-byte
// vectors (three vector loads per group instead of a dozen scalar ones).
struct __align__(16) BuildPart {
  float4 w;  // bilinear weights w00, w10, w01, w11
  int4 a;    // first group g0, kstart, staging offset - klo, row offset
  int4 b;    // n_e, flags (kPartCell | kPartPlain), khi, alpha (bits)
};
constexpr int kPartCell = 1;   // inside the SSP grid (else G = 0)
constexpr int kPartPlain = 2;  // kstart >= 0 and kend + 1 <= nW - 1: no grid end in the row

// One thread: the build parameters of a planned batch and its total group count.
// kstart >= -1 and kend >= kstart give khi >= klo, so the clamped corner index of every
// entry lies in the particle's staged segment [klo, khi].
template <int kBU>
__device__ __forceinline__ void prep_parts(const ParticleRec* recs, const BatchPlan& bp, int nW,
                                           BuildPart* out, int* gtot) {
  int g = 0;
  for (int p = 0; p < bp.cnt; ++p) {
    const ParticleRec r = recs[p];
    BuildPart q;
    const float tz = r.a.w, ta = __int_as_float(r.b.w);
    const int ke = r.b.z & ~kGenericFlag;
    const int ks = r.b.y;
    const int klo = max(ks, 0);
    const int n_e = ke - ks + 1;
    const int off = p == 0 ? 0 : (p == 1 ? bp.off[1] : bp.off[2]);
    q.w = make_float4((1.f - tz) * (1.f - ta), tz * (1.f - ta), (1.f - tz) * ta, tz * ta);
    q.a = make_int4(g, ks, off - klo, off);
    q.b = make_int4(n_e,
                    (r.b.x >= 0 ? kPartCell : 0) | ((ks >= 0 && ke + 1 <= nW - 1) ? kPartPlain : 0),
                    min(ke + 1, nW - 1), __float_as_int(r.a.y));
    g += (n_e + kBU - 1) / kBU;
    out[p] = q;
  }
  *gtot = g;
}

// G = sum_c w_c F_c of one staged entry (0 for particles outside the SSP grid: their
// staging slot holds no copy, and the select discards whatever it holds).
__device__ __forceinline__ float mix_corners(const float4 w, bool has_cell, const float4 c) {
  float G = w.x * c.x;
  G = fmaf(w.y, c.y, G);
  G = fmaf(w.z, c.z, G);
  G = fmaf(w.w, c.w, G);
  return has_cell ? G : 0.f;
}

template <int kBU>
__device__ __forceinline__ void build_groups(const MainArgs& a,
                                             const BuildPart* __restrict__ parts, int cnt,
                                             int gtot, const float* __restrict__ s_wz,
                                             const float4* __restrict__ stage,
                                             float4* __restrict__ rows, int tid) {
  const int nW = a.n_wave;
  for (int g = tid; g < gtot; g += kAccThreads) {
    const int p = (cnt > 2 && g >= parts[2].a.x) ? 2 : ((cnt > 1 && g >= parts[1].a.x) ? 1 : 0);
    const int4 qa = parts[p].a;
    const int4 qb = parts[p].b;
    const float4 w = parts[p].w;
    const bool has_cell = (qb.y & kPartCell) != 0;
    const float alpha = __int_as_float(qb.w);
    const int ks = qa.y, n_e = qb.x, khi = qb.z;
    const int e0 = (g - qa.x) * kBU;
    const int k0 = ks + e0;
    const float4* st = stage + qa.z;  // st[k]: staged corners, k in [klo, khi]
    float4* row = rows + qa.w;
    if ((qb.y & kPartPlain) || (k0 >= 0 && k0 + kBU <= khi && e0 + kBU <= n_e)) {
      // A row that touches neither grid end: every stored entry k <= kend and its
      // neighbour k + 1 <= kend + 1 = khi are in the staged segment.  The entries of a
      // last, partial group past the row's end are computed and not stored; their loads
      // stay in shared memory (at most kBU - 2 float4 past the staging pool, which the
      // row pool follows, and kBU - 1 floats past the SSP wavelengths, which the bucket
      // table follows).  Otherwise an interior group: every entry and its neighbour are
      // SSP wavelengths of the staged range, and every entry is stored.
      float Gv[kBU + 1], Lv[kBU + 1];
#pragma unroll
      for (int j = 0; j <= kBU; ++j) {
        Gv[j] = mix_corners(w, has_cell, st[k0 + j]);
        Lv[j] = __fmul_rn(s_wz[k0 + j], alpha);
      }
#pragma unroll
      for (int j = 0; j < kBU; ++j) {
        const float dl = Lv[j + 1] - Lv[j];
        const float slope = dl > 0.f ? __fdividef(Gv[j + 1] - Gv[j], dl) : 0.f;
        if (e0 + j < n_e) row[e0 + j] = make_float4(Lv[j], slope, Gv[j], Lv[j + 1]);
      }
    } else {
      // ends of the row: clamped corners and the sentinels of build_step
      const int klo = max(ks, 0);
      for (int j = 0; j < kBU; ++j) {
        const int e = e0 + j;
        if (e >= n_e) break;
        const int k = ks + e;
        const float G = mix_corners(w, has_cell, st[min(max(k, klo), khi)]);
        const float Gn = mix_corners(w, has_cell, st[min(max(k + 1, klo), khi)]);
        const float lp = (k < 0) ? -kFltMax : (k >= nW ? kFltMax : __fmul_rn(s_wz[k], alpha));
        const int k1 = k + 1;
        const float lpn =
            (k1 < 0) ? -kFltMax : (k1 >= nW ? kFltMax : __fmul_rn(s_wz[k1], alpha));
        float slope = 0.f;
        if (k >= 0 && k + 1 < nW) {
          const float dl = lpn - lp;
          slope = dl > 0.f ? __fdividef(Gn - G, dl) : 0.f;
        }
        const float lpw = (k + 1 >= nW) ? kFltMax : lpn;
        row[e] = make_float4(lp, slope, G, lpw);
      }
    }
  }
}

// Sums 4 values over the 32 lanes with 6 shuffles; lane 0 ends with the total of v0,
// lane 8 with v1, lane 16 with v2, lane 24 with v3.
__device__ __forceinline__ float warp_reduce4(float v0, float v1, float v2, float v3, int lane) {
  const bool b4 = lane & 16;
  const float a0 = (b4 ? v2 : v0) + __shfl_xor_sync(0xffffffffu, b4 ? v0 : v2, 16);
  const float a1 = (b4 ? v3 : v1) + __shfl_xor_sync(0xffffffffu, b4 ? v1 : v3, 16);
  const bool b3 = lane & 8;
  float c = (b3 ? a1 : a0) + __shfl_xor_sync(0xffffffffu, b3 ? a0 : a1, 8);
  c += __shfl_xor_sync(0xffffffffu, c, 4);
  c += __shfl_xor_sync(0xffffffffu, c, 2);
  c += __shfl_xor_sync(0xffffffffu, c, 1);
  return c;
}

// Bracket of this thread's first wavelength on a particle's row: bucket table in log
// wavelength, then exact comparisons on lambda'.
__device__ __forceinline__ int first_bracket(const float4* __restrict__ rowp, int ks, int ke,
                                             float B, float A0, const int2* __restrict__ s_bucket,
                                             float x0, float4& e) {
  const float u = A0 - B;
  int b = __float_as_int(u + 12582912.0f) - 0x4B400000;
  b = min(max(b, 0), kBuckets - 1);
  const int2 te = s_bucket[b];
  int k = te.x + (u >= __int_as_float(te.y) ? 1 : 0);
  k = min(max(k, ks), ke);
  e = rowp[k];
  while (k > ks && x0 < e.x) { --k; e = rowp[k]; }
  while (k < ke && x0 >= e.w) { ++k; e = rowp[k]; }
  return k;
}

// One-step walk on a row in shared memory, branch-free: if x >= e.w (the right end of
// the current interval) advance the entry address by one and load the next entry.  The
// predicate covers the add and the load, so lanes that stay issue no divergent branch.
__device__ __forceinline__ void walk_step(float x, unsigned& addr, float4& e) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ge.f32 p, %5, %4;\n\t"
      "@p add.u32 %0, %0, 16;\n\t"
      "@p ld.shared.v4.f32 {%1, %2, %3, %4}, [%0];\n\t"
      "}"
      : "+r"(addr), "+f"(e.x), "+f"(e.y), "+f"(e.z), "+f"(e.w)
      : "f"(x)
      : "memory");
}

// Interpolated values of one particle at this thread's R wavelengths; returns the
// partial sum of I_t * dlambda_t.
template <int R, bool kGeneric>
__device__ __forceinline__ float eval_particle(const float4* __restrict__ rowp, int ks, int ke,
                                               float B, float A0,
                                               const int2* __restrict__ s_bucket,
                                               const float (&lam)[R], float lam_prev,
                                               float (&I)[R]) {
  float4 e;
  int k = first_bracket(rowp, ks, ke, B, A0, s_bucket, lam[0], e);
  unsigned addr = static_cast<unsigned>(__cvta_generic_to_shared(rowp + k));
  float tp = 0.f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float x = lam[r];
    if (kGeneric) {
      while (k < ke && x >= e.w) { ++k; e = rowp[k]; }
    } else if (r > 0) {
      walk_step(x, addr, e);
    }
    const float v = fmaf(x - e.x, e.y, e.z);
    I[r] = v;
    tp = fmaf(v, x - (r > 0 ? lam[r - 1] : lam_prev), tp);
  }
  return tp;
}

// Both particles of a batch on the one-step walk, interleaved for instruction-level
// parallelism (their shared-memory loads and FMA chains overlap).
template <int R>
__device__ __forceinline__ void eval_pair(const float4* __restrict__ row0, int ks0, int ke0,
                                          float B0, const float4* __restrict__ row1, int ks1,
                                          int ke1, float B1, float A0,
                                          const int2* __restrict__ s_bucket,
                                          const float (&lam)[R], float lam_prev,
                                          float (&I0)[R], float (&I1)[R], float& tp0,
                                          float& tp1) {
  float4 e0, e1;
  const int k0 = first_bracket(row0, ks0, ke0, B0, A0, s_bucket, lam[0], e0);
  const int k1 = first_bracket(row1, ks1, ke1, B1, A0, s_bucket, lam[0], e1);
  unsigned a0 = static_cast<unsigned>(__cvta_generic_to_shared(row0 + k0));
  unsigned a1 = static_cast<unsigned>(__cvta_generic_to_shared(row1 + k1));
  tp0 = 0.f;
  tp1 = 0.f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float x = lam[r];
    if (r > 0) {
      walk_step(x, a0, e0);
      walk_step(x, a1, e1);
    }
    const float v0 = fmaf(x - e0.x, e0.y, e0.z);
    const float v1 = fmaf(x - e1.x, e1.y, e1.z);
    const float d = x - (r > 0 ? lam[r - 1] : lam_prev);
    I0[r] = v0;
    I1[r] = v1;
    tp0 = fmaf(v0, d, tp0);
    tp1 = fmaf(v1, d, tp1);
  }
}

// Three particles on the one-step walk, interleaved; dlambda_t recomputed from the
// wavelengths (lam_prev = the wavelength before this thread's first one).
template <int R>
__device__ __forceinline__ void eval_triple(const float4* __restrict__ row0, int ks0, int ke0,
                                            float B0, const float4* __restrict__ row1, int ks1,
                                            int ke1, float B1, const float4* __restrict__ row2,
                                            int ks2, int ke2, float B2, float A0,
                                            const int2* __restrict__ s_bucket,
                                            const float (&lam)[R], float lam_prev,
                                            float (&I0)[R], float (&I1)[R], float (&I2)[R],
                                            float& tp0, float& tp1, float& tp2) {
  float4 e0, e1, e2;
  const int k0 = first_bracket(row0, ks0, ke0, B0, A0, s_bucket, lam[0], e0);
  const int k1 = first_bracket(row1, ks1, ke1, B1, A0, s_bucket, lam[0], e1);
  const int k2 = first_bracket(row2, ks2, ke2, B2, A0, s_bucket, lam[0], e2);
  unsigned a0 = static_cast<unsigned>(__cvta_generic_to_shared(row0 + k0));
  unsigned a1 = static_cast<unsigned>(__cvta_generic_to_shared(row1 + k1));
  unsigned a2 = static_cast<unsigned>(__cvta_generic_to_shared(row2 + k2));
  tp0 = tp1 = tp2 = 0.f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float x = lam[r];
    const float d = x - (r > 0 ? lam[r - 1] : lam_prev);
    if (r > 0) {
      walk_step(x, a0, e0);
      walk_step(x, a1, e1);
      walk_step(x, a2, e2);
    }
    const float v0 = fmaf(x - e0.x, e0.y, e0.z);
    const float v1 = fmaf(x - e1.x, e1.y, e1.z);
    const float v2 = fmaf(x - e2.x, e2.y, e2.z);
    I0[r] = v0;
    I1[r] = v1;
    I2[r] = v2;
    tp0 = fmaf(v0, d, tp0);
    tp1 = fmaf(v1, d, tp1);
    tp2 = fmaf(v2, d, tp2);
  }
}

// LSF along wavelength of one spectrum: s_pad holds the spectrum at offset
// lead = K-1-crop with zeros around it, so out[t] = sum_j taps[j] * s_pad[t + K-1 - j].
template <int R>
__device__ __forceinline__ void lsf_epilogue(const MainArgs& a, const float* __restrict__ s_pad,
                                             int t0, float (&out)[R]) {
#pragma unroll
  for (int r = 0; r < R; ++r) out[r] = 0.f;
  const int K = a.lsf_k;
  const float* base = s_pad + t0 + K - 1;
  for (int j = 0; j < K; ++j) {
    const float w = a.lsf[j];
#pragma unroll
    for (int r = 0; r < R; ++r) out[r] = fmaf(w, base[r - j], out[r]);
  }
}

// The same with K taps known at compile time: the R + K - 1 window in registers.
template <int R, int K>
__device__ __forceinline__ void lsf_epilogue_k(const MainArgs& a,
                                               const float* __restrict__ s_pad, int t0,
                                               float (&out)[R]) {
  float win[R + K - 1];
#pragma unroll
  for (int i = 0; i < R + K - 1; ++i) win[i] = s_pad[t0 + i];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    float o = 0.f;
#pragma unroll
    for (int j = 0; j < K; ++j) o = fmaf(a.lsf[j], win[r + K - 1 - j], o);
    out[r] = o;
  }
}

template <int R, bool kDust, bool kStaged>
__global__ void __launch_bounds__(kAccThreads, 2) cube_main_kernel(MainArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SmemLayout SL = smem_layout(kStaged ? a.n_wave : 0, kStaged ? a.pool : 0, a.pool);
  float* s_wz = reinterpret_cast<float*>(smem + SL.wz);
  int2* s_bucket = reinterpret_cast<int2*>(smem + SL.bucket);
  float4* s_stage = reinterpret_cast<float4*>(smem + SL.stage);      // pool of P entries
  float4* s_rows = reinterpret_cast<float4*>(smem + SL.rows);        // pool of P entries
  float* s_red = reinterpret_cast<float*>(smem + SL.red);            // [2][warps][4]
  ParticleRec* s_rec = reinterpret_cast<ParticleRec*>(smem + SL.rec);  // records of the item
  float* s_spec = reinterpret_cast<float*>(s_rows);  // LSF epilogue reuses the rows
  __shared__ uint64_t s_bar;
  __shared__ int s_item, s_last, s_fail;
  __shared__ BuildPart s_bp[2][kPBMax];  // staged path: build parameters per batch buffer
  __shared__ int s_gtot[2];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if constexpr (kStaged)
    for (int i = tid; i < a.n_wave; i += kAccThreads) s_wz[i] = a.wave_z[i];
  for (int b = tid; b < kBuckets; b += kAccThreads) s_bucket[b] = a.bucket[b];
  const float* wzp = kStaged ? s_wz : a.wave_z;  // SSP wavelengths: shared or L1
  if (tid == 0) {
    mbar_init(&s_bar, 1);
    fence_mbar_init();
    s_fail = 0;
  }

  const int n_t = a.n_t;
  const int t0 = tid * R;
  const int P = a.pool;
  constexpr bool staged = kStaged;
  constexpr int kBU = build_group_len<R>();
  // rows built by groups of kBU entries (the dust kernel at R = 11 keeps build_plan: the
  // group build spills 72 bytes there)
  constexpr bool kGroups = kStaged && (!kDust || R <= 10);
  float lam[R], acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int t = t0 + r;
    lam[r] = a.wave_t[t < n_t ? t : n_t - 1];
  }
  // wavelength before the first one (dlambda_0 = 0: rubix's prepend-diff)
  const float lam_prev = a.wave_t[t0 == 0 ? 0 : min(t0 - 1, n_t - 1)];
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
    const int cnt_s = seg_e - seg_b;
    const long long jb = (long long)seg_b + (long long)chunk * a.chunk;
    const long long je = min((long long)seg_e, jb + a.chunk);
    const int np = (int)(je - jb);

#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = 0.f;
    // records of this item into shared memory (one 48-byte record per thread)
    for (int i = tid; i < np; i += kAccThreads) s_rec[i] = a.rec[jb + i];
    __syncthreads();
    BatchPlan bp = plan_batch(s_rec, np, P);
    if (staged && np > 0 && tid == 0) issue_plan(a, s_rec, bp, s_stage, &s_bar);
    if constexpr (kGroups) {
      // warp 1 prepares the build parameters while warp 0 issues the copies
      if (tid == 32) prep_parts<kBU>(s_rec, bp, a.n_wave, s_bp[step & 1], &s_gtot[step & 1]);
      __syncthreads();
    }

    // Batch at p0: wait for its staged corners, build its rows, stage the next batch,
    // evaluate, reduce T'.
    for (int p0 = 0; p0 < np; ++step) {
      const int buf = step & 1;
      const int cnt = bp.cnt;
      const ParticleRec* recs = s_rec + p0;
      if (staged) {
        if (!mbar_wait_bounded(&s_bar, phase)) s_fail = 1;
        phase ^= 1u;
      }
      if constexpr (kGroups)
        build_groups<kBU>(a, s_bp[buf], cnt, s_gtot[buf], wzp, s_stage, s_rows, tid);
      else
        build_plan<kStaged>(a, recs, bp, wzp, s_stage, s_rows, lane, warp);
      __syncthreads();  // rows ready; staging consumed
      if (s_fail) {
        if (tid == 0) {
          atomicExch(&a.ctrl->error, 1);
          mbar_wait_bounded(&s_bar, phase ^ 1u);  // give copies in flight a last chance
        }
        return;
      }
      const int p1 = p0 + cnt;
      const BatchPlan bn = plan_batch(s_rec + p1, np - p1, P);
      if (staged && p1 < np && tid == 0) issue_plan(a, s_rec + p1, bn, s_stage, &s_bar);
      // the other buffer: last read by the previous batch's build, before the barrier
      // above; read by the next build after the T' reduction barrier below
      if constexpr (kGroups)
        if (tid == 32)
          prep_parts<kBU>(s_rec + p1, bn, a.n_wave, s_bp[buf ^ 1], &s_gtot[buf ^ 1]);

      float I[kPBMax][R];
      float tp[kPBMax];
      const int4 rb0 = recs[0].b;
      const int4 rb1 = cnt > 1 ? recs[1].b : rb0;
      const int4 rb2 = cnt > 2 ? recs[2].b : rb0;
      const bool generic = ((rb0.z | rb1.z | rb2.z) & kGenericFlag) != 0;
      const float4* row0 = s_rows - rb0.y;
      const float4* row1 = s_rows + bp.off[1] - rb1.y;
      const float4* row2 = s_rows + bp.off[2] - rb2.y;
      if (cnt == 3 && !generic) {
        eval_triple<R>(row0, rb0.y, rb0.z, recs[0].a.z, row1, rb1.y, rb1.z, recs[1].a.z, row2,
                       rb2.y, rb2.z, recs[2].a.z, A0, s_bucket, lam, lam_prev, I[0], I[1], I[2],
                       tp[0], tp[1], tp[2]);
      } else if (cnt == 2 && !generic) {
        eval_pair<R>(row0, rb0.y, rb0.z, recs[0].a.z, row1, rb1.y, rb1.z, recs[1].a.z, A0,
                     s_bucket, lam, lam_prev, I[0], I[1], tp[0], tp[1]);
        tp[2] = 0.f;
#pragma unroll
        for (int r = 0; r < R; ++r) I[2][r] = 0.f;
      } else {
#pragma unroll
        for (int p = 0; p < kPBMax; ++p) {
          tp[p] = 0.f;
#pragma unroll
          for (int r = 0; r < R; ++r) I[p][r] = 0.f;
          if (p < cnt) {
            const int4 rb = recs[p].b;
            const int ke = rb.z & ~kGenericFlag;
            const float4* rowp = s_rows + bp.off[p] - rb.y;
            tp[p] = (rb.z & kGenericFlag)
                        ? eval_particle<R, true>(rowp, rb.y, ke, recs[p].a.z, A0, s_bucket, lam,
                                                 lam_prev, I[p])
                        : eval_particle<R, false>(rowp, rb.y, ke, recs[p].a.z, A0, s_bucket,
                                                  lam, lam_prev, I[p]);
          }
        }
      }
      // T'0..T'2 over the warp, then over the block (fixed order: deterministic).
      const float wsum = warp_reduce4(tp[0], tp[1], tp[2], 0.f, lane);
      if ((lane & 7) == 0) s_red[(buf * kAccWarps + warp) * 4 + (lane >> 3)] = wsum;
      __syncthreads();
      // lane l: value p = l >> 3 of warps (l & 7) and (l & 7) + 8
      const int pv = lane >> 3, w0 = lane & 7;
      float v = s_red[(buf * kAccWarps + w0) * 4 + pv];
      if (w0 + 8 < kAccWarps) v += s_red[(buf * kAccWarps + w0 + 8) * 4 + pv];
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 2);
      v += __shfl_xor_sync(0xffffffffu, v, 1);
      // lanes 0, 8, 16: T'0, T'1, T'2
      float beta_l = 0.f;
      if ((lane & 7) == 0 && pv < cnt) {
        const float4 ra = recs[pv].a, rc = recs[pv].c;  // lane-dependent index: shared memory
        float sc = rc.x / v;
        if (sc != sc) sc = 0.f;
        if (isinf(sc)) sc = copysignf(kFltMax, sc);
        beta_l = ra.x != 0.f ? ra.x * sc : 0.f;
      }
      const float beta0 = __shfl_sync(0xffffffffu, beta_l, 0);
      const float beta1 = __shfl_sync(0xffffffffu, beta_l, 8);
      const float beta2 = __shfl_sync(0xffffffffu, beta_l, 16);
      if constexpr (kDust) {
        // transmission 10^(-0.4 A(lambda)/A(V) A_V) of each particle's dust column
        // (spectra/dust/dust_baseclasses.py:163-164) applied to its resampled spectrum
        // (one 2^x per particle of the batch: cnt is the same for the whole block)
        const float av0 = recs[0].c.w;
        const float av1 = cnt > 1 ? recs[1].c.w : 0.f;
        const float av2 = cnt > 2 ? recs[2].c.w : 0.f;
        if (cnt == 3) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float e2 = __ldg(a.dust_e2 + min(t0 + r, n_t - 1));
            const float g0 = __fmul_rn(beta0, dust_transmission(e2, av0));
            const float g1 = __fmul_rn(beta1, dust_transmission(e2, av1));
            const float g2 = __fmul_rn(beta2, dust_transmission(e2, av2));
            acc[r] = fmaf(g2, I[2][r], fmaf(g1, I[1][r], fmaf(g0, I[0][r], acc[r])));
          }
        } else if (cnt == 2) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float e2 = __ldg(a.dust_e2 + min(t0 + r, n_t - 1));
            const float g0 = __fmul_rn(beta0, dust_transmission(e2, av0));
            const float g1 = __fmul_rn(beta1, dust_transmission(e2, av1));
            acc[r] = fmaf(g1, I[1][r], fmaf(g0, I[0][r], acc[r]));
          }
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const float e2 = __ldg(a.dust_e2 + min(t0 + r, n_t - 1));
            acc[r] = fmaf(__fmul_rn(beta0, dust_transmission(e2, av0)), I[0][r], acc[r]);
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r)
          acc[r] = fmaf(beta2, I[2][r], fmaf(beta1, I[1][r], fmaf(beta0, I[0][r], acc[r])));
      }
      p0 = p1;
      bp = bn;
    }

    const int nch = cnt_s <= a.chunk ? 1 : (cnt_s + a.chunk - 1) / a.chunk;
    bool have_final = true;
    if (nch > 1) {
      float* part = a.partials + (long long)item * n_t;
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (t0 + r < n_t) part[t0 + r] = acc[r];
      __threadfence();
      __syncthreads();
      if (tid == 0) s_last = (atomicAdd(&a.done[s], 1) == nch - 1) ? 1 : 0;
      __syncthreads();
      have_final = s_last != 0;
      if (have_final) {
        __threadfence();
        const long long slot0 = a.slot_start[s];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int t = t0 + r;
          float sum = 0.f, comp = 0.f;
          if (t < n_t) {
            for (int c = 0; c < nch; ++c) {
              const float y = __ldcg(a.partials + (slot0 + c) * n_t + t) - comp;
              const float tt = sum + y;
              comp = (tt - sum) - y;
              sum = tt;
            }
          }
          acc[r] = sum;
        }
      }
    }
    if (have_final) {
      float* out = a.cube + (long long)s * a.spaxel_stride;
      if (a.lsf_k > 0) {
        __syncthreads();  // rows free (last batch evaluated) before reuse as spectrum
        const int lead = a.lsf_k - 1 - a.lsf_crop;
        // zero padding: [0, lead) and [lead + n_t, lead + R*384 + K)
        for (int i = tid; i < lead; i += kAccThreads) s_spec[i] = 0.f;
        for (int i = lead + n_t + tid; i < lead + kAccThreads * R + a.lsf_k; i += kAccThreads)
          s_spec[i] = 0.f;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (t0 + r < n_t) s_spec[lead + t0 + r] = acc[r];
        __syncthreads();
        if (a.lsf_k == 25)  // rubix's LSF: 2 * 12 + 1 taps (telescope/lsf/lsf.py:12-26)
          lsf_epilogue_k<R, 25>(a, s_spec, t0, acc);
        else
          lsf_epilogue<R>(a, s_spec, t0, acc);
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (t0 + r < n_t) out[t0 + r] = acc[r];
    }
    __syncthreads();
  }
}

template <int R, bool kDust, bool kStaged>
int launch_main_t(const MainArgs& args, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(cube_main_kernel<R, kDust, kStaged>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess)
    return set_error(RUBIX_E_CUDA, "cudaFuncSetAttribute(cube_main_kernel): %s",
                     cudaGetErrorString(e));
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cube_main_kernel<R, kDust, kStaged>,
                                                    kAccThreads,
                                                    smem);
  if (e != cudaSuccess || per_sm < 1)
    return set_error(RUBIX_E_UNSUPPORTED,
                     "cube_main_kernel does not fit on an SM with %zu bytes of shared memory",
                     smem);
  const int grid = sm_count() * per_sm;
  cube_main_kernel<R, kDust, kStaged><<<grid, kAccThreads, smem, st>>>(args);
  RUBIX_LAUNCH_CHECK("cube_main_kernel");
  return RUBIX_OK;
}

template <int R>
int launch_main(const MainArgs& args, size_t smem, cudaStream_t st) {
  if (args.staged)
    return args.dust_e2 ? launch_main_t<R, true, true>(args, smem, st)
                        : launch_main_t<R, false, true>(args, smem, st);
  return args.dust_e2 ? launch_main_t<R, true, false>(args, smem, st)
                      : launch_main_t<R, false, false>(args, smem, st);
}

int cube_fwd_impl(const char* who, const float* ssp_flux, const float* ssp_metallicity,
                  const float* ssp_age, const float* ssp_wave_z, int32_t n_met, int32_t n_age,
                  int32_t n_wave, const float* wave_t, int32_t n_wave_t, const float* mass,
                  const float* metallicity, const float* age, const float* velocity,
                  int64_t vel_stride, int32_t vel_component, const int32_t* perm,
                  const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                  const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop, const float* av,
                  const float* dust_e2, float* cube, int64_t spaxel_stride, void* workspace,
                  size_t workspace_bytes, void* stream);

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" size_t rubix_cube_workspace_size(int64_t n, int32_t n_segments, int32_t n_wave_t,
                                            int32_t n_met, int32_t n_age, int32_t n_wave) {
  if (n < 0 || n_segments < 0 || n_wave_t < 0 || n_met < 0 || n_age < 0 || n_wave < 0) return 0;
  return carve_cube(nullptr, n, n_segments, n_wave_t, n_met, n_age, n_wave,
                    cube_tuning_current().chunk)
      .bytes;
}

namespace rubix {

// The argument checks of rubix_cube_fwd that come before its workspace check, shared
// with rubix_cube_fwd_noalloc so that both entry points return the same code for the
// same arguments.  *nothing_to_do is set when there is no spaxel to write.
int cube_fwd_check_args(const char* who, const float* ssp_flux, const float* ssp_metallicity,
                        const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                        int32_t n_age, int32_t n_wave, const float* wave_t, int32_t n_wave_t,
                        const float* mass, const float* metallicity, const float* age,
                        const float* velocity, int64_t vel_stride, int32_t vel_component,
                        const int32_t* perm, const int32_t* seg_offsets, int32_t n_segments,
                        int64_t n, const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop,
                        const float* cube, int64_t spaxel_stride, bool* nothing_to_do) {
  *nothing_to_do = false;
  RUBIX_REQUIRE(n >= 0 && n < (1LL << 31), RUBIX_E_SHAPE, "%s: bad n", who);
  RUBIX_REQUIRE(n_segments >= 0, RUBIX_E_SHAPE, "%s: n_segments < 0", who);
  RUBIX_REQUIRE(n_met >= 2 && n_age >= 2, RUBIX_E_SHAPE,
                "%s: SSP grid needs >= 2 metallicities and >= 2 ages", who);
  RUBIX_REQUIRE(n_wave >= 2, RUBIX_E_SHAPE, "%s: SSP grid needs >= 2 wavelengths", who);
  RUBIX_REQUIRE(n_wave_t >= 1 && n_wave_t <= kMaxWaveT, RUBIX_E_SHAPE,
                "%s: n_wave_t must be in [1, %d], got %d", who, kMaxWaveT, n_wave_t);
  RUBIX_REQUIRE(spaxel_stride >= n_wave_t, RUBIX_E_SHAPE,
                "%s: spaxel_stride < n_wave_t", who);
  RUBIX_REQUIRE(vel_component >= 0 && vel_component < vel_stride, RUBIX_E_INVALID,
                "%s: vel_component outside the velocity row", who);
  RUBIX_REQUIRE(n_lsf_taps >= 0 && n_lsf_taps <= kMaxLsfTaps, RUBIX_E_SHAPE,
                "%s: at most %d LSF taps", who, kMaxLsfTaps);
  RUBIX_REQUIRE(n_lsf_taps == 0 || (lsf_taps && lsf_crop >= 0 && lsf_crop < n_lsf_taps),
                RUBIX_E_INVALID, "%s: bad LSF taps/crop", who);
  if (n_segments == 0) {
    *nothing_to_do = true;
    return RUBIX_OK;
  }
  RUBIX_REQUIRE(ssp_flux && ssp_metallicity && ssp_age && ssp_wave_z && wave_t && seg_offsets &&
                    cube,
                RUBIX_E_INVALID, "%s: null pointer", who);
  RUBIX_REQUIRE(n == 0 || (mass && metallicity && age && velocity && perm), RUBIX_E_INVALID,
                "%s: null particle pointer", who);
  return RUBIX_OK;
}

namespace {

int cube_fwd_impl(const char* who, const float* ssp_flux, const float* ssp_metallicity,
                  const float* ssp_age, const float* ssp_wave_z, int32_t n_met, int32_t n_age,
                  int32_t n_wave, const float* wave_t, int32_t n_wave_t, const float* mass,
                  const float* metallicity, const float* age, const float* velocity,
                  int64_t vel_stride, int32_t vel_component, const int32_t* perm,
                  const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                  const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop, const float* av,
                  const float* dust_e2, float* cube, int64_t spaxel_stride, void* workspace,
                  size_t workspace_bytes, void* stream) {
  {
    bool nothing_to_do = false;
    const int rc = cube_fwd_check_args(who, ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z,
                                       n_met, n_age, n_wave, wave_t, n_wave_t, mass,
                                       metallicity, age, velocity, vel_stride, vel_component,
                                       perm, seg_offsets, n_segments, n, lsf_taps, n_lsf_taps,
                                       lsf_crop, cube, spaxel_stride, &nothing_to_do);
    if (rc != RUBIX_OK || nothing_to_do) return rc;
  }
  const size_t need = rubix_cube_workspace_size(n, n_segments, n_wave_t, n_met, n_age, n_wave);
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= need, RUBIX_E_WORKSPACE,
                "%s: workspace of %zu bytes needed, %zu given", who, need, workspace_bytes);
  RUBIX_REQUIRE((reinterpret_cast<uintptr_t>(workspace) & 255) == 0, RUBIX_E_INVALID,
                "%s: workspace must be 256-byte aligned", who);
  // Up to about 1300 SSP wavelengths two blocks with staged corners fit on an SM, up to
  // about 3000 one.  Larger grids (to about 13 000 wavelengths) read the corners and the
  // SSP wavelengths through L1/L2 instead of staging them, with one or two rows in the
  // pool.
  const int row_cap = n_wave + 2;
  constexpr size_t kSmemMax = 227 * 1024;
  int staged = 1, pool = kPB * row_cap;
  if (smem_layout(n_wave, pool, pool).total > kSmemMax) {
    staged = 0;
    if (smem_layout(0, 0, pool).total > kSmemMax) pool = row_cap;
  }
  const SmemLayout SL = smem_layout(staged ? n_wave : 0, staged ? pool : 0, pool);
  RUBIX_REQUIRE(SL.total <= kSmemMax, RUBIX_E_UNSUPPORTED,
                "%s: SSP grid of %d wavelengths needs %zu bytes of shared memory "
                "(limit 232448)",
                who, n_wave, SL.total);

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const CubeTuning tune = cube_tuning_current();
  const CubeLayout L =
      carve_cube(workspace, n, n_segments, n_wave_t, n_met, n_age, n_wave, tune.chunk);
  const CubeInputs in{ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, n_met, n_age, n_wave,
                      wave_t, n_wave_t, mass, metallicity, age, velocity, vel_stride,
                      vel_component, perm, seg_offsets, n_segments, n, av};
  {
    const int rc = cube_prepare(in, L, tune, /*with_grad=*/false, st);
    if (rc != RUBIX_OK) return rc;
  }
  MainArgs args;
  args.ct = L.ct;
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
  args.staged = staged;
  args.pool = pool;
  args.chunk = tune.chunk;
  args.lsf_k = n_lsf_taps;
  args.lsf_crop = lsf_crop;
  for (int i = 0; i <= kMaxLsfTaps; ++i) args.lsf[i] = i < n_lsf_taps ? lsf_taps[i] : 0.f;
  args.dust_e2 = dust_e2;
  const int need_r = (n_wave_t + kAccThreads - 1) / kAccThreads;
  const size_t smem = SL.total;
  if (need_r <= 1) return launch_main<1>(args, smem, st);
  if (need_r <= 2) return launch_main<2>(args, smem, st);
  if (need_r <= 4) return launch_main<4>(args, smem, st);
  if (need_r <= 6) return launch_main<6>(args, smem, st);
  if (need_r <= 8) return launch_main<8>(args, smem, st);
  if (need_r <= 10) return launch_main<10>(args, smem, st);
  return launch_main<11>(args, smem, st);  // kAccThreads * 11 >= kMaxWaveT
}

}  // namespace

// rubix_cube_fwd under another entry point's name (error messages carry `who`).
int cube_fwd_named(const char* who, const float* ssp_flux, const float* ssp_metallicity,
                   const float* ssp_age, const float* ssp_wave_z, int32_t n_met, int32_t n_age,
                   int32_t n_wave, const float* wave_t, int32_t n_wave_t, const float* mass,
                   const float* metallicity, const float* age, const float* velocity,
                   int64_t vel_stride, int32_t vel_component, const int32_t* perm,
                   const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                   const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop, float* cube,
                   int64_t spaxel_stride, void* workspace, size_t workspace_bytes,
                   void* stream) {
  return cube_fwd_impl(who, ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, n_met, n_age,
                       n_wave, wave_t, n_wave_t, mass, metallicity, age, velocity, vel_stride,
                       vel_component, perm, seg_offsets, n_segments, n, lsf_taps, n_lsf_taps,
                       lsf_crop, nullptr, nullptr, cube, spaxel_stride, workspace,
                       workspace_bytes, stream);
}

}  // namespace rubix

extern "C" int rubix_cube_fwd(const float* ssp_flux, const float* ssp_metallicity,
                              const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                              int32_t n_age, int32_t n_wave, const float* wave_t,
                              int32_t n_wave_t, const float* mass, const float* metallicity,
                              const float* age, const float* velocity, int64_t vel_stride,
                              int32_t vel_component, const int32_t* perm,
                              const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                              const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop,
                              float* cube, int64_t spaxel_stride, void* workspace,
                              size_t workspace_bytes, void* stream) {
  return cube_fwd_impl("rubix_cube_fwd", ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, n_met,
                       n_age, n_wave, wave_t, n_wave_t, mass, metallicity, age, velocity,
                       vel_stride, vel_component, perm, seg_offsets, n_segments, n, lsf_taps,
                       n_lsf_taps, lsf_crop, nullptr, nullptr, cube, spaxel_stride, workspace,
                       workspace_bytes, stream);
}

extern "C" int rubix_cube_fwd_dust(const float* ssp_flux, const float* ssp_metallicity,
                                   const float* ssp_age, const float* ssp_wave_z, int32_t n_met,
                                   int32_t n_age, int32_t n_wave, const float* wave_t,
                                   int32_t n_wave_t, const float* mass, const float* metallicity,
                                   const float* age, const float* velocity, int64_t vel_stride,
                                   int32_t vel_component, const float* av,
                                   const float* ext_exponent, const int32_t* perm,
                                   const int32_t* seg_offsets, int32_t n_segments, int64_t n,
                                   const float* lsf_taps, int32_t n_lsf_taps, int32_t lsf_crop,
                                   float* cube, int64_t spaxel_stride, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(ext_exponent != nullptr && (n == 0 || av != nullptr), RUBIX_E_INVALID,
                "rubix_cube_fwd_dust: null A_V or extinction exponent");
  return cube_fwd_impl("rubix_cube_fwd_dust", ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z,
                       n_met, n_age, n_wave, wave_t, n_wave_t, mass, metallicity, age, velocity,
                       vel_stride, vel_component, perm, seg_offsets, n_segments, n, lsf_taps,
                       n_lsf_taps, lsf_crop, av, ext_exponent, cube, spaxel_stride, workspace,
                       workspace_bytes, stream);
}

extern "C" int rubix_cube_status(const void* workspace, int* device_error, void* stream) {
  RUBIX_REQUIRE(workspace != nullptr && device_error != nullptr, RUBIX_E_INVALID,
                "rubix_cube_status: null pointer");
  const CubeCtrl* ctrl = static_cast<const CubeCtrl*>(workspace);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  RUBIX_CUDA_TRY(cudaMemcpyAsync(device_error, &ctrl->error, sizeof(int),
                                 cudaMemcpyDeviceToHost, st));
  RUBIX_CUDA_TRY(cudaStreamSynchronize(st));
  return *device_error ? set_error(RUBIX_E_DEVICE, "cube kernel: a TMA wait timed out")
                       : RUBIX_OK;
}
