// Dust extinction of the stars by the gas in front of them: rubix's
// calculate_extinction step (rubix/core/dust.py:16-65) through apply_spaxel_extinction
// (rubix/spectra/dust/dust_extinction.py:169-358).
//
// rubix, per spaxel s (a sequential scan over all spaxels, each step over all cells):
//   * gas and stars lexsorted by (pixel assignment, z); segments by searchsorted;
//   * the spaxel's cells keep (z, cumulative extinction within the spaxel), every other
//     cell becomes (z * 1e30, 0); the pairs are sorted by the first value (stable);
//   * each star of the spaxel takes jnp.interp of its z on those pairs, extrapolating
//     linearly on the left and clamping on the right: its A_V.
// Here the same A_V comes from one pass per star over precomputed orders:
//   P order  the cells by (pixel assignment, z): segments and cumulative sums;
//   Q order  P order re-sorted by (segment, z): the interpolation nodes of a spaxel
//            (equal to P order unless assignments reach past the last spaxel);
//   G order  every cell by fl32(z * fl32(1e30)), stable from P order, with the run
//            structure of the segment ids, so that "the last cell of another spaxel with
//            key <= x" is one binary search and one run lookup.
// A star's interpolation nodes are its spaxel's Q-ordered cells merged with the G
// entries of the other spaxels, the merge order being (key, P position), exactly the
// order of rubix's stable sort.  Only the two nodes bracketing the star (or the first
// two / last two) are ever formed.
#include "common.cuh"
#include "radix.cuh"
#include "scan.cuh"

namespace rubix {
namespace {

// Monotone map of a float onto unsigned keys (-0 and +0 tie; NaN after +inf).
__device__ __forceinline__ unsigned float_key(float f) {
  if (f == 0.f) f = 0.f;
  unsigned u = __float_as_uint(f);
  if (f != f) u = 0x7fc00000u;
  return u ^ ((unsigned)((int)u >> 31) | 0x80000000u);
}

struct DgrParams {  // 1 / 10^(a + alpha (x_sol - g)); "broken": (a_lo, alpha_lo) at g <= x_t
  float x_sol, a_hi, alpha_hi, a_lo, alpha_lo, x_t;
  int broken;
};

__global__ void gas_extinction_kernel(const float* __restrict__ mass,
                                      const float* __restrict__ metals, long long mstride,
                                      int h_col, int o_col, long long n, DgrParams p, float scale,
                                      float area, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float h = metals[i * mstride + h_col], o = metals[i * mstride + o_col];
    const float g = __fadd_rn(12.f, log10f(__fdiv_rn(o, __fmul_rn(16.f, h))));
    const float d = __fsub_rn(p.x_sol, g);
    const float yh = __fadd_rn(p.a_hi, __fmul_rn(p.alpha_hi, d));
    float y = yh;
    if (p.broken && !(g > p.x_t)) y = __fadd_rn(p.a_lo, __fmul_rn(p.alpha_lo, d));
    const float dgr = __fdiv_rn(1.f, exp10f(y));
    const float dm = __fmul_rn(mass[i], dgr);
    out[i] = __fdiv_rn(__fmul_rn(dm, scale), area);
  }
}

// Keys of the z pass: float_key(z), values = cell index.
__global__ void dust_zkeys_kernel(const float* __restrict__ coords, long long stride, long long n,
                                  unsigned* __restrict__ keys, int* __restrict__ vals) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    keys[i] = float_key(coords[i * stride + 2]);
    vals[i] = (int)i;
  }
}

// Keys of the assignment pass for the z-sorted cells: the pixel assignment clamped to
// [0, pa_max]; with `perm`, order holds P positions (cell = perm[order[j]]).
__global__ void dust_pakeys_kernel(const int* __restrict__ pa, const int* __restrict__ order,
                                   const int* __restrict__ perm, long long n, int pa_max,
                                   unsigned* __restrict__ keys) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    int c = order[j];
    if (perm) c = perm[c];
    keys[j] = (unsigned)min(max(pa[c], 0), pa_max);
  }
}

// z keys of cells given in P order (for the Q and G sorts); values = P position.
__global__ void dust_pzkeys_kernel(const float* __restrict__ coords, long long stride,
                                   const int* __restrict__ perm, long long n, int scaled,
                                   unsigned* __restrict__ keys, int* __restrict__ vals) {
  const float big = 1e30f;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    const float z = coords[(long long)perm[j] * stride + 2];
    keys[j] = float_key(scaled ? __fmul_rn(z, big) : z);
    vals[j] = (int)j;
  }
}

// seg_off[s] = first P position whose segment min(key, nseg-1) >= s; seg_off[nseg] = n.
__global__ void dust_segoff_kernel(const unsigned* __restrict__ keys, long long n, int nseg,
                                   int* __restrict__ seg_off) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j <= n;
       j += (long long)gridDim.x * blockDim.x) {
    const long long lo = (j == 0) ? 0 : (long long)min(keys[j - 1], (unsigned)(nseg - 1)) + 1;
    const long long hi = (j == n) ? nseg : (long long)min(keys[j], (unsigned)(nseg - 1));
    for (long long s = lo; s <= hi; ++s) seg_off[s] = (int)j;
  }
}

// The cells' extinction in P order (so that the segmented sums read contiguously).
__global__ void dust_gather_kernel(const float* __restrict__ ext, const int* __restrict__ perm,
                                   long long n, float* __restrict__ ext_p) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x)
    ext_p[j] = ext[perm[j]];
}

// Inclusive cumulative sum of the cells' extinction within each segment, in P order:
// one warp per segment, 4 x 32 cells loaded ahead, then scanned 32 at a time with a
// running carry.
__global__ void dust_cumsum_kernel(const float* __restrict__ ext_p,
                                   const int* __restrict__ seg_off, int nseg,
                                   float* __restrict__ cum) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nseg; s += warps) {
    const int b = seg_off[s], e = seg_off[s + 1];
    float carry = 0.f;
    for (int base = b; base < e; base += 128) {
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = base + 32 * q + lane;
        v[q] = j < e ? ext_p[j] : 0.f;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float x = v[q];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x = __fadd_rn(x, y);
        }
        x = __fadd_rn(x, carry);
        const int j = base + 32 * q + lane;
        if (j < e) cum[j] = x;
        carry = __shfl_sync(0xffffffffu, x, 31);
      }
    }
  }
}

// Interpolation nodes in Q order: z, cumulative value and P position of each.
__global__ void dust_nodes_kernel(const float* __restrict__ coords, long long stride,
                                  const int* __restrict__ perm, const int* __restrict__ qpos,
                                  const float* __restrict__ cum, long long n,
                                  float* __restrict__ nz, float* __restrict__ nf,
                                  int* __restrict__ np_) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int j = qpos ? qpos[q] : (int)q;
    nz[q] = coords[(long long)perm[j] * stride + 2];
    nf[q] = cum[j];
    np_[q] = j;
  }
}

// G order arrays: key fl32(z * 1e30), segment, P position; run-start flags.
__global__ void dust_gorder_kernel(const float* __restrict__ coords, long long stride,
                                   const int* __restrict__ perm, const int* __restrict__ pa,
                                   const int* __restrict__ gpos, long long n, int nseg,
                                   float* __restrict__ gk, int* __restrict__ gs,
                                   int* __restrict__ gp) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const int j = gpos[k];
    const int c = perm[j];
    gk[k] = __fmul_rn(coords[(long long)c * stride + 2], 1e30f);
    gs[k] = min(max(pa[c], 0), nseg - 1);
    gp[k] = j;
  }
}

// Runs of equal segment ids in G order: flags[k] = 1 at a run start (exclusive scan
// gives run ids).
__global__ void dust_runflag_kernel(const int* __restrict__ gs, long long n,
                                    int* __restrict__ flags) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x)
    flags[k] = (k == 0 || gs[k] != gs[k - 1]) ? 1 : 0;
}

// run_id[k] (in place over the scanned flags) and run_start[run] = first k of the run;
// run_start[n_runs] = n.
__global__ void dust_runs_kernel(const int* __restrict__ gs, long long n, int* __restrict__ rid,
                                 int* __restrict__ run_start) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const bool start = (k == 0 || gs[k] != gs[k - 1]);
    const int r = rid[k] + (start ? 1 : 0) - 1;  // exclusive count of starts before k
    rid[k] = r;
    if (start) run_start[r] = (int)k;
    if (k == n - 1) run_start[r + 1] = (int)n;
  }
}

struct DustView {
  const float* nz;  // Q order: node z, cumulative value, P position
  const float* nf;
  const int* np_;
  const int* seg_off;
  const float* gk;  // G order: key, segment, P position, run id; run starts
  const int* gs;
  const int* gp;
  const int* rid;
  const int* run_start;
  int ng, nseg;
};

struct Node {
  float x, f;
  int p;  // P position (tie order)
  bool ok;
  bool own;  // a cell of the star's own spaxel (its value is a cumulative sum)
};

__device__ __forceinline__ bool node_before(const Node& a, const Node& b) {
  return a.x < b.x || (a.x == b.x && a.p < b.p);
}

__device__ __forceinline__ Node own_node(const DustView& v, int q) {
  return Node{v.nz[q], v.nf[q], v.np_[q], true, true};
}

__device__ __forceinline__ Node other_node(const DustView& v, int k) {
  if (k < 0 || k >= v.ng) return Node{0.f, 0.f, 0, false, false};
  return Node{v.gk[k], 0.f, v.gp[k], true, false};
}

__device__ __forceinline__ Node no_node() { return Node{0.f, 0.f, 0, false, false}; }

// First G index >= k outside segment s (ng if none); last G index <= k outside s (-1).
__device__ __forceinline__ int other_next(const DustView& v, int k, int s) {
  if (k >= v.ng) return v.ng;
  return v.gs[k] != s ? k : v.run_start[v.rid[k] + 1];
}
__device__ __forceinline__ int other_prev(const DustView& v, int k, int s) {
  if (k < 0) return -1;
  return v.gs[k] != s ? k : v.run_start[v.rid[k]] - 1;
}

// Number of entries of a[b, e) that are <= x (ascending a).
__device__ __forceinline__ int upper_bound(const float* __restrict__ a, int b, int e, float x) {
  int lo = b, hi = e;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ float interp_pair(const Node& L, const Node& R, float x) {
  // jnp.interp's formula: fp[i-1] + (x - xp[i-1]) / dx * df, fp[i-1] where |dx| is tiny
  const float df = __fsub_rn(R.f, L.f);
  const float dx = __fsub_rn(R.x, L.x);
  const float delta = __fsub_rn(x, L.x);
  if (fabsf(dx) <= 1.4210855e-14f) return L.f;  // spacing(float32 eps)
  return __fadd_rn(L.f, __fmul_rn(__fdiv_rn(delta, dx), df));
}

// How a star's A_V follows from the merged nodes of its spaxel.
enum StarMode { kNoGas = 0, kLast = 1, kFlat = 2, kInterp = 3 };

struct StarInterp {
  Node A, B, last;
  int mode;  // kNoGas: 0; kLast: last.f (one node, or right of every node); kFlat: A.f
             // (a pair closer than float32 spacing); kInterp: A.f + (x - A.x)/dx * df
};

// The nodes of one star at height x in spaxel s (jnp.interp with left extrapolation
// on rubix's merged (key, value) pairs, the pairs formed only where needed).
__device__ __forceinline__ StarInterp star_interp(const DustView& v, float x, int s) {
  StarInterp r;
  r.A = r.B = r.last = no_node();
  r.mode = kNoGas;
  if (v.ng == 0) return r;
  const int ob = v.seg_off[s], oe = v.seg_off[s + 1];
  // last node of the merged order (right clamp) and the single-node case
  Node last = oe > ob ? own_node(v, oe - 1) : no_node();
  {
    const Node t = other_node(v, other_prev(v, v.ng - 1, s));
    if (t.ok && (!last.ok || node_before(last, t))) last = t;
  }
  r.last = last;
  if (v.ng == 1) {
    r.mode = kLast;
    return r;
  }
  const int qo = upper_bound(v.nz, ob, oe, x);  // own nodes <= x: [ob, qo)
  const int kg = upper_bound(v.gk, 0, v.ng, x);  // G entries <= x: [0, kg)
  Node L = qo > ob ? own_node(v, qo - 1) : no_node();
  Node R = qo < oe ? own_node(v, qo) : no_node();
  {
    const Node t = other_node(v, other_prev(v, kg - 1, s));
    if (t.ok && (!L.ok || node_before(L, t))) L = t;
    const Node u = other_node(v, other_next(v, kg, s));
    if (u.ok && (!R.ok || node_before(u, R))) R = u;
  }
  Node A, B;
  if (!L.ok) {
    // x below every node: the first two nodes (left extrapolation)
    const Node o0 = ob < oe ? own_node(v, ob) : no_node();
    const Node o1 = ob + 1 < oe ? own_node(v, ob + 1) : no_node();
    const int g0 = other_next(v, 0, s);
    const Node t0 = other_node(v, g0);
    const Node t1 = other_node(v, other_next(v, g0 + 1, s));
    if (o0.ok && (!t0.ok || node_before(o0, t0))) {
      A = o0;
      B = (o1.ok && (!t0.ok || node_before(o1, t0))) ? o1 : t0;
    } else {
      A = t0;
      B = (o0.ok && (!t1.ok || node_before(o0, t1))) ? o0 : t1;
    }
  } else if (!R.ok) {
    // x at or above every node: the last two nodes
    const Node o1 = oe > ob ? own_node(v, oe - 1) : no_node();
    const Node o0 = oe - 1 > ob ? own_node(v, oe - 2) : no_node();
    const int g1 = other_prev(v, v.ng - 1, s);
    const Node t1 = other_node(v, g1);
    const Node t0 = other_node(v, other_prev(v, g1 - 1, s));
    if (o1.ok && (!t1.ok || node_before(t1, o1))) {
      B = o1;
      A = (o0.ok && (!t1.ok || node_before(t1, o0))) ? o0 : t1;
    } else {
      B = t1;
      A = (o1.ok && (!t0.ok || node_before(t0, o1))) ? o1 : t0;
    }
  } else {
    A = L;
    B = R;
  }
  r.A = A;
  r.B = B;
  if (x > last.x)
    r.mode = kLast;
  else
    r.mode = fabsf(__fsub_rn(B.x, A.x)) <= 1.4210855e-14f ? kFlat : kInterp;
  return r;
}

__global__ void dust_star_av_kernel(DustView v, const float* __restrict__ coords,
                                    long long stride, const int* __restrict__ pa, long long n,
                                    float* __restrict__ av) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float x = coords[i * stride + 2];
    const int s = min(max(pa[i], 0), v.nseg - 1);
    const StarInterp r = star_interp(v, x, s);
    float f = 0.f;
    if (r.mode == kLast)
      f = r.last.f;
    else if (r.mode != kNoGas)
      f = interp_pair(r.A, r.B, x);
    av[i] = f;
  }
}

// Adjoint of dust_star_av_kernel for an upstream gradient g_i = dL/dA_V,i.  A_V is
// a_A f_A + a_B f_B of (at most) two node values, f = 0 for cells of other spaxels and
// the cumulative extinction of the spaxel's cells up to the node otherwise; its
// derivative in the star's z is g df/dx between two nodes (the node positions, i.e.
// the gas heights, are held fixed).  Each star emits two records (P position of the
// node, or n_gas for a node whose value does not depend on the cells; weight) and its
// z derivative.
__global__ void dust_star_av_bwd_kernel(DustView v, const float* __restrict__ coords,
                                        long long stride, const int* __restrict__ pa,
                                        long long n, const float* __restrict__ dav,
                                        float* __restrict__ dz, unsigned* __restrict__ rkey,
                                        int* __restrict__ rval, float* __restrict__ rw) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float x = coords[i * stride + 2];
    const int s = min(max(pa[i], 0), v.nseg - 1);
    const float g = dav[i];
    const StarInterp r = star_interp(v, x, s);
    const unsigned none = (unsigned)v.ng;
    unsigned ka = none, kb = none;
    float wa = 0.f, wb = 0.f, gz = 0.f;
    if (r.mode == kLast) {
      if (r.last.own) { ka = (unsigned)r.last.p; wa = g; }
    } else if (r.mode == kFlat) {
      if (r.A.own) { ka = (unsigned)r.A.p; wa = g; }
    } else if (r.mode == kInterp) {
      const float dx = __fsub_rn(r.B.x, r.A.x);
      const float q = __fdiv_rn(__fsub_rn(x, r.A.x), dx);
      const float df = __fsub_rn(r.B.f, r.A.f);
      gz = g * (df / dx);
      if (r.A.own) { ka = (unsigned)r.A.p; wa = g * (1.f - q); }
      if (r.B.own) { kb = (unsigned)r.B.p; wb = g * q; }
    }
    dz[i] = gz;
    rkey[2 * i] = ka;
    rkey[2 * i + 1] = kb;
    rval[2 * i] = (int)(2 * i);
    rval[2 * i + 1] = (int)(2 * i + 1);
    rw[2 * i] = wa;
    rw[2 * i + 1] = wb;
  }
}

// Records sorted by node (stable): each thread sums the runs of equal keys inside its
// tile of kRunTile records in order (float64) and writes the sum at the position where
// the run's part in this tile begins.
constexpr int kRunTile = 256;

__global__ void dust_run_partial_kernel(const unsigned* __restrict__ key,
                                        const int* __restrict__ val,
                                        const float* __restrict__ w, long long n,
                                        double* __restrict__ partial) {
  const long long tiles = (n + kRunTile - 1) / kRunTile;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tiles;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t * kRunTile, e = min(n, b + kRunTile);
    long long start = b;
    double sum = 0.0;
    for (long long j = b; j < e; ++j) {
      if (j > b && key[j] != key[j - 1]) {
        partial[start] = sum;
        start = j;
        sum = 0.0;
      }
      sum += (double)w[val[j]];
    }
    partial[start] = sum;
  }
}

// The total of every run that starts in this thread's tile: its partial there plus the
// partials at the starts of the following tiles it reaches into, in tile order; runs
// of key >= n_gas are dropped.  gnode[key] = total (gnode zeroed before).
__global__ void dust_run_total_kernel(const unsigned* __restrict__ key,
                                      const double* __restrict__ partial, long long n,
                                      unsigned n_gas, double* __restrict__ gnode) {
  const long long tiles = (n + kRunTile - 1) / kRunTile;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tiles;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t * kRunTile, e = min(n, b + kRunTile);
    for (long long j = b; j < e; ++j) {
      if (j > 0 && key[j] == key[j - 1]) continue;  // not a run start
      const unsigned k = key[j];
      if (k >= n_gas) continue;
      double tot = partial[j];
      for (long long nb = e; nb < n && key[nb] == k; nb += kRunTile) tot += partial[nb];
      gnode[k] = tot;
    }
  }
}

// Per segment of the P order (one warp each), the suffix sums of the node gradients:
// d ext_P[j] = sum over P positions q >= j of the segment of gnode[q] (cum[q] holds
// ext_P[j] for every j <= q of the segment), written to the cell perm[j].
__global__ void dust_suffix_kernel(const double* __restrict__ gnode,
                                   const int* __restrict__ seg_off, int nseg,
                                   const int* __restrict__ perm, float* __restrict__ dext) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nseg; s += warps) {
    const int b = seg_off[s], e = seg_off[s + 1];
    double carry = 0.0;
    for (int top = e; top > b; top -= 32) {
      const int j = top - 1 - lane;  // lane 0 the highest position of this chunk
      double x = j >= b ? gnode[j] : 0.0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      x += carry;
      if (j >= b) dext[perm[j]] = (float)x;
      carry = __shfl_sync(0xffffffffu, x, 31);
    }
  }
}

// d ext / d(mass, H, O) of gas_extinction_kernel times the upstream dL/d ext:
// ext = mass dgr scale / area, dgr = 10^-y, y = a + alpha (x_sol - g),
// g = 12 + log10(O / (16 H)): d ext/d mass = dgr scale / area, d ext/dO = alpha ext / O,
// d ext/dH = -alpha ext / H (alpha of the branch the forward took).
__global__ void gas_extinction_bwd_kernel(const float* __restrict__ mass,
                                          const float* __restrict__ metals, long long mstride,
                                          int h_col, int o_col, long long n, DgrParams p,
                                          float scale, float area,
                                          const float* __restrict__ dext,
                                          float* __restrict__ dmass, float* __restrict__ dh,
                                          float* __restrict__ dox) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float h = metals[i * mstride + h_col], o = metals[i * mstride + o_col];
    const float g = __fadd_rn(12.f, log10f(__fdiv_rn(o, __fmul_rn(16.f, h))));
    const float d = __fsub_rn(p.x_sol, g);
    float y = __fadd_rn(p.a_hi, __fmul_rn(p.alpha_hi, d));
    float alpha = p.alpha_hi;
    if (p.broken && !(g > p.x_t)) {
      y = __fadd_rn(p.a_lo, __fmul_rn(p.alpha_lo, d));
      alpha = p.alpha_lo;
    }
    const float dgr = __fdiv_rn(1.f, exp10f(y));
    const float k = __fdiv_rn(__fmul_rn(dgr, scale), area);  // d ext / d mass
    const float ext = __fmul_rn(mass[i], k);
    const float gi = dext[i];
    dmass[i] = gi * k;
    dox[i] = gi * alpha * ext / o;
    dh[i] = -gi * alpha * ext / h;
  }
}

// rows[i][t] *= 2^(e[t] * av[i]): the dust transmission on materialised spectra.
__global__ void dust_rows_kernel(float* __restrict__ rows, long long n, int L,
                                 long long row_stride, const float* __restrict__ av,
                                 const float* __restrict__ e) {
  const long long total = n * (long long)L;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const long long i = k / L;
    const int t = (int)(k - i * L);
    float* p = rows + i * row_stride + t;
    *p = __fmul_rn(*p, dust_transmission(e[t], av[i]));
  }
}

int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  const long long cap = (long long)sm_count() * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

int key_bits(unsigned max_key) {
  int b = 0;
  while (b < 32 && (max_key >> b) != 0) ++b;
  return (b + kRadixBits - 1) / kRadixBits * kRadixBits;
}

struct DustLayout {
  unsigned *k0, *k1;
  int *v0, *v1, *hist;
  int *perm, *seg_off;
  float *cum, *nz, *nf, *gk;
  int *np_, *gs, *gp, *rid, *run_start;
  size_t bytes;
};

DustLayout carve_dust(void* base, long long ng, int nseg) {
  Carve c(base);
  DustLayout L;
  const size_t n = (size_t)(ng > 0 ? ng : 1);
  L.k0 = c.take<unsigned>(n);
  L.k1 = c.take<unsigned>(n);
  L.v0 = c.take<int>(n);
  L.v1 = c.take<int>(n);
  L.hist = c.take<int>((size_t)radix_hist_ints(ng));
  L.perm = c.take<int>(n);
  L.seg_off = c.take<int>((size_t)nseg + 1);
  L.cum = c.take<float>(n);
  L.nz = c.take<float>(n);
  L.nf = c.take<float>(n);
  L.np_ = c.take<int>(n);
  L.gk = c.take<float>(n);
  L.gs = c.take<int>(n);
  L.gp = c.take<int>(n);
  L.rid = c.take<int>(n + 1);
  L.run_start = c.take<int>(n + 1);
  L.bytes = c.off;
  return L;
}

struct DustBwdLayout {
  DustLayout fwd;
  unsigned *rk0, *rk1;
  int *rv0, *rv1, *rhist;
  float* rw;
  double *partial, *gnode;
  size_t bytes;
};

DustBwdLayout carve_dust_bwd(void* base, long long ng, int nseg, long long ns) {
  DustBwdLayout B;
  B.fwd = carve_dust(base, ng, nseg);
  Carve c(base ? static_cast<char*>(base) + B.fwd.bytes : nullptr);
  const size_t nr = (size_t)(2 * (ns > 0 ? ns : 1));
  B.rk0 = c.take<unsigned>(nr);
  B.rk1 = c.take<unsigned>(nr);
  B.rv0 = c.take<int>(nr);
  B.rv1 = c.take<int>(nr);
  B.rhist = c.take<int>((size_t)radix_hist_ints((long long)nr));
  B.rw = c.take<float>(nr);
  B.partial = c.take<double>(nr);
  B.gnode = c.take<double>((size_t)(ng > 0 ? ng : 1));
  B.bytes = B.fwd.bytes + c.off;
  return B;
}

}  // namespace
}  // namespace rubix

namespace rubix {
namespace {

// The node structure of rubix_dust_av (P, Q and G orders, segment offsets, cumulative
// sums) built in the layout L; v describes it to the star kernels.
int dust_setup(const float* gas_coords, int64_t gas_stride, const int32_t* gas_pa,
               const float* gas_ext, int64_t n_gas, int32_t n_segments, int32_t pa_limit,
               const DustLayout& L, DustView& v, cudaStream_t st) {
  const long long ng = n_gas;
  v = DustView{};
  v.ng = (int)ng;
  v.nseg = n_segments;
  if (ng > 0) {
    const int G = grid_for(ng, 256);
    // P order: z pass, then the (clamped) assignment pass, both stable.
    dust_zkeys_kernel<<<G, 256, 0, st>>>(gas_coords, gas_stride, ng, L.k0, L.v0);
    int w = radix_sort_pairs(L.k0, L.v0, L.k1, L.v1, ng, 32, L.hist, st);
    unsigned* kz = w ? L.k1 : L.k0;
    int* vz = w ? L.v1 : L.v0;
    unsigned* ko = w ? L.k0 : L.k1;
    int* vo = w ? L.v0 : L.v1;
    dust_pakeys_kernel<<<G, 256, 0, st>>>(gas_pa, vz, nullptr, ng, pa_limit - 1, kz);
    w = radix_sort_pairs(kz, vz, ko, vo, ng, key_bits((unsigned)(pa_limit - 1)), L.hist, st);
    const unsigned* kp = w ? ko : kz;
    const int* vp = w ? vo : vz;
    RUBIX_CUDA_TRY(cudaMemcpyAsync(L.perm, vp, sizeof(int) * ng, cudaMemcpyDeviceToDevice, st));
    dust_segoff_kernel<<<grid_for(ng + 1, 256), 256, 0, st>>>(kp, ng, n_segments, L.seg_off);
    // L.nz holds the P-ordered extinction until the node pass overwrites it
    dust_gather_kernel<<<G, 256, 0, st>>>(gas_ext, L.perm, ng, L.nz);
    dust_cumsum_kernel<<<grid_for((long long)n_segments * 32, 256), 256, 0, st>>>(
        L.nz, L.seg_off, n_segments, L.cum);
    // Q order: only differs from P order when assignments reach past the last spaxel.
    const int* qpos = nullptr;
    if (pa_limit > n_segments) {
      dust_pzkeys_kernel<<<G, 256, 0, st>>>(gas_coords, gas_stride, L.perm, ng, 0, L.k0, L.v0);
      w = radix_sort_pairs(L.k0, L.v0, L.k1, L.v1, ng, 32, L.hist, st);
      unsigned* kq = w ? L.k1 : L.k0;
      int* vq = w ? L.v1 : L.v0;
      unsigned* kq2 = w ? L.k0 : L.k1;
      int* vq2 = w ? L.v0 : L.v1;
      dust_pakeys_kernel<<<G, 256, 0, st>>>(gas_pa, vq, L.perm, ng, n_segments - 1, kq);
      w = radix_sort_pairs(kq, vq, kq2, vq2, ng, key_bits((unsigned)(n_segments - 1)), L.hist,
                           st);
      // the Q positions go to gp (free until the G pass) so the node pass can read them
      RUBIX_CUDA_TRY(cudaMemcpyAsync(L.gp, w ? vq2 : vq, sizeof(int) * ng,
                                     cudaMemcpyDeviceToDevice, st));
      qpos = L.gp;
    }
    dust_nodes_kernel<<<G, 256, 0, st>>>(gas_coords, gas_stride, L.perm, qpos, L.cum, ng, L.nz,
                                         L.nf, L.np_);
    // G order: keys fl32(z * 1e30), stable from P order.
    dust_pzkeys_kernel<<<G, 256, 0, st>>>(gas_coords, gas_stride, L.perm, ng, 1, L.k0, L.v0);
    w = radix_sort_pairs(L.k0, L.v0, L.k1, L.v1, ng, 32, L.hist, st);
    dust_gorder_kernel<<<G, 256, 0, st>>>(gas_coords, gas_stride, L.perm, gas_pa,
                                          w ? L.v1 : L.v0, ng, n_segments, L.gk, L.gs, L.gp);
    dust_runflag_kernel<<<G, 256, 0, st>>>(L.gs, ng, L.rid);
    scan_exclusive_1block<<<1, 1024, 0, st>>>(L.rid, ng, 0);
    dust_runs_kernel<<<G, 256, 0, st>>>(L.gs, ng, L.rid, L.run_start);
    RUBIX_LAUNCH_CHECK("dust column passes");
    v.nz = L.nz;
    v.nf = L.nf;
    v.np_ = L.np_;
    v.seg_off = L.seg_off;
    v.gk = L.gk;
    v.gs = L.gs;
    v.gp = L.gp;
    v.rid = L.rid;
    v.run_start = L.run_start;
  }
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_dust_gas_extinction(const float* mass, const float* metals,
                                         int64_t metals_stride, int32_t h_col, int32_t o_col,
                                         int64_t n, const float* dgr_params, int32_t broken,
                                         float scale, float spaxel_area, float* ext_out,
                                         void* stream) {
  RUBIX_REQUIRE(n >= 0, RUBIX_E_INVALID, "rubix_dust_gas_extinction: n < 0");
  RUBIX_REQUIRE(h_col >= 0 && o_col >= 0 && h_col < metals_stride && o_col < metals_stride,
                RUBIX_E_INVALID, "rubix_dust_gas_extinction: H/O columns outside the rows");
  RUBIX_REQUIRE(dgr_params != nullptr, RUBIX_E_INVALID,
                "rubix_dust_gas_extinction: null dgr_params");
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(mass && metals && ext_out, RUBIX_E_INVALID,
                "rubix_dust_gas_extinction: null pointer");
  DgrParams p{dgr_params[0], dgr_params[1], dgr_params[2], dgr_params[3], dgr_params[4],
              dgr_params[5], broken};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gas_extinction_kernel<<<grid_for(n, 256), 256, 0, st>>>(mass, metals, metals_stride, h_col,
                                                          o_col, n, p, scale, spaxel_area,
                                                          ext_out);
  RUBIX_LAUNCH_CHECK("gas_extinction_kernel");
  return RUBIX_OK;
}

extern "C" size_t rubix_dust_av_workspace_size(int64_t n_gas, int32_t n_segments) {
  if (n_gas < 0 || n_segments < 1) return 0;
  return carve_dust(nullptr, n_gas, n_segments).bytes;
}

extern "C" int rubix_dust_av(const float* gas_coords, int64_t gas_stride, const int32_t* gas_pa,
                             const float* gas_ext, int64_t n_gas, const float* star_coords,
                             int64_t star_stride, const int32_t* star_pa, int64_t n_stars,
                             int32_t n_segments, int32_t pa_limit, float* av_out,
                             void* workspace, size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n_gas >= 0 && n_gas < (1LL << 31) - 1, RUBIX_E_SHAPE,
                "rubix_dust_av: n_gas must be in [0, 2^31 - 1)");
  RUBIX_REQUIRE(n_stars >= 0, RUBIX_E_SHAPE, "rubix_dust_av: n_stars < 0");
  RUBIX_REQUIRE(n_segments >= 1 && pa_limit >= n_segments, RUBIX_E_SHAPE,
                "rubix_dust_av: need 1 <= n_segments <= pa_limit");
  RUBIX_REQUIRE(gas_stride >= 3 && star_stride >= 3, RUBIX_E_SHAPE,
                "rubix_dust_av: coordinate rows need 3 components");
  if (n_stars == 0) return RUBIX_OK;
  RUBIX_REQUIRE(star_coords && star_pa && av_out, RUBIX_E_INVALID,
                "rubix_dust_av: null star pointer");
  RUBIX_REQUIRE(n_gas == 0 || (gas_coords && gas_pa && gas_ext), RUBIX_E_INVALID,
                "rubix_dust_av: null gas pointer");
  const size_t need = rubix_dust_av_workspace_size(n_gas, n_segments);
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= need, RUBIX_E_WORKSPACE,
                "rubix_dust_av: workspace of %zu bytes needed, %zu given", need,
                workspace_bytes);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const DustLayout L = carve_dust(workspace, n_gas, n_segments);
  DustView v{};
  {
    const int rc = dust_setup(gas_coords, gas_stride, gas_pa, gas_ext, n_gas, n_segments,
                              pa_limit, L, v, st);
    if (rc != RUBIX_OK) return rc;
  }
  // one star per thread: the binary searches are latency-bound, so no grid cap
  const long long star_blocks = (n_stars + 255) / 256;
  dust_star_av_kernel<<<(unsigned)std::min<long long>(star_blocks, 1LL << 30), 256, 0, st>>>(
      v, star_coords, star_stride, star_pa, n_stars, av_out);
  RUBIX_LAUNCH_CHECK("dust_star_av_kernel");
  return RUBIX_OK;
}

extern "C" size_t rubix_dust_av_bwd_workspace_size(int64_t n_gas, int32_t n_segments,
                                                   int64_t n_stars) {
  if (n_gas < 0 || n_segments < 1 || n_stars < 0) return 0;
  return carve_dust_bwd(nullptr, n_gas, n_segments, n_stars).bytes;
}

extern "C" int rubix_dust_av_bwd(const float* gas_coords, int64_t gas_stride,
                                 const int32_t* gas_pa, const float* gas_ext, int64_t n_gas,
                                 const float* star_coords, int64_t star_stride,
                                 const int32_t* star_pa, int64_t n_stars, int32_t n_segments,
                                 int32_t pa_limit, const float* grad_av, float* grad_star_z,
                                 float* grad_gas_ext, void* workspace, size_t workspace_bytes,
                                 void* stream) {
  RUBIX_REQUIRE(n_gas >= 0 && n_gas < (1LL << 31) - 1, RUBIX_E_SHAPE,
                "rubix_dust_av_bwd: n_gas must be in [0, 2^31 - 1)");
  RUBIX_REQUIRE(n_stars >= 0 && n_stars < (1LL << 30), RUBIX_E_SHAPE,
                "rubix_dust_av_bwd: n_stars must be in [0, 2^30)");
  RUBIX_REQUIRE(n_segments >= 1 && pa_limit >= n_segments, RUBIX_E_SHAPE,
                "rubix_dust_av_bwd: need 1 <= n_segments <= pa_limit");
  RUBIX_REQUIRE(gas_stride >= 3 && star_stride >= 3, RUBIX_E_SHAPE,
                "rubix_dust_av_bwd: coordinate rows need 3 components");
  RUBIX_REQUIRE(n_stars == 0 || (star_coords && star_pa && grad_av && grad_star_z),
                RUBIX_E_INVALID, "rubix_dust_av_bwd: null star pointer");
  RUBIX_REQUIRE(n_gas == 0 || (gas_coords && gas_pa && gas_ext && grad_gas_ext),
                RUBIX_E_INVALID, "rubix_dust_av_bwd: null gas pointer");
  const size_t need = rubix_dust_av_bwd_workspace_size(n_gas, n_segments, n_stars);
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= need, RUBIX_E_WORKSPACE,
                "rubix_dust_av_bwd: workspace of %zu bytes needed, %zu given", need,
                workspace_bytes);
  RUBIX_REQUIRE((reinterpret_cast<uintptr_t>(workspace) & 255) == 0, RUBIX_E_INVALID,
                "rubix_dust_av_bwd: workspace must be 256-byte aligned");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n_gas > 0)
    RUBIX_CUDA_TRY(cudaMemsetAsync(grad_gas_ext, 0, sizeof(float) * (size_t)n_gas, st));
  if (n_stars == 0) return RUBIX_OK;
  const DustBwdLayout B = carve_dust_bwd(workspace, n_gas, n_segments, n_stars);
  DustView v{};
  {
    const int rc = dust_setup(gas_coords, gas_stride, gas_pa, gas_ext, n_gas, n_segments,
                              pa_limit, B.fwd, v, st);
    if (rc != RUBIX_OK) return rc;
  }
  const long long star_blocks = (n_stars + 255) / 256;
  dust_star_av_bwd_kernel<<<(unsigned)std::min<long long>(star_blocks, 1LL << 30), 256, 0,
                            st>>>(v, star_coords, star_stride, star_pa, n_stars, grad_av,
                                  grad_star_z, B.rk0, B.rv0, B.rw);
  RUBIX_LAUNCH_CHECK("dust_star_av_bwd_kernel");
  if (n_gas == 0) return RUBIX_OK;
  // records by node, stable (the star order within a node), summed per node in order
  const long long nr = 2 * n_stars;
  const int w = radix_sort_pairs(B.rk0, B.rv0, B.rk1, B.rv1, nr, key_bits((unsigned)n_gas),
                                 B.rhist, st);
  const unsigned* rk = w ? B.rk1 : B.rk0;
  const int* rv = w ? B.rv1 : B.rv0;
  const long long tiles = (nr + kRunTile - 1) / kRunTile;
  dust_run_partial_kernel<<<grid_for(tiles, 128), 128, 0, st>>>(rk, rv, B.rw, nr, B.partial);
  RUBIX_CUDA_TRY(cudaMemsetAsync(B.gnode, 0, sizeof(double) * (size_t)n_gas, st));
  dust_run_total_kernel<<<grid_for(tiles, 128), 128, 0, st>>>(rk, B.partial, nr,
                                                              (unsigned)n_gas, B.gnode);
  dust_suffix_kernel<<<grid_for((long long)n_segments * 32, 256), 256, 0, st>>>(
      B.gnode, B.fwd.seg_off, n_segments, B.fwd.perm, grad_gas_ext);
  RUBIX_LAUNCH_CHECK("dust A_V adjoint passes");
  return RUBIX_OK;
}

extern "C" int rubix_dust_gas_extinction_bwd(const float* mass, const float* metals,
                                             int64_t metals_stride, int32_t h_col,
                                             int32_t o_col, int64_t n, const float* dgr_params,
                                             int32_t broken, float scale, float spaxel_area,
                                             const float* grad_ext, float* grad_mass,
                                             float* grad_h, float* grad_o, void* stream) {
  RUBIX_REQUIRE(n >= 0, RUBIX_E_INVALID, "rubix_dust_gas_extinction_bwd: n < 0");
  RUBIX_REQUIRE(h_col >= 0 && o_col >= 0 && h_col < metals_stride && o_col < metals_stride,
                RUBIX_E_INVALID, "rubix_dust_gas_extinction_bwd: H/O columns outside the rows");
  RUBIX_REQUIRE(dgr_params != nullptr, RUBIX_E_INVALID,
                "rubix_dust_gas_extinction_bwd: null dgr_params");
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(mass && metals && grad_ext && grad_mass && grad_h && grad_o, RUBIX_E_INVALID,
                "rubix_dust_gas_extinction_bwd: null pointer");
  DgrParams p{dgr_params[0], dgr_params[1], dgr_params[2], dgr_params[3], dgr_params[4],
              dgr_params[5], broken};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  gas_extinction_bwd_kernel<<<grid_for(n, 256), 256, 0, st>>>(
      mass, metals, metals_stride, h_col, o_col, n, p, scale, spaxel_area, grad_ext, grad_mass,
      grad_h, grad_o);
  RUBIX_LAUNCH_CHECK("gas_extinction_bwd_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_dust_apply_rows(float* rows, int64_t n, int32_t n_wave_t,
                                     int64_t row_stride, const float* av,
                                     const float* ext_exponent, void* stream) {
  RUBIX_REQUIRE(n >= 0 && n_wave_t >= 0 && row_stride >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_dust_apply_rows: bad shape");
  if (n == 0 || n_wave_t == 0) return RUBIX_OK;
  RUBIX_REQUIRE(rows && av && ext_exponent, RUBIX_E_INVALID,
                "rubix_dust_apply_rows: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  dust_rows_kernel<<<grid_for(n * (long long)n_wave_t, 256), 256, 0, st>>>(
      rows, n, n_wave_t, row_stride, av, ext_exponent);
  RUBIX_LAUNCH_CHECK("dust_rows_kernel");
  return RUBIX_OK;
}
