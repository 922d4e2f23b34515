// Kernel (c): separable 2-D convolution of every wavelength plane of a datacube
// ("same" mode, zero padding).  A Gaussian PSF kernel normalised by its 2-D sum is
// the outer product of two normalised 1-D Gaussians, so rubix's per-plane
// convolve2d with gaussian_kernel_2d (telescope/psf/psf.py:33-58, kernels.py:5-31)
// is an x-pass followed by a y-pass.
//
// A block owns a strip of kTileX spaxel columns by kTileL wavelengths (one warp
// lane per wavelength: coalesced 128-byte row segments along the contiguous
// wavelength axis) and streams down the y axis: each input row is staged in shared
// memory with its x halo, convolved along x into a ring of the last m_y rows, and
// the ring gives the y-convolved output row.  Every input element is read from
// global memory once per strip (plus the x halo) and every output written once.
// When the input's spaxel stride is a multiple of 16 bytes, one thread stages each row
// with a single tiled TMA copy (psf_tma_kernel); otherwise every thread issues 4-byte
// cp.async copies of its share of the row.
#include "common.cuh"
#include "dot_reduce.cuh"
#include "tma.cuh"

#include <cuda.h>  // CUtensorMap and its enums; cuTensorMapEncodeTiled comes through the runtime

namespace rubix {
namespace {

constexpr int kPsfTileX = 32;
constexpr int kPsfTileL = 32;
constexpr int kPsfThreads = 256;
constexpr int kPsfWarps = kPsfThreads / 32;
constexpr int kPsfXPerThread = kPsfTileX / kPsfWarps;
constexpr int kMaxTaps = 63;

struct PsfArgs {
  const float* in;
  float* out;
  int ny, nx, nl;
  long long sin, sout;
  int my, mx, oy, ox;
  float ty[kMaxTaps + 1];
  float tx[kMaxTaps + 1];
  const float* ty_dev;  // when set, the taps are read from device memory instead
  const float* tx_dev;
};

__global__ void __launch_bounds__(kPsfThreads) psf_strip_kernel(PsfArgs a) {
  extern __shared__ float smem[];
  const int wrow = kPsfTileX + a.mx - 1;
  float* s_in = smem;                   // [wrow][kPsfTileL]
  float* s_ring = smem + wrow * kPsfTileL;  // [my][kPsfTileX][kPsfTileL]
  __shared__ float s_ty[kMaxTaps + 1], s_tx[kMaxTaps + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < a.my) s_ty[tid] = a.ty_dev ? a.ty_dev[tid] : a.ty[tid];
  if (tid < a.mx) s_tx[tid] = a.tx_dev ? a.tx_dev[tid] : a.tx[tid];
  const int x0 = blockIdx.x * kPsfTileX;
  const int l0 = blockIdx.y * kPsfTileL;
  const int l = l0 + lane;
  const int xsrc0 = x0 - (a.mx - 1) + a.ox;  // global x of s_in column 0
  const int total = a.ny - 1 + a.oy;
  for (int r = 0; r <= total; ++r) {
    // 1. stage input row r (zero outside the cube)
    for (int q = tid; q < wrow * kPsfTileL; q += kPsfThreads) {
      const int jj = q / kPsfTileL, ll = q % kPsfTileL;
      const int xg = xsrc0 + jj, lg = l0 + ll;
      float v = 0.f;
      if (r < a.ny && xg >= 0 && xg < a.nx && lg < a.nl)
        v = a.in[((long long)r * a.nx + xg) * a.sin + lg];
      s_in[q] = v;
    }
    __syncthreads();
    // 2. x-pass into ring slot r % my
    const int slot = r % a.my;
#pragma unroll
    for (int j = 0; j < kPsfXPerThread; ++j) {
      const int xl = warp + kPsfWarps * j;
      float h = 0.f;
      for (int i = 0; i < a.mx; ++i)
        h = fmaf(s_tx[i], s_in[(xl + (a.mx - 1) - i) * kPsfTileL + lane], h);
      s_ring[(slot * kPsfTileX + xl) * kPsfTileL + lane] = h;
    }
    __syncthreads();
    // 3. y-pass: output row y = r - oy
    const int y = r - a.oy;
    if (y >= 0 && y < a.ny && l < a.nl) {
      const int imax = min(a.my - 1, r);
#pragma unroll
      for (int j = 0; j < kPsfXPerThread; ++j) {
        const int xl = warp + kPsfWarps * j;
        const int x = x0 + xl;
        float o = 0.f;
        int sl = slot;
        for (int i = 0; i <= imax; ++i) {
          o = fmaf(s_ty[i], s_ring[(sl * kPsfTileX + xl) * kPsfTileL + lane], o);
          sl = (sl == 0) ? a.my - 1 : sl - 1;
        }
        if (x < a.nx) a.out[((long long)y * a.nx + x) * a.sout + l] = o;
      }
    }
  }
}


// Register-blocked variant for equal tap counts M <= 21: each thread owns one
// wavelength lane and kPsfXB consecutive x positions; the y window of the last M
// x-convolved rows lives in registers (the row loop is unrolled by M so every window
// index is static).  Input rows are staged by 4-byte cp.async copies into a ring of
// S shared-memory rows (up to 8, as many as 48 KB of static shared memory hold),
// S-1 rows ahead of the row being convolved,
// so each SM keeps several rows of every strip in flight; one barrier per row.
constexpr int kPsfXB = 4;
// Ring depth for a tap count M: as many staged rows as fit in 48 KB, at most 8.
__host__ __device__ constexpr int psf_stages(int M) {
  return (48 * 1024) / ((kPsfTileX + M - 1) * kPsfTileL * 4) >= 8
             ? 8
             : (48 * 1024) / ((kPsfTileX + M - 1) * kPsfTileL * 4);
}

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  const int n = valid ? 4 : 0;  // 0: zero-fill, nothing read
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// The strip (bx, by) of one cube: ny x nx spaxels (spaxel strides sin/sout), nl
// wavelengths, taps ty/tx (M each, any address space), 'same' offsets oy/ox.
// kDot: instead of storing an output o[y][x][l], add w[y][x][l] * o to `dot` (w has
// the output's layout, spaxel stride sout); `out` is not written.
template <int M, bool kDot = false>
__device__ __forceinline__ void psf_reg_body(const float* __restrict__ in, float* __restrict__ out,
                                             int ny, int nx, int nl, long long sin,
                                             long long sout, int oy, int ox,
                                             const float* ty_src, const float* tx_src, int bx,
                                             int by, const float* __restrict__ w = nullptr,
                                             float* dot = nullptr) {
  constexpr int W = kPsfTileX + M - 1;  // staged row width
  constexpr int PER = (W * kPsfTileL + kPsfThreads - 1) / kPsfThreads;
  constexpr int kPsfStages = psf_stages(M);
  static_assert(kPsfStages >= 3, "PSF ring needs at least 3 rows");
  __shared__ float s_in[kPsfStages][W * kPsfTileL];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int x0 = bx * kPsfTileX;
  const int l0 = by * kPsfTileL;
  const int l = l0 + lane;
  const int xsrc0 = x0 - (M - 1) + ox;
  const int xb = warp * kPsfXB;  // first local x of this thread
  float ty[M], tx[M];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    ty[i] = ty_src[i];
    tx[i] = tx_src[i];
  }
  const int total = ny + oy;  // input rows 0 .. ny-1+oy
  // This thread's copies of a staged row: element q = tid + k*256 (column jj = q / 32,
  // lane ll = q % 32) comes from row_base + off[k]; the column/wavelength validity is
  // the same for every row.
  int off[PER];
  unsigned valid = 0u;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int q = tid + k * kPsfThreads;
    const int jj = q / kPsfTileL, ll = q % kPsfTileL;
    const int xg = xsrc0 + jj, lg = l0 + ll;
    const bool ok = q < W * kPsfTileL && xg >= 0 && xg < nx && lg < nl;
    off[k] = ok ? (int)((long long)xg * sin + lg) : 0;
    valid |= ok ? (1u << k) : 0u;
  }
  const long long row_stride = (long long)nx * sin;
  auto issue_row = [&](int r) {
    float* dst = s_in[r % kPsfStages];
    const float* base = in + (long long)r * row_stride;
    const bool row_ok = r < ny;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int q = tid + k * kPsfThreads;
      if (q < W * kPsfTileL) {
        const bool ok = row_ok && ((valid >> k) & 1u);
        cp_async4(dst + q, ok ? base + off[k] : in, ok);
      }
    }
  };
  float win[M][kPsfXB];
#pragma unroll
  for (int i = 0; i < M; ++i)
#pragma unroll
    for (int j = 0; j < kPsfXB; ++j) win[i][j] = 0.f;

#pragma unroll
  for (int r = 0; r < kPsfStages - 1; ++r) {
    if (r < total) issue_row(r);
    cp_async_commit();
  }
  for (int r0 = 0; r0 < total; r0 += M) {
#pragma unroll
    for (int jj = 0; jj < M; ++jj) {
      const int r = r0 + jj;
      if (r >= total) break;
      cp_async_wait<kPsfStages - 2>();  // row r has landed (this thread's copies)
      __syncthreads();                   // ... and every thread's; row r-1 is consumed
      {
        const int rn = r + kPsfStages - 1;
        if (rn < total) issue_row(rn);
        cp_async_commit();
      }
      const float* row = s_in[r % kPsfStages];
      // dot mode: this row's weights, loaded now so the x-pass hides their latency
      float wv[kPsfXB];
      if constexpr (kDot) {
        const int yw = r - oy;
#pragma unroll
        for (int j = 0; j < kPsfXB; ++j) {
          const int x = x0 + xb + j;
          wv[j] = (yw >= 0 && l < nl && x < nx) ? w[((long long)yw * nx + x) * sout + l] : 0.f;
        }
      }
      // x-pass over the staged row r for this thread's kPsfXB positions
      float xv[kPsfXB + M - 1];
#pragma unroll
      for (int q = 0; q < kPsfXB + M - 1; ++q) xv[q] = row[(xb + q) * kPsfTileL + lane];
#pragma unroll
      for (int j = 0; j < kPsfXB; ++j) {
        float h = 0.f;
#pragma unroll
        for (int i = 0; i < M; ++i) h = fmaf(tx[i], xv[j + (M - 1) - i], h);
        win[jj][j] = h;
      }
      // y-pass: output row y = r - oy uses x-convolved rows r - i, i < M
      const int y = r - oy;
      if (y >= 0 && l < nl) {
#pragma unroll
        for (int j = 0; j < kPsfXB; ++j) {
          float o = 0.f;
#pragma unroll
          for (int i = 0; i < M; ++i) o = fmaf(ty[i], win[(jj - i + M) % M][j], o);
          const int x = x0 + xb + j;
          if constexpr (kDot) {
            *dot = fmaf(wv[j], o, *dot);  // wv[j] = 0 outside the cube
          } else {
            if (x < nx) out[((long long)y * nx + x) * sout + l] = o;
          }
        }
      }
    }
  }
  cp_async_wait<0>();
}

template <int M>
__global__ void __launch_bounds__(kPsfThreads) psf_reg_kernel(PsfArgs a) {
  psf_reg_body<M>(a.in, a.out, a.ny, a.nx, a.nl, a.sin, a.sout, a.oy, a.ox,
                  a.ty_dev ? a.ty_dev : a.ty, a.tx_dev ? a.tx_dev : a.tx, blockIdx.x,
                  blockIdx.y);
}

// sum over the cube of w * PSF(in), the PSF with device taps (psf_reg_body's arithmetic
// per output), reduced deterministically; the PSF output is never written.
template <int M>
__global__ void __launch_bounds__(kPsfThreads) psf_dot_kernel(PsfArgs a, const float* w,
                                                             FusedDotScratch* ws, double* out) {
  __shared__ double s_w[kPsfThreads / 32];
  __shared__ int s_last;
  float dot = 0.f;
  psf_reg_body<M, true>(a.in, nullptr, a.ny, a.nx, a.nl, a.sin, a.sout, a.oy, a.ox, a.ty_dev,
                        a.tx_dev, blockIdx.x, blockIdx.y, w, &dot);
  fused_dot_finish(dot, ws, out, s_w, &s_last);
}

// The same strip with packed two-lane FMAs (__ffma2_rn) for host taps: the four x
// positions of a thread form two pairs, so each tap of the x-pass and of the y-pass is
// one FFMA2 per pair.  The x-pass operands (x_k, x_k+1) come as aligned pairs A_m =
// (x_2m, x_2m+1) and shifted pairs B_m = (x_2m+1, x_2m+2); the taps are read from the
// kernel parameters.  Same products and summation order as psf_reg_body, so the
// result is bit-identical.
template <int M>
__global__ void __launch_bounds__(kPsfThreads, 2) psf_reg2_kernel(PsfArgs a) {
  constexpr int W = kPsfTileX + M - 1;  // staged row width
  constexpr int PER = (W * kPsfTileL + kPsfThreads - 1) / kPsfThreads;
  constexpr int kPsfStages = psf_stages(M);
  constexpr int NA = (kPsfXB + M - 1) / 2;  // aligned input pairs per thread and row
  static_assert(kPsfXB == 4 && (M & 1), "two output pairs, odd tap count");
  __shared__ float s_in[kPsfStages][W * kPsfTileL];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float* __restrict__ in = a.in;
  float* __restrict__ out = a.out;
  const int ny = a.ny, nx = a.nx, nl = a.nl, oy = a.oy;
  const long long sin = a.sin, sout = a.sout;
  const int x0 = blockIdx.x * kPsfTileX;
  const int l0 = blockIdx.y * kPsfTileL;
  const int l = l0 + lane;
  const int xsrc0 = x0 - (M - 1) + a.ox;
  const int xb = warp * kPsfXB;
  const int total = ny + oy;
  int off[PER];
  unsigned valid = 0u;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int q = tid + k * kPsfThreads;
    const int jj = q / kPsfTileL, ll = q % kPsfTileL;
    const int xg = xsrc0 + jj, lg = l0 + ll;
    const bool ok = q < W * kPsfTileL && xg >= 0 && xg < nx && lg < nl;
    off[k] = ok ? (int)((long long)xg * sin + lg) : 0;
    valid |= ok ? (1u << k) : 0u;
  }
  const long long row_stride = (long long)nx * sin;
  auto issue_row = [&](int r) {
    float* dst = s_in[r % kPsfStages];
    const float* base = in + (long long)r * row_stride;
    const bool row_ok = r < ny;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int q = tid + k * kPsfThreads;
      if (q < W * kPsfTileL) {
        const bool ok = row_ok && ((valid >> k) & 1u);
        cp_async4(dst + q, ok ? base + off[k] : in, ok);
      }
    }
  };
  float2 win[M][2];  // x-convolved rows r-M+1 .. r of this thread's two output pairs
#pragma unroll
  for (int i = 0; i < M; ++i) {
    win[i][0] = make_float2(0.f, 0.f);
    win[i][1] = win[i][0];
  }
#pragma unroll
  for (int r = 0; r < kPsfStages - 1; ++r) {
    if (r < total) issue_row(r);
    cp_async_commit();
  }
  for (int r0 = 0; r0 < total; r0 += M) {
#pragma unroll
    for (int jj = 0; jj < M; ++jj) {
      const int r = r0 + jj;
      if (r >= total) break;
      cp_async_wait<kPsfStages - 2>();
      __syncthreads();
      {
        const int rn = r + kPsfStages - 1;
        if (rn < total) issue_row(rn);
        cp_async_commit();
      }
      const float* row = s_in[r % kPsfStages];
      float2 A[NA], B[NA - 1];
#pragma unroll
      for (int m = 0; m < NA; ++m) {
        A[m].x = row[(xb + 2 * m) * kPsfTileL + lane];
        A[m].y = row[(xb + 2 * m + 1) * kPsfTileL + lane];
      }
#pragma unroll
      for (int m = 0; m < NA - 1; ++m) B[m] = make_float2(A[m].y, A[m + 1].x);
      float2 h0 = make_float2(0.f, 0.f), h1 = h0;
#pragma unroll
      for (int i = 0; i < M; ++i) {
        const float2 t = make_float2(a.tx[i], a.tx[i]);
        const int k0 = M - 1 - i, k1 = M + 1 - i;  // first input of outputs 0-1 and 2-3
        h0 = __ffma2_rn(t, (k0 & 1) ? B[k0 >> 1] : A[k0 >> 1], h0);
        h1 = __ffma2_rn(t, (k1 & 1) ? B[k1 >> 1] : A[k1 >> 1], h1);
      }
      win[jj][0] = h0;
      win[jj][1] = h1;
      const int y = r - oy;
      if (y >= 0 && l < nl) {
        float2 o0 = make_float2(0.f, 0.f), o1 = o0;
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const float2 t = make_float2(a.ty[i], a.ty[i]);
          o0 = __ffma2_rn(t, win[(jj - i + M) % M][0], o0);
          o1 = __ffma2_rn(t, win[(jj - i + M) % M][1], o1);
        }
        const int x = x0 + xb;
        float* o = out + ((long long)y * nx + x) * sout + l;
        if (x < nx) o[0] = o0.x;
        if (x + 1 < nx) o[sout] = o0.y;
        if (x + 2 < nx) o[2 * sout] = o1.x;
        if (x + 3 < nx) o[3 * sout] = o1.y;
      }
    }
  }
  cp_async_wait<0>();
}

// Device error word of the TMA-staged PSF: set when a bounded wait for a staged row
// runs out (the block then waits for its copies in flight and returns without writing
// the rest of its strip).  Sticky until rubix_psf_status reads it.
__device__ int g_psf_error;

// The strip of psf_reg_body with its input rows staged by TMA: thread 0 loads input
// row r (W spaxel columns from x0 - (M-1) + ox, kTileL wavelengths from l0, zero outside
// the cube) with one tiled copy of the 3-D tensor map (wavelength, x, y) into ring slot
// r % S, completing on that slot's mbarrier, S - 1 rows ahead.  The copies replace the
// per-thread 4-byte copies, their address arithmetic and validity masks.  The
// wavelength coordinate l0 is a multiple of 32 floats (128 bytes), as a tiled copy
// needs; x and y may start outside the cube, where the copy fills zeros.  The x-pass
// runs scalar FMAs on the parameter taps, the y-pass packed FMAs (__ffma2_rn) on tap
// pairs held in registers.  Same products and summation order as psf_reg_body and
// psf_reg2_kernel: bit-identical.
// Ring depth of the TMA-staged kernel: as many staged rows as fit in 48 KB of static
// shared memory next to the slots' mbarriers, at most 8.
__host__ __device__ constexpr int psf_tma_stages(int M) {
  return (48 * 1024 - 256) / ((kPsfTileX + M - 1) * kPsfTileL * 4) >= 8
             ? 8
             : (48 * 1024 - 256) / ((kPsfTileX + M - 1) * kPsfTileL * 4);
}

// kDevTaps: the taps come from device memory (a.ty_dev, a.tx_dev; the differentiable
// render) and the x taps are held in registers too.  kDot: instead of storing an output
// o[y][x][l], add w[y][x][l] * o into a deterministic sum (w has the output's layout,
// spaxel stride a.sout; the row's weights are loaded before its x-pass).
template <int M, bool kDevTaps = false, bool kDot = false>
__global__ void __launch_bounds__(kPsfThreads, 2)
    psf_tma_kernel(const __grid_constant__ CUtensorMap map, PsfArgs a,
                   const float* __restrict__ w = nullptr, FusedDotScratch* dot_ws = nullptr,
                   double* dot_out = nullptr) {
  constexpr int W = kPsfTileX + M - 1;  // staged row width
  constexpr int kS = psf_tma_stages(M);
  static_assert(kS >= 3, "PSF ring needs at least 3 rows");
  constexpr uint32_t kRowBytes = W * kPsfTileL * sizeof(float);
  static_assert(kPsfXB == 4 && (M & 1), "two output pairs, odd tap count");
  static_assert((W * kPsfTileL * sizeof(float)) % 128 == 0, "ring slots stay 128-byte aligned");
  __shared__ __align__(128) float s_in[kS][W * kPsfTileL];
  __shared__ uint64_t s_bar[kS];
  __shared__ int s_fail;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float* __restrict__ out = a.out;
  const int ny = a.ny, nx = a.nx, nl = a.nl, oy = a.oy;
  const long long sout = a.sout;
  const int x0 = blockIdx.x * kPsfTileX;
  const int l0 = blockIdx.y * kPsfTileL;
  const int l = l0 + lane;
  const int xsrc0 = x0 - (M - 1) + a.ox;
  const int xb = warp * kPsfXB;
  const int total = ny + oy;  // input rows 0 .. ny-1+oy (rows >= ny are zero)
  if (tid == 0) {
    for (int i = 0; i < kS; ++i) mbar_init(&s_bar[i], 1);
    fence_mbar_init();
    s_fail = 0;
  }
  __syncthreads();
  if (tid == 0) {
    fence_proxy_async_smem();
    for (int r = 0; r < kS - 1 && r < total; ++r) {
      mbar_arrive_expect_tx(&s_bar[r], kRowBytes);
      tensor_copy_3d_g2s(s_in[r], &map, l0, xsrc0, r, &s_bar[r]);
    }
  }
  float2 win[M][2];  // x-convolved rows r-M+1 .. r of this thread's two output pairs
#pragma unroll
  for (int i = 0; i < M; ++i) {
    win[i][0] = make_float2(0.f, 0.f);
    win[i][1] = win[i][0];
  }
  // y taps as register pairs for the packed FMAs, formed once: made opaque by the move,
  // so the compiler keeps them instead of re-forming pairs from the parameters per use
  float2 typ[M];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    unsigned long long v;
    const float t = kDevTaps ? a.ty_dev[i] : a.ty[i];
    asm volatile("mov.b64 %0, {%1, %1};" : "=l"(v) : "f"(t));
    typ[i] = *reinterpret_cast<const float2*>(&v);
  }
  float txr[M];  // device x taps in registers (host taps are read from the parameters)
#pragma unroll
  for (int i = 0; i < M; ++i) txr[i] = kDevTaps ? a.tx_dev[i] : 0.f;
  float dot = 0.f;
  for (int r0 = 0; r0 < total; r0 += M) {
#pragma unroll
    for (int jj = 0; jj < M; ++jj) {
      const int r = r0 + jj;
      if (r >= total) break;
      const int slot = r % kS;
      if (!mbar_wait_bounded(&s_bar[slot], (uint32_t)(r / kS) & 1u)) s_fail = 1;
      __syncthreads();  // row r landed for every thread; row r - 1 is consumed
      if (s_fail) {
        if (tid == 0) {
          atomicExch(&g_psf_error, 1);
          for (int q = r; q < r + kS - 1 && q < total; ++q)  // rows still in flight
            mbar_wait_bounded(&s_bar[q % kS], (uint32_t)(q / kS) & 1u);
        }
        return;
      }
      if (tid == 0) {  // row r + S - 1 into the slot row r - 1 left
        const int rn = r + kS - 1;
        if (rn < total) {
          fence_proxy_async_smem();
          mbar_arrive_expect_tx(&s_bar[rn % kS], kRowBytes);
          tensor_copy_3d_g2s(s_in[rn % kS], &map, l0, xsrc0, rn, &s_bar[rn % kS]);
        }
      }
      // dot mode: this row's output weights, loaded now so the x-pass hides them
      float wv[kPsfXB];
      if constexpr (kDot) {
        const int yw = r - oy;
#pragma unroll
        for (int j = 0; j < kPsfXB; ++j) {
          const int x = x0 + xb + j;
          wv[j] = (yw >= 0 && l < nl && x < nx) ? w[((long long)yw * nx + x) * sout + l] : 0.f;
        }
      }
      // x-pass: scalar FMAs, the taps straight from the kernel parameters
      const float* row = s_in[slot];
      float xv[kPsfXB + M - 1];
#pragma unroll
      for (int q = 0; q < kPsfXB + M - 1; ++q) xv[q] = row[(xb + q) * kPsfTileL + lane];
      float hs[kPsfXB];
#pragma unroll
      for (int j = 0; j < kPsfXB; ++j) {
        float v = 0.f;
#pragma unroll
        for (int i = 0; i < M; ++i)
          v = fmaf(kDevTaps ? txr[i] : a.tx[i], xv[j + (M - 1) - i], v);
        hs[j] = v;
      }
      win[jj][0] = make_float2(hs[0], hs[1]);
      win[jj][1] = make_float2(hs[2], hs[3]);
      // y-pass: packed FMAs over the two output pairs
      const int y = r - oy;
      if (y >= 0 && l < nl) {
        float2 o0 = make_float2(0.f, 0.f), o1 = o0;
#pragma unroll
        for (int i = 0; i < M; ++i) {
          o0 = __ffma2_rn(typ[i], win[(jj - i + M) % M][0], o0);
          o1 = __ffma2_rn(typ[i], win[(jj - i + M) % M][1], o1);
        }
        if constexpr (kDot) {
          dot = fmaf(wv[0], o0.x, dot);  // wv = 0 outside the cube
          dot = fmaf(wv[1], o0.y, dot);
          dot = fmaf(wv[2], o1.x, dot);
          dot = fmaf(wv[3], o1.y, dot);
        } else {
          const int x = x0 + xb;
          float* o = out + ((long long)y * nx + x) * sout + l;
          if (x < nx) o[0] = o0.x;
          if (x + 1 < nx) o[sout] = o0.y;
          if (x + 2 < nx) o[2 * sout] = o1.x;
          if (x + 3 < nx) o[3 * sout] = o1.y;
        }
      }
    }
  }
  if constexpr (kDot) {
    __shared__ double s_red[kPsfThreads / 32];
    __shared__ int s_last;
    fused_dot_finish(dot, dot_ws, dot_out, s_red, &s_last);
  }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry points (null if unavailable).
EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000,
                                                           cudaEnableDefault, &q);
    return (e == cudaSuccess && q == cudaDriverEntryPointSuccess)
               ? reinterpret_cast<EncodeTiledFn>(f)
               : nullptr;
  }();
  return fn;
}

// The TMA-staged kernel when the input allows tiled copies (16-byte aligned base, spaxel
// stride a multiple of 4 floats); false (nothing launched) otherwise.  With `w` the dot
// mode (device taps) into *dot_out.
template <int M>
bool launch_psf_tma(const PsfArgs& a, cudaStream_t st, const float* w = nullptr,
                    FusedDotScratch* dot_ws = nullptr, double* dot_out = nullptr) {
  if (a.sin % 4 != 0 || (reinterpret_cast<uintptr_t>(a.in) & 15) != 0) return false;
  const EncodeTiledFn enc = encode_tiled();
  if (enc == nullptr) return false;
  constexpr int W = kPsfTileX + M - 1;
  CUtensorMap map;
  const cuuint64_t dims[3] = {(cuuint64_t)a.nl, (cuuint64_t)a.nx, (cuuint64_t)a.ny};
  const cuuint64_t strides[2] = {(cuuint64_t)a.sin * sizeof(float),
                                 (cuuint64_t)a.nx * (cuuint64_t)a.sin * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)kPsfTileL, (cuuint32_t)W, 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(a.in), dims, strides, box,
          elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  dim3 grid(div_up(a.nx, kPsfTileX), div_up(a.nl, kPsfTileL));
  if (w != nullptr)
    psf_tma_kernel<M, true, true><<<grid, kPsfThreads, 0, st>>>(map, a, w, dot_ws, dot_out);
  else if (a.ty_dev != nullptr)
    psf_tma_kernel<M, true><<<grid, kPsfThreads, 0, st>>>(map, a);
  else
    psf_tma_kernel<M><<<grid, kPsfThreads, 0, st>>>(map, a);
  return true;
}

// Ragged batch: galaxy g owns blocks [block_off[g], block_off[g+1]) (x strips fastest),
// its square S_g x S_g cube starts at spaxel seg_base[g], and its taps are
// taps[g][0][:] (y) and taps[g][1][:] (x), zero-padded and centred to M.
struct RaggedPsfArgs {
  const float* in;
  float* out;
  int nl;
  long long sin, sout;
  int n_gal;
  const int* sbin;
  const long long* seg_base;
  const int* block_off;
  const float* taps;
};

template <int M>
__global__ void __launch_bounds__(kPsfThreads) ragged_psf_kernel(RaggedPsfArgs a) {
  const int b = blockIdx.x;
  int lo = 0, hi = a.n_gal;  // galaxy: last g with block_off[g] <= b
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (a.block_off[mid] <= b) lo = mid; else hi = mid;
  }
  const int g = lo;
  const int S = a.sbin[g];
  const int nsx = (S + kPsfTileX - 1) / kPsfTileX;
  const int local = b - a.block_off[g];
  const long long base = a.seg_base[g];
  const float* t = a.taps + (long long)g * 2 * M;
  psf_reg_body<M>(a.in + base * a.sin, a.out + base * a.sout, S, S, a.nl, a.sin, a.sout,
                  (M - 1) / 2, (M - 1) / 2, t, t + M, local % nsx, local / nsx);
}

template <int M>
int launch_psf_reg(const PsfArgs& a, cudaStream_t st) {
  dim3 grid(div_up(a.nx, kPsfTileX), div_up(a.nl, kPsfTileL));
  // rows staged by TMA where the stride allows (up to 17 taps, where the window and the
  // tap pairs stay in registers), host or device taps
  if (M <= 17 && launch_psf_tma<(M <= 17 ? M : 17)>(a, st)) {
    RUBIX_LAUNCH_CHECK("psf_tma_kernel");
    return RUBIX_OK;
  }
  // host taps: the packed-FMA kernel with the taps as parameters
  if (a.ty_dev == nullptr && M <= 17) {
    psf_reg2_kernel<(M <= 17 ? M : 17)><<<grid, kPsfThreads, 0, st>>>(a);
    RUBIX_LAUNCH_CHECK("psf_reg2_kernel");
    return RUBIX_OK;
  }
  psf_reg_kernel<M><<<grid, kPsfThreads, 0, st>>>(a);
  RUBIX_LAUNCH_CHECK("psf_reg_kernel");
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix

using namespace rubix;

namespace rubix {
namespace {

int psf_fwd_impl(const float* in, float* out, int32_t ny, int32_t nx, int32_t n_wave_t,
                 int64_t spaxel_stride_in, int64_t spaxel_stride_out, const float* ty,
                 int32_t m_y, const float* tx, int32_t m_x, bool device_taps, void* stream) {
  const char* sfx = device_taps ? "_dtaps" : "";
  RUBIX_REQUIRE(ny >= 0 && nx >= 0 && n_wave_t >= 0, RUBIX_E_SHAPE,
                "rubix_psf_fwd%s: negative size", sfx);
  RUBIX_REQUIRE(m_y >= 1 && m_y <= 31 && m_x >= 1 && m_x <= kMaxTaps, RUBIX_E_SHAPE,
                "rubix_psf_fwd%s: kernel sizes must satisfy 1 <= m_y <= 31, 1 <= m_x <= %d", sfx,
                kMaxTaps);
  RUBIX_REQUIRE(spaxel_stride_in >= n_wave_t && spaxel_stride_out >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_psf_fwd%s: spaxel stride smaller than n_wave_t", sfx);
  if (ny == 0 || nx == 0 || n_wave_t == 0) return RUBIX_OK;
  RUBIX_REQUIRE(in && out && ty && tx, RUBIX_E_INVALID, "rubix_psf_fwd%s: null pointer", sfx);
  RUBIX_REQUIRE(in != out, RUBIX_E_INVALID, "rubix_psf_fwd%s: in and out must differ", sfx);
  PsfArgs a;
  a.in = in;
  a.out = out;
  a.ny = ny;
  a.nx = nx;
  a.nl = n_wave_t;
  a.sin = spaxel_stride_in;
  a.sout = spaxel_stride_out;
  a.my = m_y;
  a.mx = m_x;
  a.oy = (m_y - 1) / 2;
  a.ox = (m_x - 1) / 2;
  a.ty_dev = device_taps ? ty : nullptr;
  a.tx_dev = device_taps ? tx : nullptr;
  for (int i = 0; i <= kMaxTaps; ++i) {
    a.ty[i] = (!device_taps && i < m_y) ? ty[i] : 0.f;
    a.tx[i] = (!device_taps && i < m_x) ? tx[i] : 0.f;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the register kernel keeps per-row element offsets in 32 bits
  const bool small_rows = (long long)nx * spaxel_stride_in < (1LL << 31);
  if (m_x == m_y && small_rows) {
    switch (m_x) {
      case 1: return launch_psf_reg<1>(a, st);
      case 3: return launch_psf_reg<3>(a, st);
      case 5: return launch_psf_reg<5>(a, st);
      case 7: return launch_psf_reg<7>(a, st);
      case 9: return launch_psf_reg<9>(a, st);
      case 11: return launch_psf_reg<11>(a, st);
      case 13: return launch_psf_reg<13>(a, st);
      case 15: return launch_psf_reg<15>(a, st);
      case 17: return launch_psf_reg<17>(a, st);
      case 19: return launch_psf_reg<19>(a, st);
      case 21: return launch_psf_reg<21>(a, st);
      default: break;
    }
  }
  const size_t smem = sizeof(float) * ((size_t)(kPsfTileX + m_x - 1) * kPsfTileL +
                                       (size_t)m_y * kPsfTileX * kPsfTileL);
  cudaError_t e = cudaFuncSetAttribute(psf_strip_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess)
    return set_error(RUBIX_E_CUDA, "cudaFuncSetAttribute(psf_strip_kernel): %s", cudaGetErrorString(e));
  dim3 grid(div_up(nx, kPsfTileX), div_up(n_wave_t, kPsfTileL));
  psf_strip_kernel<<<grid, kPsfThreads, smem, st>>>(a);
  RUBIX_LAUNCH_CHECK("psf_strip_kernel");
  return RUBIX_OK;
}

}  // namespace
}  // namespace rubix

extern "C" int rubix_psf_fwd(const float* in, float* out, int32_t ny, int32_t nx,
                             int32_t n_wave_t, int64_t spaxel_stride_in,
                             int64_t spaxel_stride_out, const float* ty, int32_t m_y,
                             const float* tx, int32_t m_x, void* stream) {
  return psf_fwd_impl(in, out, ny, nx, n_wave_t, spaxel_stride_in, spaxel_stride_out, ty, m_y,
                      tx, m_x, false, stream);
}

extern "C" int rubix_psf_fwd_dtaps(const float* in, float* out, int32_t ny, int32_t nx,
                                   int32_t n_wave_t, int64_t spaxel_stride_in,
                                   int64_t spaxel_stride_out, const float* ty, int32_t m_y,
                                   const float* tx, int32_t m_x, void* stream) {
  return psf_fwd_impl(in, out, ny, nx, n_wave_t, spaxel_stride_in, spaxel_stride_out, ty, m_y,
                      tx, m_x, true, stream);
}

extern "C" size_t rubix_fused_dot_workspace_size(void) { return sizeof(FusedDotScratch); }

extern "C" int rubix_psf_dot_dtaps(const float* in, int64_t spaxel_stride_in, const float* w,
                                   int64_t spaxel_stride_w, int32_t ny, int32_t nx,
                                   int32_t n_wave_t, const float* ty, const float* tx, int32_t m,
                                   double* out, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  RUBIX_REQUIRE(ny >= 0 && nx >= 0 && n_wave_t >= 0, RUBIX_E_SHAPE,
                "rubix_psf_dot_dtaps: negative size");
  RUBIX_REQUIRE(m >= 1 && m <= 21 && (m & 1), RUBIX_E_UNSUPPORTED,
                "rubix_psf_dot_dtaps: tap count must be odd and <= 21, got %d", m);
  RUBIX_REQUIRE(spaxel_stride_in >= n_wave_t && spaxel_stride_w >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_psf_dot_dtaps: spaxel stride smaller than n_wave_t");
  RUBIX_REQUIRE((long long)nx * spaxel_stride_in < (1LL << 31), RUBIX_E_SHAPE,
                "rubix_psf_dot_dtaps: rows too long");
  RUBIX_REQUIRE(out != nullptr, RUBIX_E_INVALID, "rubix_psf_dot_dtaps: null output");
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= sizeof(FusedDotScratch) &&
                    (reinterpret_cast<uintptr_t>(workspace) & 7) == 0,
                RUBIX_E_WORKSPACE,
                "rubix_psf_dot_dtaps: workspace of %zu bytes (8-byte aligned) needed",
                sizeof(FusedDotScratch));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (ny == 0 || nx == 0 || n_wave_t == 0) {
    RUBIX_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double), st));
    return RUBIX_OK;
  }
  RUBIX_REQUIRE(in && w && ty && tx, RUBIX_E_INVALID, "rubix_psf_dot_dtaps: null pointer");
  const dim3 grid(div_up(nx, kPsfTileX), div_up(n_wave_t, kPsfTileL));
  RUBIX_REQUIRE((long long)grid.x * grid.y <= kFusedDotMaxBlocks, RUBIX_E_SHAPE,
                "rubix_psf_dot_dtaps: cube too large (%u x %u strips > %d)", grid.x, grid.y,
                kFusedDotMaxBlocks);
  PsfArgs a;
  a.in = in;
  a.out = nullptr;
  a.ny = ny;
  a.nx = nx;
  a.nl = n_wave_t;
  a.sin = spaxel_stride_in;
  a.sout = spaxel_stride_w;
  a.my = a.mx = m;
  a.oy = a.ox = (m - 1) / 2;
  a.ty_dev = ty;
  a.tx_dev = tx;
  auto* scratch = static_cast<FusedDotScratch*>(workspace);
  RUBIX_CUDA_TRY(cudaMemsetAsync(&scratch->counter, 0, sizeof(unsigned), st));
  // rows staged by TMA where the input's stride allows (m <= 17), else 4-byte copies
  bool tma = false;
  switch (m) {
#define RUBIX_PSF_DOT_TMA(MM) \
  case MM: tma = launch_psf_tma<MM>(a, st, w, scratch, out); break;
    RUBIX_PSF_DOT_TMA(1)
    RUBIX_PSF_DOT_TMA(3)
    RUBIX_PSF_DOT_TMA(5)
    RUBIX_PSF_DOT_TMA(7)
    RUBIX_PSF_DOT_TMA(9)
    RUBIX_PSF_DOT_TMA(11)
    RUBIX_PSF_DOT_TMA(13)
    RUBIX_PSF_DOT_TMA(15)
    RUBIX_PSF_DOT_TMA(17)
#undef RUBIX_PSF_DOT_TMA
    default:
      break;
  }
  if (tma) {
    RUBIX_LAUNCH_CHECK("psf_tma_kernel");
    return RUBIX_OK;
  }
  switch (m) {
#define RUBIX_PSF_DOT(MM)                                                   \
  case MM:                                                                  \
    psf_dot_kernel<MM><<<grid, kPsfThreads, 0, st>>>(a, w, scratch, out);   \
    break;
    RUBIX_PSF_DOT(1)
    RUBIX_PSF_DOT(3)
    RUBIX_PSF_DOT(5)
    RUBIX_PSF_DOT(7)
    RUBIX_PSF_DOT(9)
    RUBIX_PSF_DOT(11)
    RUBIX_PSF_DOT(13)
    RUBIX_PSF_DOT(15)
    RUBIX_PSF_DOT(17)
    RUBIX_PSF_DOT(19)
    RUBIX_PSF_DOT(21)
#undef RUBIX_PSF_DOT
    default:
      break;
  }
  RUBIX_LAUNCH_CHECK("psf_dot_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_psf_status(int* device_error, void* stream) {
  RUBIX_REQUIRE(device_error != nullptr, RUBIX_E_INVALID, "rubix_psf_status: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int v = 0;
  RUBIX_CUDA_TRY(cudaMemcpyFromSymbolAsync(&v, g_psf_error, sizeof(int), 0,
                                           cudaMemcpyDeviceToHost, st));
  RUBIX_CUDA_TRY(cudaStreamSynchronize(st));
  *device_error = v;
  if (v == 0) return RUBIX_OK;
  const int zero = 0;
  RUBIX_CUDA_TRY(cudaMemcpyToSymbolAsync(g_psf_error, &zero, sizeof(int), 0,
                                         cudaMemcpyHostToDevice, st));
  RUBIX_CUDA_TRY(cudaStreamSynchronize(st));
  return set_error(RUBIX_E_DEVICE, "psf kernel: a TMA wait timed out");
}

extern "C" int rubix_ragged_psf_fwd(const float* in, float* out, int32_t n_wave_t,
                                    int64_t spaxel_stride_in, int64_t spaxel_stride_out,
                                    int32_t n_gal, const int32_t* sbin, const int64_t* seg_base,
                                    const int32_t* block_offsets, int32_t n_blocks,
                                    const float* taps, int32_t m, void* stream) {
  RUBIX_REQUIRE(n_gal >= 0 && n_wave_t >= 0 && n_blocks >= 0, RUBIX_E_SHAPE,
                "rubix_ragged_psf_fwd: negative size");
  RUBIX_REQUIRE(m >= 1 && m <= 21 && (m & 1), RUBIX_E_SHAPE,
                "rubix_ragged_psf_fwd: padded tap count must be odd and <= 21, got %d", m);
  RUBIX_REQUIRE(spaxel_stride_in >= n_wave_t && spaxel_stride_out >= n_wave_t, RUBIX_E_SHAPE,
                "rubix_ragged_psf_fwd: spaxel stride smaller than n_wave_t");
  if (n_gal == 0 || n_wave_t == 0 || n_blocks == 0) return RUBIX_OK;
  RUBIX_REQUIRE(in && out && sbin && seg_base && block_offsets && taps, RUBIX_E_INVALID,
                "rubix_ragged_psf_fwd: null pointer");
  RUBIX_REQUIRE(in != out, RUBIX_E_INVALID, "rubix_ragged_psf_fwd: in and out must differ");
  RUBIX_REQUIRE(64LL * spaxel_stride_in < (1LL << 31), RUBIX_E_SHAPE,
                "rubix_ragged_psf_fwd: spaxel stride too large");
  RaggedPsfArgs a{in, out, n_wave_t, spaxel_stride_in, spaxel_stride_out, n_gal, sbin,
                  reinterpret_cast<const long long*>(seg_base), block_offsets, taps};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (m) {
#define RUBIX_RAGGED_PSF(MM)                                              \
  case MM:                                                                \
    ragged_psf_kernel<MM><<<n_blocks, kPsfThreads, 0, st>>>(a);           \
    break;
    RUBIX_RAGGED_PSF(1)
    RUBIX_RAGGED_PSF(3)
    RUBIX_RAGGED_PSF(5)
    RUBIX_RAGGED_PSF(7)
    RUBIX_RAGGED_PSF(9)
    RUBIX_RAGGED_PSF(11)
    RUBIX_RAGGED_PSF(13)
    RUBIX_RAGGED_PSF(15)
    RUBIX_RAGGED_PSF(17)
    RUBIX_RAGGED_PSF(19)
    RUBIX_RAGGED_PSF(21)
#undef RUBIX_RAGGED_PSF
    default:
      break;
  }
  RUBIX_LAUNCH_CHECK("ragged_psf_kernel");
  return RUBIX_OK;
}
