// Ragged batches of galaxies (particles of galaxy g at [poff[g], poff[g+1]), its square
// S_g x S_g spaxel grid at global spaxels [seg_base[g], seg_base[g] + S_g^2)):
//   * spaxel assignment with each galaxy's own bin edges, giving global spaxel ids
//     that the ordinary stable sort and the cube kernels consume unchanged, so one
//     persistent launch renders every galaxy of the batch;
//   * per-galaxy dot products (the PSF-width gradients of a batch).
#include "common.cuh"
#include "particle_frame.cuh"

namespace rubix {
namespace {

// Per particle: galaxy by binary search on poff; ix, iy = clip(digitize - 1) on the
// galaxy's edges (rubix/telescope/utils.py:138-151); kept when inside the inclusive
// aperture [edges[0], edges[-1]] (ascending edges; utils.py:173-174) and when the flat
// id ix + nb*iy is below S_g^2 (ids beyond are dropped by segment_sum, spectra/ifu.py:286).
__global__ void ragged_assign_kernel(const float* __restrict__ coords, long long n,
                                     long long stride, const long long* __restrict__ poff,
                                     int n_gal, const float* __restrict__ edges,
                                     const int* __restrict__ eoff, const int* __restrict__ sbin,
                                     const long long* __restrict__ seg_base,
                                     int* __restrict__ idx_out,
                                     unsigned char* __restrict__ keep_out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = n_gal;  // last g with poff[g] <= i
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (poff[mid] <= i) lo = mid; else hi = mid;
    }
    const int g = lo;
    const float* e = edges + eoff[g];
    const int ne = eoff[g + 1] - eoff[g];
    const float x = coords[i * stride], y = coords[i * stride + 1];
    const int local = spaxel_index(e, ne, x, y);
    const bool inside = inside_aperture(x, y, e[0], e[ne - 1]);
    const int S = sbin[g];
    const bool keep = inside && local < S * S;
    idx_out[i] = keep ? (int)(seg_base[g] + local) : 0;
    keep_out[i] = keep ? 1 : 0;
  }
}

constexpr int kSegDotThreads = 256;
constexpr int kSegDotSplit = 16;  // blocks per segment

// partial[g][j] = sum over block j's share of segment g, double block sums.
__global__ void __launch_bounds__(kSegDotThreads) seg_dot_kernel(
    const float* __restrict__ a, const float* __restrict__ b, const long long* __restrict__ off,
    double* __restrict__ partial) {
  __shared__ double s_w[kSegDotThreads / 32];
  const int g = blockIdx.y, j = blockIdx.x;
  const long long s0 = off[g], s1 = off[g + 1];
  float c0 = 0.f, c1 = 0.f;
  const long long stride = (long long)kSegDotSplit * kSegDotThreads;
  long long i = s0 + (long long)j * kSegDotThreads + threadIdx.x;
  for (; i + stride < s1; i += 2 * stride) {
    c0 = fmaf(a[i], b[i], c0);
    c1 = fmaf(a[i + stride], b[i + stride], c1);
  }
  if (i < s1) c0 = fmaf(a[i], b[i], c0);
  double v = (double)c0 + (double)c1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kSegDotThreads / 32; ++w) t += s_w[w];
    partial[(long long)g * kSegDotSplit + j] = t;
  }
}

__global__ void seg_dot_finish_kernel(const double* __restrict__ partial, int n_seg,
                                      double* __restrict__ out) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n_seg; g += gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int j = 0; j < kSegDotSplit; ++j) t += partial[(long long)g * kSegDotSplit + j];
    out[g] = t;
  }
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_ragged_assign(const float* coords, int64_t n, int64_t coord_stride,
                                   const int64_t* particle_offsets, int32_t n_gal,
                                   const float* edges, const int32_t* edge_offsets,
                                   const int32_t* sbin, const int64_t* seg_base, int32_t* idx_out,
                                   uint8_t* keep_out, void* stream) {
  RUBIX_REQUIRE(n >= 0 && n_gal >= 0 && coord_stride >= 2, RUBIX_E_SHAPE,
                "rubix_ragged_assign: bad sizes");
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(n_gal >= 1, RUBIX_E_SHAPE, "rubix_ragged_assign: particles but no galaxies");
  RUBIX_REQUIRE(coords && particle_offsets && edges && edge_offsets && sbin && seg_base &&
                    idx_out && keep_out,
                RUBIX_E_INVALID, "rubix_ragged_assign: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
  ragged_assign_kernel<<<g, 256, 0, st>>>(coords, n, coord_stride,
                                          reinterpret_cast<const long long*>(particle_offsets),
                                          n_gal, edges, edge_offsets, sbin,
                                          reinterpret_cast<const long long*>(seg_base), idx_out,
                                          keep_out);
  RUBIX_LAUNCH_CHECK("ragged_assign_kernel");
  return RUBIX_OK;
}

extern "C" size_t rubix_segmented_dot_workspace_size(int32_t n_seg) {
  return n_seg > 0 ? sizeof(double) * (size_t)n_seg * kSegDotSplit : 0;
}

extern "C" int rubix_segmented_dot(const float* a, const float* b, const int64_t* offsets,
                                   int32_t n_seg, double* out, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n_seg >= 0, RUBIX_E_SHAPE, "rubix_segmented_dot: n_seg < 0");
  if (n_seg == 0) return RUBIX_OK;
  RUBIX_REQUIRE(a && b && offsets && out, RUBIX_E_INVALID, "rubix_segmented_dot: null pointer");
  RUBIX_REQUIRE(workspace && workspace_bytes >= rubix_segmented_dot_workspace_size(n_seg) &&
                    (reinterpret_cast<uintptr_t>(workspace) & 7) == 0,
                RUBIX_E_WORKSPACE, "rubix_segmented_dot: workspace of %zu bytes needed",
                rubix_segmented_dot_workspace_size(n_seg));
  RUBIX_REQUIRE(n_seg <= 65535, RUBIX_E_SHAPE, "rubix_segmented_dot: at most 65535 segments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partial = static_cast<double*>(workspace);
  seg_dot_kernel<<<dim3(kSegDotSplit, n_seg), kSegDotThreads, 0, st>>>(
      a, b, reinterpret_cast<const long long*>(offsets), partial);
  RUBIX_LAUNCH_CHECK("seg_dot_kernel");
  seg_dot_finish_kernel<<<(n_seg + 255) / 256, 256, 0, st>>>(partial, n_seg, out);
  RUBIX_LAUNCH_CHECK("seg_dot_finish_kernel");
  return RUBIX_OK;
}
