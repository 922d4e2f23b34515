// Kernel (a): aperture mask, spaxel assignment and a stable LSD radix sort of the
// particles by spaxel index, ending in per-spaxel segment offsets.
//
// The radix sort is written from the published LSD scheme: per pass, a per-tile
// digit histogram, one exclusive scan over (digit, tile), and a stable scatter in
// which each tile ranks its keys with warp-level match/popc and per-warp digit
// counters.  No float atomics anywhere; the result is deterministic.
#include "common.cuh"
#include "particle_frame.cuh"
#include "radix.cuh"
#include "scan.cuh"

namespace rubix {
namespace {

constexpr int kMaxSmemEdges = 8192;

__global__ void aperture_mask_kernel(const float* __restrict__ coords, long long n,
                                     long long stride, const float* __restrict__ edges,
                                     int n_edges, unsigned char* __restrict__ mask) {
  __shared__ float s_lo, s_hi;
  if (threadIdx.x == 0) {
    float lo = edges[0], hi = edges[0];
    for (int i = 1; i < n_edges; ++i) {
      lo = fminf(lo, edges[i]);
      hi = fmaxf(hi, edges[i]);
    }
    s_lo = lo;
    s_hi = hi;
  }
  __syncthreads();
  const float lo = s_lo, hi = s_hi;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    mask[i] = inside_aperture(coords[i * stride], coords[i * stride + 1], lo, hi) ? 1 : 0;
  }
}

__global__ void spaxel_assign_kernel(const float* __restrict__ coords, long long n,
                                     long long stride, const float* __restrict__ edges,
                                     int n_edges, int* __restrict__ idx_out) {
  extern __shared__ float s_edges[];
  const bool in_smem = n_edges <= kMaxSmemEdges;
  if (in_smem) {
    for (int i = threadIdx.x; i < n_edges; i += blockDim.x) s_edges[i] = edges[i];
    __syncthreads();
  }
  const float* e = in_smem ? s_edges : edges;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    idx_out[i] = spaxel_index(e, n_edges, coords[i * stride], coords[i * stride + 1]);
}

constexpr int kMaxFrameFields = 8;

// Per-particle float32 fields copied with the particles outside the aperture set to 0.
struct FrameFields {
  const float* in[kMaxFrameFields];
  float* out[kMaxFrameFields];
  int width[kMaxFrameFields];
  int n;
};

// rotate_galaxy + filter_particles + spaxel_assignment in one pass over the particles:
// coordinates and velocities turned by M (when rotate), the aperture mask of the turned
// coordinates, the masked copies of the fields, and the flat spaxel index.  The same
// per-particle arithmetic as rotate_kernel, aperture_mask_kernel and spaxel_assign_kernel.
__global__ void frame_assign_kernel(const float* coords, const float* velocity, long long n,
                                    int rotate, Mat3 M, float* coords_out, float* velocity_out,
                                    const float* __restrict__ edges, int n_edges, FrameFields F,
                                    unsigned char* __restrict__ mask_out,
                                    int* __restrict__ idx_out) {
  extern __shared__ float s_edges[];
  __shared__ float s_lo, s_hi;
  const bool in_smem = n_edges <= kMaxSmemEdges;
  if (in_smem)
    for (int i = threadIdx.x; i < n_edges; i += blockDim.x) s_edges[i] = edges[i];
  if (threadIdx.x == 0) {
    float lo = edges[0], hi = edges[0];
    for (int i = 1; i < n_edges; ++i) {
      lo = fminf(lo, edges[i]);
      hi = fmaxf(hi, edges[i]);
    }
    s_lo = lo;
    s_hi = hi;
  }
  __syncthreads();
  const float* e = in_smem ? s_edges : edges;
  const float lo = s_lo, hi = s_hi;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float x = coords[3 * i], y = coords[3 * i + 1], z = coords[3 * i + 2];
    if (rotate) {
      rotate_row(x, y, z, M, x, y, z);
      coords_out[3 * i] = x;
      coords_out[3 * i + 1] = y;
      coords_out[3 * i + 2] = z;
      float vx, vy, vz;
      rotate_row(velocity[3 * i], velocity[3 * i + 1], velocity[3 * i + 2], M, vx, vy, vz);
      velocity_out[3 * i] = vx;
      velocity_out[3 * i + 1] = vy;
      velocity_out[3 * i + 2] = vz;
    }
    const bool inside = inside_aperture(x, y, lo, hi);
    if (mask_out) mask_out[i] = inside ? 1 : 0;
    for (int f = 0; f < F.n; ++f) {
      const int w = F.width[f];
      for (int k = 0; k < w; ++k) F.out[f][i * w + k] = inside ? F.in[f][i * w + k] : 0.f;
    }
    idx_out[i] = spaxel_index(e, n_edges, x, y);
  }
}

// key = idx if kept and inside [0, n_segments), else n_segments (sorts last).
__global__ void make_keys_kernel(const int* __restrict__ idx,
                                 const unsigned char* __restrict__ keep, long long n,
                                 int n_segments, unsigned* __restrict__ keys,
                                 int* __restrict__ vals) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    int k = idx[i];
    bool ok = (k >= 0) && (k < n_segments) && (keep == nullptr || keep[i] != 0);
    keys[i] = ok ? (unsigned)k : (unsigned)n_segments;
    vals[i] = (int)i;
  }
}

// seg_offsets[s] = first sorted position whose key >= s, for s in [0, n_segments].
__global__ void seg_offsets_kernel(const unsigned* __restrict__ keys, long long n,
                                   int n_segments, int* __restrict__ offsets) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j <= n;
       j += (long long)gridDim.x * blockDim.x) {
    long long lo = (j == 0) ? 0 : (long long)keys[j - 1] + 1;
    long long hi = (j == n) ? n_segments : min((long long)keys[j], (long long)n_segments);
    for (long long s = lo; s <= hi; ++s) offsets[s] = (int)j;
  }
}

int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  long long cap = (long long)sm_count() * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

int sort_passes(int n_segments) {
  unsigned maxkey = (unsigned)n_segments;  // sentinel key value
  int bits = 0;
  while (bits < 32 && (maxkey >> bits) != 0) ++bits;
  if (bits == 0) bits = 1;
  return (bits + kRadixBits - 1) / kRadixBits;
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_aperture_mask(const float* coords, int64_t n, int64_t coord_stride,
                                   const float* edges, int32_t n_edges, uint8_t* mask_out,
                                   void* stream) {
  RUBIX_REQUIRE(n >= 0, RUBIX_E_INVALID, "rubix_aperture_mask: n < 0");
  RUBIX_REQUIRE(n_edges >= 1, RUBIX_E_SHAPE, "rubix_aperture_mask: need at least one edge");
  RUBIX_REQUIRE(coord_stride >= 2, RUBIX_E_SHAPE, "rubix_aperture_mask: coord_stride < 2");
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(coords && edges && mask_out, RUBIX_E_INVALID,
                "rubix_aperture_mask: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  aperture_mask_kernel<<<grid_for(n, 256), 256, 0, st>>>(coords, n, coord_stride, edges,
                                                          n_edges, mask_out);
  RUBIX_LAUNCH_CHECK("aperture_mask_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_spaxel_assign(const float* coords, int64_t n, int64_t coord_stride,
                                   const float* edges, int32_t n_edges, int32_t* idx_out,
                                   void* stream) {
  RUBIX_REQUIRE(n >= 0, RUBIX_E_INVALID, "rubix_spaxel_assign: n < 0");
  RUBIX_REQUIRE(n_edges >= 2, RUBIX_E_SHAPE, "rubix_spaxel_assign: need at least two edges");
  RUBIX_REQUIRE((long long)(n_edges - 1) * (n_edges - 1) < (1LL << 31), RUBIX_E_SHAPE,
                "rubix_spaxel_assign: (n_edges-1)^2 overflows int32");
  RUBIX_REQUIRE(coord_stride >= 2, RUBIX_E_SHAPE, "rubix_spaxel_assign: coord_stride < 2");
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(coords && edges && idx_out, RUBIX_E_INVALID,
                "rubix_spaxel_assign: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  size_t smem = n_edges <= kMaxSmemEdges ? (size_t)n_edges * sizeof(float) : 0;
  spaxel_assign_kernel<<<grid_for(n, 256), 256, smem, st>>>(coords, n, coord_stride, edges,
                                                             n_edges, idx_out);
  RUBIX_LAUNCH_CHECK("spaxel_assign_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_orient_filter_assign(const float* coords, const float* velocity,
                                          int64_t n, const double* matrix9, float* coords_out,
                                          float* velocity_out, const float* edges,
                                          int32_t n_edges, int32_t n_fields,
                                          const float* const* fields_in,
                                          float* const* fields_out,
                                          const int32_t* field_widths, uint8_t* mask_out,
                                          int32_t* idx_out, void* stream) {
  RUBIX_REQUIRE(n >= 0, RUBIX_E_INVALID, "rubix_orient_filter_assign: n < 0");
  RUBIX_REQUIRE(n_edges >= 2, RUBIX_E_SHAPE,
                "rubix_orient_filter_assign: need at least two edges");
  RUBIX_REQUIRE((long long)(n_edges - 1) * (n_edges - 1) < (1LL << 31), RUBIX_E_SHAPE,
                "rubix_orient_filter_assign: (n_edges-1)^2 overflows int32");
  RUBIX_REQUIRE(n_fields >= 0 && n_fields <= kMaxFrameFields, RUBIX_E_INVALID,
                "rubix_orient_filter_assign: n_fields must be in [0, %d]", kMaxFrameFields);
  RUBIX_REQUIRE(n_fields == 0 || (fields_in && fields_out && field_widths), RUBIX_E_INVALID,
                "rubix_orient_filter_assign: null field arrays");
  RUBIX_REQUIRE(n_fields == 0 || mask_out, RUBIX_E_INVALID,
                "rubix_orient_filter_assign: filtered fields need mask_out");
  FrameFields F;
  F.n = n_fields;
  for (int f = 0; f < kMaxFrameFields; ++f) {
    F.in[f] = nullptr;
    F.out[f] = nullptr;
    F.width[f] = 0;
  }
  for (int f = 0; f < n_fields; ++f) {
    RUBIX_REQUIRE(field_widths[f] >= 1, RUBIX_E_SHAPE,
                  "rubix_orient_filter_assign: field %d has width < 1", f);
    RUBIX_REQUIRE(n == 0 || (fields_in[f] && fields_out[f]), RUBIX_E_INVALID,
                  "rubix_orient_filter_assign: field %d has a null pointer", f);
    F.in[f] = fields_in[f];
    F.out[f] = fields_out[f];
    F.width[f] = field_widths[f];
  }
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(coords && edges && idx_out, RUBIX_E_INVALID,
                "rubix_orient_filter_assign: null pointer");
  Mat3 M;
  for (int i = 0; i < 9; ++i) M.m[i] = matrix9 ? matrix9[i] : (i % 4 == 0 ? 1.0 : 0.0);
  if (matrix9)
    RUBIX_REQUIRE(velocity && coords_out && velocity_out, RUBIX_E_INVALID,
                  "rubix_orient_filter_assign: a rotation needs velocity, coords_out and "
                  "velocity_out");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  size_t smem = n_edges <= kMaxSmemEdges ? (size_t)n_edges * sizeof(float) : 0;
  frame_assign_kernel<<<grid_for(n, 256), 256, smem, st>>>(
      coords, velocity, n, matrix9 ? 1 : 0, M, coords_out, velocity_out, edges, n_edges, F,
      mask_out, idx_out);
  RUBIX_LAUNCH_CHECK("frame_assign_kernel");
  return RUBIX_OK;
}

extern "C" size_t rubix_spaxel_sort_workspace_size(int64_t n, int32_t n_segments) {
  if (n < 0 || n_segments < 0) return 0;
  long long n_tiles = (n + kSortTile - 1) / kSortTile;
  if (n_tiles < 1) n_tiles = 1;
  Carve c(nullptr);
  c.take<unsigned>((size_t)n);               // keys A
  c.take<unsigned>((size_t)n);               // keys B
  c.take<int>((size_t)n);                    // vals scratch
  c.take<int>((size_t)kRadix * (n_tiles + 1));  // histogram + digit totals
  return c.off;
}

extern "C" int rubix_spaxel_sort(const int32_t* idx, const uint8_t* keep, int64_t n,
                                 int32_t n_segments, int32_t* perm_out,
                                 int32_t* seg_offsets_out, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n >= 0 && n < (1LL << 31), RUBIX_E_SHAPE,
                "rubix_spaxel_sort: n must be in [0, 2^31)");
  RUBIX_REQUIRE(n_segments >= 0 && n_segments < 0x7fffffff, RUBIX_E_SHAPE,
                "rubix_spaxel_sort: bad n_segments");
  RUBIX_REQUIRE(seg_offsets_out != nullptr, RUBIX_E_INVALID,
                "rubix_spaxel_sort: seg_offsets_out is null");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n == 0) {
    RUBIX_CUDA_TRY(cudaMemsetAsync(seg_offsets_out, 0, sizeof(int) * ((size_t)n_segments + 1), st));
    return RUBIX_OK;
  }
  RUBIX_REQUIRE(idx && perm_out, RUBIX_E_INVALID, "rubix_spaxel_sort: null pointer");
  size_t need = rubix_spaxel_sort_workspace_size(n, n_segments);
  RUBIX_REQUIRE(workspace != nullptr && workspace_bytes >= need, RUBIX_E_WORKSPACE,
                "rubix_spaxel_sort: workspace of %zu bytes needed, %zu given", need,
                workspace_bytes);
  const int n_tiles = (int)((n + kSortTile - 1) / kSortTile);
  Carve c(workspace);
  unsigned* keys_a = c.take<unsigned>((size_t)n);
  unsigned* keys_b = c.take<unsigned>((size_t)n);
  int* vals_ws = c.take<int>((size_t)n);
  int* hist = c.take<int>((size_t)kRadix * (n_tiles + 1));
  int* totals = hist + (long long)kRadix * n_tiles;  // per-digit totals of a pass

  const int passes = sort_passes(n_segments);
  // The last pass must write into perm_out: pass p writes perm_out when
  // (passes-1-p) is even, vals_ws otherwise.
  auto dst_vals = [&](int p) { return ((passes - 1 - p) % 2 == 0) ? perm_out : vals_ws; };
  int* vals_src = (dst_vals(0) == perm_out) ? vals_ws : perm_out;
  make_keys_kernel<<<grid_for(n, 256), 256, 0, st>>>(idx, keep, n, n_segments, keys_a, vals_src);
  RUBIX_LAUNCH_CHECK("make_keys_kernel");
  unsigned* kin = keys_a;
  unsigned* kout = keys_b;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * kRadixBits;
    const unsigned dmask = (unsigned)(kRadix - 1);
    int* vout = dst_vals(p);
    radix_hist_kernel<<<n_tiles, kSortThreads, 0, st>>>(kin, n, shift, dmask, n_tiles, hist);
    RUBIX_LAUNCH_CHECK("radix_hist_kernel");
    radix_rowscan_kernel<<<kRadix, kSortThreads, 0, st>>>(hist, n_tiles, totals);
    RUBIX_LAUNCH_CHECK("radix_rowscan_kernel");
    radix_scatter_kernel<<<n_tiles, kSortThreads, 0, st>>>(kin, vals_src, kout, vout, n, shift,
                                                           dmask, n_tiles, hist, totals);
    RUBIX_LAUNCH_CHECK("radix_scatter_kernel");
    unsigned* tk = kin;
    kin = kout;
    kout = tk;
    vals_src = vout;
  }
  seg_offsets_kernel<<<grid_for(n + 1, 256), 256, 0, st>>>(kin, n, n_segments, seg_offsets_out);
  RUBIX_LAUNCH_CHECK("seg_offsets_kernel");
  return RUBIX_OK;
}
