// Galaxy orientation (rubix/galaxy/alignment.py:66-265 via rubix/core/rotation.py:11-117):
// the moment-of-inertia tensor of the particles within the half-mass radius, and the
// rotation of coordinates and velocities by a 3x3 matrix (x' = x M, row vectors).
//
// The tensor reproduces a property of rubix's implementation: it selects the particles
// with jnp.where(distance <= radius, size=N), which pads the index list with index 0, so
// particle 0 enters (N - n_inside) more times (alignment.py:92-100).  Sums are float64:
// per-thread partials, block partials, then one block adding the block partials in
// index order (deterministic).
#include "common.cuh"
#include "particle_frame.cuh"

namespace rubix {
namespace {

constexpr int kInThreads = 256;
constexpr int kInBlocks = 512;
constexpr int kInVals = 7;  // xx, yy, zz, xy, xz, yz (mass-weighted sums), count

__device__ __forceinline__ void inertia_terms(double x, double y, double z, double m,
                                              double (&t)[6]) {
  const double r2 = x * x + y * y + z * z;
  t[0] = m * r2 - m * x * x;
  t[1] = m * r2 - m * y * y;
  t[2] = m * r2 - m * z * z;
  t[3] = -m * x * y;
  t[4] = -m * x * z;
  t[5] = -m * y * z;
}

__global__ void __launch_bounds__(kInThreads) inertia_partial_kernel(
    const float* __restrict__ pos, long long stride, const float* __restrict__ mass,
    long long n, float radius, double* __restrict__ partial) {
  __shared__ double s[kInThreads / 32][kInVals];
  double acc[kInVals] = {0, 0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)kInThreads + threadIdx.x; i < n;
       i += (long long)gridDim.x * kInThreads) {
    const float x = pos[i * stride], y = pos[i * stride + 1], z = pos[i * stride + 2];
    // distances = sqrt(sum pos^2) in float32, compared with the radius (alignment.py:91-95)
    const float d = sqrtf(x * x + y * y + z * z);
    if (d <= radius) {
      double t[6];
      inertia_terms(x, y, z, mass[i], t);
#pragma unroll
      for (int j = 0; j < 6; ++j) acc[j] += t[j];
      acc[6] += 1.0;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kInVals; ++j) {
    double v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) s[w][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < kInVals) {
    double v = 0.0;
    for (int k = 0; k < kInThreads / 32; ++k) v += s[k][threadIdx.x];
    partial[(long long)blockIdx.x * kInVals + threadIdx.x] = v;
  }
}

// Block partials summed by one warp per value (lane-strided, then a fixed shuffle tree:
// deterministic), then the padding correction and the 3x3 layout by thread 0.
__global__ void __launch_bounds__(kInVals * 32) inertia_finish_kernel(
    const double* __restrict__ partial, int n_blocks, const float* __restrict__ pos,
    const float* __restrict__ mass, long long n, double* __restrict__ out) {
  __shared__ double s_v[kInVals];
  const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
  double acc = 0.0;
  for (int b = lane; b < n_blocks; b += 32) acc += partial[(long long)b * kInVals + j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) s_v[j] = acc;
  __syncthreads();
  if (threadIdx.x != 0) return;
  double v[kInVals];
  for (int q = 0; q < kInVals; ++q) v[q] = s_v[q];
  // index padding of jnp.where(..., size=N): particle 0 once more per particle outside
  const double extra = (double)n - v[6];
  if (n > 0 && extra > 0.0) {
    double t[6];
    inertia_terms(pos[0], pos[1], pos[2], mass[0], t);
    for (int j = 0; j < 6; ++j) v[j] += extra * t[j];
  }
  out[0] = v[0];
  out[1] = v[3];
  out[2] = v[4];
  out[3] = v[3];
  out[4] = v[1];
  out[5] = v[5];
  out[6] = v[4];
  out[7] = v[5];
  out[8] = v[2];
}

__global__ void rotate_kernel(const float* __restrict__ in, float* __restrict__ out,
                              long long n, long long stride_in, long long stride_out, Mat3 M) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    rotate_row(in[i * stride_in], in[i * stride_in + 1], in[i * stride_in + 2], M,
               out[i * stride_out], out[i * stride_out + 1], out[i * stride_out + 2]);
  }
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" size_t rubix_inertia_workspace_size(void) {
  return sizeof(double) * (size_t)kInBlocks * kInVals;
}

extern "C" int rubix_inertia_tensor(const float* positions, int64_t n, int64_t stride,
                                    const float* masses, float halfmass_radius, double* out9,
                                    void* workspace, size_t workspace_bytes, void* stream) {
  RUBIX_REQUIRE(n >= 0 && stride >= 3, RUBIX_E_SHAPE, "rubix_inertia_tensor: bad sizes");
  RUBIX_REQUIRE(out9 && (n == 0 || (positions && masses)), RUBIX_E_INVALID,
                "rubix_inertia_tensor: null pointer");
  RUBIX_REQUIRE(workspace && workspace_bytes >= rubix_inertia_workspace_size() &&
                    (reinterpret_cast<uintptr_t>(workspace) & 7) == 0,
                RUBIX_E_WORKSPACE, "rubix_inertia_tensor: workspace of %zu bytes needed",
                rubix_inertia_workspace_size());
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* partial = static_cast<double*>(workspace);
  inertia_partial_kernel<<<kInBlocks, kInThreads, 0, st>>>(positions, stride, masses, n,
                                                          halfmass_radius, partial);
  RUBIX_LAUNCH_CHECK("inertia_partial_kernel");
  inertia_finish_kernel<<<1, kInVals * 32, 0, st>>>(partial, kInBlocks, positions, masses, n,
                                                    out9);
  RUBIX_LAUNCH_CHECK("inertia_finish_kernel");
  return RUBIX_OK;
}

extern "C" int rubix_rotate_vectors(const float* in, float* out, int64_t n, int64_t stride_in,
                                    int64_t stride_out, const double* matrix9, void* stream) {
  RUBIX_REQUIRE(n >= 0 && stride_in >= 3 && stride_out >= 3, RUBIX_E_SHAPE,
                "rubix_rotate_vectors: bad sizes");
  RUBIX_REQUIRE(matrix9 != nullptr, RUBIX_E_INVALID, "rubix_rotate_vectors: null matrix");
  if (n == 0) return RUBIX_OK;
  RUBIX_REQUIRE(in && out, RUBIX_E_INVALID, "rubix_rotate_vectors: null pointer");
  Mat3 M;
  for (int i = 0; i < 9; ++i) M.m[i] = matrix9[i];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int g = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
  rotate_kernel<<<g, 256, 0, st>>>(in, out, n, stride_in, stride_out, M);
  RUBIX_LAUNCH_CHECK("rotate_kernel");
  return RUBIX_OK;
}
