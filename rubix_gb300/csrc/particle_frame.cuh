// Per-particle arithmetic shared by the orientation, aperture and spaxel-assignment
// kernels, so the separate launches and the fused pass give bit-identical results.
#pragma once

#include "common.cuh"

namespace rubix {

// A 3x3 matrix (row-major) applied to row vectors: x' = x M (rubix's
// jnp.dot(positions, R), rubix/galaxy/alignment.py:208-265), in float64 and rounded once.
struct Mat3 {
  double m[9];
};

__device__ __forceinline__ void rotate_row(double x, double y, double z, const Mat3& M,
                                           float& ox, float& oy, float& oz) {
  ox = (float)(x * M.m[0] + y * M.m[3] + z * M.m[6]);
  oy = (float)(x * M.m[1] + y * M.m[4] + z * M.m[7]);
  oz = (float)(x * M.m[2] + y * M.m[5] + z * M.m[8]);
}

// Number of edges <= x (searchsorted side='right'); NaN counts as above all edges,
// matching the NaN-last comparator of jnp.digitize.
__device__ __forceinline__ int count_le(const float* e, int n, float x) {
  if (x != x) return n;
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (e[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// square_spaxel_assignment (rubix/telescope/utils.py:138-151): clip(digitize - 1) per
// axis, flat index ix + nb * iy.
__device__ __forceinline__ int spaxel_index(const float* e, int n_edges, float x, float y) {
  const int nb = n_edges - 1;
  int ix = count_le(e, n_edges, x) - 1;
  int iy = count_le(e, n_edges, y) - 1;
  ix = min(max(ix, 0), nb - 1);
  iy = min(max(iy, 0), nb - 1);
  return ix + nb * iy;
}

// mask_particles_outside_aperture (rubix/telescope/utils.py:173-174): inclusive bounds.
__device__ __forceinline__ bool inside_aperture(float x, float y, float lo, float hi) {
  return x >= lo && x <= hi && y >= lo && y <= hi;
}

}  // namespace rubix
