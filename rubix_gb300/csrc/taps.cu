// Normalised 1-D Gaussian taps and their derivative with respect to sigma, from a sigma
// held in device memory, so that a differentiable render never reads sigma back to the
// host.  rubix's PSF kernel is the outer product of two such taps
// (telescope/psf/kernels.py:5-31) and its LSF kernel one (telescope/lsf/lsf.py:12-26):
//   e_i = exp(-x_i^2 / (2 sigma^2)),  t_i = e_i / sum e,
//   dt_i/dsigma = (e_i x_i^2 / sigma^3 - t_i sum_j e_j x_j^2 / sigma^3) / sum e,
// in float64, rounded to float32.
#include "common.cuh"

namespace rubix {
namespace {

constexpr int kMaxGaussTaps = 64;

struct TapsArgs {
  double x[kMaxGaussTaps];
  int m;
  float* taps;
  float* dtaps;
  float* rtaps;  // reversed taps, plus a trailing zero when rpad (even m: the adjoint)
  int rpad;
};

__global__ void __launch_bounds__(kMaxGaussTaps) gauss_taps_kernel(const double* __restrict__ sigma,
                                                                   TapsArgs a) {
  __shared__ double s_e[kMaxGaussTaps], s_de[kMaxGaussTaps], s_sum[2];
  const int i = threadIdx.x;
  const double sg = *sigma;
  double e = 0.0, de = 0.0;
  if (i < a.m) {
    const double x = a.x[i];
    e = exp(-(x * x) / (2.0 * sg * sg));
    de = e * x * x / (sg * sg * sg);
  }
  s_e[i] = e;
  s_de[i] = de;
  __syncthreads();
  if (i == 0) {  // sums in index order
    double se = 0.0, sde = 0.0;
    for (int j = 0; j < a.m; ++j) {
      se += s_e[j];
      sde += s_de[j];
    }
    s_sum[0] = se;
    s_sum[1] = sde;
  }
  __syncthreads();
  const double S = s_sum[0], Sde = s_sum[1];
  if (i < a.m) {
    const double t = e / S;
    a.taps[i] = (float)t;
    if (a.dtaps) a.dtaps[i] = (float)((de - t * Sde) / S);
    if (a.rtaps) a.rtaps[a.m - 1 - i] = (float)t;
  }
  if (i == 0 && a.rtaps && a.rpad) a.rtaps[a.m] = 0.f;
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_gauss_taps(const double* sigma, const double* x, int32_t m, float* taps,
                                float* dtaps, float* rtaps, int32_t rtaps_pad, void* stream) {
  RUBIX_REQUIRE(m >= 1 && m < kMaxGaussTaps, RUBIX_E_SHAPE,
                "rubix_gauss_taps: m must be in [1, %d]", kMaxGaussTaps - 1);
  RUBIX_REQUIRE(sigma && x && taps, RUBIX_E_INVALID, "rubix_gauss_taps: null pointer");
  TapsArgs a;
  for (int i = 0; i < kMaxGaussTaps; ++i) a.x[i] = i < m ? x[i] : 0.0;
  a.m = m;
  a.taps = taps;
  a.dtaps = dtaps;
  a.rtaps = rtaps;
  a.rpad = rtaps_pad;
  gauss_taps_kernel<<<1, kMaxGaussTaps, 0, static_cast<cudaStream_t>(stream)>>>(sigma, a);
  RUBIX_LAUNCH_CHECK("gauss_taps_kernel");
  return RUBIX_OK;
}
