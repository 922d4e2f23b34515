// FITS layout of a datacube: rubix writes datacube.T as a FITS image
// (rubix/core/fits.py:88), i.e. for a cube [A][B][L] (spaxel row, spaxel column,
// wavelength) the array [L][B][A] in big-endian IEEE float32 (FITS BITPIX = -32).  One
// tiled transpose: a block reads a 32 (a) x 32 (l) tile of one spaxel column b, rows of
// 32 consecutive wavelengths (128-byte reads), and writes it back as 32 wavelength
// planes of 32 consecutive a (128-byte writes), byte-swapping on the way out.
#include "common.cuh"

namespace rubix {
namespace {

constexpr int kTile = 32;

__global__ void __launch_bounds__(256) fits_layout_kernel(const float* __restrict__ cube,
                                                          long long spaxel_stride, int A, int B,
                                                          int L, unsigned* __restrict__ out) {
  __shared__ float tile[kTile][kTile + 1];
  const int l0 = blockIdx.x * kTile;
  const int a0 = blockIdx.y * kTile;
  const int b = blockIdx.z;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int i = ty; i < kTile; i += 8) {
    const int a = a0 + i, l = l0 + tx;
    tile[i][tx] = (a < A && l < L) ? cube[((long long)a * B + b) * spaxel_stride + l] : 0.f;
  }
  __syncthreads();
  for (int i = ty; i < kTile; i += 8) {
    const int l = l0 + i, a = a0 + tx;
    if (l < L && a < A) {
      const unsigned u = __float_as_uint(tile[tx][i]);
      out[((long long)l * B + b) * A + a] = __byte_perm(u, 0, 0x0123);
    }
  }
}

}  // namespace
}  // namespace rubix

using namespace rubix;

extern "C" int rubix_fits_cube_layout(const float* cube, int32_t A, int32_t B, int32_t L,
                                      int64_t spaxel_stride, void* out, void* stream) {
  RUBIX_REQUIRE(A >= 0 && B >= 0 && L >= 0, RUBIX_E_SHAPE, "rubix_fits_cube_layout: bad shape");
  RUBIX_REQUIRE(spaxel_stride >= L, RUBIX_E_SHAPE,
                "rubix_fits_cube_layout: spaxel_stride < L");
  RUBIX_REQUIRE(B <= 65535, RUBIX_E_SHAPE, "rubix_fits_cube_layout: at most 65535 columns");
  if ((long long)A * B * L == 0) return RUBIX_OK;
  RUBIX_REQUIRE(cube && out, RUBIX_E_INVALID, "rubix_fits_cube_layout: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const dim3 grid((unsigned)div_up(L, kTile), (unsigned)div_up(A, kTile), (unsigned)B);
  fits_layout_kernel<<<grid, 256, 0, st>>>(cube, spaxel_stride, A, B, L,
                                           static_cast<unsigned*>(out));
  RUBIX_LAUNCH_CHECK("fits_layout_kernel");
  return RUBIX_OK;
}
