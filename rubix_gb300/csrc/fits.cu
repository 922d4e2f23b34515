// FITS layout of a datacube: rubix writes datacube.T as a FITS image
// (rubix/core/fits.py:88), i.e. for a cube [A][B][L] (spaxel row, spaxel column,
// wavelength) the array [L][B][A] in big-endian IEEE float32 (FITS BITPIX = -32).  One
// tiled transpose: a block reads a 64 (a) x 64 (l) tile of one spaxel column b, rows of
// 64 consecutive wavelengths (256-byte reads), and writes it back as 64 wavelength
// planes of 64 consecutive a (256-byte writes), byte-swapping on the way out.  The rows
// and planes a block touches lie megabytes apart; 64 x 64 tiles move twice the bytes
// per page touched of 32 x 32 ones (0.46 against 0.58 ms for a 300 x 300 x 3721 cube).
#include "common.cuh"

namespace rubix {
namespace {

constexpr int kTileA = 64;  // spaxel rows a per tile
constexpr int kTileL = 64;  // wavelengths per tile

__global__ void __launch_bounds__(256) fits_layout_kernel(const float* __restrict__ cube,
                                                          long long spaxel_stride, int A, int B,
                                                          int L, unsigned* __restrict__ out) {
  __shared__ float tile[kTileA][kTileL + 1];  // odd row pitch: conflict-free columns
  const int l0 = blockIdx.x * kTileL;
  const int a0 = blockIdx.y * kTileA;
  const int b = blockIdx.z;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
#pragma unroll
  for (int i = ty; i < kTileA; i += 8) {
    const int a = a0 + i;
#pragma unroll
    for (int c = tx; c < kTileL; c += 32) {
      const int l = l0 + c;
      tile[i][c] = (a < A && l < L) ? cube[((long long)a * B + b) * spaxel_stride + l] : 0.f;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = ty; i < kTileL; i += 8) {
    const int l = l0 + i;
#pragma unroll
    for (int c = tx; c < kTileA; c += 32) {
      const int a = a0 + c;
      if (l < L && a < A) {
        const unsigned u = __float_as_uint(tile[c][i]);
        out[((long long)l * B + b) * A + a] = __byte_perm(u, 0, 0x0123);
      }
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
  const dim3 grid((unsigned)div_up(L, kTileL), (unsigned)div_up(A, kTileA), (unsigned)B);
  fits_layout_kernel<<<grid, 256, 0, st>>>(cube, spaxel_stride, A, B, L,
                                           static_cast<unsigned*>(out));
  RUBIX_LAUNCH_CHECK("fits_layout_kernel");
  return RUBIX_OK;
}
