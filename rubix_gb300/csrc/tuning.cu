// Per-device tuning of the cube kernels' work items, set by an autotuner (or by hand)
// through rubix_cube_tuning_set.  The only mutable state of the library besides the
// error buffer; guarded by a mutex.
#include <mutex>

#include "cube_common.cuh"

namespace rubix {
namespace {

constexpr int kMaxDevices = 64;
std::mutex g_tuning_mutex;
CubeTuning g_tuning[kMaxDevices];
bool g_tuning_set[kMaxDevices] = {};

constexpr CubeTuning kDefaultTuning{256, 64};

}  // namespace

CubeTuning cube_tuning_current() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return kDefaultTuning;
  std::lock_guard<std::mutex> lock(g_tuning_mutex);
  return g_tuning_set[dev] ? g_tuning[dev] : kDefaultTuning;
}

}  // namespace rubix

using namespace rubix;

extern "C" int rubix_cube_tuning_set(int32_t device, const rubix_cube_tuning* t) {
  RUBIX_REQUIRE(device >= 0 && device < kMaxDevices, RUBIX_E_INVALID,
                "rubix_cube_tuning_set: device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_tuning_mutex);
  if (t == nullptr) {  // back to the defaults
    g_tuning_set[device] = false;
    return RUBIX_OK;
  }
  RUBIX_REQUIRE(t->chunk >= kMinChunk && t->chunk <= kMaxChunk && t->chunk % 32 == 0,
                RUBIX_E_INVALID, "rubix_cube_tuning_set: chunk must be a multiple of 32 in "
                "[%d, %d], got %d", kMinChunk, kMaxChunk, t->chunk);
  RUBIX_REQUIRE(t->big_item >= 1, RUBIX_E_INVALID, "rubix_cube_tuning_set: big_item < 1");
  g_tuning[device] = CubeTuning{t->chunk, t->big_item};
  g_tuning_set[device] = true;
  return RUBIX_OK;
}

extern "C" int rubix_cube_tuning_get(int32_t device, rubix_cube_tuning* t) {
  RUBIX_REQUIRE(device >= 0 && device < kMaxDevices && t != nullptr, RUBIX_E_INVALID,
                "rubix_cube_tuning_get: bad arguments");
  std::lock_guard<std::mutex> lock(g_tuning_mutex);
  const CubeTuning c = g_tuning_set[device] ? g_tuning[device] : kDefaultTuning;
  t->chunk = c.chunk;
  t->big_item = c.big_item;
  return RUBIX_OK;
}
