// Fixed device scratch for vg_nav_compute_step_and_next_volume_noalloc: the work-queue
// counter, the relocation points of the split step, the per-track proposal slots, and the
// sort keys, track order and radix counts of a scheduled navigation step, held in one
// file-scope device array instead of a caller-supplied or allocated workspace.
//
// Capacity: kNoAllocMaxTracks tracks per call (41.5 MiB of scratch per device). The array
// exists once per device, so calls that overlap in time (on different streams or host
// threads) share it and race; callers serialise them. The first call on a device looks up
// the array's address (cudaGetSymbolAddress, which may load this module), so it belongs
// in setup, before any stream capture. Nothing in the scratch has to start at zero: the
// work-queue counter is cleared on the stream before every step launch and the sort
// buffers are written before they are read.
#include "launch.h"
#include <mutex>

namespace vg {
namespace {

constexpr size_t kNoAllocMaxTracks = size_t(1) << 20;
// The layout of a step workspace with every scheduling flag at kNoAllocMaxTracks tracks:
// 256-byte counter block, three relocation coordinates (doubles) per track, one proposal
// slot byte per track (256-aligned), four track arrays of 4 bytes per track (keys and
// values, twice), 512 digit counts per 4096-track tile and 512 digit totals. noalloc_check_capacity() compares this with the workspace
// size the step launch asks for, so the two cannot drift apart unnoticed.
constexpr size_t kNoAllocTiles        = (kNoAllocMaxTracks + 4095) / 4096;
constexpr size_t kNoAllocScratchBytes = 256 + 3 * 8 * kNoAllocMaxTracks + kNoAllocMaxTracks +
                                        4 * (kNoAllocMaxTracks * 4) + 512 * kNoAllocTiles * 4 + 512 * 4;
static_assert(kNoAllocMaxTracks % 256 == 0 && (512 * kNoAllocTiles * 4) % 256 == 0,
              "no-allocation scratch segments must stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

} // namespace

size_t noalloc_max_tracks() { return kNoAllocMaxTracks; }

// Address of the current device's scratch (looked up once per device) and its size.
cudaError_t noalloc_scratch(void **ptr, size_t *bytes)
{
  *ptr   = nullptr;
  *bytes = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e       = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *ptr   = g_scratch_ptr[dev];
  *bytes = kNoAllocScratchBytes;
  return cudaSuccess;
}

} // namespace vg
