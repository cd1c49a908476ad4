// sort_gaussian for callers that cannot allocate device memory.
//
// Who needs this: code that runs inside a host application owning the GPU
// memory budget (a game engine, a viewer plug-in, a real-time loop with a
// fixed memory plan) or that must not enter the CUDA allocator on its hot
// path (cudaMalloc synchronises the device and can fail under memory
// pressure).  Such callers can still pass their inputs and outputs, but not
// the scratch that pgb_sort_gaussian_begin/finish take.  Here the scratch is
// a fixed static device array, created when the library is loaded, on every
// GPU that loads it, and held until the process exits.
//
// The entry point reuses pgb_sort_gaussian_begin/finish unchanged, giving
// them slices of that array.  It is synchronous (it reads the entry count K
// back before the second phase and checks the device status at the end) and
// it calls no allocating CUDA or library routine.
#include <mutex>

#include "pgb_common.cuh"

namespace {

constexpr int64_t kMaxGaussians = PGB_NOALLOC_MAX_GAUSSIANS;
constexpr size_t kScratchBytes = PGB_NOALLOC_SCRATCH_BYTES;
constexpr size_t kInfoBytes = 256;  // two int64 info words, padded to 256 bytes

// The shared scratch.  In host code `g_noalloc_scratch` names a host-side
// stand-in, not device memory: kernels only ever get the address that
// cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 128;
std::mutex g_mutex;
void* g_device_address[kMaxDevices] = {};

// Device address of the static scratch on the current device; looked up once
// per device (the first call on a device does this set-up).
int scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return PGB_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return PGB_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (g_device_address[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr)
      return PGB_ERR_CUDA;
    g_device_address[dev] = p;
  }
  *out = g_device_address[dev];
  return PGB_OK;
}

size_t round256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

}  // namespace

extern "C" int pgb_sort_gaussian_noalloc(const float* uv, const float* depth,
                                         const int32_t* radius, const int32_t* tiles_touched,
                                         int64_t n, int width, int height, int32_t* ids_out,
                                         int64_t ids_capacity, int32_t* tile_range_out,
                                         int64_t* k_out, void* stream) {
  if (k_out) *k_out = -1;
  if (n < 0 || width <= 0 || height <= 0 || ids_capacity < 0 || !tile_range_out)
    return PGB_ERR_INVALID;
  if (n > kMaxGaussians) return PGB_ERR_INVALID;  // beyond the fixed capacity
  if (n > 0 && (!uv || !depth || !radius || !tiles_touched)) return PGB_ERR_INVALID;
  if (ids_capacity > 0 && !ids_out) return PGB_ERR_INVALID;
  if (pgb::misaligned(uv, 8) || pgb::misaligned(tile_range_out, 8)) return PGB_ERR_INVALID;
  size_t bytes_n = 0, bytes_k = 0;
  int st = pgb_sort_scratch_bytes(n, 0, width, height, &bytes_n, nullptr);
  if (st != PGB_OK) return st;
  if (kInfoBytes + round256(bytes_n) > kScratchBytes) return PGB_ERR_INVALID;

  void* base = nullptr;
  st = scratch_address(&base);
  if (st != PGB_OK) return st;
  char* p = static_cast<char*>(base);
  int64_t* info = reinterpret_cast<int64_t*>(p);
  void* scratch_n = p + kInfoBytes;
  void* scratch_k = p + kInfoBytes + round256(bytes_n);
  cudaStream_t s = pgb::as_stream(stream);

  // phase 1 clears the info words and every counter, histogram and status
  // word it uses, then sorts by depth and sums K on the device
  st = pgb_sort_gaussian_begin(depth, radius, tiles_touched, n, width, height, scratch_n, bytes_n,
                               info, stream);
  if (st != PGB_OK) return st;
  int64_t host_info[2] = {0, 0};
  if (cudaMemcpyAsync(host_info, info, sizeof(host_info), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PGB_ERR_CUDA;
  if (host_info[1] != 0) return static_cast<int>(host_info[1]);
  const int64_t k = host_info[0];
  if (k_out) *k_out = k;
  st = pgb_sort_scratch_bytes(n, k, width, height, nullptr, &bytes_k);
  if (st != PGB_OK) return st;
  // K beyond what the static array or the caller's output can hold
  if (kInfoBytes + round256(bytes_n) + bytes_k > kScratchBytes || k > ids_capacity)
    return PGB_ERR_OVERFLOW;
  if (k > 0 && !ids_out) return PGB_ERR_INVALID;

  // phase 2 clears its pass status words and tile_range_out before use
  st = pgb_sort_gaussian_finish(uv, radius, tiles_touched, n, width, height, k, scratch_n, bytes_n,
                                scratch_k, bytes_k, info, ids_out, tile_range_out, stream);
  if (st != PGB_OK) return st;
  if (cudaMemcpyAsync(host_info, info, sizeof(host_info), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PGB_ERR_CUDA;
  return static_cast<int>(host_info[1]);
}
