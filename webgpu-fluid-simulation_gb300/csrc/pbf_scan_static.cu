// pbf_scan_static.cu — an exclusive scan that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a
// prefix sum: a host framework that owns every device byte through its own
// pool and forbids other allocators, or a real-time frame loop that must not
// enter the CUDA allocator.  pbf_exclusive_scan_u32_noalloc serves them: the
// caller passes the input and output arrays and the scan's look-back scratch
// lives in the fixed file-scope device array below, which every GPU that
// loads this library holds until the process exits.
//
// The call is synchronous: after the scan it copies the device error word
// back to the host and synchronises the caller's stream, so it cannot be
// recorded into a CUDA graph.  The array's device address is looked up once
// per device (first call, that device current) and cached for the life of
// the process; do not keep using the library on a device after
// cudaDeviceReset there.
//
// The array is shared by all calls on a device and keeps the last call's
// contents; each call clears the parts that must start at zero (tile
// counter, tile status words, error word) on the caller's stream before the
// scan runs.  Two calls whose work overlaps on the GPU (different streams,
// no ordering between them) race on the array and produce wrong results.
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/pbf_gb300.h"
#include "pbf_kernels.h"

namespace {

// Tile counter and status words for PBF_SCAN_NOALLOC_MAX elements, then the
// error word: about 256 KB in all.
constexpr size_t kStatusBytes =
    256 + ((size_t)PBF_SCAN_NOALLOC_MAX / pbf::kScanTileElements + 1) * sizeof(unsigned long long);
constexpr size_t kErrOffset = (kStatusBytes + 255) / 256 * 256;
constexpr size_t kStaticBytes = kErrOffset + 256;

static __device__ __align__(256) unsigned char g_scan_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};  // device address of g_scan_scratch per device ordinal

// Host code only sees a stand-in for g_scan_scratch; its device address is
// looked up once per device with that device current.
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PBF_ECUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scan_scratch) != cudaSuccess || !p) return PBF_ECUDA;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return PBF_OK;
}

}  // namespace

extern "C" int pbf_exclusive_scan_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, size_t n, void* stream) {
  if ((!d_in || !d_out) && n) return PBF_EINVAL;
  if (n > (size_t)PBF_SCAN_NOALLOC_MAX) return PBF_ECAPACITY;
  if (n == 0) return PBF_OK;
  if (pbf::scan_scratch_bytes(n) > kErrOffset) return PBF_ECAPACITY;
  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t* err = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(base) + kErrOffset);
  if (cudaMemsetAsync(err, 0, sizeof(uint32_t), st) != cudaSuccess) return PBF_ECUDA;
  // launch_exclusive_scan clears the counter and status words it uses
  if (pbf::launch_exclusive_scan(d_in, d_out, n, base, err, st) != cudaSuccess) return PBF_ECUDA;
  uint32_t e = 0;
  if (cudaMemcpyAsync(&e, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess) return PBF_ECUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return PBF_ECUDA;
  return e ? PBF_ETIMEOUT : PBF_OK;
}
