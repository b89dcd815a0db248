// pa_sort_u32_noalloc: the 32-bit key sort for callers that must not
// allocate GPU memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or harmful --
// inside a framework whose caching allocator owns all device memory and
// forbids allocations behind its back, latency-critical loops in which the
// implicit device-wide synchronisation of cudaMalloc/cudaFree would stall
// other streams, or callers that have already reserved every byte they may
// use.  pa_sort_u32 keeps a grow-only per-stream workspace that it
// (re)allocates on demand; this entry point instead works in a fixed scratch
// area compiled into the library, so it never allocates.
//
// The scratch is one file-scope __device__ array (kScratchBytes, about
// 4 MiB): digit counts, bin starts, the pass-control block, tile tickets, an
// error word and the look-back status words.  Every GPU that loads the
// library holds it until the process exits.  It bounds the size: at most
// kMaxKeys keys per call.  Every call reuses the same array and finds the
// previous call's contents there; the call clears what must start at zero.
// Two calls whose work overlaps on the GPU (different streams or host
// threads) would race on the array: issue them one after the other.
//
// Host code cannot use the array's name as a device address, so the first
// call on each device that needs the scratch looks the address up with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture.  Up to 8192 keys the call sorts in
// one CTA's shared memory, as pa_sort_u32 does, and touches no scratch.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "pa_common.cuh"
#include "pa_gpu.h"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr size_t kMaxKeys = (size_t)1 << 22;      // 4,194,304 keys
constexpr int kPasses = 4;                          // 32-bit keys, 8-bit digits
constexpr size_t kMinTileKeys = 4096;               // smallest onesweep tile geometry
constexpr size_t kMaxTiles = kMaxKeys / kMinTileKeys;
constexpr size_t kStatusBytes = (size_t)kPasses * kMaxTiles * 256 * 4;  // 32-bit status words

// Layout of the scratch (offsets in bytes, each 256-aligned).
constexpr size_t kCountsOff = 0;                                   // [4][256] u64, zeroed
constexpr size_t kTicketsOff = kCountsOff + kPasses * 256 * 8;     // [4] u32, zeroed
constexpr size_t kErrOff = kTicketsOff + 256;                      // u32, zeroed
constexpr size_t kStatusOff = kErrOff + 256;                       // status words, zeroed
constexpr size_t kBinStartOff = kStatusOff + kStatusBytes;         // [4][256] u64
constexpr size_t kCtrlOff = kBinStartOff + kPasses * 256 * 8;      // SortCtrl
constexpr size_t kScratchBytes = kCtrlOff + ((sizeof(SortCtrl) + 255) / 256) * 256;

static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[64] = {};

// Device address of the scratch for the current device (looked up once).
int scratch_for_current_device(unsigned char** out, char* why, size_t why_len) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    snprintf(why, why_len, "cudaGetDevice: %s", cudaGetErrorString(e));
    return PA_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || p == nullptr) {
      snprintf(why, why_len, "cudaGetSymbolAddress of the sort scratch: %s", cudaGetErrorString(e));
      return PA_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return PA_OK;
}

bool on_current_device(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

int fail(int status, const char* what) { return record_error(status, what); }

}  // namespace
}  // namespace pa

using namespace pa;

extern "C" int pa_sort_u32_noalloc(uint32_t* keys, uint32_t* tmp, size_t n, const pa_opts* opts) {
  if (n == 0) return PA_OK;
  if (!keys || !tmp) return fail(PA_ERR_ARG, "pa_sort_u32_noalloc: keys and tmp are required");
  if (n > kMaxKeys) return fail(PA_ERR_ARG, "pa_sort_u32_noalloc: n exceeds the 4,194,304-key limit of its fixed scratch");
  if (opts && (opts->digit_bits != 0 && opts->digit_bits != 8))
    return fail(PA_ERR_ARG, "pa_sort_u32_noalloc: digit_bits must be 0 or 8");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(PA_ERR_NO_DEVICE, "pa_sort_u32_noalloc: no CUDA device");
  }
  if (!on_current_device(keys) || !on_current_device(tmp))
    return fail(PA_ERR_ARG,
                "pa_sort_u32_noalloc: keys and tmp must be device memory of the current device (host buffers "
                "would need staging memory; use pa_sort_u32)");
  cudaStream_t stream = opts ? static_cast<cudaStream_t>(opts->stream) : (cudaStream_t)0;
  char why[200];
  if (n <= small_sort_max_keys(4, false)) {
    // Up to 8192 keys pa_sort_u32 sorts in one CTA's shared memory; that
    // kernel needs no global scratch, so this call runs it as is.
    cudaError_t e = launch_small_sort(keys, nullptr, n, 4, false, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
      snprintf(why, sizeof(why), "pa_sort_u32_noalloc: %s", cudaGetErrorString(e));
      return fail(PA_ERR_CUDA, why);
    }
    return PA_OK;
  }
  const size_t tile = onesweep_tile_keys(4, false);
  const size_t tiles = (n + tile - 1) / tile;
  if ((size_t)kPasses * tiles * 256 * 4 > kStatusBytes)
    return fail(PA_ERR_ARG, "pa_sort_u32_noalloc: the selected tile geometry needs more look-back words than the scratch holds");

  unsigned char* base = nullptr;
  if (int rc = scratch_for_current_device(&base, why, sizeof(why))) return fail(rc, why);
  auto* counts = reinterpret_cast<unsigned long long*>(base + kCountsOff);
  auto* tickets = reinterpret_cast<uint32_t*>(base + kTicketsOff);
  auto* err = reinterpret_cast<uint32_t*>(base + kErrOff);
  unsigned char* status = base + kStatusOff;
  auto* bin_start = reinterpret_cast<unsigned long long*>(base + kBinStartOff);
  auto* ctrl = reinterpret_cast<SortCtrl*>(base + kCtrlOff);

  // The previous call's counts, tickets, error word and status words are
  // still in the scratch: clear the part this call uses.
  const size_t zero_bytes = kStatusOff + (size_t)kPasses * tiles * 256 * 4;
  cudaError_t e = cudaMemsetAsync(base, 0, zero_bytes, stream);
  if (e == cudaSuccess) e = launch_digit_counts(keys, n, 4, kPasses, 8, 0, 8, false, counts, stream);
  if (e == cudaSuccess) e = launch_scan_digits(counts, kPasses, 8, n, false, true, bin_start, ctrl, stream);
  for (int p = 0; p < kPasses && e == cudaSuccess; ++p) {
    OnesweepArgs a{};
    a.keys_a = keys;
    a.keys_b = tmp;
    a.n = n;
    a.shift = 8u * (uint32_t)p;
    a.pass = p;
    a.bin_start = bin_start + (size_t)p * 256;
    a.status = status + (size_t)p * tiles * 256 * 4;
    a.tile_counter = tickets + p;
    a.ctrl = ctrl;
    a.err = err;
    e = launch_onesweep_pass(a, 4, false, stream);
  }
  if (e == cudaSuccess) e = launch_final_copy(keys, tmp, nullptr, nullptr, n, 4, ctrl, stream);
  uint32_t err_host = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err_host, err, sizeof(err_host), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) {
    snprintf(why, sizeof(why), "pa_sort_u32_noalloc: %s", cudaGetErrorString(e));
    return fail(e == cudaErrorMemoryAllocation ? PA_ERR_OOM : PA_ERR_CUDA, why);
  }
  if (err_host) return fail(PA_ERR_TIMEOUT, "pa_sort_u32_noalloc: a bounded device-side wait gave up");
  return PA_OK;
}
