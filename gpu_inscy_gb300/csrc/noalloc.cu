// inscy_selftest_noalloc: the device self-test without any device allocation.
//
// Who needs it: processes that must not (or cannot) call cudaMalloc when they
// check a GPU -- for example a serving process whose device memory is already
// handed out in full to a caching allocator or a memory-capped job, where a
// new cudaMalloc would fail or fragment the pool, or code on a latency path
// where cudaMalloc's implicit synchronisation is not acceptable.  They can
// still run the self-test: its only scratch, the mismatch counter, lives in
// a file-scope device array that is part of the loaded library.
//
// The array stays allocated on every GPU that loads this library until the
// process exits.  All calls share it: the counter is cleared at the start of
// every call, and calls that overlap on the GPU (several streams or host
// threads at once) race on it and may report each other's mismatches.
//
// The array's device address is looked up once per device and kept.  A
// cudaDeviceReset loads the library's device code into a new context, where
// the kept address is no longer the array's: a process that resets a device
// must not call this entry on that device afterwards.  The kept address is
// dropped whenever a CUDA call of the entry fails, so the next call looks it
// up again.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/inscy_gb300.h"
#include "inscy_kernels.h"

namespace {

// 256 bytes; the self-test uses the first 8 (one 64-bit counter)
__device__ __align__(256) unsigned long long g_noalloc_scratch[32];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices];  // device address of g_noalloc_scratch, per device
std::mutex g_scratch_mu;

// The symbol's host-side name is not a device address: the device address
// is looked up once per device, with that device current.
void* scratch_for(int dev) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
    g_scratch_addr[dev] = p;
  }
  return g_scratch_addr[dev];
}

// A CUDA call of the entry failed: forget the device's address.
int64_t failed(int dev) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  g_scratch_addr[dev] = nullptr;
  return INSCY_SELFTEST_NOALLOC_CUDA;
}

}  // namespace

extern "C" int64_t inscy_selftest_noalloc(int64_t count, void* stream) {
  if (count < 0 || count > INSCY_SELFTEST_NOALLOC_MAX) return INSCY_SELFTEST_NOALLOC_TOO_LARGE;
  // an error left pending by earlier work is the caller's: report it without
  // clearing it, and launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return INSCY_SELFTEST_NOALLOC_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return INSCY_SELFTEST_NOALLOC_CUDA;
  void* scratch = scratch_for(dev);
  if (!scratch) return failed(dev);
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* counter = (unsigned long long*)scratch;
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s) != cudaSuccess) return failed(dev);
  if (count > 0) inscy::launch_phi_selftest((unsigned long long)count, 0x5eedull, counter, s);
  if (cudaGetLastError() != cudaSuccess) return failed(dev);  // the launch's own error
  unsigned long long bad = 0;
  if (cudaMemcpyAsync(&bad, counter, sizeof(bad), cudaMemcpyDeviceToHost, s) != cudaSuccess) return failed(dev);
  if (cudaStreamSynchronize(s) != cudaSuccess) return failed(dev);
  return (int64_t)bad;
}
