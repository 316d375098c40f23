// Device-wide primitives: exclusive scans and a stable byte-digit counting
// sort (the building block of the radix sorts that order the SCY-tree and
// the neighbourhood trie).  Plain CUDA, warp shuffles / match for the
// intra-block steps.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "inscy_common.cuh"

namespace inscy {

// ---------------------------------------------------------------------------
// Block-wide inclusive scan of one value per thread (blockDim.x <= 1024).
// `sh` needs 32 entries.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T block_inclusive_scan(T v, T* sh, T* total) {
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= (unsigned)o) v += u;
  }
  if (lane == 31) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    T w = (lane < nw) ? sh[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= (unsigned)o) w += u;
    }
    if (lane < nw) sh[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v += sh[warp - 1];
  if (total) *total = sh[nw - 1];
  __syncthreads();
  return v;
}

// ---------------------------------------------------------------------------
// Device-wide exclusive scan, three phases (tile sums, scan of sums, tiles).
// ---------------------------------------------------------------------------
constexpr int kScanTile = 2048;  // 256 threads x 8 items

template <class Tin, class Tout>
__global__ void k_scan_tile_sums(const Tin* __restrict__ in, long long n, Tout* __restrict__ sums) {
  __shared__ Tout sh[32];
  long long base = (long long)blockIdx.x * kScanTile;
  Tout s = 0;
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x) {
    long long j = base + i;
    if (j < n) s += (Tout)in[j];
  }
  Tout tot;
  block_inclusive_scan<Tout>(s, sh, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <class T>
__global__ void k_scan_single(T* __restrict__ a, long long n, T* __restrict__ total) {
  // exclusive scan of a[0..n) in place by one block (n up to a few million)
  __shared__ T sh[32];
  __shared__ T carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long long base = 0; base < n; base += blockDim.x) {
    long long j = base + threadIdx.x;
    T v = (j < n) ? a[j] : T(0);
    T tot;
    T inc = block_inclusive_scan<T>(v, sh, &tot);
    if (j < n) a[j] = carry + inc - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

template <class Tin, class Tout>
__global__ void k_scan_tiles(const Tin* __restrict__ in, Tout* __restrict__ out, long long n,
                             const Tout* __restrict__ sums) {
  __shared__ Tout sh[32];
  __shared__ Tout carry;
  const int per = kScanTile / 256;
  long long base = (long long)blockIdx.x * kScanTile;
  if (threadIdx.x == 0) carry = sums[blockIdx.x];
  __syncthreads();
  // each thread scans `per` consecutive items
  Tout loc[kScanTile / 256];
  Tout s = 0;
  for (int i = 0; i < per; ++i) {
    long long j = base + (long long)threadIdx.x * per + i;
    Tout v = (j < n) ? (Tout)in[j] : Tout(0);
    loc[i] = s;
    s += v;
  }
  Tout tot;
  Tout inc = block_inclusive_scan<Tout>(s, sh, &tot);
  Tout pre = carry + inc - s;
  for (int i = 0; i < per; ++i) {
    long long j = base + (long long)threadIdx.x * per + i;
    if (j < n) out[j] = pre + loc[i];
  }
}

// ---------------------------------------------------------------------------
// Stable counting sort of int values by an 8-bit digit, device-wide.
//   hist:  256 * nblocks counters (digit-major), scanned in place.
// Digit functors return 0..255.
// ---------------------------------------------------------------------------
constexpr int kSortTile = 512;  // one element per thread

template <class DigitFn>
__global__ void k_digit_hist(const int* __restrict__ in, int m, DigitFn fn, int* __restrict__ hist, int nblocks) {
  __shared__ int cnt[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  int j = blockIdx.x * kSortTile + threadIdx.x;
  if (j < m) atomicAdd(&cnt[fn(in[j])], 1);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i * nblocks + blockIdx.x] = cnt[i];
}

template <class DigitFn>
__global__ void k_digit_scatter(const int* __restrict__ in, int* __restrict__ out, int m, DigitFn fn,
                                const int* __restrict__ offs, int nblocks) {
  __shared__ int wc[kSortTile / 32][256];
  const int nw = kSortTile / 32;
  for (int i = threadIdx.x; i < nw * 256; i += blockDim.x) (&wc[0][0])[i] = 0;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  int j = blockIdx.x * kSortTile + threadIdx.x;
  bool valid = j < m;
  int v = valid ? in[j] : 0;
  int dg = valid ? fn(v) : 256 + (int)lane;  // invalid lanes never match valid ones
  unsigned peers = __match_any_sync(0xffffffffu, dg);
  int rank = __popc(peers & lanemask_lt());
  if (valid && rank == 0) wc[warp][dg] = __popc(peers);
  __syncthreads();
  for (int dgt = threadIdx.x; dgt < 256; dgt += blockDim.x) {
    int run = 0;
    for (int w = 0; w < nw; ++w) {
      int t = wc[w][dgt];
      wc[w][dgt] = run;
      run += t;
    }
  }
  __syncthreads();
  if (valid) out[offs[dg * nblocks + blockIdx.x] + wc[warp][dg] + rank] = v;
}

}  // namespace inscy
