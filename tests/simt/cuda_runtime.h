// CPU execution of the engine's CUDA sources (a test harness, not a product
// path): the subset of the CUDA runtime and device intrinsics the engine
// uses.  Threads of a block are fibers that switch only at __syncthreads and
// warp collectives (simt.cpp); device memory is host memory with guard pages.
#pragma once
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __restrict__ __restrict
#define __shared__ static thread_local
#define __align__(n) alignas(n)

struct uint3 {
  unsigned x, y, z;
};
struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct int2 {
  int x, y;
};
struct alignas(16) float4 {
  float x, y, z, w;
};
struct alignas(16) uint4 {
  unsigned x, y, z, w;
};
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline int2 make_int2(int a, int b) { return int2{a, b}; }
using std::max;
using std::min;

namespace simt {
extern thread_local uint3 g_tid, g_bid;
extern dim3 g_bdim, g_gdim;
enum Op { OP_SHFL = 1, OP_SHFL_UP, OP_SHFL_XOR, OP_BALLOT, OP_ANY, OP_MATCH_ANY };
unsigned long long collective(int op, unsigned mask, unsigned long long v, int arg);
void syncthreads();
typedef void (*CallFn)(void*);
void launch_impl(const char* name, dim3 grid, dim3 block, CallFn fn, void* obj);
template <class F>
void launch(const char* name, dim3 grid, dim3 block, F f) {
  launch_impl(name, grid, block, [](void* p) { (*(F*)p)(); }, (void*)&f);
}
template <class T>
unsigned long long to_bits(T v) {
  unsigned long long b = 0;
  std::memcpy(&b, &v, sizeof(T));
  return b;
}
template <class T>
T from_bits(unsigned long long b) {
  T v;
  std::memcpy(&v, &b, sizeof(T));
  return v;
}
}  // namespace simt

#define threadIdx (::simt::g_tid)
#define blockIdx (::simt::g_bid)
#define blockDim (::simt::g_bdim)
#define gridDim (::simt::g_gdim)

inline void __syncthreads() { ::simt::syncthreads(); }
template <class T>
inline T __shfl_sync(unsigned m, T v, int src) {
  return simt::from_bits<T>(simt::collective(simt::OP_SHFL, m, simt::to_bits(v), src));
}
template <class T>
inline T __shfl_up_sync(unsigned m, T v, unsigned o) {
  return simt::from_bits<T>(simt::collective(simt::OP_SHFL_UP, m, simt::to_bits(v), (int)o));
}
template <class T>
inline T __shfl_xor_sync(unsigned m, T v, int o) {
  return simt::from_bits<T>(simt::collective(simt::OP_SHFL_XOR, m, simt::to_bits(v), o));
}
inline unsigned __ballot_sync(unsigned m, int p) { return (unsigned)simt::collective(simt::OP_BALLOT, m, p ? 1 : 0, 0); }
inline int __any_sync(unsigned m, int p) { return (int)simt::collective(simt::OP_ANY, m, p ? 1 : 0, 0); }
inline void __syncwarp(unsigned m = 0xffffffffu) { (void)simt::collective(simt::OP_ANY, m, 0, 0); }
template <class T>
inline unsigned __match_any_sync(unsigned m, T v) {
  return (unsigned)simt::collective(simt::OP_MATCH_ANY, m, simt::to_bits(v), (int)sizeof(T));
}

inline int __popc(unsigned v) { return __builtin_popcount(v); }
inline int __popcll(unsigned long long v) { return __builtin_popcountll(v); }
inline int __ffsll(long long v) { return __builtin_ffsll(v); }
inline int __ffs(int v) { return __builtin_ffs(v); }
inline int __clzll(long long v) { return v == 0 ? 64 : __builtin_clzll((unsigned long long)v); }
inline int __clz(int v) { return v == 0 ? 32 : __builtin_clz((unsigned)v); }
// IEEE single/double operations, each rounded once (build with -ffp-contract=off)
inline float __fdiv_rn(float a, float b) { return a / b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fsqrt_rn(float a) { return std::sqrt(a); }
inline double __dsub_rn(double a, double b) { return a - b; }
inline double __dadd_rn(double a, double b) { return a + b; }
inline float __double2float_rn(double a) { return (float)a; }
inline float __uint_as_float(unsigned u) { return simt::from_bits<float>(u); }
inline unsigned __float_as_uint(float f) { return (unsigned)simt::to_bits(f); }
inline float __int_as_float(int i) { return simt::from_bits<float>((unsigned)i); }
inline int __float_as_int(float f) { return (int)(unsigned)simt::to_bits(f); }

// blocks run on several host threads: real atomics
template <class T>
inline T atomicAdd(T* p, T v) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
template <class T>
inline T atomicExch(T* p, T v) {
  return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST);
}
template <class T>
inline T atomicCAS(T* p, T c, T v) {
  __atomic_compare_exchange_n(p, &c, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return c;
}
template <class T>
inline T atomicMin(T* p, T v) {
  T o = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (v < o && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return o;
}
template <class T>
inline T atomicOr(T* p, T v) {
  return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST);
}

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
typedef struct simt_stream* cudaStream_t;
typedef struct simt_event* cudaEvent_t;
typedef struct simt_pool* cudaMemPool_t;
enum cudaMemcpyKind {
  cudaMemcpyHostToHost,
  cudaMemcpyHostToDevice,
  cudaMemcpyDeviceToHost,
  cudaMemcpyDeviceToDevice,
  cudaMemcpyDefault
};
enum { cudaMemAllocationTypePinned = 1 };
enum { cudaMemLocationTypeDevice = 1 };
enum cudaMemPoolAttr { cudaMemPoolAttrReleaseThreshold = 1 };
enum cudaDeviceAttr { cudaDevAttrMultiProcessorCount = 16 };
struct cudaMemLocation {
  int type, id;
};
struct cudaMemPoolProps {
  int allocType;
  int handleTypes;
  cudaMemLocation location;
  void* win32SecurityAttributes;
  unsigned char reserved[64];
};
cudaError_t cudaGetDevice(int* d);
cudaError_t cudaDeviceGetAttribute(int* v, cudaDeviceAttr a, int device);
const char* cudaGetErrorString(cudaError_t e);
cudaError_t cudaGetLastError();
cudaError_t cudaMemPoolCreate(cudaMemPool_t* p, const cudaMemPoolProps* props);
cudaError_t cudaMemPoolDestroy(cudaMemPool_t p);
cudaError_t cudaMemPoolSetAttribute(cudaMemPool_t p, cudaMemPoolAttr a, void* v);
cudaError_t cudaMallocFromPoolAsync(void** p, size_t bytes, cudaMemPool_t pool, cudaStream_t s);
cudaError_t cudaFreeAsync(void* p, cudaStream_t s);
cudaError_t cudaMalloc(void** p, size_t bytes);
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t bytes) {
  return cudaMalloc((void**)p, bytes);
}
cudaError_t cudaFree(void* p);
cudaError_t cudaMallocHost(void** p, size_t bytes);
template <class T>
inline cudaError_t cudaMallocHost(T** p, size_t bytes) {
  return cudaMallocHost((void**)p, bytes);
}
cudaError_t cudaFreeHost(void* p);
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind k, cudaStream_t st = 0);
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind k);
cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t st = 0);
cudaError_t cudaMemset(void* d, int v, size_t n);
cudaError_t cudaStreamSynchronize(cudaStream_t s);
enum { cudaStreamNonBlocking = 1 };
cudaError_t cudaSetDevice(int d);
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned flags);
cudaError_t cudaStreamDestroy(cudaStream_t s);
cudaError_t cudaEventCreate(cudaEvent_t* e);
cudaError_t cudaEventDestroy(cudaEvent_t e);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s = 0);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b);
