// Setup kernels: grid cells, s-connection flags, the neighbourhood-trie
// order and the per-dim candidate lists.
//
// The SCY-tree of the reference is a pointer trie built point by point
// (ScyTreeNode.cu:105-143).  Here it is never materialised: every point's
// coarse cell per dim and its s-connection ("ghost") flags are computed once,
// and the trie orders the reference walks are recovered by radix sorts of
// cell keys (see the engine).
#include <cstdint>
#include <cuda_runtime.h>

#include "inscy_common.cuh"
#include "inscy_prims.cuh"
#include "inscy_kernels.h"

namespace inscy {

// Cells and ghost flags of every (point, dim).
//   coarse: get_cell_no (ScyTreeNode.cu:100-102) with cell_size = 1.f/cells;
//   ghost:  construct_s_connection's test x >= (cell+1)*cell_size - eps
//           (ScyTreeNode.cu:36) -- float arithmetic, no contraction;
//   fine:   the same cell rule on the ceil(1/eps) grid (inscy_map.cpp:243).
__global__ void k_prep(const float* __restrict__ X, int n, int d, int cells, float csz, int G, float fsz, float eps,
                       uint8_t* __restrict__ cc, uint8_t* __restrict__ fc, unsigned long long* __restrict__ gz) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  unsigned long long g = 0;
  for (int k = 0; k < d; ++k) {
    float x = X[(size_t)p * d + k];
    int c = (int)__fdiv_rn(x, csz);
    c = c < cells - 1 ? c : cells - 1;
    c = c > 0 ? c : 0;  // inputs are checked to lie in [0, 1]; the clamps only keep indices in range
    int f = (int)__fdiv_rn(x, fsz);
    f = f < G - 1 ? f : G - 1;
    f = f > 0 ? f : 0;
    cc[(size_t)p * d + k] = (uint8_t)c;
    fc[(size_t)p * d + k] = (uint8_t)f;
    float edge = __fsub_rn(__fmul_rn((float)(c + 1), csz), eps);
    if (x >= edge) g |= 1ull << k;
  }
  gz[p] = g;
}

// Candidate lists of the 1-dim subspace {k}: for each fine cell c, the
// points of cells c-1, c, c+1 in neighbourhood-trie order.  Each point of
// bucket c' lands in the lists of c'-1, c', c'+1 at
//   (its index in bucket c') + (#points with smaller trie rank in the other
//   two buckets of the list),
// i.e. a three-way merge by rank done with binary searches.
__global__ void k_candidate_lists(int n, int d, int G, const int* __restrict__ bucket_pts,
                                  const int* __restrict__ bucket_off, const int* __restrict__ rank,
                                  const uint8_t* __restrict__ fc, const long long* __restrict__ list_off,
                                  int* __restrict__ list_pts) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)n * d;
  if (t >= total) return;
  int k = (int)(t / n);
  int e = (int)(t % n);
  const int* bp = bucket_pts + (size_t)k * n;
  const int* bo = bucket_off + (size_t)k * (G + 1);
  int p = bp[e];
  int cp = fc[(size_t)p * d + k];
  int r = rank[p];
  int own = e - bo[cp];
  for (int c = cp - 1; c <= cp + 1; ++c) {
    if (c < 0 || c >= G) continue;
    int pos = own;
    for (int b = c - 1; b <= c + 1; ++b) {
      if (b < 0 || b >= G || b == cp) continue;
      int lo = bo[b], hi = bo[b + 1];
      while (lo < hi) {  // number of entries with rank < r
        int mid = (lo + hi) >> 1;
        if (rank[bp[mid]] < r)
          lo = mid + 1;
        else
          hi = mid;
      }
      pos += lo - bo[b];
    }
    list_pts[list_off[(size_t)k * G + c] + pos] = p;
  }
}

__global__ void k_check_range(const float* __restrict__ X, long long m, int* __restrict__ bad) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) {
    float x = X[i];
    if (!(x >= 0.f && x <= 1.f)) atomicExch(bad, 1);
  }
}

void launch_check_range(const float* X, long long m, int* bad, cudaStream_t s) {
  if (m > 0) k_check_range<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(X, m, bad);
}

__global__ void k_iota(int* a, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = i;
}

__global__ void k_scatter_rank(const int* __restrict__ order, int n, int* __restrict__ rank) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rank[order[i]] = i;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
__global__ void k_digit_starts(const int* hist, int nb, int m, int* starts) {
  int i = threadIdx.x;
  if (i < 256) starts[i] = hist[i * nb];
  if (i == 0) starts[256] = m;
}

void launch_digit_starts(const int* hist, int nb, int m, int* starts, cudaStream_t s) {
  k_digit_starts<<<1, 256, 0, s>>>(hist, nb, m, starts);
}

struct ByteDigit {  // digit = byte matrix entry [v * d + k]
  const uint8_t* a;
  int d, k;
  __device__ int operator()(int v) const { return a[(size_t)v * d + k]; }
};

void launch_prep(const float* X, int n, int d, int cells, float csz, int G, float fsz, float eps, uint8_t* cc,
                 uint8_t* fc, unsigned long long* gz, cudaStream_t s) {
  if (n <= 0) return;
  k_prep<<<(n + 255) / 256, 256, 0, s>>>(X, n, d, cells, csz, G, fsz, eps, cc, fc, gz);
}

// Point rows of `slots` (16, 24 or 32) >= d: the coordinates of every point,
// zero-padded, and its fine-cell window per dim as a coordinate interval
// [lo, hi) (fine_lo[k] = least x whose fine cell before the cap is >= k):
// q is within +-1 fine cell of p on dim k iff lo_p <= x_q < hi_p.
__global__ void k_point_rows(const float* __restrict__ X, const uint8_t* __restrict__ fc, int n, int d, int slots,
                             int G, const float* __restrict__ fine_lo, float* __restrict__ xrow,
                             float* __restrict__ win) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * slots) return;
  const long long p = t / slots;
  const int k = (int)(t % slots);
  const float ninf = __uint_as_float(0xff800000u), pinf = __uint_as_float(0x7f800000u);
  float x = 0.f, lo = ninf, hi = pinf;
  if (k < d) {
    x = X[p * d + k];
    const int f = fc[p * d + k];
    if (f - 1 >= 1) lo = fine_lo[f - 1];
    if (f + 2 <= G - 1) hi = fine_lo[f + 2];
  }
  xrow[t] = x;
  win[2 * t] = lo;
  win[2 * t + 1] = hi;
}

void launch_point_rows(const float* X, const uint8_t* fc, int n, int d, int slots, int G, const float* fine_lo,
                       float* xrow, float* win, cudaStream_t s) {
  long long m = (long long)n * slots;
  if (m > 0) k_point_rows<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(X, fc, n, d, slots, G, fine_lo, xrow, win);
}

void launch_iota(int* a, int n, cudaStream_t s) {
  if (n > 0) k_iota<<<(n + 255) / 256, 256, 0, s>>>(a, n);
}

// Points per (dim, coarse cell): the counts behind the entropy level order of
// get_subspace_order (inscy_map.cpp:61-121), whose cell rule is the coarse
// cell's.  Counts go to shared memory first when d * cells fit kHistShared.
constexpr int kHistShared = 8192;
__global__ void k_cell_hist(const uint8_t* __restrict__ cc, int n, int d, int cells, int* __restrict__ hist) {
  __shared__ int sh[kHistShared];
  const int m = d * cells;
  const bool local = m <= kHistShared;
  if (local)
    for (int i = threadIdx.x; i < m; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const long long total = (long long)n * d;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t % d);
    const int c = cc[t];
    if (c < cells) atomicAdd(local ? &sh[k * cells + c] : &hist[k * cells + c], 1);
  }
  __syncthreads();
  if (local)
    for (int i = threadIdx.x; i < m; i += blockDim.x)
      if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

void launch_cell_hist(const uint8_t* cc, int n, int d, int cells, int sms, int* hist, cudaStream_t s) {
  const long long total = (long long)n * d;
  if (total <= 0) return;
  long long blocks = (total + 255) / 256;
  if (blocks > 4LL * sms) blocks = 4LL * sms;
  k_cell_hist<<<(unsigned)blocks, 256, 0, s>>>(cc, n, d, cells, hist);
}

void launch_scatter_rank(const int* order, int n, int* rank, cudaStream_t s) {
  if (n > 0) k_scatter_rank<<<(n + 255) / 256, 256, 0, s>>>(order, n, rank);
}

// One stable pass: out = in stably sorted by bytes[v*d + k].
// `hist` needs 256 * ceil(m / kSortTile) ints; `digit_start` (optional)
// receives the 257 start offsets of the digits.
void launch_byte_sort_pass(const int* in, int* out, int m, const uint8_t* bytes, int d, int k, int* hist,
                           int* hist_total, int* digit_start, void* sums, cudaStream_t s) {
  if (m <= 0) return;
  int nb = (m + kSortTile - 1) / kSortTile;
  ByteDigit fn{bytes, d, k};
  k_digit_hist<<<nb, kSortTile, 0, s>>>(in, m, fn, hist, nb);
  launch_exclusive_scan_int(hist, hist, 256LL * nb, hist_total, sums, s);
  k_digit_scatter<<<nb, kSortTile, 0, s>>>(in, out, m, fn, hist, nb);
  if (digit_start) launch_digit_starts(hist, nb, m, digit_start, s);
}

void launch_candidate_lists(int n, int d, int G, const int* bucket_pts, const int* bucket_off, const int* rank,
                            const uint8_t* fc, const long long* list_off, int* list_pts, cudaStream_t s) {
  long long total = (long long)n * d;
  if (total <= 0) return;
  k_candidate_lists<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n, d, G, bucket_pts, bucket_off, rank, fc,
                                                                    list_off, list_pts);
}

// ---------------------------------------------------------------------------
// scans (the caller owns `sums`: ceil(n / kScanTile) elements of the output type)
// ---------------------------------------------------------------------------
template <class Tin, class Tout>
static void exclusive_scan_impl(const Tin* in, Tout* out, long long n, Tout* total, Tout* sums, cudaStream_t s) {
  long long nt = (n + kScanTile - 1) / kScanTile;
  k_scan_tile_sums<Tin, Tout><<<(unsigned)nt, 256, 0, s>>>(in, n, sums);
  k_scan_single<Tout><<<1, 1024, 0, s>>>(sums, nt, total);
  k_scan_tiles<Tin, Tout><<<(unsigned)nt, 256, 0, s>>>(in, out, n, sums);
}

__global__ void k_zero_ll(long long* p) { *p = 0; }
__global__ void k_zero_i(int* p) { *p = 0; }

void launch_exclusive_scan_int(const int* in, int* out, long long n, int* total, void* sums, cudaStream_t s) {
  if (n <= 0) {
    if (total) k_zero_i<<<1, 1, 0, s>>>(total);
    return;
  }
  exclusive_scan_impl<int, int>(in, out, n, total, (int*)sums, s);
}

void launch_exclusive_scan_ll(const long long* in, long long* out, long long n, long long* total, void* sums,
                              cudaStream_t s) {
  if (n <= 0) {
    if (total) k_zero_ll<<<1, 1, 0, s>>>(total);
    return;
  }
  exclusive_scan_impl<long long, long long>(in, out, n, total, (long long*)sums, s);
}

void launch_exclusive_scan_i2ll(const int* in, long long* out, long long n, long long* total, void* sums,
                                cudaStream_t s) {
  if (n <= 0) {
    if (total) k_zero_ll<<<1, 1, 0, s>>>(total);
    return;
  }
  exclusive_scan_impl<int, long long>(in, out, n, total, (long long*)sums, s);
}

}  // namespace inscy
