// Shared device-side types and helpers of the GB300 INSCY engine.
//
// Terminology (follows the reference, mrjakobdk/GPU_INSCY):
//   * coarse cell  -- the SCY-tree grid cell, min(int(x / (1/cells)), cells-1)
//                     (ScyTreeNode.cu:100-102);
//   * fine cell    -- the same rule on the ceil(1/eps) grid of the
//                     neighbourhood tree (inscy_map.cpp:243);
//   * ghost        -- an s-connection chain (ScyTreeNode.cu:34-49): point p
//                     owns one on dim k when x[p][k] >= (cell+1)/cells - eps;
//   * subspace     -- a set of restricted dims, always restricted in
//                     ascending order, kept as a 64-bit mask;
//   * call         -- one INSCY recursion node (InscyNodeCpu.cu:159-235):
//                     a restricted, merged and pruned SCY-tree;
//   * region       -- one restriction of a call to (dim, run of cells), after
//                     mergeWithNeighbors (ScyTreeNode.cu:837-851).
#pragma once
#include <cstring>
#include <cstdint>
#include <cuda_runtime.h>

namespace inscy {

constexpr int kMaxDims = 64;    // subspaces are 64-bit masks
constexpr int kMaxCells = 255;  // coarse cells fit a byte
constexpr int kWarp = 32;
// point rows of the density pass: 16, 24 or 32 slots (the least >= d), none
// above 32
__host__ __device__ inline int row_slots(int d) { return d <= 16 ? 16 : d <= 24 ? 24 : d <= 32 ? 32 : 0; }

// Region record written by the level kernel (one per restriction run).
struct RegionRec {
  int call;       // index of the parent call in its level
  int dim;        // restricted dim
  int c0, c1;     // run of merged cells [c0, c1]
  int npts;       // points left after the weak-density prune
  int passed;     // npts >= min_size: the region recurses (becomes a call)
  long long pts_off;    // where its pruned points were written (passed only)
  long long ghost_off;  // where its detached ghosts were written (passed only)
  int nghost;
  int pad;
};

// One call of the level being expanded (device view).
struct CallDesc {
  long long pts_off;    // points, in the call's leaf order
  long long ghost_off;  // detached ghosts: (point, dim) pairs
  uint64_t rmask;       // restricted dims
  int npts;
  int f;                // first dim the call restricts (InscyNodeCpu.cu:172)
  int nghost;
  int sub;              // the call's subspace in the previous level (-1: root)
  int child_sub;        // first child subspace (dim f) in the current level
  int nrestricted;
};

// A subspace whose density is evaluated at the current level.
struct SubDesc {
  uint64_t mask;      // dims of the subspace
  int dim;            // its largest dim (the one added at this level)
  int nsub;           // |S|
  int parent;         // parent subspace in the previous level (-1 at level 1)
  int nquery;         // query points = kept points of the parent (all points at level 1)
  long long item_off;   // first work item of this subspace
  long long query_off;  // parent's kept-point list offset (level 1: unused)
  long long plist_base; // parent's list base (entry offsets are absolute)
  long long bitmap_off; // word offset of this subspace's flag bitmaps
  // 1: candidates must lie within +-1 fine cell of the query on `dim`.  The
  // neighbourhood trie's walk (ScyTreeNode.cu:896-934) tests a subspace dim
  // only while the subspace's dims, in ascending order, appear in the trie's
  // level order; under a permuted level order the dims after the first
  // inversion are left to the distance test alone.
  int win;
  int pad;
};

// The children of one parent subspace (contiguous subspace indices).
struct GroupDesc {
  long long warp_off;   // first (child, query) work item of the group
  long long qwarp_off;  // first query of the group (one warp per query)
  int sub_base;
  int nchild;
  int nquery;
  int nowin;  // bit c: child c takes no fine-cell test (its SubDesc::win is 0; children < 32)
};

// One (group, query) pair of a level >= 2 density pass, resolved once by the
// capacity kernel for the row kernel: the query point, its parent list, and
// the group's children (dims d0 .. d0 + nc - 1, subspaces sub_base ..).
// len < 0 marks a pair whose checks failed (the guard holds the reason).
struct alignas(16) RowItem {
  long long pb;  // parent-list start
  int len;       // parent-list length
  int p;         // query point
  int sub_base;  // first child subspace
  int i;         // query index within the group
  short d0;      // first child's dim
  short nc;      // children
  int nowin;     // the group's GroupDesc::nowin
};

// Device-side consistency checks: the first failed check records its code and
// the offending value; the caller skips the access and the host reports the
// failure after the launch (INSCY_ERR_INTERNAL) instead of touching memory out
// of range.
struct Guard {
  int* code;
  long long* info;
};
__device__ __forceinline__ bool guard_fail(const Guard& g, int code, long long v) {
  if (atomicCAS(g.code, 0, code) == 0) *g.info = v;
  return false;
}
#define GUARD_OK(g, cond, code, v) ((cond) || guard_fail((g), (code), (long long)(v)))

// Per-point flag bits of a (subspace, point) evaluation.
enum : uint8_t { kFlagWeak = 1, kFlagDense = 2, kFlagKeep = 4 };

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Asynchronous 16-byte global -> shared copies of one thread (cp.async, cached
// in L1): both addresses 16-byte aligned; a thread's copies complete in the
// order of its commit groups, and async_wait<N> waits until at most N of its
// groups are pending.  Host execution of these sources copies at once.
#ifdef __CUDACC__
__device__ __forceinline__ void async_copy16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
#else
inline void async_copy16(void* smem, const void* gmem) { std::memcpy(smem, gmem, 16); }
inline void async_commit() {}
template <int N>
inline void async_wait() {}
#endif

// Squared-distance step of dist() (ClusteringCpu.cu:40-50): acc + diff*diff
// with each operation rounded separately (no fused multiply-add).
__device__ __forceinline__ float dist_step(float acc, float xp, float xq) {
  float diff = __fsub_rn(xp, xq);
  return __fadd_rn(acc, __fmul_rn(diff, diff));
}

// phi() term (ClusteringCpu.cu:118-120): d = dist/eps; sq = d*d; the float
// sum absorbs (1. - sq) through a double addition, then rounds to float.
__device__ __forceinline__ double phi_term(float dist, float eps) {
  float dd = __fdiv_rn(dist, eps);
  float sq = __fmul_rn(dd, dd);
  return __dsub_rn(1.0, (double)sq);
}
__device__ __forceinline__ float phi_add(float sum, double term) {
  return __double2float_rn(__dadd_rn((double)sum, term));
}

}  // namespace inscy
