// SCY-tree restrict / merge / prune for every (call, dim) of one level.
//
// A call's SCY-tree (ScyTreeNode.h:25-121) is held as
//   * its points, stored in the tree's leaf order (get_points,
//     ScyTreeNode.cu:853-869): lexicographic in the cells of the remaining
//     dims taken in the tree's level order (get_subspace_order,
//     inscy_map.cpp:61-121; the identity unless entropy_order != 0), then the
//     cells of the restricted dims from the last restricted one back to the
//     first, then point id;
//   * its "detached ghosts": s-connection chains (ScyTreeNode.cu:34-49)
//     whose point was pruned earlier but whose chain is still in the trie,
//     each as (point, marker dim g | last level << 8).
//     The chains of points still present are implied by the per-point ghost
//     flags; where they end follows from the call's restricted dims alone.
// A chain holds the trie levels from its marker's down to its last one.
// restrict_node (ScyTreeNode.cu:227-323) keeps a node whose level's dim is
// larger than the restricted dim D even when no point below it lies in the
// restricted cell (`is_included`, :285), and a node above such a node.  In
// the identity level order no such node lies above D's level and chains stay
// whole; in a permuted order restrict leaves count-0 "phantom" nodes above
// D's level and cuts chains to the levels that still hold a kept node.
// Given that representation, the reference's pointer-trie operations become:
//   restrict(D, c)            keep points with cell c on D; a chain whose
//                             marker is on D and lies in cell c marks the
//                             result s-connected; other chains are cut
//                             (chain_cut) and may survive as phantoms;
//   mergeWithNeighbors        absorb cell c+1 while the tree restricted last was
//                             s-connected (ScyTreeNode.cu:837-851); the merged
//                             leaf order is a stable sort by (remaining cells,
//                             cell on D); mergeNodes adds points only to a node
//                             whose count is positive (ScyTreeNode.cu:805-808),
//                             so the absorbed points of a leaf node that the
//                             first cell left empty (a phantom, or the root when
//                             no dim remains) are lost;
//   pruneRecursionAndRemove2  keep weak-dense points (ScyTreeNode.cu:582-667);
//                             propergate_count2 (:446-467) then erases empty
//                             child nodes (phantoms included) together with the
//                             s-connection of the same cell, which decides which
//                             ghosts survive.
// All of this is integer work: filters are block-wide stable compactions; a
// merged run is a stable partition by the cell on D (one counting pass: warp
// match + block scan) and a merge of the cells' already ordered points; the
// chain decisions test the nearest kept points in the sorted key order.
#include <cstdint>
#include <cuda_runtime.h>

#include "inscy_common.cuh"
#include "inscy_prims.cuh"
#include "inscy_kernels.h"

namespace inscy {

// Work items (one call, one dim) of up to kTreeBig points and chains get a
// block of 256 threads; larger ones a block of 1024 in a separate launch, so a
// level's few large items (the root's restrictions hold every point) do not
// leave the GPU waiting on a long tail.
constexpr int kTreeThreads = 256;
constexpr int kTreeThreadsBig = 1024;

// Leaf keys: one cell per dim, kbits bits each; the engine picks the
// narrowest of 32, 64 and 128 bits that holds d * kbits (wide shifts and
// compares cost several instructions each).
using Key128 = unsigned __int128;

struct TreeArgs {
  const CallDesc* calls;
  int ncalls;
  const long long* work_off;  // [ncalls]: first work item of each call
  int nwork;
  const int* pts_in;
  const int2* ghosts_in;
  const uint8_t* cc;
  const unsigned long long* gz;
  int n, d, cells, min_size;
  int kbits;  // bits per cell in the packed leaf keys
  const SubDesc* subs;
  const unsigned* bitmaps;
  char* scratch;  // per work item, at work_scratch[w] bytes: see k_tree_level
  const long long* work_scratch;
  RegionRec* recs;  // per work item: cells records
  int* nrecs;
  int* out_pts;
  unsigned long long* out_pts_top;
  long long out_pts_cap;
  int2* out_ghosts;
  unsigned long long* out_ghost_top;
  long long out_ghost_cap;
  int* err;
  long long pts_in_total;
  long long ghosts_in_total;
  Guard guard;
  uint8_t lvl_pos[kMaxDims];             // trie level of every dim
  uint8_t lvl_dim[kMaxDims];             // dim of every trie level
  unsigned long long gt_pos[kMaxDims];   // per dim e: the levels whose dim is > e
};

// trie levels a .. b as a bit mask (empty when a > b)
__device__ __forceinline__ unsigned long long level_span(int a, int b) {
  if (a > b) return 0ull;
  const unsigned long long hi = b >= 63 ? ~0ull : ((1ull << (b + 1)) - 1ull);
  return hi & ~((1ull << a) - 1ull);
}
__device__ __forceinline__ int top_level(unsigned long long x) { return 63 - __clzll((long long)x); }

// A chain from marker level pg to last level pt after restrict(D) removed
// level pD (rem: the levels left; gt: the levels whose dim is > D; match: its
// point's cell on D is among the restricted ones).  restrict_node keeps a
// chain node whose dim is > D or that has a kept node below; at level pD it
// keeps the node of a restricted cell, whose ancestors are then kept too, and
// reaches nothing below another cell (ScyTreeNode.cu:227-323).  Returns the
// new last level, or -1 when the chain is gone (a chain whose marker is on D
// marks the tree s-connected and is not kept).
__device__ __forceinline__ int chain_cut(int pg, int pt, int pD, unsigned long long rem, unsigned long long gt,
                                         bool match) {
  if (pD == pg) return -1;
  unsigned long long x;
  if (pD < pg) {  // below D's level, under the node of its point's cell on D
    if (!match) return -1;
    x = rem & gt & level_span(pg, pt);
  } else if (pD <= pt) {  // passes D's level
    if (match) {
      x = rem & gt & level_span(pD + 1, pt);
      if (!x) x = rem & level_span(pg, pD - 1);  // holds pg
    } else {
      x = rem & gt & level_span(pg, pD - 1);
    }
  } else {  // ends above D's level: kept in every restricted cell
    x = rem & gt & level_span(pg, pt);
  }
  return x ? top_level(x) : -1;
}

template <class Pred>
__device__ int block_filter(const int* in, int n, Pred pred, int* out, int* sh) {
  int base = 0;
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    int j = c0 + threadIdx.x;
    int x = j < n ? in[j] : 0;
    int f = (j < n && pred(x)) ? 1 : 0;
    int tot;
    int inc = block_inclusive_scan<int>(f, sh, &tot);
    if (f) out[base + inc - 1] = x;
    base += tot;
  }
  __syncthreads();  // the compacted entries are read by other threads next
  return base;
}

// one stable counting-sort pass of (key, value) pairs by an 8-bit digit of
// the key (warp match for the intra-warp rank, block scan across warps)
template <int kWarps, class Key>
__device__ void block_sort_pass(const Key* kin, const int* vin, Key* kout, int* vout, int n, int shift, int* s_base,
                                int* s_tot, int* s_wc, int dmask = 255) {
  const int R = 256;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < R; i += blockDim.x) s_base[i] = 0;
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) atomicAdd(&s_base[(int)(kin[j] >> shift) & dmask], 1);
  __syncthreads();
  if (threadIdx.x < 32) {
    // exclusive scan of the 256 digit counts by one warp
    int v[8], run = 0;
    for (int t = 0; t < 8; ++t) {
      v[t] = s_base[lane * 8 + t];
      run += v[t];
    }
    int inc = run;
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, inc, o);
      if ((int)lane >= o) inc += u;
    }
    int ex = inc - run;
    for (int t = 0; t < 8; ++t) {
      s_base[lane * 8 + t] = ex;
      ex += v[t];
    }
  }
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    for (int i = threadIdx.x; i < kWarps * R; i += blockDim.x) s_wc[i] = 0;
    __syncthreads();
    int j = c0 + threadIdx.x;
    bool valid = j < n;
    Key k = valid ? kin[j] : (Key)0;
    int x = valid ? vin[j] : 0;
    int v = valid ? ((int)(k >> shift) & dmask) : R + (int)lane;
    unsigned peers = __match_any_sync(0xffffffffu, v);
    int rank = __popc(peers & lanemask_lt());
    if (valid && rank == 0) s_wc[warp * R + v] = __popc(peers);
    __syncthreads();
    for (int u = threadIdx.x; u < R; u += blockDim.x) {
      int run = 0;
      for (int w = 0; w < kWarps; ++w) {
        int t = s_wc[w * R + u];
        s_wc[w * R + u] = run;
        run += t;
      }
      s_tot[u] = run;
    }
    __syncthreads();
    if (valid) {
      int o = s_base[v] + s_wc[warp * R + v] + rank;
      kout[o] = k;
      vout[o] = x;
    }
    __syncthreads();
    for (int u = threadIdx.x; u < R; u += blockDim.x) s_base[u] += s_tot[u];
    __syncthreads();
  }
}

template <int kWarps>
struct TreeShared {
  int cnt[256];
  int sf[256];
  int runs[256][2];
  int nruns;
  int lam[kMaxDims];
  int nlam;
  int sh[32];
  int base[256];
  int tot[256];
  int wc[kWarps * 256];
  long long off;
  long long goff;
  int gcount;
  int gwrite;
  int gneed;  // detached chains undecided before the chains' sort
  int seg[kMaxCells + 2];  // a merged run: start of each cell's points after the partition
  // per dim g: last level of the chains of the call's present points with
  // marker g (-1: none), in the call's tree (pst) and after restrict(D) (cst)
  int pst[kMaxDims];
  int cst[kMaxDims];
  unsigned long long remc;   // levels of the restricted tree
  unsigned long long cmask;  // dims g with cst[g] >= 0
  unsigned long long nmask;  // dims whose chains of unmatched points can stay as phantoms
  int kph;                   // deepest level above D's whose dim is > D (-1: none)
  int lph;                   // a merge loses the absorbed points of leaves the first cell left empty
};

// leaf key of point x: its cells on the remaining dims (in level order, most
// significant first), then its cell on the restricted dim D
template <class Key>
__device__ __forceinline__ Key leaf_key(const uint8_t* cc, int d, const int* lam, int nlam, int D, int b, int x) {
  const uint8_t* row = cc + (size_t)x * d;
  Key k = 0;
  for (int t = 0; t < nlam; ++t) k = (k << b) | (Key)row[lam[t]];
  return (k << b) | (Key)row[D];
}

// [lo, hi) of the keys of K[0..m) that share `key`'s prefix above bit `sh`
template <class Key>
__device__ __forceinline__ void key_range(const Key* K, int m, Key key, int sh, int& lo, int& hi) {
  const Key pre = key >> sh;
  int a = 0, b = m;
  while (a < b) {
    int mid = (a + b) >> 1;
    if ((K[mid] >> sh) < pre)
      a = mid + 1;
    else
      b = mid;
  }
  lo = a;
  b = m;
  while (a < b) {
    int mid = (a + b) >> 1;
    if ((K[mid] >> sh) <= pre)
      a = mid + 1;
    else
      b = mid;
  }
  hi = a;
}

// one block per work item: items[blockIdx.x], or blockIdx.x without a list
template <int kThreads, class Key>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads) k_tree_level(TreeArgs a, const int* __restrict__ items, int nitems) {
  __shared__ TreeShared<kThreads / 32> s;
  if ((int)blockIdx.x >= nitems) return;
  const int w = items ? items[blockIdx.x] : (int)blockIdx.x;
  if (w < 0 || w >= a.nwork) return;
  // locate the call of this work item
  int lo = 0, hi = a.ncalls - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (a.work_off[mid] <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int ci = lo;
  const CallDesc C = a.calls[ci];
  const int D = C.f + (int)(w - a.work_off[ci]);
  const int d = a.d;
  const int b = a.kbits;
  const int* P = a.pts_in + C.pts_off;
  const int np = C.npts;
  const int2* Gh = a.ghosts_in + C.ghost_off;
  const int ng = C.nghost;
  if (!GUARD_OK(a.guard, C.pts_off >= 0 && C.pts_off + np <= a.pts_in_total, 51, C.pts_off + np)) return;
  if (!GUARD_OK(a.guard, ng == 0 || (C.ghost_off >= 0 && C.ghost_off + ng <= a.ghosts_in_total), 52,
                C.ghost_off + ng))
    return;
  const uint64_t smask = C.rmask | (1ull << D);
  const SubDesc& S = a.subs[C.child_sub + (D - C.f)];
  const unsigned* wd = a.bitmaps + S.bitmap_off;
  // scratch: keys first (16-byte aligned), then ints
  char* base = a.scratch + a.work_scratch[w];
  // key buffers in 16-byte slots whatever the key width (a free one holds
  // 8-byte chain masks later)
  Key* KA = (Key*)base;                              // np: leaf keys of the region's points
  Key* KB = (Key*)(base + 16LL * np);                // np
  Key* KG = (Key*)(base + 32LL * np);                // ng: leaf keys of the region's detached chains
  Key* KH = (Key*)(base + 32LL * np + 16LL * ng);    // ng
  int* A = (int*)(base + 32LL * (np + ng));  // np: the region's points
  int* B = A + np;
  int* SV = B + np;       // np + 1 survivor prefix counts
  int* GA = SV + np + 1;  // ng: detached chains of the region
  int* GB = GA + ng;
  int* GC = GB + ng;      // ng: per detached chain, its cell on D and its cut (see step 2)
  RegionRec* rec = a.recs + (long long)w * a.cells;

  // 0. the call's points and chains must be valid ids (checked once)
  if (threadIdx.x == 0) s.gcount = 0;
  __syncthreads();
  for (int j = threadIdx.x; j < np; j += blockDim.x)
    if (!GUARD_OK(a.guard, P[j] >= 0 && P[j] < a.n, 53, P[j])) s.gcount = 1;
  for (int j = threadIdx.x; j < ng; j += blockDim.x) {
    const int y = Gh[j].y;
    if (!GUARD_OK(a.guard, Gh[j].x >= 0 && Gh[j].x < a.n && y >= 0 && (y & 255) < d && (y >> 8) < d, 54, Gh[j].x))
      s.gcount = 1;
  }
  __syncthreads();
  if (s.gcount) return;
  // 1. the levels of the call's tree and of the restricted one, and where the
  //    chains of present points end in each
  const int pD = a.lvl_pos[D];
  const unsigned long long gtD = a.gt_pos[D];
  if (threadIdx.x == 0) {
    unsigned long long remp = 0;
    for (int k = 0; k < d; ++k)
      if (!((C.rmask >> k) & 1ull)) remp |= 1ull << a.lvl_pos[k];
    const unsigned long long remc = remp & ~(1ull << pD);
    s.remc = remc;
    const unsigned long long above = remp & gtD & level_span(0, pD - 1);
    s.kph = above ? top_level(above) : -1;
    // restricting the deepest level: the level above keeps count-0 leaves
    // when its dim is > D, and with no level left the root is the leaf
    s.lph = top_level(remp) == pD && (remc == 0ull || a.lvl_dim[top_level(remc)] > D);
  }
  if (threadIdx.x < d) {
    const int g = threadIdx.x;
    int pt = -1, ct = -1;
    if (!((C.rmask >> g) & 1ull)) {
      // a chain starts whole at the build (ScyTreeNode.cu:36-47); present
      // points matched every restriction, made in ascending dim order
      const int pg = a.lvl_pos[g];
      unsigned long long rem = d == 64 ? ~0ull : ((1ull << d) - 1ull);
      pt = d - 1;
      unsigned long long rm = C.rmask;
      while (rm && pt >= 0) {
        const int e = __ffsll((long long)rm) - 1;
        rm &= rm - 1;
        rem &= ~(1ull << a.lvl_pos[e]);
        pt = chain_cut(pg, pt, a.lvl_pos[e], rem, a.gt_pos[e], true);
      }
      if (pt >= 0 && g != D) ct = chain_cut(pg, pt, pD, rem & ~(1ull << pD), gtD, true);
    }
    s.pst[g] = pt;
    s.cst[g] = ct;
  }
  // 2. cell counts and s-connection flags on D
  for (int i = threadIdx.x; i < a.cells; i += blockDim.x) {
    s.cnt[i] = 0;
    s.sf[i] = 0;
  }
  __syncthreads();
  const bool sconn_present = s.pst[D] >= 0;
  for (int j = threadIdx.x; j < np; j += blockDim.x) {
    int x = P[j];
    int c = a.cc[(size_t)x * d + D];
    atomicAdd(&s.cnt[c], 1);
    if (sconn_present && ((a.gz[x] >> D) & 1ull)) s.sf[c] = 1;
  }
  // per detached chain, once for all runs: its point's cell on D (bits 0-7)
  // and its last level + 1 after the restriction when that cell is in the run
  // (bits 8-15) and when not (bits 16-23); 0: gone (or marker on D / restricted)
  {
    const unsigned long long remc0 = s.remc;
    uint64_t lm = ~smask;
    if (d < 64) lm &= (1ull << d) - 1;
    for (int j = threadIdx.x; j < ng; j += blockDim.x) {
      const int2 gg = Gh[j];
      const int g = gg.y & 255;
      const int cx = a.cc[(size_t)gg.x * d + D];
      if (g == D) s.sf[cx] = 1;
      int packed = cx;
      if (g != D && ((lm >> g) & 1ull)) {
        const int pm = chain_cut(a.lvl_pos[g], gg.y >> 8, pD, remc0, gtD, true);
        const int pn = chain_cut(a.lvl_pos[g], gg.y >> 8, pD, remc0, gtD, false);
        packed |= ((pm + 1) << 8) | ((pn + 1) << 16);
      }
      GC[j] = packed;
    }
  }
  __syncthreads();
  // 3. merge runs (InscyNodeCpu.cu:179-192 with mergeWithNeighbors) and the
  //    remaining dims of the restricted tree, in level order
  if (threadIdx.x == 0) {
    int nr = 0, c = 0;
    while (c < a.cells) {
      int c0 = c;
      while (s.sf[c] && c < a.cells - 1) ++c;
      s.runs[nr][0] = c0;
      s.runs[nr][1] = c;
      ++nr;
      ++c;
    }
    s.nruns = nr;
    int nl = 0;
    for (int t = 0; t < d; ++t)
      if ((s.remc >> t) & 1ull) s.lam[nl++] = a.lvl_dim[t];
    s.nlam = nl;
    unsigned long long cm = 0, nm = 0;
    for (int g = 0; g < d; ++g) {
      if (s.cst[g] >= 0) cm |= 1ull << g;
      // an unmatched point's chain stays only through a level above D's
      // whose dim is > D
      if (g != D && s.pst[g] >= 0 && s.kph >= 0 && a.lvl_pos[g] <= s.kph) nm |= 1ull << g;
    }
    s.cmask = cm;
    s.nmask = nm;
  }
  __syncthreads();
  const int nruns = s.nruns;
  const int nlam = s.nlam;
  const int key_bits = (nlam + 1) * b;
  const unsigned long long remc = s.remc;
  const int kph = s.kph;
  const bool lph = s.lph != 0;
  uint64_t lammask = ~smask;
  if (d < 64) lammask &= (1ull << d) - 1;
  const Key cellmask = ((Key)1 << b) - (Key)1;
  // trie level of dim g in the restricted tree
  auto level_of = [&](int g) { return __popcll(remc & ((1ull << a.lvl_pos[g]) - 1ull)); };

  for (int r = 0; r < nruns; ++r) {
    const int c0 = s.runs[r][0], c1 = s.runs[r][1];
    // 4. restrict (+ merge): points of the run, in the parent's order
    int m = block_filter(
        P, np,
        [&](int x) {
          int c = a.cc[(size_t)x * d + D];
          return c >= c0 && c <= c1;
        },
        A, s.sh);
    for (int j = threadIdx.x; j < m; j += blockDim.x) KA[j] = leaf_key<Key>(a.cc, d, s.lam, nlam, D, b, A[j]);
    __syncthreads();
    // 5. merged runs: stable re-sort by the leaf key (remaining cells, cell on
    //    D); equal keys keep their order (the restricted dims, then id).  The
    //    points of one cell come in the parent's order, which already orders
    //    them by this key (their cell on D is the same), so a run of up to 8
    //    cells is a stable partition by the cell on D and a merge: a point's
    //    place is its rank in its cell plus the keys smaller than its own in
    //    the other cells (binary searches; keys of different cells differ).
    //    Longer runs take the radix passes over the whole key.
    Key* kcur = KA;
    int* cur = A;
    if (c1 > c0 && m > 1 && c1 - c0 < 8) {
      block_sort_pass<kThreads / 32>(KA, A, KB, B, m, 0, s.base, s.tot, s.wc, (int)cellmask);
      if (threadIdx.x == 0) {
        int o = 0;
        for (int c = c0; c <= c1; ++c) {
          s.seg[c - c0] = o;
          o += s.cnt[c];
        }
        s.seg[c1 - c0 + 1] = o;
      }
      __syncthreads();
      const int nk = c1 - c0 + 1;
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const Key key = KB[i];
        const int ci = (int)(key & cellmask) - c0;
        int pos = i - s.seg[ci];
        for (int t = 0; t < nk; ++t) {
          if (t == ci) continue;
          int lo = s.seg[t], hi = s.seg[t + 1];
          const int base0 = lo;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (KB[mid] < key)
              lo = mid + 1;
            else
              hi = mid;
          }
          pos += lo - base0;
        }
        KA[pos] = key;
        A[pos] = B[i];
      }
      __syncthreads();
    } else if (c1 > c0 && m > 1) {
      Key* koth = KB;
      int* oth = B;
      for (int sh = 0; sh < key_bits; sh += 8) {
        block_sort_pass<kThreads / 32>(kcur, cur, koth, oth, m, sh, s.base, s.tot, s.wc);
        Key* tk = kcur;
        kcur = koth;
        koth = tk;
        int* t = cur;
        cur = oth;
        oth = t;
      }
    }
    // 6. prune: weak density of the subspace, survivor prefix counts.  A
    //    merge into a leaf node that the run's first cell left empty loses
    //    the absorbed points: they count as pruned.
    const bool drops = lph && c1 > c0;
    int npp = 0;
    for (int c = 0; c < m; c += blockDim.x) {
      int j = c + threadIdx.x;
      int f = 0;
      if (j < m) {
        int x = cur[j];
        f = (wd[x >> 5] >> (x & 31)) & 1u;
        if (f && drops) {
          int glo, ghi;
          key_range(kcur, m, kcur[j], b, glo, ghi);  // the point's leaf node
          if ((int)(kcur[glo] & cellmask) != c0) f = 0;
        }
      }
      int tot;
      int inc = block_inclusive_scan<int>(f, s.sh, &tot);
      if (j < m) SV[j] = npp + inc - f;
      npp += tot;
    }
    if (threadIdx.x == 0) SV[m] = npp;
    __syncthreads();
    const bool passed = npp >= a.min_size;
    long long pts_off = -1, ghost_off = -1;
    int nghost = 0;
    if (passed) {
      if (threadIdx.x == 0) {
        unsigned long long o = atomicAdd(a.out_pts_top, (unsigned long long)npp);
        if ((long long)(o + npp) > a.out_pts_cap) {
          atomicExch(a.err, 1);
          s.off = -1;
        } else {
          s.off = (long long)o;
        }
      }
      __syncthreads();
      pts_off = s.off;
      // kpos[r]: position (in the sorted order) of the r-th kept point, in the
      // int buffer the merge sort did not end in
      int* kpos = cur == A ? B : A;
      for (int j = threadIdx.x; j < m; j += blockDim.x) {
        if (SV[j + 1] != SV[j]) {
          kpos[SV[j]] = j;
          if (pts_off >= 0) a.out_pts[pts_off + SV[j]] = cur[j];
        }
      }
      __syncthreads();
      // 7. ghosts of the pruned tree.  A detached chain's fate mostly follows
      //    from the points' nodes (its place among the sorted point keys and
      //    the nearest kept points there); only a chain whose sibling node
      //    holds no point at all needs "does a deeper chain pass this node",
      //    a range search on the chains' own keys, so the region's chains are
      //    sorted by leaf key only when some chain needs that.
      int ngp = 0;
      if (ng > 0) {
        for (int c = 0; c < ng; c += blockDim.x) {
          int j = c + threadIdx.x;
          int f = 0;
          if (j < ng) {
            const int gc = GC[j];
            const int cx = gc & 255;
            f = ((gc >> ((cx >= c0 && cx <= c1) ? 8 : 16)) & 255) != 0 ? 1 : 0;
          }
          int tot;
          int inc = block_inclusive_scan<int>(f, s.sh, &tot);
          if (f) GA[ngp + inc - 1] = j;
          ngp += tot;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < ngp; j += blockDim.x) KG[j] = leaf_key<Key>(a.cc, d, s.lam, nlam, D, b, Gh[GA[j]].x);
        __syncthreads();
      }
      // The keep decisions are made once and stored in buffers free by now
      // (the key buffer the merge sort did not end in; the chains' sort
      // buffer), then the surviving chains are written at one reserved range.
      unsigned long long* kmask = (unsigned long long*)(kcur == KA ? KB : KA);  // per point: chain dims kept
      int* gkeep = GB;                                                          // per detached chain: kept
      if (threadIdx.x == 0) {
        s.gcount = 0;
        s.gwrite = 0;
        s.gneed = 0;
      }
      __syncthreads();
      // (a) chains of points pruned (or lost) here: a chain survives when a
      //     kept point shares the cells of every remaining dim up to the
      //     chain's level
      //     The keys are sorted, so of all kept points the nearest one on
      //     either side of a position shares the longest prefix with it: "a
      //     kept point shares the cells through level l" is a test of those
      //     two.  kept_left(p): the last kept position < p; kept_right(p): the
      //     first kept position >= p (-1: none).
      auto kept_left = [&](int p) { return SV[p] > 0 ? kpos[SV[p] - 1] : -1; };
      auto kept_right = [&](int p) { return SV[p] < npp ? kpos[SV[p]] : -1; };
      const unsigned long long cmask = s.cmask;
      for (int j = threadIdx.x; j < m; j += blockDim.x) {
        unsigned long long km = 0;
        if (SV[j + 1] == SV[j]) {
          unsigned long long gb = a.gz[cur[j]] & lammask & cmask;
          if (gb) {
            const Key kj = kcur[j];
            const int il = kept_left(j), ir = kept_right(j);
            const Key xl = il >= 0 ? kcur[il] ^ kj : ~(Key)0;
            const Key xr = ir >= 0 ? kcur[ir] ^ kj : ~(Key)0;
            while (gb) {
              const int g = __ffsll((long long)gb) - 1;
              gb &= gb - 1;
              const int sh = b * (nlam - level_of(g));  // prefix through the chain's level
              if ((xl >> sh) == 0 || (xr >> sh) == 0) km |= 1ull << g;
            }
          }
          if (km) atomicAdd(&s.gcount, __popcll(km));
        }
        kmask[j] = km;
      }
      // (b) chains detached earlier: 1 kept, 0 dropped, 2 undecided until the
      //     chains are sorted (`sorted` false)
      // a key's place among the sorted point keys, and whether a kept point
      // (kept) or any point (any) shares its prefix above bit sh
      auto lower = [&](Key kx) {
        int lo = 0, hi = m;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (kcur[mid] < kx)
            lo = mid + 1;
          else
            hi = mid;
        }
        return lo;
      };
      auto kept_shares = [&](Key kx, int p, int sh) {
        const int il = kept_left(p), ir = kept_right(p);
        return (il >= 0 && ((kcur[il] ^ kx) >> sh) == 0) || (ir >= 0 && ((kcur[ir] ^ kx) >> sh) == 0);
      };
      auto decide = [&](int jj, bool sorted) -> int {
        const int2 gg = Gh[GA[jj]];
        const int g = gg.y & 255;
        const Key kx = KG[jj];
        const int l = level_of(g);
        const int p = lower(kx);
        const int sh = b * (nlam - l);
        if (l > 0 && !kept_shares(kx, p, sh + b)) return 0;  // the parent node (through level l-1) keeps no point
        if (kept_shares(kx, p, sh)) return 1;                 // the sibling node keeps points
        if ((p > 0 && ((kcur[p - 1] ^ kx) >> sh) == 0) || (p < m && ((kcur[p] ^ kx) >> sh) == 0))
          return 0;  // the sibling node existed and is erased with it
        if (a.lvl_pos[g] <= kph) {
          // restrict kept the path of every point of the call down to level
          // kph, so the sibling node existed (as a phantom) when a point of
          // the call shares its cells; the call's points are in leaf order,
          // whose first levels are these
          const uint8_t* rx = a.cc + (size_t)gg.x * d;
          Key want = 0;
          for (int t = 0; t <= l; ++t) want = (want << b) | (Key)rx[s.lam[t]];
          int lo2 = 0, hi2 = np;
          Key got = 0;
          while (lo2 < hi2) {
            const int mid = (lo2 + hi2) >> 1;
            const uint8_t* ry = a.cc + (size_t)P[mid] * d;
            Key ky = 0;
            for (int t = 0; t <= l; ++t) ky = (ky << b) | (Key)ry[s.lam[t]];
            if (ky < want)
              lo2 = mid + 1;
            else
              hi2 = mid;
          }
          if (lo2 < np) {
            const uint8_t* ry = a.cc + (size_t)P[lo2] * d;
            for (int t = 0; t <= l; ++t) got = (got << b) | (Key)ry[s.lam[t]];
            if (got == want) return 0;
          }
        }
        // the sibling node exists only if a deeper detached chain passes it
        if (!sorted) return 2;
        int glo, ghi;
        key_range(KG, ngp, kx, b * (nlam - l), glo, ghi);
        for (int t = glo; t < ghi; ++t)
          if (level_of(Gh[GA[t]].y & 255) > l) return 0;
        return 1;
      };
      for (int jj = threadIdx.x; jj < ngp; jj += blockDim.x) {
        const int k = decide(jj, ngp <= 1);
        gkeep[jj] = k;
        if (k == 2) atomicAdd(&s.gneed, 1);
      }
      __syncthreads();
      if (s.gneed > 0) {
        // sort the chains by leaf key (the sort buffers hold no decision yet
        // worth keeping: all are made again on the sorted order)
        Key* kc = KG;
        Key* ko = KH;
        int* gc = GA;
        int* go = GB;
        for (int sh = 0; sh < key_bits; sh += 8) {
          block_sort_pass<kThreads / 32>(kc, gc, ko, go, ngp, sh, s.base, s.tot, s.wc);
          Key* tk = kc;
          kc = ko;
          ko = tk;
          int* t = gc;
          gc = go;
          go = t;
        }
        if (gc != GA) {
          for (int j = threadIdx.x; j < ngp; j += blockDim.x) {
            GA[j] = gc[j];
            KG[j] = kc[j];
          }
          __syncthreads();
        }
        for (int jj = threadIdx.x; jj < ngp; jj += blockDim.x) gkeep[jj] = decide(jj, true);
        __syncthreads();
      }
      // (c) chains of the call's points outside the run: restrict kept their
      //     path down to level kph (phantom nodes, no points), so their
      //     sibling node existed; a chain survives when a kept point shares
      //     the cells up to its level.  Counted here, written below.
      const unsigned long long nmask = s.nmask;
      auto unmatched = [&](int j, bool write) {
        const int x = P[j];
        unsigned long long gb = a.gz[x] & nmask;
        if (!gb) return 0;
        const int cx = a.cc[(size_t)x * d + D];
        if (cx >= c0 && cx <= c1) return 0;
        const Key kx = leaf_key<Key>(a.cc, d, s.lam, nlam, D, b, x);
        int kept = 0;
        while (gb) {
          const int g = __ffsll((long long)gb) - 1;
          gb &= gb - 1;
          const int pt = chain_cut(a.lvl_pos[g], s.pst[g], pD, remc, gtD, false);
          if (pt < 0) continue;
          if (!kept_shares(kx, lower(kx), b * (nlam - level_of(g)))) continue;
          ++kept;
          if (write) {
            const int o = atomicAdd(&s.gwrite, 1);
            if (o < s.gcount) a.out_ghosts[s.goff + o] = make_int2(x, g | (pt << 8));
          }
        }
        return kept;
      };
      {
        int kept = 0;
        for (int jj = threadIdx.x; jj < ngp; jj += blockDim.x) kept += gkeep[jj];
        if (nmask)
          for (int j = threadIdx.x; j < np; j += blockDim.x) kept += unmatched(j, false);
        if (kept) atomicAdd(&s.gcount, kept);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned long long o = atomicAdd(a.out_ghost_top, (unsigned long long)s.gcount);
        if ((long long)(o + s.gcount) > a.out_ghost_cap) {
          atomicExch(a.err, 2);
          s.gcount = 0;  // nothing is written; the host retries with more room
          o = 0;
        }
        s.goff = (long long)o;
      }
      __syncthreads();
      if (s.gcount > 0) {
        for (int j = threadIdx.x; j < m; j += blockDim.x) {
          unsigned long long km = kmask[j];
          while (km) {
            const int g = __ffsll((long long)km) - 1;
            km &= km - 1;
            const int o = atomicAdd(&s.gwrite, 1);
            if (o < s.gcount) a.out_ghosts[s.goff + o] = make_int2(cur[j], g | (s.cst[g] << 8));
          }
        }
        for (int jj = threadIdx.x; jj < ngp; jj += blockDim.x)
          if (gkeep[jj]) {
            const int2 gg = Gh[GA[jj]];
            const int g = gg.y & 255;
            const int gc = GC[GA[jj]];
            const int cx = gc & 255;
            const int pt = ((gc >> ((cx >= c0 && cx <= c1) ? 8 : 16)) & 255) - 1;
            const int o = atomicAdd(&s.gwrite, 1);
            if (o < s.gcount) a.out_ghosts[s.goff + o] = make_int2(gg.x, g | (pt << 8));
          }
        if (nmask)
          for (int j = threadIdx.x; j < np; j += blockDim.x) unmatched(j, true);
      }
      ghost_off = s.goff;
      nghost = s.gcount;
    }
    if (threadIdx.x == 0) {
      RegionRec R;
      R.call = ci;
      R.dim = D;
      R.c0 = c0;
      R.c1 = c1;
      R.npts = npp;
      R.passed = passed ? 1 : 0;
      R.pts_off = pts_off;
      R.ghost_off = ghost_off;
      R.nghost = nghost;
      R.pad = 0;
      rec[r] = R;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) a.nrecs[w] = nruns;
}

template <class Key>
static void tree_launches(const TreeArgs& a, const TreeLaunch& L, cudaStream_t s) {
  if (L.nbig > 0) {
    k_tree_level<kTreeThreadsBig, Key><<<L.nbig, kTreeThreadsBig, 0, s>>>(a, L.items_big, L.nbig);
    if (L.nsmall > 0) k_tree_level<kTreeThreads, Key><<<L.nsmall, kTreeThreads, 0, s>>>(a, L.items_small, L.nsmall);
  } else {
    k_tree_level<kTreeThreads, Key><<<L.nwork, kTreeThreads, 0, s>>>(a, nullptr, L.nwork);
  }
}

void launch_tree_level(const TreeLaunch& L, cudaStream_t s) {
  if (L.nwork <= 0) return;
  TreeArgs a;
  a.calls = L.calls;
  a.ncalls = L.ncalls;
  a.work_off = L.work_off;
  a.nwork = L.nwork;
  a.pts_in = L.pts_in;
  a.ghosts_in = L.ghosts_in;
  a.cc = L.cc;
  a.gz = L.gz;
  a.n = L.n;
  a.d = L.d;
  a.cells = L.cells;
  a.min_size = L.min_size;
  a.kbits = L.kbits;
  a.subs = L.subs;
  a.bitmaps = L.bitmaps;
  a.scratch = L.scratch;
  a.work_scratch = L.work_scratch;
  a.recs = L.recs;
  a.nrecs = L.nrecs;
  a.out_pts = L.out_pts;
  a.out_pts_top = L.out_pts_top;
  a.out_pts_cap = L.out_pts_cap;
  a.out_ghosts = L.out_ghosts;
  a.out_ghost_top = L.out_ghost_top;
  a.out_ghost_cap = L.out_ghost_cap;
  a.err = L.err;
  a.pts_in_total = L.pts_in_total;
  a.ghosts_in_total = L.ghosts_in_total;
  a.guard = L.guard;
  for (int k = 0; k < kMaxDims; ++k) {
    a.lvl_pos[k] = L.lvl_pos[k];
    a.lvl_dim[k] = L.lvl_dim[k];
    a.gt_pos[k] = L.gt_pos[k];
  }
  if (L.key_bytes <= 4)
    tree_launches<uint32_t>(a, L, s);
  else if (L.key_bytes <= 8)
    tree_launches<unsigned long long>(a, L, s);
  else
    tree_launches<Key128>(a, L, s);
}

}  // namespace inscy
