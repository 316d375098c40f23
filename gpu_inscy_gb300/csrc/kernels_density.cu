// epsilon-neighbourhood density of every (subspace, point) of one lattice level.
//
// Reference semantics (ClusteringCpu.cu:40-125, ScyTreeNode.cu:896-946):
//   * candidates of p in subspace S are the points whose fine cells are within
//     +-1 of p's on every dim of S, in neighbourhood-trie order;
//   * q != p is a neighbour when eps >= sqrt(sum over S, ascending, of
//     (p_k - q_k)^2), every operation rounded separately;
//   * phi(p) = sum over neighbours, in candidate order, of (1 - (dist/eps)^2)
//     accumulated in float through a double addition;
//   * dense / weak-dense / rectangular tests compare phi (or the neighbour
//     count) with host-computed float thresholds.
//
// Because subspaces are extended by their largest dim D, N(p, S u {D}) is the
// ordered subsequence of N(p, S) that passes the +-1 test on D and the
// distance test; the partial squared distance is stored with each list entry
// so a child adds exactly one term, in the reference's summation order.
// Level-1 subspaces {D} read the precomputed candidate list of p's fine cell.
//
// Kernels: the candidate pass writes every item's ordered list (level 1:
// k_neighbours, one warp per (subspace, query point); levels >= 2:
// k_neighbours_rows over point rows when d <= 32, else k_neighbours_multi, one
// warp per (parent subspace, query point) testing all children), candidates
// 32 at a time with a ballot; k_density_phi then sums each list on one lane
// and k_density_flags turns the sums into flags and bitmap bits.
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>
#ifdef __CUDACC__
#include <cuda.h>  // CUtensorMap (the type only: the encoder is reached through the runtime)
#endif

#include "inscy_common.cuh"
#include "inscy_kernels.h"
#include "phi_exact.cuh"

namespace inscy {

struct DensityArgs {
  const SubDesc* subs;
  int nsubs;
  long long nitems;
  const GroupDesc* groups;  // children of one parent subspace, walked child-fastest
  int ngroups;
  long long nwarps;
  const float* X;
  const uint8_t* fc;
  int n, d, G;
  float eps;
  int rect;
  float acc_max;  // eps >= sqrt(acc)  <=>  acc <= acc_max (sqrt is monotone)
  float thr_weak;
  const float* thr_dense;  // [|S|]
  const float* thr_keep;   // [|S|]
  // level-1 candidate lists
  const long long* cand_off;  // d*G + 1
  const int* cand_pts;
  // previous level (parent subspaces): kept points and their lists
  const int* prev_keep;
  const long long* prev_loff;
  const int* prev_lcnt;
  const int2* prev_ent;  // parent-level list entries (ListEnt)
  // outputs
  int* cnt;           // [nitems] neighbours
  uint8_t* flags;     // [nitems]
  unsigned* bitmaps;  // per subspace 3 * W words (weak, dense, keep)
  int words;          // W = ceil(n / 32)
  const long long* loff;  // [nitems] list start of every item
  int2* ent;  // this level's list entries (ListEnt)
  unsigned long long* cand_counter;  // candidate tests (candidate x child subspace)
  unsigned long long* list_counter;  // list entries read
  unsigned long long* out_counter;   // list entries written (single-pass write)
  // single-pass write (levels >= 2): the list of child c of (group, query) w
  // starts at cap_base[w] + c * (the query's parent-list length), a bound on
  // its length; the kernel writes every item's count and list start (cap_loff)
  const long long* cap_base;
  long long* cap_loff;
  // point rows (d <= 32) and the work counter of k_neighbours_rows
  const float* xrow;
  const float* win;
  unsigned long long* work;
  RowItem* items;        // per (group, query): written by k_list_capacity, read by k_neighbours_rows
  int slots;             // row width of xrow / win (16, 24 or 32; 0: no rows)
  int chunk;             // (group, query) pairs a warp takes per counter update
  long long prev_total;  // entries in the previous level's lists
  long long total;       // entries in this level's lists (write passes)
  long long prev_nkeep;  // kept points of the previous level
  Guard guard;
};

__device__ __forceinline__ int find_sub(const SubDesc* subs, int nsubs, long long item) {
  int lo = 0, hi = nsubs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (subs[mid].item_off <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// warp w -> (subspace, query index): the children of one parent are adjacent,
// so the parent's list of a point is read by its siblings back to back (L2)
__device__ __forceinline__ void locate(const DensityArgs& a, long long w, int& si, long long& i) {
  int lo = 0, hi = a.ngroups - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (a.groups[mid].warp_off <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  const GroupDesc g = a.groups[lo];
  long long j = w - g.warp_off;
  i = j / g.nchild;
  si = g.sub_base + (int)(j % g.nchild);
}

// count (kWrite = false) or write (kWrite = true) the ordered neighbour list
// of one (subspace, point): candidates 32 at a time, accepted lanes by ballot
// Per-block sums of the statistics counters: one shared add per warp and one
// global add per block (per-warp global atomics on the same few counters
// saturate the L2 slice that holds them).
struct BlockStats {
  unsigned long long cand, list, out;
};
__device__ __forceinline__ void block_stats_begin(BlockStats& s) {
  if (threadIdx.x == 0) s.cand = s.list = s.out = 0;
  __syncthreads();
}
__device__ __forceinline__ void block_stats_end(BlockStats& s, const DensityArgs& a, unsigned long long cand,
                                                unsigned long long list, unsigned long long out = 0) {
  if (lane_id() == 0 && (cand || list || out)) {
    atomicAdd(&s.cand, cand);
    atomicAdd(&s.list, list);
    atomicAdd(&s.out, out);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (a.cand_counter && s.cand) atomicAdd(a.cand_counter, s.cand);
    if (a.list_counter && s.list) atomicAdd(a.list_counter, s.list);
    if (a.out_counter && s.out) atomicAdd(a.out_counter, s.out);
  }
}

template <bool kWrite>
__global__ void __launch_bounds__(256) k_neighbours(DensityArgs a) {
  // single-pass write (cap_base set): the list of an item starts at
  // cap_base[item], its candidate-list length being a bound; the kernel also
  // writes the count and the list start (cap_loff)
  const bool single = kWrite && a.cap_base != nullptr;
  __shared__ BlockStats bs;
  if (!kWrite || single) block_stats_begin(bs);
  unsigned long long n_len = 0, n_out = 0;  // the warp's list length and entries written
  [&] {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= a.nwarps) return;
  const unsigned lane = lane_id();
  int si;
  long long i;
  locate(a, w, si, i);
  const SubDesc& S = a.subs[si];
  const long long item = S.item_off + i;
  const bool level1 = S.parent < 0;
  const int D = S.dim;
  if (!GUARD_OK(a.guard, level1 || S.query_off + i < a.prev_nkeep, 21, S.query_off + i)) return;
  const int p = level1 ? (int)i : a.prev_keep[S.query_off + i];
  if (!GUARD_OK(a.guard, p >= 0 && p < a.n, 22, p)) return;
  const float xp = a.X[(size_t)p * a.d + D];
  const int fp = a.fc[(size_t)p * a.d + D];
  const int* ids = nullptr;
  const int2* ents = nullptr;
  long long len;
  if (level1) {
    long long b = a.cand_off[(size_t)D * a.G + fp], e = a.cand_off[(size_t)D * a.G + fp + 1];
    ids = a.cand_pts + b;
    len = e - b;
  } else {
    long long b = a.prev_loff[S.query_off + i];
    ents = a.prev_ent + b;
    len = a.prev_lcnt[S.query_off + i];
    if (!GUARD_OK(a.guard, b >= 0 && len >= 0 && b + len <= a.prev_total, 23, b + len)) return;
  }
  int count = 0;
  const long long wbase = single ? a.cap_base[item] : kWrite ? a.loff[item] : 0;
  for (long long j0 = 0; j0 < len; j0 += 32) {
    long long j = j0 + lane;
    bool ok = j < len;
    const int2 e = ok && !level1 ? ents[j] : make_int2(-1, 0);
    int q = ok ? (level1 ? ids[j] : e.x) : -1;
    if (ok && !GUARD_OK(a.guard, q >= 0 && q < a.n, 24, q)) ok = false;
    ok = ok && q != p;
    if (ok && !level1 && S.win) {
      int fq = a.fc[(size_t)q * a.d + D];
      ok = fq >= fp - 1 && fq <= fp + 1;
    }
    float acc2 = 0.f;
    if (ok) {
      float acc = level1 ? 0.f : __int_as_float(e.y);
      acc2 = dist_step(acc, xp, a.X[(size_t)q * a.d + D]);
      ok = acc2 <= a.acc_max;
    }
    unsigned m = __ballot_sync(0xffffffffu, ok);
    if (kWrite && ok) {
      long long o = wbase + count + __popc(m & lanemask_lt());
      if (GUARD_OK(a.guard, o >= 0 && o < a.total, 25, o)) a.ent[o] = make_int2(q, __float_as_int(acc2));
    }
    count += __popc(m);
  }
  if ((!kWrite || single) && lane == 0) {
    a.cnt[item] = count;
    if (single) a.cap_loff[item] = wbase;
  }
  n_len = (unsigned long long)len;
  n_out = (unsigned long long)count;
  }();
  if (!kWrite || single) block_stats_end(bs, a, n_len, n_len, single ? n_out : 0);
}

// Levels >= 2: every child subspace of a parent filters the same parent list
// of p, so one warp per (parent, p) reads that list once and tests each
// candidate against all children (the candidate's row of X and of the fine
// cells is loaded once).  Lane c keeps the running count of child c (and
// c + 32).
template <bool kWrite>
__global__ void __launch_bounds__(256, 4) k_neighbours_multi(DensityArgs a) {
  const bool single = kWrite && a.cap_base != nullptr;
  const bool stats = !kWrite || single;
  __shared__ BlockStats bs;
  __shared__ unsigned long long bs_out;
  if (stats) {
    if (threadIdx.x == 0) bs_out = 0;
    block_stats_begin(bs);
  }
  unsigned long long n_cand = 0, n_list = 0;
  [&] {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= a.nwarps) return;
  const unsigned lane = lane_id();
  int lo = 0, hi = a.ngroups - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (a.groups[mid].qwarp_off <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  const GroupDesc g = a.groups[lo];
  const long long i = w - g.qwarp_off;
  if (i < 0 || i >= g.nquery) return;  // unreachable when the offsets are consistent
  const int nc = g.nchild;
  const SubDesc& S0 = a.subs[g.sub_base];
  if (!GUARD_OK(a.guard, S0.query_off + i < a.prev_nkeep && nc <= 64, 31, S0.query_off + i)) return;
  const int p = a.prev_keep[S0.query_off + i];
  if (!GUARD_OK(a.guard, p >= 0 && p < a.n, 32, p)) return;
  const long long pb = a.prev_loff[S0.query_off + i];
  const int2* ents = a.prev_ent + pb;
  const long long len = a.prev_lcnt[S0.query_off + i];
  if (!GUARD_OK(a.guard, pb >= 0 && len >= 0 && pb + len <= a.prev_total, 33, pb + len)) return;
  const float* xrow_p = a.X + (size_t)p * a.d;
  const uint8_t* frow_p = a.fc + (size_t)p * a.d;
  int run0 = 0, run1 = 0;  // lane c: children c and c + 32
  long long ob0 = 0, ob1 = 0;
  if (single) {
    ob0 = a.cap_base[w] + (long long)lane * len;
    ob1 = a.cap_base[w] + (long long)(lane + 32) * len;
  } else if (kWrite) {
    if ((int)lane < nc) ob0 = a.loff[a.subs[g.sub_base + lane].item_off + i];
    if ((int)lane + 32 < nc) ob1 = a.loff[a.subs[g.sub_base + lane + 32].item_off + i];
  }
  for (long long j0 = 0; j0 < len; j0 += 32) {
    const long long j = j0 + lane;
    bool in = j < len;
    const int2 e = in ? ents[j] : make_int2(p, 0);
    int q = e.x;
    const float acc0 = __int_as_float(e.y);  // read before the id check, which may store
    if (in && !GUARD_OK(a.guard, q >= 0 && q < a.n, 34, q)) {
      in = false;
      q = p;
    }
    const float acc = in ? acc0 : 0.f;
    const float* xrow_q = a.X + (size_t)q * a.d;
    const uint8_t* frow_q = a.fc + (size_t)q * a.d;
    for (int c = 0; c < nc; ++c) {
      const SubDesc& Sc = a.subs[g.sub_base + c];
      const int D = Sc.dim;
      const int fp = frow_p[D];
      const int fq = frow_q[D];
      bool ok = in && q != p && (!Sc.win || (fq >= fp - 1 && fq <= fp + 1));
      float acc2 = 0.f;
      if (ok) {
        acc2 = dist_step(acc, xrow_p[D], xrow_q[D]);
        ok = acc2 <= a.acc_max;
      }
      const unsigned m = __ballot_sync(0xffffffffu, ok);
      if (!m) continue;
      if (kWrite) {
        const int owner = c & 31;
        long long base = __shfl_sync(0xffffffffu, c < 32 ? ob0 + run0 : ob1 + run1, owner);
        if (ok) {
          long long o = base + __popc(m & lanemask_lt());
          if (GUARD_OK(a.guard, o >= 0 && o < a.total, 35, o)) a.ent[o] = make_int2(q, __float_as_int(acc2));
        }
      }
      if ((int)lane == (c & 31)) {
        if (c < 32)
          run0 += __popc(m);
        else
          run1 += __popc(m);
      }
    }
  }
  if (!kWrite || single) {
    if ((int)lane < nc) {
      const long long item = a.subs[g.sub_base + lane].item_off + i;
      a.cnt[item] = run0;
      if (single) a.cap_loff[item] = ob0;
    }
    if ((int)lane + 32 < nc) {
      const long long item = a.subs[g.sub_base + lane + 32].item_off + i;
      a.cnt[item] = run1;
      if (single) a.cap_loff[item] = ob1;
    }
    n_cand = (unsigned long long)len * nc;
    n_list = (unsigned long long)len;
    if (single && a.out_counter) {
      int tot = ((int)lane < nc ? run0 : 0) + ((int)lane + 32 < nc ? run1 : 0);
      for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
      if (lane == 0 && tot) atomicAdd(&bs_out, (unsigned long long)tot);
    }
  }
  }();
  if (stats) {
    block_stats_end(bs, a, n_cand, n_list);  // its barrier also orders the adds to bs_out
    if (threadIdx.x == 0 && single && a.out_counter && bs_out) atomicAdd(a.out_counter, bs_out);
  }
}

// Levels >= 2 when d <= 32 (rows of kS = 16, 24 or 32 slots): the same tests and
// outputs as k_neighbours_multi, with
//   * the (group, query) pair read from its record (RowItem, resolved by
//     k_list_capacity), so a pair starts after one load instead of a search
//     and a chain of dependent loads;
//   * every candidate's row of coordinates (kS floats; the 16-byte quarters
//     below the first child's dim are skipped) loaded once into registers,
//     and the children walked by a loop over the kS dims unrolled at compile
//     time (a group's children extend the parent by the consecutive dims
//     d0 .. d0 + nc - 1, child c = dim d0 + c), so a
//     (candidate, child) test reads registers and one warp-uniform 16-byte
//     shared load (the query's coordinate and fine-cell window on that dim).
//     The +-1 fine-cell test is the equivalent interval test
//     lo_p <= x_q < hi_p, so no fine cell of the candidate is read;
//   * a software pipeline over the 32-candidate chunks of a list: the ids and
//     partial distances of chunk k + 2 and (kS = 16, 24; 32-slot rows take
//     too many registers to hold two) the rows of chunk k + 1 are loaded
//     while chunk k is tested;
//   * warps taking `chunk` (group, query) pairs at a time from a work counter,
//     so a warp whose list was short takes the next pair instead of idling
//     until the longest list of its block is done;
//   * in the single pass, one bounds check per (group, query) block: child c
//     writes at most len entries from its block's start.
// resident blocks per SM: 64 registers a thread for 16-slot rows, 85 for 24
// and 32
constexpr int rows_blocks_per_sm(int slots) { return slots == 16 ? 4 : 3; }
int rows_max_blocks_per_sm(int slots) { return rows_blocks_per_sm(slots); }

// kMode: 0 count, 1 write at the counted offsets (loff), 2 single-pass write
// at capacity offsets (cap_base)
template <int kMode, int kS>
__global__ void __launch_bounds__(256, rows_blocks_per_sm(kS)) k_neighbours_rows(DensityArgs a) {
  constexpr bool kWrite = kMode >= 1;
  constexpr int kQ = kS / 4;           // 16-byte quarters of a row
  constexpr bool kPre = kS <= 24;      // rows of the next chunk held in registers
  __shared__ float4 squery[8][kS];     // per warp and dim: the query's (x, lo, hi, -)
  // per warp: candidate tests, list entries read, entries written; added to
  // the global counters once when the warp exits (per-pair atomics on three
  // adjacent counters saturate one L2 slice)
  __shared__ unsigned long long sstat[8][3];
  const unsigned lane = lane_id();
  const unsigned lt = lanemask_lt();  // read once: the lanes below this one
  const int wb = (int)(threadIdx.x >> 5);
  constexpr bool single = kMode == 2;
  const float4* xrow4 = reinterpret_cast<const float4*>(a.xrow);
  const float4* qv = squery[wb];
  const float acc_max = a.acc_max;
  // lanes past the end of a list load row n of xrow, whose coordinates are
  // all 3.4e38: (x_p - 3.4e38)^2 overflows to +inf, so they pass no distance
  // test and need no flag of their own
  const int sentinel = a.n;
  if (lane == 0) sstat[wb][0] = sstat[wb][1] = sstat[wb][2] = 0;  // lane 0 alone touches them
  for (;;) {
    unsigned long long take = 0;
    if (lane == 0) take = atomicAdd(a.work, (unsigned long long)a.chunk);
    const long long w0 = (long long)__shfl_sync(0xffffffffu, take, 0);
    if (w0 >= a.nwarps) break;
    const long long w1 = w0 + a.chunk < a.nwarps ? w0 + a.chunk : a.nwarps;
    for (long long w = w0; w < w1; ++w) {
      const RowItem r = a.items[w];
      if (r.len < 0) continue;  // failed its checks (reported by the capacity kernel)
      const int p = r.p, nc = r.nc, D0 = r.d0;
      const long long len = r.len;
      const int2* ents = a.prev_ent + r.pb;
      // lane c: the work item of child c (read now, used after the list)
      const long long item_c = (int)lane < nc ? a.subs[r.sub_base + lane].item_off + r.i : 0;
      int run = 0;  // lane c: entries of child c so far
      long long ob = 0;
      if (single) {
        // child c writes at most len entries from cap_base[w] + c * len, so
        // one check of the pair's block bounds every write below
        const long long cb = a.cap_base[w];
        if (!GUARD_OK(a.guard, cb >= 0 && cb + (long long)nc * len <= a.total, 39, cb)) continue;
        ob = cb + (long long)lane * len;
      } else if (kWrite) {
        if ((int)lane < nc) ob = a.loff[item_c];
      }
      __syncwarp();  // the previous pair's reads of the query slot are done
      if (lane < (unsigned)kS) {
        const size_t t = (size_t)p * kS + lane;
        // a child without the fine-cell test gets the window (-inf, +inf)
        const int c = (int)lane - D0;
        const bool open = c >= 0 && c < nc && ((r.nowin >> c) & 1);
        squery[wb][lane] = open ? make_float4(a.xrow[t], __uint_as_float(0xff800000u), __uint_as_float(0x7f800000u), 0.f)
                                : make_float4(a.xrow[t], a.win[2 * t], a.win[2 * t + 1], 0.f);
      }
      // candidate j of the list, one 8-byte entry (lanes past the end stand
      // on the sentinel row); nothing reads the loaded values until load_row,
      // a chunk later
      auto fetch = [&](long long j, bool& in, int& q, float& acc) {
        in = j < len;
        const int2 e = in ? ents[j] : make_int2(sentinel, 0);
        q = e.x;
        acc = __int_as_float(e.y);
      };
      // the id is checked where it is first used: the load of its row
      auto load_row = [&](float4 (&x)[kQ], bool& in, int& q) {
        if (in && !GUARD_OK(a.guard, q >= 0 && q < a.n, 34, q)) {
          in = false;
          q = sentinel;
        }
#pragma unroll
        for (int t = 0; t < kQ; ++t)
          if (4 * t + 3 >= D0) x[t] = xrow4[(size_t)q * kQ + t];  // quarters below d0 are not read
      };
      const long long nchunks = (len + 31) >> 5;
      bool in_a = false, in_b = false;
      int q_a = sentinel, q_b = sentinel;
      float acc_a = 0.f, acc_b = 0.f;
      float4 xa[kQ], xb[kQ];  // xb: the next chunk's rows (kPre only)
#pragma unroll
      for (int t = 0; t < kQ; ++t) xa[t] = xb[t] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (nchunks > 0) {
        fetch(lane, in_a, q_a, acc_a);
        if (kPre) load_row(xa, in_a, q_a);
      }
      if (nchunks > 1) fetch(32 + lane, in_b, q_b, acc_b);
      __syncwarp();  // the query slot is visible to the whole warp
      for (long long k = 0; k < nchunks; ++k) {
        // chunk k + 1: rows in flight (kPre); chunk k + 2: ids and distances in flight
        if (kPre) {
          if (k + 1 < nchunks) load_row(xb, in_b, q_b);
        } else {
          load_row(xa, in_a, q_a);
        }
        const int q = q_a;
        const float acc = acc_a;
        in_a = in_b;
        q_a = q_b;
        acc_a = acc_b;
        if (k + 2 < nchunks) fetch(((k + 2) << 5) + lane, in_b, q_b, acc_b);
        float xq[kS];
#pragma unroll
        for (int t = 0; t < kQ; ++t) {
          xq[4 * t] = xa[t].x;
          xq[4 * t + 1] = xa[t].y;
          xq[4 * t + 2] = xa[t].z;
          xq[4 * t + 3] = xa[t].w;
        }
#pragma unroll
        for (int D = 0; D < kS; ++D) {
          const int c = D - D0;
          if (c < 0 || c >= nc) continue;  // warp-uniform
          const float4 v = qv[D];
          const float xd = xq[D];
          const float acc2 = dist_step(acc, v.x, xd);
          const bool ok = xd >= v.y && xd < v.z && acc2 <= acc_max;
          const unsigned m = __ballot_sync(0xffffffffu, ok);
          if (!m) continue;
          if (kWrite) {
            const long long base = __shfl_sync(0xffffffffu, ob + run, c);
            if (ok) {
              const long long o = base + __popc(m & lt);
              if (single || GUARD_OK(a.guard, o >= 0 && o < a.total, 35, o))
                a.ent[o] = make_int2(q, __float_as_int(acc2));
            }
          }
          if ((int)lane == c) run += __popc(m);
        }
        if (kPre) {
#pragma unroll
          for (int t = 0; t < kQ; ++t) xa[t] = xb[t];
        }
      }
      if (!kWrite || single) {
        int out = 0;
        if ((int)lane < nc) {
          a.cnt[item_c] = run;
          if (single) a.cap_loff[item_c] = ob;
          out = run;
        }
        for (int o = 16; o > 0; o >>= 1) out += __shfl_xor_sync(0xffffffffu, out, o);
        if (lane == 0) {
          sstat[wb][0] += (unsigned long long)len * nc;
          sstat[wb][1] += (unsigned long long)len;
          sstat[wb][2] += (unsigned long long)out;
        }
      }
    }
  }
  if ((!kWrite || single) && lane == 0) {
    if (a.cand_counter) atomicAdd(a.cand_counter, sstat[wb][0]);
    if (a.list_counter) atomicAdd(a.list_counter, sstat[wb][1]);
    if (single && a.out_counter) atomicAdd(a.out_counter, sstat[wb][2]);
  }
}

#ifdef __CUDACC__
// ---------------------------------------------------------------------------
// The same pass with the candidate rows gathered by the tensor memory
// accelerator.  Each warp owns kRB chunk buffers in shared memory; the rows of
// chunk j (32 candidates, by id) arrive in buffer j % kRB through eight
// cp.async.bulk.tensor tile::gather4 copies (four rows each, issued by lanes
// 0..7), counted in by that buffer's mbarrier, while the warp tests chunk
// j - kRB + 1 ... j - 1.  The candidates' ids and partial distances go to the
// buffer's side arrays when the copies are issued.  Tests, writes and outputs
// are those of k_neighbours_rows.
// ---------------------------------------------------------------------------
#ifndef INSCY_ROWS_TMA_BUFFERS16
#define INSCY_ROWS_TMA_BUFFERS16 3
#endif
__host__ __device__ constexpr int rows_tma_buffers(int kS) { return kS == 16 ? INSCY_ROWS_TMA_BUFFERS16 : 2; }
__host__ __device__ constexpr int rows_tma_blocks(int) { return 3; }
__host__ __device__ constexpr int rows_tma_smem(int kS) { return 8 * rows_tma_buffers(kS) * 32 * kS * 4; }
// an mbarrier wait gives up after this many polls (the copies of a chunk take
// microseconds), reports guard code 36 and stops the warp
constexpr int kMbarPolls = 1 << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity) {
  for (int it = 0; it < kMbarPolls; ++it) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_addr(m)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <int kMode, int kS>
__global__ void __launch_bounds__(256, rows_tma_blocks(kS))
    k_neighbours_rows_tma(DensityArgs a, const __grid_constant__ CUtensorMap rows) {
  constexpr bool kWrite = kMode >= 1;
  constexpr int kQ = kS / 4;
  constexpr int kRB = rows_tma_buffers(kS);
  constexpr int kChunkFloats = 32 * kS;
  constexpr uint32_t kChunkBytes = 32u * kS * 4u;
  extern __shared__ __align__(128) unsigned char rows_smem[];
  __shared__ __align__(8) uint64_t mbar[8][kRB];
  __shared__ int sq[8][kRB][32];      // per warp and buffer: the candidates' ids
  __shared__ float sacc[8][kRB][32];  // and their partial distances
  __shared__ float4 squery[8][kS];
  __shared__ unsigned long long sstat[8][3];
  const unsigned lane = lane_id();
  const unsigned lt = lanemask_lt();
  const int wb = (int)(threadIdx.x >> 5);
  constexpr bool single = kMode == 2;
  float* wrows = reinterpret_cast<float*>(rows_smem) + (size_t)wb * kRB * kChunkFloats;
  const float4* qv = squery[wb];
  const float acc_max = a.acc_max;
  const int sentinel = a.n;  // row n of the rows: coordinates 3.4e38, no test passes
  if (lane == 0) {
    sstat[wb][0] = sstat[wb][1] = sstat[wb][2] = 0;
    for (int b = 0; b < kRB; ++b)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&mbar[wb][b])), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  uint32_t ph = 0;  // bit b: the parity the next wait on buffer b waits for
  bool stuck = false;
  for (;;) {
    unsigned long long take = 0;
    if (lane == 0) take = atomicAdd(a.work, (unsigned long long)a.chunk);
    const long long w0 = (long long)__shfl_sync(0xffffffffu, take, 0);
    if (w0 >= a.nwarps) break;
    const long long w1 = w0 + a.chunk < a.nwarps ? w0 + a.chunk : a.nwarps;
    for (long long w = w0; w < w1 && !stuck; ++w) {
      const RowItem r = a.items[w];
      if (r.len < 0) continue;  // failed its checks (reported by the capacity kernel)
      const int p = r.p, nc = r.nc, D0 = r.d0;
      const long long len = r.len;
      const int2* ents = a.prev_ent + r.pb;
      const long long item_c = (int)lane < nc ? a.subs[r.sub_base + lane].item_off + r.i : 0;
      int run = 0;
      long long ob = 0;
      if (single) {
        const long long cb = a.cap_base[w];
        if (!GUARD_OK(a.guard, cb >= 0 && cb + (long long)nc * len <= a.total, 39, cb)) continue;
        ob = cb + (long long)lane * len;
      } else if (kWrite) {
        if ((int)lane < nc) ob = a.loff[item_c];
      }
      __syncwarp();  // the previous pair's reads of the query slot are done
      if (lane < (unsigned)kS) {
        const size_t t = (size_t)p * kS + lane;
        // a child without the fine-cell test gets the window (-inf, +inf)
        const int c = (int)lane - D0;
        const bool open = c >= 0 && c < nc && ((r.nowin >> c) & 1);
        squery[wb][lane] = open ? make_float4(a.xrow[t], __uint_as_float(0xff800000u), __uint_as_float(0x7f800000u), 0.f)
                                : make_float4(a.xrow[t], a.win[2 * t], a.win[2 * t + 1], 0.f);
      }
      const long long nchunks = (len + 31) >> 5;
      // entry of chunk j for this lane (lanes past the end: the sentinel)
      auto entry = [&](long long j) -> int2 {
        const long long k = (j << 5) + lane;
        return k < len ? ents[k] : make_int2(sentinel, 0);
      };
      int2 e_next = nchunks > 0 ? entry(0) : make_int2(sentinel, 0);
      // chunk j into buffer j % kRB: ids and distances to the side arrays,
      // then the rows by eight 4-row gathers
      auto issue = [&](long long j) {
        const int b = (int)(j % kRB);
        int q = e_next.x;
        if (q != sentinel && !GUARD_OK(a.guard, q >= 0 && q < a.n, 34, q)) q = sentinel;
        sq[wb][b][lane] = q;
        sacc[wb][b][lane] = __int_as_float(e_next.y);
        if (j + 1 < nchunks) e_next = entry(j + 1);
        const int g = (int)(lane & 7u) * 4;
        const int r0 = __shfl_sync(0xffffffffu, q, g), r1 = __shfl_sync(0xffffffffu, q, g + 1);
        const int r2 = __shfl_sync(0xffffffffu, q, g + 2), r3 = __shfl_sync(0xffffffffu, q, g + 3);
        uint64_t* mb = &mbar[wb][b];
        // the warp's reads of buffer b (generic proxy) before the copies
        // (async proxy) overwrite it
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (lane == 0)
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mb)), "r"(kChunkBytes)
                       : "memory");
        __syncwarp();
        if (lane < 8u) {
          float* dst = wrows + (size_t)b * kChunkFloats + (size_t)lane * 4 * kS;
          asm volatile(
              "cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::bytes"
              " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_addr(dst)),
              "l"(reinterpret_cast<uint64_t>(&rows)), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_addr(mb))
              : "memory");
        }
      };
      for (long long j = 0; j < nchunks && j < kRB; ++j) issue(j);
      __syncwarp();  // the query slot is visible to the whole warp
      long long k = 0;
      for (; k < nchunks; ++k) {
        const int b = (int)(k % kRB);
        // every lane polls; the warp goes on only if all of them saw the
        // copies land (the decision stays warp-uniform)
        if (!__all_sync(0xffffffffu, mbar_wait(&mbar[wb][b], (ph >> b) & 1u))) {
          if (lane == 0) GUARD_OK(a.guard, false, 36, k);
          stuck = true;
          break;
        }
        ph ^= 1u << b;
        const int q = sq[wb][b][lane];
        const float acc = sacc[wb][b][lane];
        const float4* xr = reinterpret_cast<const float4*>(wrows + (size_t)b * kChunkFloats + (size_t)lane * kS);
        float xq[kS];
#pragma unroll
        for (int t = 0; t < kQ; ++t) {
          if (4 * t + 3 >= D0) {
            const float4 x = xr[t];
            xq[4 * t] = x.x;
            xq[4 * t + 1] = x.y;
            xq[4 * t + 2] = x.z;
            xq[4 * t + 3] = x.w;
          } else {
            xq[4 * t] = xq[4 * t + 1] = xq[4 * t + 2] = xq[4 * t + 3] = 0.f;
          }
        }
#pragma unroll
        for (int D = 0; D < kS; ++D) {
          const int c = D - D0;
          if (c < 0 || c >= nc) continue;  // warp-uniform
          const float4 v = qv[D];
          const float xd = xq[D];
          const float acc2 = dist_step(acc, v.x, xd);
          const bool ok = xd >= v.y && xd < v.z && acc2 <= acc_max;
          const unsigned m = __ballot_sync(0xffffffffu, ok);
          if (!m) continue;
          if (kWrite) {
            const long long base = __shfl_sync(0xffffffffu, ob + run, c);
            if (ok) {
              const long long o = base + __popc(m & lt);
              if (single || GUARD_OK(a.guard, o >= 0 && o < a.total, 35, o))
                a.ent[o] = make_int2(q, __float_as_int(acc2));
            }
          }
          if ((int)lane == c) run += __popc(m);
        }
        __syncwarp();  // every lane has read buffer b
        if (k + kRB < nchunks) issue(k + kRB);
      }
      if (stuck) {
        // the copies still in flight land before the warp leaves
        for (long long j = k; j < nchunks && j < k + kRB; ++j) {
          const int b = (int)(j % kRB);
          if (mbar_wait(&mbar[wb][b], (ph >> b) & 1u)) ph ^= 1u << b;
        }
        break;
      }
      if (!kWrite || single) {
        int out = 0;
        if ((int)lane < nc) {
          a.cnt[item_c] = run;
          if (single) a.cap_loff[item_c] = ob;
          out = run;
        }
        for (int o = 16; o > 0; o >>= 1) out += __shfl_xor_sync(0xffffffffu, out, o);
        if (lane == 0) {
          sstat[wb][0] += (unsigned long long)len * nc;
          sstat[wb][1] += (unsigned long long)len;
          sstat[wb][2] += (unsigned long long)out;
        }
      }
    }
    if (stuck) break;
  }
  if ((!kWrite || single) && lane == 0) {
    if (a.cand_counter) atomicAdd(a.cand_counter, sstat[wb][0]);
    if (a.list_counter) atomicAdd(a.list_counter, sstat[wb][1]);
    if (single && a.out_counter) atomicAdd(a.out_counter, sstat[wb][2]);
  }
}
#endif  // __CUDACC__


// single-pass list capacity of every (group, query): children x the query's
// parent-list length; with `a.items`, also the pair's record for the row
// kernel (query point, parent list, children), checked here once
__global__ void k_list_capacity(DensityArgs a, long long* __restrict__ cap) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= a.nwarps) return;
  int lo = 0, hi = a.ngroups - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (a.groups[mid].qwarp_off <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  const GroupDesc g = a.groups[lo];
  const long long i = w - g.qwarp_off;
  const long long k = a.subs[g.sub_base].query_off + i;
  long long len = 0;
  const bool ok = GUARD_OK(a.guard, i >= 0 && i < g.nquery && k < a.prev_nkeep, 36, k);
  if (ok) len = a.prev_lcnt[k];
  cap[w] = (long long)g.nchild * len;
  if (!a.items) return;
  RowItem r;
  r.pb = 0;
  r.len = -1;
  r.p = 0;
  r.sub_base = g.sub_base;
  r.i = (int)i;
  r.d0 = (short)a.subs[g.sub_base].dim;
  r.nc = (short)g.nchild;
  r.nowin = g.nowin;
  if (ok) {
    const int p = a.prev_keep[k];
    const long long pb = a.prev_loff[k];
    const int nc = g.nchild, d0 = a.subs[g.sub_base].dim;
    if (GUARD_OK(a.guard,
                 d0 >= 0 && nc >= 1 && d0 + nc <= a.slots && a.subs[g.sub_base + nc - 1].dim == d0 + nc - 1, 37,
                 d0) &&
        GUARD_OK(a.guard, p >= 0 && p < a.n, 32, p) &&
        GUARD_OK(a.guard, pb >= 0 && len >= 0 && pb + len <= a.prev_total, 33, pb + len)) {
      r.pb = pb;
      r.len = (int)len;
      r.p = p;
    }
  }
  a.items[w] = r;
}

// level 1: the capacity of item (subspace {D}, point p) is the length of the
// candidate list of p's fine cell on D
__global__ void k_level1_capacity(DensityArgs a, long long* __restrict__ cap) {
  const long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= a.nitems) return;
  const SubDesc& S = a.subs[find_sub(a.subs, a.nsubs, it)];
  const long long i = it - S.item_off;
  long long len = 0;
  if (GUARD_OK(a.guard, S.parent < 0 && i >= 0 && i < a.n, 38, i)) {
    const size_t c = (size_t)S.dim * a.G + a.fc[(size_t)i * a.d + S.dim];
    len = a.cand_off[c + 1] - a.cand_off[c];
  }
  cap[it] = len;
}

static DensityArgs make_args(const DensityLaunch& L);

void launch_level1_capacity(const DensityLaunch& L, long long* cap, cudaStream_t s) {
  if (L.nitems <= 0) return;
  DensityArgs a = make_args(L);
  k_level1_capacity<<<(unsigned)((L.nitems + 255) / 256), 256, 0, s>>>(a, cap);
}

// Density of every (subspace, point) from its list, in two kernels:
//
// k_density_phi: the phi sum of one item is sequential, so each lane walks
// its own list, and all busy lanes of a warp advance together for as many
// entries as the shortest remaining list allows.  Lists differ a lot in
// length, so (1) the items are taken in the order of a permutation that
// groups them by list length (half-octave classes, longest first: the lanes
// of a warp hold lists of similar length, and the longest start first), and
// (2) lanes are refilled as they finish: the warps are persistent and take
// batches of 32 consecutive positions of the permutation (the first one by a
// fixed spread over the blocks, the rest from a work counter),
// one item's (length, list start) per lane, handed to the lanes that need one
// by shuffles; a warp stops taking batches once the counter has passed the
// last position and finishes the items its lanes hold.
//
// k_density_flags: one thread per item turns the sum (or, for rectangular
// density, the neighbour count) into the weak / dense / keep flags and sets
// the point's bits in the subspace's bitmaps: the items of a warp are
// consecutive, so the points that share a bitmap word are adjacent lanes,
// and one lane per word ORs their bits in.
constexpr int kPhiBlocksPerSM = 6;
constexpr int kPhiClasses = 64;  // list-length classes of the permutation

// class of a list of length c: two per octave of c + 1, longest first
__device__ __forceinline__ int phi_class(int c) {
  const unsigned v = (unsigned)c + 1u;
  const int lg = 31 - __clz((int)v);
  const int half = lg >= 1 ? (int)((v >> (lg - 1)) & 1u) : 0;
  const int k = 2 * lg + half;
  return kPhiClasses - 1 - (k < kPhiClasses - 1 ? k : kPhiClasses - 1);
}

// per-class item counts (hist[kPhiClasses], zeroed by the caller)
__global__ void k_phi_class_count(const int* __restrict__ cnt, long long nitems, int* __restrict__ hist) {
  __shared__ int local[kPhiClasses];
  if (threadIdx.x < kPhiClasses) local[threadIdx.x] = 0;
  __syncthreads();
  const long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (it < nitems) atomicAdd(&local[phi_class(cnt[it])], 1);
  __syncthreads();
  if (threadIdx.x < kPhiClasses && local[threadIdx.x]) atomicAdd(&hist[threadIdx.x], local[threadIdx.x]);
}

// class starts: cursor[k] = items of the classes before k (one block)
__global__ void k_phi_class_starts(const int* __restrict__ hist, int* __restrict__ cursor) {
  if (threadIdx.x == 0) {
    int o = 0;
    for (int k = 0; k < kPhiClasses; ++k) {
      cursor[k] = o;
      o += hist[k];
    }
  }
}

// scatter the items into their classes (the order within a class is free:
// every item's sum is stored at its own index)
__global__ void k_phi_class_scatter(const int* __restrict__ cnt, long long nitems, int* __restrict__ cursor,
                                    int* __restrict__ perm) {
  __shared__ int local[kPhiClasses], base[kPhiClasses];
  if (threadIdx.x < kPhiClasses) local[threadIdx.x] = 0;
  __syncthreads();
  const long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int k = it < nitems ? phi_class(cnt[it]) : 0;
  const int r = it < nitems ? atomicAdd(&local[k], 1) : 0;
  __syncthreads();
  if (threadIdx.x < kPhiClasses && local[threadIdx.x]) base[threadIdx.x] = atomicAdd(&cursor[threadIdx.x], local[threadIdx.x]);
  __syncthreads();
  if (it < nitems) perm[base[k] + r] = (int)it;
}

__global__ void __launch_bounds__(256, kPhiBlocksPerSM) k_density_phi(DensityArgs a, const int* __restrict__ perm,
                                                                       float* __restrict__ phi) {
  const unsigned lane = lane_id();
  const long long nitems = a.nitems;
  // the current batch: positions bbase .. bbase + 31 of the permutation, lane
  // l holding the item at bbase + l (bi) and its list; positions below bpos
  // are handed out
  long long bbase = 0;
  int bc = 0, bpos = 32, bi = 0;
  long long bl = 0;
  bool drained = false;  // the counter has passed the last item (warp-uniform)
  // the first batch of warp i of block b is batch i * gridDim.x + b, so the
  // longest lists (the first batches) spread over the blocks and thus the
  // SMs; later batches come from the counter, after the first gridDim.x * 8
  bool first = true;
  auto new_batch = [&]() {
    long long batch;
    if (first) {
      batch = (long long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x;
      first = false;
    } else {
      unsigned long long t = 0;
      if (lane == 0) t = atomicAdd(a.work, 1ull);
      batch = (long long)__shfl_sync(0xffffffffu, t, 0) + (long long)gridDim.x * (blockDim.x >> 5);
    }
    bbase = batch * 32;
    drained = bbase + 32 >= nitems;
    const long long pos = bbase + lane;
    bi = pos < nitems ? perm[pos] : 0;
    bc = pos < nitems ? a.cnt[bi] : 0;
    bl = pos < nitems ? a.loff[bi] : 0;
    bpos = 0;
  };
  long long item = 0;
  const int2* acc = nullptr;  // the item's list entries
  int c = 0, j = 0;
  float sum = 0.f;
  // phi is only compared with the weak, dense and keep thresholds
  // (k_density_flags; keep <= weak), and the sum never decreases (every term
  // 1 - sq >= 0, each rounding monotone): once it reaches the larger of the
  // weak and the subspace's dense threshold every flag is decided, and the
  // partial sum is stored
  float stop = 0.f;
  bool live = false;  // this lane holds an item whose sum is still to be stored
  // hand the next items of the queue to the lanes in `need`, in lane order
  auto hand_out = [&](unsigned need) {
    const int k = __popc(need & lanemask_lt());
    const int tot = __popc(need);
    const int avail = 32 - bpos;
    const bool cur = k < avail;  // from the current batch, else from the next one
    const int s0 = cur ? bpos + k : 0;
    const int c0 = __shfl_sync(0xffffffffu, bc, s0);
    const long long l0 = __shfl_sync(0xffffffffu, bl, s0);
    const int x0 = __shfl_sync(0xffffffffu, bi, s0);
    const bool v0 = bbase + s0 < nitems;
    int c1 = 0, x1 = 0;
    long long l1 = 0;
    bool v1 = false;
    if (tot > avail) {
      if (!drained) {
        new_batch();
        const int s1 = cur ? 0 : k - avail;
        c1 = __shfl_sync(0xffffffffu, bc, s1);
        l1 = __shfl_sync(0xffffffffu, bl, s1);
        x1 = __shfl_sync(0xffffffffu, bi, s1);
        v1 = bbase + s1 < nitems;
        bpos = tot - avail;
      } else {
        bpos = 32;
      }
    } else {
      bpos += tot;
    }
    if ((need >> lane) & 1u) {
      item = cur ? x0 : x1;
      c = cur ? c0 : c1;
      const long long lo = cur ? l0 : l1;
      live = (cur ? v0 : v1) && GUARD_OK(a.guard, c >= 0 && lo >= 0 && lo + c <= a.total, 41, lo + c);
      acc = a.ent + lo;
      j = 0;
      sum = 0.f;
      if (live) {
        const float td = a.thr_dense[a.subs[find_sub(a.subs, a.nsubs, item)].nsub];
        stop = td > a.thr_weak ? td : a.thr_weak;
      }
    }
  };
  new_batch();
  hand_out(0xffffffffu);
  for (;;) {
    if (!__any_sync(0xffffffffu, live)) break;
    // steps every busy lane can take: the shortest remaining list, at most
    // 128 so that lanes whose sums stop early are refilled soon
    int steps = live ? c - j : INT_MAX;
    for (int o = 16; o > 0; o >>= 1) steps = min(steps, __shfl_xor_sync(0xffffffffu, steps, o));
    steps = min(steps, 128);
    if (live) {
      // the terms do not depend on the sum: four at a time are loaded and
      // computed side by side, then added in order (the sum's chain alone is
      // sequential)
      const int2* ap = acc + j;
      int t = 0;
      bool hit = sum >= stop;
      for (; !hit && t + 4 <= steps; t += 4) {
        const float a0 = __int_as_float(ap[t].y), a1 = __int_as_float(ap[t + 1].y);
        const float a2 = __int_as_float(ap[t + 2].y), a3 = __int_as_float(ap[t + 3].y);
        const float d0 = __fdiv_rn(__fsqrt_rn(a0), a.eps), d1 = __fdiv_rn(__fsqrt_rn(a1), a.eps);
        const float d2 = __fdiv_rn(__fsqrt_rn(a2), a.eps), d3 = __fdiv_rn(__fsqrt_rn(a3), a.eps);
        sum = phi_step_exact(sum, __fmul_rn(d0, d0));  // integer pipe, no FP64
        sum = phi_step_exact(sum, __fmul_rn(d1, d1));
        sum = phi_step_exact(sum, __fmul_rn(d2, d2));
        sum = phi_step_exact(sum, __fmul_rn(d3, d3));
        hit = sum >= stop;
      }
      for (; !hit && t < steps; ++t) {
        const float dd = __fdiv_rn(__fsqrt_rn(__int_as_float(ap[t].y)), a.eps);
        sum = phi_step_exact(sum, __fmul_rn(dd, dd));
        hit = sum >= stop;
      }
      j = hit ? c : j + steps;
    }
    const bool done = live && j >= c;
    if (done) {
      phi[item] = sum;
      live = false;
    }
    // lanes without an item ask for one while the queue lasts
    const bool more = !(drained && bpos >= 32) ;
    const unsigned need = __ballot_sync(0xffffffffu, more && !live);
    if (need) hand_out(need);
  }
}

__global__ void __launch_bounds__(256) k_density_flags(DensityArgs a, const float* __restrict__ phi) {
  const long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if ((it & ~31LL) >= a.nitems) return;  // whole warps
  const unsigned lane = lane_id();
  const bool valid = it < a.nitems;
  const long long itc = valid ? it : a.nitems - 1;
  const int si = find_sub(a.subs, a.nsubs, itc);
  const SubDesc& S = a.subs[si];
  const long long i = itc - S.item_off;
  const int p = S.parent < 0 ? (int)i : a.prev_keep[S.query_off + i];
  uint8_t f = 0;
  if (valid && GUARD_OK(a.guard, p >= 0 && p < a.n, 42, p)) {
    const float v = a.rect ? (float)a.cnt[it] : phi[it];
    if (v >= a.thr_weak) f |= kFlagWeak;
    if (v >= a.thr_dense[S.nsub]) f |= kFlagDense;
    if (v >= a.thr_keep[S.nsub]) f |= kFlagKeep;
    a.flags[it] = f;
  }
  // the word of the point in its subspace's bitmaps; adjacent lanes share it
  // (items of a subspace ascend in point), so OR the bits over each run of
  // equal words and let the run's last lane store them
  const long long word = valid ? S.bitmap_off + (p >> 5) : -1 - (long long)lane;
  const unsigned bit = 1u << (p & 31);
  unsigned w = (f & kFlagWeak) ? bit : 0u, dn = (f & kFlagDense) ? bit : 0u, kp = (f & kFlagKeep) ? bit : 0u;
  for (int o = 1; o < 32; o <<= 1) {
    const long long wo = __shfl_up_sync(0xffffffffu, word, o);
    const unsigned a0 = __shfl_up_sync(0xffffffffu, w, o);
    const unsigned a1 = __shfl_up_sync(0xffffffffu, dn, o);
    const unsigned a2 = __shfl_up_sync(0xffffffffu, kp, o);
    if ((int)lane >= o && wo == word) {
      w |= a0;
      dn |= a1;
      kp |= a2;
    }
  }
  const long long wn = __shfl_sync(0xffffffffu, word, lane < 31 ? (int)lane + 1 : 31);
  if (valid && (lane == 31 || wn != word)) {
    unsigned* bm = a.bitmaps + word;
    if (w) atomicOr(bm, w);
    if (dn) atomicOr(bm + a.words, dn);
    if (kp) atomicOr(bm + 2 * a.words, kp);
  }
}

// kept items: list lengths (0 for the others) for the offset scan
__global__ void k_keep_counts(const int* __restrict__ cnt, const uint8_t* __restrict__ flags, long long nitems,
                              int* __restrict__ kcnt, int* __restrict__ kflag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nitems) return;
  bool k = flags[i] & kFlagKeep;
  kcnt[i] = k ? cnt[i] : 0;
  kflag[i] = k ? 1 : 0;
}

// compact the kept items into the level's kept-point arrays
__global__ void k_keep_compact(const SubDesc* __restrict__ subs, int nsubs, long long nitems,
                               const uint8_t* __restrict__ flags, const int* __restrict__ cnt,
                               const long long* __restrict__ kpos, const long long* __restrict__ loff,
                               const int* __restrict__ prev_keep, int* __restrict__ keep_ids,
                               long long* __restrict__ keep_loff, int* __restrict__ keep_lcnt) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nitems) return;
  if (!(flags[i] & kFlagKeep)) return;
  int si = find_sub(subs, nsubs, i);
  const SubDesc& S = subs[si];
  long long li = i - S.item_off;
  int p = S.parent < 0 ? (int)li : prev_keep[S.query_off + li];
  long long k = kpos[i];
  keep_ids[k] = p;
  keep_loff[k] = loff[i];
  keep_lcnt[k] = cnt[i];
}

// popcount of every bitmap word (for rank lookups in the keep bitmaps)
__global__ void k_word_popc(const unsigned* __restrict__ words, long long nw, int* __restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nw) out[i] = __popc(words[i]);
}

// popcount of the kept-bitmap words of every subspace (third bitmap of each)
__global__ void k_keep_popc(const unsigned* __restrict__ bm, int nsubs, int W, int* __restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nsubs * W) return;
  long long s = i / W, w = i % W;
  out[i] = __popc(bm[s * 3 * W + 2 * W + w]);
}

void launch_keep_popc(const unsigned* bm, int nsubs, int W, int* out, cudaStream_t s) {
  long long nw = (long long)nsubs * W;
  if (nw > 0) k_keep_popc<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(bm, nsubs, W, out);
}

// first kept index of every subspace: the kept-prefix at its first item
__global__ void k_gather_kstart(const SubDesc* __restrict__ subs, int nsubs, const long long* __restrict__ kpos,
                                long long nitems, long long K, long long* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nsubs) return;
  if (i == nsubs) {
    out[i] = K;
    return;
  }
  long long it = subs[i].item_off;
  out[i] = it < nitems ? kpos[it] : K;
}

// first component id of every subspace
__global__ void k_gather_cbase(const long long* __restrict__ kstart, int nsubs, const int* __restrict__ root_id,
                               long long K, int ncomp, int* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nsubs) return;
  long long k = kstart[i];
  out[i] = k < K ? root_id[k] : ncomp;
}

void launch_gather_kstart(const SubDesc* subs, int nsubs, const long long* kpos, long long nitems, long long K,
                          long long* out, cudaStream_t s) {
  k_gather_kstart<<<(nsubs + 1 + 255) / 256, 256, 0, s>>>(subs, nsubs, kpos, nitems, K, out);
}

void launch_gather_cbase(const long long* kstart, int nsubs, const int* root_id, long long K, int ncomp, int* out,
                         cudaStream_t s) {
  k_gather_cbase<<<(nsubs + 1 + 255) / 256, 256, 0, s>>>(kstart, nsubs, root_id, K, ncomp, out);
}

static DensityArgs make_args(const DensityLaunch& L) {
  DensityArgs a;
  a.subs = L.subs;
  a.nsubs = L.nsubs;
  a.nitems = L.nitems;
  a.groups = L.groups;
  a.ngroups = L.ngroups;
  a.nwarps = L.nitems;
  a.X = L.X;
  a.fc = L.fc;
  a.n = L.n;
  a.d = L.d;
  a.G = L.G;
  a.eps = L.eps;
  a.rect = L.rect;
  a.acc_max = L.acc_max;
  a.thr_weak = L.thr_weak;
  a.thr_dense = L.thr_dense;
  a.thr_keep = L.thr_keep;
  a.cand_off = L.cand_off;
  a.cand_pts = L.cand_pts;
  a.prev_keep = L.prev_keep;
  a.prev_loff = L.prev_loff;
  a.prev_lcnt = L.prev_lcnt;
  a.prev_ent = L.prev_ent;
  a.cnt = L.cnt;
  a.flags = L.flags;
  a.bitmaps = L.bitmaps;
  a.words = L.words;
  a.loff = L.loff;
  a.ent = L.ent;
  a.cand_counter = L.cand_counter;
  a.list_counter = L.list_counter;
  a.out_counter = L.out_counter;
  a.cap_base = L.cap_base;
  a.cap_loff = L.cap_loff;
  a.xrow = L.xrow;
  a.win = L.win;
  a.work = L.work;
  a.items = L.items;
  a.slots = L.slots;
  a.chunk = 1;
  a.prev_total = L.prev_total;
  a.total = L.total;
  a.prev_nkeep = L.prev_nkeep;
  a.guard = L.guard;
  return a;
}

void launch_neighbours(const DensityLaunch& L, bool write, cudaStream_t s) {
  if (L.nitems <= 0) return;
  DensityArgs a = make_args(L);
  unsigned blocks = (unsigned)((L.nitems * 32 + 255) / 256);
  if (write)
    k_neighbours<true><<<blocks, 256, 0, s>>>(a);
  else
    k_neighbours<false><<<blocks, 256, 0, s>>>(a);
}

// self-test: the integer phi step against the double-precision expression on
// pseudo-random and edge inputs; counts mismatches
__global__ void k_phi_selftest(unsigned long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long x = (i + 1) * 0x9e3779b97f4a7c15ull ^ seed;
  x ^= x >> 31;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  float sum;
  const int mode = (int)(x & 3);
  if (mode == 0)
    sum = (float)((x >> 8) % 100000);
  else if (mode == 1)
    sum = 0.f;
  else
    sum = __uint_as_float(((uint32_t)((int)((x >> 40) % 42) - 24 + 127) << 23) | ((uint32_t)(x >> 8) & 0x7fffffu));
  unsigned long long y = x * 0x94d049bb133111ebull;
  y ^= y >> 29;
  float sq;
  if (y & 1)
    sq = __uint_as_float((uint32_t)(y >> 8) % 0x3f800001u);
  else {
    float dd = (float)((y >> 11) * 0x1p-53);
    sq = __fmul_rn(dd, dd);
  }
  if (sq > 1.f) sq = 1.f;
  if (__float_as_uint(phi_step_exact(sum, sq)) != __float_as_uint(phi_step_double(sum, sq))) atomicAdd(bad, 1ull);
}

void launch_phi_selftest(unsigned long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t s) {
  k_phi_selftest<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, seed, bad);
}

#ifdef __CUDACC__
// The row table as a 2-d tensor of n + 1 rows of `slots` floats (the last
// row is the sentinel), read one row per box by tile::gather4 copies.
static bool rows_tensor_map(CUtensorMap* tm, const float* xrow, int n, int slots) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    encode = reinterpret_cast<Encode>(fn);
  }
  const cuuint64_t dims[2] = {(cuuint64_t)slots, (cuuint64_t)n + 1};
  const cuuint64_t strides[1] = {(cuuint64_t)slots * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)slots, 1};  // one row per box, as tile::gather4 takes it
  const cuuint32_t estr[2] = {1, 1};
  return encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(xrow), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int kMode, int kS>
static void rows_tma_kernel(const DensityArgs& a, const CUtensorMap& tm, unsigned blocks, cudaStream_t s) {
  static bool attr = false;  // the dynamic shared memory above 48 KB is opted into once
  if (!attr) {
    cudaFuncSetAttribute(k_neighbours_rows_tma<kMode, kS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         rows_tma_smem(kS));
    attr = true;
  }
  k_neighbours_rows_tma<kMode, kS><<<blocks, 256, rows_tma_smem(kS), s>>>(a, tm);
}

// The row kernel with TMA-gathered rows; false when the tensor map cannot be
// made (the caller then launches k_neighbours_rows).
static bool rows_tma_launch(const DensityLaunch& L, DensityArgs& a, long long nwarps, bool write, cudaStream_t s) {
  CUtensorMap tm;
  if (!rows_tensor_map(&tm, L.xrow, L.n, L.slots)) return false;
  const long long max_blocks = (long long)(L.sms > 0 ? L.sms : 1) * rows_tma_blocks(L.slots);
  long long chunk = nwarps / (max_blocks * 8 * 16);
  a.chunk = (int)(chunk < 1 ? 1 : chunk > 8 ? 8 : chunk);
  const long long need = (nwarps + 7) / 8;
  const unsigned blocks = (unsigned)(need < max_blocks ? need : max_blocks);
  const int mode = write ? (L.cap_base ? 2 : 1) : 0;
  if (L.slots == 16) {
    if (mode == 2) rows_tma_kernel<2, 16>(a, tm, blocks, s);
    else if (mode == 1) rows_tma_kernel<1, 16>(a, tm, blocks, s);
    else rows_tma_kernel<0, 16>(a, tm, blocks, s);
  } else if (L.slots == 24) {
    if (mode == 2) rows_tma_kernel<2, 24>(a, tm, blocks, s);
    else if (mode == 1) rows_tma_kernel<1, 24>(a, tm, blocks, s);
    else rows_tma_kernel<0, 24>(a, tm, blocks, s);
  } else {
    if (mode == 2) rows_tma_kernel<2, 32>(a, tm, blocks, s);
    else if (mode == 1) rows_tma_kernel<1, 32>(a, tm, blocks, s);
    else rows_tma_kernel<0, 32>(a, tm, blocks, s);
  }
  return true;
}
#endif

// level >= 2: one warp per (parent group, query point)
void launch_neighbours_multi(const DensityLaunch& L, long long nwarps, bool write, cudaStream_t s) {
  if (nwarps <= 0) return;
  DensityArgs a = make_args(L);
  a.nwarps = nwarps;
#ifdef __CUDACC__
  if (L.rows_tma && L.xrow && L.win && L.work && L.items && (L.slots == 16 || L.slots == 24 || L.slots == 32) &&
      L.d <= L.slots && rows_tma_launch(L, a, nwarps, write, s))
    return;
#endif
  if (L.xrow && L.win && L.work && L.items && (L.slots == 16 || L.slots == 24 || L.slots == 32) && L.d <= L.slots) {
    // persistent warps: a grid that fills every SM once, (group, query) pairs
    // handed out by the work counter, several per update when there are many
    const int bps_max = rows_blocks_per_sm(L.slots);
    const int bps = L.rows_bps > 0 && L.rows_bps < bps_max ? L.rows_bps : bps_max;
    const long long max_blocks = (long long)(L.sms > 0 ? L.sms : 1) * bps;
    // pairs per counter update: about `takes` updates per warp over the launch
    const long long takes = L.rows_takes > 0 ? L.rows_takes : 16;
    long long chunk = nwarps / (max_blocks * 8 * takes);
    a.chunk = (int)(chunk < 1 ? 1 : chunk > 64 ? 64 : chunk);
    const long long need = (nwarps + 7) / 8;
    const unsigned blocks = (unsigned)(need < max_blocks ? need : max_blocks);
    const int mode = write ? (L.cap_base ? 2 : 1) : 0;
    if (L.slots == 16) {
      if (mode == 2)
        k_neighbours_rows<2, 16><<<blocks, 256, 0, s>>>(a);
      else if (mode == 1)
        k_neighbours_rows<1, 16><<<blocks, 256, 0, s>>>(a);
      else
        k_neighbours_rows<0, 16><<<blocks, 256, 0, s>>>(a);
    } else if (L.slots == 24) {
      if (mode == 2)
        k_neighbours_rows<2, 24><<<blocks, 256, 0, s>>>(a);
      else if (mode == 1)
        k_neighbours_rows<1, 24><<<blocks, 256, 0, s>>>(a);
      else
        k_neighbours_rows<0, 24><<<blocks, 256, 0, s>>>(a);
    } else {
      if (mode == 2)
        k_neighbours_rows<2, 32><<<blocks, 256, 0, s>>>(a);
      else if (mode == 1)
        k_neighbours_rows<1, 32><<<blocks, 256, 0, s>>>(a);
      else
        k_neighbours_rows<0, 32><<<blocks, 256, 0, s>>>(a);
    }
    return;
  }
  unsigned blocks = (unsigned)((nwarps * 32 + 255) / 256);
  if (write)
    k_neighbours_multi<true><<<blocks, 256, 0, s>>>(a);
  else
    k_neighbours_multi<false><<<blocks, 256, 0, s>>>(a);
}

void launch_list_capacity(const DensityLaunch& L, long long nwarps, long long* cap, cudaStream_t s) {
  if (nwarps <= 0) return;
  DensityArgs a = make_args(L);
  a.nwarps = nwarps;
  k_list_capacity<<<(unsigned)((nwarps + 255) / 256), 256, 0, s>>>(a, cap);
}

void launch_density_flags(const DensityLaunch& L, float* phi, int* perm, cudaStream_t s) {
  if (L.nitems <= 0) return;
  DensityArgs a = make_args(L);
  if (!L.rect) {  // rectangular density compares the neighbour count: no sum
    a.work = L.phi_work;
    int* hist = reinterpret_cast<int*>(L.phi_work + 1);  // kPhiClasses counts, then kPhiClasses cursors
    const unsigned iblocks = (unsigned)((L.nitems + 255) / 256);
    k_phi_class_count<<<iblocks, 256, 0, s>>>(L.cnt, L.nitems, hist);
    k_phi_class_starts<<<1, 32, 0, s>>>(hist, hist + kPhiClasses);
    k_phi_class_scatter<<<iblocks, 256, 0, s>>>(L.cnt, L.nitems, hist + kPhiClasses, perm);
    const long long need = (L.nitems + 255) / 256;  // one 32-item batch per warp
    const long long cap = (long long)(L.sms > 0 ? L.sms : 1) * kPhiBlocksPerSM;
    const unsigned blocks = (unsigned)(need < cap ? need : cap);
    k_density_phi<<<blocks, 256, 0, s>>>(a, perm, phi);
  }
  k_density_flags<<<(unsigned)((L.nitems + 255) / 256), 256, 0, s>>>(a, phi);
}

void launch_keep_counts(const int* cnt, const uint8_t* flags, long long nitems, int* kcnt, int* kflag,
                        cudaStream_t s) {
  if (nitems <= 0) return;
  k_keep_counts<<<(unsigned)((nitems + 255) / 256), 256, 0, s>>>(cnt, flags, nitems, kcnt, kflag);
}

void launch_keep_compact(const SubDesc* subs, int nsubs, long long nitems, const uint8_t* flags, const int* cnt,
                         const long long* kpos, const long long* loff, const int* prev_keep, int* keep_ids,
                         long long* keep_loff, int* keep_lcnt, cudaStream_t s) {
  if (nitems <= 0) return;
  k_keep_compact<<<(unsigned)((nitems + 255) / 256), 256, 0, s>>>(subs, nsubs, nitems, flags, cnt, kpos, loff,
                                                                  prev_keep, keep_ids, keep_loff, keep_lcnt);
}

void launch_word_popc(const unsigned* words, long long nw, int* out, cudaStream_t s) {
  if (nw <= 0) return;
  k_word_popc<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(words, nw, out);
}

}  // namespace inscy
