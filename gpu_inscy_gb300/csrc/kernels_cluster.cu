// Clustering of the subspaces of one level (INSCYClusteringImplCPUAll,
// ClusteringCpu.cu:317-389, re-derived).
//
// The reference runs a BFS from every region point in leaf order: a dense
// point joins the current cluster and enqueues its unvisited neighbours
// (marking them -2), a non-dense point ends the branch.  Since the neighbour
// relation is symmetric and density is a pure function of (point, subspace),
// the outcome is:
//   * clusters  = connected components of the dense points under the
//                 neighbour relation, numbered in the order in which the
//                 region's leaf order first meets a dense point of each;
//   * -2 marks  = non-dense points adjacent to a dense point of a numbered
//                 component.
// So the GPU computes, per subspace, the components (lock-free atomicCAS
// union-find with pointer jumping), per component its members and its
// non-dense border points, and per region the components in first-seed order.
// The host then numbers them exactly as the BFS does.
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "inscy_common.cuh"
#include "inscy_prims.cuh"
#include "inscy_kernels.h"

namespace inscy {

constexpr int kUnionLimit = 1 << 22;  // bound on CAS retries of one union

__device__ __forceinline__ bool bit_of(const unsigned* bm, int p) { return (bm[p >> 5] >> (p & 31)) & 1u; }

// global keep index of point q in subspace si (rank in its keep bitmap)
__device__ __forceinline__ long long keep_index(const ClusterArgs& a, int si, int q) {
  const unsigned* kb = a.bitmaps + a.subs[si].bitmap_off + 2LL * a.words;
  unsigned wv = kb[q >> 5];
  return (long long)a.keep_word_rank[(long long)si * a.words + (q >> 5)] + __popc(wv & ((1u << (q & 31)) - 1u));
}

__device__ __forceinline__ int find_sub_by_keep(const long long* kstart, int nsubs, long long kk) {
  int lo = 0, hi = nsubs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (kstart[mid] <= kk)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int uf_find(int* par, int x) {
  volatile int* vp = par;
  int cur = x;
  int next = vp[cur];
  int guard = 0;
  while (next != cur) {
    int nn = vp[next];
    if (nn != next) vp[cur] = nn;  // path halving: only ever points closer to the root
    cur = next;
    next = vp[cur];
    if (++guard > kUnionLimit) break;
  }
  return cur;
}

// unite the trees of roots-or-nodes ra and rb
__device__ __forceinline__ void uf_unite(int* par, int ra, int rb, int* err) {
  int it = 0;
  while (ra != rb) {
    if (ra < rb) {
      int t = ra;
      ra = rb;
      rb = t;
    }
    int old = atomicCAS(&par[ra], ra, rb);  // hook the larger root under the smaller
    if (old == ra) return;
    ra = uf_find(par, old);
    rb = uf_find(par, rb);
    if (++it > kUnionLimit) {
      atomicExch(err, 3);
      return;
    }
  }
}

// the subspace of every kept point (its kept index lies in the subspace's
// range [kstart[si], kstart[si + 1])), looked up by the clustering kernels
__global__ void k_sub_of_keep(const long long* __restrict__ kstart, int nsubs, long long nkeep, int* __restrict__ sub_of) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk < nkeep) sub_of[kk] = find_sub_by_keep(kstart, nsubs, kk);
}

void launch_sub_of_keep(const long long* kstart, int nsubs, long long nkeep, int* sub_of, cudaStream_t s) {
  if (nkeep > 0) k_sub_of_keep<<<(unsigned)((nkeep + 255) / 256), 256, 0, s>>>(kstart, nsubs, nkeep, sub_of);
}

__global__ void k_uf_init(int* par, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) par[i] = (int)i;
}

// Connected components of the dense points of every clustered subspace, in
// the Afforest order: (1) every dense point is united with its first two dense
// neighbours; (2) per subspace, the component most of 32 sampled dense points
// fall in is taken as the dominant one; (3) only points outside the dominant
// component (checked when they are processed) unite with all their dense
// neighbours.  Every edge that is skipped joins two points that were both in
// the dominant component at some time, and components only grow, so the final
// partition is the connected components of the full neighbour relation.
// That holds for any number of links in (1): INSCY_UF_LINKS = 0 (a build for
// the host tests) leaves every edge but the sampled point's to (3).
#ifndef INSCY_UF_LINKS
#define INSCY_UF_LINKS 2
#endif

// (1) one thread per kept point
__global__ void __launch_bounds__(256) k_uf_link2(ClusterArgs a) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= a.nkeep) return;
  const int si = a.sub_of[kk];
  if (!a.clustered[si]) return;
  const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
  if (!bit_of(dn, a.keep_ids[kk])) return;
  const long long b = a.keep_loff[kk];
  const int len = a.keep_lcnt[kk];
  int linked = 0;
  for (int j = 0; j < len && linked < INSCY_UF_LINKS; ++j) {
    int q = a.ent[b + j].x;
    if (!GUARD_OK(a.guard, q >= 0 && q < a.n, 63, q) || !bit_of(dn, q)) continue;
    long long kq = keep_index(a, si, q);
    if (!GUARD_OK(a.guard, kq >= a.kstart[si] && kq < a.kstart[si + 1], 64, kq)) continue;
    uf_unite(a.uf, uf_find(a.uf, (int)kk), uf_find(a.uf, (int)kq), a.err);
    ++linked;
  }
}

// (1b) compress: every dense kept point points at its root, so the finds of
// the sampling and of the skip test in (3) take one step
__global__ void __launch_bounds__(256) k_uf_compress(ClusterArgs a) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= a.nkeep) return;
  const int si = a.sub_of[kk];
  if (!a.clustered[si]) return;
  const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
  if (!bit_of(dn, a.keep_ids[kk])) return;
  const int r = uf_find(a.uf, (int)kk);
  if (r != (int)kk) ((volatile int*)a.uf)[kk] = r;  // an ancestor: finds stay valid
}

// (2) one warp per clustered subspace: a dense point of the dominant component
__global__ void k_uf_sample(ClusterArgs a, int nclustered, int* __restrict__ sample) {
  const int cs = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (cs >= nclustered) return;
  const unsigned lane = lane_id();
  const int si = a.clustered_list[cs];
  const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
  const long long s0 = a.kstart[si], len = a.kstart[si + 1] - s0;
  long long pick = -1;
  if (len > 0) {
    long long idx = s0 + ((2 * (long long)lane + 1) * len) / 64;
    for (int t = 0; t < 16 && idx < s0 + len; ++t, ++idx)
      if (bit_of(dn, a.keep_ids[idx])) {
        pick = idx;
        break;
      }
  }
  const int root = pick >= 0 ? uf_find(a.uf, (int)pick) : -1 - (int)lane;  // no point: a unique non-root
  const unsigned peers = __match_any_sync(0xffffffffu, root);
  int votes = pick >= 0 ? __popc(peers) : 0;
  int best = votes, who = (int)lane;
  for (int o = 16; o > 0; o >>= 1) {
    int bv = __shfl_xor_sync(0xffffffffu, best, o), bw = __shfl_xor_sync(0xffffffffu, who, o);
    if (bv > best || (bv == best && bw < who)) {
      best = bv;
      who = bw;
    }
  }
  long long win = __shfl_sync(0xffffffffu, pick, who);
  if (lane == 0) sample[cs] = best > 0 ? (int)win : -1;
}

// (2b) one thread per kept point: 1 when it is in its subspace's dominant
// component (or is no dense point of a clustered subspace), else 0
__global__ void __launch_bounds__(256) k_uf_dominant(ClusterArgs a, const int* __restrict__ cslot_of,
                                                     const int* __restrict__ sample, uint8_t* __restrict__ dom) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= a.nkeep) return;
  uint8_t f = 1;
  const int si = a.sub_of[kk];
  if (a.clustered[si]) {
    const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
    if (bit_of(dn, a.keep_ids[kk])) {
      const int smp = sample[cslot_of[si]];
      f = (smp >= 0 && uf_find(a.uf, (int)kk) == uf_find(a.uf, smp)) ? 1 : 0;
    }
  }
  dom[kk] = f;
}

// (3) one warp per dense point outside the dominant component (dom = 0): its
// dense neighbours.  An edge between two such points is taken by the one with
// the larger keep index (the other one's warp skips it; the neighbour relation
// is symmetric), an edge to a dominant point always; edges between dominant
// points join one component already.  The point's own root is found once per
// 64 neighbours.
__global__ void __launch_bounds__(256) k_uf_union(ClusterArgs a, const uint8_t* __restrict__ dom) {
  const long long kk = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (kk >= a.nkeep) return;
  if (dom[kk]) return;
  const int si = a.sub_of[kk];
  const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
  const unsigned lane = lane_id();
  const long long b = a.keep_loff[kk];
  const int len = a.keep_lcnt[kk];
  // two chunks of 32 entries per step: their loads and finds are independent
  // chains, issued together (the walk is bound by their latency)
  constexpr int kUnionChunks = 2;
  for (int j0 = 0; j0 < len; j0 += kUnionChunks * 32) {
    int qv[kUnionChunks], kq[kUnionChunks];
#pragma unroll
    for (int u = 0; u < kUnionChunks; ++u) {
      const int j = j0 + u * 32 + (int)lane;
      qv[u] = j < len ? a.ent[b + j].x : 0;
    }
#pragma unroll
    for (int u = 0; u < kUnionChunks; ++u) {
      kq[u] = -1;
      if (j0 + u * 32 + (int)lane < len) {
        const int q = qv[u];
        if (GUARD_OK(a.guard, q >= 0 && q < a.n, 61, q) && bit_of(dn, q)) {
          long long k2 = keep_index(a, si, q);
          if (GUARD_OK(a.guard, k2 >= a.kstart[si] && k2 < a.kstart[si + 1], 62, k2))
            kq[u] = (k2 < kk || dom[k2]) ? (int)k2 : -1;  // a larger non-dominant neighbour takes the edge
        }
      }
    }
    bool any = false;
#pragma unroll
    for (int u = 0; u < kUnionChunks; ++u) any = any || kq[u] >= 0;
    if (!__any_sync(0xffffffffu, any)) continue;
    int rk = 0;
    if (lane == 0) rk = uf_find(a.uf, (int)kk);
    rk = __shfl_sync(0xffffffffu, rk, 0);
    int rq[kUnionChunks];
#pragma unroll
    for (int u = 0; u < kUnionChunks; ++u) rq[u] = kq[u] >= 0 ? uf_find(a.uf, kq[u]) : rk;
    // uf_unite takes stale roots: a failed hook finds the current ones
#pragma unroll
    for (int u = 0; u < kUnionChunks; ++u)
      if (rq[u] != rk) uf_unite(a.uf, rk, rq[u], a.err);
  }
}

// Level 1 (one-dim subspaces {D}): the neighbour relation on a line is
// monotone -- for p <= q <= r in coordinate, p and r neighbours makes q a
// neighbour of both (the +-1 fine-cell test and the distance only grow with
// the gap) -- so the components of the dense points are the runs of
// consecutive dense points, in coordinate order, whose consecutive pairs are
// neighbours.  Every point's parent becomes the least keep index of its run,
// the root union-find ends at (it hooks larger roots under smaller).

// (1) dense points of clustered subspaces
__global__ void k_l1_flags(ClusterArgs a, int* __restrict__ flag) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= a.nkeep) return;
  int f = 0;
  const int si = a.sub_of[kk];
  if (a.clustered[si]) f = bit_of(a.bitmaps + a.subs[si].bitmap_off + a.words, a.keep_ids[kk]) ? 1 : 0;
  flag[kk] = f;
}

// (2) element e (compacted): its keep index and its sort key's bytes, least
// significant first: the coordinate's bits (x >= 0: ordered as integers), then
// the subspace
__global__ void k_l1_pack(ClusterArgs a, const float* __restrict__ X, int d, const int* __restrict__ flag,
                          const int* __restrict__ pos, int* __restrict__ kidx, uint8_t* __restrict__ kbytes) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= a.nkeep || !flag[kk]) return;
  const int e = pos[kk];
  const int si = a.sub_of[kk];
  const unsigned u = __float_as_uint(X[(size_t)a.keep_ids[kk] * d + a.subs[si].dim]);
  kidx[e] = (int)kk;
  uint8_t* kb = kbytes + (size_t)e * 5;
  kb[0] = (uint8_t)u;
  kb[1] = (uint8_t)(u >> 8);
  kb[2] = (uint8_t)(u >> 16);
  kb[3] = (uint8_t)(u >> 24);
  kb[4] = (uint8_t)si;  // one byte: level 1 has d <= 64 subspaces (the engine checks nsubs <= 256)
}

// (3) run starts in sorted order: not the same subspace as the previous
// element, or not its neighbour
__global__ void k_l1_starts(ClusterArgs a, const float* __restrict__ X, int d, const uint8_t* __restrict__ fc,
                            float acc_max, const int* __restrict__ perm, const int* __restrict__ kidx, int m,
                            int* __restrict__ start) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  int st = 1;
  if (t > 0) {
    const long long k1 = kidx[perm[t]], k0 = kidx[perm[t - 1]];
    const int s1 = a.sub_of[k1], s0 = a.sub_of[k0];
    if (s1 == s0) {
      const int D = a.subs[s1].dim;
      const size_t p = (size_t)a.keep_ids[k1] * d + D, q = (size_t)a.keep_ids[k0] * d + D;
      const int fp = fc[p], fq = fc[q];
      st = (fq >= fp - 1 && fq <= fp + 1 && dist_step(0.f, X[p], X[q]) <= acc_max) ? 0 : 1;
    }
  }
  start[t] = st;
}

// (4) least keep index of every run, then every point's parent
__global__ void k_l1_runmin(const int* __restrict__ perm, const int* __restrict__ kidx, const int* __restrict__ start,
                            const int* __restrict__ runx, int m, int* __restrict__ runmin) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) atomicMin(&runmin[runx[t] + start[t] - 1], kidx[perm[t]]);
}
__global__ void k_l1_parent(const int* __restrict__ perm, const int* __restrict__ kidx, const int* __restrict__ start,
                            const int* __restrict__ runx, int m, const int* __restrict__ runmin, int* __restrict__ par) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) par[kidx[perm[t]]] = runmin[runx[t] + start[t] - 1];
}

// roots: every dense point's root goes to a separate array (writing it into
// `par` would race with the path-halving writes of concurrent finds, which
// may store a non-root ancestor over it); roots are flagged
__global__ void k_uf_flatten(ClusterArgs a, int* is_root, int* root_of) {
  long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= a.nkeep) return;
  int si = a.sub_of[kk];
  int root = 0, r = -1;
  if (a.clustered[si]) {
    const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
    if (bit_of(dn, a.keep_ids[kk])) {
      r = uf_find(a.uf, (int)kk);
      root = (r == (int)kk);
    }
  }
  root_of[kk] = r;
  is_root[kk] = root;
}

// component id (global, dense) of every dense kept point; -1 otherwise
// atomicAdd(&ctr[key], 1) for every lane whose key is >= 0, with one atomic
// per distinct key of the warp (large components put most lanes of a warp on
// one counter); returns the lane's slot (the counter's old value + its rank
// among the lanes with that key).  Every lane of the warp calls it.
__device__ __forceinline__ int warp_inc(int* ctr, int key) {
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  const int leader = __ffs((int)peers) - 1;
  int base = 0;
  if (key >= 0 && (int)lane_id() == leader) base = atomicAdd(&ctr[key], __popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  return base + __popc(peers & lanemask_lt());
}

__global__ void k_comp_ids(ClusterArgs a, const int* __restrict__ root_id, const int* __restrict__ root_of,
                           int* __restrict__ comp, int* __restrict__ mcount) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = kk < a.nkeep;  // whole warps stay for warp_inc
  int c = -1;
  if (valid) {
    const int r = root_of[kk];
    if (r >= 0) c = root_id[r];
  }
  warp_inc(mcount, c);
  if (valid) comp[kk] = c;
}

__global__ void k_members(ClusterArgs a, const int* __restrict__ comp, const long long* __restrict__ moff,
                          int* __restrict__ mfill, int* __restrict__ members) {
  const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = kk < a.nkeep ? comp[kk] : -1;  // whole warps stay for warp_inc
  const int o = warp_inc(mfill, c);
  if (c >= 0) members[moff[c] + o] = a.keep_ids[kk];
}

// border pairs (component, non-dense neighbour), de-duplicated through two
// slots per (clustered subspace, point); rare third components overflow
__global__ void __launch_bounds__(256) k_borders(ClusterArgs a, const int* __restrict__ comp,
                                                 const int* __restrict__ cslot_of, int* __restrict__ slots,
                                                 int2* __restrict__ ovf, int* __restrict__ novf, int ovf_cap) {
  const long long kk = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (kk >= a.nkeep) return;
  const int c = comp[kk];
  if (c < 0) return;
  const int si = a.sub_of[kk];
  const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
  const long long b = a.keep_loff[kk];
  const int len = a.keep_lcnt[kk];
  int* sl = slots + (long long)cslot_of[si] * a.n * 2;
  // the list is read kBorderChunks x 32 entries at a time, all loads issued
  // before the first is used (the walk is bound by their latency)
  constexpr int kBorderChunks = 4;
  for (int j0 = 0; j0 < len; j0 += kBorderChunks * 32) {
    int qv[kBorderChunks];
#pragma unroll
    for (int u = 0; u < kBorderChunks; ++u) {
      const int j = j0 + u * 32 + (int)lane_id();
      qv[u] = j < len ? a.ent[b + j].x : 0;
    }
#pragma unroll
    for (int u = 0; u < kBorderChunks; ++u) {
      if (j0 + u * 32 + (int)lane_id() >= len) continue;
      const int q = qv[u];
      if (!GUARD_OK(a.guard, q >= 0 && q < a.n, 65, q) || bit_of(dn, q)) continue;
      int* s2 = sl + 2LL * q;
      int v0 = ((volatile int*)s2)[0];
      if (v0 == c) continue;
      if (v0 == -1) {
        int old = atomicCAS(&s2[0], -1, c);
        if (old == -1 || old == c) continue;
      }
      int v1 = ((volatile int*)s2)[1];
      if (v1 == c) continue;
      if (v1 == -1) {
        int old = atomicCAS(&s2[1], -1, c);
        if (old == -1 || old == c) continue;
      }
      int o = atomicAdd(novf, 1);
      if (o < ovf_cap)
        ovf[o] = make_int2(c, q);
      else
        atomicExch(a.err, 4);
    }
  }
}

__global__ void k_border_count(const int* __restrict__ slots, long long nslots2, int* __restrict__ bcount) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  warp_inc(bcount, i < nslots2 ? slots[i] : -1);  // whole warps stay for warp_inc
}

__global__ void k_border_count_ovf(const int2* __restrict__ ovf, int novf, int* __restrict__ bcount) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < novf) atomicAdd(&bcount[ovf[i].x], 1);
}

__global__ void k_border_fill(const int* __restrict__ slots, long long nslots2, int n, const long long* __restrict__ boff,
                              int* __restrict__ bfill, int* __restrict__ borders) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = i < nslots2 ? slots[i] : -1;  // whole warps stay for warp_inc
  const int o = warp_inc(bfill, c);
  if (c >= 0) borders[boff[c] + o] = (int)((i >> 1) % n);
}

__global__ void k_border_fill_ovf(const int2* __restrict__ ovf, int novf, const long long* __restrict__ boff,
                                  int* __restrict__ bfill, int* __restrict__ borders) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= novf) return;
  int2 e = ovf[i];
  int o = atomicAdd(&bfill[e.x], 1);
  borders[boff[e.x] + o] = e.y;
}

// Components of each region in first-dense-seed order.  One block per
// clustered subspace walks its regions (they may share components).
__global__ void __launch_bounds__(256) k_region_order(ClusterArgs a, const int* __restrict__ comp,
                                                      const int* __restrict__ cbase_of,
                                                      const int* __restrict__ sub_calls_off,
                                                      const int* __restrict__ sub_calls, const CallDesc* __restrict__ ncalls,
                                                      const int* __restrict__ pts, int* __restrict__ firstpos,
                                                      int* __restrict__ order, int* __restrict__ order_cnt) {
  __shared__ int sh[32];
  const int cs = blockIdx.x;  // clustered-subspace slot
  const int si = a.clustered_list[cs];
  const unsigned* dn = a.bitmaps + a.subs[si].bitmap_off + a.words;
  const int cb = cbase_of[si];
  for (int t = sub_calls_off[cs]; t < sub_calls_off[cs + 1]; ++t) {
    const int call = sub_calls[t];
    const CallDesc C = ncalls[call];
    const int* P = pts + C.pts_off;
    const int m = C.npts;
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      int p = P[j];
      if (bit_of(dn, p)) {
        long long kp = keep_index(a, si, p);
        if (GUARD_OK(a.guard, kp >= a.kstart[si] && kp < a.kstart[si + 1] && comp[kp] >= 0, 66, kp))
          atomicMin(&firstpos[comp[kp]], j);
      }
    }
    __syncthreads();
    int base = 0;
    for (int c0 = 0; c0 < m; c0 += blockDim.x) {
      int j = c0 + threadIdx.x;
      int f = 0, c = -1;
      if (j < m) {
        int p = P[j];
        if (bit_of(dn, p)) {
          long long kp = keep_index(a, si, p);
          if (kp >= a.kstart[si] && kp < a.kstart[si + 1] && comp[kp] >= 0) {
            c = comp[kp];
            f = firstpos[c] == j;
          }
        }
      }
      int tot;
      int inc = block_inclusive_scan<int>(f, sh, &tot);
      if (f) order[C.pts_off + base + inc - 1] = c - cb;
      base += tot;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      int p = P[j];
      if (bit_of(dn, p)) {
        long long kp = keep_index(a, si, p);
        if (kp >= a.kstart[si] && kp < a.kstart[si + 1] && comp[kp] >= 0) firstpos[comp[kp]] = INT_MAX;
      }
    }
    if (threadIdx.x == 0) order_cnt[call] = base;
    __syncthreads();
  }
}

// pack the per-region component orders (written at each region's point
// offset) into consecutive lists
__global__ void k_pack_order(const CallDesc* __restrict__ ncalls, int ncall, const int* __restrict__ order,
                             const int* __restrict__ order_cnt, const long long* __restrict__ order_off,
                             int* __restrict__ packed) {
  const int c = blockIdx.x;
  if (c >= ncall) return;
  const long long src = ncalls[c].pts_off, dst = order_off[c];
  for (int j = threadIdx.x; j < order_cnt[c]; j += blockDim.x) packed[dst + j] = order[src + j];
}

void launch_pack_order(const CallDesc* ncalls, int ncall, const int* order, const int* order_cnt,
                       const long long* order_off, int* packed, cudaStream_t s) {
  if (ncall > 0) k_pack_order<<<ncall, 128, 0, s>>>(ncalls, ncall, order, order_cnt, order_off, packed);
}

// ---------------------------------------------------------------------------
void launch_uf_init(int* par, long long n, cudaStream_t s) {
  if (n > 0) k_uf_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(par, n);
}
void launch_uf_union(const ClusterArgs& a, int nclustered, const int* cslot_of, int* sample, uint8_t* dom,
                     cudaStream_t s) {
  if (a.nkeep <= 0) return;
  k_uf_link2<<<(unsigned)((a.nkeep + 255) / 256), 256, 0, s>>>(a);
  k_uf_compress<<<(unsigned)((a.nkeep + 255) / 256), 256, 0, s>>>(a);
  if (nclustered > 0) k_uf_sample<<<(unsigned)((nclustered * 32LL + 255) / 256), 256, 0, s>>>(a, nclustered, sample);
  k_uf_dominant<<<(unsigned)((a.nkeep + 255) / 256), 256, 0, s>>>(a, cslot_of, sample, dom);
  k_uf_union<<<(unsigned)((a.nkeep * 32 + 255) / 256), 256, 0, s>>>(a, dom);
}
void launch_uf_level1_count(const ClusterArgs& a, const UfLevel1Scratch& w, void* sums, cudaStream_t s) {
  if (a.nkeep <= 0) return;
  k_l1_flags<<<(unsigned)((a.nkeep + 255) / 256), 256, 0, s>>>(a, w.flag);
  launch_exclusive_scan_int(w.flag, w.pos, a.nkeep, w.total, sums, s);
}

void launch_uf_level1(const ClusterArgs& a, const float* X, int d, const uint8_t* fc, float acc_max,
                      const UfLevel1Scratch& w, int m, void* sums, cudaStream_t s) {
  if (a.nkeep <= 0 || m <= 0) return;
  const unsigned kb = (unsigned)((a.nkeep + 255) / 256);
  k_l1_pack<<<kb, 256, 0, s>>>(a, X, d, w.flag, w.pos, w.kidx, w.kbytes);
  int* in = w.perm0;
  int* out = w.perm1;
  launch_iota(in, m, s);
  for (int k = 0; k < 5; ++k) {  // LSD: coordinate bytes, then the subspace
    launch_byte_sort_pass(in, out, m, w.kbytes, 5, k, w.hist, w.total, nullptr, sums, s);
    int* t = in;
    in = out;
    out = t;
  }
  const unsigned mb = (unsigned)((m + 255) / 256);
  k_l1_starts<<<mb, 256, 0, s>>>(a, X, d, fc, acc_max, in, w.kidx, m, w.start);
  launch_exclusive_scan_int(w.start, w.runx, m, w.total, sums, s);
  cudaMemsetAsync(w.runmin, 0x7f, sizeof(int) * (size_t)m, s);
  k_l1_runmin<<<mb, 256, 0, s>>>(in, w.kidx, w.start, w.runx, m, w.runmin);
  k_l1_parent<<<mb, 256, 0, s>>>(in, w.kidx, w.start, w.runx, m, w.runmin, a.uf);
}

void launch_uf_flatten(const ClusterArgs& a, int* is_root, int* root_of, cudaStream_t s) {
  if (a.nkeep > 0) k_uf_flatten<<<(unsigned)((a.nkeep + 255) / 256), 256, 0, s>>>(a, is_root, root_of);
}
void launch_comp_ids(const ClusterArgs& a, const int* root_id, const int* root_of, int* comp, int* mcount,
                     cudaStream_t s) {
  if (a.nkeep > 0)
    k_comp_ids<<<(unsigned)((a.nkeep + 255) / 256), 256, 0, s>>>(a, root_id, root_of, comp, mcount);
}
void launch_members(const ClusterArgs& a, const int* comp, const long long* moff, int* mfill, int* members,
                    cudaStream_t s) {
  if (a.nkeep > 0) k_members<<<(unsigned)((a.nkeep + 255) / 256), 256, 0, s>>>(a, comp, moff, mfill, members);
}
void launch_borders(const ClusterArgs& a, const int* comp, const int* cslot_of, int* slots, int2* ovf, int* novf,
                    int ovf_cap, cudaStream_t s) {
  if (a.nkeep > 0)
    k_borders<<<(unsigned)((a.nkeep * 32 + 255) / 256), 256, 0, s>>>(a, comp, cslot_of, slots, ovf, novf, ovf_cap);
}
void launch_border_count(const int* slots, long long nslots2, const int2* ovf, int novf, int* bcount,
                         cudaStream_t s) {
  if (nslots2 > 0) k_border_count<<<(unsigned)((nslots2 + 255) / 256), 256, 0, s>>>(slots, nslots2, bcount);
  if (novf > 0) k_border_count_ovf<<<(novf + 255) / 256, 256, 0, s>>>(ovf, novf, bcount);
}
void launch_border_fill(const int* slots, long long nslots2, int n, const int2* ovf, int novf, const long long* boff,
                        int* bfill, int* borders, cudaStream_t s) {
  if (nslots2 > 0)
    k_border_fill<<<(unsigned)((nslots2 + 255) / 256), 256, 0, s>>>(slots, nslots2, n, boff, bfill, borders);
  if (novf > 0) k_border_fill_ovf<<<(novf + 255) / 256, 256, 0, s>>>(ovf, novf, boff, bfill, borders);
}
void launch_region_order(const ClusterArgs& a, int nclustered, const int* comp, const int* cbase_of,
                         const int* sub_calls_off, const int* sub_calls, const CallDesc* ncalls, const int* pts,
                         int* firstpos, int* order, int* order_cnt, cudaStream_t s) {
  if (nclustered > 0)
    k_region_order<<<nclustered, 256, 0, s>>>(a, comp, cbase_of, sub_calls_off, sub_calls, ncalls, pts, firstpos,
                                              order, order_cnt);
}

}  // namespace inscy
