// Host engine of the GB300 INSCY path and its C ABI (include/inscy_gb300.h).
//
// The reference runs INSCY as a depth-first recursion (INSCYCPU3Weak,
// InscyNodeCpu.cu:159-235; the GPU forms InscyArrayGpu4/5,
// InscyArrayGpuMulti2.cu:569-836, keep that recursion on the host and launch
// small kernels per node).  Here the recursion is split in two:
//
//  1. Expansion, level by level over the subspace lattice, on the GPU.
//     Everything that decides *which* recursion nodes exist -- restrict,
//     mergeWithNeighbors, the weak-density prune and the min_size test -- is
//     a pure function of the node, so all nodes of one depth are expanded
//     together: one density launch for every (subspace, point) of the level,
//     one restrict/merge/prune launch for every (node, dim), one union-find
//     for every subspace that has a surviving node.
//  2. Commit, in the reference's depth-first order, on the host: the
//     pruneRedundancy gate (ScyTreeNode.cu:669-734), the BFS label
//     numbering (ClusteringCpu.cu:317-389) and join (util.cu:655-743) read
//     and write the global result map, so they replay the exact DFS order
//     over the data the GPU produced.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <new>
#include <thread>

#include "../../include/inscy_gb300.h"
#include "host_threads.h"
#include "inscy_common.cuh"
#include "inscy_kernels.h"
#include "inscy_prims.cuh"

namespace inscy {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                                            \
  do {                                                                                                   \
    cudaError_t e_ = (x);                                                                                \
    if (e_ != cudaSuccess)                                                                               \
      throw ::inscy::Error(INSCY_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + \
                                      ":" + std::to_string(__LINE__) + ")");                             \
  } while (0)

// ---------------------------------------------------------------------------
// density thresholds, computed on the host with the reference's formulas and
// types (ClusteringCpu.cu:27, 36-38, 136-164)
// ---------------------------------------------------------------------------
const double kPi = 3.14;  // ClusteringCpu.cu:27
// device memory the single-pass neighbour lists of one level may take
#ifndef INSCY_SINGLE_PASS_BYTES
#define INSCY_SINGLE_PASS_BYTES (32LL << 30)
#endif
constexpr long long kSinglePassBytes = INSCY_SINGLE_PASS_BYTES;
// density pass over point rows (k_neighbours_rows) when d <= 32; 0 keeps the
// general kernel for every d (both give the same lists)
#ifndef INSCY_DENSITY_ROWS
#define INSCY_DENSITY_ROWS 1
#endif
constexpr bool kDensityRows = INSCY_DENSITY_ROWS != 0;
// Candidate rows of the row kernel: prefetched into registers through L1
// (default), or gathered by TMA tile::gather4 copies into shared memory when
// the environment variable INSCY_ROWS_TMA is 1 at the start of a run.  Both
// write the same lists; the TMA form measured 3.6x slower on the 25,000 x 15
// workload (its copies go from L2 to shared memory and lose the L1 reuse of
// the candidate rows that neighbouring queries share).
static bool rows_tma_requested() {
  const char* e = std::getenv("INSCY_ROWS_TMA");
  return e && e[0] == '1';
}

// Launch shape of the row kernel (work-counter updates per warp that the
// pairs-per-update chunk aims at, resident blocks per SM), measured once per
// (device, row width) in the process: on
// the first single-pass level with at least kTunePairs (group, query) pairs,
// each candidate shape runs the level's pass twice (every run writes the same
// lists) and the fastest is kept.  INSCY_ROWS_TUNE=0 keeps the default shape.
constexpr long long kTunePairs = 100000;
struct RowShape {
  int takes = 0, bps = 0;  // 0: 16 updates per warp / the most the registers allow
};
static std::mutex g_tune_m;
static std::map<std::pair<int, int>, RowShape> g_tuned;  // (device, slots) -> shape
static bool rows_tune_enabled() {
  const char* e = std::getenv("INSCY_ROWS_TUNE");
  return !(e && e[0] == '0');
}
// narrowest leaf key the level kernel may use (4; raised only to test the wider forms)
#ifndef INSCY_TREE_MIN_KEY_BYTES
#define INSCY_TREE_MIN_KEY_BYTES 4
#endif
constexpr int kTreeMinKeyBytes = INSCY_TREE_MIN_KEY_BYTES;
static float omega_of(int k) { return (float)(2.0 / ((double)k + 2.0)); }
static float gamma_of(int m) {
  if (m == 2) return 1.0f;
  if (m == 1) return (float)std::sqrt(kPi);
  return (float)(((double)m / 2.0 - 1.0) * (double)gamma_of(m - 2));
}
static float cball_of(int k) {
  float r = (float)std::pow(kPi, (double)k / 2.0);
  return r / gamma_of(k + 2);
}
static float alpha_of(int k, float eps, int n) {
  float r = (float)((double)(2 * n) * std::pow((double)eps, (double)k) * (double)cball_of(k));
  r = (float)((double)r / (std::pow(1.0, (double)k) * (double)(k + 2)));
  return r;
}
static float expden_of(int k, float eps, int n) {
  float r = (float)((double)((float)n * cball_of(k)) * std::pow((double)eps, (double)k));
  r = (float)((double)r / std::pow(1.0, (double)k));
  return r;
}

// ---------------------------------------------------------------------------
// result map ordering (vec_cmp, util.cu:633-653): compare from the last dim
// ---------------------------------------------------------------------------
struct SubspaceOrder {
  bool operator()(const std::vector<int>& a, const std::vector<int>& b) const {
    int i = (int)a.size() - 1, j = (int)b.size() - 1;
    while (a[i] == b[j]) {
      --i;
      --j;
      if (i < 0 || j < 0) return i < j;
    }
    return a[i] < b[j];
  }
};

static std::vector<int> dims_of(uint64_t m) {
  std::vector<int> v;
  for (int k = 0; k < 64; ++k)
    if ((m >> k) & 1ull) v.push_back(k);
  return v;
}

// ---------------------------------------------------------------------------
// device memory: stream-ordered allocations from a retained pool (no
// cudaMalloc on the hot path once the pool has grown)
// ---------------------------------------------------------------------------
class Pool {
 public:
  explicit Pool(int device) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    CK(cudaMemPoolCreate(&pool_, &props));
    uint64_t thr = UINT64_MAX;
    CK(cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &thr));
  }
  ~Pool() { cudaMemPoolDestroy(pool_); }
  void* get(size_t bytes, cudaStream_t s) {
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    CK(cudaMallocFromPoolAsync(&p, bytes, pool_, s));
    return p;
  }
  void put(void* p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
  }

 private:
  cudaMemPool_t pool_;
};

// a set of allocations released together
class Scope {
 public:
  Scope(Pool& p, cudaStream_t s) : pool_(p), s_(s) {}
  ~Scope() { release(); }
  template <class T>
  T* get(size_t count) {
    void* p = pool_.get(count * sizeof(T), s_);
    ptrs_.push_back(p);
    return (T*)p;
  }
  void release() {
    for (void* p : ptrs_) pool_.put(p, s_);
    ptrs_.clear();
  }
  void adopt(Scope& o) {
    ptrs_.insert(ptrs_.end(), o.ptrs_.begin(), o.ptrs_.end());
    o.ptrs_.clear();
  }

 private:
  Pool& pool_;
  cudaStream_t s_;
  std::vector<void*> ptrs_;
};

// pinned staging for device-to-host copies
class Pinned {
 public:
  ~Pinned() {
    if (p_) cudaFreeHost(p_);
  }
  void* get(size_t bytes) {
    if (bytes > cap_) {
      if (p_) cudaFreeHost(p_);
      p_ = nullptr;
      cap_ = std::max(bytes, cap_ * 2);
      CK(cudaMallocHost(&p_, cap_));
    }
    return p_;
  }

 private:
  void* p_ = nullptr;
  size_t cap_ = 0;
};

// ---------------------------------------------------------------------------
// host-side record of the recursion (for the ordered commit)
// ---------------------------------------------------------------------------
struct HRegion {
  int dim;
  int passed;
  int child;  // index of the child call in its phase (passed only)
};

struct HCall {
  uint64_t rmask = 0;
  int f = 0;
  int level = 0;
  int npts = 0;
  long long pts_off = 0;  // into its level's pts (its leaf order)
  int norder = 0;         // components in first-seed order, at its level's order[order_off ...]
  long long order_off = 0;
  int csub = -1;          // clustered subspace (its own subspace) in its phase's subs
  std::vector<HRegion> regions;  // ordered by (dim, cell run)
};

// ints read back from the device: resize() gives fresh storage without
// filling it (the copy fills it)
struct IntBuf {
  std::unique_ptr<int[]> p;
  size_t n = 0;
  void resize(size_t m) {
    p.reset(new int[m > 0 ? m : 1]);
    n = m;
  }
  int* data() { return p.get(); }
  const int* data() const { return p.get(); }
  size_t size() const { return n; }
};

// a read-only range of such a buffer
struct IntView {
  const int* p = nullptr;
  size_t n = 0;
  const int* data() const { return p; }
  const int& operator[](size_t i) const { return p[i]; }
  size_t size() const { return n; }
};

struct HLevel {
  IntBuf pts;
  IntBuf order;
};

struct HSub {  // components of one clustered subspace
  std::vector<long long> moff;
  IntView members;  // ranges of the level's member and border read-backs,
  std::vector<long long> boff;
  IntView borders;
  std::shared_ptr<const IntBuf> keep_m, keep_b;  // which these keep alive
};

// Where the points of a label come from: component `comp` of a clustered
// subspace (its member list is the GPU's).  A phase's subspaces do not move
// once the phase is complete, which is before any label points to them.
struct LabelRef {
  const HSub* hs;
  int comp;
};

// The calls whose first restricted dim lies in [d0, d1) (the root's
// restrictions to those dims and everything below them).  INSCY's depth-first
// commit handles them after the calls of every smaller first dim, and a
// superset of their subspaces either holds a smaller dim (an earlier phase)
// or starts in the same range (this phase), so a phase can be committed as
// soon as its expansion is done, while the GPU expands the next one.  The
// lattice below dim D shrinks quickly with D: the phases are {0}, {1}, {2},
// {3, 4}, {5, 6, 7} and the rest, so the commit of each phase overlaps the
// expansion of the next and the last one, whose commit is all that is left
// once the GPU is done, holds little (a phase per dim costs the GPU more in
// small launches than it saves).
struct Phase {
  int d0 = 0, d1 = 0;
  std::vector<HCall> calls;    // level >= 1
  std::vector<HLevel> levels;  // [level] for level >= 2 (level 1: the shared level1_)
  std::vector<HSub> subs;      // its clustered subspaces
};

// The label vectors of a run's result-map entries: rows of n ints in blocks
// of `rows` rows (about 32 MB a block), taken in the order the entries are
// created.  A result hands them over as a few 2-d arrays and one slot per
// clustered subspace, so a binding builds its label views without a call
// per subspace.
struct LabelBlocks {
  long long n = 0;
  int rows = 1;  // rows per block
  int used = 0;  // rows taken
  std::vector<std::unique_ptr<int[]>> blocks;
  BlockFiller* filler = nullptr;  // source of blocks already filled with -1
  void reset(long long points, BlockFiller* f) {
    n = points;
    const long long per = (32LL << 20) / (4 * std::max(1LL, points));
    rows = (int)std::max(1LL, std::min(256LL, per));
    used = 0;
    blocks.clear();
    filler = f;
    if (filler) filler->start((size_t)rows * (size_t)n);
  }
  // a new row, all -1, and its slot
  int* take(int& slot) {
    if (used == (int)blocks.size() * rows) {
      if (filler) {
        blocks.push_back(filler->take());
      } else {
        blocks.emplace_back(new int[(size_t)rows * (size_t)n]);
        std::fill(blocks.back().get(), blocks.back().get() + (size_t)rows * (size_t)n, -1);
      }
    }
    slot = used++;
    return row(slot);
  }
  int* row(int slot) const { return blocks[slot / rows].get() + (size_t)(slot % rows) * (size_t)n; }
};

// One result-map entry (a clustered subspace) during the commit.
struct Entry {
  uint64_t mask = 0;
  int* lab = nullptr;          // one label per point (-1 noise, -2 border): a row of the run's LabelBlocks
  int slot = -1;               // that row
  std::vector<int> size;       // points per label (index = label)
  std::vector<LabelRef> src;   // members of each label (may include points relabelled since)
  int maxv = -100000;          // v_max(lab) (util.cu:566-574)
  int maxsz = 0;               // largest cluster
  std::vector<int> by_size;    // labels in ascending size (rebuilt when dirty)
  bool dirty = true;
};

// The clustering vector of one dim loop (InscyNodeCpu.cu:175): n labels,
// -1 by default.  Each point holds (generation << 32 | label) in one word; a
// label only counts when its generation is the current one, which makes
// clearing the vector O(1).
struct LoopVec {
  std::vector<uint64_t> gv;
  uint64_t cur = 1ull << 32;
  void init(long long n) {
    if ((long long)gv.size() != n) {
      gv.assign(n, 0);
      cur = 1ull << 32;
    }
  }
  void clear() {
    cur += 1ull << 32;
    if (cur == 0) {  // wrapped: reset the stamps
      std::fill(gv.begin(), gv.end(), 0ull);
      cur = 1ull << 32;
    }
  }
  int get(int p) const {
    const uint64_t w = gv[p];
    return (w & 0xffffffff00000000ull) == cur ? (int)(uint32_t)w : -1;
  }
  void set(int p, int v) { gv[p] = cur | (uint32_t)v; }
};


// Points [k0, k1) of a member list: for join's redundancy test the members of
// a superset cluster (those still labelled l in that entry's `lab` count, hsz
// = its size); elsewhere a range of points to label l.
struct Walk {
  const int* mem;
  long long k0, k1;
  const int* lab;
  int l;
  float hsz;
};

struct LoopState {
  std::vector<LabelRef> ref{LabelRef{nullptr, -1}};
  std::vector<int> size{0};
  int nlabels = 0;
  // loop-vector writes of the members of min_size clusters (their first
  // member is written at once), made only when join's redundancy test reads
  // the loop vector (its superset side)
  std::vector<Walk> pend;
  long long pend_work = 0;
};

// Drop every live cluster c of the loop with a point in w and
// size(c) * r < |w's cluster| (util.cu:680-705); true if one was dropped.
static bool walk_test(const Walk& w, const LoopVec& V, const int* size, float r, char* alive) {
  bool hit = false;
  const uint64_t* gv = V.gv.data();
  const uint64_t cur = V.cur;
  // the two lookups of a point are random reads of n-long vectors (several
  // superset entries per join: more than a core's L2 holds), so the points a
  // few iterations ahead are prefetched
  constexpr long long kAhead = 16;
  for (long long k = w.k0; k < w.k1; ++k) {
    if (k + kAhead < w.k1) {
      const int qa = w.mem[k + kAhead];
      __builtin_prefetch(w.lab + qa);
      __builtin_prefetch(gv + qa);
    }
    const int q = w.mem[k];
    if (w.lab[q] != w.l) continue;
    const uint64_t x = gv[q];
    if ((x & 0xffffffff00000000ull) != cur) continue;
    const int c = (int)(uint32_t)x;
    if (c > 0 && __atomic_load_n(&alive[c], __ATOMIC_RELAXED) && (float)size[c] * r < w.hsz) {
      __atomic_store_n(&alive[c], (char)0, __ATOMIC_RELAXED);
      hit = true;
    }
  }
  return hit;
}

// joins whose redundancy test covers fewer points run it on one thread
constexpr long long kParallelWalk = 32768;
// device-to-host reads of at least this many bytes skip the pinned staging
constexpr size_t kDirectD2H = 1u << 20;

struct HostParams {
  float eps, F, r;
  int num_obj, min_size, cells, rect, entropy_order;
};

// get_subspace_order (inscy_map.cpp:61-121): the SCY-tree's level order.
// Identity for entropy_order 0; else dims by ascending entropy of their
// coarse-cell histogram (float sums of -p log p with p = count / n, float
// log), ties by dim, reversed for entropy_order -1.  An empty cell makes
// p log p a NaN exactly as in the reference; the (entropy, dim) pairs are
// ordered by the same std::sort the reference's pairsort calls.
std::vector<int> level_order_of(const std::vector<int>& hist, int n, int d, int cells, int entropy_order) {
  std::vector<int> order(d);
  for (int k = 0; k < d; ++k) order[k] = k;
  if (entropy_order == 0) return order;
  std::vector<std::pair<float, int>> e(d);
  for (int k = 0; k < d; ++k) {
    float h = 0.f;
    for (int c = 0; c < cells; ++c) {
      const float p = (float)hist[(size_t)k * cells + c] / (float)n;
      h -= p * std::log(p);
    }
    e[k] = {h, k};
  }
  std::sort(e.begin(), e.end());
  if (entropy_order == -1) std::reverse(e.begin(), e.end());
  for (int k = 0; k < d; ++k) order[k] = e[k].second;
  return order;
}

// host-pool workers of engines created on this thread (-1: by the core count)
// and the single-pass list budget of their runs: batch lanes divide both
// among the concurrent engines
thread_local int t_pool_workers = -1;
thread_local long long t_single_pass_bytes = kSinglePassBytes;

// ---------------------------------------------------------------------------
// the engine (one run at a time; device resources are kept between runs)
// ---------------------------------------------------------------------------
class Engine {
 public:
  Engine() {
    CK(cudaGetDevice(&device_));
    CK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_));
    pool_.reset(new Pool(device_));
    {
      const int hw = (int)std::thread::hardware_concurrency();
      hpool_.reset(new HostPool(t_pool_workers >= 0 ? t_pool_workers : std::max(0, std::min(15, hw - 2))));
    }
    CK(cudaEventCreate(&ev0_));
    CK(cudaEventCreate(&ev1_));
  }
  ~Engine() {
    cudaEventDestroy(ev0_);
    cudaEventDestroy(ev1_);
  }

  void run(const float* X, bool on_device, long long n, int d, const HostParams& hp, cudaStream_t s,
           std::vector<std::vector<int>>& out_dims, LabelBlocks& out_labels, std::vector<int>& out_slots,
           inscy_stats& st);

 private:
  // The row kernel's launch shape for rows of `slots` on this device (see
  // RowShape), measured on this level's single pass when no engine of the
  // process has measured it yet.  The statistics counters are off during the
  // trials; each trial writes the same lists, and the caller's launch follows
  // with the chosen shape.
  template <class Fn>
  void tune_rows(DensityLaunch& DL, int slots, long long pairs, cudaStream_t s, Fn& neighbours) {
    if (!rows_tune_enabled() || pairs < kTunePairs) return;
    {
      std::lock_guard<std::mutex> g(g_tune_m);
      if (g_tuned.count({device_, slots})) return;
    }
    unsigned long long* counters[3] = {DL.cand_counter, DL.list_counter, DL.out_counter};
    DL.cand_counter = DL.list_counter = DL.out_counter = nullptr;
    const int bmax = rows_max_blocks_per_sm(slots);
    std::vector<RowShape> cands = {{4, 0}, {8, 0}, {16, 0}, {32, 0}, {64, 0}};
    if (bmax > 2) {
      cands.push_back({16, bmax - 1});
      cands.push_back({64, bmax - 1});
    }
    std::vector<double> best(cands.size(), 1e30);
    for (int rep = 0; rep < 2; ++rep)
      for (size_t i = 0; i < cands.size(); ++i) {
        DL.rows_takes = cands[i].takes;
        DL.rows_bps = cands[i].bps;
        const double ms = timed(s, [&] { neighbours(true); });
        stats_.ms_tune += ms;
        best[i] = std::min(best[i], ms);
      }
    size_t pick = 0;
    for (size_t i = 1; i < cands.size(); ++i)
      if (best[i] < best[pick]) pick = i;
    DL.rows_takes = cands[pick].takes;
    DL.rows_bps = cands[pick].bps;
    DL.cand_counter = counters[0];
    DL.list_counter = counters[1];
    DL.out_counter = counters[2];
    std::lock_guard<std::mutex> g(g_tune_m);
    g_tuned.emplace(std::make_pair(device_, slots), cands[pick]);
  }
  // timing helper: device time of the work queued by f()
  template <class Fn>
  double timed(cudaStream_t s, Fn f) {
    CK(cudaEventRecord(ev0_, s));
    f();
    CK(cudaEventRecord(ev1_, s));
    CK(cudaEventSynchronize(ev1_));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
    return ms;
  }
  // Small reads go through a pinned staging buffer; large ones (the levels'
  // points, component members, borders and orders for the commit) are copied
  // straight into their destination: on a host whose memory the GPU reaches
  // coherently this skips a host copy of every byte (measured on the GB300
  // host: the expansion of a 25,000 x 15 run 171 -> 160 ms).
  void d2h(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    if (!bytes) return;
    auto t0 = std::chrono::steady_clock::now();
    if (bytes >= kDirectD2H) {
      CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    } else {
      void* st = pinned_.get(bytes);
      CK(cudaMemcpyAsync(st, src, bytes, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      std::memcpy(dst, st, bytes);
    }
    stats_.d2h_bytes += (long long)bytes;
    stats_.ms_d2h += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  void h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    if (!bytes) return;
    void* st = pinned_.get(bytes);
    std::memcpy(st, src, bytes);
    CK(cudaMemcpyAsync(dst, st, bytes, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    stats_.h2d_bytes += (long long)bytes;
  }
  template <class T>
  T scalar(const T* dev, cudaStream_t s) {
    T v;
    d2h(&v, dev, sizeof(T), s);
    return v;
  }
  void* scan_sums(long long n, cudaStream_t, Scope& sc) {
    long long nt = (n + 2047) / 2048 + 1;
    return sc.get<long long>((size_t)nt);
  }

  // commit
  void replay_root(int D);
  void replay(const Phase& ph, int ci);
  const HLevel& level_of(const Phase& ph, const HCall& c) const { return c.level == 1 ? level1_ : ph.levels[c.level]; }
  bool prune_redundancy(const Phase& ph, const HCall& c, uint64_t smask);
  const std::vector<int>& superset_candidates(uint64_t smask);
  void cluster_into(const Phase& ph, const HCall& c, LoopVec& V, LoopState& st);
  void join(LoopVec& V, LoopState& st, uint64_t smask);
  void flush_pending(LoopVec& V, LoopState& st);
  void split_pieces(long long work);

  int device_ = 0;
  int sms_ = 1;  // SMs of the device (persistent grids fill each once)
  std::unique_ptr<Pool> pool_;
  Pinned pinned_;
  cudaEvent_t ev0_, ev1_;

  // per run
  HostParams hp_;
  long long n_ = 0;
  int d_ = 0;
  HCall root_;                 // the root call (all points, nothing restricted)
  HLevel level1_;              // points and component orders of the level-1 calls
  std::vector<Phase> phases_;  // ranges of first restricted dims
  std::vector<int> phase_of_;  // phase of every first restricted dim
  std::vector<std::unique_ptr<Entry>> ents_;  // result map entries, in insertion order
  LabelBlocks labs_;                           // their label vectors
  BlockFiller filler_;                         // fills label blocks ahead of the commit
  std::vector<uint64_t> emask_;               // their subspaces
  std::map<uint64_t, int> eidx_;              // subspace -> entry
  std::vector<std::vector<uint64_t>> dim_bits_;  // per dim: bitset of the entries whose subspace holds it
  std::vector<int> sup_;                         // superset_candidates' result
  std::vector<int> prune_order_;                 // pruneRedundancy: superset entries by largest cluster
  std::vector<uint64_t> tbits_;               // region bitmap scratch
  std::vector<LoopVec> vbuf_;                  // one clustering vector per recursion depth
  std::vector<char> alive_;                    // join: clusters of the loop still alive
  std::vector<int> sdesc_, hsel_;              // join: alive clusters by size; superset entries tested
  std::vector<long long> spre_;                // join: prefix sums of those sizes
  std::vector<Walk> walk_, pieces_, split_;   // point ranges of the commit's loops
  std::unique_ptr<HostPool> hpool_;
  double t_prune_ = 0, t_cluster_ = 0, t_join_ = 0;
  long long* rc_ = nullptr;  // stats_.replay_counters
  inscy_stats stats_;
};

// ---------------------------------------------------------------------------
void Engine::run(const float* X, bool on_device, long long n, int d, const HostParams& hp, cudaStream_t s,
                 std::vector<std::vector<int>>& out_dims, LabelBlocks& out_labels, std::vector<int>& out_slots,
                 inscy_stats& st) {
  auto t_start = std::chrono::steady_clock::now();
  std::memset(&stats_, 0, sizeof(stats_));
  hp_ = hp;
  n_ = n;
  d_ = d;
  root_ = HCall();
  level1_ = HLevel();
  phases_.clear();
  phase_of_.clear();
  ents_.clear();
  emask_.clear();
  eidx_.clear();
  dim_bits_.assign(d, std::vector<uint64_t>());
  labs_.reset(n, n > 0 ? &filler_ : nullptr);
  out_dims.clear();
  out_slots.clear();
  out_labels.reset(n, nullptr);
  if (n == 0) {
    st = stats_;
    return;
  }
  const int ni = (int)n;
  const int cells = hp.cells;
  const bool rows_tma = rows_tma_requested();
  const int G = (int)std::ceil(1.0 / (double)hp.eps);  // inscy_map.cpp:243
  if (G > 256) throw Error(INSCY_ERR_LIMIT, "ceil(1/neighborhood_size) = " + std::to_string(G) + " > 256");
  const float csz = 1.0f / (float)cells;
  const float fsz = 1.0f / (float)G;
  // leaf keys pack one cell per dim into 128 bits
  int kbits = 1;
  while ((1 << kbits) < cells) ++kbits;
  if (d * kbits > 128)
    throw Error(INSCY_ERR_LIMIT, "d * ceil(log2(number_of_cells)) = " + std::to_string(d * kbits) + " > 128");
  const int W = (ni + 31) / 32;
  long long launches = 0;

  // thresholds: weak density uses all d dims (ScyTreeNode.cu:604-606), the
  // clustering density |S| (ClusteringCpu.cu:166-183).  A point that can be
  // dense in some descendant subspace has phi >= thr_keep at every prefix.
  std::vector<float> thr_dense(d + 2, 0.f), thr_keep(d + 2, 0.f);
  float thr_weak;
  if (hp.rect) {
    thr_weak = std::max(hp.F * expden_of(d, hp.eps, ni), (float)hp.num_obj);
    for (int k = 1; k <= d; ++k) thr_dense[k] = std::max(hp.F * expden_of(k, hp.eps, ni), (float)hp.num_obj);
  } else {
    thr_weak = std::max(hp.F * alpha_of(d, hp.eps, ni), (float)hp.num_obj * omega_of(d));
    for (int k = 1; k <= d; ++k)
      thr_dense[k] = std::max(hp.F * alpha_of(k, hp.eps, ni), (float)hp.num_obj * omega_of(k));
  }
  for (int k = 1; k <= d; ++k) {
    float t = thr_weak;
    for (int j = k; j <= d; ++j) t = std::min(t, thr_dense[j]);
    thr_keep[k] = t;
  }

  // eps >= sqrtf(acc) (ClusteringCpu.cu:72) holds exactly for acc <= acc_max:
  // correctly rounded sqrt is monotone, so the passing accs are a prefix of
  // the non-negative floats; find its last element by bisection on the bits
  float acc_max;
  {
    uint32_t lo = 0, hi = 0x7f800000u;  // [0, +inf)
    while (lo < hi) {
      uint32_t mid = lo + (hi - lo + 1) / 2;
      float x;
      std::memcpy(&x, &mid, 4);
      if (hp.eps >= std::sqrt(x))
        lo = mid;
      else
        hi = mid - 1;
    }
    std::memcpy(&acc_max, &lo, 4);
  }

  Scope persist(*pool_, s);
  // ------------------------------------------------------------------ setup
  auto t_setup0 = std::chrono::steady_clock::now();
  const float* dX = X;
  if (!on_device) {
    float* x = persist.get<float>((size_t)n * d);
    void* stg = pinned_.get((size_t)n * d * sizeof(float));
    std::memcpy(stg, X, (size_t)n * d * sizeof(float));
    CK(cudaMemcpyAsync(x, stg, (size_t)n * d * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the staging buffer is reused below
    stats_.h2d_bytes += (long long)n * d * sizeof(float);
    dX = x;
  } else {
    // device input: every value must be a number in [0, 1] (cell indices
    // index the per-dim buckets)
    int* bad = persist.get<int>(1);
    CK(cudaMemsetAsync(bad, 0, sizeof(int), s));
    launch_check_range(dX, (long long)n * d, bad, s);
    if (scalar(bad, s)) throw Error(INSCY_ERR_ARG, "X has a value outside [0, 1]");
  }
  uint8_t* dcc = persist.get<uint8_t>((size_t)n * d);
  uint8_t* dfc = persist.get<uint8_t>((size_t)n * d);
  unsigned long long* dgz = persist.get<unsigned long long>((size_t)n);
  float* dthr = persist.get<float>(2 * (d + 2));
  h2d(dthr, thr_dense.data(), sizeof(float) * (d + 2), s);
  h2d(dthr + d + 2, thr_keep.data(), sizeof(float) * (d + 2), s);
  // device-side consistency checks (code, offending value)
  long long* dguard = persist.get<long long>(2);
  CK(cudaMemsetAsync(dguard, 0, 2 * sizeof(long long), s));
  Guard guard{(int*)dguard, dguard + 1};
  auto check_guard = [&](const char* where) {
    long long g[2];
    d2h(g, dguard, sizeof(g), s);
    if ((int)g[0] != 0)
      throw Error(INSCY_ERR_INTERNAL, std::string("device check ") + std::to_string((int)g[0]) + " failed in " +
                                          where + " (value " + std::to_string(g[1]) + ")");
  };
  launch_prep(dX, ni, d, cells, csz, G, fsz, hp.eps, dcc, dfc, dgz, s);
  ++launches;
  // the SCY-tree's and the neighbourhood trie's level order
  std::vector<int> lvl_dim(d), lvl_pos(d);
  {
    std::vector<int> hist;
    if (hp.entropy_order != 0) {
      Scope tmp(*pool_, s);
      int* dh = tmp.get<int>((size_t)d * cells);
      CK(cudaMemsetAsync(dh, 0, sizeof(int) * (size_t)d * cells, s));
      launch_cell_hist(dcc, ni, d, cells, sms_, dh, s);
      ++launches;
      hist.resize((size_t)d * cells);
      d2h(hist.data(), dh, sizeof(int) * hist.size(), s);
    }
    lvl_dim = level_order_of(hist, ni, d, cells, hp.entropy_order);
    for (int t = 0; t < d; ++t) lvl_pos[lvl_dim[t]] = t;
  }
  // point rows for the density pass when a row fits 16, 24 or 32 slots
  float* dxrow = nullptr;
  float* dwin = nullptr;
  unsigned long long* dwork = persist.get<unsigned long long>(1);
  unsigned long long* dphiwork = persist.get<unsigned long long>(kPhiWorkBytes / 8);
  const int slots = kDensityRows ? row_slots(d) : 0;
  if (slots) {
    // fine_lo[k]: the least float x in [0, 1] whose fine cell before the cap,
    // (int)(x / fsz), is >= k (+inf if none); the cell is monotone in x, so
    // the +-1 fine-cell test becomes an interval test on the coordinate
    std::vector<float> fine_lo(G + 2);
    for (int k = 0; k <= G + 1; ++k) {
      auto reaches = [&](uint32_t b) {
        float x;
        std::memcpy(&x, &b, 4);
        return (int)(x / fsz) >= k;
      };
      const uint32_t one = 0x3f800000u;  // 1.0f: inputs lie in [0, 1]
      if (!reaches(one)) {
        fine_lo[k] = std::numeric_limits<float>::infinity();
        continue;
      }
      uint32_t lo = 0, hi = one;  // least b in [lo, hi] that reaches k
      while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (reaches(mid))
          hi = mid;
        else
          lo = mid + 1;
      }
      std::memcpy(&fine_lo[k], &lo, 4);
    }
    float* dfine = persist.get<float>(G + 2);
    h2d(dfine, fine_lo.data(), sizeof(float) * (G + 2), s);
    // n rows and a sentinel row n whose coordinates are all 3.4e38 (bytes
    // 0x7f): lanes past the end of a candidate list read it and, the square
    // of their difference overflowing to +inf, pass no distance test
    dxrow = persist.get<float>((size_t)(n + 1) * slots);
    dwin = persist.get<float>((size_t)n * slots * 2);
    launch_point_rows(dX, dfc, ni, d, slots, G, dfine, dxrow, dwin, s);
    CK(cudaMemsetAsync(dxrow + (size_t)n * slots, 0x7f, sizeof(float) * slots, s));
    ++launches;
  }
  int* drank = persist.get<int>(n);
  int* dbucket = persist.get<int>((size_t)n * d);
  int* dboff = persist.get<int>((size_t)d * (G + 1));
  long long* dcoff = persist.get<long long>((size_t)d * G + 1);
  int* dcand = nullptr;
  int* droot = nullptr;
  {
    Scope tmp(*pool_, s);
    int nb = (ni + kSortTile - 1) / kSortTile;
    int* hist = tmp.get<int>((size_t)256 * nb);
    int* htot = tmp.get<int>(1);
    int* starts = tmp.get<int>(257);
    void* sums = scan_sums(256LL * nb, s, tmp);
    int* a = tmp.get<int>(n);
    int* b = tmp.get<int>(n);
    // neighbourhood-trie leaf order: lexicographic fine cells, dims in
    // level order, ties by id -> LSD passes from the last level
    launch_iota(a, ni, s);
    ++launches;
    for (int t = d - 1; t >= 0; --t) {
      launch_byte_sort_pass(a, b, ni, dfc, d, lvl_dim[t], hist, htot, nullptr, sums, s);
      launches += 5;
      std::swap(a, b);
    }
    launch_scatter_rank(a, ni, drank, s);
    ++launches;
    // per-dim cell buckets, each in trie order
    for (int k = 0; k < d; ++k) {
      launch_byte_sort_pass(a, dbucket + (size_t)k * n, ni, dfc, d, k, hist, htot, starts, sums, s);
      launches += 6;
      CK(cudaMemcpyAsync(dboff + (size_t)k * (G + 1), starts, sizeof(int) * (G + 1), cudaMemcpyDeviceToDevice, s));
    }
    std::vector<int> hboff((size_t)d * (G + 1));
    d2h(hboff.data(), dboff, hboff.size() * sizeof(int), s);
    std::vector<long long> hcoff((size_t)d * G + 1);
    long long tot = 0;
    for (int k = 0; k < d; ++k)
      for (int c = 0; c < G; ++c) {
        hcoff[(size_t)k * G + c] = tot;
        const int* bo = hboff.data() + (size_t)k * (G + 1);
        for (int b2 = c - 1; b2 <= c + 1; ++b2)
          if (b2 >= 0 && b2 < G) tot += bo[b2 + 1] - bo[b2];
      }
    hcoff[(size_t)d * G] = tot;
    h2d(dcoff, hcoff.data(), hcoff.size() * sizeof(long long), s);
    dcand = persist.get<int>((size_t)tot);
    launch_candidate_lists(ni, d, G, dbucket, dboff, drank, dfc, dcoff, dcand, s);
    ++launches;
    // root SCY-tree leaf order: coarse cells in level order, ties by id
    launch_iota(a, ni, s);
    ++launches;
    for (int t = d - 1; t >= 0; --t) {
      launch_byte_sort_pass(a, b, ni, dcc, d, lvl_dim[t], hist, htot, nullptr, sums, s);
      launches += 5;
      std::swap(a, b);
    }
    droot = persist.get<int>(n);
    CK(cudaMemcpyAsync(droot, a, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
  }
  stats_.ms_setup = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_setup0).count();

  // ------------------------------------------------------------ expansion
  // The frontier of the expansion: the calls of one level (device
  // descriptors and the index of their host record) and what the next level
  // needs from this one.
  struct Frontier {
    int level = 0;
    std::vector<CallDesc> hcalls;
    std::vector<int> call_ids;       // host record of each call in its phase; -1: the root
    std::shared_ptr<Scope> pts_mem;  // the calls' points and detached chains
    int* d_pts = nullptr;
    int2* d_ghosts = nullptr;
    long long pts_total = 0, ghosts_total = 0;
    std::shared_ptr<Scope> prev_mem;     // this level's kept lists
    std::vector<long long> prev_kstart;  // kept-index start of every subspace of the level (+ the total)
    int* keep_ids = nullptr;
    long long* keep_loff = nullptr;
    int* keep_lcnt = nullptr;
    int2* lent = nullptr;      // this level's list entries (ListEnt)
    long long prev_total = 0;  // list entries
    long long prev_nkeep = 0;  // kept points
  };
  root_.npts = ni;
  phase_of_.assign(d, 0);
  for (int k = 0, d0 = 0; d0 < d; ++k) {
    static const int kPhaseDims[] = {1, 1, 1, 2, 3};  // then the rest
    Phase ph;
    ph.d0 = d0;
    ph.d1 = k < 5 ? std::min(d, d0 + kPhaseDims[k]) : d;
    for (int D = ph.d0; D < ph.d1; ++D) phase_of_[D] = k;
    d0 = ph.d1;
    phases_.push_back(std::move(ph));
  }
  const int nphases = (int)phases_.size();
  Frontier F1;
  {
    CallDesc c;
    c.pts_off = 0;
    c.ghost_off = 0;
    c.rmask = 0;
    c.npts = ni;
    c.f = 0;
    c.nghost = 0;
    c.sub = -1;
    c.child_sub = 0;
    c.nrestricted = 0;
    F1.hcalls.push_back(c);
    F1.call_ids.push_back(-1);
    F1.pts_mem.reset(new Scope(*pool_, s));
    F1.d_pts = droot;
    F1.d_ghosts = F1.pts_mem->get<int2>(1);
    F1.pts_total = n;
  }

  // Expands the frontier level by level (one level only for the root).  The
  // host records go to `phase` (at the root level: to the phase of each dim).
  auto expand = [&](int phase, Frontier& F, bool one_level) {
    while (!F.hcalls.empty()) {
      const int level = ++F.level;
      stats_.levels = std::max<long long>(stats_.levels, level);
      Scope lv(*pool_, s);  // this level's temporaries
      std::unique_ptr<Scope> keepmem(new Scope(*pool_, s));  // this level's kept lists (live one more level)

      // ---- 1. subspaces of this level: children of the calls' subspaces
      std::vector<SubDesc> subs;
      // the neighbourhood trie's walk (ScyTreeNode.cu:896-934) tests dim D of
      // parent dims pm + D only when pm, ascending, lies in level order and
      // D's level follows the last of them
      auto win_of = [&](uint64_t pm, int D) {
        int last = -1;
        for (uint64_t m = pm; m; m &= m - 1) {
          const int e = __builtin_ctzll(m);
          if (lvl_pos[e] <= last) return 0;
          last = lvl_pos[e];
        }
        return lvl_pos[D] > last ? 1 : 0;
      };
      std::map<int, int> child_base;  // parent subspace -> first child
      for (auto& c : F.hcalls) {
        auto it = child_base.find(c.sub);
        if (it == child_base.end()) {
          int base = (int)subs.size();
          child_base[c.sub] = base;
          uint64_t pm = c.rmask;
          int first = c.f;
          long long nq = c.sub < 0 ? n : F.prev_kstart[c.sub + 1] - F.prev_kstart[c.sub];
          long long qo = c.sub < 0 ? 0 : F.prev_kstart[c.sub];
          for (int D = first; D < d; ++D) {
            SubDesc S;
            S.mask = pm | (1ull << D);
            S.dim = D;
            S.nsub = __builtin_popcountll(S.mask);
            S.parent = c.sub;
            S.nquery = (int)nq;
            S.item_off = 0;
            S.query_off = qo;
            S.plist_base = 0;
            S.bitmap_off = 0;
            S.win = win_of(pm, D);
            S.pad = 0;
            subs.push_back(S);
          }
          c.child_sub = base;
        } else {
          c.child_sub = it->second;
        }
      }
      const int nsubs = (int)subs.size();
      long long nitems = 0;
      for (int i = 0; i < nsubs; ++i) {
        subs[i].item_off = nitems;
        subs[i].bitmap_off = (long long)i * 3 * W;
        nitems += subs[i].nquery;
      }
      stats_.subspaces += nsubs;
      SubDesc* dsubs = lv.get<SubDesc>(nsubs);
      h2d(dsubs, subs.data(), sizeof(SubDesc) * nsubs, s);

      // groups: the children of one parent subspace, walked child-fastest
      std::vector<GroupDesc> groups;
      long long ngroup_warps = 0;  // one warp per (group, query point)
      {
        long long wo = 0;
        for (int i = 0; i < nsubs;) {
          int j = i;
          while (j < nsubs && subs[j].parent == subs[i].parent) ++j;
          GroupDesc g;
          g.warp_off = wo;
          g.qwarp_off = ngroup_warps;
          g.sub_base = i;
          g.nchild = j - i;
          g.nquery = subs[i].nquery;
          g.nowin = 0;
          for (int c = i; c < j && c - i < 32; ++c)
            if (!subs[c].win) g.nowin |= (int)(1u << (c - i));
          wo += (long long)g.nchild * g.nquery;
          ngroup_warps += g.nquery;
          groups.push_back(g);
          i = j;
        }
        if (wo != nitems) throw Error(INSCY_ERR_INTERNAL, "work item count mismatch");
      }
      GroupDesc* dgroups = lv.get<GroupDesc>(groups.size());
      h2d(dgroups, groups.data(), sizeof(GroupDesc) * groups.size(), s);

      // ---- 2. neighbour counts of every (subspace, point)
      int* dcnt = lv.get<int>(nitems);
      uint8_t* dflags = lv.get<uint8_t>(nitems);
      unsigned* dbm = keepmem->get<unsigned>((size_t)nsubs * 3 * W);
      CK(cudaMemsetAsync(dbm, 0, sizeof(unsigned) * (size_t)nsubs * 3 * W, s));
      DensityLaunch DL;
      std::memset(&DL, 0, sizeof(DL));
      DL.subs = dsubs;
      DL.nsubs = nsubs;
      DL.nitems = nitems;
      DL.groups = dgroups;
      DL.ngroups = (int)groups.size();
      DL.X = dX;
      DL.fc = dfc;
      DL.n = ni;
      DL.d = d;
      DL.G = G;
      DL.eps = hp.eps;
      DL.rect = hp.rect;
      DL.acc_max = acc_max;
      DL.thr_weak = thr_weak;
      DL.thr_dense = dthr;
      DL.thr_keep = dthr + d + 2;
      DL.cand_off = dcoff;
      DL.cand_pts = dcand;
      DL.prev_keep = F.keep_ids;
      DL.prev_loff = F.keep_loff;
      DL.prev_lcnt = F.keep_lcnt;
      DL.prev_ent = F.lent;
      DL.cnt = dcnt;
      DL.flags = dflags;
      DL.bitmaps = dbm;
      DL.words = W;
      DL.prev_total = F.prev_total;
      DL.prev_nkeep = F.prev_nkeep;
      DL.total = 0;
      DL.guard = guard;
      unsigned long long* dcand_cnt = lv.get<unsigned long long>(3);
      CK(cudaMemsetAsync(dcand_cnt, 0, 3 * sizeof(unsigned long long), s));
      DL.cand_counter = dcand_cnt;
      DL.list_counter = dcand_cnt + 1;
      DL.out_counter = dcand_cnt + 2;
      DL.cap_base = nullptr;
      DL.cap_loff = nullptr;
      DL.xrow = dxrow;
      DL.win = dwin;
      DL.slots = slots;
      DL.work = dxrow ? dwork : nullptr;
      DL.items = nullptr;
      DL.phi_work = dphiwork;
      DL.sms = sms_;
      DL.rows_tma = rows_tma ? 1 : 0;
      {
        std::lock_guard<std::mutex> g(g_tune_m);
        auto it = g_tuned.find({device_, slots});
        const RowShape sh = it != g_tuned.end() && rows_tune_enabled() ? it->second : RowShape();
        DL.rows_takes = sh.takes;
        DL.rows_bps = sh.bps;
      }
      auto neighbours = [&](bool write) {
        if (level == 1) {
          launch_neighbours(DL, write, s);
        } else {
          if (DL.work) CK(cudaMemsetAsync(DL.work, 0, sizeof(unsigned long long), s));
          launch_neighbours_multi(DL, ngroup_warps, write, s);
        }
      };
      // algorithmic bytes of the candidate pass: per (subspace, point) 26 B (its
      // id, list offset and length, own coordinate and fine cell, count out);
      // per list entry read 8 B (id + partial distance; at level 1 id +
      // coordinate); per further (candidate, child subspace) test at levels
      // >= 2 the candidate's coordinate on that dim, 4 B (the row kernel tests
      // the fine cell as a window on the coordinate), or coordinate and fine
      // cell, 5 B (the general kernel); per entry written by the single pass 8 B
      auto count_bytes = [&](bool single) {
        unsigned long long nc[3];
        d2h(nc, dcand_cnt, sizeof(nc), s);
        stats_.candidates += (long long)nc[0];
        stats_.density_bytes += 26.0 * (double)nitems + 8.0 * (double)nc[1] +
                                (level == 1 ? 0.0 : (DL.xrow ? 4.0 : 5.0) * (double)nc[0]) +
                                (single ? 8.0 * (double)nc[2] : 0.0);
      };

      // ---- 3. ordered lists of every item, then densities and flags.  A
      // list is a subsequence of a known list (the parent's at levels >= 2,
      // the fine cell's candidates at level 1), so when those lengths bound
      // the level within the single-pass budget one pass tests and writes
      // (lists at capacity offsets); otherwise a count pass sizes the lists
      // exactly and a second pass writes them.
      long long* dloff = lv.get<long long>(nitems);
      long long* dtot = lv.get<long long>(2);
      void* sums = scan_sums(std::max(std::max(nitems, (long long)nsubs * W), ngroup_warps) + 1, s, lv);
      long long L = 0;
      int2* lent = nullptr;
      bool single = false;
      {
        // capacities: per (group, query) at levels >= 2, per item (the
        // candidate-list length) at level 1
        const long long ncap = level > 1 ? ngroup_warps : nitems;
        long long* cap = lv.get<long long>(ncap + 1);
        long long* cbase = lv.get<long long>(ncap + 1);
        if (level > 1) {
          if (DL.work) DL.items = lv.get<RowItem>(ngroup_warps);  // the row kernel's pair records
          launch_list_capacity(DL, ngroup_warps, cap, s);
        } else {
          launch_level1_capacity(DL, cap, s);
        }
        launch_exclusive_scan_ll(cap, cbase, ncap, dtot, sums, s);
        launches += 4;
        const long long capt = scalar(dtot, s);
        if (capt * 8 <= t_single_pass_bytes) {
          single = true;
          L = capt;
          lent = keepmem->get<int2>(L);
          DL.cap_base = cbase;
          DL.cap_loff = dloff;
          DL.ent = lent;
          DL.total = L;
          if (level > 1 && DL.work && !rows_tma) tune_rows(DL, slots, ngroup_warps, s, neighbours);
          const double ms1 = timed(s, [&] { neighbours(true); });
          stats_.ms_density += ms1;
          stats_.ms_density_pass1 += ms1;
          stats_.density_launches_pass1 += 1;
          ++launches;
          count_bytes(true);
          check_guard("density lists");
          DL.cap_base = nullptr;
          DL.cap_loff = nullptr;
          DL.cand_counter = DL.list_counter = DL.out_counter = nullptr;
          DL.loff = dloff;
          float* dphi = lv.get<float>(nitems);
          int* dperm = lv.get<int>(nitems);
          CK(cudaMemsetAsync(dphiwork, 0, kPhiWorkBytes, s));
          stats_.ms_density += timed(s, [&] { launch_density_flags(DL, dphi, dperm, s); });
          launches += hp.rect ? 1 : 5;
        }
      }
      if (!single) {
        const double ms1 = timed(s, [&] { neighbours(false); });
        stats_.ms_density += ms1;
        stats_.ms_density_pass1 += ms1;
        stats_.density_launches_pass1 += 1;
        ++launches;
        count_bytes(false);
        check_guard("density count");  // the counts size every later buffer
        DL.cand_counter = DL.list_counter = DL.out_counter = nullptr;
        launch_exclusive_scan_i2ll(dcnt, dloff, nitems, dtot, sums, s);
        launches += 3;
        L = scalar(dtot, s);
        lent = keepmem->get<int2>(L);
        DL.loff = dloff;
        DL.ent = lent;
        DL.total = L;
        float* dphi = lv.get<float>(nitems);
        int* dperm = lv.get<int>(nitems);
        CK(cudaMemsetAsync(dphiwork, 0, kPhiWorkBytes, s));
        stats_.ms_density += timed(s, [&] {
          neighbours(true);
          launch_density_flags(DL, dphi, dperm, s);
        });
        launches += hp.rect ? 2 : 6;
      }
      // kept items
      int* dkcnt = lv.get<int>(nitems);
      int* dkflag = lv.get<int>(nitems);
      long long* dkpos = lv.get<long long>(nitems + 1);
      launch_keep_counts(dcnt, dflags, nitems, dkcnt, dkflag, s);
      launch_exclusive_scan_i2ll(dkflag, dkpos, nitems, dtot + 1, sums, s);
      launches += 4;
      const long long K = scalar(dtot + 1, s);
      check_guard("density");
      // kept (subspace, point) pairs are indexed by int in the clustering
      // kernels (union-find parents, level-1 sort indices, member counts)
      if (K >= (long long)INT_MAX)
        throw Error(INSCY_ERR_LIMIT, "level " + std::to_string(level) + " keeps " + std::to_string(K) +
                                         " (subspace, point) pairs; the limit is 2^31 - 2");
      int* keep_ids = keepmem->get<int>(K);
      long long* keep_loff = keepmem->get<long long>(K);
      int* keep_lcnt = keepmem->get<int>(K);
      launch_keep_compact(dsubs, nsubs, nitems, dflags, dcnt, dkpos, dloff, F.keep_ids, keep_ids, keep_loff,
                          keep_lcnt, s);
      launches += 2;
      // kept-index start of every subspace
      long long* dkstart = keepmem->get<long long>(nsubs + 1);
      launch_gather_kstart(dsubs, nsubs, dkpos, nitems, K, dkstart, s);
      ++launches;
      std::vector<long long> kstart(nsubs + 1);
      d2h(kstart.data(), dkstart, sizeof(long long) * (nsubs + 1), s);
      // global rank of every kept bit: prefix of the kept-bitmap popcounts
      int* dkwr = keepmem->get<int>((size_t)nsubs * W + 1);
      {
        int* pc = lv.get<int>((size_t)nsubs * W + 1);
        launch_keep_popc(dbm, nsubs, W, pc, s);
        ++launches;
        int* dt = lv.get<int>(1);
        launch_exclusive_scan_int(pc, dkwr, (long long)nsubs * W, dt, sums, s);
        launches += 3;
      }

      // ---- 4. restrict / merge / prune of every (call, dim)
      const int ncalls = (int)F.hcalls.size();
      std::vector<long long> work_off(ncalls), work_scr;
      std::vector<int> items_big, items_small;  // work items by block size (see launch_tree_level)
      long long nwork = 0, scr = 0, pts_cap = 0, ghost_in = 0;
      int key_bits = 0;  // widest leaf key of the level: (remaining dims incl. D) x bits per cell
      for (int i = 0; i < ncalls; ++i) {
        key_bits = std::max(key_bits, (d - F.hcalls[i].nrestricted) * kbits);
        work_off[i] = nwork;
        int nd = d - F.hcalls[i].f;
        for (int t = 0; t < nd; ++t) {
          work_scr.push_back(scr);
          // keys (16 B) of points and chains, then ints (see k_tree_level)
          long long bytes = 16LL * (2LL * F.hcalls[i].npts + 2LL * F.hcalls[i].nghost) +
                            4LL * (3LL * F.hcalls[i].npts + 1 + 3LL * F.hcalls[i].nghost);
          scr += (bytes + 15) / 16 * 16;
        }
        for (int t = 0; t < nd; ++t)
          ((long long)F.hcalls[i].npts + F.hcalls[i].nghost > kTreeBig ? items_big : items_small)
              .push_back((int)(nwork + t));
        nwork += nd;
        pts_cap += (long long)F.hcalls[i].npts * nd;
        ghost_in += (long long)F.hcalls[i].nghost * nd;
      }
      int* ditems = nullptr;
      if (!items_big.empty()) {
        std::vector<int> both(items_big);
        both.insert(both.end(), items_small.begin(), items_small.end());
        ditems = lv.get<int>(both.size());
        h2d(ditems, both.data(), sizeof(int) * both.size(), s);
      }
      CallDesc* dcalls = lv.get<CallDesc>(ncalls);
      h2d(dcalls, F.hcalls.data(), sizeof(CallDesc) * ncalls, s);
      long long* dwork = lv.get<long long>(ncalls);
      h2d(dwork, work_off.data(), sizeof(long long) * ncalls, s);
      long long* dwscr = lv.get<long long>(nwork);
      h2d(dwscr, work_scr.data(), sizeof(long long) * nwork, s);
      char* dscr = lv.get<char>(scr);
      RegionRec* drecs = lv.get<RegionRec>((size_t)nwork * cells);
      int* dnrecs = lv.get<int>(nwork);
      std::unique_ptr<Scope> next_pts(new Scope(*pool_, s));
      int* dout_pts = next_pts->get<int>(pts_cap);
      unsigned long long* dtops = lv.get<unsigned long long>(2);
      int* derr = lv.get<int>(1);
      long long ghost_cap = std::max(1024LL, ghost_in + 2 * pts_cap);
      int2* dout_gh = nullptr;
      std::vector<RegionRec> recs;
      std::vector<int> nrecs(nwork);
      unsigned long long tops[2];
      for (int attempt = 0;; ++attempt) {
        dout_gh = next_pts->get<int2>(ghost_cap);
        CK(cudaMemsetAsync(dtops, 0, sizeof(unsigned long long) * 2, s));
        CK(cudaMemsetAsync(derr, 0, sizeof(int), s));
        TreeLaunch TL;
        TL.calls = dcalls;
        TL.ncalls = ncalls;
        TL.work_off = dwork;
        TL.nwork = (int)nwork;
        TL.pts_in = F.d_pts;
        TL.ghosts_in = F.d_ghosts;
        TL.cc = dcc;
        TL.gz = dgz;
        TL.n = ni;
        TL.d = d;
        TL.cells = cells;
        TL.min_size = hp.min_size;
        TL.kbits = kbits;
        TL.subs = dsubs;
        TL.bitmaps = dbm;
        TL.scratch = dscr;
        TL.work_scratch = dwscr;
        TL.recs = drecs;
        TL.nrecs = dnrecs;
        TL.out_pts = dout_pts;
        TL.out_pts_top = dtops;
        TL.out_pts_cap = pts_cap;
        TL.out_ghosts = dout_gh;
        TL.out_ghost_top = dtops + 1;
        TL.out_ghost_cap = ghost_cap;
        TL.err = derr;
        TL.pts_in_total = F.pts_total;
        TL.ghosts_in_total = F.ghosts_total;
        TL.guard = guard;
        // a work item's leaf key holds its call's remaining dims and D: the
        // level's widest key decides the key type
        TL.key_bytes = std::max(kTreeMinKeyBytes, key_bits <= 32 ? 4 : key_bits <= 64 ? 8 : 16);
        TL.items_big = ditems;
        TL.nbig = ditems ? (int)items_big.size() : 0;
        TL.items_small = ditems ? ditems + items_big.size() : nullptr;
        TL.nsmall = ditems ? (int)items_small.size() : 0;
        for (int k = 0; k < kMaxDims; ++k) {
          TL.lvl_pos[k] = (uint8_t)(k < d ? lvl_pos[k] : 0);
          TL.lvl_dim[k] = (uint8_t)(k < d ? lvl_dim[k] : 0);
          unsigned long long gt = 0;
          for (int e = k + 1; e < d; ++e) gt |= 1ull << lvl_pos[e];
          TL.gt_pos[k] = k < d ? gt : 0ull;
        }
        stats_.ms_tree += timed(s, [&] { launch_tree_level(TL, s); });
        launches += (TL.nbig > 0 && TL.nsmall > 0) ? 2 : 1;
        int err = scalar(derr, s);
        d2h(tops, dtops, sizeof(tops), s);
        if (err == 2 && attempt < 4) {
          ghost_cap = (long long)tops[1] + 1024;
          continue;
        }
        if (err) throw Error(INSCY_ERR_INTERNAL, "level kernel reported error " + std::to_string(err));
        check_guard("restrict/merge/prune");
        break;
      }
      recs.resize((size_t)nwork * cells);
      d2h(recs.data(), drecs, sizeof(RegionRec) * recs.size(), s);
      d2h(nrecs.data(), dnrecs, sizeof(int) * nwork, s);
      // algorithmic bytes of the level kernel: per (call, dim) work item and
      // point of the call its id, its cell on the dim and its s-connection
      // flags (4 + 1 + 8 B), per chain 8 B; per point and chain written 4 / 8 B
      stats_.tree_bytes += 13.0 * (double)pts_cap + 8.0 * (double)ghost_in + 4.0 * (double)tops[0] +
                           8.0 * (double)tops[1];

      // ---- 5. next level's calls (host records in the reference's order)
      std::vector<CallDesc> ncall;
      std::vector<int> ncall_ids, ncall_phase;
      for (int i = 0; i < ncalls; ++i) {
        int nd = d - F.hcalls[i].f;
        for (int t = 0; t < nd; ++t) {
          long long w = work_off[i] + t;
          for (int r = 0; r < nrecs[w]; ++r) {
            const RegionRec& R = recs[(size_t)w * cells + r];
            stats_.regions++;
            HRegion hr;
            hr.dim = R.dim;
            hr.passed = R.passed;
            hr.child = -1;
            if (R.passed) {
              CallDesc c;
              c.pts_off = R.pts_off;
              c.ghost_off = R.ghost_off;
              c.rmask = F.hcalls[i].rmask | (1ull << R.dim);
              c.npts = R.npts;
              c.f = R.dim + 1;
              c.nghost = R.nghost;
              c.sub = F.hcalls[i].child_sub + (R.dim - F.hcalls[i].f);
              c.child_sub = 0;
              c.nrestricted = F.hcalls[i].nrestricted + 1;
              ncall.push_back(c);
              HCall hc;
              hc.rmask = c.rmask;
              hc.f = c.f;
              hc.level = level;
              hc.npts = c.npts;
              hc.pts_off = c.pts_off;
              const int cp = phase < 0 ? phase_of_[R.dim] : phase;  // the root's restrictions start the phases
              hr.child = (int)phases_[cp].calls.size();
              ncall_ids.push_back(hr.child);
              ncall_phase.push_back(cp);
              phases_[cp].calls.push_back(hc);
            }
            (F.call_ids[i] < 0 ? root_ : phases_[phase].calls[F.call_ids[i]]).regions.push_back(hr);
          }
        }
      }
      stats_.calls += (long long)ncall.size();

      // ---- 6. clustering of the subspaces that gained calls
      if (phase >= 0 && (int)phases_[phase].levels.size() <= level) phases_[phase].levels.resize(level + 1);
      HLevel& hl = phase < 0 ? level1_ : phases_[phase].levels[level];
      if (!ncall.empty()) {
        hl.pts.resize(tops[0]);
        d2h(hl.pts.data(), dout_pts, sizeof(int) * tops[0], s);
        std::vector<uint8_t> clustered(nsubs, 0);
        std::vector<std::vector<int>> sub_calls(nsubs);
        for (size_t j = 0; j < ncall.size(); ++j) {
          clustered[ncall[j].sub] = 1;
          sub_calls[ncall[j].sub].push_back((int)j);
        }
        std::vector<int> clist, cslot(nsubs, -1), sc_off(1, 0), sc_list;
        for (int i = 0; i < nsubs; ++i)
          if (clustered[i]) {
            cslot[i] = (int)clist.size();
            clist.push_back(i);
            for (int j : sub_calls[i]) sc_list.push_back(j);
            sc_off.push_back((int)sc_list.size());
          }
        const int ncl = (int)clist.size();
        uint8_t* dcl = lv.get<uint8_t>(nsubs);
        h2d(dcl, clustered.data(), nsubs, s);
        int* dclist = lv.get<int>(ncl);
        h2d(dclist, clist.data(), sizeof(int) * ncl, s);
        int* dcslot = lv.get<int>(nsubs);
        h2d(dcslot, cslot.data(), sizeof(int) * nsubs, s);
        int* dscoff = lv.get<int>(sc_off.size());
        h2d(dscoff, sc_off.data(), sizeof(int) * sc_off.size(), s);
        int* dsclist = lv.get<int>(sc_list.size());
        h2d(dsclist, sc_list.data(), sizeof(int) * sc_list.size(), s);
        CallDesc* dncall = lv.get<CallDesc>(ncall.size());
        h2d(dncall, ncall.data(), sizeof(CallDesc) * ncall.size(), s);

        ClusterArgs CA;
        CA.nsubs = nsubs;
        CA.subs = dsubs;
        CA.kstart = dkstart;
        CA.keep_ids = keep_ids;
        CA.keep_loff = keep_loff;
        CA.keep_lcnt = keep_lcnt;
        CA.ent = lent;
        CA.bitmaps = dbm;
        CA.words = W;
        CA.keep_word_rank = dkwr;
        CA.clustered = dcl;
        CA.clustered_list = dclist;
        CA.nkeep = K;
        CA.n = ni;
        CA.uf = lv.get<int>(K + 1);
        CA.err = derr;
        CA.guard = guard;
        {
          int* sub_of = lv.get<int>(K + 1);
          launch_sub_of_keep(dkstart, nsubs, K, sub_of, s);
          ++launches;
          CA.sub_of = sub_of;
        }
        CK(cudaMemsetAsync(derr, 0, sizeof(int), s));
        int* is_root = lv.get<int>(K + 1);
        int* root_id = lv.get<int>(K + 1);
        int* comp = lv.get<int>(K + 1);
        int* root_of = lv.get<int>(K + 1);
        int* dsample = lv.get<int>(ncl + 1);
        uint8_t* ddom = lv.get<uint8_t>(K + 1);  // per kept point: in its subspace's dominant component
        int* dnc = lv.get<int>(1);
        long long ncomp = 0;
        std::vector<int> cbase(nsubs + 1);
        if (level == 1) {
          // one-dim subspaces: components are runs in coordinate order.  The
          // sort key holds the subspace in one byte: level 1 has d <= 64
          // subspaces
          if (nsubs > 256) throw Error(INSCY_ERR_INTERNAL, "level 1 has more than 256 subspaces");
          UfLevel1Scratch w;
          w.flag = lv.get<int>(K + 1);
          w.pos = lv.get<int>(K + 1);
          w.total = lv.get<int>(1);
          w.kidx = lv.get<int>(K + 1);
          w.kbytes = lv.get<uint8_t>(5 * (K + 1));
          w.perm0 = lv.get<int>(K + 1);
          w.perm1 = lv.get<int>(K + 1);
          w.hist = lv.get<int>(256 * ((K + kSortTile - 1) / kSortTile + 1));
          w.start = lv.get<int>(K + 1);
          w.runx = lv.get<int>(K + 1);
          w.runmin = lv.get<int>(K + 1);
          stats_.ms_cluster += timed(s, [&] {
            launch_uf_init(CA.uf, K, s);
            launch_uf_level1_count(CA, w, sums, s);
          });
          const int m = scalar(w.total, s);
          stats_.ms_cluster += timed(s, [&] {
            launch_uf_level1(CA, dX, d, dfc, acc_max, w, m, sums, s);
            launch_uf_flatten(CA, is_root, root_of, s);
            launch_exclusive_scan_int(is_root, root_id, K, dnc, sums, s);
          });
          launches += 40;
        } else {
          stats_.ms_cluster += timed(s, [&] {
            launch_uf_init(CA.uf, K, s);
            launch_uf_union(CA, ncl, dcslot, dsample, ddom, s);
            launch_uf_flatten(CA, is_root, root_of, s);
            launch_exclusive_scan_int(is_root, root_id, K, dnc, sums, s);
          });
          launches += 10;
        }
        ncomp = scalar(dnc, s);
        int* dcbase = lv.get<int>(nsubs + 1);
        launch_gather_cbase(dkstart, nsubs, root_id, K, (int)ncomp, dcbase, s);
        ++launches;
        d2h(cbase.data(), dcbase, sizeof(int) * (nsubs + 1), s);
        int* mcount = lv.get<int>(ncomp + 1);
        int* mfill = lv.get<int>(ncomp + 1);
        long long* moff = lv.get<long long>(ncomp + 1);
        int* bcount = lv.get<int>(ncomp + 1);
        int* bfill = lv.get<int>(ncomp + 1);
        long long* boff = lv.get<long long>(ncomp + 1);
        CK(cudaMemsetAsync(mcount, 0, sizeof(int) * (ncomp + 1), s));
        CK(cudaMemsetAsync(mfill, 0, sizeof(int) * (ncomp + 1), s));
        CK(cudaMemsetAsync(bcount, 0, sizeof(int) * (ncomp + 1), s));
        CK(cudaMemsetAsync(bfill, 0, sizeof(int) * (ncomp + 1), s));
        long long nslots2 = (long long)ncl * n * 2;
        int* slots = lv.get<int>(nslots2);
        CK(cudaMemsetAsync(slots, 0xff, sizeof(int) * nslots2, s));
        const int ovf_cap = 1 << 20;
        int2* ovf = lv.get<int2>(ovf_cap);
        int* novf = lv.get<int>(1);
        CK(cudaMemsetAsync(novf, 0, sizeof(int), s));
        long long* dmtot = lv.get<long long>(2);
        stats_.ms_cluster += timed(s, [&] {
          launch_comp_ids(CA, root_id, root_of, comp, mcount, s);
          launch_exclusive_scan_i2ll(mcount, moff, ncomp, dmtot, sums, s);
        });
        launches += 4;
        long long hm[2];
        d2h(hm, dmtot, sizeof(long long), s);
        int* members = lv.get<int>(hm[0] + 1);
        launch_members(CA, comp, moff, mfill, members, s);
        launches += 1;
        int hovf = 0;
        stats_.ms_cluster += timed(s, [&] { launch_borders(CA, comp, dcslot, slots, ovf, novf, ovf_cap, s); });
        launches += 1;
        hovf = scalar(novf, s);
        if (scalar(derr, s)) throw Error(INSCY_ERR_INTERNAL, "clustering kernels reported an error");
        check_guard("clustering");
        hovf = std::min(hovf, ovf_cap);
        launch_border_count(slots, nslots2, ovf, hovf, bcount, s);
        launch_exclusive_scan_i2ll(bcount, boff, ncomp, dmtot + 1, sums, s);
        launches += 5;
        long long hb;
        d2h(&hb, dmtot + 1, sizeof(long long), s);
        int* borders = lv.get<int>(hb + 1);
        launch_border_fill(slots, nslots2, ni, ovf, hovf, boff, bfill, borders, s);
        // components of each region in first-seed order
        int* firstpos = lv.get<int>(ncomp + 1);
        CK(cudaMemsetAsync(firstpos, 0x7f, sizeof(int) * (ncomp + 1), s));
        int* order = lv.get<int>(tops[0] + 1);
        int* order_cnt = lv.get<int>(ncall.size());
        stats_.ms_cluster += timed(s, [&] {
          launch_region_order(CA, ncl, comp, dcbase, dscoff, dsclist, dncall, dout_pts, firstpos, order, order_cnt, s);
        });
        launches += 3;
        // to the host
        std::vector<long long> hmoff(ncomp + 1), hboff(ncomp + 1);
        d2h(hmoff.data(), moff, sizeof(long long) * ncomp, s);
        hmoff[ncomp] = hm[0];
        d2h(hboff.data(), boff, sizeof(long long) * ncomp, s);
        hboff[ncomp] = hb;
        auto hmem = std::make_shared<IntBuf>(), hbor = std::make_shared<IntBuf>();
        hmem->resize(hm[0]);
        hbor->resize(hb);
        d2h(hmem->data(), members, sizeof(int) * hm[0], s);
        d2h(hbor->data(), borders, sizeof(int) * hb, s);
        std::vector<int> hocnt(ncall.size());
        long long* order_off = lv.get<long long>(ncall.size() + 1);
        long long* dot = lv.get<long long>(1);
        launch_exclusive_scan_i2ll(order_cnt, order_off, (long long)ncall.size(), dot,
                                   scan_sums((long long)ncall.size() + 1, s, lv), s);
        const long long norder_tot = scalar(dot, s);
        int* packed = lv.get<int>(norder_tot + 1);
        launch_pack_order(dncall, (int)ncall.size(), order, order_cnt, order_off, packed, s);
        launches += 4;
        hl.order.resize(norder_tot);
        d2h(hl.order.data(), packed, sizeof(int) * norder_tot, s);
        check_guard("component order");
        d2h(hocnt.data(), order_cnt, sizeof(int) * ncall.size(), s);
        std::vector<long long> hooff(ncall.size());
        d2h(hooff.data(), order_off, sizeof(long long) * ncall.size(), s);
        // one HSub per clustered subspace (component-local offsets)
        std::vector<int> csub_of(nsubs, -1);
        for (int i : clist) {
          HSub hs;
          long long c0 = cbase[i], c1 = cbase[i + 1];
          hs.moff.resize(c1 - c0 + 1);
          hs.boff.resize(c1 - c0 + 1);
          for (long long c = c0; c <= c1; ++c) {
            hs.moff[c - c0] = hmoff[c] - hmoff[c0];
            hs.boff[c - c0] = hboff[c] - hboff[c0];
          }
          hs.members = IntView{hmem->data() + hmoff[c0], (size_t)(hmoff[c1] - hmoff[c0])};
          hs.borders = IntView{hbor->data() + hboff[c0], (size_t)(hboff[c1] - hboff[c0])};
          hs.keep_m = hmem;
          hs.keep_b = hbor;
          Phase& sp = phases_[phase < 0 ? phase_of_[subs[i].dim] : phase];
          csub_of[i] = (int)sp.subs.size();
          sp.subs.push_back(std::move(hs));
        }
        for (size_t j = 0; j < ncall.size(); ++j) {
          HCall& hc = phases_[ncall_phase[j]].calls[ncall_ids[j]];
          hc.csub = csub_of[ncall[j].sub];
          hc.norder = hocnt[j];
          hc.order_off = hooff[j];
        }
      }

      // ---- 7. advance: this level's lists become the parent lists
      F.prev_mem.reset(keepmem.release());
      F.prev_kstart = kstart;
      F.keep_ids = keep_ids;
      F.keep_loff = keep_loff;
      F.keep_lcnt = keep_lcnt;
      F.lent = lent;
      F.prev_total = L;
      F.prev_nkeep = K;
      F.pts_total = (long long)tops[0];
      F.ghosts_total = (long long)tops[1];
      F.pts_mem.reset(next_pts.release());
      F.d_pts = dout_pts;
      F.d_ghosts = dout_gh;
      F.hcalls.swap(ncall);
      F.call_ids.swap(ncall_ids);
      lv.release();
      stats_.kernel_launches = launches;
      if (one_level) break;
    }
  };
  expand(-1, F1, true);  // level 1: every 1-dim subspace and the root's restrictions

  // ---------------------------------------------------------------- commit
  // A phase is committed on a second host thread as soon as its expansion is
  // done, while this thread drives the GPU through the next phase.
  if ((int)vbuf_.size() != d + 2) vbuf_.assign(d + 2, LoopVec());
  tbits_.assign(((size_t)n + 63) / 64, 0);
  t_prune_ = t_cluster_ = t_join_ = 0;
  rc_ = stats_.replay_counters;
  std::mutex mu;
  std::condition_variable cv;
  int ready = 0;
  bool stop = false;
  std::atomic<bool> commit_failed{false};
  std::exception_ptr commit_err;
  double ms_commit = 0;
  std::thread committer([&] {
    try {
      for (int k = 0; k < nphases; ++k) {
        {
          std::unique_lock<std::mutex> lk(mu);
          cv.wait(lk, [&] { return ready > k || stop; });
          if (stop) return;
        }
        auto t0 = std::chrono::steady_clock::now();
        for (int D = phases_[k].d0; D < phases_[k].d1; ++D) replay_root(D);
        ms_commit += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      }
    } catch (...) {
      commit_err = std::current_exception();
      commit_failed = true;
    }
  });
  try {
    for (int k = 0; k < nphases && !commit_failed; ++k) {
      Frontier F = F1;
      F.hcalls.clear();
      F.call_ids.clear();
      for (size_t i = 0; i < F1.hcalls.size(); ++i)
        if (phase_of_[__builtin_ctzll(F1.hcalls[i].rmask)] == k) {
          F.hcalls.push_back(F1.hcalls[i]);
          F.call_ids.push_back(F1.call_ids[i]);
        }
      expand(k, F, false);
      {
        std::lock_guard<std::mutex> lk(mu);
        ready = k + 1;
      }
      cv.notify_all();
    }
  } catch (...) {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    cv.notify_all();
    committer.join();
    throw;
  }
  F1 = Frontier();
  persist.release();
  CK(cudaStreamSynchronize(s));
  auto t_expanded = std::chrono::steady_clock::now();
  stats_.ms_expand = std::chrono::duration<double, std::milli>(t_expanded - t_start).count();
  committer.join();
  stats_.ms_commit_tail = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_expanded).count();
  if (slots) {
    std::lock_guard<std::mutex> g(g_tune_m);
    auto it = g_tuned.find({device_, slots});
    const RowShape sh = it != g_tuned.end() && rows_tune_enabled() ? it->second : RowShape();
    stats_.rows_takes = sh.takes > 0 ? sh.takes : 16;
    stats_.rows_blocks_per_sm = sh.bps > 0 ? sh.bps : rows_max_blocks_per_sm(slots);
  }
  if (commit_err) std::rethrow_exception(commit_err);
  stats_.ms_replay_prune = t_prune_;
  stats_.ms_replay_cluster = t_cluster_;
  stats_.ms_replay_join = t_join_;
  stats_.ms_replay = ms_commit;
  {
    // the result map's order (vec_cmp)
    std::map<std::vector<int>, int, SubspaceOrder> order;
    for (size_t i = 0; i < ents_.size(); ++i) order.emplace(dims_of(emask_[i]), (int)i);
    for (auto& kv : order) {
      out_dims.push_back(kv.first);
      out_slots.push_back(ents_[kv.second]->slot);
    }
  }
  out_labels = std::move(labs_);
  out_labels.filler = nullptr;
  labs_ = LabelBlocks();
  ents_.clear();
  emask_.clear();
  eidx_.clear();
  stats_.kernel_launches = launches;
  stats_.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  st = stats_;
}

// ---------------------------------------------------------------------------
// ordered commit (InscyNodeCpu.cu:159-235)
// ---------------------------------------------------------------------------
// the root's loop over dim D (InscyNodeCpu.cu:171-233 at the root): every
// region of the root on D, then join
void Engine::replay_root(int D) {
  const Phase& ph = phases_[phase_of_[D]];
  LoopVec& V = vbuf_[0];
  V.init(n_);
  V.clear();
  LoopState st;
  const uint64_t smask = 1ull << D;
  for (const HRegion& R : root_.regions) {
    if (R.dim != D || !R.passed) continue;
    replay(ph, R.child);
    auto t0 = std::chrono::steady_clock::now();
    bool ok = prune_redundancy(ph, ph.calls[R.child], smask);
    auto t1 = std::chrono::steady_clock::now();
    if (ok) cluster_into(ph, ph.calls[R.child], V, st);
    auto t2 = std::chrono::steady_clock::now();
    t_prune_ += std::chrono::duration<double, std::milli>(t1 - t0).count();
    t_cluster_ += std::chrono::duration<double, std::milli>(t2 - t1).count();
  }
  auto t3 = std::chrono::steady_clock::now();
  join(V, st, smask);
  t_join_ += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t3).count();
}

void Engine::replay(const Phase& ph, int ci) {
  const HCall& c = ph.calls[ci];
  const int f = c.f;
  const uint64_t rmask = c.rmask;
  const int depth = __builtin_popcountll(rmask);
  LoopVec& V = vbuf_[depth];
  V.init(n_);
  size_t ri = 0;
  const size_t nreg = c.regions.size();
  for (int D = f; D < d_; ++D) {
    const uint64_t smask = rmask | (1ull << D);
    LoopState st;
    V.clear();
    while (ri < nreg && c.regions[ri].dim == D) {
      const HRegion R = c.regions[ri++];
      if (!R.passed) continue;
      replay(ph, R.child);
      auto t0 = std::chrono::steady_clock::now();
      bool ok = prune_redundancy(ph, ph.calls[R.child], smask);
      auto t1 = std::chrono::steady_clock::now();
      if (ok) cluster_into(ph, ph.calls[R.child], V, st);
      auto t2 = std::chrono::steady_clock::now();
      t_prune_ += std::chrono::duration<double, std::milli>(t1 - t0).count();
      t_cluster_ += std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    auto t3 = std::chrono::steady_clock::now();
    join(V, st, smask);
    t_join_ += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t3).count();
  }
}

// pruneRedundancy (ScyTreeNode.cu:669-734): over result entries whose
// subspace contains S, the smallest cluster touching the region's points;
// the region is clustered unless the largest of these reaches |region| * r.
// The answer only depends on that maximum, so the scan stops as soon as it
// is decided; per entry the smallest touched cluster is found either by
// scanning the region's points or, for large regions, by walking the entry's
// clusters smallest-first against a bitmap of the region.
// the entries whose subspace contains `smask`, in insertion order: the AND of
// the per-dim entry bitsets over the dims of smask
const std::vector<int>& Engine::superset_candidates(uint64_t smask) {
  sup_.clear();
  const size_t nw = (ents_.size() + 63) / 64;
  for (size_t w = 0; w < nw; ++w) {
    uint64_t x = ~0ull;
    for (uint64_t m = smask; m && x; m &= m - 1) x &= dim_bits_[__builtin_ctzll(m)][w];
    while (x) {
      sup_.push_back((int)(w * 64 + __builtin_ctzll(x)));
      x &= x - 1;
    }
  }
  return sup_;
}

static void refresh_order(Entry& E) {
  if (!E.dirty) return;
  E.by_size.clear();
  for (int l = 0; l < (int)E.size.size(); ++l)
    if (E.size[l] > 0) E.by_size.push_back(l);
  std::stable_sort(E.by_size.begin(), E.by_size.end(), [&](int a, int b) { return E.size[a] < E.size[b]; });
  E.dirty = false;
}

bool Engine::prune_redundancy(const Phase& ph, const HCall& c, uint64_t smask) {
  const int* pts = level_of(ph, c).pts.data() + c.pts_off;
  const int m = c.npts;
  rc_[6]++;
  const double thr = (double)((float)m * hp_.r);
  const bool use_bits = (long long)m * 8 > n_;
  bool bits_set = false;  // the region's bitmap, built when first needed
  int max_min = 0;
  bool result = true;
  // An entry's minimum (its smallest cluster touching the region) is at most
  // its largest cluster, so an entry whose largest cluster is at or below
  // max_min cannot raise it and is skipped.  The answer depends only on the
  // maximum over the entries, not on their order: the entry with the largest
  // cluster goes first (it tends to set a high max_min at once), the others
  // in the order found.
  std::vector<int>& order = prune_order_;
  const std::vector<int>& sup = superset_candidates(smask);
  order.assign(sup.begin(), sup.end());
  if (order.size() > 1) {
    size_t top = 0;
    for (size_t t = 1; t < order.size(); ++t)
      if (ents_[order[t]]->maxsz > ents_[order[top]]->maxsz) top = t;
    std::swap(order[0], order[top]);
  }
  for (int i : order) {
    Entry& E = *ents_[i];
    if (E.maxsz <= max_min) continue;
    int mn = -1;
    if (!use_bits) {
      // the entry matters only if its minimum ends above max_min, so the scan
      // stops once the minimum so far is at or below it
      const int* lab = E.lab;
      const int* esz = E.size.data();
      int j = 0;
      for (; j < m; ++j) {
        if (j + 16 < m) __builtin_prefetch(lab + pts[j + 16]);  // random reads of an n-long vector
        const int l = lab[pts[j]];
        if (l >= 0) {
          const int v = esz[l];
          if (mn == -1 || v < mn) {
            mn = v;
            if (mn <= max_min) break;
          }
        }
      }
      rc_[7] += j < m ? j + 1 : m;
    } else {
      if (!bits_set) {
        for (int j = 0; j < m; ++j) tbits_[pts[j] >> 6] |= 1ull << (pts[j] & 63);
        bits_set = true;
      }
      refresh_order(E);
      for (int l : E.by_size) {
        bool hit = false;
        const HSub& hs = *E.src[l].hs;
        const int cp = E.src[l].comp;
        for (long long k = hs.moff[cp]; k < hs.moff[cp + 1]; ++k) {
          int q = hs.members[k];
          rc_[7]++;
          if (E.lab[q] == l && ((tbits_[q >> 6] >> (q & 63)) & 1ull)) {
            hit = true;
            break;
          }
        }
        if (hit) {
          mn = E.size[l];
          break;
        }
      }
    }
    if (mn > max_min) {
      max_min = mn;
      if (!(thr > (double)max_min * 1.0)) {
        result = false;
        break;
      }
    }
  }
  if (bits_set) std::fill(tbits_.begin(), tbits_.end(), 0ull);
  return max_min == 0 ? true : result;
}

// BFS numbering of INSCYClusteringImplCPUAll (ClusteringCpu.cu:317-389):
// components in the order their first dense seed appears, members get the
// next label, non-dense neighbours that are still -1 become -2.
void Engine::cluster_into(const Phase& ph, const HCall& c, LoopVec& V, LoopState& st) {
  const HSub& hs = ph.subs[c.csub];
  const int* order = level_of(ph, c).order.data() + c.order_off;
  // labels in first-seed order.  Components are disjoint, so no write below
  // changes another component's first member: all labels can be decided
  // before the writes.
  const int first = st.nlabels + 1;
  // three dependent random reads per component (its member range, its first
  // member, that member's label): each is prefetched a few components ahead
  // of its use, the next read in the chain once the previous one has landed
  const int* mem = hs.members.data();
  const long long* moff = hs.moff.data();
  const uint64_t* lv = V.gv.data();
  for (int t = 0; t < c.norder; ++t) {
    if (t + 16 < c.norder) __builtin_prefetch(moff + order[t + 16]);
    if (t + 8 < c.norder) __builtin_prefetch(mem + moff[order[t + 8]]);
    if (t + 4 < c.norder) {
      const long long a4 = moff[order[t + 4]];
      if (a4 < moff[order[t + 4] + 1]) __builtin_prefetch(lv + mem[a4]);
    }
    int comp = order[t];
    long long m0 = hs.moff[comp], m1 = hs.moff[comp + 1];
    if (m1 == m0) continue;
    if (V.get(hs.members[m0]) != -1) continue;  // already numbered in this dim loop
    ++st.nlabels;
    rc_[8]++;
    rc_[9] += hs.boff[comp + 1] - hs.boff[comp];
    st.ref.push_back(LabelRef{&hs, comp});
    st.size.push_back((int)(m1 - m0));
  }
  // The loop vector is read in two places only: the check above (a
  // component's first member) and join's redundancy test, which looks at
  // clusters of min_size points or more (smaller ones are dropped first).  So
  // those clusters get every member labelled and the others their first
  // member; the -2 marks of border points reach the result entry from the
  // component lists in join and are never read from the loop vector.
  // The other members of the clusters that join may test are written only if
  // join reads the loop vector (flush_pending): its test from the loop's side
  // does not.
  uint64_t* gv = V.gv.data();
  const uint64_t cur = V.cur;
  for (int label = first; label <= st.nlabels; ++label) {
    const int comp = st.ref[label].comp;
    const long long m0 = hs.moff[comp], m = hs.moff[comp + 1] - m0;
    gv[hs.members[m0]] = cur | (uint32_t)label;
    if (m >= hp_.min_size && m > 1) {
      st.pend.push_back(Walk{hs.members.data() + m0, 1, m, nullptr, label, 0.f});
      st.pend_work += m - 1;
    }
  }
}

// the loop-vector writes cluster_into left pending
void Engine::flush_pending(LoopVec& V, LoopState& st) {
  if (st.pend.empty()) return;
  uint64_t* gv = V.gv.data();
  const uint64_t cur = V.cur;
  auto write = [&](const Walk& w) {
    const uint64_t v = cur | (uint32_t)w.l;
    for (long long k = w.k0; k < w.k1; ++k) __atomic_store_n(&gv[w.mem[k]], v, __ATOMIC_RELAXED);
  };
  if (st.pend_work < kParallelWalk || hpool_->workers() == 0) {
    for (const Walk& w : st.pend) write(w);
  } else {
    pieces_.assign(st.pend.begin(), st.pend.end());
    split_pieces(st.pend_work);
    hpool_->run((int)split_.size(), [&](int i) { write(split_[i]); });
  }
  st.pend.clear();
  st.pend_work = 0;
}

// pieces_ cut into parts of about work / (4 * threads) entries (split_)
void Engine::split_pieces(long long work) {
  split_.clear();
  const long long part = std::max(4096LL, work / (4LL * (hpool_->workers() + 1)));
  for (const Walk& w : pieces_)
    for (long long k = w.k0; k < w.k1; k += part)
      split_.push_back(Walk{w.mem, k, std::min(w.k1, k + part), w.lab, w.l, w.hsz});
}

// join (util.cu:655-743): drop clusters below min_size, drop clusters a
// superset subspace already covers with a cluster more than r times larger,
// then insert the clustering or merge it into the subspace's entry (new
// labels offset by the old maximum + 1, -2 marks overwrite).  Works on whole
// clusters: the loop's labels are components with known sizes.
void Engine::join(LoopVec& V, LoopState& st, uint64_t smask) {
  const int nl = st.nlabels;
  if (nl == 0) return;
  rc_[0]++;
  std::vector<char>& alive = alive_;
  alive.assign(nl + 1, 0);
  int minsz = INT32_MAX;
  for (int l = 1; l <= nl; ++l)
    if (st.size[l] >= hp_.min_size) {
      alive[l] = 1;
      minsz = std::min(minsz, st.size[l]);
    }
  if (minsz == INT32_MAX) return;
  if (hp_.r >= 0.f) {
    // Only clusters of a superset entry larger than (smallest cluster here) * r
    // can drop anything (float comparisons as the reference).  Whether a
    // cluster here is dropped does not depend on the order of the tests, so
    // the points of all such clusters are tested together, split over the
    // host pool when there are many.
    walk_.clear();
    long long total = 0;
    // The same test from this loop's side: for a superset entry H, scan the
    // members of every alive cluster here small enough for H's largest
    // cluster to drop it.  Its cost (costB) is known from the clusters'
    // sizes; the cheaper side runs (both drop exactly the same clusters).
    sdesc_.clear();
    for (int l = 1; l <= nl; ++l)
      if (alive[l]) sdesc_.push_back(l);
    std::sort(sdesc_.begin(), sdesc_.end(), [&](int x, int y) { return st.size[x] < st.size[y]; });
    spre_.assign(sdesc_.size() + 1, 0);
    for (size_t t = 0; t < sdesc_.size(); ++t) spre_[t + 1] = spre_[t] + st.size[sdesc_[t]];
    // alive clusters (ascending size) with size * r < hmax: a prefix of sdesc_
    auto below = [&](int hmax) {
      size_t lo = 0, hi = sdesc_.size();
      while (lo < hi) {
        const size_t mid = (lo + hi) / 2;
        if ((float)st.size[sdesc_[mid]] * hp_.r < (float)hmax)
          lo = mid + 1;
        else
          hi = mid;
      }
      return lo;
    };
    long long costB = 0;
    hsel_.clear();
    for (int i : superset_candidates(smask)) {
      Entry& H = *ents_[i];
      rc_[4]++;
      if (!((float)minsz * hp_.r < (float)H.maxsz)) continue;
      hsel_.push_back(i);
      costB += spre_[below(H.maxsz)];
      refresh_order(H);
      for (int t = (int)H.by_size.size() - 1; t >= 0; --t) {
        const int l = H.by_size[t];
        const int hsz = H.size[l];
        if (!((float)minsz * hp_.r < (float)hsz)) break;
        const HSub& hs = *H.src[l].hs;
        const int cp = H.src[l].comp;
        const long long m = hs.moff[cp + 1] - hs.moff[cp];
        walk_.push_back(Walk{hs.members.data() + hs.moff[cp], 0, m, H.lab, l, (float)hsz});
        total += m;
      }
    }
    bool hit = false;
    const int* ssz = st.size.data();
    const float r = hp_.r;
    // the superset side also pays for the loop-vector writes left pending
    const long long costA = total + st.pend_work;
    if (costB < costA && costB < kParallelWalk) {
      rc_[5] += costB;
      for (int i : hsel_) {
        const Entry& H = *ents_[i];
        const size_t nb = below(H.maxsz);
        for (size_t t = 0; t < nb; ++t) {
          const int l = sdesc_[t];
          if (!alive[l]) continue;
          const float lsz = (float)ssz[l] * r;
          const HSub& hs = *st.ref[l].hs;
          const int cp = st.ref[l].comp;
          const int* mem = hs.members.data();
          for (long long k = hs.moff[cp]; k < hs.moff[cp + 1]; ++k) {
            const int h = H.lab[mem[k]];
            if (h >= 0 && lsz < (float)H.size[h]) {
              alive[l] = 0;
              hit = true;
              break;
            }
          }
        }
      }
    } else if (costB < costA && hpool_->workers() > 0) {
      // the loop's side on the host pool: one task per alive cluster (largest
      // first), which alone writes its own flag
      rc_[5] += costB;
      std::atomic<bool> any{false};
      const int nsd = (int)sdesc_.size();
      hpool_->run(nsd, [&](int t) {
        const int l = sdesc_[nsd - 1 - t];
        const float lsz = (float)ssz[l] * r;
        const HSub& hs = *st.ref[l].hs;
        const int cp = st.ref[l].comp;
        const int* mem = hs.members.data();
        for (int i : hsel_) {
          const Entry& H = *ents_[i];
          if (!(lsz < (float)H.maxsz)) continue;
          for (long long k = hs.moff[cp]; k < hs.moff[cp + 1]; ++k) {
            const int h = H.lab[mem[k]];
            if (h >= 0 && lsz < (float)H.size[h]) {
              alive[l] = 0;
              any.store(true, std::memory_order_relaxed);
              return;
            }
          }
        }
      });
      hit = any.load();
    } else if (total < kParallelWalk || hpool_->workers() == 0) {
      flush_pending(V, st);
      rc_[5] += total;
      // one thread: raise the size bar as clusters drop
      for (const Walk& w : walk_) {
        if (!((float)minsz * r < w.hsz)) continue;
        if (walk_test(w, V, ssz, r, alive.data())) {
          hit = true;
          minsz = INT32_MAX;
          for (int l = 1; l <= nl; ++l)
            if (alive[l]) minsz = std::min(minsz, st.size[l]);
          if (minsz == INT32_MAX) return;
        }
      }
    } else {
      flush_pending(V, st);
      rc_[5] += total;
      pieces_.assign(walk_.begin(), walk_.end());
      split_pieces(total);
      std::atomic<bool> any{false};
      hpool_->run((int)split_.size(), [&](int i) {
        if (walk_test(split_[i], V, ssz, r, alive.data())) any.store(true, std::memory_order_relaxed);
      });
      hit = any.load();
    }
    if (hit) {
      minsz = INT32_MAX;
      for (int l = 1; l <= nl; ++l)
        if (alive[l]) minsz = std::min(minsz, st.size[l]);
      if (minsz == INT32_MAX) return;
    }
  } else {
    flush_pending(V, st);
    for (int i : superset_candidates(smask)) {
      Entry& H = *ents_[i];
      rc_[4]++;
      bool hit = false;
      for (int l = 1; l <= nl; ++l) {
        if (!alive[l]) continue;
        const HSub& hs = *st.ref[l].hs;
        const int cp = st.ref[l].comp;
        for (long long k = hs.moff[cp]; k < hs.moff[cp + 1]; ++k) {
          const int q = hs.members[k];
          const int h = H.lab[q];
          rc_[5]++;
          if (h < 0) continue;
          const int c = V.get(q);
          if (c > 0 && alive[c] && (float)st.size[c] * hp_.r < (float)H.size[h]) {
            alive[c] = 0;
            hit = true;
          }
        }
      }
      if (hit) {
        minsz = INT32_MAX;
        for (int l = 1; l <= nl; ++l)
          if (alive[l]) minsz = std::min(minsz, st.size[l]);
        if (minsz == INT32_MAX) return;
      }
    }
  }
  Entry* E;
  int off = 0;
  auto it = eidx_.find(smask);
  if (it != eidx_.end()) {
    E = ents_[it->second].get();
    off = E->maxv + 1;  // m + 1 + label
  } else {
    std::unique_ptr<Entry> ne(new Entry());
    ne->mask = smask;
    ne->lab = labs_.take(ne->slot);  // all -1
    E = ne.get();
    rc_[1]++;
    eidx_[smask] = (int)ents_.size();
    const size_t e = ents_.size();
    for (auto& b : dim_bits_)
      if (b.size() * 64 <= e) b.push_back(0);
    for (uint64_t m = smask; m; m &= m - 1) dim_bits_[__builtin_ctzll(m)][e >> 6] |= 1ull << (e & 63);
    ents_.push_back(std::move(ne));
    emask_.push_back(smask);
    off = 0;
  }
  const int top = off + nl;
  if ((int)E->size.size() <= top) {
    E->size.resize(top + 1, 0);
    E->src.resize(top + 1, LabelRef{nullptr, -1});
  }
  // label sizes and sources, then the point writes: members of the live
  // clusters get their new label, border marks of every cluster overwrite
  // (util.cu:726-739); a relabelled point leaves its old cluster
  pieces_.clear();
  long long work = 0;
  for (int l = 1; l <= nl; ++l) {
    const HSub& hs = *st.ref[l].hs;
    const int cp = st.ref[l].comp;
    if (alive[l]) {
      const int nv = off + l;
      E->size[nv] += st.size[l];
      E->src[nv] = st.ref[l];
      rc_[2] += st.size[l];
      pieces_.push_back(Walk{hs.members.data() + hs.moff[cp], 0, hs.moff[cp + 1] - hs.moff[cp], nullptr, nv, 0.f});
      work += hs.moff[cp + 1] - hs.moff[cp];
    }
    rc_[3] += hs.boff[cp + 1] - hs.boff[cp];
    pieces_.push_back(Walk{hs.borders.data() + hs.boff[cp], 0, hs.boff[cp + 1] - hs.boff[cp], nullptr, -2, 0.f});
    work += hs.boff[cp + 1] - hs.boff[cp];
  }
  int* lab = E->lab;
  int* esz = E->size.data();
  if (work < kParallelWalk || hpool_->workers() == 0) {
    for (const Walk& w : pieces_) {
      if (w.l >= 0) {
        for (long long k = w.k0; k < w.k1; ++k) {
          const int p = w.mem[k];
          const int ov = lab[p];
          if (ov >= 0) esz[ov]--;
          lab[p] = w.l;
        }
      } else {
        for (long long k = w.k0; k < w.k1; ++k) {
          const int q = w.mem[k];
          const int ov = lab[q];
          if (ov >= 0) esz[ov]--;
          lab[q] = -2;
        }
      }
    }
  } else {
    // members of different clusters are disjoint and never border points;
    // a border point may be listed by several clusters, hence the exchange
    split_pieces(work);
    hpool_->run((int)split_.size(), [&](int i) {
      const Walk& w = split_[i];
      // the sizes of the labels overwritten, subtracted once per run of
      // equal old labels (the points of a piece mostly share one)
      int run_l = -1, run_n = 0;
      auto drop = [&](int ov) {
        if (ov < 0) return;
        if (ov != run_l) {
          if (run_n) __atomic_fetch_sub(&esz[run_l], run_n, __ATOMIC_RELAXED);
          run_l = ov;
          run_n = 0;
        }
        ++run_n;
      };
      if (w.l >= 0) {
        for (long long k = w.k0; k < w.k1; ++k) {
          const int p = w.mem[k];
          drop(lab[p]);
          lab[p] = w.l;
        }
      } else {
        for (long long k = w.k0; k < w.k1; ++k) drop(__atomic_exchange_n(&lab[w.mem[k]], -2, __ATOMIC_RELAXED));
      }
      if (run_n) __atomic_fetch_sub(&esz[run_l], run_n, __ATOMIC_RELAXED);
    });
  }
  // v_max over the whole vector: the largest label that still has points,
  // else the largest of -1/-2 present
  int mx = -100000, msz = 0;
  for (int l = (int)E->size.size() - 1; l >= 0; --l)
    if (E->size[l] > 0) {
      if (mx == -100000) mx = l;
      msz = std::max(msz, E->size[l]);
    }
  if (mx == -100000) {
    for (long long q = 0; q < n_; ++q) mx = std::max(mx, E->lab[q]);
  }
  E->maxv = mx;
  E->maxsz = msz;
  E->dirty = true;
}

}  // namespace inscy

// ===========================================================================
// C ABI
// ===========================================================================
struct inscy_result {
  long long n = 0;
  std::vector<std::vector<int>> dims;
  inscy::LabelBlocks labels;  // label rows of the clustered subspaces
  std::vector<int> slots;     // row of each clustered subspace, in the result map's order
  inscy_stats stats;
};

namespace {
thread_local std::string g_err;
thread_local std::unique_ptr<inscy::Engine> g_engine;
thread_local int g_engine_device = -1;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int check_params(int64_t n, int d, const inscy_params* p) {
  if (!p) return fail(INSCY_ERR_ARG, "params is NULL");
  if (n < 0) return fail(INSCY_ERR_ARG, "n < 0");
  if (n > 0x7fffffffLL) return fail(INSCY_ERR_LIMIT, "n > 2^31-1");
  if (d <= 0) return fail(INSCY_ERR_ARG, "d <= 0");
  if (d > 64) return fail(INSCY_ERR_LIMIT, "d > 64 (subspaces are 64-bit masks)");
  if (!(p->neighborhood_size > 0.f)) return fail(INSCY_ERR_ARG, "neighborhood_size must be > 0");
  if (p->number_of_cells <= 0) return fail(INSCY_ERR_ARG, "number_of_cells must be > 0");
  if (p->number_of_cells > 255) return fail(INSCY_ERR_LIMIT, "number_of_cells > 255");
  return INSCY_OK;
}

int run_common(const float* X, bool on_device, int64_t n, int d, const inscy_params* p, void* stream,
               inscy_result** out) {
  if (!out) return fail(INSCY_ERR_ARG, "out is NULL");
  *out = nullptr;
  int rc = check_params(n, d, p);
  if (rc) return rc;
  if (n > 0 && !X) return fail(INSCY_ERR_ARG, "X is NULL");
  if (!on_device) {
    for (long long i = 0; i < (long long)n * d; ++i)
      if (!(X[i] >= 0.f && X[i] <= 1.f)) return fail(INSCY_ERR_ARG, "X has a value outside [0, 1] (index " + std::to_string(i) + ")");
  }
  try {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (!g_engine || g_engine_device != dev) {
      g_engine.reset(new inscy::Engine());
      g_engine_device = dev;
    }
    inscy::HostParams hp;
    hp.eps = p->neighborhood_size;
    hp.F = p->F;
    hp.r = p->r;
    hp.num_obj = p->num_obj;
    hp.min_size = p->min_size;
    hp.cells = p->number_of_cells;
    hp.rect = p->rectangular ? 1 : 0;
    hp.entropy_order = p->entropy_order;
    std::unique_ptr<inscy_result> res(new inscy_result());
    res->n = n;
    g_engine->run(X, on_device, n, d, hp, (cudaStream_t)stream, res->dims, res->labels, res->slots, res->stats);
    *out = res.release();
    g_err.clear();
    return INSCY_OK;
  } catch (const inscy::Error& e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return fail(INSCY_ERR_CUDA, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(INSCY_ERR_INTERNAL, e.what());
  }
}
// Batch lanes: host threads that each own an engine (memory pool, events,
// commit thread) and a non-blocking CUDA stream, so that several datasets
// run at once -- their kernels overlap on the GPU and their commits on the
// host cores.  A lane takes the next dataset of the schedule when its last
// one is done.  The lanes stay parked between calls (engines keep their
// warmed pools); a call with another device or lane count replaces the set
// (the old lanes exit and free their engines).
struct BatchJob {
  const float* X;
  int64_t n;
  int d;
  inscy_result** out;
  int rc;
  std::string err;
};

class LanePool {
 public:
  LanePool(int device, int lanes) : device_(device), lanes_(lanes) {
    for (int i = 0; i < lanes; ++i) th_.emplace_back([this] { lane_main(); });
  }
  // the lanes exit; their engines (memory pools, streams) go with them
  ~LanePool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  int device() const { return device_; }
  int lanes() const { return lanes_; }
  void run(std::vector<BatchJob>& jobs, const inscy_params* p) {
    std::unique_lock<std::mutex> lk(m_);
    jobs_ = &jobs;
    p_ = p;
    next_ = 0;
    active_ = lanes_;
    ++gen_;
    cv_.notify_all();
    done_.wait(lk, [&] { return active_ == 0; });
    jobs_ = nullptr;
  }

 private:
  void lane_main() {
    cudaSetDevice(device_);
    const int hw = (int)std::thread::hardware_concurrency();
    inscy::t_pool_workers = std::max(0, std::min(7, hw / (2 * lanes_) - 1));
    inscy::t_single_pass_bytes = inscy::kSinglePassBytes / lanes_;
    cudaStream_t s = nullptr;
    const cudaError_t serr = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    long long seen = 0;
    for (;;) {
      std::vector<BatchJob>* jobs;
      const inscy_params* p;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) break;
        jobs = jobs_;
        p = p_;
      }
      for (;;) {
        const int i = next_.fetch_add(1);
        if (i >= (int)jobs->size()) break;
        BatchJob& j = (*jobs)[i];
        if (serr != cudaSuccess) {  // the lane has no stream: its datasets fail
          j.rc = INSCY_ERR_CUDA;
          j.err = std::string("lane stream: ") + cudaGetErrorString(serr);
          continue;
        }
        j.rc = run_common(j.X, false, j.n, j.d, p, s, j.out);
        if (j.rc) j.err = g_err;
      }
      std::lock_guard<std::mutex> lk(m_);
      if (--active_ == 0) done_.notify_all();
    }
    g_engine.reset();
    if (serr == cudaSuccess) cudaStreamDestroy(s);
  }
  int device_, lanes_;
  bool stop_ = false;
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  std::vector<BatchJob>* jobs_ = nullptr;
  const inscy_params* p_ = nullptr;
  std::atomic<int> next_{0};
  int active_ = 0;
  long long gen_ = 0;
};

std::mutex g_lanes_m;
LanePool* g_lanes = nullptr;  // the current lane set (not torn down at exit)

constexpr int kDefaultLanes = 4;
}  // namespace

extern "C" {

int inscy_run(const float* X, int64_t n, int d, const inscy_params* p, int mode, inscy_result** out) {
  (void)mode;
  return run_common(X, false, n, d, p, nullptr, out);
}

int inscy_run_device(const float* X_dev, int64_t n, int d, const inscy_params* p, int mode, void* stream,
                     inscy_result** out) {
  (void)mode;
  return run_common(X_dev, true, n, d, p, stream, out);
}

int inscy_run_batch_scheduled(const float* const* Xs, const int64_t* ns, const int* ds, int count,
                              const inscy_params* p, const int* order, int lanes, inscy_result** outs) {
  if (count < 0 || (count > 0 && (!Xs || !ns || !ds || !outs))) return fail(INSCY_ERR_ARG, "bad batch arguments");
  for (int i = 0; i < count; ++i) outs[i] = nullptr;  // on every failure below they stay NULL
  if (lanes < 1 || lanes > 64) return fail(INSCY_ERR_ARG, "lanes must be in [1, 64]");
  if (count == 0) return INSCY_OK;
  std::vector<char> seen(count, 0);
  std::vector<BatchJob> jobs(count);
  for (int k = 0; k < count; ++k) {
    const int i = order ? order[k] : k;
    if (i < 0 || i >= count || seen[i]) return fail(INSCY_ERR_ARG, "order is not a permutation of 0..count-1");
    seen[i] = 1;
    jobs[k] = BatchJob{Xs[i], ns[i], ds[i], &outs[i], 0, std::string()};
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(INSCY_ERR_CUDA, "cudaGetDevice failed");
  {
    std::lock_guard<std::mutex> g(g_lanes_m);  // one scheduled batch at a time per process
    if (!g_lanes || g_lanes->device() != dev || g_lanes->lanes() != lanes) {
      delete g_lanes;
      g_lanes = nullptr;
      g_lanes = new LanePool(dev, lanes);
    }
    g_lanes->run(jobs, p);
  }
  for (const BatchJob& j : jobs)
    if (j.rc) {
      for (int i = 0; i < count; ++i) {
        delete outs[i];
        outs[i] = nullptr;
      }
      return fail(j.rc, j.err);
    }
  g_err.clear();
  return INSCY_OK;
}

int inscy_run_batch(const float* const* Xs, const int64_t* ns, const int* ds, int count, const inscy_params* p,
                    int mode, inscy_result** outs) {
  if (mode == INSCY_MODE_BATCHED)
    return inscy_run_batch_scheduled(Xs, ns, ds, count, p, nullptr, std::max(1, std::min(kDefaultLanes, count)), outs);
  if (count < 0 || (count > 0 && (!Xs || !ns || !ds || !outs))) return fail(INSCY_ERR_ARG, "bad batch arguments");
  for (int i = 0; i < count; ++i) outs[i] = nullptr;
  for (int i = 0; i < count; ++i) {
    int rc = inscy_run(Xs[i], ns[i], ds[i], p, mode, &outs[i]);
    if (rc) {
      for (int j = 0; j < i; ++j) {
        delete outs[j];
        outs[j] = nullptr;
      }
      return rc;
    }
  }
  return INSCY_OK;
}

int inscy_result_count(const inscy_result* r) { return r ? (int)r->dims.size() : 0; }
int64_t inscy_result_n(const inscy_result* r) { return r ? r->n : 0; }

int inscy_result_subspace(const inscy_result* r, int i, int* dims, int cap) {
  if (!r || i < 0 || i >= (int)r->dims.size() || (cap > 0 && !dims)) return -1;
  const auto& v = r->dims[i];
  for (int k = 0; k < (int)v.size() && k < cap; ++k) dims[k] = v[k];
  return (int)v.size();
}

int inscy_result_labels(const inscy_result* r, int i, int32_t* out) {
  if (!r || !out || i < 0 || i >= (int)r->slots.size()) return fail(INSCY_ERR_ARG, "bad result index");
  std::memcpy(out, r->labels.row(r->slots[i]), sizeof(int32_t) * (size_t)r->n);
  return INSCY_OK;
}

int inscy_result_stats(const inscy_result* r, inscy_stats* out) {
  if (!r || !out) return fail(INSCY_ERR_ARG, "NULL argument");
  *out = r->stats;
  return INSCY_OK;
}

void inscy_result_free(inscy_result* r) { delete r; }

const char* inscy_last_error(void) { return g_err.c_str(); }

const char* inscy_version(void) { return "inscy_gb300 0.1"; }

int64_t inscy_selftest(int64_t count) {
  try {
    unsigned long long* d = nullptr;
    CK(cudaMalloc(&d, sizeof(unsigned long long)));
    CK(cudaMemset(d, 0, sizeof(unsigned long long)));
    inscy::launch_phi_selftest((unsigned long long)count, 0x5eedull, d, 0);
    CK(cudaGetLastError());
    unsigned long long bad = 0;
    CK(cudaMemcpy(&bad, d, sizeof(bad), cudaMemcpyDeviceToHost));
    cudaFree(d);
    g_err.clear();
    return (int64_t)bad;
  } catch (const inscy::Error& e) {
    fail(e.code, e.what());
    return -1;
  }
}

const int32_t* inscy_result_labels_ptr(const inscy_result* r, int i) {
  if (!r || i < 0 || i >= (int)r->slots.size()) return nullptr;
  return r->labels.row(r->slots[i]);
}

int inscy_result_subspaces(const inscy_result* r, int32_t* dims, int cap, int32_t* lens) {
  if (!r || !lens || (cap > 0 && !dims)) return -1;
  int w = 0;
  for (size_t i = 0; i < r->dims.size(); ++i) {
    lens[i] = (int32_t)r->dims[i].size();
    for (int v : r->dims[i])
      if (w < cap) dims[w++] = v;
  }
  return w;
}

int inscy_result_label_blocks(const inscy_result* r, int* rows) {
  if (!r) return -1;
  if (rows) *rows = r->labels.rows;
  return (int)r->labels.blocks.size();
}

const int32_t* inscy_result_label_block(const inscy_result* r, int b) {
  if (!r || b < 0 || b >= (int)r->labels.blocks.size()) return nullptr;
  return r->labels.blocks[b].get();
}

int inscy_result_label_slots(const inscy_result* r, int32_t* slots) {
  if (!r || (!slots && !r->slots.empty())) return fail(INSCY_ERR_ARG, "NULL argument");
  for (size_t i = 0; i < r->slots.size(); ++i) slots[i] = r->slots[i];
  return INSCY_OK;
}

}  // extern "C"
