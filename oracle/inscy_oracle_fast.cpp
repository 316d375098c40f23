// INSCY CPU oracle, fast form -- TEST INFRASTRUCTURE ONLY.
//
// A second restatement of the reference CPU INSCY path (`CPU()` ->
// `run_cpu3_weak` -> `INSCYCPU3Weak`, InscyNodeCpu.cu:159-235) with the same
// decisions, orders and float operations as inscy_oracle.cpp, organised so
// that the workloads of tens of thousands to a hundred thousand points finish
// in minutes.  It is the checker for the CUDA implementation at those sizes:
// only tests/, the fixture scripts under tests/golden/ and bench.py's CPU leg
// load it.  Pinned, like inscy_oracle.cpp, against the reference's own
// outputs in tests/golden/, and cross-checked against inscy_oracle.cpp.
//
// What is organised differently (and why the result is the same):
//
//  * The SCY-tree is the same trie (ScyTreeNode.cu:22-143) with the same
//    restrict / mergeNodes / get_leafs / propergate_count2 rules
//    (ScyTreeNode.cu:227-379, 422-467, 803-851), held in one node array per
//    tree with sibling lists ordered by cell, the order std::map iteration
//    gives the reference.
//
//  * Neighbourhoods.  The reference walks the whole neighbourhood trie per
//    query (ScyTreeNode.cu:896-946) and keeps the points within +-1 fine cell
//    on the matched dims, in trie leaf order; `neighborhood` then keeps those
//    within eps (ClusteringCpu.cu:52-81).  A call's subspace S+[D] extends its
//    parent's S by its largest dim, the matched dims of S+[D] are those of S
//    plus at most D, and the float sum of squares over S+[D] is the one over
//    S plus the D term (the dims are summed in ascending order, :40-50), which
//    can only grow.  So the neighbour list of p in S+[D] is the ordered
//    subsequence of its list in S that passes the cell test on D and the eps
//    test on the extended sum.  Each call keeps, for every point of its
//    region, its list as (neighbour, partial sum of squares) pairs, and its
//    children derive theirs from them.  One-dim subspaces start from the three
//    fine-cell buckets around p, merged in trie order.  Points outside every
//    ancestor region (met by the clustering walk) start from those buckets.
//
//  * Clustering (INSCYClusteringImplCPUAll, ClusteringCpu.cu:317-389) walks
//    the queue one BFS level at a time: the density of every point of a level
//    is a pure function of (point, subspace) and is evaluated in parallel; the
//    label writes and queue pushes then run in the queue's order, so labels
//    and their numbering are those of the sequential walk.
//
//  * Independent work (the restricts of a call, the per-point lists and
//    sums of a prune) runs on a thread pool; the DFS order of every commit
//    step (pruneRedundancy, clustering, join) is the reference's.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "oracle_common.h"

namespace {

using namespace orc_common;

// ------------------------------------------------------------------------
// Thread pool: run(count, grain, fn) calls fn(begin, end) over [0, count)
// in chunks of `grain`, on the caller and the workers.
// ------------------------------------------------------------------------
class Pool {
 public:
  explicit Pool(int threads) {
    for (int i = 1; i < threads; ++i) workers_.emplace_back([this] { loop(); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }
  int size() const { return (int)workers_.size() + 1; }

  void run(int count, int grain, const std::function<void(int, int)>& fn) {
    if (count <= 0) return;
    if (grain < 1) grain = 1;
    if (workers_.empty() || count <= grain) {
      fn(0, count);
      return;
    }
    // Each run has its own claim counter: a worker that wakes late takes the
    // job current at that moment, and a job whose counter is exhausted hands
    // out nothing (its function is never called again).
    auto job = std::make_shared<Job>();
    job->fn = &fn;
    job->count = count;
    job->grain = grain;
    {
      std::lock_guard<std::mutex> lk(mu_);
      cur_ = job;
      ++gen_;
    }
    cv_.notify_all();
    work(*job);
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return running_ == 0; });
    cur_.reset();
  }

 private:
  struct Job {
    const std::function<void(int, int)>* fn = nullptr;
    int count = 0, grain = 1;
    std::atomic<int> next{0};
  };
  static void work(Job& j) {
    for (;;) {
      int b = j.next.fetch_add(j.grain);
      if (b >= j.count) break;
      (*j.fn)(b, std::min(j.count, b + j.grain));
    }
  }
  void loop() {
    long long seen = 0;
    for (;;) {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      std::shared_ptr<Job> job = cur_;
      if (!job) continue;
      ++running_;
      lk.unlock();
      work(*job);
      lk.lock();
      if (--running_ == 0) done_.notify_all();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  std::shared_ptr<Job> cur_;
  long long gen_ = 0;
  int running_ = 0;
  bool stop_ = false;
};

// ------------------------------------------------------------------------
// SCY-tree as a node array (Node.h:15-60, ScyTreeNode.cu)
// ------------------------------------------------------------------------
struct TN {
  int cell;
  int count;          // -1 marks an s-connection node
  int kid = -1;       // first child (children in ascending cell order)
  int sc = -1;        // first s-connection
  int next = -1;      // next sibling
  int pb = 0, pn = 0;  // its points: Trie::flat[pb .. pb + pn)
  bool leaf = false;
};

struct Trie {
  std::vector<TN> nd;                // nd[0] is the root
  std::vector<int> flat;             // the nodes' point lists
  std::vector<int> levels;           // dims still in the trie, in level order
  std::vector<int> restricted;       // restricted dims, in restriction order
  int cells = 0;
  float cell_size = 0.f;
  bool sconnected = false;
  int npts = 0;

  Trie() { nd.push_back(TN{-1, 0}); }
  int add(int cell, int count) {
    nd.push_back(TN{cell, count});
    return (int)nd.size() - 1;
  }
  const int* pts(int v) const { return flat.data() + nd[v].pb; }
  // appends src[0 .. len) to the points of v (v's list moves to the end of
  // `flat` first when something follows it there)
  void append_pts(int v, const int* src, int len) {
    if (len <= 0) return;
    TN& t = nd[v];
    if (t.pn > 0 && t.pb + t.pn != (int)flat.size()) {
      const int old = t.pb;
      t.pb = (int)flat.size();
      flat.insert(flat.end(), flat.begin() + old, flat.begin() + old + t.pn);
    } else if (t.pn == 0) {
      t.pb = (int)flat.size();
    }
    flat.insert(flat.end(), src, src + len);
    nd[v].pn += len;
  }
};

int find_child(const Trie& T, int head, int cell) {
  for (int c = head; c != -1; c = T.nd[c].next) {
    if (T.nd[c].cell == cell) return c;
    if (T.nd[c].cell > cell) return -1;
  }
  return -1;
}

// Links x into the (s-connection) children of p in cell order.  Like
// std::map::emplace, nothing is linked when p already has that cell.
bool link(Trie& T, int p, int x, bool sconn) {
  const int cell = T.nd[x].cell;
  int prev = -1, c = sconn ? T.nd[p].sc : T.nd[p].kid;
  while (c != -1 && T.nd[c].cell < cell) {
    prev = c;
    c = T.nd[c].next;
  }
  if (c != -1 && T.nd[c].cell == cell) return false;
  T.nd[x].next = c;
  if (prev == -1)
    (sconn ? T.nd[p].sc : T.nd[p].kid) = x;
  else
    T.nd[prev].next = x;
  return true;
}

void unlink_cell(Trie& T, int p, int cell, bool sconn) {
  int prev = -1, c = sconn ? T.nd[p].sc : T.nd[p].kid;
  while (c != -1 && T.nd[c].cell != cell) {
    prev = c;
    c = T.nd[c].next;
  }
  if (c == -1) return;
  if (prev == -1)
    (sconn ? T.nd[p].sc : T.nd[p].kid) = T.nd[c].next;
  else
    T.nd[prev].next = T.nd[c].next;
}

int child_of(Trie& T, int p, int cell, bool sconn) {
  int c = find_child(T, sconn ? T.nd[p].sc : T.nd[p].kid, cell);
  if (c != -1) return c;
  int x = T.add(cell, sconn ? -1 : 0);
  link(T, p, x, sconn);
  return x;
}

// ScyTreeNode(X, subspace, cells, ...) constructor, ScyTreeNode.cu:105-143,
// with construct_s_connection (:34-49).
void build_trie(const Data& D, int cells, Trie& T) {
  T.cells = cells;
  T.cell_size = 1.0f / (float)cells;
  T.levels = D.order;
  const int m = (int)T.levels.size();
  std::map<int, std::vector<int>> leaf_pts;
  for (int i = 0; i < D.n; ++i) {
    T.nd[0].count += 1;
    int node = 0;
    for (int j = 0; j < m; ++j) {
      float xij = D.x(i, T.levels[j]);
      int c = cell_no(xij, T.cell_size, cells);
      int ch = child_of(T, node, c, false);
      T.nd[ch].count += 1;
      if (xij >= ((float)(c + 1) * T.cell_size - D.eps)) {
        int s = child_of(T, node, c, true);
        for (int k = j + 1; k < m; ++k) s = child_of(T, s, cell_no(D.x(i, T.levels[k]), T.cell_size, cells), true);
        T.nd[s].leaf = true;
      }
      node = ch;
    }
    leaf_pts[node].push_back(i);
    T.nd[node].leaf = true;
  }
  T.npts = T.nd[0].count;
  for (auto& kv : leaf_pts) T.append_pts(kv.first, kv.second.data(), (int)kv.second.size());
}

// restrict_node, ScyTreeNode.cu:227-323 (same branches as inscy_oracle.cpp)
bool restrict_node(const Trie& T, int old, Trie& R, int np, int dim, int cell, int depth, bool& sflag) {
  const TN& o = T.nd[old];
  if (T.levels[depth] == dim) {
    if (o.cell != cell) return false;
    if (R.nd[np].count != -1 && o.count == -1) {
      sflag = true;
      return false;
    }
    if (o.leaf) {
      R.nd[np].leaf = true;
      if (o.count > 0) {
        R.append_pts(np, T.pts(old), o.pn);
        R.nd[np].count += o.count;
      }
      return true;
    }
    for (int c = o.kid; c != -1; c = T.nd[c].next) restrict_node(T, c, R, np, dim, cell, depth + 1, sflag);
    for (int c = o.sc; c != -1; c = T.nd[c].next) restrict_node(T, c, R, np, dim, cell, depth + 1, sflag);
    return true;
  }
  // copy of old (Node(shared_ptr<Node>), Node.h:33-38); when it ends up not
  // included, it and everything made below it are dropped again
  const size_t mark_nd = R.nd.size(), mark_flat = R.flat.size();
  const int nn = R.add(o.cell, o.count);
  R.nd[nn].leaf = o.leaf;
  R.append_pts(nn, T.pts(old), o.pn);
  bool inc = T.levels[depth] > dim;
  if (o.count == -1) {
    for (int c = o.sc; c != -1; c = T.nd[c].next) inc = restrict_node(T, c, R, nn, dim, cell, depth + 1, sflag) || inc;
    if (inc) link(R, np, nn, true);
  } else {
    if (!o.leaf)
      R.nd[nn].count = 0;
    else
      inc = true;
    for (int c = o.kid; c != -1; c = T.nd[c].next) inc = restrict_node(T, c, R, nn, dim, cell, depth + 1, sflag) || inc;
    for (int c = o.sc; c != -1; c = T.nd[c].next) inc = restrict_node(T, c, R, nn, dim, cell, depth + 1, sflag) || inc;
    if (inc) {
      const int add = R.nd[nn].count;
      link(R, np, nn, false);
      R.nd[np].count += add;
    }
  }
  if (!inc) {
    R.nd.resize(mark_nd);
    R.flat.resize(mark_flat);
  }
  return inc;
}

constexpr int kMaxAllCells = 64;

// What restrict_node(T, old, R, np, dim, c, depth, sflag) returns, for every
// cell c of `dim` at once, as a bit mask; `parent_sconn` tells whether np is an
// s-connection copy (count -1).  Read-only: sets sflag[c] where restrict_node
// would, and records the masks of the nodes above the restricted level.
uint64_t include_mask(const Trie& T, int old, int dim, int depth, bool parent_sconn, bool* sflag,
                      std::vector<uint64_t>& mask) {
  const TN& o = T.nd[old];
  const uint64_t all = (T.cells >= 64) ? ~0ull : ((1ull << T.cells) - 1);
  uint64_t m;
  if (T.levels[depth] == dim) {
    if (o.cell < 0 || o.cell >= T.cells) return 0;
    if (!parent_sconn && o.count == -1) {
      sflag[o.cell] = true;
      return 0;
    }
    return 1ull << o.cell;
  }
  m = T.levels[depth] > dim ? all : 0;
  if (o.count == -1) {
    for (int k = o.sc; k != -1; k = T.nd[k].next) m |= include_mask(T, k, dim, depth + 1, true, sflag, mask);
  } else {
    if (o.leaf) m = all;
    for (int k = o.kid; k != -1; k = T.nd[k].next) m |= include_mask(T, k, dim, depth + 1, false, sflag, mask);
    for (int k = o.sc; k != -1; k = T.nd[k].next) m |= include_mask(T, k, dim, depth + 1, false, sflag, mask);
  }
  mask[old] = m;
  return m;
}

// restrict_node for every cell of `dim` in one walk: out[c] receives what
// restrict_node(T, old, *out[c], np[c], dim, c, depth, sflag) gives it.
// Above the restricted level a node is copied into exactly the outputs whose
// bit include_mask set; at that level only the output of the node's own cell
// sees it.
void restrict_node_all(const Trie& T, int old, Trie* const* out, const int* np, int dim, int depth,
                       const std::vector<uint64_t>& mask) {
  const TN& o = T.nd[old];
  const int cells = T.cells;
  if (T.levels[depth] == dim) {
    if (o.cell >= 0 && o.cell < cells) {
      bool sflag = false;
      restrict_node(T, old, *out[o.cell], np[o.cell], dim, o.cell, depth, sflag);
    }
    return;
  }
  const uint64_t m = mask[old];
  if (!m) return;
  int nn[kMaxAllCells];
  for (int c = 0; c < cells; ++c) {
    if (!(m >> c & 1)) continue;
    Trie& R = *out[c];
    nn[c] = R.add(o.cell, o.count);
    R.nd[nn[c]].leaf = o.leaf;
    R.append_pts(nn[c], T.pts(old), o.pn);
    if (o.count != -1 && !o.leaf) R.nd[nn[c]].count = 0;
  }
  if (o.count == -1) {
    for (int k = o.sc; k != -1; k = T.nd[k].next) restrict_node_all(T, k, out, nn, dim, depth + 1, mask);
    for (int c = 0; c < cells; ++c)
      if (m >> c & 1) link(*out[c], np[c], nn[c], true);
  } else {
    for (int k = o.kid; k != -1; k = T.nd[k].next) restrict_node_all(T, k, out, nn, dim, depth + 1, mask);
    for (int k = o.sc; k != -1; k = T.nd[k].next) restrict_node_all(T, k, out, nn, dim, depth + 1, mask);
    for (int c = 0; c < cells; ++c)
      if (m >> c & 1) {
        Trie& R = *out[c];
        const int add = R.nd[nn[c]].count;
        link(R, np[c], nn[c], false);
        R.nd[np[c]].count += add;
      }
  }
}

// restrict(), ScyTreeNode.cu:335-379, for every cell of `dim`: out[c] is
// restrict(T, dim, c).
void restrict_trie_all(const Trie& T, int dim, std::vector<std::unique_ptr<Trie>>& out) {
  const int cells = T.cells;
  out.clear();
  std::vector<Trie*> raw;
  std::vector<int> roots(cells, 0);
  for (int c = 0; c < cells; ++c) {
    auto R = std::make_unique<Trie>();
    R->cells = T.cells;
    R->cell_size = T.cell_size;
    R->restricted = T.restricted;
    R->restricted.push_back(dim);
    for (int l : T.levels)
      if (l != dim) R->levels.push_back(l);
    R->nd.reserve(T.nd.size() / cells + 16);
    R->flat.reserve(T.flat.size() / cells + 16);
    raw.push_back(R.get());
    out.push_back(std::move(R));
  }
  if (cells <= kMaxAllCells) {
    bool sflag[kMaxAllCells] = {};
    std::vector<uint64_t> mask(T.nd.size(), 0);
    for (int k = T.nd[0].kid; k != -1; k = T.nd[k].next) include_mask(T, k, dim, 0, false, sflag, mask);
    for (int k = T.nd[0].sc; k != -1; k = T.nd[k].next) include_mask(T, k, dim, 0, false, sflag, mask);
    for (int k = T.nd[0].kid; k != -1; k = T.nd[k].next) restrict_node_all(T, k, raw.data(), roots.data(), dim, 0, mask);
    for (int k = T.nd[0].sc; k != -1; k = T.nd[k].next) restrict_node_all(T, k, raw.data(), roots.data(), dim, 0, mask);
    for (int c = 0; c < cells; ++c) raw[c]->sconnected = sflag[c];
  } else {
    for (int c = 0; c < cells; ++c) {
      bool sflag = false;
      for (int k = T.nd[0].kid; k != -1; k = T.nd[k].next) restrict_node(T, k, *raw[c], 0, dim, c, 0, sflag);
      for (int k = T.nd[0].sc; k != -1; k = T.nd[k].next) restrict_node(T, k, *raw[c], 0, dim, c, 0, sflag);
      raw[c]->sconnected = sflag;
    }
  }
  for (int c = 0; c < cells; ++c) raw[c]->npts = raw[c]->nd[0].count;
}

// mergeNodes, ScyTreeNode.cu:803-829, with b in A's own node array: b's
// subtrees are relinked under a.
void merge_nodes(Trie& A, int a, int b) {
  if (A.nd[a].count > 0) {
    A.nd[a].count += A.nd[b].count;
    if (A.nd[b].pn > 0) {
      std::vector<int> tmp(A.pts(b), A.pts(b) + A.nd[b].pn);
      A.append_pts(a, tmp.data(), (int)tmp.size());
    }
  }
  for (int c = A.nd[b].kid; c != -1;) {
    const int nxt = A.nd[c].next;
    const int x = find_child(A, A.nd[a].kid, A.nd[c].cell);
    if (x != -1)
      merge_nodes(A, x, c);
    else
      link(A, a, c, false);
    c = nxt;
  }
  for (int c = A.nd[b].sc; c != -1;) {
    const int nxt = A.nd[c].next;
    const int x = find_child(A, A.nd[a].sc, A.nd[c].cell);
    if (x != -1)
      merge_nodes(A, x, c);
    else
      link(A, a, c, true);
    c = nxt;
  }
}

// Moves B's nodes and points to the end of A's arrays; returns the index
// that B's root has there.
int absorb(Trie& A, const Trie& B) {
  const int base = (int)A.nd.size(), pbase = (int)A.flat.size();
  A.nd.insert(A.nd.end(), B.nd.begin(), B.nd.end());
  A.flat.insert(A.flat.end(), B.flat.begin(), B.flat.end());
  for (size_t i = base; i < A.nd.size(); ++i) {
    TN& t = A.nd[i];
    if (t.kid != -1) t.kid += base;
    if (t.sc != -1) t.sc += base;
    if (t.next != -1) t.next += base;
    t.pb += pbase;
  }
  return base;
}

void collect_leaves(const Trie& T, int v, std::vector<int>& out) {  // get_leafs, ScyTreeNode.cu:422-431
  if (T.nd[v].kid == -1 && T.nd[v].sc == -1) {
    out.push_back(v);
    return;
  }
  for (int c = T.nd[v].kid; c != -1; c = T.nd[c].next) collect_leaves(T, c, out);
}

void recount(Trie& T, int v) {  // propergate_count2, ScyTreeNode.cu:446-467
  if (T.nd[v].kid == -1 && T.nd[v].sc == -1) return;
  T.nd[v].count = 0;
  // children whose count drops to 0 are erased together with the
  // s-connection of the same cell
  for (int c = T.nd[v].kid, prev = -1; c != -1;) {
    const int nxt = T.nd[c].next;
    recount(T, c);
    if (T.nd[c].count == 0) {
      if (prev == -1)
        T.nd[v].kid = nxt;
      else
        T.nd[prev].next = nxt;
      unlink_cell(T, v, T.nd[c].cell, true);
    } else {
      T.nd[v].count += T.nd[c].count;
      prev = c;
    }
    c = nxt;
  }
}

void points_of(const Trie& T, int v, std::vector<int>& out) {  // get_points_node, ScyTreeNode.cu:859-869
  if (T.nd[v].kid == -1) out.insert(out.end(), T.pts(v), T.pts(v) + T.nd[v].pn);
  for (int c = T.nd[v].kid; c != -1; c = T.nd[c].next) points_of(T, c, out);
}

// ------------------------------------------------------------------------
// Neighbour lists
// ------------------------------------------------------------------------
struct Entry {
  int q;      // neighbour
  float acc;  // float sum of squared differences over the subspace's dims, ascending
};

// The neighbour lists (and density values) of one region's points in the
// region's subspace, stored in blocks of consecutive region points.
struct RegionLists {
  static constexpr int kBlock = 32;
  std::vector<int> sub;                      // the subspace
  std::vector<char> matched;                 // per dim of sub: filtered on its fine cell
  std::vector<int> ids;                      // region points, in the trie's leaf order
  std::vector<int> by_id;                    // indices into ids, ordered by point id
  std::vector<int> blk_start;                // per point: start in its block's storage
  std::vector<int> len;                      // per point: list length
  std::vector<float> phi;                    // per point: phi (or the list length, as float)
  std::vector<std::vector<Entry>> store;     // per block
  const RegionLists* up = nullptr;           // the parent region's lists
  int find(int p) const {
    auto it = std::lower_bound(by_id.begin(), by_id.end(), p, [&](int i, int v) { return ids[i] < v; });
    return (it != by_id.end() && ids[*it] == p) ? *it : -1;
  }
  const Entry* list(int i) const { return store[i / kBlock].data() + blk_start[i]; }
};

struct Ctx {
  Data D;
  float F = 1.f;
  int num_obj = 1;
  bool rect = false;
  Commit commit;
  std::unique_ptr<Pool> pool;
  // column-major copies: coordinate and fine cell of point q on dim k at [k * n + q]
  std::vector<float> xc;
  std::vector<uint16_t> fc;
  // per (dim, fine cell): the points in fine cells cell-1 .. cell+1 of dim, in trie order
  std::vector<std::vector<std::vector<int>>> cand;
  // thresholds by subspace size
  std::vector<float> thr_dense, thr_rect_dense;
  float acc_max = 0.f;  // the largest float a with sqrt(a) <= eps
  float thr_weak = 0.f, thr_rect_weak = 0.f;
  // statistics
  long long calls = 0, regions = 0, prunes_passed = 0, clusterings = 0, dense_tests = 0;

  float X(int q, int k) const { return xc[(size_t)k * D.n + q]; }
  int FC(int q, int k) const { return fc[(size_t)k * D.n + q]; }
};

// Neighbour list of p in `sub` (size k) from a list of p in the prefix of
// `sub` of size `from` (src, its partial sums) -- or, with from == 0, from the
// fine-cell candidates of sub[0].  Returns phi (or |N| for rectangular density).
float derive(const Ctx& C, int p, const std::vector<int>& sub, const std::vector<char>& matched, int from,
             const Entry* src, int src_len, std::vector<Entry>& out) {
  const int k = (int)sub.size();
  const float eps = C.D.eps;
  float xp[64];
  int cp[64];
  for (int j = 0; j < k; ++j) {
    xp[j] = C.X(p, sub[j]);
    cp[j] = C.FC(p, sub[j]);
  }
  const size_t first = out.size();
  // eps >= sqrt(acc) exactly when acc <= acc_max (sqrt is monotone)
  const float acc_max = C.acc_max;
  auto extend = [&](int q, float acc) {
    for (int j = from; j < k; ++j) {
      const int dj = sub[j];
      if (matched[j]) {
        int cq = C.FC(q, dj);
        if (cq < cp[j] - 1 || cq > cp[j] + 1) return;
      }
      float diff = xp[j] - C.X(q, dj);
      acc = acc + diff * diff;
    }
    if (acc <= acc_max) out.push_back(Entry{q, acc});
  };
  if (from == 0) {
    // ScyTreeNode.cu:896-946 on a one-dim prefix: the +-1 fine cells of sub[0]
    const std::vector<int>& cl = C.cand[sub[0]][cp[0]];
    for (int q : cl)
      if (q != p) extend(q, 0.f);
  } else if (from == k - 1) {  // one more dim: the common case
    const int dj = sub[k - 1];
    const float* xcol = C.xc.data() + (size_t)dj * C.D.n;
    const uint16_t* fcol = C.fc.data() + (size_t)dj * C.D.n;
    const float x0 = xp[k - 1];
    const int lo = cp[k - 1] - 1, hi = cp[k - 1] + 1;
    const bool m = matched[k - 1] != 0;
    for (int i = 0; i < src_len; ++i) {
      const int q = src[i].q;
      if (m) {
        const int cq = fcol[q];
        if (cq < lo || cq > hi) continue;
      }
      const float diff = x0 - xcol[q];
      const float acc = src[i].acc + diff * diff;
      if (acc <= acc_max) out.push_back(Entry{q, acc});
    }
  } else {
    for (int i = 0; i < src_len; ++i) extend(src[i].q, src[i].acc);
  }
  if (C.rect) return (float)(out.size() - first);
  float sum = 0.f;
  for (size_t i = first; i < out.size(); ++i) sum = phi_step(sum, std::sqrt(out[i].acc), eps);
  return sum;
}

// Lists of the points `pts` of a region of subspace `sub`, from the parent
// region's lists (or the fine-cell candidates at one dim).
void region_lists(Ctx& C, const std::vector<int>& sub, const std::vector<int>& pts, const RegionLists* up,
                  RegionLists& L) {
  L.sub = sub;
  {
    std::vector<int> m = matched_dims(C.D, sub);
    L.matched.assign(sub.size(), 0);
    for (size_t j = 0, t = 0; j < sub.size(); ++j)
      if (t < m.size() && m[t] == sub[j]) {
        L.matched[j] = 1;
        ++t;
      }
  }
  L.up = up;
  L.ids = pts;
  const int m = (int)L.ids.size();
  L.by_id.resize(m);
  for (int i = 0; i < m; ++i) L.by_id[i] = i;
  std::sort(L.by_id.begin(), L.by_id.end(), [&](int a, int b) { return L.ids[a] < L.ids[b]; });
  L.blk_start.assign(m, 0);
  L.len.assign(m, 0);
  L.phi.assign(m, 0.f);
  const int nblk = (m + RegionLists::kBlock - 1) / RegionLists::kBlock;
  L.store.assign(nblk, {});
  const int k = (int)sub.size();
  C.pool->run(nblk, 1, [&](int b0, int b1) {
    for (int b = b0; b < b1; ++b) {
      std::vector<Entry>& st = L.store[b];
      for (int i = b * RegionLists::kBlock; i < std::min(m, (b + 1) * RegionLists::kBlock); ++i) {
        const int p = L.ids[i];
        L.blk_start[i] = (int)st.size();
        if (k == 1 || !up) {
          L.phi[i] = derive(C, p, sub, L.matched, 0, nullptr, 0, st);
        } else {
          const int u = up->find(p);
          if (u < 0) {  // cannot happen: a region's points are kept points of its parent region
            std::fprintf(stderr, "oracle: point %d missing from its parent region\n", p);
            std::abort();
          }
          L.phi[i] = derive(C, p, sub, L.matched, k - 1, up->list(u), up->len[u], st);
        }
        L.len[i] = (int)st.size() - L.blk_start[i];
      }
    }
  });
}

// ------------------------------------------------------------------------
// The recursion (InscyNodeCpu.cu:159-235)
// ------------------------------------------------------------------------

// pruneRecursionAndRemove2, ScyTreeNode.cu:582-667 (weak density with d = all dims)
// `leaves` are the trie's leaves in get_leafs order, whose points are L.ids.
bool prune_recursion(Ctx& C, Trie& T, const std::vector<int>& leaves, const RegionLists& L) {
  int kept_total = 0;
  int i = 0;
  for (int v : leaves) {
    int* pts = T.flat.data() + T.nd[v].pb;
    int kept = 0;
    for (int j = 0; j < T.nd[v].pn; ++j, ++i) {
      const int p = pts[j];
      const bool weak = C.rect ? (L.phi[i] >= C.thr_rect_weak) : (L.phi[i] >= C.thr_weak);
      if (weak) pts[kept++] = p;
    }
    C.dense_tests += T.nd[v].pn;
    T.nd[v].pn = kept;
    T.nd[v].count = kept;
    kept_total += kept;
  }
  recount(T, 0);
  T.npts = T.nd[0].count;
  return kept_total >= C.commit.min_size;
}

// INSCYClusteringImplCPUAll, ClusteringCpu.cu:317-389, one BFS level at a time
void cluster_region(Ctx& C, const Trie& T, const RegionLists& L, std::vector<int>& clu) {
  const std::vector<int>& sub = L.sub;
  const int k = (int)sub.size();
  const float thr = C.rect ? C.thr_rect_dense[k] : C.thr_dense[k];
  int clustered = 0, prev = 0;
  int label = std::max(0, max_of(clu)) + 1;
  std::vector<int> seeds;
  points_of(T, 0, seeds);
  std::vector<int> frontier, next, own;
  std::vector<std::vector<Entry>> nbs;
  std::vector<char> dense;
  for (int s : seeds) {
    if (clu[s] != -1) continue;
    prev = clustered;
    frontier.assign(1, s);
    while (!frontier.empty()) {
      const int f = (int)frontier.size();
      nbs.resize(std::max(nbs.size(), (size_t)f));
      own.assign(f, -1);
      dense.assign(f, 0);
      C.pool->run(f, f < 64 ? f : 8, [&](int b0, int b1) {
        for (int t = b0; t < b1; ++t) {
          const int p = frontier[t];
          std::vector<Entry>& nb = nbs[t];
          nb.clear();
          float phi;
          const RegionLists* A = &L;
          int i = A->find(p);
          while (i < 0 && A->up) {
            A = A->up;
            i = A->find(p);
          }
          if (i >= 0 && A == &L) {  // a point of the region: its list and density are known
            own[t] = i;
            phi = L.phi[i];
          } else if (i >= 0) {
            phi = derive(C, p, sub, L.matched, (int)A->sub.size(), A->list(i), A->len[i], nb);
          } else {
            phi = derive(C, p, sub, L.matched, 0, nullptr, 0, nb);
          }
          dense[t] = phi >= thr;
        }
      });
      C.dense_tests += f;
      next.clear();
      for (int t = 0; t < f; ++t) {
        if (!dense[t]) continue;
        const int p = frontier[t];
        clu[p] = label;
        ++clustered;
        const Entry* e = own[t] >= 0 ? L.list(own[t]) : nbs[t].data();
        const int len = own[t] >= 0 ? L.len[own[t]] : (int)nbs[t].size();
        for (int j = 0; j < len; ++j) {
          const int o = e[j].q;
          if (clu[o] == -1) {
            clu[o] = -2;
            next.push_back(o);
          }
        }
      }
      frontier.swap(next);
    }
    if (clustered > prev) ++label;
  }
}

// One restricted (and merged) region of a call, with its leaves in get_leafs
// order and their points.
struct Region {
  std::unique_ptr<Trie> R;
  std::vector<int> leaves, pts;
};

// The regions of `dim` in the call on T, in the order the cells loop of
// INSCYCPU3Weak meets them: restrict(dim, cell), then mergeWithNeighbors
// (ScyTreeNode.cu:837-851) absorbs the next cells while the tree restricted
// last was s-connected, and the loop skips the absorbed cells.
void dim_regions(const Trie& T, int dim, std::vector<Region>& out) {
  const int cells = T.cells;
  std::vector<std::unique_ptr<Trie>> rs;
  restrict_trie_all(T, dim, rs);
  int cell = 0;
  while (cell < cells) {
    Region g;
    g.R = std::move(rs[cell]);
    Trie& R = *g.R;
    if (R.sconnected) {
      bool last = true;
      while (last && cell < cells - 1) {
        std::unique_ptr<Trie> nb = std::move(rs[cell + 1]);
        merge_nodes(R, 0, absorb(R, *nb));
        last = nb->sconnected;
        ++cell;
      }
      R.npts = R.nd[0].count;
      R.sconnected = false;
    }
    collect_leaves(R, 0, g.leaves);
    for (int v : g.leaves) g.pts.insert(g.pts.end(), R.pts(v), R.pts(v) + R.nd[v].pn);
    out.push_back(std::move(g));
    ++cell;
  }
}

void inscy(Ctx& C, Trie& T, const RegionLists* TL, int first_dim) {
  C.calls++;
  const int d = C.D.d;
  const int n = C.D.n;
  // the regions of every dim of this call, computed up front, one task per dim
  const int nd = d - first_dim;
  std::vector<std::vector<Region>> regions(std::max(0, nd));
  C.pool->run(nd, 1, [&](int b0, int b1) {
    for (int t = b0; t < b1; ++t) dim_regions(T, first_dim + t, regions[t]);
  });
  for (int dim = first_dim; dim < d; ++dim) {
    std::vector<int> clu(n, -1);
    std::vector<int> sub;
    for (Region& g : regions[dim - first_dim]) {
      Trie& R = *g.R;
      sub = R.restricted;
      C.regions++;
      RegionLists L;
      region_lists(C, sub, g.pts, TL, L);
      if (prune_recursion(C, R, g.leaves, L)) {
        C.prunes_passed++;
        inscy(C, R, &L, dim + 1);
        std::vector<int> rpts;
        points_of(R, 0, rpts);
        if (C.commit.prune_redundancy(R.restricted, rpts, R.npts)) {
          C.clusterings++;
          cluster_region(C, R, L, clu);
        }
      }
      g.R.reset();
    }
    C.commit.join(clu, sub);
  }
}

}  // namespace

extern "C" {

// Same arguments and result as orc_run (inscy_oracle.cpp).
int orcf_run(const float* X, int n, int d, float eps, float F, int num_obj, int min_size, float r, int cells,
             int rectangular, int entropy_order, int threads, orc_result** out) {
  if (!out || n < 0 || d <= 0 || d > 64 || cells <= 0 || !(eps > 0.f)) return 1;
  auto* res = new orc_result();
  std::memset(res->stats, 0, sizeof(res->stats));
  *out = res;
  if (n == 0) return 0;
  Ctx C;
  C.D.X = X;
  C.D.n = n;
  C.D.d = d;
  C.D.eps = eps;
  C.F = F;
  C.num_obj = num_obj;
  C.rect = rectangular != 0;
  C.commit.r = r;
  C.commit.min_size = min_size;
  C.pool = std::make_unique<Pool>(threads > 0 ? threads : 1);
  C.D.order = level_order(X, n, d, cells, entropy_order);
  build_index(C.D);
  if (C.D.fine_cells > 65535) return 1;
  C.xc.resize((size_t)n * d);
  C.fc.resize((size_t)n * d);
  for (int q = 0; q < n; ++q)
    for (int k = 0; k < d; ++k) {
      C.xc[(size_t)k * n + q] = C.D.x(q, k);
      C.fc[(size_t)k * n + q] = (uint16_t)C.D.fine[(size_t)q * d + k];
    }
  const int G = C.D.fine_cells;
  C.cand.assign(d, std::vector<std::vector<int>>(G));
  for (int k = 0; k < d; ++k)
    for (int c = 0; c < G; ++c) {
      std::vector<int>& v = C.cand[k][c];
      for (int cc = c - 1; cc <= c + 1; ++cc)
        if (cc >= 0 && cc < G) v.insert(v.end(), C.D.bucket[k][cc].begin(), C.D.bucket[k][cc].end());
      std::sort(v.begin(), v.end(), [&](int a, int b) { return C.D.rank[a] < C.D.rank[b]; });
    }
  C.thr_dense.assign(d + 1, 0.f);
  C.thr_rect_dense.assign(d + 1, 0.f);
  for (int k = 1; k <= d; ++k) {
    C.thr_dense[k] = std::max(F * alpha_of(k, eps, n), (float)num_obj * omega_of(k));
    C.thr_rect_dense[k] = std::max(F * expden_of(k, eps, n), (float)num_obj);
  }
  {
    float a = eps * eps;
    while (std::sqrt(a) > eps) a = std::nextafter(a, 0.f);
    while (std::sqrt(std::nextafter(a, INFINITY)) <= eps) a = std::nextafter(a, INFINITY);
    C.acc_max = a;
  }
  C.thr_weak = std::max(F * alpha_of(d, eps, n), (float)num_obj * omega_of(d));
  C.thr_rect_weak = std::max(F * expden_of(d, eps, n), (float)num_obj);
  Trie root;
  build_trie(C.D, cells, root);
  inscy(C, root, nullptr, 0);
  for (auto& e : C.commit.result) {
    res->subspaces.push_back(e.first);
    res->labels.push_back(e.second);
  }
  res->stats[0] = C.calls;
  res->stats[1] = C.regions;
  res->stats[2] = C.prunes_passed;
  res->stats[3] = C.clusterings;
  res->stats[4] = C.dense_tests;
  res->stats[5] = (long long)C.commit.result.size();
  return 0;
}

}  // extern "C"
