// INSCY CPU oracle -- TEST INFRASTRUCTURE ONLY.
//
// A restatement, in plain C++, of the reference CPU INSCY path
// (`CPU()` -> `run_cpu3_weak` -> `INSCYCPU3Weak`) of mrjakobdk/GPU_INSCY.
// It is the checker for the CUDA implementation: only tests/, the smoke
// test and the CPU-baseline leg of bench.py load it.  Nothing in the product
// links against it.
//
// Pinned against the compiled reference through tests/golden/ (fixtures
// produced by tests/golden/make_golden.py from `run_cpu3_weak` itself).
//
// Every decision and every float operation follows the reference:
//   * the SCY-tree is a trie of grid cells with s-connection chains
//     (ScyTreeNode.cu:22-143), restricted and merged exactly as
//     ScyTreeNode.cu:227-379 and :803-851 do it, including the count quirks;
//   * neighbourhoods are the points whose cells on the ceil(1/eps) grid are
//     within +-1 on the (greedily matched) subspace dims, emitted in the
//     neighbourhood trie's leaf order (ScyTreeNode.cu:896-946) -- here found
//     through per-dimension cell buckets that are merged back into that
//     order, so the float sums run in the reference's order;
//   * dist / phi / alpha / omega / expDen use the reference's types and
//     operation order (ClusteringCpu.cu:27-183).  Build with
//     -ffp-contract=off so no multiply-add is fused (x86 and Arm agree).
//
// The one intentional difference: independent per-point density tests of a
// prune are evaluated by several threads (results are per point, so the
// outcome does not depend on the thread count).
//
// The thresholds, the neighbourhood grid, join and pruneRedundancy are shared
// with the fast restatement (inscy_oracle_fast.cpp) through oracle_common.h.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <queue>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "oracle_common.h"

namespace {

using namespace orc_common;

// Lazily built 2-D cell buckets for a pair of dims (a < b): points grouped by
// (fine cell of a, fine cell of b).
struct PairIndex {
  std::vector<int> start;  // (G*G + 1) offsets
  std::vector<int> pts;
};

struct NbIndex {
  std::map<std::pair<int, int>, PairIndex> pairs;
  const PairIndex& get(const Data& D, int a, int b) {
    auto key = std::make_pair(a, b);
    auto it = pairs.find(key);
    if (it != pairs.end()) return it->second;
    PairIndex P;
    const int G = D.fine_cells;
    P.start.assign((size_t)G * G + 1, 0);
    for (int p = 0; p < D.n; ++p) P.start[(size_t)D.fine[(size_t)p * D.d + a] * G + D.fine[(size_t)p * D.d + b] + 1]++;
    for (size_t i = 1; i < P.start.size(); ++i) P.start[i] += P.start[i - 1];
    P.pts.assign(D.n, 0);
    std::vector<int> fill(P.start.begin(), P.start.end() - 1);
    for (int p = 0; p < D.n; ++p) P.pts[fill[(size_t)D.fine[(size_t)p * D.d + a] * G + D.fine[(size_t)p * D.d + b]]++] = p;
    return pairs.emplace(key, std::move(P)).first->second;
  }
};

// neighborhood() (ClusteringCpu.cu:52-81) over get_possible_neighbors()
// (ScyTreeNode.cu:896-946): the candidates are the points whose fine cells are
// within +-1 on every matched dim; the reference emits them in trie order.
// Here they are collected through cell buckets, filtered with the same
// tests, and the survivors are put back into trie order (by rank) before
// anything order-dependent (phi) runs, so the returned list is identical.
void neighbours(const Data& D, NbIndex* pix, int p, const std::vector<int>& sub, const std::vector<int>& match,
                std::vector<int>& out) {
  out.clear();
  auto accept = [&](int q) {
    if (q == p) return;
    for (int k : match) {
      int c = D.fine[(size_t)p * D.d + k], cq = D.fine[(size_t)q * D.d + k];
      if (cq < c - 1 || cq > c + 1) return;
    }
    float dd = dist_of(D, p, q, sub);
    if (D.eps >= dd) out.push_back(q);
  };
  if (match.empty()) {  // no filtering dim: every point
    for (int q = 0; q < D.n; ++q) accept(q);
  } else if (match.size() == 1 || !pix) {
    int best = -1;
    size_t best_sz = (size_t)-1;
    for (int k : match) {
      int c = D.fine[(size_t)p * D.d + k];
      size_t s = 0;
      for (int cc = c - 1; cc <= c + 1; ++cc)
        if (cc >= 0 && cc < D.fine_cells) s += D.bucket[k][cc].size();
      if (s < best_sz) { best_sz = s; best = k; }
    }
    int c = D.fine[(size_t)p * D.d + best];
    for (int cc = c - 1; cc <= c + 1; ++cc)
      if (cc >= 0 && cc < D.fine_cells)
        for (int q : D.bucket[best][cc]) accept(q);
  } else {
    // the two matched dims with the smallest 1-D neighbourhoods
    int a = -1, b = -1;
    size_t sa = (size_t)-1, sb = (size_t)-1;
    for (int k : match) {
      int c = D.fine[(size_t)p * D.d + k];
      size_t s = 0;
      for (int cc = c - 1; cc <= c + 1; ++cc)
        if (cc >= 0 && cc < D.fine_cells) s += D.bucket[k][cc].size();
      if (s < sa) { sb = sa; b = a; sa = s; a = k; }
      else if (s < sb) { sb = s; b = k; }
    }
    if (a > b) std::swap(a, b);
    const PairIndex& P = pix->get(D, a, b);
    const int G = D.fine_cells;
    int ca = D.fine[(size_t)p * D.d + a], cb = D.fine[(size_t)p * D.d + b];
    for (int x = ca - 1; x <= ca + 1; ++x) {
      if (x < 0 || x >= G) continue;
      int y0 = std::max(cb - 1, 0), y1 = std::min(cb + 1, G - 1);
      int s = P.start[(size_t)x * G + y0], e = P.start[(size_t)x * G + y1 + 1];
      for (int i = s; i < e; ++i) accept(P.pts[i]);
    }
  }
  std::sort(out.begin(), out.end(), [&](int u, int v) { return D.rank[u] < D.rank[v]; });
}

float phi_of(const Data& D, int p, const std::vector<int>& nb, const std::vector<int>& sub) {  // :112-125
  float sum = 0.f;
  for (int q : nb) sum = phi_step(sum, dist_of(D, p, q, sub), D.eps);
  return sum;
}

// ------------------------------------------------------------------------
// SCY-tree (pointer trie), ScyTreeNode.cu / Node.h
// ------------------------------------------------------------------------
struct Node {
  int cell;
  int count = 0;  // -1 marks an s-connection node
  bool leaf = false;
  std::map<int, std::unique_ptr<Node>> kids;   // children
  std::map<int, std::unique_ptr<Node>> sconn;  // s-connections
  std::vector<int> pts;
  explicit Node(int c) : cell(c) {}
};

std::unique_ptr<Node> copy_shallow(const Node* o) {  // Node(shared_ptr<Node>) in Node.h:33-38
  auto n = std::make_unique<Node>(o->cell);
  n->count = o->count;
  n->pts = o->pts;
  n->leaf = o->leaf;
  return n;
}

struct Tree {
  std::vector<int> levels;      // dims still in the trie, in level order
  std::vector<int> restricted;  // restricted dims, in restriction order
  int cells = 0;
  float cell_size = 0.f;
  bool sconnected = false;
  int npts = 0;
  std::unique_ptr<Node> root = std::make_unique<Node>(-1);
};

Node* child_of(std::map<int, std::unique_ptr<Node>>& m, int c, bool sconn) {
  auto it = m.find(c);
  if (it != m.end()) return it->second.get();
  auto nn = std::make_unique<Node>(c);
  if (sconn) nn->count = -1;
  Node* raw = nn.get();
  m.emplace(c, std::move(nn));
  return raw;
}

// ScyTreeNode(X, subspace, cells, ...) constructor, ScyTreeNode.cu:105-143,
// with construct_s_connection (:34-49).
void build_tree(const Data& D, int cells, Tree& T) {
  T.cells = cells;
  T.cell_size = 1.0f / (float)cells;
  T.levels = D.order;
  T.restricted.clear();
  Node* root = T.root.get();
  const int m = (int)T.levels.size();
  for (int i = 0; i < D.n; ++i) {
    root->count += 1;
    Node* node = root;
    for (int j = 0; j < m; ++j) {
      float xij = D.x(i, T.levels[j]);
      int c = cell_no(xij, T.cell_size, cells);
      Node* ch = child_of(node->kids, c, false);
      ch->count += 1;
      if (xij >= ((float)(c + 1) * T.cell_size - D.eps)) {
        Node* s = child_of(node->sconn, c, true);
        for (int k = j + 1; k < m; ++k) s = child_of(s->sconn, cell_no(D.x(i, T.levels[k]), T.cell_size, cells), true);
        s->leaf = true;
      }
      node = ch;
    }
    node->pts.push_back(i);
    node->leaf = true;
  }
  T.npts = root->count;
}

// restrict_node, ScyTreeNode.cu:227-323
bool restrict_node(const Tree& T, const Node* old, Node* np, int dim, int cell, int depth, bool& sflag) {
  if (T.levels[depth] == dim) {
    if (old->cell != cell) return false;
    if (np->count != -1 && old->count == -1) {
      sflag = true;
      return false;
    }
    if (old->leaf) {
      np->leaf = true;
      if (old->count > 0) {
        np->pts.insert(np->pts.end(), old->pts.begin(), old->pts.end());
        np->count += old->count;
      }
      return true;
    }
    for (auto& kv : old->kids) restrict_node(T, kv.second.get(), np, dim, cell, depth + 1, sflag);
    for (auto& kv : old->sconn) restrict_node(T, kv.second.get(), np, dim, cell, depth + 1, sflag);
    return true;
  }
  std::unique_ptr<Node> nn = copy_shallow(old);
  bool inc = T.levels[depth] > dim;
  if (old->count == -1) {
    for (auto& kv : old->sconn) inc = restrict_node(T, kv.second.get(), nn.get(), dim, cell, depth + 1, sflag) || inc;
    if (inc) np->sconn.emplace(nn->cell, std::move(nn));
  } else {
    if (!old->leaf)
      nn->count = 0;
    else
      inc = true;
    for (auto& kv : old->kids) inc = restrict_node(T, kv.second.get(), nn.get(), dim, cell, depth + 1, sflag) || inc;
    for (auto& kv : old->sconn) inc = restrict_node(T, kv.second.get(), nn.get(), dim, cell, depth + 1, sflag) || inc;
    if (inc) {
      int add = nn->count;
      np->kids.emplace(nn->cell, std::move(nn));
      np->count += add;
    }
  }
  return inc;
}

// restrict(), ScyTreeNode.cu:335-379
std::unique_ptr<Tree> restrict_tree(const Tree& T, int dim, int cell) {
  auto R = std::make_unique<Tree>();
  R->cells = T.cells;
  R->cell_size = T.cell_size;
  R->restricted = T.restricted;
  R->restricted.push_back(dim);
  for (int l : T.levels)
    if (l != dim) R->levels.push_back(l);
  R->sconnected = false;
  for (auto& kv : T.root->kids) restrict_node(T, kv.second.get(), R->root.get(), dim, cell, 0, R->sconnected);
  for (auto& kv : T.root->sconn) restrict_node(T, kv.second.get(), R->root.get(), dim, cell, 0, R->sconnected);
  R->npts = R->root->count;
  return R;
}

// mergeNodes, ScyTreeNode.cu:803-829 (ownership of b's subtrees moves to a)
void merge_nodes(Node* a, Node* b) {
  if (a->count > 0) {
    a->count += b->count;
    a->pts.insert(a->pts.end(), b->pts.begin(), b->pts.end());
  }
  for (auto& kv : b->kids) {
    auto it = a->kids.find(kv.first);
    if (it != a->kids.end())
      merge_nodes(it->second.get(), kv.second.get());
    else
      a->kids.emplace(kv.first, std::move(kv.second));
  }
  for (auto& kv : b->sconn) {
    auto it = a->sconn.find(kv.first);
    if (it != a->sconn.end())
      merge_nodes(it->second.get(), kv.second.get());
    else
      a->sconn.emplace(kv.first, std::move(kv.second));
  }
}

// mergeWithNeighbors, ScyTreeNode.cu:837-851: keep absorbing the next cell
// while the tree restricted last was s-connected.
void merge_with_neighbours(Tree& R, const Tree& parent, int dim, int& cell) {
  if (!R.sconnected) return;
  bool last = true;
  while (last && cell < R.cells - 1) {
    auto nb = restrict_tree(parent, dim, cell + 1);
    merge_nodes(R.root.get(), nb->root.get());
    last = nb->sconnected;
    ++cell;
  }
  R.npts = R.root->count;
  R.sconnected = false;
}

void collect_leaves(Node* n, std::vector<Node*>& out) {  // get_leafs, ScyTreeNode.cu:422-431
  if (n->kids.empty() && n->sconn.empty()) {
    out.push_back(n);
    return;
  }
  for (auto& kv : n->kids) collect_leaves(kv.second.get(), out);
}

void recount(Node* n) {  // propergate_count2, ScyTreeNode.cu:446-467
  if (n->kids.empty() && n->sconn.empty()) return;
  n->count = 0;
  std::vector<int> gone;
  for (auto& kv : n->kids) {
    recount(kv.second.get());
    if (kv.second->count == 0)
      gone.push_back(kv.second->cell);
    else
      n->count += kv.second->count;
  }
  for (int c : gone) {
    n->kids.erase(c);
    n->sconn.erase(c);
  }
}

void points_of(const Node* n, std::vector<int>& out) {  // get_points_node, ScyTreeNode.cu:859-869
  if (n->kids.empty()) out.insert(out.end(), n->pts.begin(), n->pts.end());
  for (auto& kv : n->kids) points_of(kv.second.get(), out);
}

struct Ctx {
  Data D;
  float F = 1.f;
  int num_obj = 1;
  bool rect = false;
  int threads = 1;
  Commit commit;  // result map, join, pruneRedundancy
  // statistics
  long long calls = 0, regions = 0, prunes_passed = 0, clusterings = 0, dense_tests = 0;
  NbIndex nbx;
};

void prepare_pairs(Ctx& C, const std::vector<int>& match) {
  for (size_t i = 0; i < match.size(); ++i)
    for (size_t j = i + 1; j < match.size(); ++j) C.nbx.get(C.D, std::min(match[i], match[j]), std::max(match[i], match[j]));
}

// per-point density decisions of a prune, several threads
template <class Fn>
void parallel_for(int threads, int count, Fn fn) {
  if (threads <= 1 || count < 64) {
    for (int i = 0; i < count; ++i) fn(i);
    return;
  }
  std::atomic<int> next(0);
  std::vector<std::thread> ws;
  for (int t = 0; t < threads; ++t)
    ws.emplace_back([&]() {
      for (;;) {
        int i = next.fetch_add(16);
        if (i >= count) break;
        for (int j = i; j < std::min(count, i + 16); ++j) fn(j);
      }
    });
  for (auto& w : ws) w.join();
}

// pruneRecursionAndRemove2, ScyTreeNode.cu:582-667 (weak density with d = all dims)
bool prune_recursion(Ctx& C, Tree& T) {
  const Data& D = C.D;
  std::vector<Node*> leaves;
  collect_leaves(T.root.get(), leaves);
  const float a = alpha_of(D.d, D.eps, D.n);
  const float w = omega_of(D.d);
  const float ex = expden_of(D.d, D.eps, D.n);
  const float thr = std::max(C.F * a, (float)C.num_obj * w);
  const float thr_rect = std::max(C.F * ex, (float)C.num_obj);
  const std::vector<int>& sub = T.restricted;
  const std::vector<int> match = matched_dims(D, sub);
  std::vector<std::pair<Node*, int>> work;
  for (Node* l : leaves)
    for (int p : l->pts) work.push_back({l, p});
  std::vector<char> keep(work.size(), 0);
  prepare_pairs(C, match);
  parallel_for(C.threads, (int)work.size(), [&](int i) {
    thread_local std::vector<int> nb;
    int p = work[i].second;
    neighbours(D, &C.nbx, p, sub, match, nb);
    if (C.rect)
      keep[i] = (float)nb.size() >= thr_rect;
    else
      keep[i] = phi_of(D, p, nb, sub) >= thr;
  });
  C.dense_tests += (long long)work.size();
  int kept_total = 0;
  size_t w0 = 0;
  for (Node* l : leaves) {
    std::vector<int> kept;
    for (size_t j = 0; j < l->pts.size(); ++j, ++w0)
      if (keep[w0]) kept.push_back(l->pts[j]);
    l->pts = kept;
    l->count = (int)kept.size();
    kept_total += (int)kept.size();
  }
  recount(T.root.get());
  T.npts = T.root->count;
  return kept_total >= C.commit.min_size;
}

// INSCYClusteringImplCPUAll, ClusteringCpu.cu:317-389
void cluster_region(Ctx& C, const Tree& T, std::vector<int>& clu) {
  const Data& D = C.D;
  const std::vector<int>& sub = T.restricted;
  const int k = (int)sub.size();
  const std::vector<int> match = matched_dims(D, sub);
  const float thr = std::max(C.F * alpha_of(k, D.eps, D.n), (float)C.num_obj * omega_of(k));
  const float thr_rect = std::max(C.F * expden_of(k, D.eps, D.n), (float)C.num_obj);
  int clustered = 0, prev = 0;
  int label = std::max(0, max_of(clu)) + 1;
  std::vector<int> seeds;
  points_of(T.root.get(), seeds);
  std::vector<int> nb;
  prepare_pairs(C, match);
  std::queue<int> q;
  for (int s : seeds) {
    if (clu[s] != -1) continue;
    prev = clustered;
    q.push(s);
    while (!q.empty()) {
      int p = q.front();
      q.pop();
      neighbours(D, &C.nbx, p, sub, match, nb);
      C.dense_tests++;
      bool dense = C.rect ? ((float)nb.size() >= thr_rect) : (phi_of(D, p, nb, sub) >= thr);
      if (dense) {
        clu[p] = label;
        ++clustered;
        for (int o : nb)
          if (clu[o] == -1) {
            clu[o] = -2;
            q.push(o);
          }
      }
    }
    if (clustered > prev) ++label;
  }
}

// INSCYCPU3Weak, InscyNodeCpu.cu:159-235
void inscy(Ctx& C, Tree& T, int first_dim) {
  C.calls++;
  const int d = C.D.d;
  const int n = C.D.n;
  for (int dim = first_dim; dim < d; ++dim) {
    std::vector<int> clu(n, -1);
    std::vector<int> sub;
    int cell = 0;
    while (cell < T.cells) {
      auto R = restrict_tree(T, dim, cell);
      sub = R->restricted;
      merge_with_neighbours(*R, T, dim, cell);
      C.regions++;
      if (prune_recursion(C, *R)) {
        C.prunes_passed++;
        inscy(C, *R, dim + 1);
        std::vector<int> rpts;
        points_of(R->root.get(), rpts);
        if (C.commit.prune_redundancy(R->restricted, rpts, R->npts)) {
          C.clusterings++;
          cluster_region(C, *R, clu);
        }
      }
      ++cell;
    }
    C.commit.join(clu, sub);
  }
}

}  // namespace

// ------------------------------------------------------------------------
// C ABI used by the tests and the bench's CPU-baseline leg
// ------------------------------------------------------------------------
extern "C" {

int orc_run(const float* X, int n, int d, float eps, float F, int num_obj, int min_size, float r, int cells,
            int rectangular, int entropy_order, int threads, orc_result** out) {
  if (!out || n < 0 || d <= 0 || cells <= 0 || !(eps > 0.f)) return 1;
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
  C.commit.r = r;
  C.num_obj = num_obj;
  C.commit.min_size = min_size;
  C.rect = rectangular != 0;
  C.threads = threads > 0 ? threads : 1;
  C.D.order = level_order(X, n, d, cells, entropy_order);
  build_index(C.D);
  Tree root;
  build_tree(C.D, cells, root);
  inscy(C, root, 0);
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

int orc_count(const orc_result* r) { return r ? (int)r->subspaces.size() : 0; }

int orc_subspace(const orc_result* r, int i, int* dims, int cap) {
  const auto& s = r->subspaces[i];
  for (int k = 0; k < (int)s.size() && k < cap; ++k) dims[k] = s[k];
  return (int)s.size();
}

void orc_labels(const orc_result* r, int i, int* out) {
  std::memcpy(out, r->labels[i].data(), r->labels[i].size() * sizeof(int));
}

void orc_stats(const orc_result* r, long long* out6) { std::memcpy(out6, r->stats, sizeof(r->stats)); }

void orc_free(orc_result* r) { delete r; }

// Thresholds as the reference computes them (for host-side checks in tests).
float orc_alpha(int k, float eps, int n) { return alpha_of(k, eps, n); }
float orc_omega(int k) { return omega_of(k); }
float orc_expden(int k, float eps, int n) { return expden_of(k, eps, n); }

}  // extern "C"
