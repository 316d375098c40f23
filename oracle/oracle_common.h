// Shared pieces of the two INSCY CPU oracles -- TEST INFRASTRUCTURE ONLY.
//
// Thresholds, the neighbourhood grid, the result-map order and the commit
// steps (join, pruneRedundancy) of the reference CPU INSCY, used by both
// restatements in this directory:
//   inscy_oracle.cpp       pointer trie, candidates searched per query;
//   inscy_oracle_fast.cpp  arena trie, candidate lists derived from the
//                          parent call's lists, thread pool.
// Every float operation follows the reference's types and order
// (ClusteringCpu.cu:27-183, util.cu:619-743); build with -ffp-contract=off.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <set>
#include <vector>

namespace orc_common {

// ------------------------------------------------------------------------
// Density constants (ClusteringCpu.cu:27, 36-38, 136-164)
// ------------------------------------------------------------------------
const double kPi = 3.14;  // ClusteringCpu.cu:27 (sic)

inline float omega_of(int k) { return (float)(2.0 / ((double)k + 2.0)); }  // :36-38

inline float gamma_of(int m) {  // :136-143, called with subspace_size + 2
  if (m == 2) return 1.0f;
  if (m == 1) return (float)std::sqrt(kPi);
  return (float)(((double)m / 2.0 - 1.0) * (double)gamma_of(m - 2));
}

inline float cball_of(int k) {  // c(), :145-150
  float r = (float)std::pow(kPi, (double)k / 2.0);
  return r / gamma_of(k + 2);
}

inline float alpha_of(int k, float eps, int n) {  // :152-157
  float r = (float)((double)(2 * n) * std::pow((double)eps, (double)k) * (double)cball_of(k));
  r = (float)((double)r / (std::pow(1.0, (double)k) * (double)(k + 2)));
  return r;
}

inline float expden_of(int k, float eps, int n) {  // :159-164 and ScyTreeNode.cu:608-611
  float r = (float)((double)((float)n * cball_of(k)) * std::pow((double)eps, (double)k));
  r = (float)((double)r / std::pow(1.0, (double)k));
  return r;
}

// ------------------------------------------------------------------------
// Input + neighbourhood index
// ------------------------------------------------------------------------
struct Data {
  const float* X = nullptr;
  int n = 0, d = 0;
  float eps = 0.f;
  std::vector<int> order;  // level order of the dims (get_subspace_order)
  // neighbourhood grid (ScyTreeNode ctor with ceil(1/eps) cells, inscy_map.cpp:243)
  int fine_cells = 0;
  float fine_size = 0.f;
  std::vector<int> fine;             // n x d fine cell numbers
  std::vector<int> rank;             // position of each point in the neighbourhood trie's leaf order
  std::vector<std::vector<std::vector<int>>> bucket;  // [dim][cell] -> points sorted by rank
  float x(int p, int k) const { return X[(size_t)p * d + k]; }
};

inline int cell_no(float x, float size, int cells) {  // ScyTreeNode.cu:100-102
  return std::min((int)(x / size), cells - 1);
}

inline void build_index(Data& D) {
  D.fine_cells = (int)std::ceil(1.0 / (double)D.eps);
  D.fine_size = 1.0f / (float)D.fine_cells;
  D.fine.assign((size_t)D.n * D.d, 0);
  for (int p = 0; p < D.n; ++p)
    for (int k = 0; k < D.d; ++k) D.fine[(size_t)p * D.d + k] = cell_no(D.x(p, k), D.fine_size, D.fine_cells);
  // Trie leaf order of the neighbourhood tree: lexicographic in the level order
  // of the dims, ties (same leaf) in insertion order = point id.
  std::vector<int> idx(D.n);
  for (int i = 0; i < D.n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
    for (int l = 0; l < D.d; ++l) {
      int k = D.order[l];
      int ca = D.fine[(size_t)a * D.d + k], cb = D.fine[(size_t)b * D.d + k];
      if (ca != cb) return ca < cb;
    }
    return false;
  });
  D.rank.assign(D.n, 0);
  for (int i = 0; i < D.n; ++i) D.rank[idx[i]] = i;
  D.bucket.assign(D.d, std::vector<std::vector<int>>(D.fine_cells));
  for (int i = 0; i < D.n; ++i) {
    int p = idx[i];
    for (int k = 0; k < D.d; ++k) D.bucket[k][D.fine[(size_t)p * D.d + k]].push_back(p);
  }
}

// Dims of `sub` (ascending) that the neighbourhood trie walk filters on: the
// walk advances through `sub` only when the level's dim equals the next
// element (ScyTreeNode.cu:907-913).
inline std::vector<int> matched_dims(const Data& D, const std::vector<int>& sub) {
  std::vector<int> m;
  size_t si = 0;
  for (int l = 0; l < D.d && si < sub.size(); ++l)
    if (D.order[l] == sub[si]) m.push_back(sub[si++]);
  return m;
}

inline float dist_of(const Data& D, int p, int q, const std::vector<int>& sub) {  // ClusteringCpu.cu:40-50
  float acc = 0.f;
  for (int k : sub) {
    float diff = D.x(p, k) - D.x(q, k);
    acc = acc + diff * diff;
  }
  return std::sqrt(acc);
}

// One step of phi (ClusteringCpu.cu:112-125): the distance divided by eps,
// squared, and 1 - sq added to the float sum through a double.
inline float phi_step(float sum, float dist, float eps) {
  float dd = dist / eps;
  float sq = dd * dd;
  return (float)((double)sum + (1.0 - (double)sq));
}

// get_subspace_order, inscy_map.cpp:61-121
inline std::vector<int> level_order(const float* X, int n, int d, int cells, int entropy_order) {
  std::vector<int> sub(d);
  for (int i = 0; i < d; ++i) sub[i] = i;
  if (entropy_order == 0) return sub;
  std::vector<std::vector<int>> cnt(d, std::vector<int>(cells, 0));
  float size = 1.0f / (float)cells;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < d; ++j) cnt[j][cell_no(X[(size_t)i * d + j], size, cells)] += 1;
  std::vector<std::pair<float, int>> ent(d);
  for (int i = 0; i < d; ++i) {
    float e = 0.f;
    for (int j = 0; j < cells; ++j) {
      float p = (float)cnt[i][j] / (float)n;
      e -= p * std::log(p);
    }
    ent[i] = {e, i};
  }
  std::sort(ent.begin(), ent.end());
  if (entropy_order == -1) std::reverse(ent.begin(), ent.end());
  for (int i = 0; i < d; ++i) sub[i] = ent[i].second;
  return sub;
}

// ------------------------------------------------------------------------
// result map ordering, subspace test, join (util.cu:619-743)
// ------------------------------------------------------------------------
struct SubspaceOrder {  // vec_cmp, util.cu:633-653: compare from the last dim backwards
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
using Result = std::map<std::vector<int>, std::vector<int>, SubspaceOrder>;

inline bool is_subsequence(const std::vector<int>& sub, const std::vector<int>& sup) {  // subspace_of, util.cu:619-631
  size_t i = 0, j = 0;
  while (j < sup.size() && i < sub.size()) {
    if (sub[i] == sup[j]) ++i;
    ++j;
  }
  return i == sub.size();
}

inline int max_of(const std::vector<int>& v) {  // v_max(vector<int>), util.cu:566-574
  int m = -100000;
  for (int x : v)
    if (x > m) m = x;
  return m;
}

// The global result map with the two commit steps that read it.
struct Commit {
  float r = 1.f;
  int min_size = 0;
  Result result;
  // per result entry: size of the cluster each point belongs to (0 when the
  // point is not in a cluster); rebuilt whenever the entry changes
  std::map<std::vector<int>, std::vector<int>, SubspaceOrder> sizes_cache;

  const std::vector<int>& sizes_of(const std::vector<int>& sub, const std::vector<int>& lab) {
    auto it = sizes_cache.find(sub);
    if (it != sizes_cache.end()) return it->second;
    std::map<int, int> s;
    for (int c : lab)
      if (c >= 0) s[c]++;
    std::vector<int> per(lab.size(), 0);
    for (size_t i = 0; i < lab.size(); ++i)
      if (lab[i] >= 0) per[i] = s[lab[i]];
    return sizes_cache.emplace(sub, std::move(per)).first->second;
  }

  // join(), util.cu:655-743
  void join(std::vector<int>& clu, const std::vector<int>& sub) {
    if (max_of(clu) < 0) return;
    const int n = (int)clu.size();
    std::map<int, int> sizes;
    for (int i = 0; i < n; ++i)
      if (clu[i] >= 0) sizes[clu[i]]++;
    for (int i = 0; i < n; ++i)
      if (clu[i] >= 0 && sizes[clu[i]] < min_size) clu[i] = -1;
    for (auto& e : result) {
      if (!is_subsequence(sub, e.first)) continue;
      const std::vector<int>& H = e.second;
      const std::vector<int>& sH = sizes_of(e.first, H);
      std::set<int> drop;
      for (int i = 0; i < n; ++i) {
        int c = clu[i], h = H[i];
        if (c >= 0 && h >= 0 && (float)sizes[c] * r < (float)sH[i]) drop.insert(c);
      }
      if (!drop.empty())
        for (int i = 0; i < n; ++i)
          if (clu[i] >= 0 && drop.count(clu[i])) clu[i] = -1;
    }
    if (max_of(clu) < 0) return;
    auto it = result.find(sub);
    if (it != result.end()) {
      std::vector<int>& old = it->second;
      int m = max_of(old);
      for (int i = 0; i < n; ++i) {
        if (clu[i] == -2)
          old[i] = -2;
        else if (clu[i] >= 0)
          old[i] = m + 1 + clu[i];
      }
    } else {
      result.emplace(sub, clu);
    }
    sizes_cache.erase(sub);
  }

  // pruneRedundancy, ScyTreeNode.cu:669-734, for a region of subspace `sub`
  // holding the points `pts` (npts = the tree's root count)
  bool prune_redundancy(const std::vector<int>& sub, const std::vector<int>& pts, int npts) {
    int max_min = 0;
    for (auto& e : result) {
      if (!is_subsequence(sub, e.first)) continue;
      // smallest cluster of this entry that holds a point of the region
      const std::vector<int>& sz = sizes_of(e.first, e.second);
      int mn = -1;
      for (int p : pts)
        if (e.second[p] >= 0 && (mn == -1 || sz[p] < mn)) mn = sz[p];
      if (mn > max_min) max_min = mn;
    }
    if (max_min == 0) return true;
    return (double)((float)npts * r) > (double)max_min * 1.0;
  }
};

}  // namespace orc_common

// Result of one oracle run, read through the orc_* accessors (C ABI).
struct orc_result {
  std::vector<std::vector<int>> subspaces;
  std::vector<std::vector<int>> labels;
  long long stats[6];
};
