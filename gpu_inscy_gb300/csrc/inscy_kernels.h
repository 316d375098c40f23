// Launchers of the engine's kernels (host-callable, C++ linkage).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "inscy_common.cuh"

namespace inscy {

// ---- primitives / setup (kernels_setup.cu)
void launch_exclusive_scan_int(const int* in, int* out, long long n, int* total, void* sums, cudaStream_t s);
void launch_exclusive_scan_ll(const long long* in, long long* out, long long n, long long* total, void* sums,
                              cudaStream_t s);
void launch_exclusive_scan_i2ll(const int* in, long long* out, long long n, long long* total, void* sums,
                                cudaStream_t s);
void launch_prep(const float* X, int n, int d, int cells, float csz, int G, float fsz, float eps, uint8_t* cc,
                 uint8_t* fc, unsigned long long* gz, cudaStream_t s);
void launch_iota(int* a, int n, cudaStream_t s);
// hist[k * cells + c] += points whose coarse cell on dim k is c (hist zeroed by the caller)
void launch_cell_hist(const uint8_t* cc, int n, int d, int cells, int sms, int* hist, cudaStream_t s);
// rows of `slots` (16, 24 or 32 >= d) coordinates and fine-cell windows per point
void launch_point_rows(const float* X, const uint8_t* fc, int n, int d, int slots, int G, const float* fine_lo,
                       float* xrow, float* win, cudaStream_t s);
void launch_check_range(const float* X, long long m, int* bad, cudaStream_t s);
void launch_scatter_rank(const int* order, int n, int* rank, cudaStream_t s);
void launch_byte_sort_pass(const int* in, int* out, int m, const uint8_t* bytes, int d, int k, int* hist,
                           int* hist_total, int* digit_start, void* sums, cudaStream_t s);
void launch_digit_starts(const int* hist, int nb, int m, int* starts, cudaStream_t s);
void launch_candidate_lists(int n, int d, int G, const int* bucket_pts, const int* bucket_off, const int* rank,
                            const uint8_t* fc, const long long* list_off, int* list_pts, cudaStream_t s);

// ---- density (kernels_density.cu)
// One entry of a neighbour list, 8 bytes: .x the neighbour's id, .y the bits
// of the float sum of squared differences between query and neighbour over
// the list's subspace (its dims in ascending order).  One load or store moves
// a whole entry.
using ListEnt = int2;

struct DensityLaunch {
  const SubDesc* subs;
  int nsubs;
  long long nitems;
  const GroupDesc* groups;
  int ngroups;
  const float* X;
  const uint8_t* fc;
  int n, d, G;
  float eps;
  int rect;
  float acc_max;
  float thr_weak;
  const float* thr_dense;
  const float* thr_keep;
  const long long* cand_off;
  const int* cand_pts;
  const int* prev_keep;
  const long long* prev_loff;
  const int* prev_lcnt;
  const int2* prev_ent;  // parent-level list entries (ListEnt)
  int* cnt;
  uint8_t* flags;
  unsigned* bitmaps;
  int words;
  const long long* loff;
  int2* ent;  // this level's list entries (ListEnt)
  unsigned long long* cand_counter;
  unsigned long long* list_counter;
  unsigned long long* out_counter;  // single-pass write: entries written
  const long long* cap_base;        // single-pass write: list base of every (group, query)
  long long* cap_loff;              // single-pass write: list start of every item (out)
  const float* xrow;                // d <= 32: point rows (coordinates), else null
  const float* win;                 // d <= 32: fine-cell windows [lo, hi) per (point, dim)
  int slots;                        // row width (16, 24 or 32)
  unsigned long long* work;         // work counter of the row kernel (the caller zeroes it before each launch)
  RowItem* items;                   // row kernel: one record per (group, query), written by the capacity kernel
  unsigned long long* phi_work;     // scratch of the phi kernels (kPhiWorkBytes, zeroed by the caller before each launch)
  int sms;                          // SMs of the device: persistent grids fill each once
  int rows_tma;                     // levels >= 2, d <= 32: gather the candidate rows with TMA (k_neighbours_rows_tma)
  int rows_takes;                   // row kernel: work-counter updates per warp the chunk aims at (0: 16)
  int rows_bps;                     // row kernel: resident blocks per SM (0: the most its registers allow)
  long long prev_total;
  long long total;
  long long prev_nkeep;
  Guard guard;
};
void launch_neighbours(const DensityLaunch& L, bool write, cudaStream_t s);
// phi of every item (non-rectangular; `phi` holds nitems floats, `perm`
// nitems ints), then its flags and bitmap bits.  L.phi_work points at
// kPhiWorkBytes of zeroed scratch (the work counter and the class counts).
constexpr int kPhiWorkBytes = 8 + 2 * 64 * 4;
void launch_density_flags(const DensityLaunch& L, float* phi, int* perm, cudaStream_t s);
void launch_list_capacity(const DensityLaunch& L, long long nwarps, long long* cap, cudaStream_t s);
void launch_level1_capacity(const DensityLaunch& L, long long* cap, cudaStream_t s);
void launch_phi_selftest(unsigned long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t s);
void launch_neighbours_multi(const DensityLaunch& L, long long nwarps, bool write, cudaStream_t s);
// resident blocks per SM the row kernel's registers allow (rows of `slots`)
int rows_max_blocks_per_sm(int slots);
void launch_keep_counts(const int* cnt, const uint8_t* flags, long long nitems, int* kcnt, int* kflag,
                        cudaStream_t s);
void launch_keep_compact(const SubDesc* subs, int nsubs, long long nitems, const uint8_t* flags, const int* cnt,
                         const long long* kpos, const long long* loff, const int* prev_keep, int* keep_ids,
                         long long* keep_loff, int* keep_lcnt, cudaStream_t s);
void launch_word_popc(const unsigned* words, long long nw, int* out, cudaStream_t s);
void launch_keep_popc(const unsigned* bm, int nsubs, int W, int* out, cudaStream_t s);
void launch_gather_kstart(const SubDesc* subs, int nsubs, const long long* kpos, long long nitems, long long K,
                          long long* out, cudaStream_t s);
void launch_gather_cbase(const long long* kstart, int nsubs, const int* root_id, long long K, int ncomp, int* out,
                         cudaStream_t s);

// ---- SCY-tree level (kernels_tree.cu)
struct TreeLaunch {
  const CallDesc* calls;
  int ncalls;
  const long long* work_off;
  int nwork;
  const int* pts_in;
  const int2* ghosts_in;
  const uint8_t* cc;
  const unsigned long long* gz;
  int n, d, cells, min_size;
  int kbits;
  const SubDesc* subs;
  const unsigned* bitmaps;
  char* scratch;
  const long long* work_scratch;
  RegionRec* recs;
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
  // work items with more than kTreeBig points + chains (nbig of them, listed
  // in items_big) run in 1024-thread blocks, the others (items_small) in
  // 256-thread blocks; nbig = 0: every item in one 256-thread launch
  const int* items_big;
  int nbig;
  const int* items_small;
  int nsmall;
  int key_bytes;  // leaf key width: 4, 8 or 16 bytes (d * kbits bits must fit)
  // the SCY-tree's level order (get_subspace_order, inscy_map.cpp:61-121):
  // level of every dim, dim of every level, and per dim e the levels of the
  // dims > e (restrict_node's inclusion test, ScyTreeNode.cu:285)
  uint8_t lvl_pos[kMaxDims];
  uint8_t lvl_dim[kMaxDims];
  unsigned long long gt_pos[kMaxDims];
};
#ifndef INSCY_TREE_BIG
#define INSCY_TREE_BIG 4096
#endif
constexpr long long kTreeBig = INSCY_TREE_BIG;
void launch_tree_level(const TreeLaunch& L, cudaStream_t s);

// ---- clustering (kernels_cluster.cu)
struct ClusterArgs {
  int nsubs;
  const SubDesc* subs;
  const long long* kstart;  // [nsubs + 1] first kept index of each subspace
  const int* keep_ids;
  const long long* keep_loff;
  const int* keep_lcnt;
  const int2* ent;  // list entries (ListEnt); .x is the neighbour
  const unsigned* bitmaps;
  int words;
  const int* keep_word_rank;  // [nsubs * words] global prefix of kept popcounts
  const uint8_t* clustered;   // [nsubs]
  const int* clustered_list;  // [nclustered] subspace of each clustered slot
  long long nkeep;
  int n;
  int* uf;
  int* err;
  Guard guard;
  const int* sub_of;  // [nkeep] subspace of every kept point (launch_sub_of_keep)
};
void launch_sub_of_keep(const long long* kstart, int nsubs, long long nkeep, int* sub_of, cudaStream_t s);
void launch_uf_init(int* par, long long n, cudaStream_t s);
void launch_uf_union(const ClusterArgs& a, int nclustered, const int* cslot_of, int* sample, uint8_t* dom,
                     cudaStream_t s);
// level 1 (one-dim subspaces): components as runs in coordinate order
// instead of union-find (kept points K; element buffers of K; hist of
// 256 * ceil(K / kSortTile) ints)
struct UfLevel1Scratch {
  int* flag;       // K
  int* pos;        // K + 1
  int* total;      // 1
  int* kidx;       // K
  uint8_t* kbytes; // 5 K
  int* perm0;      // K
  int* perm1;      // K
  int* hist;
  int* start;      // K
  int* runx;       // K + 1
  int* runmin;     // K
};
// first the dense points of clustered subspaces are counted (*w.total), then
// with that count m the runs are found and the parents set
void launch_uf_level1_count(const ClusterArgs& a, const UfLevel1Scratch& w, void* sums, cudaStream_t s);
void launch_uf_level1(const ClusterArgs& a, const float* X, int d, const uint8_t* fc, float acc_max,
                      const UfLevel1Scratch& w, int m, void* sums, cudaStream_t s);
void launch_uf_flatten(const ClusterArgs& a, int* is_root, int* root_of, cudaStream_t s);
void launch_comp_ids(const ClusterArgs& a, const int* root_id, const int* root_of, int* comp, int* mcount,
                     cudaStream_t s);
void launch_members(const ClusterArgs& a, const int* comp, const long long* moff, int* mfill, int* members,
                    cudaStream_t s);
void launch_borders(const ClusterArgs& a, const int* comp, const int* cslot_of, int* slots, int2* ovf, int* novf,
                    int ovf_cap, cudaStream_t s);
void launch_border_count(const int* slots, long long nslots2, const int2* ovf, int novf, int* bcount, cudaStream_t s);
void launch_border_fill(const int* slots, long long nslots2, int n, const int2* ovf, int novf, const long long* boff,
                        int* bfill, int* borders, cudaStream_t s);
void launch_region_order(const ClusterArgs& a, int nclustered, const int* comp, const int* cbase_of,
                         const int* sub_calls_off, const int* sub_calls, const CallDesc* ncalls, const int* pts,
                         int* firstpos, int* order, int* order_cnt, cudaStream_t s);

void launch_pack_order(const CallDesc* ncalls, int ncall, const int* order, const int* order_cnt,
                       const long long* order_off, int* packed, cudaStream_t s);

}  // namespace inscy
