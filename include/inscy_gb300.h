/*
 * inscy_gb300.h -- C ABI of the GB300 INSCY engine (libinscy_gb300.so).
 *
 * Drop-in for the GPU run of mrjakobdk/GPU_INSCY: the entry points below
 * replace the torch-extension functions
 *   run_gpu_5(X, neighborhood_size, F, num_obj, min_size, r, number_of_cells,
 *             rectangular, entropy_order)          inscy_map.cpp:1070-1158
 *   run_gpu_4(...same...)                          inscy_map.cpp:979-1067
 * reached from GPU5() / GPU() in python/inscy.py:189-197, and return the same
 * [subspaces, clusterings] content: one entry per clustered subspace (dims in
 * ascending order), entries ordered as the reference's result map
 * (vec_cmp, util.cu:633-653), each with one int32 label per point
 * (cluster ids >= 1, -1 noise, -2 border points) -- bit-identical to the
 * reference CPU INSCY (run_cpu3_weak, inscy_map.cpp:230-270).
 *
 * Plain pointers and sizes only.  Every function returns INSCY_OK (0) or an
 * error code; inscy_last_error() then describes the failure (thread-local).
 * Nothing calls exit(): where the reference aborts through gpuAssert
 * (InscyArrayGpuMulti2.cu:19-29) these return INSCY_ERR_CUDA.
 */
#ifndef INSCY_GB300_H
#define INSCY_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  INSCY_OK = 0,
  INSCY_ERR_ARG = 1,         /* bad argument (null pointer, n < 0, d out of range, values outside [0,1]) */
  INSCY_ERR_CUDA = 2,        /* a CUDA call failed (no device, out of memory, launch failure) */
  INSCY_ERR_UNSUPPORTED = 3, /* option not implemented (no option returns it at present) */
  INSCY_ERR_LIMIT = 4,       /* input beyond a documented limit (d > 64, ceil(1/eps) > 256, cells > 255) */
  INSCY_ERR_INTERNAL = 5     /* a device-side consistency check failed */
};

/* Parameters of run_gpu_5 / run_cpu3_weak, same meaning and types. */
typedef struct inscy_params {
  float neighborhood_size; /* eps of the epsilon-neighbourhood */
  float F;                 /* density factor */
  int num_obj;             /* minimum number of objects term of the threshold */
  int min_size;            /* absolute minimum cluster/region size */
  float r;                 /* redundancy factor */
  int number_of_cells;     /* grid cells per dimension of the SCY-tree */
  int rectangular;         /* 0: phi density (ClusteringCpu.cu:166-176); 1: neighbour count (:178-183) */
  int entropy_order;       /* level order of the trees (inscy_map.cpp:61-121): 0 identity, -1 by
                              descending cell entropy, any other value by ascending entropy */
} inscy_params;

/* Execution form of inscy_run_batch.  PLAIN: the datasets one after another.
 * BATCHED: the datasets on concurrent lanes (inscy_run_batch_scheduled with
 * the given order and 4 lanes).  Results are the same either way. */
enum { INSCY_MODE_PLAIN = 0, INSCY_MODE_BATCHED = 1 };

typedef struct inscy_result inscy_result;

/* Run statistics of the last run that produced a result. */
typedef struct inscy_stats {
  double ms_total;          /* wall time of the run (host clock) */
  double ms_setup;          /* grid cells, trie order, candidate lists */
  double ms_density;        /* density kernels (pass 1 + pass 2), device time */
  double ms_density_pass1;  /* the candidate pass alone (count pass, or the single-pass write), device time */
  double ms_tree;           /* restrict/merge/prune kernels, device time */
  double ms_cluster;        /* union-find + component kernels, device time */
  double ms_replay;         /* host commit (pruneRedundancy, numbering, join) */
  double ms_replay_prune;   /* ... of which pruneRedundancy */
  double ms_replay_cluster; /* ... of which cluster numbering */
  double ms_replay_join;    /* ... of which join */
  double ms_d2h;            /* device-to-host copies (synchronous, host clock) */
  double density_bytes;     /* algorithmic bytes of the density count launches */
  double tree_bytes;        /* algorithmic bytes of the tree launches */
  long long density_launches_pass1;
  long long kernel_launches; /* kernels launched by this run */
  long long calls;           /* INSCY recursion nodes */
  long long regions;         /* restricted (and merged) regions */
  long long subspaces;       /* subspaces evaluated */
  long long candidates;      /* candidate pairs tested */
  long long levels;
  long long h2d_bytes, d2h_bytes;
  /* commit work counters: joins with clusters, new entries, label writes,
   * border writes, superset entries examined by join, points visited by
   * join's redundancy test, pruneRedundancy calls, points visited by
   * pruneRedundancy, clusters numbered, border checks while numbering */
  long long replay_counters[10];
  double ms_expand;       /* wall time of the expansion (the GPU-driving thread) */
  double ms_commit_tail;  /* time the run waited for the commit once the expansion was done */
  /* launch shape of the candidate pass's row kernel (d <= 32): work-counter
   * updates per warp that the pairs-per-update chunk aims at, and resident
   * blocks per SM, chosen by the engine's tuner (measured once per row width
   * and device in the process, on the first level with enough pairs), and the
   * device time of the tuner's trial launches in this run */
  int rows_takes;
  int rows_blocks_per_sm;
  double ms_tune;
} inscy_stats;

/* Replaces run_gpu_5 / run_gpu_4 (inscy_map.cpp:1070-1158 / :979-1067).
 * X: host, float32, row-major [n, d], values in [0, 1] (the reference's
 * cell rule, ScyTreeNode.cu:100-102, assumes this).  X is only read.  The
 * result is owned by the caller and released with inscy_result_free. */
int inscy_run(const float* X, int64_t n, int d, const inscy_params* p, int mode, inscy_result** out);

/* Same, with X already in device memory (a CUDA device pointer) and the work
 * queued on `stream` (a cudaStream_t, NULL = legacy default stream).  The
 * call is synchronous: it returns once the result is on the host. */
int inscy_run_device(const float* X_dev, int64_t n, int d, const inscy_params* p, int mode, void* stream,
                     inscy_result** out);

/* Many independent datasets (the batched workload): outs[i] receives the
 * result of Xs[i] ([ns[i], ds[i]], host).  Same semantics as `count` calls of
 * inscy_run; on failure every outs[i] is NULL. */
int inscy_run_batch(const float* const* Xs, const int64_t* ns, const int* ds, int count, const inscy_params* p,
                    int mode, inscy_result** outs);

/* The batched form (no counterpart in the reference, whose batched runs are
 * sequential): `lanes` host threads, each with its own engine and CUDA
 * stream, run the datasets concurrently -- their kernels overlap on the GPU
 * and their ordered commits on the host cores.  Each lane takes the next
 * dataset of `order` (a permutation of 0..count-1; NULL: 0, 1, ...), so the
 * order is the schedule (a cost model can put the longest datasets first).
 * outs[i] receives the result of Xs[i], identical to inscy_run's.  1 <= lanes
 * <= 64.  Calls are serialised within a process.  On failure every outs[i]
 * is NULL (results of datasets that had finished are freed). */
int inscy_run_batch_scheduled(const float* const* Xs, const int64_t* ns, const int* ds, int count,
                              const inscy_params* p, const int* order, int lanes, inscy_result** outs);

/* Cost model of the batch scheduler (no counterpart in the reference): an MLP
 * in -> 64 -> 64 -> 1 with ReLU, parameters flat float32 in the order W1 (64 x
 * in, row-major), b1 (64), W2 (64 x 64), b2 (64), w3 (64), b3 (1):
 * inscy_mlp_params(in, 64) of them (-1 for a bad shape).  Rows of X are
 * feature vectors, row-major [rows, in].  Training runs `steps` full-batch Adam
 * steps (beta 0.9/0.999, eps 1e-8, learning rate lr) of the mean squared error
 * on the GPU and updates `params` in place; loss_hist[t] receives the loss
 * before step t.  inscy_mlp_grad returns the loss and its gradient at
 * `params` (for checking the training kernels).  hidden must be 64 and
 * 1 <= in <= 64.  These functions allocate device memory per call.  On error
 * they return a nonzero code and inscy_mlp_last_error() describes it. */
int inscy_mlp_params(int in, int hidden);
int inscy_mlp_train(float* params, int in, int hidden, const float* X, const float* y, int rows, int steps, float lr,
                    float* loss_hist);
int inscy_mlp_predict(const float* params, int in, int hidden, const float* X, int rows, float* out);
int inscy_mlp_grad(const float* params, int in, int hidden, const float* X, const float* y, int rows, float* grad,
                   float* loss);
const char* inscy_mlp_last_error(void);

/* Result access. */
int inscy_result_count(const inscy_result* r);              /* number of clustered subspaces */
int64_t inscy_result_n(const inscy_result* r);              /* number of points */
int inscy_result_subspace(const inscy_result* r, int i, int* dims, int cap); /* returns |S|, writes min(|S|,cap) dims;
                                                                          -1: bad index, or dims NULL with cap > 0 */
int inscy_result_labels(const inscy_result* r, int i, int32_t* out);        /* copies n labels */
const int32_t* inscy_result_labels_ptr(const inscy_result* r, int i);       /* n labels, valid until free; NULL on bad i */
/* The whole result in a few calls (no counterpart in the reference, whose
 * binding converts to Python lists): every clustered subspace's dims, back
 * to back, with lens[i] = |S_i| (returns the dims written, at most cap, or
 * -1); the label vectors as blocks of `*rows` rows of n int32 each
 * (inscy_result_label_blocks returns the block count, inscy_result_label_block
 * the first row of block b), and the row ("slot") of each clustered
 * subspace's labels: row s lies in block s / rows at (s % rows) * n.  All
 * valid until inscy_result_free. */
int inscy_result_subspaces(const inscy_result* r, int32_t* dims, int cap, int32_t* lens);
int inscy_result_label_blocks(const inscy_result* r, int* rows);
const int32_t* inscy_result_label_block(const inscy_result* r, int b);
int inscy_result_label_slots(const inscy_result* r, int32_t* slots);
int inscy_result_stats(const inscy_result* r, inscy_stats* out);
void inscy_result_free(inscy_result* r);

/* Description of the last error of the calling thread ("" if none). */
const char* inscy_last_error(void);

/* Library version string. */
const char* inscy_version(void);

/* Device self-test: checks `count` pseudo-random and edge inputs of the
 * integer form of the reference's phi accumulation step against the
 * double-precision expression on the current GPU.  Returns the number of
 * mismatches (0 expected), or -1 with inscy_last_error() set. */
int64_t inscy_selftest(int64_t count);

/* inscy_selftest without any device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc while they check a
 * GPU, e.g. a process whose device memory is already fully handed to a
 * caching allocator or capped, or a latency-critical path that must avoid
 * cudaMalloc's implicit synchronisation.  The only scratch, the mismatch
 * counter, is a 256-byte file-scope device array inside the library (held on
 * every GPU that loads it until exit).  The first call on a device looks up
 * the array's device address, so make that first call before any stream
 * capture.  Every call clears the counter; calls that overlap on the GPU
 * share it and race.  The looked-up address belongs to the device's current
 * context: after a cudaDeviceReset of that device, do not call this entry on
 * it again in the same process (the address is looked up anew only after a
 * failed call).  An error already pending in the CUDA runtime when the entry
 * is called is left in place and reported as INSCY_SELFTEST_NOALLOC_CUDA.
 * Same result as inscy_selftest(count) (work queued on `stream`, a
 * cudaStream_t or NULL).  count is limited to
 * INSCY_SELFTEST_NOALLOC_MAX; returns the mismatch count (0 expected),
 * INSCY_SELFTEST_NOALLOC_TOO_LARGE for count < 0 or above the limit, or
 * INSCY_SELFTEST_NOALLOC_CUDA when a CUDA call fails.  It does not touch
 * inscy_last_error(). */
#define INSCY_SELFTEST_NOALLOC_MAX (1LL << 31)
#define INSCY_SELFTEST_NOALLOC_TOO_LARGE (-1)
#define INSCY_SELFTEST_NOALLOC_CUDA (-2)
int64_t inscy_selftest_noalloc(int64_t count, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* INSCY_GB300_H */
