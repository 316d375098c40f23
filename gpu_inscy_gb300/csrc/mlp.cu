// Cost model for the batch scheduler: a small MLP (in -> 64 -> 64 -> 1, ReLU)
// trained and evaluated by the kernels below.  It predicts the log run time of
// a dataset from cheap features; the schedule (longest predicted first) only
// orders work, so a wrong prediction costs time, never labels.
//
// Parameters, flat float32: W1[H][in], b1[H], W2[H][H], b2[H], w3[H], b3.
// Loss: mean squared error over the rows.
//
// The problem is tiny (hundreds of rows, ~5k parameters), so one block does a
// whole training run: per step every row's forward and backward pass (four
// rows at a time, 64 threads each), gradients summed in shared memory, then an
// Adam update -- one launch for all steps.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/inscy_gb300.h"

namespace inscy {

constexpr int kH = 64;           // hidden width
constexpr int kMaxIn = 64;       // feature count limit
constexpr int kRowsPar = 4;      // rows in flight per block
constexpr int kMlpThreads = kH * kRowsPar;

__host__ __device__ inline int mlp_nparams(int in) { return kH * in + kH + kH * kH + kH + kH + 1; }

struct MlpView {
  const float *W1, *b1, *W2, *b2, *w3, *b3;
  __device__ MlpView(const float* p, int in)
      : W1(p), b1(p + kH * in), W2(p + kH * in + kH), b2(p + kH * in + kH + kH * kH),
        w3(p + kH * in + kH + kH * kH + kH), b3(p + kH * in + kH + kH * kH + kH + kH) {}
};

// Forward and (optionally) backward pass of row r on the 64 threads of group
// g; gradients are added to grad (shared or global), the loss to *loss.
__device__ void mlp_row(const MlpView& P, int in, const float* x, float y, float scale, float* grad, float* loss,
                        float* out, bool backward, float* s_a1, float* s_z1, float* s_a2, float* s_z2, float* s_red) {
  const int j = threadIdx.x % kH;
  // layer 1
  float z1 = P.b1[j];
  for (int i = 0; i < in; ++i) z1 = fmaf(P.W1[j * in + i], x[i], z1);
  s_z1[j] = z1;
  s_a1[j] = z1 > 0.f ? z1 : 0.f;
  __syncwarp(0xffffffffu);
  // the 64 threads of a group are two warps: the group barrier is a named one
  asm volatile("bar.sync %0, %1;" ::"r"(1 + threadIdx.x / kH), "r"(kH));
  float z2 = P.b2[j];
  for (int k = 0; k < kH; ++k) z2 = fmaf(P.W2[j * kH + k], s_a1[k], z2);
  s_z2[j] = z2;
  const float a2 = z2 > 0.f ? z2 : 0.f;
  s_a2[j] = a2;
  // output: sum over the group
  float part = P.w3[j] * a2;
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((j & 31) == 0) s_red[j >> 5] = part;
  asm volatile("bar.sync %0, %1;" ::"r"(1 + threadIdx.x / kH), "r"(kH));
  const float o_ = P.b3[0] + s_red[0] + s_red[1];
  if (j == 0 && out) *out = o_;
  if (!backward) return;
  const float e = o_ - y;
  if (j == 0) atomicAdd(loss, scale * e * e);
  const float dout = 2.f * scale * e;
  const int nW1 = kH * in, ob1 = nW1, oW2 = ob1 + kH, ob2 = oW2 + kH * kH, ow3 = ob2 + kH, ob3 = ow3 + kH;
  atomicAdd(&grad[ow3 + j], dout * a2);
  if (j == 0) atomicAdd(&grad[ob3], dout);
  const float dz2 = s_z2[j] > 0.f ? dout * P.w3[j] : 0.f;
  atomicAdd(&grad[ob2 + j], dz2);
  for (int k = 0; k < kH; ++k) atomicAdd(&grad[oW2 + j * kH + k], dz2 * s_a1[k]);
  s_red[2 + j] = dz2;  // shared dz2 for the layer-1 pass (s_red has 2 + 64 slots)
  asm volatile("bar.sync %0, %1;" ::"r"(1 + threadIdx.x / kH), "r"(kH));
  float da1 = 0.f;
  for (int k = 0; k < kH; ++k) da1 = fmaf(P.W2[k * kH + j], s_red[2 + k], da1);
  const float dz1 = s_z1[j] > 0.f ? da1 : 0.f;
  atomicAdd(&grad[ob1 + j], dz1);
  for (int i = 0; i < in; ++i) atomicAdd(&grad[j * in + i], dz1 * x[i]);
  asm volatile("bar.sync %0, %1;" ::"r"(1 + threadIdx.x / kH), "r"(kH));
}

struct RowScratch {
  float a1[kRowsPar][kH], z1[kRowsPar][kH], a2[kRowsPar][kH], z2[kRowsPar][kH], red[kRowsPar][2 + kH];
  float x[kRowsPar][kMaxIn];
};

// loss and gradient over all rows at params p (one block)
__device__ void mlp_loss_grad(const float* p, int in, const float* X, const float* y, int rows, float* grad,
                              float* loss, RowScratch& s) {
  const MlpView P(p, in);
  const int g = threadIdx.x / kH, j = threadIdx.x % kH;
  const float scale = 1.f / (float)rows;
  for (int r0 = 0; r0 < rows; r0 += kRowsPar) {
    const int r = r0 + g;
    const bool live = r < rows;  // the group of a missing row idles through the same barriers
    for (int i = j; i < in; i += kH) s.x[g][i] = live ? X[(size_t)r * in + i] : 0.f;
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kH));
    mlp_row(P, in, s.x[g], live ? y[r] : 0.f, live ? scale : 0.f, grad, loss, nullptr, true, s.a1[g], s.z1[g],
            s.a2[g], s.z2[g], s.red[g]);
  }
}

constexpr int kMaxParams = kH * kMaxIn + kH + kH * kH + kH + kH + 1;

__global__ void __launch_bounds__(kMlpThreads) k_mlp_grad(const float* p, int in, const float* X, const float* y,
                                                           int rows, float* grad, float* loss) {
  __shared__ RowScratch s;
  __shared__ float sg[kMaxParams];
  __shared__ float sl;
  const int np = mlp_nparams(in);
  for (int i = threadIdx.x; i < np; i += blockDim.x) sg[i] = 0.f;
  if (threadIdx.x == 0) sl = 0.f;
  __syncthreads();
  mlp_loss_grad(p, in, X, y, rows, sg, &sl, s);
  __syncthreads();
  for (int i = threadIdx.x; i < np; i += blockDim.x) grad[i] = sg[i];
  if (threadIdx.x == 0) *loss = sl;
}

// `steps` Adam steps (beta 0.9 / 0.999, eps 1e-8) on the whole batch;
// loss_hist[t] = loss before step t
__global__ void __launch_bounds__(kMlpThreads) k_mlp_train(float* p, int in, const float* X, const float* y, int rows,
                                                            int steps, float lr, float* m, float* v, float* loss_hist) {
  __shared__ RowScratch s;
  __shared__ float grad[kMaxParams];
  __shared__ float loss;
  const int np = mlp_nparams(in);
  float b1t = 1.f, b2t = 1.f;
  for (int t = 0; t < steps; ++t) {
    for (int i = threadIdx.x; i < np; i += blockDim.x) grad[i] = 0.f;
    if (threadIdx.x == 0) loss = 0.f;
    __syncthreads();
    mlp_loss_grad(p, in, X, y, rows, grad, &loss, s);
    __syncthreads();
    if (threadIdx.x == 0) loss_hist[t] = loss;
    b1t *= 0.9f;
    b2t *= 0.999f;
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      const float gi = grad[i];
      const float mi = 0.9f * m[i] + 0.1f * gi, vi = 0.999f * v[i] + 0.001f * gi * gi;
      m[i] = mi;
      v[i] = vi;
      p[i] -= lr * (mi / (1.f - b1t)) / (sqrtf(vi / (1.f - b2t)) + 1e-8f);
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kMlpThreads) k_mlp_predict(const float* p, int in, const float* X, int rows,
                                                              float* out) {
  __shared__ RowScratch s;
  const MlpView P(p, in);
  const int g = threadIdx.x / kH, j = threadIdx.x % kH;
  const int stride = gridDim.x * kRowsPar;
  for (int r0 = blockIdx.x * kRowsPar; r0 < rows; r0 += stride) {
    const int r = r0 + g;
    const bool live = r < rows;
    for (int i = j; i < in; i += kH) s.x[g][i] = live ? X[(size_t)r * in + i] : 0.f;
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kH));
    float o = 0.f;
    mlp_row(P, in, s.x[g], 0.f, 0.f, nullptr, nullptr, live ? &o : nullptr, false, s.a1[g], s.z1[g], s.a2[g],
            s.z2[g], s.red[g]);
    if (live && j == 0) out[r] = o;
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kH));
  }
}

}  // namespace inscy

// ---------------------------------------------------------------- C ABI
namespace {
thread_local std::string g_mlp_err;

struct DevBufs {
  float* b[8] = {nullptr};
  ~DevBufs() {
    for (float* x : b)
      if (x) cudaFree(x);
  }
};

int mlp_check(int rows, int in, int hidden) {
  if (hidden != inscy::kH) {
    g_mlp_err = "hidden width must be 64";
    return INSCY_ERR_ARG;
  }
  if (in < 1 || in > inscy::kMaxIn || rows < 0) {
    g_mlp_err = "bad feature count or row count";
    return INSCY_ERR_ARG;
  }
  return INSCY_OK;
}

#define MCK(x)                                                      \
  do {                                                              \
    cudaError_t e_ = (x);                                           \
    if (e_ != cudaSuccess) {                                        \
      g_mlp_err = std::string(#x) + ": " + cudaGetErrorString(e_); \
      return INSCY_ERR_CUDA;                                        \
    }                                                               \
  } while (0)

int up(float** d, const float* h, size_t n) {
  MCK(cudaMalloc(d, (n ? n : 1) * sizeof(float)));
  if (h && n) MCK(cudaMemcpy(*d, h, n * sizeof(float), cudaMemcpyHostToDevice));
  return INSCY_OK;
}
}  // namespace

extern "C" {

int inscy_mlp_params(int in, int hidden) { return hidden == inscy::kH && in >= 1 ? inscy::mlp_nparams(in) : -1; }

int inscy_mlp_grad(const float* params, int in, int hidden, const float* X, const float* y, int rows, float* grad,
                   float* loss) {
  int rc = mlp_check(rows, in, hidden);
  if (rc) return rc;
  if (!params || !grad || !loss || (rows > 0 && (!X || !y))) return g_mlp_err = "NULL argument", INSCY_ERR_ARG;
  const int np = inscy::mlp_nparams(in);
  DevBufs B;
  if ((rc = up(&B.b[0], params, np)) || (rc = up(&B.b[1], X, (size_t)rows * in)) || (rc = up(&B.b[2], y, rows)) ||
      (rc = up(&B.b[3], nullptr, np)) || (rc = up(&B.b[4], nullptr, 1)))
    return rc;
  inscy::k_mlp_grad<<<1, inscy::kMlpThreads>>>(B.b[0], in, B.b[1], B.b[2], rows, B.b[3], B.b[4]);
  MCK(cudaGetLastError());
  MCK(cudaMemcpy(grad, B.b[3], np * sizeof(float), cudaMemcpyDeviceToHost));
  MCK(cudaMemcpy(loss, B.b[4], sizeof(float), cudaMemcpyDeviceToHost));
  return INSCY_OK;
}

int inscy_mlp_train(float* params, int in, int hidden, const float* X, const float* y, int rows, int steps, float lr,
                    float* loss_hist) {
  int rc = mlp_check(rows, in, hidden);
  if (rc) return rc;
  if (!params || !loss_hist || steps < 0 || rows < 1 || !X || !y) return g_mlp_err = "bad argument", INSCY_ERR_ARG;
  const int np = inscy::mlp_nparams(in);
  DevBufs B;
  if ((rc = up(&B.b[0], params, np)) || (rc = up(&B.b[1], X, (size_t)rows * in)) || (rc = up(&B.b[2], y, rows)) ||
      (rc = up(&B.b[4], nullptr, np)) || (rc = up(&B.b[5], nullptr, np)) || (rc = up(&B.b[6], nullptr, steps)))
    return rc;
  MCK(cudaMemset(B.b[4], 0, np * sizeof(float)));
  MCK(cudaMemset(B.b[5], 0, np * sizeof(float)));
  inscy::k_mlp_train<<<1, inscy::kMlpThreads>>>(B.b[0], in, B.b[1], B.b[2], rows, steps, lr, B.b[4], B.b[5], B.b[6]);
  MCK(cudaGetLastError());
  MCK(cudaMemcpy(params, B.b[0], np * sizeof(float), cudaMemcpyDeviceToHost));
  if (steps) MCK(cudaMemcpy(loss_hist, B.b[6], steps * sizeof(float), cudaMemcpyDeviceToHost));
  return INSCY_OK;
}

int inscy_mlp_predict(const float* params, int in, int hidden, const float* X, int rows, float* out) {
  int rc = mlp_check(rows, in, hidden);
  if (rc) return rc;
  if (rows == 0) return INSCY_OK;
  if (!params || !X || !out) return g_mlp_err = "NULL argument", INSCY_ERR_ARG;
  const int np = inscy::mlp_nparams(in);
  DevBufs B;
  if ((rc = up(&B.b[0], params, np)) || (rc = up(&B.b[1], X, (size_t)rows * in)) || (rc = up(&B.b[2], nullptr, rows)))
    return rc;
  const int blocks = (rows + inscy::kRowsPar - 1) / inscy::kRowsPar;
  inscy::k_mlp_predict<<<blocks < 304 ? blocks : 304, inscy::kMlpThreads>>>(B.b[0], in, B.b[1], rows, B.b[2]);
  MCK(cudaGetLastError());
  MCK(cudaMemcpy(out, B.b[2], rows * sizeof(float), cudaMemcpyDeviceToHost));
  return INSCY_OK;
}

const char* inscy_mlp_last_error(void) { return g_mlp_err.c_str(); }

}  // extern "C"
