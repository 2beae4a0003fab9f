// warmstart.cu -- learned warm start: a small MLP maps per-row sparsity and
// value statistics of a tensor to initial factor rows.  No reference
// counterpart (the reference always starts from uniform [0,1) draws,
// tucker.cuh:84-97; that stays the fallback).
//
// Features of row i of mode n (F = 4 + 6(N-1) + N values):
//   log(1 + c_i), mean x, std x over the row's c_i nonzeros;
//   for every other mode m (increasing): over the row's nonzeros, the mean and std
//   of mu_m[i_m] (the mean value of the co-indexed row of mode m), the mean of
//   lc_m = log(1 + c_m[i_m]) (its density), and the cross moments E[x mu_m],
//   E[x mu_m^2], E[x lc_m] (how the row's values vary with the co-indexed rows);
//   E[x prod_m mu_m];
//   one-hot of n.
// Each feature is standardised with the mean/std of the training examples.
//
// Network: y = W3 relu(W2 relu(W1 f + b1) + b2) + b3, H hidden units, J outputs
// (one factor row).  Loss = mean over the batch and the J outputs of (y - t)^2,
// t = the factor row the plain ALS method converged to on a training tensor.
// Training and inference run in the kernels below (FP32): the forward pass, the
// loss gradient, the backward pass as small tiled GEMMs (activation gradients and
// weight gradients reduced over the batch), and Adam.
//
// Row statistics: the mode-m view is sorted by row, so a thread takes a
// contiguous chunk of nonzeros, sums per row in registers and flushes with an
// atomic add only when the row changes.  The sums are FP64: the standard
// deviations come from E[a^2] - E[a]^2, which cancels in FP32 when the spread is
// small against the mean (a one-time pass: the FP64 adds cost nothing visible).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

struct gtk_ws {
  int dev = 0, N = 0, J = 0, H = 0, F = 0;
  size_t np = 0;                  // trainable parameters
  float *w = nullptr;             // [W1 H*F | b1 H | W2 H*H | b2 H | W3 J*H | b3 J]
  float *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // gradient, Adam moments
  std::vector<float> fmean, fstd;  // feature standardisation (host)
  float *d_fmean = nullptr, *d_fstd = nullptr;
  bool have_norm = false;
  uint64_t adam_t = 0;
  uint64_t seed = 0;
  cudaStream_t stream = nullptr;
  // training examples: features (raw) and targets, grown by gtk_ws_add_example
  float *ex_f = nullptr, *ex_t = nullptr;
  uint64_t ex_n = 0, ex_cap = 0;
  // batch scratch
  int bcap = 0;
  float *bx = nullptr, *bt = nullptr, *h1 = nullptr, *h2 = nullptr, *y = nullptr, *dy = nullptr, *d2 = nullptr,
        *d1 = nullptr;
  double *loss = nullptr;
};

using namespace gtk;

namespace {

constexpr int kWsThreads = 256;
constexpr int kChunk = 64;  // nonzeros per thread in the row-statistics kernels

inline size_t ws_np(int F, int H, int J) { return (size_t)H * F + H + (size_t)H * H + H + (size_t)J * H + J; }

struct WsParams {
  const float *W1, *b1, *W2, *b2, *W3, *b3;
};
WsParams params_of(const gtk_ws *m, const float *w) {
  WsParams p;
  p.W1 = w;
  p.b1 = p.W1 + (size_t)m->H * m->F;
  p.W2 = p.b1 + m->H;
  p.b2 = p.W2 + (size_t)m->H * m->H;
  p.W3 = p.b2 + m->H;
  p.b3 = p.W3 + (size_t)m->J * m->H;
  return p;
}

// ---------------------------------------------------------------- row statistics
// per row of the view: count, sum x, sum x^2 (FP64 sums)
template <class V>
__global__ void k_row_stats(const uint32_t *__restrict__ row, const V *__restrict__ val, uint64_t nnz,
                            double *__restrict__ cnt, double *__restrict__ s1, double *__restrict__ s2) {
  const uint64_t t0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kChunk;
  if (t0 >= nnz) return;
  const uint64_t t1 = min(nnz, t0 + kChunk);
  uint32_t r = row[t0];
  double c = 0, a = 0, b = 0;
  for (uint64_t t = t0; t < t1; ++t) {
    const uint32_t rr = row[t];
    if (rr != r) {
      atomicAdd(cnt + r, c);
      atomicAdd(s1 + r, a);
      atomicAdd(s2 + r, b);
      r = rr;
      c = a = b = 0;
    }
    const double x = (double)val[t];
    c += 1;
    a += x;
    b += x * x;
  }
  atomicAdd(cnt + r, c);
  atomicAdd(s1 + r, a);
  atomicAdd(s2 + r, b);
}

// mu = sum / count, lc = log(1 + count) per row of a mode
__global__ void k_row_mean(const double *__restrict__ cnt, const double *__restrict__ s1, double *__restrict__ mu,
                           double *__restrict__ lc, uint64_t rows) {
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x) {
    const double c = cnt[r];
    mu[r] = c > 0 ? s1[r] / c : 0.0;
    lc[r] = log1p(c);
  }
}

inline int ws_nfeat(int N) { return 4 + 6 * (N - 1) + N; }

struct CoArgs {
  const uint32_t *row;             // view of mode n: global row of mode n
  const void *val;                 // view of mode n: values
  const uint32_t *coord[kMaxOrder];  // view of mode n: coordinates of the other modes (compact, D entries)
  const double *mu[kMaxOrder];
  const double *lc[kMaxOrder];
  int D;
};

// per row of mode n, for each other mode d: sums of mu, mu^2, lc, x mu, x mu^2,
// x lc over the row's nonzeros (6 per mode), then the sum of x prod_d mu_d
template <class V>
__global__ void k_coindex(CoArgs a, uint64_t nnz, double *__restrict__ acc /* rows x (6D + 1) */) {
  const uint64_t t0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kChunk;
  if (t0 >= nnz) return;
  const uint64_t t1 = min(nnz, t0 + kChunk);
  const int D = a.D, W = 6 * D + 1;
  const V *val = reinterpret_cast<const V *>(a.val);
  uint32_t r = a.row[t0];
  double s[6 * (kMaxOrder - 1) + 1];
  for (int k = 0; k < W; ++k) s[k] = 0;
  for (uint64_t t = t0; t < t1; ++t) {
    const uint32_t rr = a.row[t];
    if (rr != r) {
      for (int k = 0; k < W; ++k) {
        atomicAdd(acc + (size_t)r * W + k, s[k]);
        s[k] = 0;
      }
      r = rr;
    }
    const double x = (double)val[t];
    double prod = x;
    for (int d = 0; d < D; ++d) {
      const uint32_t c = a.coord[d][t];
      const double m = a.mu[d][c], l = a.lc[d][c];
      s[6 * d] += m;
      s[6 * d + 1] += m * m;
      s[6 * d + 2] += l;
      s[6 * d + 3] += x * m;
      s[6 * d + 4] += x * m * m;
      s[6 * d + 5] += x * l;
      prod *= m;
    }
    s[6 * D] += prod;
  }
  for (int k = 0; k < W; ++k) atomicAdd(acc + (size_t)r * W + k, s[k]);
}

// raw features of rows [0, rows) of mode n, F per row
__global__ void k_features(const double *__restrict__ cnt, const double *__restrict__ s1,
                           const double *__restrict__ s2, const double *__restrict__ acc, uint64_t rows, int N, int n,
                           int F, float *__restrict__ out) {
  const int D = N - 1;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x) {
    float *o = out + r * F;
    const double c = cnt[r];
    const double inv = c > 0 ? 1.0 / c : 0.0;
    const double mean = s1[r] * inv;
    const double var = fmax(0.0, s2[r] * inv - mean * mean);
    o[0] = (float)log1p(c);
    o[1] = (float)mean;
    o[2] = (float)sqrt(var);
    const double *q0 = acc + r * (6 * D + 1);
    for (int d = 0; d < D; ++d) {
      const double *q = q0 + 6 * d;
      const double m = q[0] * inv;
      o[3 + 6 * d] = (float)m;
      o[4 + 6 * d] = (float)sqrt(fmax(0.0, q[1] * inv - m * m));
      o[5 + 6 * d] = (float)(q[2] * inv);
      o[6 + 6 * d] = (float)(q[3] * inv);
      o[7 + 6 * d] = (float)(q[4] * inv);
      o[8 + 6 * d] = (float)(q[5] * inv);
    }
    o[3 + 6 * D] = (float)(q0[6 * D] * inv);
    for (int k = 0; k < N; ++k) o[4 + 6 * D + k] = k == n ? 1.f : 0.f;
  }
}

// ---------------------------------------------------------------- MLP kernels
// C[M x N] = act(A[M x K] * op(B) + bias): op(B) = B^T (B is N x K, a weight
// matrix W[out][in]).  16 x 16 output tiles, K in steps of 16 through shared memory.
constexpr int kT = 16;
__global__ void k_gemm_abt(const float *__restrict__ A, const float *__restrict__ B, const float *__restrict__ bias,
                           float *__restrict__ C, int M, int Nc, int K, int relu) {
  __shared__ float As[kT][kT + 1], Bs[kT][kT + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * kT + ty, col = blockIdx.x * kT + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += kT) {
    As[ty][tx] = (row < M && k0 + tx < K) ? A[(size_t)row * K + k0 + tx] : 0.f;
    const int bn = blockIdx.x * kT + ty;
    Bs[ty][tx] = (bn < Nc && k0 + tx < K) ? B[(size_t)bn * K + k0 + tx] : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kT; ++k) acc += As[ty][k] * Bs[tx][k];
    __syncthreads();
  }
  if (row < M && col < Nc) {
    if (bias) acc += bias[col];
    if (relu) acc = fmaxf(acc, 0.f);
    C[(size_t)row * Nc + col] = acc;
  }
}

// C[M x N] = (A[M x K] * B[K x N]) .* mask(Z > 0): activation gradients dH = dY W .* relu'
__global__ void k_gemm_ab_mask(const float *__restrict__ A, const float *__restrict__ B, const float *__restrict__ Z,
                               float *__restrict__ C, int M, int Nc, int K) {
  __shared__ float As[kT][kT + 1], Bs[kT][kT + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.y * kT + ty, col = blockIdx.x * kT + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += kT) {
    As[ty][tx] = (row < M && k0 + tx < K) ? A[(size_t)row * K + k0 + tx] : 0.f;
    Bs[ty][tx] = (k0 + ty < K && col < Nc) ? B[(size_t)(k0 + ty) * Nc + col] : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kT; ++k) acc += As[ty][k] * Bs[k][tx];
    __syncthreads();
  }
  if (row < M && col < Nc) C[(size_t)row * Nc + col] = Z[(size_t)row * Nc + col] > 0.f ? acc : 0.f;
}

// weight gradient G[M x N] = sum_b A[b][m] * B[b][n] over the batch, and the bias
// gradient gb[m] = sum_b A[b][m] (column block 0 computes it)
__global__ void k_gemm_atb(const float *__restrict__ A, const float *__restrict__ B, float *__restrict__ G,
                           float *__restrict__ gb, int Bn, int M, int Nc) {
  __shared__ float As[kT][kT + 1], Bs[kT][kT + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int m = blockIdx.y * kT + ty, n = blockIdx.x * kT + tx;
  float acc = 0.f, bacc = 0.f;
  for (int b0 = 0; b0 < Bn; b0 += kT) {
    // As[k][i] = A[b0 + k][mblock + i], Bs[k][j] = B[b0 + k][nblock + j]
    As[ty][tx] = (b0 + ty < Bn && blockIdx.y * kT + tx < M) ? A[(size_t)(b0 + ty) * M + blockIdx.y * kT + tx] : 0.f;
    Bs[ty][tx] = (b0 + ty < Bn && n < Nc) ? B[(size_t)(b0 + ty) * Nc + n] : 0.f;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kT; ++k) {
      acc += As[k][ty] * Bs[k][tx];
      bacc += As[k][ty];
    }
    __syncthreads();
  }
  if (m < M && n < Nc) G[(size_t)m * Nc + n] = acc;
  if (gb && blockIdx.x == 0 && tx == 0 && m < M) gb[m] = bacc;
}

// dY = 2 (Y - T) / (B J); loss partial sums of (Y - T)^2 / (B J) into *loss (FP64)
__global__ void k_loss_grad(const float *__restrict__ Y, const float *__restrict__ T, float *__restrict__ dY,
                            uint64_t n, float scale, double *__restrict__ loss) {
  double acc = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    dY[i] = 2.f * d * scale;
    acc += (double)d * (double)d * (double)scale;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m1,
                       float *__restrict__ m2, uint64_t n, float lr, float b1, float b2, float c1, float c2, float eps) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    w[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
  }
}

// standardise rows of F features: (f - mean) / std
__global__ void k_standardise(const float *__restrict__ in, float *__restrict__ out, uint64_t rows, int F,
                              const float *__restrict__ mean, const float *__restrict__ sd) {
  const uint64_t n = rows * F;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const int f = (int)(i % F);
    out[i] = (in[i] - mean[f]) / sd[f];
  }
}

// gather batch rows idx[] of the example set (standardised features, targets)
__global__ void k_gather_batch(const float *__restrict__ ef, const float *__restrict__ et, const uint64_t *__restrict__ idx,
                               int B, int F, int J, const float *__restrict__ mean, const float *__restrict__ sd,
                               float *__restrict__ bx, float *__restrict__ bt) {
  const int b = blockIdx.x;
  if (b >= B) return;
  const uint64_t r = idx[b];
  for (int k = threadIdx.x; k < F; k += blockDim.x) bx[(size_t)b * F + k] = (ef[r * F + k] - mean[k]) / sd[k];
  for (int k = threadIdx.x; k < J; k += blockDim.x) bt[(size_t)b * J + k] = et[r * J + k];
}

// SplitMix64: batch indices for step `step`
__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__global__ void k_batch_idx(uint64_t *__restrict__ idx, int B, uint64_t n, uint64_t seed, uint64_t step) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) idx[b] = splitmix(seed ^ (step * 0x100000001B3ull) ^ ((uint64_t)b << 40)) % n;
}

// predicted rows -> factor matrix (value_t, stride ldf); rows >= dims (padding) are 0
template <class V>
__global__ void k_put_rows(const float *__restrict__ y, uint64_t rows, uint64_t valid, int J, int ldf, V *__restrict__ fac) {
  const uint64_t n = rows * (uint64_t)ldf;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = i / ldf;
    const int c = (int)(i % ldf);
    fac[i] = (r < valid && c < J) ? (V)y[r * J + c] : V(0);
  }
}
// factor matrix (value_t, stride ldf) -> targets [rows][J] float
template <class V>
__global__ void k_get_rows(const V *__restrict__ fac, const uint32_t *__restrict__ pick, uint64_t n, int J, int ldf,
                           float *__restrict__ out) {
  const uint64_t tot = n * (uint64_t)J;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = i / J;
    out[i] = (float)fac[(size_t)pick[k] * ldf + (i % J)];
  }
}
__global__ void k_gather_feat(const float *__restrict__ f, const uint32_t *__restrict__ pick, uint64_t n, int F,
                              float *__restrict__ out) {
  const uint64_t tot = n * (uint64_t)F;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = f[(size_t)pick[i / F] * F + (i % F)];
}

unsigned grid_for(uint64_t n, int threads = kWsThreads) {
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + threads - 1) / threads, 152ull * 32));
}

// raw features of every row of mode n into d_feat (rows[n] x F)
int mode_features(gtk_tensor *t, int n, float *d_feat) {
  const int N = t->N, D = N - 1, F = ws_nfeat(N);
  (void)F;
  cudaStream_t s = t->stream;
  // per-mode row statistics (every mode: the co-indexed means need them all)
  std::vector<double *> bufs;
  auto alloc = [&](size_t n) -> double * {
    void *p = nullptr;
    if (malloc_retry(&p, std::max<size_t>(n, 1) * sizeof(double)) != cudaSuccess) return nullptr;
    bufs.push_back(static_cast<double *>(p));
    return static_cast<double *>(p);
  };
  auto release = [&]() {
    for (double *p : bufs) cudaFree(p);
  };
  std::vector<double *> cnt(N), s1(N), s2(N), mu(N), lc(N);
  for (int m = 0; m < N; ++m) {
    cnt[m] = alloc(t->rows[m]);
    s1[m] = alloc(t->rows[m]);
    s2[m] = alloc(t->rows[m]);
    mu[m] = alloc(t->rows[m]);
    lc[m] = alloc(t->rows[m]);
    if (!cnt[m] || !s1[m] || !s2[m] || !mu[m] || !lc[m]) {
      release();
      return fail(GTK_ERR_OOM, "warm-start feature buffers");
    }
  }
  double *acc = alloc(t->rows[n] * (size_t)(6 * std::max(1, D) + 1));
  if (!acc) {
    release();
    return fail(GTK_ERR_OOM, "warm-start feature buffers");
  }
  int rc = 0;
  for (int m = 0; m < N && !rc; ++m) {
    rc = ck(cudaMemsetAsync(cnt[m], 0, t->rows[m] * 8, s), "memset");
    if (!rc) rc = ck(cudaMemsetAsync(s1[m], 0, t->rows[m] * 8, s), "memset");
    if (!rc) rc = ck(cudaMemsetAsync(s2[m], 0, t->rows[m] * 8, s), "memset");
    if (rc || !t->nnz) continue;
    const unsigned g = (unsigned)((t->nnz + (uint64_t)kChunk * kWsThreads - 1) / ((uint64_t)kChunk * kWsThreads));
    if (t->dtype == GTK_F32)
      k_row_stats<float><<<g, kWsThreads, 0, s>>>(t->vidx[m][m], (const float *)t->vval[m], t->nnz, cnt[m], s1[m],
                                                 s2[m]);
    else
      k_row_stats<double><<<g, kWsThreads, 0, s>>>(t->vidx[m][m], (const double *)t->vval[m], t->nnz, cnt[m], s1[m],
                                                  s2[m]);
    rc = ck(cudaGetLastError(), "k_row_stats");
  }
  for (int m = 0; m < N && !rc; ++m) {
    k_row_mean<<<grid_for(t->rows[m]), kWsThreads, 0, s>>>(cnt[m], s1[m], mu[m], lc[m], t->rows[m]);
    rc = ck(cudaGetLastError(), "k_row_mean");
  }
  if (!rc) rc = ck(cudaMemsetAsync(acc, 0, t->rows[n] * (size_t)(6 * std::max(1, D) + 1) * 8, s), "memset");
  if (!rc && t->nnz && D > 0) {
    CoArgs a;
    memset(&a, 0, sizeof(a));
    a.row = t->vidx[n][n];
    a.val = t->vval[n];
    a.D = D;
    int d = 0;
    for (int m = 0; m < N; ++m) {
      if (m == n) continue;
      a.coord[d] = t->vidx[n][m];
      a.mu[d] = mu[m];
      a.lc[d] = lc[m];
      ++d;
    }
    const unsigned g = (unsigned)((t->nnz + (uint64_t)kChunk * kWsThreads - 1) / ((uint64_t)kChunk * kWsThreads));
    if (t->dtype == GTK_F32)
      k_coindex<float><<<g, kWsThreads, 0, s>>>(a, t->nnz, acc);
    else
      k_coindex<double><<<g, kWsThreads, 0, s>>>(a, t->nnz, acc);
    rc = ck(cudaGetLastError(), "k_coindex");
  }
  if (!rc) {
    k_features<<<grid_for(t->rows[n]), kWsThreads, 0, s>>>(cnt[n], s1[n], s2[n], acc, t->rows[n], N, n,
                                                           F, d_feat);
    rc = ck(cudaGetLastError(), "k_features");
  }
  if (!rc) rc = ck(cudaStreamSynchronize(s), "sync");
  release();
  return rc;
}

int ensure_batch(gtk_ws *m, int B) {
  if (B <= m->bcap) return 0;
  float **ps[] = {&m->bx, &m->bt, &m->h1, &m->h2, &m->y, &m->dy, &m->d2, &m->d1};
  for (float **p : ps)
    if (*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  const size_t sz[] = {(size_t)B * m->F, (size_t)B * m->J, (size_t)B * m->H, (size_t)B * m->H,
                       (size_t)B * m->J, (size_t)B * m->J, (size_t)B * m->H, (size_t)B * m->H};
  for (int i = 0; i < 8; ++i) GTK_CUDA(malloc_retry((void **)ps[i], sz[i] * sizeof(float)));
  m->bcap = B;
  return 0;
}

dim3 tiles(int rows, int cols) { return dim3((cols + kT - 1) / kT, (rows + kT - 1) / kT); }

// forward of B standardised rows in m->bx (or x) -> h1, h2, y
int forward(gtk_ws *m, const float *x, int B, float *y_out) {
  const WsParams p = params_of(m, m->w);
  const dim3 th(kT, kT);
  k_gemm_abt<<<tiles(B, m->H), th, 0, m->stream>>>(x, p.W1, p.b1, m->h1, B, m->H, m->F, 1);
  k_gemm_abt<<<tiles(B, m->H), th, 0, m->stream>>>(m->h1, p.W2, p.b2, m->h2, B, m->H, m->H, 1);
  k_gemm_abt<<<tiles(B, m->J), th, 0, m->stream>>>(m->h2, p.W3, p.b3, y_out, B, m->J, m->H, 0);
  return ck(cudaGetLastError(), "mlp forward");
}

// loss and gradient (into m->g) of the batch in m->bx / m->bt
int forward_backward(gtk_ws *m, int B) {
  if (int rc = forward(m, m->bx, B, m->y)) return rc;
  GTK_CUDA(cudaMemsetAsync(m->loss, 0, 8, m->stream));
  const uint64_t n = (uint64_t)B * m->J;
  k_loss_grad<<<grid_for(n), kWsThreads, 0, m->stream>>>(m->y, m->bt, m->dy, n, 1.f / (float)n, m->loss);
  const WsParams p = params_of(m, m->w);
  float *gW1 = m->g, *gb1 = gW1 + (size_t)m->H * m->F, *gW2 = gb1 + m->H, *gb2 = gW2 + (size_t)m->H * m->H,
        *gW3 = gb2 + m->H, *gb3 = gW3 + (size_t)m->J * m->H;
  const dim3 th(kT, kT);
  // layer 3: dW3 = dY^T H2, db3 = sum dY; dH2 = dY W3 .* (H2 > 0)
  k_gemm_atb<<<tiles(m->J, m->H), th, 0, m->stream>>>(m->dy, m->h2, gW3, gb3, B, m->J, m->H);
  k_gemm_ab_mask<<<tiles(B, m->H), th, 0, m->stream>>>(m->dy, p.W3, m->h2, m->d2, B, m->H, m->J);
  // layer 2
  k_gemm_atb<<<tiles(m->H, m->H), th, 0, m->stream>>>(m->d2, m->h1, gW2, gb2, B, m->H, m->H);
  k_gemm_ab_mask<<<tiles(B, m->H), th, 0, m->stream>>>(m->d2, p.W2, m->h1, m->d1, B, m->H, m->H);
  // layer 1
  k_gemm_atb<<<tiles(m->H, m->F), th, 0, m->stream>>>(m->d1, m->bx, gW1, gb1, B, m->H, m->F);
  return ck(cudaGetLastError(), "mlp backward");
}

}  // namespace

extern "C" {

int gtk_ws_create(int order, int rank, int hidden, uint64_t seed, int device, gtk_ws **out) {
  if (order < 2 || order > kMaxOrder || rank < 1 || rank > kMaxRank || hidden < 1 || hidden > 1024 || !out)
    return fail(GTK_ERR_ARG, "order 2..8, rank 1..64, hidden 1..1024");
  gtk_ws *m = new gtk_ws();
  m->dev = device;
  m->N = order;
  m->J = rank;
  m->H = hidden;
  m->F = ws_nfeat(order);
  m->np = ws_np(m->F, m->H, m->J);
  m->seed = seed;
  auto bail = [&](int rc) {
    gtk_ws_destroy(m);
    return rc;
  };
  if (int rc = ck(cudaSetDevice(device), "cudaSetDevice")) return bail(rc);
  if (int rc = ck(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "stream")) return bail(rc);
  float **ps[] = {&m->w, &m->g, &m->m1, &m->m2};
  for (float **p : ps)
    if (int rc = ck(malloc_retry((void **)p, m->np * sizeof(float)), "cudaMalloc")) return bail(rc);
  if (int rc = ck(malloc_retry((void **)&m->d_fmean, m->F * 4), "cudaMalloc")) return bail(rc);
  if (int rc = ck(malloc_retry((void **)&m->d_fstd, m->F * 4), "cudaMalloc")) return bail(rc);
  if (int rc = ck(malloc_retry((void **)&m->loss, 8), "cudaMalloc")) return bail(rc);
  // He-uniform weights, zero biases, from a seeded host generator
  std::vector<float> w(m->np, 0.f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto unif = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (float)((st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
  };
  size_t off = 0;
  const int fan[3][2] = {{m->F, m->H}, {m->H, m->H}, {m->H, m->J}};
  for (int l = 0; l < 3; ++l) {
    const int fin = fan[l][0], fout = fan[l][1];
    const float a = std::sqrt(6.f / (float)fin) * (l == 2 ? 0.5f : 1.f);
    for (size_t k = 0; k < (size_t)fin * fout; ++k) w[off + k] = a * unif();
    off += (size_t)fin * fout + fout;
  }
  m->fmean.assign(m->F, 0.f);
  m->fstd.assign(m->F, 1.f);
  int rc = ck(cudaMemcpy(m->w, w.data(), m->np * 4, cudaMemcpyHostToDevice), "H2D");
  if (!rc) rc = ck(cudaMemset(m->m1, 0, m->np * 4), "memset");
  if (!rc) rc = ck(cudaMemset(m->m2, 0, m->np * 4), "memset");
  if (!rc) rc = ck(cudaMemcpy(m->d_fmean, m->fmean.data(), m->F * 4, cudaMemcpyHostToDevice), "H2D");
  if (!rc) rc = ck(cudaMemcpy(m->d_fstd, m->fstd.data(), m->F * 4, cudaMemcpyHostToDevice), "H2D");
  if (rc) return bail(rc);
  *out = m;
  return 0;
}

void gtk_ws_destroy(gtk_ws *m) {
  if (!m) return;
  cudaSetDevice(m->dev);
  if (m->stream) cudaStreamSynchronize(m->stream);
  float *ps[] = {m->w, m->g, m->m1, m->m2, m->d_fmean, m->d_fstd, m->ex_f, m->ex_t, m->bx, m->bt,
                 m->h1, m->h2, m->y, m->dy, m->d2, m->d1};
  for (float *p : ps)
    if (p) cudaFree(p);
  if (m->loss) cudaFree(m->loss);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

// model file: "GTKWS001", u32 order, rank, hidden, features, u64 params, then the
// params, the feature means and standard deviations (float), then the FNV-1a 64
// checksum of everything before it
static const char kWsMagic[8] = {'G', 'T', 'K', 'W', 'S', '0', '0', '1'};
static uint64_t fnv1a(const unsigned char *p, size_t n, uint64_t h) {
  for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 1099511628211ull;
  return h;
}

int gtk_ws_save(const gtk_ws *m, const char *path) {
  if (!m || !path) return fail(GTK_ERR_ARG, "null argument");
  if (!m->have_norm) return fail(GTK_ERR_STATE, "the model is untrained");
  std::vector<unsigned char> buf;
  auto put = [&](const void *p, size_t n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    buf.insert(buf.end(), c, c + n);
  };
  const uint32_t hdr[4] = {(uint32_t)m->N, (uint32_t)m->J, (uint32_t)m->H, (uint32_t)m->F};
  const uint64_t np = m->np;
  put(kWsMagic, 8);
  put(hdr, sizeof(hdr));
  put(&np, 8);
  std::vector<float> w(m->np);
  GTK_CUDA(cudaSetDevice(m->dev));
  GTK_CUDA(cudaMemcpy(w.data(), m->w, m->np * 4, cudaMemcpyDeviceToHost));
  put(w.data(), w.size() * 4);
  put(m->fmean.data(), (size_t)m->F * 4);
  put(m->fstd.data(), (size_t)m->F * 4);
  const uint64_t h = fnv1a(buf.data(), buf.size(), 1469598103934665603ull);
  put(&h, 8);
  const std::string tmp = std::string(path) + ".tmp";
  FILE *f = fopen(tmp.c_str(), "wb");
  if (!f) return fail(GTK_ERR_IO, "cannot write " + tmp);
  const bool ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
  if (fclose(f) != 0 || !ok || rename(tmp.c_str(), path) != 0) return fail(GTK_ERR_IO, "cannot write " + std::string(path));
  return 0;
}

int gtk_ws_load(const char *path, int device, gtk_ws **out) {
  if (!path || !out) return fail(GTK_ERR_ARG, "null argument");
  FILE *f = fopen(path, "rb");
  if (!f) return fail(GTK_ERR_IO, "cannot open " + std::string(path));
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t n;
  while ((n = fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
  fclose(f);
  const size_t head = 8 + 16 + 8;
  if (buf.size() < head + 8 || memcmp(buf.data(), kWsMagic, 8) != 0) return fail(GTK_ERR_PARSE, "not a warm-start model");
  uint32_t hdr[4];
  uint64_t np = 0, h = 0;
  memcpy(hdr, buf.data() + 8, 16);
  memcpy(&np, buf.data() + 24, 8);
  const uint64_t F = hdr[3];
  if (hdr[0] < 2 || hdr[0] > kMaxOrder || hdr[1] < 1 || hdr[1] > kMaxRank || hdr[2] < 1 || hdr[2] > 1024 ||
      np > (1ull << 32) || F > 1024 || buf.size() != head + np * 4 + 2 * F * 4 + 8)
    return fail(GTK_ERR_PARSE, "damaged warm-start model");
  memcpy(&h, buf.data() + buf.size() - 8, 8);
  if (fnv1a(buf.data(), buf.size() - 8, 1469598103934665603ull) != h) return fail(GTK_ERR_PARSE, "checksum mismatch");
  gtk_ws *m = nullptr;
  if (int rc = gtk_ws_create((int)hdr[0], (int)hdr[1], (int)hdr[2], 0, device, &m)) return rc;
  if (m->np != np || (uint64_t)m->F != F) {
    gtk_ws_destroy(m);
    return fail(GTK_ERR_PARSE, "model layout does not match its order, rank and width");
  }
  const float *p = reinterpret_cast<const float *>(buf.data() + head);
  if (int rc = gtk_ws_set_params(m, p, p + np, p + np + F)) {
    gtk_ws_destroy(m);
    return rc;
  }
  *out = m;
  return 0;
}

int gtk_ws_info(const gtk_ws *m, int *features, uint64_t *params, uint64_t *examples) {
  if (!m) return fail(GTK_ERR_ARG, "null model");
  if (features) *features = m->F;
  if (params) *params = m->np;
  if (examples) *examples = m->ex_n;
  return 0;
}

int gtk_ws_get_params(const gtk_ws *m, float *params, float *feat_mean, float *feat_std) {
  if (!m) return fail(GTK_ERR_ARG, "null model");
  GTK_CUDA(cudaSetDevice(m->dev));
  if (params) GTK_CUDA(cudaMemcpy(params, m->w, m->np * 4, cudaMemcpyDeviceToHost));
  if (feat_mean) memcpy(feat_mean, m->fmean.data(), m->F * 4);
  if (feat_std) memcpy(feat_std, m->fstd.data(), m->F * 4);
  return 0;
}

int gtk_ws_set_params(gtk_ws *m, const float *params, const float *feat_mean, const float *feat_std) {
  if (!m) return fail(GTK_ERR_ARG, "null model");
  GTK_CUDA(cudaSetDevice(m->dev));
  if (params) GTK_CUDA(cudaMemcpy(m->w, params, m->np * 4, cudaMemcpyHostToDevice));
  if (feat_mean && feat_std) {
    for (int k = 0; k < m->F; ++k)
      if (!(feat_std[k] > 0.f)) return fail(GTK_ERR_ARG, "feature std must be > 0");
    memcpy(m->fmean.data(), feat_mean, m->F * 4);
    memcpy(m->fstd.data(), feat_std, m->F * 4);
    GTK_CUDA(cudaMemcpy(m->d_fmean, feat_mean, m->F * 4, cudaMemcpyHostToDevice));
    GTK_CUDA(cudaMemcpy(m->d_fstd, feat_std, m->F * 4, cudaMemcpyHostToDevice));
    m->have_norm = true;
  }
  return 0;
}

int gtk_ws_features(gtk_tensor *t, int mode, float *out) {
  if (!t || !out || mode < 0 || mode >= t->N) return fail(GTK_ERR_ARG, "bad argument");
  if (int rc = need_resident(*t, "the warm start")) return rc;
  if (t->N < 2) return fail(GTK_ERR_UNSUPPORTED, "warm start needs order >= 2");
  GTK_CUDA(cudaSetDevice(t->dev));
  const int F = ws_nfeat(t->N);
  float *d = nullptr;
  GTK_CUDA(malloc_retry(&d, std::max<size_t>(1, t->rows[mode] * F) * 4));
  int rc = mode_features(t, mode, d);
  if (!rc) rc = ck(cudaMemcpy(out, d, t->rows[mode] * F * 4, cudaMemcpyDeviceToHost), "D2H");
  cudaFree(d);
  return rc;
}

int gtk_ws_add_example(gtk_ws *m, gtk_tensor *t) {
  if (!m || !t) return fail(GTK_ERR_ARG, "null argument");
  if (int rc = need_resident(*t, "the warm start")) return rc;
  if (t->N != m->N || t->J != m->J) return fail(GTK_ERR_ARG, "model and tensor differ in order or rank");
  if (!t->have_factors) return fail(GTK_ERR_STATE, "the tensor has no factors to learn from");
  if (t->dev != m->dev) return fail(GTK_ERR_ARG, "model and tensor on different devices");
  GTK_CUDA(cudaSetDevice(m->dev));
  for (int n = 0; n < t->N; ++n) {
    // rows of mode n with at least one nonzero (the others carry no signal)
    const uint64_t rows = t->dims[n];
    std::vector<float> feat((size_t)t->rows[n] * m->F);
    float *d = nullptr;
    GTK_CUDA(malloc_retry(&d, std::max<size_t>(1, feat.size()) * 4));
    int rc = mode_features(t, n, d);
    if (!rc) rc = ck(cudaMemcpy(feat.data(), d, feat.size() * 4, cudaMemcpyDeviceToHost), "D2H");
    std::vector<uint32_t> pick;
    for (uint64_t r = 0; r < rows && !rc; ++r)
      if (feat[r * m->F] > 0.f) pick.push_back((uint32_t)r);
    const uint64_t k = pick.size();
    if (!rc && k) {
      if (m->ex_n + k > m->ex_cap) {  // grow the example arrays
        const uint64_t cap = std::max<uint64_t>(m->ex_n + k, m->ex_cap * 2);
        float *nf = nullptr, *nt = nullptr;
        rc = ck(malloc_retry(&nf, cap * m->F * 4), "cudaMalloc");
        if (!rc) rc = ck(malloc_retry(&nt, cap * m->J * 4), "cudaMalloc");
        if (!rc && m->ex_n) rc = ck(cudaMemcpy(nf, m->ex_f, m->ex_n * m->F * 4, cudaMemcpyDeviceToDevice), "D2D");
        if (!rc && m->ex_n) rc = ck(cudaMemcpy(nt, m->ex_t, m->ex_n * m->J * 4, cudaMemcpyDeviceToDevice), "D2D");
        if (rc) {
          if (nf) cudaFree(nf);
          if (nt) cudaFree(nt);
        } else {
          if (m->ex_f) cudaFree(m->ex_f);
          if (m->ex_t) cudaFree(m->ex_t);
          m->ex_f = nf;
          m->ex_t = nt;
          m->ex_cap = cap;
        }
      }
      uint32_t *dp = nullptr;
      if (!rc) rc = ck(malloc_retry(&dp, k * 4), "cudaMalloc");
      if (!rc) rc = ck(cudaMemcpy(dp, pick.data(), k * 4, cudaMemcpyHostToDevice), "H2D");
      if (!rc) {
        k_gather_feat<<<grid_for(k * m->F), kWsThreads, 0, m->stream>>>(d, dp, k, m->F, m->ex_f + m->ex_n * m->F);
        if (t->dtype == GTK_F32)
          k_get_rows<float><<<grid_for(k * m->J), kWsThreads, 0, m->stream>>>((const float *)t->fac[n], dp, k, m->J,
                                                                             t->ldf, m->ex_t + m->ex_n * m->J);
        else
          k_get_rows<double><<<grid_for(k * m->J), kWsThreads, 0, m->stream>>>((const double *)t->fac[n], dp, k,
                                                                              m->J, t->ldf, m->ex_t + m->ex_n * m->J);
        rc = ck(cudaGetLastError(), "gather examples");
      }
      if (!rc) rc = ck(cudaStreamSynchronize(m->stream), "sync");
      if (dp) cudaFree(dp);
      if (!rc) m->ex_n += k;
    }
    cudaFree(d);
    if (rc) return rc;
  }
  return 0;
}

int gtk_ws_loss_grad(gtk_ws *m, const float *x, const float *target, int B, double *loss, float *grad) {
  if (!m || !x || !target || B < 1) return fail(GTK_ERR_ARG, "bad argument");
  GTK_CUDA(cudaSetDevice(m->dev));
  if (int rc = ensure_batch(m, B)) return rc;
  GTK_CUDA(cudaMemcpyAsync(m->bx, x, (size_t)B * m->F * 4, cudaMemcpyHostToDevice, m->stream));
  GTK_CUDA(cudaMemcpyAsync(m->bt, target, (size_t)B * m->J * 4, cudaMemcpyHostToDevice, m->stream));
  if (int rc = forward_backward(m, B)) return rc;
  double l = 0;
  GTK_CUDA(cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->stream));
  if (grad) GTK_CUDA(cudaMemcpyAsync(grad, m->g, m->np * 4, cudaMemcpyDeviceToHost, m->stream));
  GTK_CUDA(cudaStreamSynchronize(m->stream));
  if (loss) *loss = l;
  return 0;
}

int gtk_ws_predict(gtk_ws *m, const float *x, int B, float *y) {
  if (!m || !x || !y || B < 1) return fail(GTK_ERR_ARG, "bad argument");
  GTK_CUDA(cudaSetDevice(m->dev));
  if (int rc = ensure_batch(m, B)) return rc;
  GTK_CUDA(cudaMemcpyAsync(m->bx, x, (size_t)B * m->F * 4, cudaMemcpyHostToDevice, m->stream));
  if (int rc = forward(m, m->bx, B, m->y)) return rc;
  GTK_CUDA(cudaMemcpyAsync(y, m->y, (size_t)B * m->J * 4, cudaMemcpyDeviceToHost, m->stream));
  GTK_CUDA(cudaStreamSynchronize(m->stream));
  return 0;
}

int gtk_ws_train(gtk_ws *m, int steps, int batch, float lr, double *final_loss) {
  NvtxRange nvtx("gtk_ws_train");
  if (!m || steps < 0 || batch < 1) return fail(GTK_ERR_ARG, "bad argument");
  if (!m->ex_n) return fail(GTK_ERR_STATE, "no training examples (gtk_ws_add_example)");
  GTK_CUDA(cudaSetDevice(m->dev));
  if (!m->have_norm) {  // standardisation from the examples (host pass over a copy)
    std::vector<float> f(m->ex_n * m->F);
    GTK_CUDA(cudaMemcpy(f.data(), m->ex_f, f.size() * 4, cudaMemcpyDeviceToHost));
    for (int k = 0; k < m->F; ++k) {
      double s = 0, q = 0;
      for (uint64_t r = 0; r < m->ex_n; ++r) {
        const double v = f[r * m->F + k];
        s += v;
        q += v * v;
      }
      const double mean = s / (double)m->ex_n;
      const double var = std::max(0.0, q / (double)m->ex_n - mean * mean);
      m->fmean[k] = (float)mean;
      m->fstd[k] = var > 1e-12 ? (float)std::sqrt(var) : 1.f;
    }
    GTK_CUDA(cudaMemcpy(m->d_fmean, m->fmean.data(), m->F * 4, cudaMemcpyHostToDevice));
    GTK_CUDA(cudaMemcpy(m->d_fstd, m->fstd.data(), m->F * 4, cudaMemcpyHostToDevice));
    m->have_norm = true;
  }
  if (int rc = ensure_batch(m, batch)) return rc;
  uint64_t *idx = nullptr;
  GTK_CUDA(malloc_retry(&idx, (size_t)batch * 8));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  int rc = 0;
  double l = 0;
  for (int s = 0; s < steps && !rc; ++s) {
    k_batch_idx<<<(batch + 255) / 256, 256, 0, m->stream>>>(idx, batch, m->ex_n, m->seed, m->adam_t);
    k_gather_batch<<<batch, 32, 0, m->stream>>>(m->ex_f, m->ex_t, idx, batch, m->F, m->J, m->d_fmean, m->d_fstd,
                                               m->bx, m->bt);
    rc = ck(cudaGetLastError(), "batch gather");
    if (!rc) rc = forward_backward(m, batch);
    if (rc) break;
    ++m->adam_t;
    const float c1 = 1.f - std::pow(b1, (float)m->adam_t), c2 = 1.f - std::pow(b2, (float)m->adam_t);
    k_adam<<<grid_for(m->np), kWsThreads, 0, m->stream>>>(m->w, m->g, m->m1, m->m2, m->np, lr, b1, b2, c1, c2, eps);
    rc = ck(cudaGetLastError(), "adam");
  }
  if (!rc) rc = ck(cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->stream), "D2H");
  if (!rc) rc = ck(cudaStreamSynchronize(m->stream), "sync");
  cudaFree(idx);
  if (!rc && final_loss) *final_loss = l;
  return rc;
}

int gtk_ws_apply(gtk_ws *m, gtk_tensor *t) {
  if (!m || !t) return fail(GTK_ERR_ARG, "null argument");
  if (int rc = need_resident(*t, "the warm start")) return rc;
  if (t->N != m->N || t->J != m->J) return fail(GTK_ERR_ARG, "model and tensor differ in order or rank");
  if (t->dev != m->dev) return fail(GTK_ERR_ARG, "model and tensor on different devices");
  if (!t->have_core) return fail(GTK_ERR_STATE, "initialise the core first (gtk_init_random or gtk_set_core)");
  if (!m->have_norm) return fail(GTK_ERR_STATE, "the model is untrained");
  GTK_CUDA(cudaSetDevice(m->dev));
  for (int n = 0; n < t->N; ++n) {
    const uint64_t rows = t->rows[n];
    float *d = nullptr, *z = nullptr, *y = nullptr;
    int rc = ck(malloc_retry(&d, std::max<uint64_t>(1, rows) * m->F * 4), "cudaMalloc");
    if (!rc) rc = ck(malloc_retry(&z, std::max<uint64_t>(1, rows) * m->F * 4), "cudaMalloc");
    if (!rc) rc = ck(malloc_retry(&y, std::max<uint64_t>(1, rows) * m->J * 4), "cudaMalloc");
    if (!rc) rc = mode_features(t, n, d);
    if (!rc) {
      k_standardise<<<grid_for(rows * m->F), kWsThreads, 0, t->stream>>>(d, z, rows, m->F, m->d_fmean, m->d_fstd);
      rc = ck(cudaGetLastError(), "standardise");
    }
    // inference in chunks through the batch scratch of the model
    const int chunk = 65536;
    if (!rc) rc = ensure_batch(m, chunk);
    if (!rc) rc = ck(cudaStreamSynchronize(t->stream), "sync");
    for (uint64_t r0 = 0; r0 < rows && !rc; r0 += chunk) {
      const int B = (int)std::min<uint64_t>(chunk, rows - r0);
      rc = forward(m, z + r0 * m->F, B, y + r0 * m->J);
    }
    if (!rc) rc = ck(cudaStreamSynchronize(m->stream), "sync");
    if (!rc) {
      if (t->dtype == GTK_F32)
        k_put_rows<float><<<grid_for(rows * t->ldf), kWsThreads, 0, t->stream>>>(y, rows, t->dims[n], m->J, t->ldf,
                                                                               (float *)t->fac[n]);
      else
        k_put_rows<double><<<grid_for(rows * t->ldf), kWsThreads, 0, t->stream>>>(y, rows, t->dims[n], m->J, t->ldf,
                                                                                (double *)t->fac[n]);
      rc = ck(cudaGetLastError(), "put rows");
    }
    if (!rc) rc = ck(cudaStreamSynchronize(t->stream), "sync");
    if (d) cudaFree(d);
    if (z) cudaFree(z);
    if (y) cudaFree(y);
    if (rc) return rc;
  }
  t->have_factors = true;
  fit_invalidate(*t);
  return 0;
}

}  // extern "C"
