// core_update.cu -- optional update of the core tensor G.  GPUTucker keeps G at
// its initial values (the ALS of tucker.cuh:166-187 updates factors only), so this
// is an extension, off unless called, and it changes results.
//
// With the factors fixed, G minimises
//   sum_t (x_t - <G, phi_t>)^2 + lambda ||G||^2,   phi_t = a_0[i_0] (x) ... (x) a_{N-1}[i_{N-1}],
// whose normal equations (Phi^T Phi + lambda I) vec(G) = Phi^T x are solved by
// conjugate gradients from the current core (G in linear order, mode N-1 fastest).
// Per CG step one product with Phi^T Phi:
//   * Phi v: the delta kernels of the last mode with v as the core (plain FP32 /
//     FP64 form), then x_hat_t = delta_t . a_{N-1}[i_{N-1}] (k_core_y);
//   * Phi^T y = sum_t y_t phi_t (k_core_grad): the modes split into a left group
//     0..N1-1 and a right group N1..N-1, phi_t = l_t (x) r_t, so the sum is the
//     outer product accumulation sum_t (y_t l_t) r_t^T of a (J^N1) x (J^(N-N1))
//     matrix.  Per CTA a tile of nonzeros' l and r rows is built in shared memory;
//     each thread owns an 8 x 8 block of the output, accumulates in value_t over
//     kFlushEvery nonzeros, then adds into FP64 with atomics.
// The CG vectors (J^N <= 65536 entries) stay on the host in FP64.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "blocks.cuh"
#include "internal.h"

namespace gtk {
namespace {

constexpr int kGradThreads = 256;
constexpr int kBlk = 8;  // output block per thread: kBlk x kBlk
constexpr int kFlushEvery = 1024;  // nonzeros per value_t partial sum before the FP64 flush
constexpr uint64_t kCoreUpdateMaxCore = 65536;

struct ModePtrs {
  const uint32_t *idx[kMaxOrder];  // block-local coordinates
  const void *fac[kMaxOrder];
  uint32_t bd[kMaxOrder], P[kMaxOrder];
  uint64_t stride[kMaxOrder];      // block id = sum_k c_k * stride[k], last mode fastest
};


__device__ __forceinline__ uint32_t global_row(const ModePtrs &m, int k, uint32_t b, uint64_t t) {
  const uint32_t c = (uint32_t)((b / m.stride[k]) % m.P[k]);
  return c * m.bd[k] + m.idx[k][t];
}

// y_t = delta_t . a_{N-1}[i_{N-1}(t)], block-major order
template <class V>
__global__ void k_core_y(const V *__restrict__ delta, ModePtrs m, const uint64_t *__restrict__ blk_ptr, uint32_t nblk,
                         int N, int J, int ldf, uint64_t nnz, V *__restrict__ y) {
  const V *fac = reinterpret_cast<const V *>(m.fac[N - 1]);
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnz; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t b = block_of(blk_ptr, nblk, t);
    const V *a = fac + (uint64_t)global_row(m, N - 1, b, t) * ldf;
    const V *d = delta + t * (uint64_t)J;
    V s = V(0);
    for (int j = 0; j < J; ++j) s += d[j] * a[j];
    y[t] = s;
  }
}

// out[l * SR + r] += sum_t w_t l_t[l] r_t[r] over the nonzeros [t_begin, t_end) of
// this CTA's range; blockIdx.x = range * nchunks + chunk, chunk = which 256 of the
// (SLp/8) x (SRp/8) output blocks of kBlk x kBlk this CTA's threads own
template <class V>
__global__ void __launch_bounds__(kGradThreads) k_core_grad(const V *__restrict__ w, ModePtrs m,
                                                            const uint64_t *__restrict__ blk_ptr, uint32_t nblk, int N,
                                                            int J, int ldf, uint64_t nnz, int N1, int SL, int SR,
                                                            int nbl, int nbr, int nchunks, uint64_t per,
                                                            double *__restrict__ out) {
  constexpr int TN = sizeof(V) == 4 ? 32 : 16;  // nonzeros per tile
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int SLp = nbl * kBlk, SRp = nbr * kBlk;
  V *PL = reinterpret_cast<V *>(smem_raw);      // [TN][SLp]
  V *PR = PL + (size_t)TN * SLp;                // [TN][SRp]
  uint32_t *rows = reinterpret_cast<uint32_t *>(PR + (size_t)TN * SRp);  // [TN][N]
  V *wt = reinterpret_cast<V *>(rows + TN * kMaxOrder + 4);  // [TN] (8-byte aligned)
  const int tid = threadIdx.x;
  const int chunk = blockIdx.x % nchunks;
  const uint64_t range = blockIdx.x / nchunks;
  const uint64_t t_begin = range * per, t_end = min(nnz, t_begin + per);
  const int bi = chunk * kGradThreads + tid;  // this thread's output block
  const bool active = bi < nbl * nbr;
  const int l0 = active ? (bi / nbr) * kBlk : 0, r0 = active ? (bi % nbr) * kBlk : 0;
  V acc[kBlk][kBlk];
#pragma unroll
  for (int i = 0; i < kBlk; ++i)
#pragma unroll
    for (int j = 0; j < kBlk; ++j) acc[i][j] = V(0);
  auto flush = [&]() {
    if (!active) return;
#pragma unroll
    for (int i = 0; i < kBlk; ++i)
#pragma unroll
      for (int j = 0; j < kBlk; ++j) {
        if (l0 + i < SL && r0 + j < SR && acc[i][j] != V(0))
          atomicAdd(out + (size_t)(l0 + i) * SR + (r0 + j), (double)acc[i][j]);
        acc[i][j] = V(0);
      }
  };
  int since_flush = 0;
  for (uint64_t base = t_begin; base < t_end; base += TN) {
    const int nt = (int)min((uint64_t)TN, t_end - base);
    if (tid < TN) {
      const uint64_t t = base + tid;
      if (tid < nt) {
        const uint32_t b = block_of(blk_ptr, nblk, t);
        for (int k = 0; k < N; ++k) rows[tid * kMaxOrder + k] = global_row(m, k, b, t);
        wt[tid] = w[t];
      } else {
        for (int k = 0; k < N; ++k) rows[tid * kMaxOrder + k] = 0;
        wt[tid] = V(0);
      }
    }
    __syncthreads();
    // l rows (weighted) and r rows of the tile: digits of l over modes 0..N1-1 and of
    // r over modes N1..N-1, the last mode of each group fastest
    for (int e = tid; e < TN * SLp; e += kGradThreads) {
      const int tt = e / SLp, l = e % SLp;
      V v = V(0);
      if (l < SL) {
        v = wt[tt];
        int rem = l;
        for (int k = N1 - 1; k >= 0; --k) {
          const int d = rem % J;
          rem /= J;
          v *= reinterpret_cast<const V *>(m.fac[k])[(uint64_t)rows[tt * kMaxOrder + k] * ldf + d];
        }
      }
      PL[e] = v;
    }
    for (int e = tid; e < TN * SRp; e += kGradThreads) {
      const int tt = e / SRp, r = e % SRp;
      V v = V(0);
      if (r < SR) {
        v = V(1);
        int rem = r;
        for (int k = N - 1; k >= N1; --k) {
          const int d = rem % J;
          rem /= J;
          v *= reinterpret_cast<const V *>(m.fac[k])[(uint64_t)rows[tt * kMaxOrder + k] * ldf + d];
        }
      }
      PR[e] = v;
    }
    __syncthreads();
    if (active) {
      for (int tt = 0; tt < nt; ++tt) {
        V lv[kBlk], rv[kBlk];
#pragma unroll
        for (int i = 0; i < kBlk; ++i) lv[i] = PL[tt * SLp + l0 + i];
#pragma unroll
        for (int j = 0; j < kBlk; ++j) rv[j] = PR[tt * SRp + r0 + j];
#pragma unroll
        for (int i = 0; i < kBlk; ++i)
#pragma unroll
          for (int j = 0; j < kBlk; ++j) acc[i][j] += lv[i] * rv[j];
      }
    }
    since_flush += nt;
    if (since_flush >= kFlushEvery) {
      flush();
      since_flush = 0;
    }
    __syncthreads();  // the next tile overwrites the rows
  }
  flush();
}

struct CoreScratch {
  void *delta = nullptr, *y = nullptr;
  double *acc = nullptr;
  ~CoreScratch() {
    if (delta) cudaFree(delta);
    if (y) cudaFree(y);
    if (acc) cudaFree(acc);
  }
};

template <class V> int update_core_impl(DevTensor &t, int iters, int *iters_run, double *rel_residual) {
  const int N = t.N, J = t.J;
  const uint64_t M = t.core_n, nnz = t.nnz;
  ModePtrs m;
  memset(&m, 0, sizeof(m));
  uint64_t stride = 1;
  for (int k = N - 1; k >= 0; --k) {
    m.idx[k] = t.blk_idx[k];
    m.fac[k] = t.fac[k];
    m.bd[k] = t.bd[k];
    m.P[k] = t.P[k];
    m.stride[k] = stride;
    stride *= t.P[k];
  }
  const int N1 = N / 2;
  int SL = 1, SR = 1;
  for (int k = 0; k < N1; ++k) SL *= J;
  for (int k = N1; k < N; ++k) SR *= J;
  const int nbl = (SL + kBlk - 1) / kBlk, nbr = (SR + kBlk - 1) / kBlk;
  const int nchunks = (nbl * nbr + kGradThreads - 1) / kGradThreads;
  constexpr int TN = sizeof(V) == 4 ? 32 : 16;
  const size_t smem =
      ((size_t)TN * (nbl + nbr) * kBlk * sizeof(V) + TN * kMaxOrder * 4 + 16 + TN * sizeof(V) + 15) / 16 * 16;
  if (smem > 200 * 1024) return fail(GTK_ERR_UNSUPPORTED, "core update: the core's factor groups are too wide");
  GTK_CUDA(cudaFuncSetAttribute((const void *)k_core_grad<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const uint64_t target = (uint64_t)t.num_sms * 4;
  const uint64_t nranges = std::max<uint64_t>(1, std::min<uint64_t>((nnz + 255) / 256, (target + nchunks - 1) / nchunks));
  const uint64_t per = (nnz + nranges - 1) / nranges;
  const unsigned grid = (unsigned)(nranges * nchunks);

  CoreScratch sc;
  GTK_CUDA(malloc_retry(&sc.delta, nnz * (size_t)J * sizeof(V)));
  GTK_CUDA(malloc_retry(&sc.y, nnz * sizeof(V)));
  GTK_CUDA(malloc_retry((void **)&sc.acc, M * sizeof(double)));
  std::vector<double> hacc(M);
  // Phi^T w for device weights w (block-major order)
  auto phi_t = [&](const V *w, std::vector<double> &res) -> int {
    GTK_CUDA(cudaMemsetAsync(sc.acc, 0, M * sizeof(double), t.stream));
    k_core_grad<V><<<grid, kGradThreads, smem, t.stream>>>(w, m, t.blk_ptr, (uint32_t)t.nblk, N, J, t.ldf, nnz, N1, SL,
                                                         SR, nbl, nbr, nchunks, per, sc.acc);
    GTK_CUDA(cudaGetLastError());
    GTK_CUDA(cudaMemcpyAsync(res.data(), sc.acc, M * sizeof(double), cudaMemcpyDeviceToHost, t.stream));
    GTK_CUDA(cudaStreamSynchronize(t.stream));
    return 0;
  };
  std::vector<V> hv(M);
  // res = (Phi^T Phi + lambda I) v; the handle's core holds v afterwards
  auto apply = [&](const std::vector<double> &v, std::vector<double> &res) -> int {
    for (uint64_t i = 0; i < M; ++i) hv[i] = (V)v[i];
    if (int rc = put_core(t, hv.data())) return rc;
    if (int rc = run_delta(t, N - 1, sc.delta)) return rc;
    const unsigned g = (unsigned)std::min<uint64_t>((nnz + 255) / 256, (uint64_t)t.num_sms * 16);
    k_core_y<V><<<g, 256, 0, t.stream>>>((const V *)sc.delta, m, t.blk_ptr, (uint32_t)t.nblk, N, J, t.ldf, nnz,
                                         (V *)sc.y);
    GTK_CUDA(cudaGetLastError());
    if (int rc = phi_t((const V *)sc.y, res)) return rc;
    for (uint64_t i = 0; i < M; ++i) res[i] += kLambda * v[i];
    return 0;
  };
  // the plain delta kernels (FP32 / FP64 SIMT) for Phi v, whatever form the sweep uses
  const int prec = t.precision, var = t.variant;
  t.precision = GTK_PREC_PLAIN;
  if (t.variant == kVarTc) t.variant = kVarAuto;
  auto restore = [&]() {
    t.precision = prec;
    t.variant = var;
  };
  std::vector<double> g(M), b(M), r(M), p(M), ap(M);
  std::vector<V> core0(M);  // put back if a step fails
  if (cudaMemcpyAsync(core0.data(), t.core, M * sizeof(V), cudaMemcpyDeviceToHost, t.stream) != cudaSuccess ||
      cudaStreamSynchronize(t.stream) != cudaSuccess) {
    restore();
    return cuda_fail(cudaGetLastError(), "core read-back");
  }
  for (uint64_t i = 0; i < M; ++i) g[i] = (double)core0[i];
  int rc = phi_t((const V *)t.blk_val, b);
  if (!rc) rc = apply(g, ap);
  int k = 0;
  double bn = 0, rs = 0;
  if (!rc) {
    for (uint64_t i = 0; i < M; ++i) {
      r[i] = b[i] - ap[i];
      p[i] = r[i];
      rs += r[i] * r[i];
      bn += b[i] * b[i];
    }
    for (; k < iters && rs > 1e-28 * bn; ++k) {
      if ((rc = apply(p, ap))) break;
      double pap = 0;
      for (uint64_t i = 0; i < M; ++i) pap += p[i] * ap[i];
      if (!(pap > 0)) break;
      const double alpha = rs / pap;
      double rs1 = 0;
      for (uint64_t i = 0; i < M; ++i) {
        g[i] += alpha * p[i];
        r[i] -= alpha * ap[i];
        rs1 += r[i] * r[i];
      }
      const double beta = rs1 / rs;
      rs = rs1;
      for (uint64_t i = 0; i < M; ++i) p[i] = r[i] + beta * p[i];
    }
  }
  restore();
  if (!rc) {
    for (uint64_t i = 0; i < M; ++i) hv[i] = (V)g[i];
    rc = put_core(t, hv.data());  // the solution (the precision form's images rebuilt as well)
  } else {
    put_core(t, core0.data());  // the core the call started from
  }
  if (iters_run) *iters_run = k;
  if (rel_residual) *rel_residual = bn > 0 ? std::sqrt(rs / bn) : 0.0;
  return rc;
}

}  // namespace

int run_update_core(DevTensor &t, int iters, int *iters_run, double *rel_residual) {
  NvtxRange nvtx("gtk_update_core");
  if (t.core_n > kCoreUpdateMaxCore)
    return fail(GTK_ERR_UNSUPPORTED, "core update: at most 65536 core entries (rank^order)");
  if (!t.nnz) return fail(GTK_ERR_STATE, "core update of an empty tensor");
  return t.dtype == GTK_F32 ? update_core_impl<float>(t, iters, iters_run, rel_residual)
                            : update_core_impl<double>(t, iters, iters_run, rel_residual);
}

}  // namespace gtk
