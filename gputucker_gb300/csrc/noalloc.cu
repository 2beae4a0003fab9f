// noalloc.cu -- the reconstruction error of caller-owned device data, without
// allocating anything.
//
// Who needs it: code that cannot call cudaMalloc where it runs --
// latency-critical loops that must not touch the allocator (cudaMalloc and
// cudaFree synchronise the device and cost milliseconds), and hosts whose device
// memory belongs to another runtime's pool or is capped by it.  They hand in
// device pointers to their own tensor, factors and core and get the sum of
// squared errors back in device memory.
//
// The kernel is the generic reconstruction kernel of sweep.cu (x_hat =
// delta . a[i] with delta the staged contraction of the core with the other
// modes' factor rows) reading the caller's arrays; its scratch -- the per-CTA
// error sums and the core with rows padded for float4 loads -- lives in one
// file-scope device array instead of handle allocations:
//   kNaCtas doubles of partial sums + kNaCoreFloats floats of padded core
//   (8 KB + 4 MB; every GPU that loads the library holds it until exit).
// A core whose padded size exceeds kNaCoreFloats is rejected with
// GTK_ERR_UNSUPPORTED.
//
// The array is shared by every call in the process: two calls whose kernels
// overlap on the GPU (different streams, or different host threads) race on it
// and must be serialised by the caller.  Each call overwrites every scratch
// entry it reads (the partial sums of all its CTAs, the padded core) before
// reading it, so nothing carries over from one call to the next.
//
// Host code cannot use the array's name as a device address; the first call on
// each device looks the address up with cudaGetSymbolAddress (with that device
// current) and caches it.  Make that first call before any stream capture
// starts: the lookup may load the module, which a capturing stream forbids.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"

namespace gtk {
namespace {

constexpr int kNaCtas = 1024;
constexpr int kNaThreads = 256;
constexpr size_t kNaCoreFloats = (size_t)1 << 20;
constexpr size_t kNaScratchBytes = kNaCtas * sizeof(double) + kNaCoreFloats * sizeof(float);

static __device__ __align__(256) unsigned char g_na_scratch[kNaScratchBytes];

struct NaArgs {
  const uint32_t *idx[kMaxOrder];
  const float *fac[kMaxOrder];  // rows x J, row-major, no padding
  const float *val;
  uint64_t nnz;
  int N, J, ldg;                // ldg: padded core row length (multiple of 4)
};

// the caller's core (J^N, last mode fastest) as rows of J padded to ldg
__global__ void k_na_core(const float *__restrict__ core, uint64_t rows, int J, int ldg, float *__restrict__ out) {
  const uint64_t n = rows * (uint64_t)ldg;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = k / ldg, c = k % ldg;
    out[k] = c < (uint64_t)J ? core[r * J + c] : 0.f;
  }
}

// x_hat_t = sum_{j0} delta_t[j0] * A_0[i_0, j0], delta over modes 1..N-1 (mode 0 is
// the core's first index, so the linear core is already mode-0-first)
__global__ void __launch_bounds__(kNaThreads) k_na_fit(NaArgs a, const float *__restrict__ gp,
                                                       double *__restrict__ partial) {
  const int J = a.J, M = a.N - 1;
  uint64_t rows_per = 1;
  for (int k = 0; k < M - 1; ++k) rows_per *= (uint64_t)J;
  double err = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.nnz;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const float *ap[kMaxOrder];
    for (int k = 0; k < a.N; ++k) ap[k] = a.fac[k] + (size_t)a.idx[k][t] * J;
    float xhat = 0.f;
    for (int j0 = 0; j0 < J; ++j0) {
      float acc = 0.f;
      if (M == 0) {
        acc = gp[j0];
      } else {
        int dig[kMaxOrder];
        for (int k = 0; k < M; ++k) dig[k] = 0;
        const float *alast = ap[M];
        for (uint64_t r = 0; r < rows_per; ++r) {
          float pp = 1.f;
          for (int k = 0; k < M - 1; ++k) pp *= ap[k + 1][dig[k]];
          const float *grow = gp + ((size_t)j0 * rows_per + r) * a.ldg;
          float dot = 0.f;
          for (int c = 0; c < J; ++c) dot += grow[c] * alast[c];
          acc += pp * dot;
          for (int k = M - 2; k >= 0; --k) {
            if (++dig[k] < J) break;
            dig[k] = 0;
          }
        }
      }
      xhat += acc * ap[0][j0];
    }
    const float d = a.val[t] - xhat;
    err += (double)d * (double)d;
  }
  __shared__ double sw[kNaThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) err += __shfl_down_sync(0xFFFFFFFFu, err, o);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = err;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int w = 0; w < kNaThreads / 32; ++w) s += sw[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void k_na_sum(const double *__restrict__ partial, int m, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += partial[i];
    *out = s;
  }
}

std::mutex g_na_mutex;
void *g_na_addr[256] = {};

// once per device, with that device current: the scratch array's device address
int na_scratch(int dev, unsigned char **out) {
  if (dev < 0 || dev >= 256) return fail(GTK_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
    g_na_addr[dev] = p;
  }
  *out = static_cast<unsigned char *>(g_na_addr[dev]);
  return 0;
}

}  // namespace
}  // namespace gtk

using namespace gtk;

extern "C" int gtk_reconstruction_error_noalloc(int order, int rank, uint64_t nnz, const uint32_t *const *d_idx,
                                                const float *d_vals, const float *const *d_factors,
                                                const float *d_core, double *d_err, void *stream) {
  if (order < 1 || order > GTK_MAX_ORDER) return fail(GTK_ERR_ARG, "order must be 1..8");
  if (rank < 1 || rank > GTK_MAX_RANK) return fail(GTK_ERR_ARG, "rank must be 1..64");
  if (!d_core || !d_err || (nnz && (!d_idx || !d_vals || !d_factors)))
    return fail(GTK_ERR_ARG, "null argument");
  for (int n = 0; nnz && n < order; ++n)
    if (!d_idx[n] || !d_factors[n]) return fail(GTK_ERR_ARG, "null coordinate or factor array");
  uint64_t rows = 1;  // J^(N-1) rows of J in the core
  for (int n = 0; n < order - 1; ++n) rows *= (uint64_t)rank;
  const int ldg = (rank + 3) / 4 * 4;
  if (rows * (uint64_t)ldg > kNaCoreFloats)
    return fail(GTK_ERR_UNSUPPORTED, "core too large for the no-allocation scratch: rank^(order-1) * " +
                                         std::to_string(ldg) + " = " + std::to_string(rows * ldg) +
                                         " floats > " + std::to_string(kNaCoreFloats));
  int dev = 0;
  GTK_CUDA(cudaGetDevice(&dev));
  unsigned char *scratch = nullptr;
  if (int rc = na_scratch(dev, &scratch)) return rc;
  double *partial = reinterpret_cast<double *>(scratch);
  float *gp = reinterpret_cast<float *>(scratch + kNaCtas * sizeof(double));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_na_core<<<256, 256, 0, s>>>(d_core, rows, rank, ldg, gp);
  GTK_CUDA(cudaGetLastError());
  NaArgs a;
  memset(&a, 0, sizeof(a));
  for (int n = 0; n < order; ++n) {
    a.idx[n] = nnz ? d_idx[n] : nullptr;
    a.fac[n] = nnz ? d_factors[n] : nullptr;
  }
  a.val = d_vals;
  a.nnz = nnz;
  a.N = order;
  a.J = rank;
  a.ldg = ldg;
  uint64_t grid = (nnz + kNaThreads - 1) / kNaThreads;
  if (grid > (uint64_t)kNaCtas) grid = kNaCtas;
  if (grid < 1) grid = 1;
  k_na_fit<<<(unsigned)grid, kNaThreads, 0, s>>>(a, gp, partial);
  GTK_CUDA(cudaGetLastError());
  k_na_sum<<<1, 32, 0, s>>>(partial, (int)grid, d_err);
  GTK_CUDA(cudaGetLastError());
  return 0;
}
