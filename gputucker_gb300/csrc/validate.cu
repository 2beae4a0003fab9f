// validate.cu -- device-side consistency checks of a handle's persistent arrays
// (gtk_validate).  compute-sanitizer is not available everywhere this library
// runs; these checks read every index array once and count violations instead of
// trapping, so a damaged or mis-built handle is reported, not run.  Checks (the
// order of the counters):
//   0 block-local coordinate >= block_dims[n]          (blk_idx)
//   1 view coordinate >= dims[k]                       (vidx)
//   2 view not sorted by its mode's row                (vidx[m][m])
//   3 view permutation entry >= nnz                    (vperm)
//   4 where_nnz entry >= its block's size              (where)
//   5 count_nnz row pointer decreasing, not starting at 0 or not ending at the
//     block's size                                     (count)
//   6 non-finite factor or core entry                  (fac, core)
//   7 block pointers decreasing or not ending at nnz   (blk_ptr)

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "blocks.cuh"
#include "internal.h"

namespace gtk {
namespace {

constexpr int kChecks = GTK_VALIDATE_CHECKS;

__device__ __forceinline__ void bump(unsigned long long *cnt, int check, unsigned long long n) {
  if (n) atomicAdd(cnt + check, n);
}

__global__ void k_check_below(const uint32_t *__restrict__ a, uint64_t n, uint32_t limit, int check,
                              unsigned long long *cnt) {
  unsigned long long bad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    bad += a[i] >= limit;
  bump(cnt, check, bad);
}

__global__ void k_check_sorted(const uint32_t *__restrict__ a, uint64_t n, unsigned long long *cnt) {
  unsigned long long bad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    bad += a[i - 1] > a[i];
  bump(cnt, 2, bad);
}

__global__ void k_check_where(const uint32_t *__restrict__ where, const uint64_t *__restrict__ blk_ptr, uint32_t nblk,
                              uint64_t nnz, unsigned long long *cnt) {
  unsigned long long bad = 0;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t b = block_of(blk_ptr, nblk, j);
    bad += (uint64_t)where[j] >= blk_ptr[b + 1] - blk_ptr[b];
  }
  bump(cnt, 4, bad);
}

// count[b * (bd + 1) + r], r = 0..bd: starts at 0, non-decreasing, ends at the block's size
__global__ void k_check_count(const uint64_t *__restrict__ count, const uint64_t *__restrict__ blk_ptr, uint32_t nblk,
                              uint32_t bd, unsigned long long *cnt) {
  unsigned long long bad = 0;
  const uint64_t m = (uint64_t)nblk * (bd + 1);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = i / (bd + 1), r = i % (bd + 1);
    if (r == 0)
      bad += count[i] != 0;
    else
      bad += count[i - 1] > count[i];
    if (r == bd) bad += count[i] != blk_ptr[b + 1] - blk_ptr[b];
  }
  bump(cnt, 5, bad);
}

template <class V>
__global__ void k_check_finite(const V *__restrict__ a, uint64_t rows, int cols, int ld, unsigned long long *cnt) {
  unsigned long long bad = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (uint64_t)gridDim.x * blockDim.x)
    bad += !isfinite((double)a[(i / cols) * ld + i % cols]);
  bump(cnt, 6, bad);
}

template <class V> int validate_impl(DevTensor &t, uint64_t *out) {
  DevBuf cbuf;  // freed on every return path
  GTK_CUDA(cbuf.alloc(kChecks * sizeof(unsigned long long)));
  unsigned long long *cnt = cbuf.as<unsigned long long>();
  GTK_CUDA(cudaMemsetAsync(cnt, 0, kChecks * sizeof(unsigned long long), t.stream));
  const unsigned g = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((t.nnz + 255) / 256, (uint64_t)t.num_sms * 8));
  const uint32_t nblk = (uint32_t)t.nblk;
  if (t.nnz) {
    for (int n = 0; n < t.N; ++n) {
      k_check_below<<<g, 256, 0, t.stream>>>(t.blk_idx[n], t.nnz, t.bd[n], 0, cnt);
      for (int k = 0; k < t.N; ++k) k_check_below<<<g, 256, 0, t.stream>>>(t.vidx[n][k], t.nnz, t.dims[k], 1, cnt);
      k_check_sorted<<<g, 256, 0, t.stream>>>(t.vidx[n][n], t.nnz, cnt);
      k_check_below<<<g, 256, 0, t.stream>>>(t.vperm[n], t.nnz, (uint32_t)t.nnz, 3, cnt);
      k_check_where<<<g, 256, 0, t.stream>>>(t.where[n], t.blk_ptr, nblk, t.nnz, cnt);
    }
  }
  for (int n = 0; n < t.N; ++n) {
    const uint64_t m = t.nblk * (uint64_t)(t.bd[n] + 1);
    const unsigned gc = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((m + 255) / 256, (uint64_t)t.num_sms * 8));
    k_check_count<<<gc, 256, 0, t.stream>>>(t.count[n], t.blk_ptr, nblk, t.bd[n], cnt);
    if (t.have_factors)
      k_check_finite<V><<<gc, 256, 0, t.stream>>>((const V *)t.fac[n], t.rows[n], t.J, t.ldf, cnt);
  }
  if (t.have_core) k_check_finite<V><<<g, 256, 0, t.stream>>>((const V *)t.core, t.core_n, 1, 1, cnt);
  GTK_CUDA(cudaGetLastError());
  unsigned long long h[kChecks];
  GTK_CUDA(cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, t.stream));
  GTK_CUDA(cudaStreamSynchronize(t.stream));
  for (int c = 0; c < kChecks; ++c) out[c] = h[c];
  // block pointers: the host copy the partition read back, and the device array against it
  std::vector<uint64_t> bp(t.nblk + 1);
  GTK_CUDA(cudaMemcpy(bp.data(), t.blk_ptr, bp.size() * 8, cudaMemcpyDeviceToHost));
  uint64_t bad = bp[0] != 0 || bp[t.nblk] != t.nnz;
  for (uint64_t b = 0; b < t.nblk; ++b) bad += bp[b] > bp[b + 1];
  if (t.h_blk_ptr.size() == bp.size()) bad += memcmp(bp.data(), t.h_blk_ptr.data(), bp.size() * 8) != 0;
  out[7] = bad;
  return 0;
}

}  // namespace

int run_validate(DevTensor &t, uint64_t *violations) {
  return t.dtype == GTK_F32 ? validate_impl<float>(t, violations) : validate_impl<double>(t, violations);
}

}  // namespace gtk
