// partition.cu -- tensor-block partition and per-mode segmenting on the GPU.
//
// Produces, bit-exactly, what the reference builds on the host:
//   * block id of a nonzero = sum_k (i_k / block_dims[k]) * prod_{l>k} P_l, last
//     mode fastest (tensor_manager.tpp:229-245, tensor.tpp:157-174);
//   * blocks keep input order: a stable sort by block id equals the reference's
//     serial insertion with position nnz_count - remaining
//     (tensor_manager.tpp:267-290, block.tpp:100-108);
//   * block-local coordinates i_k - block_coord_k * block_dims[k] (block.tpp:105);
//   * count_nnz[n] (CSR row pointer of each block, block_dims[n]+1 entries) and
//     where_nnz[n] (positions of the block's nonzeros, stably sorted by local
//     mode-n index) of every block (block.tpp:115-186).
// It also builds what the sweep runs on: for every mode n a copy of the tensor
// stably sorted by global mode-n row, so that the nonzeros of one factor row
// are contiguous and appear in (block_id, position) order -- the order in which
// ComputingBC (update.cuh:73-100) visits them.
//
// All sorts are one stable LSD radix sort (8-bit digits at most, tiles of 2048
// keys, in-tile ranks from warp match_any) -- integer work bound by HBM.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "internal.h"

namespace gtk {
namespace {

constexpr int kRsThreads = 256;
constexpr int kRsRounds = 8;
constexpr int kRsTile = kRsThreads * kRsRounds;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanChunk = kScanThreads * kScanItems;
constexpr uint32_t kHistSmemKeys = 8192;  // block histograms up to this many blocks count in shared memory

struct Ptrs {
  const uint32_t *p[kMaxOrder];
};
struct MPtrs {
  uint32_t *p[kMaxOrder];
};
struct Dims {
  uint32_t bd[kMaxOrder];
  uint32_t P[kMaxOrder];
};

// ---------------------------------------------------------------- radix sort
__global__ void k_radix_hist(const uint32_t *__restrict__ keys, uint64_t n, int shift, uint32_t mask,
                             uint32_t *__restrict__ hist, uint32_t ntiles) {
  __shared__ uint32_t cnt[256];
  for (int d = threadIdx.x; d <= (int)mask; d += blockDim.x) cnt[d] = 0;
  __syncthreads();
  uint64_t base = (uint64_t)blockIdx.x * kRsTile;
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    uint64_t i = base + (uint64_t)r * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & mask], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d <= (int)mask; d += blockDim.x) hist[(uint64_t)d * ntiles + blockIdx.x] = cnt[d];
}

// offs[d * ntiles + tile] = absolute output position of the tile's first key of digit d.
// The tile is first ordered by digit in shared memory (stable: rounds, then warps,
// then lanes, in key order), so that each digit's keys leave as one contiguous run
// and the global writes coalesce.
__global__ void k_radix_scatter(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                                uint32_t *__restrict__ okeys, uint32_t *__restrict__ ovals, uint64_t n, int shift,
                                uint32_t mask, const uint32_t *__restrict__ offs, uint32_t ntiles) {
  __shared__ uint32_t running[256];  // next tile-local position per digit
  __shared__ uint32_t lstart[256];   // tile-local start of each digit
  __shared__ uint32_t wcnt[kRsThreads / 32][256];
  __shared__ uint32_t skey[kRsTile], sval[kRsTile];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t base = (uint64_t)blockIdx.x * kRsTile;
  const int nt = (int)min((uint64_t)kRsTile, n - base);  // keys in this tile
  uint32_t key[kRsRounds], val[kRsRounds];
  for (int d = tid; d < 256; d += blockDim.x) running[d] = 0;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    const int i = r * kRsThreads + tid;
    key[r] = i < nt ? keys[base + i] : 0u;
    val[r] = i < nt ? vals[base + i] : 0u;
    if (i < nt) atomicAdd(&running[(key[r] >> shift) & mask], 1u);
  }
  __syncthreads();
  if (tid == 0) {  // exclusive scan of the tile's digit counts (at most 256)
    uint32_t acc = 0;
    for (int d = 0; d <= (int)mask; ++d) {
      const uint32_t c = running[d];
      lstart[d] = acc;
      running[d] = acc;
      acc += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    for (int k = tid; k < (kRsThreads / 32) * 256; k += blockDim.x) (&wcnt[0][0])[k] = 0;
    __syncthreads();
    const int i = r * kRsThreads + tid;
    const bool valid = i < nt;
    const uint32_t d = valid ? ((key[r] >> shift) & mask) : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
    const uint32_t lrank = __popc(peers & ((1u << lane) - 1u));
    if (valid && lrank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    for (int dd = tid; dd <= (int)mask; dd += blockDim.x) {
      uint32_t p = running[dd];
#pragma unroll
      for (int w = 0; w < kRsThreads / 32; ++w) {
        const uint32_t c = wcnt[w][dd];
        wcnt[w][dd] = p;
        p += c;
      }
      running[dd] = p;
    }
    __syncthreads();
    if (valid) {
      const uint32_t lpos = wcnt[warp][d] + lrank;
      skey[lpos] = key[r];
      sval[lpos] = val[r];
    }
    __syncthreads();  // wcnt is cleared for the next round
  }
  for (int j = tid; j < nt; j += blockDim.x) {
    const uint32_t k = skey[j];
    const uint32_t d = (k >> shift) & mask;
    const uint64_t pos = (uint64_t)offs[(uint64_t)d * ntiles + blockIdx.x] + (uint32_t)(j - lstart[d]);
    okeys[pos] = k;
    ovals[pos] = sval[j];
  }
}

// ---------------------------------------------------------------- exclusive scan
template <class T> __device__ T block_exclusive_scan(T v, T *smem_warp, T *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? smem_warp[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) smem_warp[lane] = w;
  }
  __syncthreads();
  T warp_off = warp > 0 ? smem_warp[warp - 1] : T(0);
  if (total) *total = smem_warp[nw - 1];
  __syncthreads();
  return warp_off + x - v;
}

template <class T> __global__ void k_scan_reduce(const T *__restrict__ in, uint64_t m, T *__restrict__ sums) {
  __shared__ T sw[32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + (uint64_t)threadIdx.x * kScanItems;
  T s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < m) s += in[base + k];
  T tot;
  block_exclusive_scan<T>(s, sw, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <class T> __global__ void k_scan_sums(T *sums, uint64_t nc) {
  __shared__ T sw[32];
  __shared__ T carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint64_t base = 0; base < nc; base += blockDim.x) {
    uint64_t i = base + threadIdx.x;
    T v = i < nc ? sums[i] : T(0);
    T tot;
    T ex = block_exclusive_scan<T>(v, sw, &tot);
    if (i < nc) sums[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

template <class T> __global__ void k_scan_down(const T *in, T *out, uint64_t m, const T *__restrict__ sums) {
  __shared__ T sw[32];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + (uint64_t)threadIdx.x * kScanItems;
  T v[kScanItems];
  T s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < m) ? in[base + k] : T(0);
    s += v[k];
  }
  T ex = block_exclusive_scan<T>(s, sw, nullptr) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < m) out[base + k] = ex;
    ex += v[k];
  }
}

template <class T> int exclusive_scan(T *data, uint64_t m, T *chunk_sums, cudaStream_t s) {
  if (m == 0) return 0;
  uint64_t nc = (m + kScanChunk - 1) / kScanChunk;
  k_scan_reduce<T><<<(unsigned)nc, kScanThreads, 0, s>>>(data, m, chunk_sums);
  k_scan_sums<T><<<1, 1024, 0, s>>>(chunk_sums, nc);
  k_scan_down<T><<<(unsigned)nc, kScanThreads, 0, s>>>(data, data, m, chunk_sums);
  GTK_CUDA(cudaGetLastError());
  return 0;
}

inline int bits_for(uint64_t max_value) {
  int b = 0;
  while (b < 64 && (max_value >> b) != 0) ++b;
  return b;
}

struct SortScratch {
  uint32_t *k2 = nullptr, *v2 = nullptr, *hist = nullptr, *sums = nullptr;
};

// Stable sort of (keys, vals) by the low `bits` bits of keys.  Result lands in
// (keys, vals) (ping-pong through the scratch pair).
int radix_sort(uint32_t *keys, uint32_t *vals, uint64_t n, int bits, SortScratch &sc, cudaStream_t s) {
  if (n <= 1 || bits == 0) return 0;
  const int passes = (bits + 7) / 8;
  const int width = (bits + passes - 1) / passes;
  const uint32_t ntiles = (uint32_t)((n + kRsTile - 1) / kRsTile);
  uint32_t *ka = keys, *va = vals, *kb = sc.k2, *vb = sc.v2;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * width;
    const int w = std::min(width, bits - shift);
    const uint32_t mask = (1u << w) - 1u;
    k_radix_hist<<<ntiles, kRsThreads, 0, s>>>(ka, n, shift, mask, sc.hist, ntiles);
    if (int rc = exclusive_scan<uint32_t>(sc.hist, (uint64_t)(mask + 1) * ntiles, sc.sums, s)) return rc;
    k_radix_scatter<<<ntiles, kRsThreads, 0, s>>>(ka, va, kb, vb, n, shift, mask, sc.hist, ntiles);
    GTK_CUDA(cudaGetLastError());
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    GTK_CUDA(cudaMemcpyAsync(keys, ka, n * 4, cudaMemcpyDeviceToDevice, s));
    GTK_CUDA(cudaMemcpyAsync(vals, va, n * 4, cudaMemcpyDeviceToDevice, s));
  }
  return 0;
}

// ---------------------------------------------------------------- partition kernels
__global__ void k_block_id(Ptrs g, int N, Dims dm, uint64_t n, uint32_t *__restrict__ bid,
                           uint32_t *__restrict__ iota) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t b = 0, mult = 1;
    for (int k = N - 1; k >= 0; --k) {
      b += (uint64_t)(g.p[k][t] / dm.bd[k]) * mult;
      mult *= dm.P[k];
    }
    bid[t] = (uint32_t)b;
    iota[t] = (uint32_t)t;
  }
}

// histogram of keys < nkeys into cnt (u64); per-CTA shared counters when they fit
__global__ void k_count_u64(const uint32_t *__restrict__ key, uint64_t n, uint64_t *__restrict__ cnt, uint32_t nkeys) {
  extern __shared__ unsigned int hs[];
  const bool local = nkeys <= kHistSmemKeys;
  if (local) {
    for (uint32_t k = threadIdx.x; k < nkeys; k += blockDim.x) hs[k] = 0;
    __syncthreads();
  }
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    if (local)
      atomicAdd(&hs[key[t]], 1u);
    else
      atomicAdd((unsigned long long *)&cnt[key[t]], 1ull);
  }
  if (local) {
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < nkeys; k += blockDim.x)
      if (hs[k]) atomicAdd((unsigned long long *)&cnt[k], (unsigned long long)hs[k]);
  }
}

// gather the coordinates into block-major order; global copy gblk and local blk_idx
template <class V>
__global__ void k_gather_blocks(Ptrs g, const V *__restrict__ val, int N, Dims dm, uint64_t n,
                                const uint32_t *__restrict__ perm, const uint32_t *__restrict__ sbid, MPtrs gblk,
                                MPtrs lidx, V *__restrict__ oval) {
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t src = perm[p];
    uint32_t b = sbid[p];
    for (int k = N - 1; k >= 0; --k) {
      const uint32_t c = b % dm.P[k];
      b /= dm.P[k];
      const uint32_t gi = g.p[k][src];
      gblk.p[k][p] = gi;
      lidx.p[k][p] = gi - c * dm.bd[k];
    }
    oval[p] = val[src];
  }
}

// A nonzero as one 32-byte record: global coordinates in words 0 .. N-1 (N <= 5),
// the block id in word 5 (block order only), the value's bits in words 6 (FP32)
// or 6-7 (FP64).  A gather by permutation then reads one DRAM sector per nonzero
// instead of one per coordinate array and one for the value.
constexpr int kRecMaxOrder = 5;
__device__ __forceinline__ void rec_load(const uint4 *__restrict__ rec, uint64_t i, uint32_t (&w)[8]) {
  const uint4 a = __ldg(rec + 2 * i), b = __ldg(rec + 2 * i + 1);
  w[0] = a.x, w[1] = a.y, w[2] = a.z, w[3] = a.w, w[4] = b.x, w[5] = b.y, w[6] = b.z, w[7] = b.w;
}
__device__ __forceinline__ void rec_store(uint4 *__restrict__ rec, uint64_t i, const uint32_t (&w)[8]) {
  rec[2 * i] = make_uint4(w[0], w[1], w[2], w[3]);
  rec[2 * i + 1] = make_uint4(w[4], w[5], w[6], w[7]);
}
template <class V> __device__ __forceinline__ void rec_put_val(uint32_t (&w)[8], V v) {
  if (sizeof(V) == 4) {
    w[6] = __float_as_uint((float)v);
  } else {
    const unsigned long long u = __double_as_longlong((double)v);
    w[6] = (uint32_t)u, w[7] = (uint32_t)(u >> 32);
  }
}
template <class V> __device__ __forceinline__ V rec_get_val(const uint32_t (&w)[8]) {
  if (sizeof(V) == 4) return (V)__uint_as_float(w[6]);
  return (V)__longlong_as_double((long long)(((unsigned long long)w[7] << 32) | w[6]));
}

// The caller's COO read in place from host memory (a device that reaches
// pageable host memory: Grace's address translation over NVLink-C2C): the
// input-order record, the device copy of the value (val_in) and the block id of
// every nonzero in one pass -- the upload, k_pack_records and k_block_id fused
template <class V>
__global__ void k_pack_records_host(Ptrs g, const V *__restrict__ val, int N, Dims dm, uint64_t n,
                                    uint4 *__restrict__ rec, V *__restrict__ val_dev, uint32_t *__restrict__ bid,
                                    uint32_t *__restrict__ iota) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < kRecMaxOrder; ++k)
      if (k < N) w[k] = g.p[k][t];
    uint64_t b = 0, mult = 1;
    for (int k = N - 1; k >= 0; --k) {
      b += (uint64_t)(w[k] / dm.bd[k]) * mult;
      mult *= dm.P[k];
    }
    const V v = val[t];
    rec_put_val<V>(w, v);
    rec_store(rec, t, w);
    val_dev[t] = v;
    bid[t] = (uint32_t)b;
    iota[t] = (uint32_t)t;
  }
}

// input-order records from the uploaded coordinate arrays and values
template <class V>
__global__ void k_pack_records(Ptrs g, const V *__restrict__ val, int N, uint64_t n, uint4 *__restrict__ rec) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < kRecMaxOrder; ++k)
      if (k < N) w[k] = g.p[k][t];
    rec_put_val<V>(w, val[t]);
    rec_store(rec, t, w);
  }
}

// k_gather_blocks from records; also writes the block-order records (with block id)
template <class V>
__global__ void k_gather_blocks_rec(const uint4 *__restrict__ rin, int N, Dims dm, uint64_t n,
                                    const uint32_t *__restrict__ perm, const uint32_t *__restrict__ sbid, MPtrs gblk,
                                    MPtrs lidx, V *__restrict__ oval, uint4 *__restrict__ rblk) {
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t w[8];
    rec_load(rin, perm[p], w);
    const uint32_t bid = sbid[p];
    uint32_t b = bid;
#pragma unroll
    for (int k = kRecMaxOrder - 1; k >= 0; --k) {
      if (k < N) {
        const uint32_t c = b % dm.P[k];
        b /= dm.P[k];
        gblk.p[k][p] = w[k];
        lidx.p[k][p] = w[k] - c * dm.bd[k];
      }
    }
    oval[p] = rec_get_val<V>(w);
    w[5] = bid;
    rec_store(rblk, p, w);
  }
}

// k_gather_view from block-order records, fused with the where-sort's keys
// (block id of each view element) and values (its block-order position)
template <class V>
__global__ void k_gather_view_rec(const uint32_t *__restrict__ perm, uint64_t n, int N, const uint4 *__restrict__ rblk,
                                  MPtrs vidx, V *__restrict__ vval, uint32_t *__restrict__ keys,
                                  uint32_t *__restrict__ vals) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = perm[i];
    uint32_t w[8];
    rec_load(rblk, p, w);
#pragma unroll
    for (int k = 0; k < kRecMaxOrder; ++k)
      if (k < N) vidx.p[k][i] = w[k];
    vval[i] = rec_get_val<V>(w);
    keys[i] = w[5];
    vals[i] = p;
  }
}

template <class V>
__global__ void k_sumsq(const V *__restrict__ v, uint64_t n, double *__restrict__ partial) {
  __shared__ double sw[32];
  double s = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    double x = (double)v[t];
    s += x * x;
  }
  double tot;
  block_exclusive_scan<double>(s, sw, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void k_sum_partials(const double *__restrict__ partial, int m, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += partial[i];
    *out = s;
  }
}

// key of view element i: global row of mode n of block-major element i
__global__ void k_iota(uint32_t *__restrict__ a, uint64_t n) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    a[t] = (uint32_t)t;
}

template <class V>
__global__ void k_gather_view(const uint32_t *__restrict__ perm, uint64_t n, int N, Ptrs gblk, MPtrs vidx,
                              const V *__restrict__ val, V *__restrict__ vval) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = perm[i];
    for (int k = 0; k < N; ++k) vidx.p[k][i] = gblk.p[k][p];
    vval[i] = val[p];
  }
}

// keys for the where-sort: block id of each view element
__global__ void k_view_block_keys(const uint32_t *__restrict__ perm, const uint32_t *__restrict__ sbid, uint64_t n,
                                  uint32_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = perm[i];
    keys[i] = sbid[p];
    vals[i] = p;
  }
}

// where[j] = position inside its block
__global__ void k_where(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ pos, uint64_t n,
                        const uint64_t *__restrict__ blk_ptr, uint32_t *__restrict__ where) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x)
    where[j] = (uint32_t)(pos[j] - blk_ptr[keys[j]]);
}

// histogram of (block, local row) into count[b*(bd+1) + row]; one atomic per
// distinct counter in a warp (heavy rows of a skewed tensor recur within a warp)
// count_nnz of mode m from its view: in view order (global row, then
// block-major position) the nonzeros of one (block, local row) pair form one
// contiguous run -- a block spans bd consecutive rows, so the local row is
// row % bd -- and its count is the run's length.  The run's first element adds
// -p and its last p + 1 (two atomics per run, on distinct counters; the uint64
// wrap-around leaves the length), against one atomic per nonzero.
__global__ void k_count_view(const uint32_t *__restrict__ bid, const uint32_t *__restrict__ row, uint64_t n,
                             uint32_t bd, uint64_t *__restrict__ cnt) {
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t b = bid[p], r = row[p];
    const bool head = p == 0 || bid[p - 1] != b || row[p - 1] != r;
    const bool tail = p + 1 == n || bid[p + 1] != b || row[p + 1] != r;
    if (!head && !tail) continue;
    unsigned long long *c = (unsigned long long *)&cnt[(uint64_t)b * (bd + 1) + r % bd];
    if (head) atomicAdd(c, 0ull - (unsigned long long)p);
    if (tail) atomicAdd(c, (unsigned long long)p + 1ull);
  }
}

// after a global exclusive scan: count[b][r] -= blk_ptr[b]
__global__ void k_count_rebase(uint64_t *__restrict__ cnt, uint64_t nblk, uint32_t bd,
                               const uint64_t *__restrict__ blk_ptr) {
  const uint64_t m = nblk * (uint64_t)(bd + 1);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
    cnt[i] -= blk_ptr[i / (bd + 1)];
}

inline unsigned grid_for(uint64_t n, int threads, int num_sms) {
  uint64_t g = (n + threads - 1) / threads;
  uint64_t cap = (uint64_t)num_sms * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

template <class V> int build_impl(DevTensor &t, const gtk_coo &coo) {
  cudaStream_t s = t.stream;
  const uint64_t n = t.nnz;
  const int N = t.N;
  const int T = 256;
  const unsigned G = grid_for(n, T, t.num_sms);
  Dims dm;
  for (int k = 0; k < kMaxOrder; ++k) {
    dm.bd[k] = k < N ? t.bd[k] : 1;
    dm.P[k] = k < N ? t.P[k] : 1;
  }
  // temporaries, freed at the end
  // temporaries from the process-wide block cache (a repeated create of one
  // shape reuses them), returned to it at the end
  std::vector<std::pair<void *, size_t>> tmp;
  auto talloc = [&](void **p, size_t bytes) -> int {
    bytes = (std::max<size_t>(bytes, 16) + 255) / 256 * 256;
    *p = dev_alloc(t.dev, bytes);
    if (!*p) return fail(GTK_ERR_OOM, "device allocation of " + std::to_string(bytes) + " bytes of temporaries failed");
    tmp.push_back({*p, bytes});
    return 0;
  };
  auto cleanup = [&]() {
    cudaStreamSynchronize(s);
    for (const auto &b : tmp) dev_free(t.dev, b.first, b.second);
  };
#define TRY(x)          \
  do {                  \
    int rc_ = (x);      \
    if (rc_) {          \
      cleanup();        \
      return rc_;       \
    }                   \
  } while (0)

  // phase timers (upload, kernels), read back at the end
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  struct EvGuard {
    cudaEvent_t *e;
    ~EvGuard() {
      for (int i = 0; i < 3; ++i)
        if (e[i]) cudaEventDestroy(e[i]);
    }
  } ev_guard{ev};
  for (auto &e : ev) TRY(ck(cudaEventCreate(&e), "cudaEventCreate"));
  // Where the device reads pageable host memory coherently (Grace: address
  // translation over NVLink-C2C), the first kernel reads the caller's arrays in
  // place (k_pack_records_host); elsewhere, or with GTK_HOST_DIRECT=0, they are
  // uploaded first.  Either way the host arrays are read once.
  int pageable = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, t.dev) != cudaSuccess) {
    cudaGetLastError();
    pageable = 0;
  }
  const char *hd = getenv("GTK_HOST_DIRECT");
  const bool direct = pageable == 1 && !(hd && *hd == '0') && N <= kRecMaxOrder && n;
  t.create_direct = direct;
  // the values stay on the device in input order: the reference's serial norm sums them in that order
  TRY(dalloc(t, &t.val_in, n * sizeof(V)));
  V *dval = reinterpret_cast<V *>(t.val_in);
  // 32-byte records (N <= 5): input order, then block order; without room for
  // them the gathers read the coordinate arrays one by one
  uint4 *rin = nullptr, *rblk = nullptr;
  if (N <= kRecMaxOrder && n) {
    const size_t rb = (n * 32 + 255) / 256 * 256;
    rin = static_cast<uint4 *>(dev_alloc(t.dev, rb));
    if (rin) {
      tmp.push_back({rin, rb});
      rblk = static_cast<uint4 *>(dev_alloc(t.dev, rb));
      if (rblk) tmp.push_back({rblk, rb});
    }
    if (!rblk) rin = nullptr;
  }
  uint32_t *sbid, *perm;
  TRY(talloc((void **)&sbid, n * 4));
  TRY(talloc((void **)&perm, n * 4));
  TRY(ck(cudaEventRecord(ev[0], s), "cudaEventRecord"));
  Ptrs gin;
  const bool fused = direct && rin;
  if (fused) {
    Ptrs hst;
    for (int k = 0; k < N; ++k) hst.p[k] = coo.idx[k].data();
    k_pack_records_host<V><<<G, T, 0, s>>>(hst, reinterpret_cast<const V *>(coo.values()), N, dm, n, rin, dval, sbid,
                                           perm);
    TRY(ck(cudaGetLastError(), "k_pack_records_host"));
  } else {
    // upload COO
    for (int k = 0; k < N; ++k) {
      void *p;
      TRY(talloc(&p, n * 4));
      if (n) TRY(ck(cudaMemcpyAsync(p, coo.idx[k].data(), n * 4, cudaMemcpyHostToDevice, s), "upload coords"));
      gin.p[k] = (const uint32_t *)p;
    }
    if (n) TRY(ck(cudaMemcpyAsync(dval, coo.values(), n * sizeof(V), cudaMemcpyHostToDevice, s), "upload values"));
  }
  TRY(ck(cudaEventRecord(ev[1], s), "cudaEventRecord"));
  SortScratch sc;
  const uint64_t ntiles = (n + kRsTile - 1) / kRsTile;
  TRY(talloc((void **)&sc.k2, n * 4));
  TRY(talloc((void **)&sc.v2, n * 4));
  TRY(talloc((void **)&sc.hist, 256 * ntiles * 4 + 16));
  uint64_t max_scan = std::max<uint64_t>(256 * ntiles, 1);
  for (int k = 0; k < N; ++k) max_scan = std::max<uint64_t>(max_scan, t.nblk * (uint64_t)(t.bd[k] + 1));
  max_scan = std::max<uint64_t>(max_scan, t.nblk + 1);
  TRY(talloc((void **)&sc.sums, ((max_scan + kScanChunk - 1) / kScanChunk + 1) * 8));

  if (rin && !fused) {
    k_pack_records<V><<<G, T, 0, s>>>(gin, dval, N, n, rin);
    TRY(ck(cudaGetLastError(), "k_pack_records"));
  }
  if (n && !fused) {
    k_block_id<<<G, T, 0, s>>>(gin, N, dm, n, sbid, perm);
    TRY(ck(cudaGetLastError(), "k_block_id"));
  }
  TRY(radix_sort(sbid, perm, n, bits_for(t.nblk - 1), sc, s));
  // blk_ptr
  TRY(ck(cudaMemsetAsync(t.blk_ptr, 0, (t.nblk + 1) * 8, s), "memset"));
  if (n) {
    const size_t hsm = t.nblk <= kHistSmemKeys ? t.nblk * 4 : 0;
    k_count_u64<<<G, T, hsm, s>>>(sbid, n, t.blk_ptr, (uint32_t)t.nblk);
  }
  TRY(exclusive_scan<unsigned long long>((unsigned long long *)t.blk_ptr, t.nblk + 1, (unsigned long long *)sc.sums, s));
  // block-major arrays (global copy in gblk for the views)
  MPtrs gblk, lidx;
  for (int k = 0; k < N; ++k) {
    TRY(talloc((void **)&gblk.p[k], n * 4));
    lidx.p[k] = t.blk_idx[k];
  }
  if (n && rblk) {
    k_gather_blocks_rec<V><<<G, T, 0, s>>>(rin, N, dm, n, perm, sbid, gblk, lidx, (V *)t.blk_val, rblk);
    TRY(ck(cudaGetLastError(), "k_gather_blocks_rec"));
  } else if (n) {
    k_gather_blocks<V><<<G, T, 0, s>>>(gin, dval, N, dm, n, perm, sbid, gblk, lidx, (V *)t.blk_val);
    TRY(ck(cudaGetLastError(), "k_gather_blocks"));
  }
  // norm in FP64, fixed reduction order
  {
    const int np = t.num_sms * 2;
    k_sumsq<V><<<np, 256, 0, s>>>((const V *)t.blk_val, n, t.partial);
    k_sum_partials<<<1, 32, 0, s>>>(t.partial, np, t.partial + np);
    double ss = 0;
    TRY(ck(cudaMemcpyAsync(&ss, t.partial + np, 8, cudaMemcpyDeviceToHost, s), "norm"));
    TRY(ck(cudaStreamSynchronize(s), "norm sync"));
    t.norm = std::sqrt(ss);
  }
  Ptrs gb;
  for (int k = 0; k < N; ++k) gb.p[k] = gblk.p[k];
  uint32_t *keys;
  TRY(talloc((void **)&keys, n * 4));
  for (int m = 0; m < N; ++m) {
    // view: stable sort of block-major order by global row of mode m
    if (n) {
      TRY(ck(cudaMemcpyAsync(keys, gblk.p[m], n * 4, cudaMemcpyDeviceToDevice, s), "copy"));
      k_iota<<<G, T, 0, s>>>(t.vperm[m], n);
    }
    TRY(radix_sort(keys, t.vperm[m], n, bits_for(t.dims[m] - 1), sc, s));
    MPtrs vi;
    for (int k = 0; k < N; ++k) vi.p[k] = t.vidx[m][k];
    // where_nnz: stable sort of the view by block id -> (block, row, position)
    if (n && rblk) {
      k_gather_view_rec<V><<<G, T, 0, s>>>(t.vperm[m], n, N, rblk, vi, (V *)t.vval[m], keys, perm);
    } else if (n) {
      k_gather_view<V><<<G, T, 0, s>>>(t.vperm[m], n, N, gb, vi, (const V *)t.blk_val, (V *)t.vval[m]);
      k_view_block_keys<<<G, T, 0, s>>>(t.vperm[m], sbid, n, keys, perm);
    }
    // count_nnz, from the view order (keys: block ids in view order)
    const uint64_t cm = t.nblk * (uint64_t)(t.bd[m] + 1);
    TRY(ck(cudaMemsetAsync(t.count[m], 0, cm * 8, s), "memset"));
    if (n) k_count_view<<<G, T, 0, s>>>(keys, t.vidx[m][m], n, t.bd[m], t.count[m]);
    TRY(radix_sort(keys, perm, n, bits_for(t.nblk - 1), sc, s));
    if (n) k_where<<<G, T, 0, s>>>(keys, perm, n, t.blk_ptr, t.where[m]);
    TRY(exclusive_scan<unsigned long long>((unsigned long long *)t.count[m], cm, (unsigned long long *)sc.sums, s));
    k_count_rebase<<<grid_for(cm, T, t.num_sms), T, 0, s>>>(t.count[m], t.nblk, t.bd[m], t.blk_ptr);
    TRY(ck(cudaGetLastError(), "segmenting"));
  }
  t.h_blk_ptr.resize(t.nblk + 1);
  TRY(ck(cudaMemcpyAsync(t.h_blk_ptr.data(), t.blk_ptr, (t.nblk + 1) * 8, cudaMemcpyDeviceToHost, s), "blk_ptr"));
  TRY(ck(cudaEventRecord(ev[2], s), "cudaEventRecord"));
  TRY(ck(cudaStreamSynchronize(s), "partition sync"));
  {
    float up = 0, kern = 0;
    TRY(ck(cudaEventElapsedTime(&up, ev[0], ev[1]), "cudaEventElapsedTime"));
    TRY(ck(cudaEventElapsedTime(&kern, ev[1], ev[2]), "cudaEventElapsedTime"));
    t.create_upload_ms = up;
    t.create_kernels_ms = kern;
  }
  cleanup();
#undef TRY
  return 0;
}

}  // namespace

int build_partition(DevTensor &t, const gtk_coo &coo) {
  return t.dtype == GTK_F32 ? build_impl<float>(t, coo) : build_impl<double>(t, coo);
}

}  // namespace gtk
