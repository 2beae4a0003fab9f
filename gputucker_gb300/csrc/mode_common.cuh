// mode_common.cuh -- device pieces shared by the mode kernels (SIMT and tcgen05):
// the kernel argument block, the shared tile layout and the row-segmented
// Gram/RHS reduction of a tile of delta rows.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace gtk {
namespace {

constexpr int kThreads = 256;
constexpr int kFitGridMax = 1024;

enum Kind { kUpdate = 0, kFit = 1, kDelta = 2 };

template <int B, int E> struct Pow { static constexpr int v = B * Pow<B, E - 1>::v; };
template <int B> struct Pow<B, 0> { static constexpr int v = 1; };

struct ModeArgs {
  const uint32_t *coord[kMaxOrder];  // view coordinates (global), coord[mode] = row
  const void *val;                   // view values
  // factor matrices, row stride ldf; in the tensor-core kernels' arguments the
  // other modes' entries of an ldf = 12 handle point at its gather copies
  // (DevTensor::gfac, 64-byte rows)
  const void *fac[kMaxOrder];
  const void *corep;                 // [J^(N-1)][ldf], mode first
  const uint32_t *vperm;             // view -> block-major position (kDelta)
  void *out;                         // kDelta: delta [nnz][J] block-major
  double *gram;                      // kUpdate: [rows][E]
  double *partial;                   // kFit: per-CTA error sums
  int *status;                       // device status word (bit 1: a bounded wait gave up)
  void *dstore;                      // kUpdate: when set, delta of every nonzero in view order [nnz][J]
  uint64_t nnz;
  int N, J, ldf, mode, E, ldd;
  int others[kMaxOrder];             // the other modes in increasing order
  uint64_t gp_elems;                 // J^(N-1) * ldf
  int gp_in_smem;                    // generic kernel: core in shared memory?
  int ref_order;                     // generic kernel: delta in the reference's operation order
  const void *core;                  // the core, linear order (last mode fastest): ref_order
};

// row r of a gather copy (PadItem); floats 12..15 of a copied row are never read
__device__ __forceinline__ void pad_row(const PadItem &it, uint64_t r) {
  const float4 *s = reinterpret_cast<const float4 *>(it.src + r * 12);
  float4 *d = reinterpret_cast<float4 *>(it.dst + r * 16);
  const float4 a = __ldg(s), b = __ldg(s + 1), c = __ldg(s + 2);
  d[0] = a, d[1] = b, d[2] = c;
}

// A multi-tensor launch (batches): up to kMultiMax handles of one kernel class,
// handle i owning CTAs [first[i], first[i + 1]).  Passed by value as a
// __grid_constant__ kernel parameter (under the 32 KB parameter limit), so the
// kernels read the argument blocks from the constant bank as a single-handle
// launch reads its ModeArgs.
constexpr int kMultiMax = 96;
struct MultiParams {
  ModeArgs args[kMultiMax];
  const unsigned char *img[kMultiMax];  // streamed-core class: each handle's core image
  uint32_t first[kMultiMax + 1];
  int count;
};
static_assert(sizeof(MultiParams) <= 32000, "kernel parameter limit");

// This CTA's handle of a multi-tensor launch: its argument block copied into
// shared memory (the kernels then read fields as a single-handle launch reads
// its parameters, reloading them after barriers instead of holding them in
// registers); returns the CTA's index and count within the handle's range.
__device__ __forceinline__ const ModeArgs &multi_select(const MultiParams &p, ModeArgs &sa, uint32_t &cta,
                                                        uint32_t &nctas, const unsigned char **img = nullptr) {
  int lo = 0, hi = p.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p.first[mid] <= blockIdx.x)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int i = lo;
  constexpr int W = (int)(sizeof(ModeArgs) / 8);
  static_assert(sizeof(ModeArgs) % 8 == 0, "argument block in 8-byte words");
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(&p.args[i]);
  unsigned long long *dst = reinterpret_cast<unsigned long long *>(&sa);
  for (int k = threadIdx.x; k < W; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  cta = blockIdx.x - p.first[i];
  nctas = p.first[i + 1] - p.first[i];
  if (img) *img = p.img[i];
  return sa;
}

// the entry i with first[i] <= b < first[i + 1] of a parameter-space table
__device__ __forceinline__ int slot_of_param(const uint32_t *first, int count, uint32_t b) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// the entry i of a multi-tensor launch whose CTA range [first[i], first[i + 1])
// holds CTA b (first[0] = 0, first[count] = the grid)
__device__ __forceinline__ int slot_of(const uint32_t *__restrict__ first, int count, uint32_t b) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(first + mid) <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------- vector loads
template <class V> struct Vec;
template <> struct Vec<float> {
  using T = float4;
  static constexpr int W = 4;
  __device__ static void unpack(const T &v, float *o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
};
template <> struct Vec<double> {
  using T = double2;
  static constexpr int W = 2;
  __device__ static void unpack(const T &v, double *o) { o[0] = v.x; o[1] = v.y; }
};

// ---------------------------------------------------------------- shared tile layout
template <class V> struct TileSmem {
  // carve: [gp][arow][dx][rows][seg_start][pairs]
  V *gp;
  V *arow;
  V *dx;
  uint32_t *rows;
  uint32_t *seg;
  unsigned char *pi, *pj;
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Shared memory needed by a tile of `tn` nonzeros.
inline size_t tile_smem_bytes(size_t vsize, size_t gp_elems, int arow_levels, int npt, int J, int ldd, int E,
                              int tn) {
  size_t b = align_up(gp_elems * vsize, 16);
  b += align_up((size_t)arow_levels * npt * J * kThreads * vsize, 16);
  b += align_up((size_t)tn * ldd * vsize, 16);
  b += align_up((size_t)tn * 4, 16);
  b += align_up((size_t)(tn + 1) * 4, 16);
  b += align_up((size_t)E * 2, 16);
  return b;
}

template <class V>
__device__ TileSmem<V> carve(unsigned char *base, size_t gp_elems, int arow_levels, int npt, int J, int ldd, int E,
                             int tn) {
  TileSmem<V> s;
  size_t off = 0;
  s.gp = reinterpret_cast<V *>(base + off);
  off += align_up(gp_elems * sizeof(V), 16);
  s.arow = reinterpret_cast<V *>(base + off);
  off += align_up((size_t)arow_levels * npt * J * kThreads * sizeof(V), 16);
  s.dx = reinterpret_cast<V *>(base + off);
  off += align_up((size_t)tn * ldd * sizeof(V), 16);
  s.rows = reinterpret_cast<uint32_t *>(base + off);
  off += align_up((size_t)tn * 4, 16);
  s.seg = reinterpret_cast<uint32_t *>(base + off);
  off += align_up((size_t)(tn + 1) * 4, 16);
  s.pi = base + off;
  s.pj = base + off + E;
  return s;
}

// pair table of the Gram/RHS entries: e -> (i, j), i <= j <= J, except (J, J),
// row-major over the upper triangle.  Column J of the delta tile holds x, so
// (i, J) is the right-hand side C_i = sum x*delta_i.
__device__ void fill_pairs(unsigned char *pi, unsigned char *pj, int J) {
  if (threadIdx.x == 0) {
    int e = 0;
    for (int i = 0; i <= J; ++i)
      for (int j = i; j <= J; ++j) {
        if (i == J && j == J) continue;
        pi[e] = (unsigned char)i;
        pj[e] = (unsigned char)j;
        ++e;
      }
  }
}

// an un-contractible product (never fused into an FMA with the following add)
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <class V> struct ProdSum {
  double s = 0;
  __device__ void add(V p) { s += (double)p; }
  __device__ double value() const { return s; }
};
template <> struct ProdSum<float> {
  float s = 0.f, c = 0.f;
  __device__ void add(float p) {
    const float t = s + p;
    c += (fabsf(s) >= fabsf(p)) ? ((s - t) + p) : ((p - t) + s);
    s = t;
  }
  __device__ double value() const { return (double)s + (double)c; }
};

// Row-segmented reduction of the tile into the FP64 Gram/RHS rows.
// tile_start: view position of tile element 0; nv: valid elements in the tile.
template <class V>
__device__ void gram_phase(const ModeArgs &a, const TileSmem<V> &s, uint64_t tile_start, int nv, int npt) {
  const int tid = threadIdx.x;
  __shared__ uint32_t sw[32];
  __shared__ uint32_t nseg_s;
  // segment heads over contiguous chunks of npt positions per thread
  uint32_t cnt = 0;
  for (int k = 0; k < npt; ++k) {
    int t = tid * npt + k;
    if (t < nv && (t == 0 || s.rows[t] != s.rows[t - 1])) ++cnt;
  }
  // block exclusive scan of cnt
  {
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    if (warp == 0) {
      const int nw = (int)(blockDim.x >> 5);
      uint32_t w = lane < nw ? sw[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        if (lane >= o) w += y;
      }
      if (lane < nw) sw[lane] = w;
      if (lane == nw - 1) nseg_s = w;
    }
    __syncthreads();
    uint32_t id = (warp > 0 ? sw[warp - 1] : 0u) + x - cnt;
    for (int k = 0; k < npt; ++k) {
      int t = tid * npt + k;
      if (t < nv && (t == 0 || s.rows[t] != s.rows[t - 1])) s.seg[id++] = (uint32_t)t;
    }
    if (tid == 0) s.seg[nseg_s] = (uint32_t)nv;
  }
  __syncthreads();
  const int nseg = (int)nseg_s;
  const int E = a.E, ldd = a.ldd;
  // does the tile hold the whole first / last row?
  const uint32_t first_row = s.rows[0], last_row = nv > 0 ? s.rows[nv - 1] : 0u;
  const bool first_open = tile_start > 0 && a.coord[a.mode][tile_start - 1] == first_row;
  const bool last_open = tile_start + nv < a.nnz && a.coord[a.mode][tile_start + nv] == last_row;
  const int items = nseg * E;
  for (int w = tid; w < items; w += (int)blockDim.x) {
    const int sgi = w / E, e = w - sgi * E;
    const int i = s.pi[e], j = s.pj[e];
    const int t0 = (int)s.seg[sgi], t1 = (int)s.seg[sgi + 1];
    double sum;
    if (a.ref_order) {  // ComputingBC (update.cuh:85-90): value_t products added in double, in view order
      sum = 0;
      for (int t = t0; t < t1; ++t) sum += (double)mul_rn(s.dx[t * ldd + i], s.dx[t * ldd + j]);
    } else {
      ProdSum<V> acc;
      for (int t = t0; t < t1; ++t) acc.add(mul_rn(s.dx[t * ldd + i], s.dx[t * ldd + j]));
      sum = acc.value();
    }
    const uint32_t row = s.rows[t0];
    double *dst = a.gram + (size_t)row * E + e;
    const bool shared_row = (sgi == 0 && first_open) || (sgi == nseg - 1 && last_open);
    if (shared_row)
      atomicAdd(dst, sum);
    else
      *dst = sum;
  }
}


// Running Gram/RHS sums of one warp.  Lane l owns the entries e = l + 32k
// (k < KE) of the packed row; the warp walks its slice of each tile in view
// order, adding delta_i * delta_j for every entry, and flushes its sums with
// FP64 atomics whenever the row changes and at the end of the CTA's
// (contiguous) range of tiles.  A long row thus costs one flush per warp and
// CTA, a short row one or two flushes; no block-wide barrier is needed.
//   EXACT (the plain form): every product rounded to value_t as ComputingBC
//     forms it (update.cuh:85-90) and added with Neumaier compensation.
//   !EXACT (the tensor-core forms, whose delta carries BF16/TF32 rounding):
//     plain FP32 fused multiply-adds within a tile slice (<= 64 terms), merged
//     into the compensated running sum once per slice or row change.
// Slots past the last entry read column zc of the tile (kept at zero), so the
// inner loop has no branches.
template <class V, int KE, bool EXACT> struct GramAcc {
  ProdSum<V> acc[KE];
  V part[KE];
  int ei[KE], ej[KE];
  uint32_t row = 0xFFFFFFFFu;

  __device__ void init(const unsigned char *pi, const unsigned char *pj, int E, int zc, int lane) {
#pragma unroll
    for (int k = 0; k < KE; ++k) {
      const int e = lane + 32 * k;
      ei[k] = e < E ? pi[e] : zc;
      ej[k] = e < E ? pj[e] : zc;
      acc[k] = ProdSum<V>();
      part[k] = V(0);
    }
  }
  __device__ void merge() {
    if (!EXACT) {
#pragma unroll
      for (int k = 0; k < KE; ++k) {
        acc[k].add(part[k]);
        part[k] = V(0);
      }
    }
  }
  __device__ void flush(double *gram, int E, int lane) {
    merge();
    if (row != 0xFFFFFFFFu) {
#pragma unroll
      for (int k = 0; k < KE; ++k)
        if (lane + 32 * k < E) atomicAdd(gram + (size_t)row * E + lane + 32 * k, acc[k].value());
    }
#pragma unroll
    for (int k = 0; k < KE; ++k) acc[k] = ProdSum<V>();
  }
  // tile positions [t0, t1) of the shared delta tile (row stride ldd, column J = x)
  __device__ void run(const V *dx, int ldd, const uint32_t *rows, int t0, int t1, double *gram, int E, int lane) {
    if constexpr (EXACT) {
      for (int t = t0; t < t1; ++t) {
        const uint32_t r = rows[t];
        if (r != row) {
          flush(gram, E, lane);
          row = r;
        }
        const V *d = dx + t * ldd;
#pragma unroll
        for (int k = 0; k < KE; ++k) acc[k].add(mul_rn(d[ei[k]], d[ej[k]]));
      }
    } else {
    // runs of equal rows, 32 positions at a time: one ballot finds where rows change
    for (int base = t0; base < t1; base += 32) {
      const int n = min(32, t1 - base);
      const uint32_t my = lane < n ? rows[base + lane] : 0xFFFFFFFFu;
      const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, my, 1);
      const bool head = lane < n && (lane == 0 ? my != row : my != prev);
      uint32_t heads = __ballot_sync(0xFFFFFFFFu, head);
      int a = 0;
      while (a < n) {
        if (heads & 1u) {  // a new row starts at position base + a
          flush(gram, E, lane);
          row = __shfl_sync(0xFFFFFFFFu, my, a);
        }
        // run [a, b): up to the next head
        const uint32_t rest = heads >> 1;
        const int b = rest ? min(n, a + 1 + __ffs(rest) - 1) : n;
        V p4[KE][4];
#pragma unroll
        for (int k = 0; k < KE; ++k) p4[k][0] = p4[k][1] = p4[k][2] = p4[k][3] = V(0);
        int t = base + a;
        const int te = base + b;
        for (; t + 4 <= te; t += 4) {
          const V *d = dx + t * ldd;
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int k = 0; k < KE; ++k) p4[k][u] = fma(d[u * ldd + ei[k]], d[u * ldd + ej[k]], p4[k][u]);
        }
        for (; t < te; ++t) {
          const V *d = dx + t * ldd;
#pragma unroll
          for (int k = 0; k < KE; ++k) p4[k][0] = fma(d[ei[k]], d[ej[k]], p4[k][0]);
        }
#pragma unroll
        for (int k = 0; k < KE; ++k) part[k] += (p4[k][0] + p4[k][1]) + (p4[k][2] + p4[k][3]);
        merge();
        heads = b - a >= 32 ? 0u : (heads >> (b - a));
        a = b;
      }
    }
    }
  }
};

__host__ __device__ constexpr int gram_slots(int J) { return ((J + 1) * (J + 2) / 2 - 1 + 31) / 32; }

// Running Gram/RHS sums of one warp, register-blocked (the tensor-core forms):
// lane l owns 2 x 2 blocks (rb, cb), rb <= cb, of the (J+1) x (J+1) outer product
// of [delta, x] (features padded to an even count FP, the pad column zero), loads
// each operand pair with one 64-bit shared-memory load (the delta tile's row
// stride is even) and keeps four FP32 partial sums per block and run (4-way
// unrolled over the run's positions), merged with Neumaier compensation; runs of
// equal rows come from one ballot per 32 positions, a row change flushes the
// packed entries (i <= j, not (J, J)) with FP64 atomics.  Same sums as GramAcc's
// non-exact form, in a different association.
template <int J> struct GramBlk {
  static constexpr int FP = (J + 2) / 2 * 2;  // J + 1 features rounded up to even
  static constexpr int NB2 = FP / 2;
  static constexpr int NBLK = NB2 * (NB2 + 1) / 2;
  static constexpr int KB = (NBLK + 31) / 32;
  ProdSum<float> acc[KB][4];
  int orow[KB], ocol[KB];  // first feature of the block's row pair / column pair; -1: no block
  uint32_t row = 0xFFFFFFFFu;

  __device__ void init(int lane) {
#pragma unroll
    for (int k = 0; k < KB; ++k) {
      int b = lane + 32 * k, rb = 0;
      if (b < NBLK) {
        while (b >= NB2 - rb) {
          b -= NB2 - rb;
          ++rb;
        }
        orow[k] = 2 * rb;
        ocol[k] = 2 * (rb + b);
      } else {
        orow[k] = ocol[k] = -1;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[k][q] = ProdSum<float>();
    }
  }
  __device__ static int entry(int i, int j) { return i * (J + 1) - i * (i - 1) / 2 + (j - i); }
  __device__ void flush(double *gram, int E, int lane) {
    if (row != 0xFFFFFFFFu) {
#pragma unroll
      for (int k = 0; k < KB; ++k) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = orow[k] + (q >> 1), j = ocol[k] + (q & 1);
          if (orow[k] >= 0 && i <= j && j <= J && !(i == J && j == J))
            atomicAdd(gram + (size_t)row * E + entry(i, j), acc[k][q].value());
        }
      }
    }
#pragma unroll
    for (int k = 0; k < KB; ++k)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[k][q] = ProdSum<float>();
    (void)lane;
  }
  // tile positions [t0, t1) of the shared delta tile (row stride LDD, even; column J = x,
  // columns J+1 .. FP-1 zero)
  template <int LDD>
  __device__ void run(const float *dx, const uint32_t *rows, int t0, int t1, double *gram, int E, int lane) {
    static_assert(LDD % 2 == 0 && LDD >= FP, "64-bit pair loads");
    for (int base = t0; base < t1; base += 32) {
      const int n = min(32, t1 - base);
      const uint32_t my = lane < n ? rows[base + lane] : 0xFFFFFFFFu;
      const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, my, 1);
      const bool head = lane < n && (lane == 0 ? my != row : my != prev);
      uint32_t heads = __ballot_sync(0xFFFFFFFFu, head);
      int a = 0;
      while (a < n) {
        if (heads & 1u) {
          flush(gram, E, lane);
          row = __shfl_sync(0xFFFFFFFFu, my, a);
        }
        const uint32_t rest = heads >> 1;
        const int b = rest ? min(n, a + 1 + __ffs(rest) - 1) : n;
        float p[KB][4][2];
#pragma unroll
        for (int k = 0; k < KB; ++k)
#pragma unroll
          for (int q = 0; q < 4; ++q) p[k][q][0] = p[k][q][1] = 0.f;
        int t = base + a;
        const int te = base + b;
        for (; t + 2 <= te; t += 2) {
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const float *d = dx + (t + u) * LDD;
#pragma unroll
            for (int k = 0; k < KB; ++k) {
              const float2 r = *reinterpret_cast<const float2 *>(d + max(orow[k], 0));
              const float2 c = *reinterpret_cast<const float2 *>(d + max(ocol[k], 0));
              p[k][0][u] = fmaf(r.x, c.x, p[k][0][u]);
              p[k][1][u] = fmaf(r.x, c.y, p[k][1][u]);
              p[k][2][u] = fmaf(r.y, c.x, p[k][2][u]);
              p[k][3][u] = fmaf(r.y, c.y, p[k][3][u]);
            }
          }
        }
        for (; t < te; ++t) {
          const float *d = dx + t * LDD;
#pragma unroll
          for (int k = 0; k < KB; ++k) {
            const float2 r = *reinterpret_cast<const float2 *>(d + max(orow[k], 0));
            const float2 c = *reinterpret_cast<const float2 *>(d + max(ocol[k], 0));
            p[k][0][0] = fmaf(r.x, c.x, p[k][0][0]);
            p[k][1][0] = fmaf(r.x, c.y, p[k][1][0]);
            p[k][2][0] = fmaf(r.y, c.x, p[k][2][0]);
            p[k][3][0] = fmaf(r.y, c.y, p[k][3][0]);
          }
        }
#pragma unroll
        for (int k = 0; k < KB; ++k)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[k][q].add(p[k][q][0] + p[k][q][1]);
        heads = b - a >= 32 ? 0u : (heads >> (b - a));
        a = b;
      }
    }
  }
};

// GramMma's delta-row stride: 8, 24 or 40 floats (8 or 24 mod 32), so that the
// fragment loads of a warp (rows c, c + 4 of 8, columns g, g + 8, g + 16) hit 32
// distinct banks; GramMma::off gives the row offsets
__host__ __device__ constexpr int gram_mma_ldd(int J) { return J + 1 <= 8 ? 8 : J + 1 <= 16 ? 24 : 40; }

// One warp's Gram/RHS reduction of its 32 delta rows on the tensor cores, for
// J <= 16 (features f = [delta, x]).  For a run [a, b) of nonzeros of one row,
// G += F[:16, a:b] F[a:b] with mma.sync m16n8k8 (A = the first 16 features of
// F^T, masked to the run; B = F): a 16 x 8 NT block (NT = ceil((J+1)/8) 8-column
// n-tiles) holds the whole Gram/RHS triangle (row J = x is needed only at (J, J),
// which the Gram/RHS does not keep),
// per 8 nonzeros three MMAs per 8-column n-tile: the operands are split into TF32
// big + small parts (truncations: v = big + small + O(2^-20 |v|)) and the product
// taken as big*big + big*small + small*big, so the products stay within ~2^-19 of
// FP32's and the sums (FP32 in the MMA over at most 32 nonzeros) near FP32; runs fold
// into compensated FP32 sums and flush with FP64 atomics on a row change, like
// GramBlk.  (The 64/128-lane tcgen05 MMA has no 16-row form for this per-warp,
// per-row product.)  Lane (g = lane / 4, c = lane % 4) owns the accumulator entries
// (g [+8], 8 nt + 2c [+1]) of n-tile nt.
template <int J> struct GramMma {
  static constexpr int F = J + 1;
  static_assert(J <= 16, "delta in the 16 rows of one MMA block");
  static constexpr int NT = (F + 7) / 8;  // 8-column n-tiles
  static constexpr int LDD = gram_mma_ldd(J);
  static constexpr int COLS = 8 * NT;  // columns a row must hold (features, then zeros)
  static_assert(COLS + (LDD > 8 ? 4 : 0) <= LDD, "row stride");
  ProdSum<float> acc[NT][4];
  uint32_t row = 0xFFFFFFFFu;

  __device__ void init(int) {}
  __device__ static int entry(int i, int j) { return i * (J + 1) - i * (i - 1) / 2 + (j - i); }
  // v = big + small + O(2^-20 |v|), both exact TF32 values (low 13 bits zero)
  __device__ static void split(float v, uint32_t &big, uint32_t &small) {
    big = __float_as_uint(v) & 0xFFFFE000u;
    small = __float_as_uint(v - __uint_as_float(big)) & 0xFFFFE000u;  // the difference is exact
  }
  __device__ static void mma(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                             uint32_t b1) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  // Delta-tile layout: feature c of row r at r * LDD + c + pad(r), pad(r) = 4 for
  // rows with bit 2 set (LDD 24, 40; 0 at LDD 8, whose rows have no room).  A row
  // store (lane r writes its row as 16-byte chunks) then puts the 8 lanes of a
  // quarter-warp on 8 distinct 4-bank groups: (LDD r + pad(r)) mod 32 over
  // r = 0..7 is {0, 24, 16, 8, 4, 28, 20, 12} at LDD 24 and {0, 8, .., 24, 4, .., 28}
  // at LDD 40, where the plain stride repeats after 4 rows (a 2-way conflict).
  // The fragment loads stay conflict-free: rows k0 + c (k0 % 8 = 0, c < 4) have
  // no pad and rows k0 + c + 4 all have the same one.
  static constexpr int PAD = LDD > 8 ? 4 : 0;
  __host__ __device__ static constexpr int pad(int r) { return PAD * ((r >> 2) & 1); }
  __host__ __device__ static constexpr int off(int r, int c) { return r * LDD + c + pad(r); }
  // row r of the warp's delta tile dx: delta, x, zeros up to COLS (16-byte stores)
  __device__ static void store_row(float *dx, int r, const float (&delta)[J], float x) {
    float v[COLS];
#pragma unroll
    for (int k = 0; k < COLS; ++k) v[k] = k < J ? delta[k] : k == J ? x : 0.f;
    float *row = dx + off(r, 0);
#pragma unroll
    for (int k = 0; k < COLS; k += 4) *reinterpret_cast<float4 *>(row + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
  }
  __device__ void flush(double *gram, int E, int lane) {
    if (row != 0xFFFFFFFFu) {
      const int g = lane >> 2, c = lane & 3;
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = g + 8 * (q >> 1), j = 8 * nt + 2 * c + (q & 1);
          if (i <= j && j <= J && !(i == J && j == J)) atomicAdd(gram + (size_t)row * E + entry(i, j), acc[nt][q].value());
        }
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[nt][q] = ProdSum<float>();
  }
  // rows k0 .. k0 + 7 of the delta tile, restricted (MASK) to the run [a, b)
  template <bool MASK>
  __device__ static void kstep(float (&d)[NT][4], const float *dx, int k0, int a, int b, int g, int c) {
    const float *r0 = dx + (k0 + c) * LDD + g, *r1 = dx + (k0 + c + 4) * LDD + PAD + g;
    uint32_t h0, l0, h2, l2, h1 = 0, l1 = 0, h3 = 0, l3 = 0, h4 = 0, l4 = 0, h5 = 0, l5 = 0;
    split(r0[0], h0, l0);
    split(r1[0], h2, l2);
    if (NT > 1) {
      split(r0[8], h1, l1);
      split(r1[8], h3, l3);
    }
    if (NT > 2) {  // columns 16 .. 23 (B only)
      split(r0[16], h4, l4);
      split(r1[16], h5, l5);
    }
    // A = F^T of the run's nonzeros only; B = F (its other rows meet zeros of A)
    uint32_t ah0 = h0, ah1 = h1, ah2 = h2, ah3 = h3, al0 = l0, al1 = l1, al2 = l2, al3 = l3;
    if (MASK) {
      const bool in0 = (unsigned)(k0 + c - a) < (unsigned)(b - a), in1 = (unsigned)(k0 + c + 4 - a) < (unsigned)(b - a);
      ah0 = in0 ? h0 : 0u, ah1 = in0 ? h1 : 0u, al0 = in0 ? l0 : 0u, al1 = in0 ? l1 : 0u;
      ah2 = in1 ? h2 : 0u, ah3 = in1 ? h3 : 0u, al2 = in1 ? l2 : 0u, al3 = in1 ? l3 : 0u;
    }
    mma(d[0], ah0, ah1, ah2, ah3, h0, h2);
    mma(d[0], ah0, ah1, ah2, ah3, l0, l2);
    mma(d[0], al0, al1, al2, al3, h0, h2);
    if (NT > 1) {
      mma(d[1 % NT], ah0, ah1, ah2, ah3, h1, h3);
      mma(d[1 % NT], ah0, ah1, ah2, ah3, l1, l3);
      mma(d[1 % NT], al0, al1, al2, al3, h1, h3);
    }
    if (NT > 2) {
      mma(d[2 % NT], ah0, ah1, ah2, ah3, h4, h5);
      mma(d[2 % NT], ah0, ah1, ah2, ah3, l4, l5);
      mma(d[2 % NT], al0, al1, al2, al3, h4, h5);
    }
  }
  // rows [0, n) of this warp's delta tile (row stride LDD) with their tensor rows
  __device__ void run(const float *dx, const uint32_t *rows, int n, double *gram, int E, int lane) {
    const int g = lane >> 2, c = lane & 3;
    const uint32_t my = lane < n ? rows[lane] : 0xFFFFFFFFu;
    const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, my, 1);
    const bool head = lane < n && (lane == 0 ? my != row : my != prev);
    uint32_t heads = __ballot_sync(0xFFFFFFFFu, head);
    int a = 0;
    while (a < n) {
      if (heads & 1u) {
        flush(gram, E, lane);
        row = __shfl_sync(0xFFFFFFFFu, my, a);
      }
      const uint32_t rest = heads >> 1;
      const int b = rest ? min(n, a + __ffs(rest)) : n;
      float d[NT][4];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) d[nt][q] = 0.f;
      if (b - a == 32) {  // the warp's 32 nonzeros are one row: no masking
#pragma unroll
        for (int k0 = 0; k0 < 32; k0 += 8) kstep<false>(d, dx, k0, 0, 32, g, c);
      } else {
        for (int k0 = a & ~7; k0 < b; k0 += 8) kstep<true>(d, dx, k0, a, b, g, c);
      }
      if (b < n) {  // the row ends inside this warp's nonzeros: one plain add before its flush
#pragma unroll
        for (int nt = 0; nt < NT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[nt][q].s += d[nt][q];
      } else {      // the row may go on for many tiles: compensated
#pragma unroll
        for (int nt = 0; nt < NT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[nt][q].add(d[nt][q]);
      }
      heads = b - a >= 32 ? 0u : (heads >> (b - a));
      a = b;
    }
  }
};

__device__ inline double block_sum(double v) {
  __shared__ double sw[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  if (lane == 0) sw[warp] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sw[w];
  __syncthreads();
  return s;  // valid in thread 0
}


// odd stride (conflict-free column writes) with a spare zero column at J + 1
inline int ldd_for(int J) { return ((J + 2) & 1) ? J + 2 : J + 3; }
inline int pairs_for(int J) { return (J + 1) * (J + 2) / 2 - 1; }

}  // namespace
}  // namespace gtk
