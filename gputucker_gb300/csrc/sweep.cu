// sweep.cu -- the ALS mode update and the fit on the GPU (plain value_t form).
//
// Reference path being replaced (paths inside the GPUTucker project):
//   delta ......... computing_delta_kernel, delta.cuh:33-92.  Per nonzero x at
//                   (i_1..i_N): delta_j = sum over core entries g with g_n = j of
//                   G[g] * prod_{k != n} A_k[i_k, g_k] (J^N terms, summed in core order)
//   B, C .......... ComputingBC, update.cuh:35-101 (host, OpenMP, double):
//                   B_r = lambda*I + sum delta delta^T, C_r = sum x*delta over row r
//   row solve ..... update.cuh:163-194 (host, Eigen inverse): a_r = C_r^T B_r^-1
//   fit ........... ComputingReconstructionKernel reconstruction.cuh:32-83 and the
//                   error loop :259-276
//
// GB300 design:
//   * The tensor is HBM-resident; mode n runs over the mode-n view (nonzeros
//     stably sorted by global row i_n), so one factor row's nonzeros are
//     contiguous.
//   * One fused kernel per mode: a CTA takes a tile of 256*NPT consecutive
//     nonzeros, gathers the other modes' factor rows (L2-resident), contracts
//     the mode-n-first permuted core G_n (in shared memory, broadcast reads)
//     level by level -- J^N + J^(N-1) + ... + J^2 multiply-adds per nonzero
//     instead of the reference's (N-1) J^N -- writes delta and x to a shared
//     tile, and reduces delta delta^T (upper triangle) and x*delta per row
//     segment of the tile.  delta never reaches HBM.  Rows wholly inside a tile
//     are stored, rows cut by a tile edge are added with FP64 atomics.
//   * One warp per row solves (lambda I + Gram) a = C by Cholesky in FP64.
//   * The fit reuses the fused kernel on the last mode's view: x_hat =
//     delta^(N-1) . a_{N-1}[i_{N-1}], error (x - x_hat)^2 summed in FP64 per
//     CTA and then in a fixed order.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "internal.h"
#include "mode_common.cuh"

namespace gtk {
namespace {

// ---------------------------------------------------------------- contraction nest
// Nest<D> contracts D other modes.  g: the core sub-block for the current outer
// indices, J^(D-1) rows of LDG values.  The two innermost levels use factor rows
// held in registers (a1: second-to-last other mode, a2: last); outer levels read
// their factor rows from shared memory (arow, element (q, j) at arow[(q*J+j)*kThreads]).
template <class V, int J, int LDG, int NPT, int D> struct Nest {
  static __device__ __forceinline__ void run(const V *__restrict__ g, const V *arow, int lvl_stride,
                                             const V (&a1)[NPT][J], const V (&a2)[NPT][J], V (&out)[NPT]) {
#pragma unroll
    for (int q = 0; q < NPT; ++q) out[q] = V(0);
#pragma unroll 1
    for (int j = 0; j < J; ++j) {
      V sub[NPT];
      Nest<V, J, LDG, NPT, D - 1>::run(g + (size_t)j * Pow<J, D - 2>::v * LDG, arow + lvl_stride, lvl_stride, a1, a2,
                                       sub);
#pragma unroll
      for (int q = 0; q < NPT; ++q) out[q] += arow[(q * J + j) * kThreads] * sub[q];
    }
  }
};

template <class V, int J, int LDG, int NPT> struct Nest<V, J, LDG, NPT, 2> {
  static __device__ __forceinline__ void run(const V *__restrict__ g, const V *, int, const V (&a1)[NPT][J],
                                             const V (&a2)[NPT][J], V (&out)[NPT]) {
    using VT = typename Vec<V>::T;
    constexpr int W = Vec<V>::W;
#pragma unroll
    for (int q = 0; q < NPT; ++q) out[q] = V(0);
#pragma unroll
    for (int j1 = 0; j1 < J; ++j1) {
      V d[NPT];
#pragma unroll
      for (int q = 0; q < NPT; ++q) d[q] = V(0);
      const VT *row = reinterpret_cast<const VT *>(g + j1 * LDG);
#pragma unroll
      for (int c = 0; c < LDG / W; ++c) {
        V gv[W];
        Vec<V>::unpack(row[c], gv);
#pragma unroll
        for (int k = 0; k < W; ++k) {
          if (c * W + k < J) {
#pragma unroll
            for (int q = 0; q < NPT; ++q) d[q] += gv[k] * a2[q][c * W + k];
          }
        }
      }
#pragma unroll
      for (int q = 0; q < NPT; ++q) out[q] += a1[q][j1] * d[q];
    }
  }
};


// ---------------------------------------------------------------- core streaming
// 16-byte asynchronous global->shared copies (cp.async, completion by groups)
__device__ __forceinline__ void cp_async16(void *sdst, const void *gsrc) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Cores too large for shared memory (J^(N-1) * LDG values above ~200 KB) are
// streamed: chunk c is J^2 rows of LDG values -- for N = 4 the slice of one
// mode-n index jn, for N = 5 the slice of one (jn, first other index) pair -- the
// input of one Nest<3>.  Two chunk buffers; chunk c+1 is in flight while chunk c
// is contracted.
template <int N, int J, int LDG> struct CoreStream {
  static constexpr int NC = N == 4 ? J : J * J;       // chunks per pass over the core (N = 4 or 5)
  static constexpr size_t CH = (size_t)J * J * LDG;  // values per chunk
};

// ---------------------------------------------------------------- specialised kernel
// Compile-time order N and rank J; NPT nonzeros per thread share every core read.
// STREAM: the core is streamed through shared memory in chunks (CoreStream).
template <class V, int N, int J, int NPT, int KIND, bool STREAM>
__device__ __forceinline__ void mode_spec_body(const ModeArgs &a, uint32_t cta, uint32_t nctas) {
  using VT = typename Vec<V>::T;
  constexpr int W = Vec<V>::W;
  constexpr int LDG = (J + W - 1) / W * W;  // equals the factor row stride ldf
  constexpr int D = N - 1;                 // other modes
  constexpr int LEV = D > 2 ? D - 2 : 0;   // outer levels with factor rows in shared memory
  constexpr int TN = kThreads * NPT;
  using CS = CoreStream<N, J, LDG>;
  static_assert(!STREAM || D == 3 || D == 4, "streamed core: N = 4 or 5");
  static_assert(!STREAM || (CS::CH * sizeof(V)) % 16 == 0, "chunks move in 16-byte pieces");
  constexpr size_t GP = STREAM ? 2 * CS::CH : (size_t)Pow<J, N - 1>::v * LDG;
  extern __shared__ __align__(16) unsigned char smem[];
  const TileSmem<V> s = carve<V>(smem, GP, LEV, NPT, J, a.ldd, a.E, TN);
  const int tid = threadIdx.x;
  if (!STREAM) {
    const VT *src = reinterpret_cast<const VT *>(a.corep);
    VT *dst = reinterpret_cast<VT *>(s.gp);
    for (size_t k = tid; k < GP / W; k += kThreads) dst[k] = src[k];
  }
  if (KIND == kUpdate) fill_pairs(s.pi, s.pj, J);
  const int lvl_stride = NPT * J * kThreads;
  const V *facn = reinterpret_cast<const V *>(a.fac[a.mode]);
  double err = 0;
  GramAcc<V, gram_slots(J), true> gram;
  for (int k = tid; k < TN; k += kThreads) s.dx[k * a.ldd + J + 1] = V(0);
  __syncthreads();
  if (KIND == kUpdate) gram.init(s.pi, s.pj, a.E, J + 1, tid & 31);
  // a contiguous range of tiles per CTA, so a warp's running Gram sums follow a row across tiles
  const uint64_t ntiles = (a.nnz + TN - 1) / TN;
  const uint64_t per = (ntiles + nctas - 1) / nctas;
  const uint64_t tile_end = min(ntiles, (uint64_t)(cta + 1) * per);
  for (uint64_t tile = (uint64_t)cta * per; tile < tile_end; ++tile) {
    __syncthreads();  // previous tile's reduction is done with the shared tile
    const uint64_t t0 = tile * TN;
    const int nv = (int)min((uint64_t)TN, a.nnz - t0);
    V a1[NPT][J], a2[NPT][J];
    V xv[NPT];
    uint32_t rowv[NPT];
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const int tl = q * kThreads + tid;
      const bool valid = tl < nv;
      const uint64_t gi = valid ? t0 + tl : t0;
      rowv[q] = valid ? a.coord[a.mode][gi] : 0xFFFFFFFFu;
      xv[q] = valid ? reinterpret_cast<const V *>(a.val)[gi] : V(0);
#pragma unroll
      for (int l = 0; l < D; ++l) {
        const int o = a.others[l];
        const uint32_t r = a.coord[o][gi];
        const VT *frow = reinterpret_cast<const VT *>(reinterpret_cast<const V *>(a.fac[o]) + (size_t)r * LDG);
        V tmp[LDG];
#pragma unroll
        for (int c = 0; c < LDG / W; ++c) Vec<V>::unpack(__ldg(frow + c), tmp + c * W);
        if (l == D - 2) {
#pragma unroll
          for (int j = 0; j < J; ++j) a1[q][j] = tmp[j];
        } else if (l == D - 1) {
#pragma unroll
          for (int j = 0; j < J; ++j) a2[q][j] = tmp[j];
        } else {
#pragma unroll
          for (int j = 0; j < J; ++j) s.arow[l * lvl_stride + (q * J + j) * kThreads + tid] = tmp[j];
        }
      }
    }
    V xhat[NPT];
#pragma unroll
    for (int q = 0; q < NPT; ++q) xhat[q] = V(0);
    // delta_jn of the thread's nonzeros is o: store / use it
    auto finish = [&](int jn, const V (&o)[NPT]) {
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int tl = q * kThreads + tid;
        if (KIND == kUpdate) {
          s.dx[tl * a.ldd + jn] = o[q];
        } else if (KIND == kFit) {
          if (tl < nv) xhat[q] += o[q] * __ldg(facn + (size_t)rowv[q] * LDG + jn);
        } else {
          if (tl < nv) reinterpret_cast<V *>(a.out)[(size_t)a.vperm[t0 + tl] * J + jn] = o[q];
        }
      }
    };
    if constexpr (!STREAM) {
#pragma unroll 1
      for (int jn = 0; jn < J; ++jn) {
        V o[NPT];
        Nest<V, J, LDG, NPT, D>::run(s.gp + (size_t)jn * Pow<J, N - 2>::v * LDG, s.arow + tid, lvl_stride, a1, a2,
                                     o);
        finish(jn, o);
      }
    } else {
      const V *core = reinterpret_cast<const V *>(a.corep);
      auto issue = [&](int c) {
        const char *src = reinterpret_cast<const char *>(core + (size_t)c * CS::CH);
        char *dst = reinterpret_cast<char *>(s.gp + (size_t)(c & 1) * CS::CH);
        constexpr int P16 = (int)(CS::CH * sizeof(V) / 16);
        for (int k = tid; k < P16; k += kThreads) cp_async16(dst + 16 * k, src + 16 * k);
      };
      issue(0);
      cp_async_commit();
      V o[NPT];
#pragma unroll
      for (int q = 0; q < NPT; ++q) o[q] = V(0);
#pragma unroll 1
      for (int c = 0; c < CS::NC; ++c) {
        if (c + 1 < CS::NC) issue(c + 1);
        cp_async_commit();  // possibly empty: the group count stays one ahead
        cp_async_wait1();   // chunk c has landed (this thread's copies)
        __syncthreads();    // ... and every thread's
        const V *g = s.gp + (size_t)(c & 1) * CS::CH;
        if constexpr (D == 3) {
          Nest<V, J, LDG, NPT, 3>::run(g, s.arow + tid, lvl_stride, a1, a2, o);
          finish(c, o);
        } else {
          const int j0 = c % J;
          V sub[NPT];
          Nest<V, J, LDG, NPT, 3>::run(g, s.arow + tid + lvl_stride, lvl_stride, a1, a2, sub);
#pragma unroll
          for (int q = 0; q < NPT; ++q) o[q] += s.arow[(q * J + j0) * kThreads + tid] * sub[q];
          if (j0 == J - 1) {
            finish(c / J, o);
#pragma unroll
            for (int q = 0; q < NPT; ++q) o[q] = V(0);
          }
        }
        __syncthreads();  // chunk buffer c & 1 is refilled by the issue of chunk c + 2
      }
    }
    if (KIND == kUpdate) {
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int tl = q * kThreads + tid;
        s.dx[tl * a.ldd + J] = xv[q];
        s.rows[tl] = rowv[q];
      }
      __syncthreads();
      if (a.dstore) {  // the tile's delta rows, contiguous in view order
        V *dst = reinterpret_cast<V *>(a.dstore) + t0 * J;
        for (int k = tid; k < nv * J; k += kThreads) dst[k] = s.dx[(k / J) * a.ldd + (k % J)];
      }
      // warp w reduces tile positions [w*TN/8, (w+1)*TN/8)
      constexpr int R = TN / (kThreads / 32);
      const int w0 = (tid >> 5) * R;
      gram.run(s.dx, a.ldd, s.rows, w0, min(w0 + R, nv), a.gram, a.E, tid & 31);
    } else if (KIND == kFit) {
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        if (q * kThreads + tid < nv) {
          const V d = xv[q] - xhat[q];
          err += (double)d * (double)d;
        }
      }
    }
  }
  if (KIND == kUpdate) gram.flush(a.gram, a.E, tid & 31);
  if (KIND == kFit) {
    const double tot = block_sum(err);
    if (tid == 0) a.partial[cta] = tot;
  }
}

template <class V, int N, int J, int NPT, int KIND, bool STREAM = false>
__global__ void __launch_bounds__(kThreads) k_mode_spec(ModeArgs a) {
  mode_spec_body<V, N, J, NPT, KIND, STREAM>(a, blockIdx.x, gridDim.x);
}

// Many tensors of one shape class in one launch (batches): CTA b works for
// tensor i with cta_first[i] <= b < cta_first[i + 1], on that tensor's tiles
template <class V, int N, int J, int NPT, int KIND, bool STREAM = false>
__global__ void __launch_bounds__(kThreads) k_mode_spec_multi(const __grid_constant__ MultiParams p) {
  __shared__ ModeArgs sa;
  uint32_t cta, nctas;
  const ModeArgs &a = multi_select(p, sa, cta, nctas);
  mode_spec_body<V, N, J, NPT, KIND, STREAM>(a, cta, nctas);
}

// ---------------------------------------------------------------- generic kernel
// Any order N (1..8) and rank J (1..64); one nonzero per thread; the core is read
// from shared memory when it fits, else from global memory (L1/L2).  delta_jn =
// sum over rows r of G_n[jn][r][:] . a_last * prod of the outer factor entries.
template <class V, int KIND>
__global__ void __launch_bounds__(kThreads) k_mode_gen(ModeArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const size_t gp_sm = a.gp_in_smem ? a.gp_elems : 0;
  const TileSmem<V> s = carve<V>(smem, gp_sm, 0, 1, a.J, a.ldd, a.E, kThreads);
  const int tid = threadIdx.x;
  const int J = a.J, ldf = a.ldf, M = a.N - 1;
  const V *gp = reinterpret_cast<const V *>(a.corep);
  if (a.gp_in_smem) {
    for (size_t k = tid; k < a.gp_elems; k += kThreads) s.gp[k] = gp[k];
    gp = s.gp;
  }
  if (KIND == kUpdate) fill_pairs(s.pi, s.pj, J);
  uint64_t rows_per = 1;
  for (int k = 0; k < M - 1; ++k) rows_per *= (uint64_t)J;
  const V *facn = reinterpret_cast<const V *>(a.fac[a.mode]);
  double err = 0;
  const uint64_t ntiles = (a.nnz + kThreads - 1) / kThreads;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    __syncthreads();
    const uint64_t t0 = tile * kThreads;
    const int nv = (int)min((uint64_t)kThreads, a.nnz - t0);
    const bool valid = tid < nv;
    const uint64_t gi = valid ? t0 + tid : t0;
    const uint32_t row = valid ? a.coord[a.mode][gi] : 0xFFFFFFFFu;
    const V x = valid ? reinterpret_cast<const V *>(a.val)[gi] : V(0);
    const V *ap[kMaxOrder];
    for (int k = 0; k < M; ++k) {
      const int o = a.others[k];
      ap[k] = reinterpret_cast<const V *>(a.fac[o]) + (size_t)a.coord[o][gi] * ldf;
    }
    V xhat = V(0);
    if (a.ref_order) {
      // computing_delta_kernel (delta.cuh:62-90): over the core entries i in linear
      // order, beta = G_i * A_k[x_k][g_k(i)] for k = 0..N-1 skipping the mode, each
      // product rounded, then tmp[g_mode(i)] += beta -- the same roundings in the
      // same order, so FP32 delta is bit-identical to the reference's
      V tmp[kMaxRank];
      for (int j = 0; j < J; ++j) tmp[j] = V(0);
      const V *G = reinterpret_cast<const V *>(a.core);
      const V *fk[kMaxOrder];
      for (int k = 0; k < a.N; ++k)
        fk[k] = reinterpret_cast<const V *>(a.fac[k]) + (size_t)(valid ? a.coord[k][gi] : 0) * ldf;
      int dig[kMaxOrder];
      for (int k = 0; k < a.N; ++k) dig[k] = 0;
      uint64_t ncore = 1;
      for (int k = 0; k < a.N; ++k) ncore *= (uint64_t)J;
      for (uint64_t i = 0; i < ncore; ++i) {
        V beta = G[i];
        for (int k = 0; k < a.N; ++k)
          if (k != a.mode) beta = mul_rn(beta, fk[k][dig[k]]);
        tmp[dig[a.mode]] = add_rn(tmp[dig[a.mode]], beta);
        for (int k = a.N - 1; k >= 0; --k) {  // last mode fastest
          if (++dig[k] < J) break;
          dig[k] = 0;
        }
      }
      for (int jn = 0; jn < J; ++jn) {
        if (KIND == kUpdate) {
          s.dx[tid * a.ldd + jn] = tmp[jn];
        } else if (KIND == kFit) {
          if (valid) xhat += tmp[jn] * facn[(size_t)row * ldf + jn];
        } else {
          if (valid) reinterpret_cast<V *>(a.out)[(size_t)a.vperm[gi] * J + jn] = tmp[jn];
        }
      }
    }
    for (int jn = 0; jn < J && !a.ref_order; ++jn) {
      V acc = V(0);
      if (M == 0) {
        acc = gp[jn];
      } else {
        int dig[kMaxOrder];
        for (int k = 0; k < M; ++k) dig[k] = 0;
        const V *alast = ap[M - 1];
        for (uint64_t r = 0; r < rows_per; ++r) {
          V pp = V(1);
          for (int k = 0; k < M - 1; ++k) pp *= ap[k][dig[k]];
          const V *grow = gp + ((size_t)jn * rows_per + r) * ldf;
          V dot = V(0);
          for (int c = 0; c < J; ++c) dot += grow[c] * alast[c];
          acc += pp * dot;
          for (int k = M - 2; k >= 0; --k) {
            if (++dig[k] < J) break;
            dig[k] = 0;
          }
        }
      }
      if (KIND == kUpdate) {
        s.dx[tid * a.ldd + jn] = acc;
      } else if (KIND == kFit) {
        if (valid) xhat += acc * facn[(size_t)row * ldf + jn];
      } else {
        if (valid) reinterpret_cast<V *>(a.out)[(size_t)a.vperm[gi] * J + jn] = acc;
      }
    }
    if (KIND == kUpdate) {
      s.dx[tid * a.ldd + J] = x;
      s.rows[tid] = row;
      __syncthreads();
      if (a.dstore) {
        V *dst = reinterpret_cast<V *>(a.dstore) + t0 * J;
        for (int k = tid; k < nv * J; k += kThreads) dst[k] = s.dx[(k / J) * a.ldd + (k % J)];
      }
      gram_phase<V>(a, s, t0, nv, 1);
    } else if (KIND == kFit) {
      if (valid) {
        const V d = x - xhat;
        err += (double)d * (double)d;
      }
    }
  }
  if (KIND == kFit) {
    const double tot = block_sum(err);
    if (tid == 0) a.partial[blockIdx.x] = tot;
  }
}

// ---------------------------------------------------------------- row solves
// A = lambda I + Gram (FP64), right-hand side C; a = A^-1 C overwrites the
// factor row (cast to value_t), as update.cuh:163-194 does with Eigen's inverse.
//
// k_solve_rows: one thread per row.  The packed row (upper triangle + C, the
// layout the Gram kernels accumulate) is copied to the thread's slice of shared
// memory (element e of thread t at [e * blockDim + t], conflict-free) and
// factored in place by upper Cholesky A = U^T U, then U^T y = C, U a = y.  GB300
// issues FP64 at ~1/64 of FP32, so every lane works on its own row.  A row
// whose pivot rounds to <= 0 (rows with fewer nonzeros than J after
// ill-conditioned updates) is appended to a list and re-solved by
// k_solve_lu_rows with LU and partial pivoting -- the method of the reference's
// Eigen inverse (update.cuh:180) -- so the sweep never stops there either.

__device__ __forceinline__ int upk(int i, int j, int J) {  // packed index of (i, j), i <= j <= J
  return i * (J + 1) - (i * (i - 1)) / 2 + (j - i);
}

// FP64 Cholesky of lambda I + Gram of one row, in the thread-interleaved shared
// scratch A (element e at A[e * T]); the solution into the factor row, or the
// row onto the pivoted-LU list when a pivot is not positive
template <class V>
__device__ __forceinline__ void solve_row64(const double *__restrict__ gram, uint64_t row, int J, int E, int ldf,
                                            V *__restrict__ fac, double lambda, double *A, int T,
                                            uint32_t *__restrict__ fallback, unsigned int *__restrict__ nfallback) {
  const double *g = gram + row * (uint64_t)E;
  for (int e = 0; e < E; ++e) A[e * T] = g[e];
  for (int i = 0; i < J; ++i) A[upk(i, i, J) * T] += lambda;
  bool ok = true;
  for (int k = 0; k < J && ok; ++k) {
    const double d = A[upk(k, k, J) * T];
    if (!(d > 0.0) || !isfinite(d)) {
      ok = false;
      break;
    }
    const double u = sqrt(d), r = 1.0 / u;
    A[upk(k, k, J) * T] = u;
    for (int j = k + 1; j <= J; ++j) A[upk(k, j, J) * T] *= r;  // row k of U, and C_k / u_kk
    for (int i = k + 1; i < J; ++i) {
      const double uki = A[upk(k, i, J) * T];
      for (int j = i; j <= J; ++j) A[upk(i, j, J) * T] -= uki * A[upk(k, j, J) * T];
    }
  }
  // the elimination above also carried C through U^T y = C: column J now holds y
  V *frow = fac + row * (uint64_t)ldf;
  if (ok) {
    for (int k = J - 1; k >= 0; --k) {
      double v = A[upk(k, J, J) * T];
      for (int j = k + 1; j < J; ++j) v -= A[upk(k, j, J) * T] * A[upk(j, J, J) * T];
      v /= A[upk(k, k, J) * T];
      A[upk(k, J, J) * T] = v;
    }
    for (int j = 0; j < ldf; ++j) frow[j] = j < J ? (V)A[upk(j, J, J) * T] : V(0);
  } else {
    fallback[atomicAdd(nfallback, 1u)] = (uint32_t)row;
    atomicAdd(nfallback + 3, 1u);  // running count of the handle (gtk_solve_counters)
  }
}

// list_in == nullptr: rows 0..rows-1; else the *nlist_in rows listed
template <class V>
__global__ void k_solve_rows(const double *__restrict__ gram, uint64_t rows, const uint32_t *__restrict__ list_in,
                             const unsigned int *__restrict__ nlist_in, int J, int E, int ldf, V *__restrict__ fac,
                             double lambda, uint32_t *__restrict__ fallback, unsigned int *__restrict__ nfallback) {
  extern __shared__ double sm[];
  const int T = blockDim.x, tid = threadIdx.x;
  const uint64_t n = list_in ? (uint64_t)*nlist_in : rows;
  for (uint64_t k0 = (uint64_t)blockIdx.x * T + tid; k0 < n; k0 += (uint64_t)gridDim.x * T)
    solve_row64<V>(gram, list_in ? list_in[k0] : k0, J, E, ldf, fac, lambda, sm + tid, T, fallback, nfallback);
}

// The precision form's row solve: FP32 Cholesky per thread (GB300 runs FP32 at
// ~64x its FP64 rate), a 1-norm condition estimate kappa_1 = ||B||_1 est(||B^-1||_1)
// from the factor (Hager's method as refined by Higham, the estimator of
// LAPACK's xPOCON: at most three rounds of two solves with U^T U), and one step
// of iterative refinement whose residual
// r = C - (lambda I + G) a is formed from the FP64 Gram with each entry split
// into two floats, error-free products (fmaf) and Neumaier sums.  Rows with
// kappa above cond_max, or a non-positive pivot, go to the FP64 solver.
__device__ __forceinline__ void neu_add(float &s, float &c, float x) {
  const float t = s + x;
  c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
  s = t;
}

// y <- (U^T U)^-1 y in place (U packed at U[e * T], vectors strided by T)
__device__ __forceinline__ void chol_solve32(const float *U, float *y, int J, int T) {
  for (int k = 0; k < J; ++k) {  // U^T z = y
    float v = y[k * T];
    for (int p = 0; p < k; ++p) v -= U[upk(p, k, J) * T] * y[p * T];
    y[k * T] = v / U[upk(k, k, J) * T];
  }
  for (int k = J - 1; k >= 0; --k) {  // U w = z
    float v = y[k * T];
    for (int j = k + 1; j < J; ++j) v -= U[upk(k, j, J) * T] * y[j * T];
    y[k * T] = v / U[upk(k, k, J) * T];
  }
}

// Hager/Higham estimate of ||B^-1||_1 for SPD B = U^T U: a lower bound, in
// practice within a small factor (x, y: J-vector scratch strided by T)
__device__ float inv_norm1_est(const float *U, float *x, float *y, int J, int T) {
  for (int i = 0; i < J; ++i) x[i * T] = 1.f / (float)J;
  float est = 0.f;
  for (int it = 0; it < 3; ++it) {
    for (int i = 0; i < J; ++i) y[i * T] = x[i * T];
    chol_solve32(U, y, J, T);
    float n1 = 0.f;
    for (int i = 0; i < J; ++i) n1 += fabsf(y[i * T]);
    if (it > 0 && n1 <= est) break;
    est = n1;
    float zx = 0.f;  // z = B^-1 sign(y) (B symmetric), z . x, argmax |z|
    for (int i = 0; i < J; ++i) y[i * T] = y[i * T] >= 0.f ? 1.f : -1.f;
    chol_solve32(U, y, J, T);
    int jmax = 0;
    float zmax = -1.f;
    for (int i = 0; i < J; ++i) {
      zx += y[i * T] * x[i * T];
      if (fabsf(y[i * T]) > zmax) {
        zmax = fabsf(y[i * T]);
        jmax = i;
      }
    }
    if (it > 0 && zmax <= zx) break;
    for (int i = 0; i < J; ++i) x[i * T] = i == jmax ? 1.f : 0.f;
  }
  return est;
}

// FP32 Cholesky + condition estimate + one refinement step of one row (scratch
// sf: (E + 3J) floats, thread-interleaved); rows above cond_max, or with a
// non-positive pivot, onto the FP64 list
template <class V>
__device__ __forceinline__ void solve_row32(const double *__restrict__ gram, uint64_t row, int J, int E, int ldf,
                                            V *__restrict__ fac, double lambda, float cond_max, float *sf, int T,
                                            uint32_t *__restrict__ to_fp64, unsigned int *__restrict__ n_to_fp64) {
  float *U = sf;                          // packed factor, element e at U[e * T]
  float *r = sf + (size_t)E * T;          // residual / correction, element i at r[i * T]
  float *w = sf + (size_t)(E + J) * T;    // estimator scratch: two J-vectors
  const float lam = (float)lambda;
  const double *g = gram + row * (uint64_t)E;
  for (int e = 0; e < E; ++e) U[e * T] = (float)g[e];
  for (int i = 0; i < J; ++i) U[upk(i, i, J) * T] = (float)(g[upk(i, i, J)] + lambda);
  // ||B||_1 (B symmetric: the largest absolute row sum), from the FP64 Gram
  float bnorm1 = 0.f;
  for (int i = 0; i < J; ++i) {
    double rs = 0;
    for (int j = 0; j < J; ++j) rs += fabs(g[i <= j ? upk(i, j, J) : upk(j, i, J)]);
    bnorm1 = fmaxf(bnorm1, (float)(rs + lambda));
  }
  bool ok = true;
  for (int k = 0; k < J; ++k) {
    const float d = U[upk(k, k, J) * T];
    if (!(d > 0.f) || !isfinite(d)) {
      ok = false;
      break;
    }
    const float u = sqrtf(d), ru = 1.f / u;
    U[upk(k, k, J) * T] = u;
    for (int j = k + 1; j <= J; ++j) U[upk(k, j, J) * T] *= ru;
    for (int i = k + 1; i < J; ++i) {
      const float uki = U[upk(k, i, J) * T];
      for (int j = i; j <= J; ++j) U[upk(i, j, J) * T] -= uki * U[upk(k, j, J) * T];
    }
  }
  const float kappa = ok ? bnorm1 * inv_norm1_est(U, w, w + (size_t)J * T, J, T) : 0.f;
  if (!ok || !(kappa <= cond_max)) {
    to_fp64[atomicAdd(n_to_fp64, 1u)] = (uint32_t)row;
    atomicAdd(n_to_fp64 + 1, 1u);  // running count of the handle (gtk_solve_counters)
    return;
  }
  for (int k = J - 1; k >= 0; --k) {  // U a = y, a kept in column J
    float v = U[upk(k, J, J) * T];
    for (int j = k + 1; j < J; ++j) v -= U[upk(k, j, J) * T] * U[upk(j, J, J) * T];
    U[upk(k, J, J) * T] = v / U[upk(k, k, J) * T];
  }
  // r = C - lambda a - G a, compensated
  for (int i = 0; i < J; ++i) {
    float s = 0.f, c = 0.f;
    const double ci = g[upk(i, J, J)];
    const float ch = (float)ci;
    neu_add(s, c, ch);
    neu_add(s, c, (float)(ci - (double)ch));
    const float ai = U[upk(i, J, J) * T];
    neu_add(s, c, -lam * ai);
    for (int j = 0; j < J; ++j) {
      const double gij = g[i <= j ? upk(i, j, J) : upk(j, i, J)];
      const float gh = (float)gij, gl = (float)(gij - (double)gh);
      const float aj = U[upk(j, J, J) * T];
      const float ph = gh * aj;
      const float pl = fmaf(gh, aj, -ph);
      neu_add(s, c, -ph);
      neu_add(s, c, -(pl + gl * aj));
    }
    r[i * T] = s + c;
  }
  for (int k = 0; k < J; ++k) {  // U^T z = r
    float v = r[k * T];
    for (int p = 0; p < k; ++p) v -= U[upk(p, k, J) * T] * r[p * T];
    r[k * T] = v / U[upk(k, k, J) * T];
  }
  for (int k = J - 1; k >= 0; --k) {  // U d = z
    float v = r[k * T];
    for (int j = k + 1; j < J; ++j) v -= U[upk(k, j, J) * T] * r[j * T];
    r[k * T] = v / U[upk(k, k, J) * T];
  }
  V *frow = fac + row * (uint64_t)ldf;
  for (int j = 0; j < ldf; ++j) frow[j] = j < J ? (V)(U[upk(j, J, J) * T] + r[j * T]) : V(0);
}

template <class V>
__global__ void k_solve_rows32(const double *__restrict__ gram, uint64_t rows, int J, int E, int ldf,
                               V *__restrict__ fac, double lambda, float cond_max, uint32_t *__restrict__ to_fp64,
                               unsigned int *__restrict__ n_to_fp64) {
  extern __shared__ float sf[];
  const int T = blockDim.x, tid = threadIdx.x;
  for (uint64_t row = (uint64_t)blockIdx.x * T + tid; row < rows; row += (uint64_t)gridDim.x * T)
    solve_row32<V>(gram, row, J, E, ldf, fac, lambda, cond_max, sf + tid, T, to_fp64, n_to_fp64);
}

// decode entry e of the packed row into (i, j), 0 <= i <= j <= J
__device__ __forceinline__ void pair_of(int e, int J, int &i, int &j) {
  int off = 0;
  i = 0;
  while (off + (J + 1 - i) <= e) {
    off += J + 1 - i;
    ++i;
  }
  j = i + (e - off);
}

__device__ void load_system(const double *__restrict__ g, int J, int E, double lambda, double *A, double *b,
                            int lane) {
  for (int e = lane; e < E; e += 32) {
    int i, j;
    pair_of(e, J, i, j);
    const double v = g[e];
    if (j == J) {
      b[i] = v;
    } else {
      A[i * J + j] = v;
      A[j * J + i] = v;
    }
  }
  __syncwarp();
  for (int i = lane; i < J; i += 32) A[i * J + i] += lambda;
  __syncwarp();
}

// LU with partial (row) pivoting, applied to b on the fly; returns false on an exactly zero pivot
__device__ bool lu_solve(double *A, double *b, int J, int lane) {
  bool ok = true;
  for (int k = 0; k < J; ++k) {
    double best = -1.0;
    int bi = k;
    for (int i = k + lane; i < J; i += 32) {
      const double v = fabs(A[i * J + k]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xFFFFFFFFu, best, o);
      const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (bi != k) {
      for (int c = lane; c < J; c += 32) {
        const double tmp = A[k * J + c];
        A[k * J + c] = A[bi * J + c];
        A[bi * J + c] = tmp;
      }
      if (lane == 0) {
        const double tmp = b[k];
        b[k] = b[bi];
        b[bi] = tmp;
      }
    }
    __syncwarp();
    double d = A[k * J + k];
    if (d == 0.0) {
      ok = false;
      d = 1e-300;
    }
    for (int i = k + 1 + lane; i < J; i += 32) {
      const double f = A[i * J + k] / d;
      A[i * J + k] = f;
      for (int c = k + 1; c < J; ++c) A[i * J + c] -= f * A[k * J + c];
      b[i] -= f * b[k];
    }
    __syncwarp();
  }
  for (int k = J - 1; k >= 0; --k) {
    const double d = A[k * J + k];
    const double xk = b[k] / (d == 0.0 ? 1e-300 : d);
    __syncwarp();
    if (lane == 0) b[k] = xk;
    for (int i = lane; i < k; i += 32) b[i] -= A[i * J + k] * xk;
    __syncwarp();
  }
  return ok;
}

// one warp per listed row: LU with partial pivoting; sets bit 2 of *status
// (informational) and bit 0 on an exactly zero pivot (GTK_ERR_NUMERIC)
template <class V>
__global__ void k_solve_lu_rows(const double *__restrict__ gram, const uint32_t *__restrict__ list,
                                const unsigned int *__restrict__ nlist, uint64_t all_rows, int J, int E, int ldf,
                                V *__restrict__ fac, int *__restrict__ status, double lambda) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  double *A = sm + (size_t)wib * ((size_t)J * J + J);
  double *b = A + (size_t)J * J;
  const uint64_t n = list ? (uint64_t)*nlist : all_rows;  // list == nullptr: every row, in order
  for (uint64_t k = (uint64_t)blockIdx.x * wpb + wib; k < n; k += (uint64_t)gridDim.x * wpb) {
    const uint32_t row = list ? list[k] : (uint32_t)k;
    load_system(gram + (uint64_t)row * E, J, E, lambda, A, b, lane);
    const bool ok = lu_solve(A, b, J, lane);
    if (lane == 0 && (list || !ok)) atomicOr(status, ok ? 4 : 1);
    V *frow = fac + (uint64_t)row * ldf;
    for (int j = lane; j < ldf; j += 32) frow[j] = j < J ? (V)b[j] : V(0);
    __syncwarp();
  }
}

// ComputingBC (update.cuh:52-100) in the reference's order, for the
// reference-order variant: one thread per (row, packed entry); B starts at lambda
// on the diagonal, then every product delta_i * delta_j (C: delta_i * x), rounded
// to value_t, is added in double over the row's nonzeros in view order -- block
// order, then the block's where_nnz order, as the reference walks them.  delta
// comes from the mode pass's store ([nnz][J], view order).
template <class V>
__global__ void k_bc_ref(const V *__restrict__ delta, const V *__restrict__ val, const uint32_t *__restrict__ row_of,
                         uint64_t nnz, uint64_t rows, int J, int E, double lambda, double *__restrict__ gram) {
  const uint64_t total = rows * (uint64_t)E;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total;
       w += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t row = w / E;
    const int e = (int)(w % E);
    int i, j;
    pair_of(e, J, i, j);
    // [s, f): the row's nonzeros in the view (sorted by row)
    uint64_t lo = 0, hi = nnz;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (row_of[mid] < row) lo = mid + 1; else hi = mid;
    }
    const uint64_t s0 = lo;
    hi = nnz;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (row_of[mid] <= row) lo = mid + 1; else hi = mid;
    }
    double sum = (i == j) ? lambda : 0.0;
    for (uint64_t t = s0; t < lo; ++t) {
      const V di = delta[t * J + i];
      const V dj = j == J ? val[t] : delta[t * J + j];
      sum = __dadd_rn(sum, (double)mul_rn(di, dj));
    }
    gram[row * E + e] = sum;
  }
}

// The reference's row solve (update.cuh:163-194) in its own operation order, for
// the reference-order variant: B^-1 from LU with row pivoting (first largest
// pivot) and a solve of the permuted identity, then a_k = sum_l C_l B^-1(l, k)
// accumulated in value_t (`value_t res += C * B_inv`): every product and sum
// rounded separately, no fused multiply-adds.  One warp per row; lane c owns
// column c of the inverse.
template <class V>
__global__ void k_solve_ref_rows(const double *__restrict__ gram, uint64_t rows, int J, int E, int ldf,
                                 V *__restrict__ fac, double lambda) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  double *A = sm + (size_t)wib * (2 * (size_t)J * J + 2 * J);
  double *b = A + (size_t)J * J;
  double *inv = b + J;            // [J][J], inv[i * J + c]
  double *perm = inv + (size_t)J * J;  // row permutation, as doubles
  for (uint64_t row = (uint64_t)blockIdx.x * wpb + wib; row < rows; row += (uint64_t)gridDim.x * wpb) {
    load_system(gram + row * E, J, E, lambda, A, b, lane);
    for (int i = lane; i < J; i += 32) perm[i] = (double)i;
    __syncwarp();
    for (int k = 0; k < J; ++k) {
      double best = -1.0;
      int bi = k;
      for (int i = k + lane; i < J; i += 32) {
        const double v = fabs(A[i * J + k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xFFFFFFFFu, best, o);
        const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (bi != k) {
        for (int c = lane; c < J; c += 32) {
          const double tmp = A[k * J + c];
          A[k * J + c] = A[bi * J + c];
          A[bi * J + c] = tmp;
        }
        if (lane == 0) {
          const double tp = perm[k];
          perm[k] = perm[bi];
          perm[bi] = tp;
        }
      }
      __syncwarp();
      const double d = A[k * J + k];
      if (d != 0.0) {
        for (int i = k + 1 + lane; i < J; i += 32) {
          const double f = __ddiv_rn(A[i * J + k], d);
          A[i * J + k] = f;
          for (int c = k + 1; c < J; ++c) A[i * J + c] = __dsub_rn(A[i * J + c], __dmul_rn(f, A[k * J + c]));
        }
      }
      __syncwarp();
    }
    for (int col = lane; col < J; col += 32) {
      for (int i = 0; i < J; ++i) {
        double sacc = ((int)perm[i] == col) ? 1.0 : 0.0;
        for (int c = 0; c < i; ++c) sacc = __dsub_rn(sacc, __dmul_rn(A[i * J + c], inv[c * J + col]));
        inv[i * J + col] = sacc;
      }
      for (int i = J - 1; i >= 0; --i) {
        double sacc = inv[i * J + col];
        for (int c = i + 1; c < J; ++c) sacc = __dsub_rn(sacc, __dmul_rn(A[i * J + c], inv[c * J + col]));
        inv[i * J + col] = __ddiv_rn(sacc, A[i * J + i]);
      }
    }
    __syncwarp();
    V *frow = fac + row * ldf;
    for (int k = lane; k < ldf; k += 32) {
      V res = V(0);
      if (k < J)
        for (int l = 0; l < J; ++l) res = (V)__dadd_rn((double)res, __dmul_rn(b[l], inv[l * J + k]));
      frow[k] = res;
    }
    __syncwarp();
  }
}

// Reconstruction in the reference's order, for the reference-order variant
// (ComputingReconstructionKernel, reconstruction.cuh:58-81): per nonzero of the
// last mode's view, x_hat = sum over core entries i in linear order of
// G_i * A_0[x_0][g_0(i)] * ... * A_{N-1}[x_{N-1}][g_{N-1}(i)], every product and sum
// rounded; written to the nonzero's block-major position.
template <class V>
__global__ void k_recon_ref(ModeArgs a, V *__restrict__ xhat) {
  const int J = a.J, N = a.N, ldf = a.ldf;
  const V *G = reinterpret_cast<const V *>(a.core);
  uint64_t ncore = 1;
  for (int k = 0; k < N; ++k) ncore *= (uint64_t)J;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.nnz; t += (uint64_t)gridDim.x * blockDim.x) {
    const V *fk[kMaxOrder];
    for (int k = 0; k < N; ++k) fk[k] = reinterpret_cast<const V *>(a.fac[k]) + (size_t)a.coord[k][t] * ldf;
    int dig[kMaxOrder];
    for (int k = 0; k < N; ++k) dig[k] = 0;
    V res = V(0);
    for (uint64_t i = 0; i < ncore; ++i) {
      V temp = G[i];
      for (int k = 0; k < N; ++k) temp = mul_rn(temp, fk[k][dig[k]]);
      res = add_rn(res, temp);
      for (int k = N - 1; k >= 0; --k) {
        if (++dig[k] < J) break;
        dig[k] = 0;
      }
    }
    xhat[a.vperm[t]] = res;
  }
}

// the reference's error loop (reconstruction.cuh:259-268): one thread, block-major
// order, Error += (x - x_hat)^2 in value_t -- serial like the reference's
template <class V>
__global__ void k_err_ref(const V *__restrict__ val, const V *__restrict__ xhat, uint64_t nnz, double *__restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  V err = V(0);
  for (uint64_t t = 0; t < nnz; ++t) {
    const V e = val[t] - xhat[t];
    err = add_rn(err, mul_rn(e, e));
  }
  *out = (double)err;
}

// the fit from the delta of the last mode's pass (stored in view order):
// x_hat = delta . a_{N-1}[i_{N-1}] in value_t (reconstruction.cuh:58-81 reduced to
// one dot product), error (x - x_hat)^2 summed in FP64 per CTA
template <class V>
__global__ void k_fit_stored(const V *__restrict__ dstore, const uint32_t *__restrict__ row_of,
                             const V *__restrict__ val, const V *__restrict__ fac, uint64_t nnz, int J, int ldf,
                             double *__restrict__ partial) {
  double err = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnz; t += (uint64_t)gridDim.x * blockDim.x) {
    const V *d = dstore + t * (uint64_t)J;
    const V *a = fac + (uint64_t)row_of[t] * ldf;
    V xh = V(0);
    for (int j = 0; j < J; ++j) xh += d[j] * a[j];
    const V e = val[t] - xh;
    err += (double)e * (double)e;
  }
  const double tot = block_sum(err);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// The fit from the last mode's Gram/RHS, without a pass over the nonzeros: with
// G_i = sum delta delta^T and c_i = sum x delta over row i's nonzeros and a_i the
// row's new factor row,
//   sum_{nonzeros of row i} (x - delta . a_i)^2 = sum x^2 - 2 a_i . c_i + a_i^T G_i a_i,
// so err = ||X||^2 - sum_i (2 a_i . c_i - a_i^T G_i a_i).  Per CTA the negated
// row sum (CTA 0 adds ||X||^2), so that k_sum_fit yields err.  Gram layout:
// entry (i, j), i <= j <= J, at i (J+1) - i (i-1) / 2 + (j - i); column J is c.
template <class V>
__global__ void k_fit_gram(const double *__restrict__ gram, const V *__restrict__ fac, uint64_t rows, int J, int E,
                           int ldf, double normsq, double *__restrict__ partial) {
  double s = 0;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x) {
    const double *g = gram + r * (uint64_t)E;
    const V *a = fac + r * (uint64_t)ldf;
    double q = 0;
    int e = 0;
    for (int i = 0; i < J; ++i) {
      const double ai = (double)a[i];
      double t = 0.5 * g[e++] * ai;  // the diagonal once, the off-diagonal twice
      for (int j = i + 1; j < J; ++j) t += g[e++] * (double)a[j];
      q += ai * (2.0 * g[e++] - 2.0 * t);  // 2 a_i c_i - a_i (G a)_i, upper triangle
    }
    s += q;
  }
  const double tot = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = (blockIdx.x == 0 ? normsq : 0.0) - tot;
}

// out = the sum of partial[0, m) (acc: out += it, the streamed passes' chunks)
__global__ void k_sum_fit(const double *__restrict__ partial, int m, double *__restrict__ out, int acc = 0) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += partial[i];
    *out = acc ? *out + s : s;
  }
}

// ---------------------------------------------------------------- dispatch
struct Launch {
  const void *fn = nullptr;
  const void *fn_multi = nullptr;  // the multi-tensor form (FP32 updates), for batches
  size_t smem = 0;
  int tn = 0;  // nonzeros per tile
  bool spec = false;
};


template <class V, int N, int J, int KIND, int NPT, bool STREAM = false>
void spec_entry(Launch &L, const DevTensor &t) {
  constexpr int W = Vec<V>::W;
  constexpr int LDG = (J + W - 1) / W * W;
  constexpr int D = N - 1;
  constexpr int LEV = D > 2 ? D - 2 : 0;
  const size_t gp = STREAM ? 2 * CoreStream<N, J, LDG>::CH : (size_t)Pow<J, N - 1>::v * LDG;
  L.fn = (const void *)k_mode_spec<V, N, J, NPT, KIND, STREAM>;
  if constexpr (KIND == kUpdate && std::is_same<V, float>::value)
    L.fn_multi = (const void *)k_mode_spec_multi<V, N, J, NPT, KIND, STREAM>;
  L.smem = tile_smem_bytes(sizeof(V), gp, LEV, NPT, J, ldd_for(J), pairs_for(J), kThreads * NPT);
  L.tn = kThreads * NPT;
  L.spec = true;
  (void)t;
}

// The specialised (N, J) table (NPT nonzeros per thread).  Anything else runs the generic kernel.
template <class V, int KIND, int NPT> bool find_spec(Launch &L, const DevTensor &t) {
#define GTK_SPEC(NN, JJ)                                          \
  if (t.N == NN && t.J == JJ) {                                   \
    spec_entry<V, NN, JJ, KIND, NPT>(L, t);                       \
    return true;                                                  \
  }
  GTK_SPEC(3, 4) GTK_SPEC(3, 8) GTK_SPEC(3, 10) GTK_SPEC(3, 12) GTK_SPEC(3, 16)
  GTK_SPEC(4, 4) GTK_SPEC(4, 8) GTK_SPEC(4, 10) GTK_SPEC(4, 12)
  GTK_SPEC(5, 4) GTK_SPEC(5, 8)
#undef GTK_SPEC
  // cores streamed through shared memory (FP32 update and fit)
  if constexpr (std::is_same<V, float>::value && KIND != kDelta) {
#define GTK_STREAM(NN, JJ)                                        \
  if (t.N == NN && t.J == JJ) {                                   \
    spec_entry<V, NN, JJ, KIND, NPT, true>(L, t);                 \
    return true;                                                  \
  }
    GTK_STREAM(4, 16) GTK_STREAM(5, 12) GTK_STREAM(5, 16)
#undef GTK_STREAM
  }
  return false;
}

constexpr size_t kSmemLimit = 227 * 1024;
constexpr int kSolveMultiThreads = 64;  // batched row solves: threads per block
constexpr int kLuMultiThreads = 128;    // batched pivoted-LU pass: 4 warps per block
constexpr int kThreadSolveMaxJ = 24;  // larger ranks solve one row per warp
// precision form: rows whose 1-norm condition estimate exceeds this are solved
// in FP64 (one FP32 refinement step leaves ~(kappa * 2^-24)^2)
constexpr float kCondMaxFp32 = 1e5f;

// kernel of a KIND: the update honours the handle's variant (set by the autotuner);
// the reference-order variant applies to every KIND
template <class V, int KIND> int choose(Launch &L, const DevTensor &t, bool &gp_in_smem) {
  gp_in_smem = true;
  const int var = (KIND == kUpdate || t.variant == kVarRefOrder) ? t.variant : kVarAuto;
  if (var == kVarRefOrder) {
    L.spec = false;
    L.tn = kThreads;
    L.fn = (const void *)k_mode_gen<V, KIND>;
    gp_in_smem = false;
    L.smem = tile_smem_bytes(sizeof(V), 0, 0, 1, t.J, ldd_for(t.J), pairs_for(t.J), kThreads);
    return 0;
  }
  if (var == kVarSpec1) {
    if (find_spec<V, KIND, 1>(L, t) && L.smem <= kSmemLimit) return 0;
  } else if (var != kVarGeneric) {
    if (find_spec<V, KIND, 2>(L, t) && L.smem <= kSmemLimit) return 0;
  }
  const size_t gp = (size_t)t.core_n / (size_t)t.J * t.ldf;
  L.spec = false;
  L.tn = kThreads;
  L.fn = (const void *)k_mode_gen<V, KIND>;
  L.smem = tile_smem_bytes(sizeof(V), gp, 0, 1, t.J, ldd_for(t.J), pairs_for(t.J), kThreads);
  if (L.smem > 160 * 1024) {
    gp_in_smem = false;
    L.smem = tile_smem_bytes(sizeof(V), 0, 0, 1, t.J, ldd_for(t.J), pairs_for(t.J), kThreads);
  }
  return 0;
}

int prepare_fn(const void *fn, size_t smem) {
  static std::vector<std::pair<const void *, size_t>> done;
  for (auto &d : done)
    if (d.first == fn && d.second >= smem) return 0;
  GTK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  done.emplace_back(fn, smem);
  return 0;
}

ModeArgs make_args(const DevTensor &t, int mode) {
  ModeArgs a;
  memset(&a, 0, sizeof(a));
  const ViewRange vr = view_of(t, mode);
  for (int k = 0; k < t.N; ++k) {
    a.coord[k] = vr.coord[k];
    a.fac[k] = t.fac[k];
  }
  a.val = vr.val;
  a.corep = t.corep[mode];
  a.vperm = t.vperm[mode];
  a.gram = t.gram;
  a.partial = t.partial;
  a.status = t.status;
  a.nnz = vr.nnz;
  a.N = t.N;
  a.J = t.J;
  a.ldf = t.ldf;
  a.mode = mode;
  a.E = pairs_for(t.J);
  a.ldd = ldd_for(t.J);
  int m = 0;
  for (int k = 0; k < t.N; ++k)
    if (k != mode) a.others[m++] = k;
  a.gp_elems = (uint64_t)(t.core_n / (uint64_t)t.J) * (uint64_t)t.ldf;
  return a;
}

// profiling scopes: events recorded around a launch, resolved on read
struct ProfEvent {
  int kind;
  cudaEvent_t a, b;
};
std::vector<ProfEvent> &pending_events() {
  static std::vector<ProfEvent> v;
  return v;
}

}  // namespace

// record helpers used by the launch sites below and by api.cpp
int prof_begin(DevTensor &t, cudaEvent_t *a) {
  if (!t.prof) return 0;
  GTK_CUDA(cudaEventCreate(a));
  GTK_CUDA(cudaEventRecord(*a, t.stream));
  return 0;
}
int prof_end(DevTensor &t, int kind, cudaEvent_t a) {
  if (!t.prof) return 0;
  cudaEvent_t b;
  GTK_CUDA(cudaEventCreate(&b));
  GTK_CUDA(cudaEventRecord(b, t.stream));
  pending_events().push_back({kind, a, b});
  return 0;
}
int prof_resolve(DevTensor &t) {
  auto &v = pending_events();
  if (v.empty()) return 0;
  GTK_CUDA(cudaStreamSynchronize(t.stream));
  for (auto &e : v) {
    float ms = 0;
    GTK_CUDA(cudaEventElapsedTime(&ms, e.a, e.b));
    t.prof_ms[e.kind] += ms;
    t.prof_n[e.kind] += 1;
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  v.clear();
  return 0;
}

template <class V, int KIND> static int launch_mode(DevTensor &t, int mode, void *out, int *grid_out) {
  Launch L;
  bool gp_in_smem = true;
  choose<V, KIND>(L, t, gp_in_smem);
  if (int rc = prepare_fn(L.fn, L.smem)) return rc;
  ModeArgs a = make_args(t, mode);
  a.gp_in_smem = gp_in_smem ? 1 : 0;
  a.ref_order = t.variant == kVarRefOrder ? 1 : 0;
  a.core = t.core;
  if (KIND == kUpdate)
    a.dstore = out;  // optional: delta of every nonzero, view order
  else
    a.out = out;
  int per_sm = 0;
  GTK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L.fn, kThreads, L.smem));
  if (per_sm < 1) return fail(GTK_ERR_UNSUPPORTED, "mode kernel does not fit on an SM");
  const uint64_t ntiles = (a.nnz + L.tn - 1) / L.tn;
  uint64_t grid = std::min<uint64_t>(ntiles, KIND == kUpdate ? update_grid_cap(t, (uint64_t)per_sm)
                                                             : (uint64_t)per_sm * t.num_sms);
  if (KIND == kFit) grid = std::min<uint64_t>(grid, kFitGridMax);
  if (grid < 1) grid = 1;
  void *args[] = {&a};
  GTK_CUDA(cudaLaunchKernel(L.fn, dim3((unsigned)grid), dim3(kThreads), args, L.smem, t.stream));
  if (grid_out) *grid_out = (int)grid;
  return 0;
}

// the buffer for the last mode's delta ([nnz][J] value_t); without room the fit
// recomputes delta instead (never an error)
int ensure_dstore(DevTensor &t) {
  if (t.dstore || t.dstore_failed || !t.nnz) return 0;
  if (dalloc(t, &t.dstore, t.nnz * (size_t)t.J * t.vsize)) {
    t.dstore = nullptr;
    t.dstore_failed = true;
    cudaGetLastError();
    set_error("");
  }
  return 0;
}

// the update runs the tensor-core kernels (the precision forms)
static bool tc_update(const DevTensor &t) {
  return t.variant == kVarTc || (t.variant == kVarAuto && t.precision != GTK_PREC_PLAIN);
}

bool sweep_needs_dstore(const DevTensor &t) { return t.variant == kVarRefOrder || !tc_update(t); }

void fit_invalidate(DevTensor &t) {
  t.fit_from_store = false;
  t.fit_from_gram = false;
}

void fit_after_sweep(DevTensor &t) {
  t.fit_from_gram = tc_update(t);
  t.fit_from_store = !t.fit_from_gram && t.dstore != nullptr;
}

// One pass of a mode kernel over the streamed view of `mode` (the streamed
// layout): chunk c goes to staging buffer c % 2 on copy_stream -- after the
// kernel that read that buffer last has finished -- while the kernel of chunk
// c - 1 runs on the handle's stream; `launch` enqueues the kernel for t.range.
template <class F> static int stream_pass(DevTensor &t, int mode, F launch) {
  const HostPart &h = *t.hp;
  uint64_t c = 0;
  for (uint64_t c0 = 0; c0 < t.nnz; c0 += t.chunk, ++c) {
    const int b = (int)(c & 1);
    const uint64_t m = std::min<uint64_t>(t.chunk, t.nnz - c0);
    GTK_CUDA(cudaStreamWaitEvent(t.copy_stream, t.stage_free[b], 0));
    for (int k = 0; k < t.N; ++k)
      GTK_CUDA(cudaMemcpyAsync(t.stage_idx[b][k], h.vidx[mode][k].data() + c0, m * 4, cudaMemcpyHostToDevice,
                               t.copy_stream));
    GTK_CUDA(cudaMemcpyAsync(t.stage_val[b], h.vval[mode].data() + c0 * t.vsize, m * t.vsize, cudaMemcpyHostToDevice,
                             t.copy_stream));
    GTK_CUDA(cudaEventRecord(t.stage_ready[b], t.copy_stream));
    GTK_CUDA(cudaStreamWaitEvent(t.stream, t.stage_ready[b], 0));
    ViewRange r;
    for (int k = 0; k < kMaxOrder; ++k) r.coord[k] = k < t.N ? t.stage_idx[b][k] : nullptr;
    r.val = t.stage_val[b];
    r.nnz = m;
    t.range = &r;
    const int rc = launch();
    t.range = nullptr;
    if (rc) return rc;
    GTK_CUDA(cudaEventRecord(t.stage_free[b], t.stream));
    t.stream_copy_bytes += (double)m * (double)(t.N * 4 + t.vsize);
    t.launches += 1;
  }
  return 0;
}

template <class V> static int update_impl(DevTensor &t, int mode) {
  static const char *const kNames[kMaxOrder] = {"mode update 0", "mode update 1", "mode update 2", "mode update 3",
                                                 "mode update 4", "mode update 5", "mode update 6", "mode update 7"};
  NvtxRange nvtx(kNames[mode]);
  const int E = pairs_for(t.J);
  const int J = t.J;
  const bool last = mode == t.N - 1;
  const bool tc = tc_update(t);
  // the fit follows from the last mode's pass: in the tensor-core forms from its
  // Gram/RHS (k_fit_gram), otherwise from delta, which the pass then stores (the
  // reference-order variant stores it on every mode: its B and C come from it)
  void *dstore = nullptr;
  if (!t.streamed && ((last && !tc) || t.variant == kVarRefOrder) && t.nnz) {
    if (int rc = ensure_dstore(t)) return rc;
    dstore = t.dstore;
  }
  fit_invalidate(t);
  cudaEvent_t ev = nullptr;
  if (int rc = prof_begin(t, &ev)) return rc;
  GTK_CUDA(cudaMemsetAsync(t.gram, 0, t.rows[mode] * (uint64_t)E * 8, t.stream));
  if (t.nnz && t.streamed) {
    if (int rc = stream_pass(t, mode, [&]() {
          return tc ? run_mode_tc(t, mode, 0, nullptr, nullptr) : launch_mode<V, kUpdate>(t, mode, nullptr, nullptr);
        }))
      return rc;
  } else if (t.nnz) {
    if (tc) {
      if (int rc = run_mode_tc(t, mode, 0, dstore, nullptr)) return rc;
    } else if (int rc = launch_mode<V, kUpdate>(t, mode, dstore, nullptr)) {
      return rc;
    }
    t.launches += 1;
  }
  if (int rc = prof_end(t, 0, ev)) return rc;
  if (int rc = prof_begin(t, &ev)) return rc;
  GTK_CUDA(cudaMemsetAsync(t.nfallback, 0, 4, t.stream));
  const size_t lu_warp = ((size_t)J * J + J) * 8;
  const int lu_wpb = (int)std::min<size_t>(8, std::max<size_t>(1, (48 * 1024) / lu_warp));
  const size_t lu_smem = lu_warp * lu_wpb;
  if (int rc = prepare_fn((const void *)k_solve_lu_rows<V>, lu_smem)) return rc;
  if (t.variant == kVarRefOrder) {
    // B and C again, in the reference's summation order, from the stored delta
    if (!t.dstore) return fail(GTK_ERR_OOM, "the reference-order variant needs room for delta ([nnz][J])");
    if (t.nnz) {
      const uint64_t total = t.rows[mode] * (uint64_t)E;
      const unsigned g = (unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)t.num_sms * 64);
      k_bc_ref<V><<<g, 256, 0, t.stream>>>((const V *)t.dstore, (const V *)t.vval[mode], t.vidx[mode][mode], t.nnz,
                                           t.rows[mode], J, E, kLambda, t.gram);
      GTK_CUDA(cudaGetLastError());
      t.launches += 1;
    }
    // the reference's inverse-then-multiply with value_t accumulation (update.cuh:163-194);
    // lambda is already on the diagonal
    const size_t per_warp = (2 * (size_t)J * J + 2 * J) * 8;
    const int wpb = (int)std::min<size_t>(8, std::max<size_t>(1, (96 * 1024) / per_warp));
    const size_t smem = per_warp * wpb;
    if (int rc = prepare_fn((const void *)k_solve_ref_rows<V>, smem)) return rc;
    uint64_t grid = std::min<uint64_t>((t.rows[mode] + wpb - 1) / wpb, (uint64_t)t.num_sms * 32);
    if (grid < 1) grid = 1;
    k_solve_ref_rows<V><<<(unsigned)grid, wpb * 32, smem, t.stream>>>(t.gram, t.rows[mode], J, E, t.ldf,
                                                                      (V *)t.fac[mode], t.nnz ? 0.0 : kLambda);
    GTK_CUDA(cudaGetLastError());
    t.launches += 1;
  } else if (J <= kThreadSolveMaxJ) {
    const int T = J <= 12 ? 128 : 64;
    const size_t smem = (size_t)T * E * 8;
    if (int rc = prepare_fn((const void *)k_solve_rows<V>, smem)) return rc;
    uint64_t grid = (t.rows[mode] + T - 1) / T;
    if (grid < 1) grid = 1;
    if (t.precision != GTK_PREC_PLAIN) {
      // FP32 Cholesky + refinement; rows above the condition threshold in FP64
      const size_t smem32 = (size_t)T * (E + 3 * J) * 4;
      if (int rc = prepare_fn((const void *)k_solve_rows32<V>, smem32)) return rc;
      GTK_CUDA(cudaMemsetAsync(t.nfallback + 1, 0, 4, t.stream));
      k_solve_rows32<V><<<(unsigned)grid, T, smem32, t.stream>>>(t.gram, t.rows[mode], J, E, t.ldf,
                                                                 (V *)t.fac[mode], kLambda, kCondMaxFp32,
                                                                 t.fallback64, t.nfallback + 1);
      GTK_CUDA(cudaGetLastError());
      k_solve_rows<V><<<(unsigned)t.num_sms, T, smem, t.stream>>>(t.gram, 0, t.fallback64, t.nfallback + 1, J, E,
                                                                  t.ldf, (V *)t.fac[mode], kLambda, t.fallback,
                                                                  t.nfallback);
      t.launches += 1;
    } else {
      k_solve_rows<V><<<(unsigned)grid, T, smem, t.stream>>>(t.gram, t.rows[mode], nullptr, nullptr, J, E, t.ldf,
                                                             (V *)t.fac[mode], kLambda, t.fallback, t.nfallback);
    }
    GTK_CUDA(cudaGetLastError());
    k_solve_lu_rows<V><<<(unsigned)t.num_sms, lu_wpb * 32, lu_smem, t.stream>>>(
        t.gram, t.fallback, t.nfallback, 0, J, E, t.ldf, (V *)t.fac[mode], t.status, kLambda);
    GTK_CUDA(cudaGetLastError());
    t.launches += 2;
  } else {
    uint64_t grid = std::min<uint64_t>((t.rows[mode] + lu_wpb - 1) / lu_wpb, (uint64_t)t.num_sms * 32);
    if (grid < 1) grid = 1;
    k_solve_lu_rows<V><<<(unsigned)grid, lu_wpb * 32, lu_smem, t.stream>>>(
        t.gram, nullptr, t.nfallback, t.rows[mode], J, E, t.ldf, (V *)t.fac[mode], t.status, kLambda);
    GTK_CUDA(cudaGetLastError());
    t.launches += 1;
  }
  t.fit_from_store = dstore != nullptr && last;
  // the streamed layout keeps no delta: every form takes the fit from the Gram/RHS
  t.fit_from_gram = (tc || t.streamed) && last;
  if (int rc = prof_end(t, 1, ev)) return rc;
  return 0;
}

int run_update_mode(DevTensor &t, int mode) {
  return t.dtype == GTK_F32 ? update_impl<float>(t, mode) : update_impl<double>(t, mode);
}

// the fit kernels: the error of every nonzero summed into t.partial[kFitGridMax]
template <class V> static int fit_enqueue(DevTensor &t) {
  NvtxRange nvtx("fit");
  int grid = 1;
  if (t.variant == kVarRefOrder && t.nnz) {
    // x_hat into the delta store's memory (nnz values), then the serial error
    if (int rc = ensure_dstore(t)) return rc;
    if (!t.dstore) return fail(GTK_ERR_OOM, "the reference-order fit needs nnz values of scratch");
    ModeArgs a = make_args(t, t.N - 1);
    a.core = t.core;
    const unsigned g = (unsigned)std::min<uint64_t>((t.nnz + 255) / 256, (uint64_t)t.num_sms * 16);
    k_recon_ref<V><<<g, 256, 0, t.stream>>>(a, (V *)t.dstore);
    k_err_ref<V><<<1, 32, 0, t.stream>>>((const V *)t.blk_val, (const V *)t.dstore, t.nnz, t.partial + kFitGridMax);
    GTK_CUDA(cudaGetLastError());
    t.launches += 2;
    t.fit_from_store = false;  // the store now holds x_hat
    return 0;
  }
  if (t.fit_from_gram && t.nnz) {
    const int N = t.N;
    grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(kFitGridMax, (t.rows[N - 1] + 255) / 256));
    k_fit_gram<V><<<grid, 256, 0, t.stream>>>(t.gram, (const V *)t.fac[N - 1], t.rows[N - 1], t.J, pairs_for(t.J),
                                              t.ldf, t.norm * t.norm, t.partial);
    GTK_CUDA(cudaGetLastError());
    t.launches += 1;
  } else if (t.fit_from_store && t.nnz) {
    grid = (int)std::min<uint64_t>(kFitGridMax, (t.nnz + 255) / 256);
    k_fit_stored<V><<<grid, 256, 0, t.stream>>>((const V *)t.dstore, t.vidx[t.N - 1][t.N - 1], (const V *)t.vval[t.N - 1],
                                                (const V *)t.fac[t.N - 1], t.nnz, t.J, t.ldf, t.partial);
    GTK_CUDA(cudaGetLastError());
    t.launches += 1;
  } else if (t.nnz && t.streamed) {
    // the direct fit over the streamed view, each chunk's partials added to the sum
    GTK_CUDA(cudaMemsetAsync(t.partial + kFitGridMax, 0, 8, t.stream));
    if (int rc = stream_pass(t, t.N - 1, [&]() -> int {
          int g = 1;
          if (t.precision != GTK_PREC_PLAIN) {
            if (int rc2 = run_mode_tc(t, t.N - 1, 1, nullptr, &g)) return rc2;
          } else if (int rc2 = launch_mode<V, kFit>(t, t.N - 1, nullptr, &g)) {
            return rc2;
          }
          k_sum_fit<<<1, 32, 0, t.stream>>>(t.partial, g, t.partial + kFitGridMax, 1);
          t.launches += 1;
          return ck(cudaGetLastError(), "k_sum_fit");
        }))
      return rc;
    return 0;
  } else if (t.nnz) {
    t.launches += 1;
    if (t.precision != GTK_PREC_PLAIN) {
      if (int rc = run_mode_tc(t, t.N - 1, 1, nullptr, &grid)) return rc;
    } else if (int rc = launch_mode<V, kFit>(t, t.N - 1, nullptr, &grid)) {
      return rc;
    }
  } else {
    GTK_CUDA(cudaMemsetAsync(t.partial, 0, 8, t.stream));
  }
  k_sum_fit<<<1, 32, 0, t.stream>>>(t.partial, grid, t.partial + kFitGridMax);
  GTK_CUDA(cudaGetLastError());
  t.launches += 1;
  return 0;
}

double fit_from_err(const DevTensor &t, double err) {
  if (t.variant == kVarRefOrder && t.nnz) {
    // reconstruction.cuh:272-276 with the reference's value_t Error and norm
    if (t.norm_ref == 0) return 1.0;
    if (t.dtype == GTK_F32) {
      const float e = (float)err, nr = (float)t.norm_ref;
      return (double)(1.0f - std::sqrt(e) / nr);
    }
    return 1.0 - std::sqrt(err) / t.norm_ref;
  }
  return (t.norm == 0) ? 1.0 : 1.0 - std::sqrt(std::max(0.0, err)) / t.norm;
}

static int fit_read(DevTensor &t, double *fit) {
  if (t.variant == kVarRefOrder)
    if (int rc = ensure_norm_ref(t)) return rc;
  double err = 0;
  GTK_CUDA(cudaMemcpyAsync(&err, t.partial + kFitGridMax, 8, cudaMemcpyDeviceToHost, t.stream));
  GTK_CUDA(cudaStreamSynchronize(t.stream));
  *fit = fit_from_err(t, err);
  return 0;
}

static_assert(kFitSumSlot == kFitGridMax, "the fit's error sum follows the per-CTA partials");
int run_fit_enqueue(DevTensor &t) { return t.dtype == GTK_F32 ? fit_enqueue<float>(t) : fit_enqueue<double>(t); }

int run_fit(DevTensor &t, double *fit) {
  cudaEvent_t ev = nullptr;
  if (int rc = prof_begin(t, &ev)) return rc;
  if (int rc = t.dtype == GTK_F32 ? fit_enqueue<float>(t) : fit_enqueue<double>(t)) return rc;
  if (int rc = prof_end(t, 2, ev)) return rc;
  return fit_read(t, fit);
}

void drop_graph(DevTensor &t) {
  if (t.gexec) cudaGraphExecDestroy(t.gexec);
  if (t.graph) cudaGraphDestroy(t.graph);
  t.gexec = nullptr;
  t.graph = nullptr;
}

// One sweep (every mode's update, then the fit).  With t.use_graph the device
// work of a sweep -- memsets, the fused and solve kernels of every mode, the fit
// kernels -- is captured once into a CUDA graph and replayed; only the 8-byte
// read of the error sum stays outside.
int run_sweep(DevTensor &t, double *fit) {
  NvtxRange nvtx("sweep");
  if (!t.use_graph || t.streamed) {  // streamed passes copy from the host: not captured
    for (int n = 0; n < t.N; ++n)
      if (int rc = run_update_mode(t, n)) return rc;
    return run_fit(t, fit);
  }
  if (!t.gexec) {
    if (sweep_needs_dstore(t))
      if (int rc = ensure_dstore(t)) return rc;
    const bool prof = t.prof;
    t.prof = false;
    const uint64_t l0 = t.launches;
    GTK_CUDA(cudaStreamBeginCapture(t.stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int n = 0; n < t.N && !rc; ++n) rc = run_update_mode(t, n);
    if (!rc) rc = t.dtype == GTK_F32 ? fit_enqueue<float>(t) : fit_enqueue<double>(t);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(t.stream, &g);
    t.prof = prof;
    if (rc || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      t.launches = l0;
      return rc ? rc : cuda_fail(ec, "cudaStreamEndCapture");
    }
    t.graph = g;
    if (cudaGraphInstantiate(&t.gexec, t.graph, 0) != cudaSuccess) {
      drop_graph(t);
      return cuda_fail(cudaGetLastError(), "cudaGraphInstantiate");
    }
    t.graph_kernels = t.launches - l0;
    t.launches = l0;
  }
  cudaEvent_t ev = nullptr;
  if (int rc = prof_begin(t, &ev)) return rc;
  GTK_CUDA(cudaGraphLaunch(t.gexec, t.stream));
  if (int rc = prof_end(t, 3, ev)) return rc;
  t.launches += t.graph_kernels;
  fit_after_sweep(t);
  return fit_read(t, fit);
}

// factors between the device layout [rows][ldf] and the reference's slab layout
// [rows][J]: repacked on the device so that the host copy is one contiguous
// transfer (a pitched copy of 100,000 rows of 40 bytes runs far below the link)
template <class V> __global__ void k_fac_pack(const V *__restrict__ fac, uint64_t rows, int J, int ldf, V *__restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * J; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = fac[(i / J) * ldf + i % J];
}
template <class V> __global__ void k_fac_unpack(const V *__restrict__ in, uint64_t rows, int J, int ldf, V *__restrict__ fac) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * J; i += (uint64_t)gridDim.x * blockDim.x)
    fac[(i / J) * ldf + i % J] = in[i];
}

int factor_to_host(const DevTensor &t, int n, void *slabs) {
  const uint64_t m = t.rows[n] * (uint64_t)t.J;
  if (!m) return 0;
  const unsigned g = (unsigned)std::min<uint64_t>((m + 255) / 256, (uint64_t)t.num_sms * 8);
  if (t.dtype == GTK_F32)
    k_fac_pack<float><<<g, 256, 0, t.stream>>>((const float *)t.fac[n], t.rows[n], t.J, t.ldf, (float *)t.xfer);
  else
    k_fac_pack<double><<<g, 256, 0, t.stream>>>((const double *)t.fac[n], t.rows[n], t.J, t.ldf, (double *)t.xfer);
  GTK_CUDA(cudaGetLastError());
  GTK_CUDA(cudaMemcpyAsync(slabs, t.xfer, m * t.vsize, cudaMemcpyDeviceToHost, t.stream));
  GTK_CUDA(cudaStreamSynchronize(t.stream));
  return 0;
}

// The factors' draws of gtk_init_random (tucker.cuh:84-97): mode n's real rows
// are rows 0 .. dims[n]-1 of its stacked slabs, so draw d of the mode lands at
// row d / J, column d % J.  Two passes over the zeroed factors:
// * k_fac_draws: the sequence is cut into chunks of kFacChunk draws (start
//   windows from the host) and each chunk into kFacSplit pieces; thread
//   (c, j) moves chunk c's 31-value window on by j pieces (the window of x^k mod
//   p applied to it: the coefficients of x^(j len) mod p come from the host,
//   then one multiplication by x per further value), then generates its piece by
//   glibc's recurrence r[k] = r[k-31] + r[k-3] (mod 2^32), 31 steps at a time so
//   the window stays in registers, and stores rand() = r >> 1 in the draw's
//   factor entry as an integer;
// * k_fac_frand: every entry of the factors, in parallel, becomes
//   frand(0, 1) = (double)rand() / (2^31 - 1) as value_t (padding entries hold 0
//   and stay 0), so the FP64 divisions spread over the whole GPU.
struct FacInit {
  void *fac[kMaxOrder];
  uint64_t first[kMaxOrder + 1];  // draw offset of each mode
  int N, J, ldf;
};
template <class V>
__global__ void k_fac_draws(const uint32_t *__restrict__ states, const uint32_t *__restrict__ polys, int chunks,
                            const __grid_constant__ FacInit f) {
  using U = std::conditional_t<sizeof(V) == 4, uint32_t, unsigned long long>;
  constexpr uint64_t len = kFacChunk / kFacSplit;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = t / kFacSplit, piece = t % kFacSplit;
  if (c >= chunks) return;
  const uint64_t b = (uint64_t)c * kFacChunk + (uint64_t)piece * len, e = min(f.first[f.N], b + len);
  if (b >= e) return;
  uint32_t w[31];
  {
    uint32_t s[31], a[31];
#pragma unroll
    for (int j = 0; j < 31; ++j) s[j] = states[31 * (size_t)c + j], a[j] = polys[31 * piece + j];
#pragma unroll
    for (int m = 0; m < 31; ++m) {  // w[m] = r[b - 31 + m] = (x^(piece len + m) mod p) . s
      uint32_t v = 0;
#pragma unroll
      for (int j = 0; j < 31; ++j) v += a[j] * s[j];
      w[m] = v;
      const uint32_t top = a[30];  // a <- x a mod p, x^31 = x^28 + 1
#pragma unroll
      for (int j = 30; j > 0; --j) a[j] = a[j - 1];
      a[0] = top;
      a[28] += top;
    }
  }
  int n = 0;
  while (n + 1 < f.N && b >= f.first[n + 1]) ++n;
  const uint64_t off = b - f.first[n];
  uint64_t row = off / (uint64_t)f.J;
  int col = (int)(off - row * (uint64_t)f.J);
  for (uint64_t base = b; base < e; base += 31) {
#pragma unroll
    for (int k = 0; k < 31; ++k) {
      const uint32_t v = w[k] + w[(k + 28) % 31];
      w[k] = v;
      if (base + k < e) {
        while (base + k >= f.first[n + 1]) {  // the next mode's draws
          ++n;
          row = 0;
          col = 0;
        }
        reinterpret_cast<U *>(f.fac[n])[row * (uint64_t)f.ldf + col] = (U)(v >> 1);
        if (++col == f.J) {
          col = 0;
          ++row;
        }
      }
    }
  }
}
template <class V> __global__ void k_fac_frand(V *__restrict__ fac, uint64_t m) {
  using U = std::conditional_t<sizeof(V) == 4, uint32_t, unsigned long long>;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    const U r = reinterpret_cast<const U *>(fac)[i];
    fac[i] = (V)((double)r / 2147483647.0);
  }
}

int factor_init_device(DevTensor &t, GlibcRand &g) {
  FacInit f;
  memset(&f, 0, sizeof(f));
  f.N = t.N;
  f.J = t.J;
  f.ldf = t.ldf;
  for (int n = 0; n < t.N; ++n) {
    f.fac[n] = t.fac[n];
    f.first[n + 1] = f.first[n] + (uint64_t)t.dims[n] * t.J;
    GTK_CUDA(cudaMemsetAsync(t.fac[n], 0, t.rows[n] * (uint64_t)t.ldf * t.vsize, t.stream));
  }
  const uint64_t total = f.first[t.N];
  if (!total) return 0;
  const int chunks = (int)((total + kFacChunk - 1) / kFacChunk);
  std::vector<uint32_t> st((size_t)(chunks + kFacSplit) * 31);  // chunk windows, then the piece polynomials
  glibc_chunk_states(g, kFacChunk, chunks, st.data());
  glibc_step_polys(kFacChunk / kFacSplit, kFacSplit, st.data() + (size_t)chunks * 31);
  DevBuf buf;
  GTK_CUDA(buf.alloc(st.size() * 4));
  GTK_CUDA(cudaMemcpyAsync(buf.p, st.data(), st.size() * 4, cudaMemcpyHostToDevice, t.stream));
  const uint32_t *d_st = buf.as<uint32_t>();
  const unsigned blocks = (unsigned)(((uint64_t)chunks * kFacSplit + 63) / 64);
  if (t.dtype == GTK_F32)
    k_fac_draws<float><<<blocks, 64, 0, t.stream>>>(d_st, d_st + (size_t)chunks * 31, chunks, f);
  else
    k_fac_draws<double><<<blocks, 64, 0, t.stream>>>(d_st, d_st + (size_t)chunks * 31, chunks, f);
  GTK_CUDA(cudaGetLastError());
  for (int n = 0; n < t.N; ++n) {
    const uint64_t m = t.rows[n] * (uint64_t)t.ldf;
    const unsigned gr = (unsigned)std::min<uint64_t>((m + 255) / 256, (uint64_t)t.num_sms * 8);
    if (t.dtype == GTK_F32)
      k_fac_frand<float><<<gr, 256, 0, t.stream>>>((float *)t.fac[n], m);
    else
      k_fac_frand<double><<<gr, 256, 0, t.stream>>>((double *)t.fac[n], m);
    GTK_CUDA(cudaGetLastError());
  }
  GTK_CUDA(cudaStreamSynchronize(t.stream));  // the states' buffer is freed on return
  g.jump(total);
  return 0;
}

int factor_from_host(DevTensor &t, int n, const void *slabs) {
  const uint64_t m = t.rows[n] * (uint64_t)t.J;
  if (!m) return 0;
  GTK_CUDA(cudaMemcpyAsync(t.xfer, slabs, m * t.vsize, cudaMemcpyHostToDevice, t.stream));
  const unsigned g = (unsigned)std::min<uint64_t>((m + 255) / 256, (uint64_t)t.num_sms * 8);
  if (t.dtype == GTK_F32)
    k_fac_unpack<float><<<g, 256, 0, t.stream>>>((const float *)t.xfer, t.rows[n], t.J, t.ldf, (float *)t.fac[n]);
  else
    k_fac_unpack<double><<<g, 256, 0, t.stream>>>((const double *)t.xfer, t.rows[n], t.J, t.ldf, (double *)t.fac[n]);
  GTK_CUDA(cudaGetLastError());
  GTK_CUDA(cudaStreamSynchronize(t.stream));
  return 0;
}

int run_delta(DevTensor &t, int mode, void *d_out) {
  if (!t.nnz) return 0;
  if (t.precision != GTK_PREC_PLAIN) return run_mode_tc(t, mode, 2, d_out, nullptr);
  return t.dtype == GTK_F32 ? launch_mode<float, kDelta>(t, mode, d_out, nullptr)
                            : launch_mode<double, kDelta>(t, mode, d_out, nullptr);
}

// the longest row of `mode` (number of nonzeros), for the autotuner's shape key
__global__ void k_row_count(const uint32_t *__restrict__ row_of, uint64_t nnz, uint32_t *__restrict__ cnt) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnz; t += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[row_of[t]], 1u);
}
__global__ void k_max_u32(const uint32_t *__restrict__ a, uint64_t n, uint32_t *__restrict__ out) {
  uint32_t m = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, a[t]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

int run_row_stats(DevTensor &t, int mode, uint32_t *max_count) {
  *max_count = 0;
  if (!t.nnz) return 0;
  if (t.streamed) {  // the host view is sorted by row: the longest run
    const HostVec<uint32_t> &r = t.hp->vidx[mode][mode];
    uint32_t run = 0;
    for (uint64_t i = 0; i < t.nnz; ++i) {
      run = (i && r[i] == r[i - 1]) ? run + 1 : 1;
      *max_count = std::max(*max_count, run);
    }
    return 0;
  }
  uint32_t *cnt = nullptr;
  GTK_CUDA(malloc_retry(&cnt, (t.rows[mode] + 1) * 4));
  int rc = ck(cudaMemsetAsync(cnt, 0, (t.rows[mode] + 1) * 4, t.stream), "memset");
  if (!rc) {
    k_row_count<<<t.num_sms * 8, 256, 0, t.stream>>>(t.vidx[mode][mode], t.nnz, cnt);
    k_max_u32<<<t.num_sms * 4, 256, 0, t.stream>>>(cnt, t.rows[mode], cnt + t.rows[mode]);
    rc = ck(cudaGetLastError(), "row stats");
  }
  if (!rc) rc = ck(cudaMemcpyAsync(max_count, cnt + t.rows[mode], 4, cudaMemcpyDeviceToHost, t.stream), "d2h");
  if (!rc) rc = ck(cudaStreamSynchronize(t.stream), "sync");
  cudaFree(cnt);
  return rc;
}

// Builds G_n (mode n first, the other modes in increasing order, the last one
// fastest, rows padded to ldf) for every mode and uploads them.
int upload_core_perms(DevTensor &t, const void *core_host) {
  const int N = t.N, J = t.J, ldf = t.ldf;
  const uint64_t rows = t.core_n / (uint64_t)J;
  std::vector<unsigned char> buf(rows * ldf * t.vsize);
  for (int n = 0; n < N; ++n) {
    std::fill(buf.begin(), buf.end(), 0);
    int others[kMaxOrder], m = 0;
    for (int k = 0; k < N; ++k)
      if (k != n) others[m++] = k;
    for (uint64_t L = 0; L < t.core_n; ++L) {
      // digits of L over (n, others...) with the last fastest
      uint64_t rem = L, lin = 0;
      uint32_t dig[kMaxOrder];
      for (int k = N - 1; k >= 0; --k) {
        dig[k] = (uint32_t)(rem % J);
        rem /= J;
      }
      uint32_t full[kMaxOrder];
      full[n] = dig[0];
      for (int k = 0; k < m; ++k) full[others[k]] = dig[k + 1];
      for (int k = 0; k < N; ++k) lin = lin * J + full[k];
      const uint64_t row = L / J, col = L % J;
      memcpy(&buf[(row * ldf + col) * t.vsize], (const unsigned char *)core_host + lin * t.vsize, t.vsize);
    }
    GTK_CUDA(cudaMemcpyAsync(t.corep[n], buf.data(), buf.size(), cudaMemcpyHostToDevice, t.stream));
    GTK_CUDA(cudaStreamSynchronize(t.stream));
  }
  return 0;
}


// ---------------------------------------------------------------- batches
// gtk_batch_sweep's fused form: a sweep of many handles in few launches.

static_assert(sizeof(ModeArgs) <= kModeArgsBytes, "the argument block must fit MultiDesc::args");

// the entry i with first[i] <= k < first[i + 1] (first[0] = 0)
__device__ __forceinline__ int slot_of64(const uint64_t *__restrict__ first, int count, uint64_t k) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= k)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

struct ZeroItem {
  double *gram;
  unsigned int *nfb;
};
// every handle's Gram/RHS rows of the level's mode (first: prefix of the doubles),
// its per-mode LU / FP64 list counts, and the gather copies its tensor-core
// kernel reads (pfirst: prefix of their rows)
__global__ void k_batch_zero(const ZeroItem *__restrict__ items, const uint64_t *__restrict__ first, int count,
                             const PadItem *__restrict__ pads, const uint64_t *__restrict__ pfirst, int npads) {
  const uint64_t total = first[count];
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  if (g < (uint64_t)count) items[g].nfb[0] = items[g].nfb[1] = 0u;
  for (uint64_t k = g; k < total; k += stride) {
    const int i = slot_of64(first, count, k);
    items[i].gram[k - first[i]] = 0.0;
  }
  if (npads) {
    const uint64_t ptotal = pfirst[npads];
    for (uint64_t k = g; k < ptotal; k += stride) {
      const int i = slot_of64(pfirst, npads, k);
      pad_row(pads[i], k - pfirst[i]);
    }
  }
}

struct SolveItem {
  const double *gram;
  void *fac;
  int J, E, ldf, prec32, dbl;
  uint32_t *lu_list;     // rows for pivoted LU, count nfb[0]
  uint32_t *fp64_list;   // precision forms: rows for FP64 Cholesky, count nfb[1]
  unsigned int *nfb;
  int *status;
};

// every row of every handle (first: prefix of the row counts): FP32 Cholesky +
// estimate + refinement for the precision forms, FP64 Cholesky for the plain
// form, each as the handle's own solve kernel does it
__global__ void k_solve_multi(const SolveItem *__restrict__ items, const uint64_t *__restrict__ first, int count,
                              double lambda, float cond_max, int slot4) {
  extern __shared__ __align__(16) unsigned char smb[];
  const int T = blockDim.x, tid = threadIdx.x;
  const uint64_t total = first[count];
  for (uint64_t k = (uint64_t)blockIdx.x * T + tid; k < total; k += (uint64_t)gridDim.x * T) {
    const int i = slot_of64(first, count, k);
    const SolveItem &it = items[i];
    const uint64_t row = k - first[i];
    // slot4: every handle of the launch takes the FP32 path, whose scratch
    // interleaves 4-byte elements (element e at e * T + tid); otherwise every
    // thread's scratch sits in 8-byte slots for both paths, since threads of one
    // block may serve an FP32-path and an FP64-path handle at once and
    // interleaved 4- and 8-byte elements would overlap
    if (it.prec32) {
      const int st = slot4 ? T : 2 * T;
      float *sf = reinterpret_cast<float *>(smb) + (slot4 ? tid : 2 * tid);
      if (it.dbl)
        solve_row32<double>(it.gram, row, it.J, it.E, it.ldf, (double *)it.fac, lambda, cond_max, sf, st,
                            it.fp64_list, it.nfb + 1);
      else
        solve_row32<float>(it.gram, row, it.J, it.E, it.ldf, (float *)it.fac, lambda, cond_max, sf, st,
                           it.fp64_list, it.nfb + 1);
    } else {
      double *A = reinterpret_cast<double *>(smb) + tid;
      if (it.dbl)
        solve_row64<double>(it.gram, row, it.J, it.E, it.ldf, (double *)it.fac, lambda, A, T, it.lu_list, it.nfb);
      else
        solve_row64<float>(it.gram, row, it.J, it.E, it.ldf, (float *)it.fac, lambda, A, T, it.lu_list, it.nfb);
    }
  }
}

// the precision forms' FP64 list of every handle: handle i owns CTAs
// [cta_first[i], cta_first[i + 1]) (its share grows with its row count)
__global__ void k_solve_list64_multi(const SolveItem *__restrict__ items, const uint32_t *__restrict__ cta_first,
                                     int count, double lambda) {
  extern __shared__ __align__(16) unsigned char smb[];
  const int T = blockDim.x, tid = threadIdx.x;
  const int i = slot_of(cta_first, count, blockIdx.x);
  const uint32_t sub = blockIdx.x - cta_first[i], per = cta_first[i + 1] - cta_first[i];
  const SolveItem &it = items[i];
  if (!it.prec32) return;
  const uint64_t n = it.nfb[1];
  double *A = reinterpret_cast<double *>(smb) + tid;
  for (uint64_t k = (uint64_t)sub * T + tid; k < n; k += (uint64_t)per * T) {
    if (it.dbl)
      solve_row64<double>(it.gram, it.fp64_list[k], it.J, it.E, it.ldf, (double *)it.fac, lambda, A, T, it.lu_list,
                          it.nfb);
    else
      solve_row64<float>(it.gram, it.fp64_list[k], it.J, it.E, it.ldf, (float *)it.fac, lambda, A, T, it.lu_list,
                         it.nfb);
  }
}

// the pivoted-LU list of every handle, one warp per row, CTA ranges as above
__global__ void k_solve_lu_multi(const SolveItem *__restrict__ items, const uint32_t *__restrict__ cta_first,
                                 int count, double lambda, int maxJ) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int i = slot_of(cta_first, count, blockIdx.x);
  const uint32_t sub = blockIdx.x - cta_first[i], per = cta_first[i + 1] - cta_first[i];
  const SolveItem &it = items[i];
  const int J = it.J;
  double *A = sm + (size_t)wib * ((size_t)maxJ * maxJ + maxJ);
  double *b = A + (size_t)J * J;
  const uint64_t n = it.nfb[0];
  for (uint64_t k = (uint64_t)sub * wpb + wib; k < n; k += (uint64_t)per * wpb) {
    const uint32_t row = it.lu_list[k];
    load_system(it.gram + (uint64_t)row * it.E, J, it.E, lambda, A, b, lane);
    const bool ok = lu_solve(A, b, J, lane);
    if (lane == 0) atomicOr(it.status, ok ? 4 : 1);
    for (int j = lane; j < it.ldf; j += 32) {
      const double v = j < J ? b[j] : 0.0;
      if (it.dbl)
        ((double *)it.fac)[(uint64_t)row * it.ldf + j] = v;
      else
        ((float *)it.fac)[(uint64_t)row * it.ldf + j] = (float)v;
    }
    __syncwarp();
  }
}

struct FitItem {
  int use_gram, dbl;
  const double *gram;  // use_gram: the last mode's Gram/RHS rows
  const void *fac;     // the last mode's factor
  uint64_t rows;
  int J, E, ldf;
  double normsq;
  const void *dstore;    // else: the last mode's stored delta (view order)
  const uint32_t *row_of;
  const void *val;
  uint64_t nnz;
  double *partial;
  int *status;
};

template <class V> __device__ double fit_gram_part(const FitItem &f, uint64_t c, uint64_t nc) {
  double s = 0;
  const V *fac = (const V *)f.fac;
  for (uint64_t r = c * blockDim.x + threadIdx.x; r < f.rows; r += nc * blockDim.x) {
    const double *g = f.gram + r * (uint64_t)f.E;
    const V *a = fac + r * (uint64_t)f.ldf;
    double q = 0;
    int e = 0;
    for (int i = 0; i < f.J; ++i) {
      const double ai = (double)a[i];
      double t = 0.5 * g[e++] * ai;
      for (int j = i + 1; j < f.J; ++j) t += g[e++] * (double)a[j];
      q += ai * (2.0 * g[e++] - 2.0 * t);
    }
    s += q;
  }
  return s;
}
template <class V> __device__ double fit_stored_part(const FitItem &f, uint64_t c, uint64_t nc) {
  double err = 0;
  const V *d0 = (const V *)f.dstore, *fac = (const V *)f.fac, *val = (const V *)f.val;
  for (uint64_t t = c * blockDim.x + threadIdx.x; t < f.nnz; t += nc * blockDim.x) {
    const V *d = d0 + t * (uint64_t)f.J;
    const V *a = fac + (uint64_t)f.row_of[t] * f.ldf;
    V xh = V(0);
    for (int j = 0; j < f.J; ++j) xh += d[j] * a[j];
    const V e = val[t] - xh;
    err += (double)e * (double)e;
  }
  return err;
}

// every handle's fit partial sums (as k_fit_gram / k_fit_stored), CTA ranges per handle
__global__ void __launch_bounds__(256)
    k_fit_multi(const FitItem *__restrict__ items, const uint32_t *__restrict__ cta_first, int count) {
  const int i = slot_of(cta_first, count, blockIdx.x);
  const FitItem &f = items[i];
  const uint64_t c = blockIdx.x - cta_first[i], nc = cta_first[i + 1] - cta_first[i];
  double v;
  if (f.use_gram)
    v = f.dbl ? fit_gram_part<double>(f, c, nc) : fit_gram_part<float>(f, c, nc);
  else
    v = f.dbl ? fit_stored_part<double>(f, c, nc) : fit_stored_part<float>(f, c, nc);
  const double tot = block_sum(v);
  if (threadIdx.x == 0) f.partial[c] = f.use_gram ? (c == 0 ? f.normsq : 0.0) - tot : tot;
}

// per handle: the error sum (also into its own sum slot) and its status word, cleared
__global__ void k_fit_sum_multi(const FitItem *__restrict__ items, const uint32_t *__restrict__ cta_first, int count,
                                double *__restrict__ err_out, int *__restrict__ st_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const FitItem &f = items[i];
  double s = 0;
  for (uint32_t c = 0; c < cta_first[i + 1] - cta_first[i]; ++c) s += f.partial[c];
  f.partial[kFitSumSlot] = s;
  err_out[i] = s;
  const int st = *f.status;
  st_out[i] = st;
  if (st) *f.status = 0;
}

template <class V> static int spec_multi_desc(DevTensor &t, int mode, MultiDesc *d) {
  Launch L;
  bool gp = true;
  choose<V, kUpdate>(L, t, gp);
  if (!L.spec || !L.fn_multi || L.smem > kSmemLimit) return GTK_ERR_UNSUPPORTED;
  if (int rc = prepare_fn(L.fn_multi, L.smem)) return rc;
  ModeArgs a = make_args(t, mode);
  a.gp_in_smem = gp ? 1 : 0;
  a.ref_order = 0;
  a.core = t.core;
  a.dstore = mode == t.N - 1 ? t.dstore : nullptr;  // the plain form's fit reads the last mode's delta
  int per_sm = 0;
  GTK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L.fn_multi, kThreads, L.smem));
  if (per_sm < 1) return fail(GTK_ERR_UNSUPPORTED, "mode kernel does not fit on an SM");
  const uint64_t ntiles = (a.nnz + L.tn - 1) / L.tn;
  d->fn = L.fn_multi;
  d->threads = kThreads;
  d->smem = L.smem;
  d->ctas = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(ntiles, update_grid_cap(t, (uint64_t)per_sm)));
  d->with_image = false;
  d->image = nullptr;
  memcpy(d->args, &a, sizeof(a));
  return 0;
}

struct FusedBatch {
  struct Group {  // one kernel class of one level
    MultiDesc proto;
    int count = 0;
    std::vector<std::unique_ptr<MultiParams>> chunks;  // launches of up to kMultiMax handles
  };
  struct SolveGroup {  // the handles of one level with one rank and one solve path
    size_t items_off = 0, first_off = 0;
    int count = 0, threads = 0, slot4 = 0;
    uint64_t rows = 0;
    size_t smem = 0;
  };
  struct Level {
    int count = 0;  // handles with a mode of this index
    size_t zero_off = 0, zfirst_off = 0, solve_off = 0;
    size_t pad_off = 0, pfirst_off = 0;  // the gather copies to refresh (tensor-core handles with ldf 12)
    int npads = 0;
    uint64_t pad_total = 0;
    size_t list_first_off = 0, lu_first_off = 0;  // CTA ranges of the list passes
    uint32_t list_grid = 0, lu_grid = 0;
    uint64_t zero_total = 0;
    bool any32 = false;
    int maxJ = 1;
    size_t list_smem = 0, lu_smem = 0;
    std::vector<Group> groups;
    std::vector<SolveGroup> solves;
  };
  std::vector<Level> levels;
  int count = 0;
  size_t fit_off = 0, ffirst_off = 0;
  uint32_t fit_grid = 0;
  unsigned char *dev = nullptr;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> ev;  // fork per level, then joins per (level, group)
  int dev_id = 0;
};

void fused_batch_free(FusedBatch *fb) {
  if (!fb) return;
  for (cudaStream_t s : fb->side)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : fb->ev)
    if (e) cudaEventDestroy(e);
  if (fb->dev) cudaFree(fb->dev);
  delete fb;
}

int fused_batch_build(const std::vector<DevTensor *> &ts, FusedBatch **out) {
  *out = nullptr;
  int maxN = 0;
  for (DevTensor *t : ts) {
    if (t->streamed || t->variant == kVarRefOrder || t->J > kThreadSolveMaxJ || !t->nnz) return GTK_ERR_UNSUPPORTED;
    if (!tc_update(*t) && t->dtype != GTK_F32) return GTK_ERR_UNSUPPORTED;
    if (!tc_update(*t)) {
      if (int rc = ensure_dstore(*t)) return rc;
      if (!t->dstore) return GTK_ERR_UNSUPPORTED;
    }
    maxN = std::max(maxN, t->N);
  }
  std::unique_ptr<FusedBatch, void (*)(FusedBatch *)> fb(new FusedBatch(), fused_batch_free);
  fb->count = (int)ts.size();
  GTK_CUDA(cudaGetDevice(&fb->dev_id));
  std::vector<unsigned char> host;  // the device tables, 16-byte aligned pieces
  auto put = [&](const void *p, size_t n) {
    const size_t off = (host.size() + 15) / 16 * 16;
    host.resize(off + n);
    memcpy(host.data() + off, p, n);
    return off;
  };
  for (int n = 0; n < maxN; ++n) {
    FusedBatch::Level L;
    std::vector<ZeroItem> zi;
    std::vector<uint64_t> zf(1, 0);
    std::vector<SolveItem> si;
    std::vector<uint64_t> sf(1, 0);
    std::vector<PadItem> pi;
    std::vector<uint64_t> pf(1, 0);
    size_t max_e64 = 0, max_e32 = 0;
    std::vector<std::pair<MultiDesc, DevTensor *>> descs;
    for (DevTensor *t : ts) {
      if (n >= t->N) continue;
      MultiDesc d;
      int rc = tc_update(*t) ? tc_multi_desc(*t, n, &d) : spec_multi_desc<float>(*t, n, &d);
      if (rc) return rc;
      if (tc_update(*t) && (rc = tc_gather_items(*t, n, &pi, &pf))) return rc;
      descs.emplace_back(d, t);
      const int E = pairs_for(t->J);
      zi.push_back({t->gram, t->nfallback});
      zf.push_back(zf.back() + t->rows[n] * (uint64_t)E);
      SolveItem s;
      s.gram = t->gram;
      s.fac = t->fac[n];
      s.J = t->J;
      s.E = E;
      s.ldf = t->ldf;
      s.prec32 = t->precision != GTK_PREC_PLAIN ? 1 : 0;
      s.dbl = t->dtype == GTK_F64 ? 1 : 0;
      s.lu_list = t->fallback;
      s.fp64_list = t->fallback64;
      s.nfb = t->nfallback;
      s.status = t->status;
      si.push_back(s);
      sf.push_back(sf.back() + t->rows[n]);
      max_e64 = std::max<size_t>(max_e64, (size_t)E * 8);
      if (s.prec32) max_e32 = std::max<size_t>(max_e32, (size_t)(E + 3 * t->J) * 8);  // 8-byte slots
      L.any32 = L.any32 || s.prec32;
      L.maxJ = std::max(L.maxJ, t->J);
    }
    L.count = (int)si.size();
    L.zero_total = zf.back();
    L.zero_off = put(zi.data(), zi.size() * sizeof(ZeroItem));
    L.zfirst_off = put(zf.data(), zf.size() * 8);
    L.npads = (int)pi.size();
    L.pad_total = pf.back();
    if (L.npads) {
      L.pad_off = put(pi.data(), pi.size() * sizeof(PadItem));
      L.pfirst_off = put(pf.data(), pf.size() * 8);
    }
    L.solve_off = put(si.data(), si.size() * sizeof(SolveItem));  // every handle: the list passes
    {
      // list passes: as many CTAs per handle as its rows could need, up to two per
      // SM (the lists' lengths are known only on the device)
      std::vector<uint32_t> lf(1, 0), uf(1, 0);
      for (size_t q = 0; q < si.size(); ++q) {
        const uint64_t rows = sf[q + 1] - sf[q];
        const uint64_t cap = 2 * (uint64_t)ts[0]->num_sms;
        lf.push_back(lf.back() + (uint32_t)std::max<uint64_t>(
                                     1, std::min<uint64_t>((rows + kSolveMultiThreads - 1) / kSolveMultiThreads, cap)));
        uf.push_back(uf.back() + (uint32_t)std::max<uint64_t>(
                                     1, std::min<uint64_t>((rows + kLuMultiThreads / 32 - 1) / (kLuMultiThreads / 32),
                                                           cap)));
      }
      L.list_grid = lf.back();
      L.lu_grid = uf.back();
      L.list_first_off = put(lf.data(), lf.size() * 4);
      L.lu_first_off = put(uf.data(), uf.size() * 4);
    }
    // the row solves by (rank, path): each launch with the shared memory and block
    // size the single-handle solve kernels use for that rank
    {
      std::vector<std::pair<int, int>> keys;
      for (const SolveItem &x : si)
        if (std::find(keys.begin(), keys.end(), std::make_pair(x.J, x.prec32)) == keys.end())
          keys.emplace_back(x.J, x.prec32);
      for (const auto &key : keys) {
        std::vector<SolveItem> g;
        std::vector<uint64_t> gf(1, 0);
        for (size_t q = 0; q < si.size(); ++q)
          if (si[q].J == key.first && si[q].prec32 == key.second) {
            g.push_back(si[q]);
            gf.push_back(gf.back() + (sf[q + 1] - sf[q]));
          }
        FusedBatch::SolveGroup G;
        G.count = (int)g.size();
        G.rows = gf.back();
        G.threads = key.first <= 12 ? 128 : 64;
        G.slot4 = key.second;
        const size_t E = (size_t)pairs_for(key.first);
        G.smem = (size_t)G.threads * (key.second ? (E + 3 * (size_t)key.first) * 4 : E * 8);
        G.items_off = put(g.data(), g.size() * sizeof(SolveItem));
        G.first_off = put(gf.data(), gf.size() * 8);
        L.solves.push_back(G);
      }
    }
    (void)max_e32;
    L.list_smem = kSolveMultiThreads * max_e64;
    L.lu_smem = (size_t)(kLuMultiThreads / 32) * ((size_t)L.maxJ * L.maxJ + L.maxJ) * 8;
    // kernel classes: the same multi-tensor kernel, shared memory and block
    for (auto &pd : descs) {
      const MultiDesc &d = pd.first;
      FusedBatch::Group *g = nullptr;
      for (auto &x : L.groups)
        if (x.proto.fn == d.fn && x.proto.smem == d.smem && x.proto.threads == d.threads) g = &x;
      if (!g) {
        L.groups.emplace_back();
        g = &L.groups.back();
        g->proto = d;
      }
      g->count += 1;
    }
    for (auto &g : L.groups) {
      for (auto &pd : descs) {
        const MultiDesc &d = pd.first;
        if (d.fn != g.proto.fn || d.smem != g.proto.smem || d.threads != g.proto.threads) continue;
        if (g.chunks.empty() || g.chunks.back()->count == kMultiMax) {
          g.chunks.emplace_back(new MultiParams());
          memset(g.chunks.back().get(), 0, sizeof(MultiParams));
        }
        MultiParams &mp = *g.chunks.back();
        memcpy(&mp.args[mp.count], d.args, sizeof(ModeArgs));
        mp.img[mp.count] = d.image;
        mp.first[mp.count + 1] = mp.first[mp.count] + d.ctas;
        mp.count += 1;
      }
    }
    fb->levels.push_back(std::move(L));
  }
  // the fit: each handle's last mode
  {
    std::vector<FitItem> fi;
    std::vector<uint32_t> ff(1, 0);
    for (DevTensor *t : ts) {
      const int m = t->N - 1;
      FitItem f;
      memset(&f, 0, sizeof(f));
      f.use_gram = tc_update(*t) ? 1 : 0;
      f.dbl = t->dtype == GTK_F64 ? 1 : 0;
      f.gram = t->gram;
      f.fac = t->fac[m];
      f.rows = t->rows[m];
      f.J = t->J;
      f.E = pairs_for(t->J);
      f.ldf = t->ldf;
      f.normsq = t->norm * t->norm;
      f.dstore = t->dstore;
      f.row_of = t->vidx[m][m];
      f.val = t->vval[m];
      f.nnz = t->nnz;
      f.partial = t->partial;
      f.status = t->status;
      const uint64_t work = f.use_gram ? f.rows : f.nnz;
      const uint32_t ctas = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(kFitGridMax, (work + 255) / 256));
      fi.push_back(f);
      ff.push_back(ff.back() + ctas);
    }
    fb->fit_grid = ff.back();
    fb->fit_off = put(fi.data(), fi.size() * sizeof(FitItem));
    fb->ffirst_off = put(ff.data(), ff.size() * 4);
  }
  GTK_CUDA(malloc_retry(&fb->dev, std::max<size_t>(host.size(), 16)));
  GTK_CUDA(cudaMemcpy(fb->dev, host.data(), host.size(), cudaMemcpyHostToDevice));
  size_t groups = 0;
  for (auto &L : fb->levels) groups = std::max(groups, L.groups.size());
  const size_t nside = std::min<size_t>(groups, 8);
  fb->side.assign(nside, nullptr);
  for (auto &s : fb->side) GTK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  size_t nev = 0;
  for (auto &L : fb->levels) nev += 1 + L.groups.size();
  fb->ev.assign(nev, nullptr);
  for (auto &e : fb->ev) GTK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (auto &L : fb->levels) {
    for (auto &G : L.solves)
      if (int rc = prepare_fn((const void *)k_solve_multi, G.smem)) return rc;
    if (int rc = prepare_fn((const void *)k_solve_list64_multi, L.list_smem)) return rc;
    if (int rc = prepare_fn((const void *)k_solve_lu_multi, L.lu_smem)) return rc;
  }
  *out = fb.release();
  return 0;
}

int fused_batch_enqueue(FusedBatch *fb, cudaStream_t s, double *err_out, int *status_out, uint64_t *kernels) {
  uint64_t k = 0;
  size_t ev = 0;
  unsigned char *D = fb->dev;
  for (auto &L : fb->levels) {
    const int n = L.count;
    {
      const uint64_t blocks = std::max<uint64_t>(std::max<uint64_t>((L.zero_total + 255) / 256, (L.pad_total + 255) / 256),
                                                 (uint64_t)(n + 255) / 256);
      k_batch_zero<<<(unsigned)std::min<uint64_t>(blocks, 8192), 256, 0, s>>>(
          (const ZeroItem *)(D + L.zero_off), (const uint64_t *)(D + L.zfirst_off), n,
          L.npads ? (const PadItem *)(D + L.pad_off) : nullptr, L.npads ? (const uint64_t *)(D + L.pfirst_off) : nullptr,
          L.npads);
      GTK_CUDA(cudaGetLastError());
      ++k;
    }
    // the update launches, one per kernel class, on side streams
    cudaEvent_t fork = fb->ev[ev++];
    GTK_CUDA(cudaEventRecord(fork, s));
    for (size_t gi = 0; gi < L.groups.size(); ++gi) {
      const FusedBatch::Group &g = L.groups[gi];
      // the classes run side by side on the side streams, as the tensors' own
      // launch chains do in the per-handle graph
      cudaStream_t cs = fb->side.empty() ? s : fb->side[gi % fb->side.size()];
      GTK_CUDA(cudaStreamWaitEvent(cs, fork, 0));
      for (const auto &mp : g.chunks) {
        void *p[] = {mp.get()};
        GTK_CUDA(cudaLaunchKernel(g.proto.fn, dim3(mp->first[mp->count]), dim3(g.proto.threads), p, g.proto.smem, cs));
      }
      cudaEvent_t join = fb->ev[ev++];
      if (cs != s) {
        GTK_CUDA(cudaEventRecord(join, cs));
        GTK_CUDA(cudaStreamWaitEvent(s, join, 0));
      }
      k += g.chunks.size();
    }
    const SolveItem *si = (const SolveItem *)(D + L.solve_off);
    for (const auto &G : L.solves) {
      const unsigned sg =
          (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((G.rows + G.threads - 1) / G.threads, 65535));
      k_solve_multi<<<sg, G.threads, G.smem, s>>>((const SolveItem *)(D + G.items_off),
                                                  (const uint64_t *)(D + G.first_off), G.count, kLambda, kCondMaxFp32,
                                                  G.slot4);
      GTK_CUDA(cudaGetLastError());
      ++k;
    }
    if (L.any32) {
      k_solve_list64_multi<<<L.list_grid, kSolveMultiThreads, L.list_smem, s>>>(
          si, (const uint32_t *)(D + L.list_first_off), n, kLambda);
      GTK_CUDA(cudaGetLastError());
      ++k;
    }
    k_solve_lu_multi<<<L.lu_grid, kLuMultiThreads, L.lu_smem, s>>>(si, (const uint32_t *)(D + L.lu_first_off), n,
                                                                   kLambda, L.maxJ);
    GTK_CUDA(cudaGetLastError());
    ++k;
  }
  const FitItem *fi = (const FitItem *)(D + fb->fit_off);
  const uint32_t *ff = (const uint32_t *)(D + fb->ffirst_off);
  k_fit_multi<<<fb->fit_grid, 256, 0, s>>>(fi, ff, fb->count);
  k_fit_sum_multi<<<(fb->count + 127) / 128, 128, 0, s>>>(fi, ff, fb->count, err_out, status_out);
  GTK_CUDA(cudaGetLastError());
  k += 2;
  if (kernels) *kernels = k;
  return 0;
}

}  // namespace gtk
