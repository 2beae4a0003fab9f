// tc_sweep.cu -- the mode update and the fit with the delta contraction on the
// 5th-generation tensor cores (tcgen05, TMEM accumulators), BF16 or TF32 inputs,
// FP32 accumulation.  The precision form of the sweep; the plain form is sweep.cu.
//
// For mode n with other modes o_1 < ... < o_D (D = N-1 = 2 or 3), per nonzero t:
//   K_t[(j, l)]      = a_{o_{D-1}}[t, j] * a_{o_D}[t, l]                 (J^2, SIMT)
//   T[t, c]          = sum_k K_t[k] * G_n[c, k]      c = (j_n[, j_1])    (tcgen05 GEMM)
//   delta_t[j_n]     = T[t, j_n]                                  (D = 2)
//                    = sum_{j_1} a_{o_1}[t, j_1] * T[t, (j_n, j_1)]  (D = 3, SIMT)
// A tile = 128 nonzeros x K (K = J^2 padded to 16), B = G_n [J^(D-1) padded to 16] x K,
// both K-major in the canonical no-swizzle layout (8-row x 16-byte core matrices,
// K-adjacent core matrices 128 B apart, 8-row groups K*2 B / K*4 B apart).  One
// thread issues the MMAs (K/16 of them for BF16, K/8 for TF32) into a TMEM
// accumulator of 128 lanes x N columns; each warp reads its 32 lanes back with
// tcgen05.ld, finishes delta in registers and reduces its 32 rows of [delta, x]
// into the rows' Gram/RHS (GramMma: mma.sync 3xTF32 per row run).
//
// One CTA barrier per tile: the A tile is complete for the MMAs, every warp has
// read its TMEM lanes of the previous tile, and the CTA agrees on whether the
// previous tile's MMA wait gave up.  Everything after the MMAs is warp-private:
// warp w's delta rows live inside its own 32 rows of the A tile (free once the
// MMAs completed) and its Gram/RHS run reads only them.
//
// Every wait on the MMA-completion mbarrier is bounded: on timeout the CTA sets
// bit 1 of the status word, waits (bounded) for the MMAs it issued, frees its
// TMEM and returns.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "internal.h"
#include "mode_common.cuh"
#include "tc_ptx.cuh"

namespace gtk {
namespace {

constexpr int kTcThreads = 128;  // 4 warps; thread t owns TMEM lane t = nonzero t of the tile
constexpr int kTcFitGrid = 1024;
constexpr uint32_t kWaitLimit = 1u << 24;

template <int J, int D, int PREC> struct TcShape {
  static constexpr int ES = PREC == GTK_PREC_BF16 ? 2 : 4;  // element bytes
  static constexpr int EPC = 16 / ES;                       // elements per 16-byte core row
  static constexpr int KSTEP = 32 / ES;                     // K per MMA instruction (32 bytes)
  static constexpr int KD = J * J;
  static constexpr int KP = (KD + 15) / 16 * 16;
  static constexpr int ND = D == 3 ? J * J : J;
  static constexpr int NP = (ND + 15) / 16 * 16 < 16 ? 16 : (ND + 15) / 16 * 16;
  static constexpr int NCOLS = NP <= 32 ? 32 : NP <= 64 ? 64 : NP <= 128 ? 128 : NP <= 256 ? 256 : 512;
  static constexpr int SBO = (KP / EPC) * 128;  // bytes between 8-row groups
  static constexpr int A_BYTES = kTcThreads * KP * ES;
  static constexpr int B_BYTES = NP * KP * ES;
  // Gram/RHS reduction: on the tensor cores (GramMma) for J <= 16, else GramBlk
  static constexpr bool GRAM_MMA = J <= 16;
  using Gram = std::conditional_t<GRAM_MMA, GramMma<J>, GramBlk<J>>;
  // delta-tile row stride: GramMma's (rows padded by bit 2, GramMma::off), or even for
  // GramBlk's 64-bit pair loads (column J + 1 zero)
  static constexpr int LDD = GRAM_MMA ? gram_mma_ldd(J) : (J + 2) / 2 * 2;
  static constexpr int E = (J + 1) * (J + 2) / 2 - 1;
  static constexpr int OFF_B = A_BYTES;
  // warp w's delta rows reuse its own 32 rows of the A tile (a contiguous
  // 32 * KP * ES bytes in the canonical layout): written only after the tile's
  // MMAs have completed, overwritten by the next A tile only after the warp's
  // reduction has read them
  static constexpr int OFF_DX = 0;
  static constexpr int WARP_A_BYTES = 32 * KP * ES;
  static_assert(32 * LDD * 4 <= WARP_A_BYTES, "a warp's delta rows must fit in its A rows");  // pads included
  static constexpr int OFF_ROWS = (OFF_B + B_BYTES + 15) / 16 * 16;
  static constexpr int OFF_BAR = OFF_ROWS + (kTcThreads * 4 + 15) / 16 * 16;
  static constexpr int OFF_SLOT = OFF_BAR + 16;
  static constexpr int SMEM = OFF_SLOT + 16;
};


// element (r, c) of a warp's delta tile
template <class S> __device__ __forceinline__ int tile_off(int r, int c) {
  if constexpr (S::GRAM_MMA)
    return S::Gram::off(r, c);
  else
    return r * S::LDD + c;
}

// Row r of a factor matrix with LDG floats per row (LDG in {4, 8, 12, 16}), rank
// J.  A warp's gather costs the L1 one wavefront per sector each lane touches, and
// the L1 is the busiest unit of this kernel, so rows are read with as few sector
// accesses as they span: 256-bit loads of 32-byte-aligned rows (LDG 8, 16: the
// factors themselves; LDG 12: the gather copy with 64-byte rows, a 256-bit load
// and a 64-bit (J <= 10) or 128-bit one).  Factor matrices and gather copies start
// on 32-byte boundaries, which run_mode_tc checks.
template <int J, int LDG> struct FRow {
  static_assert(LDG == 4 || LDG == 8 || LDG == 12 || LDG == 16, "factor row stride");
  static constexpr int STRIDE = LDG == 12 ? 16 : LDG;  // floats between the rows read
  float v[LDG];
  __device__ __forceinline__ void load(const float *base, uint32_t r) {
    const float *row = base + (size_t)r * STRIDE;
    if constexpr (LDG == 4) {
      const float4 u = __ldg(reinterpret_cast<const float4 *>(row));
      v[0] = u.x, v[1] = u.y, v[2] = u.z, v[3] = u.w;
    } else if constexpr (LDG == 12) {
      ldg256(row, v);
      if constexpr (J <= 10) {
        const float2 u = __ldg(reinterpret_cast<const float2 *>(row + 8));
        v[8] = u.x, v[9] = u.y, v[10] = v[11] = 0.f;  // entries J.. are never read
      } else {
        const float4 u = __ldg(reinterpret_cast<const float4 *>(row + 8));
        v[8] = u.x, v[9] = u.y, v[10] = u.z, v[11] = u.w;
      }
    } else {
#pragma unroll
      for (int c = 0; c < LDG / 8; ++c) ldg256(row + 8 * c, v + 8 * c);
    }
  }
};

// a handle's gather copies (the listed factors; first: prefix of their rows)
struct PadList {
  PadItem it[kMaxOrder];
  uint64_t first[kMaxOrder + 1];
  int n;
};
__global__ void k_pad_rows(const __grid_constant__ PadList L) {
  const uint64_t total = L.first[L.n];
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (uint64_t)gridDim.x * blockDim.x) {
    int i = 0;
    while (k >= L.first[i + 1]) ++i;
    pad_row(L.it[i], k - L.first[i]);
  }
}

template <int J, int D, int PREC, int KIND>
__device__ __forceinline__ void mode_tc_body(const ModeArgs &a, uint32_t cta, uint32_t nctas) {
  using S = TcShape<J, D, PREC>;
  constexpr int LDG = (J + 3) / 4 * 4;  // factor row stride (floats)
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + S::OFF_BAR);
  uint32_t *slot = reinterpret_cast<uint32_t *>(smem + S::OFF_SLOT);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  TileSmem<float> ts;
  ts.gp = nullptr;
  ts.arow = nullptr;
  ts.dx = reinterpret_cast<float *>(smem + S::OFF_DX + warp * S::WARP_A_BYTES);  // this warp's delta rows
  ts.rows = reinterpret_cast<uint32_t *>(smem + S::OFF_ROWS);
  ts.seg = nullptr;
  ts.pi = ts.pj = nullptr;

  if (warp == 0) {
    tmem_alloc(slot, S::NCOLS);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  // B = G_n as [N rows (j_n[, j_1])] x [K (j, l)], zero padded
  {
    const float *gp = reinterpret_cast<const float *>(a.corep);
    for (int idx = tid; idx < S::NP * (S::KP / S::EPC); idx += kTcThreads) {
      const int n = idx / (S::KP / S::EPC), c = idx % (S::KP / S::EPC);
      float v[8];
#pragma unroll
      for (int e = 0; e < S::EPC; ++e) {
        const int k = c * S::EPC + e;
        v[e] = (n < S::ND && k < S::KD) ? gp[(size_t)(n * J + k / J) * LDG + (k % J)] : 0.f;
      }
      *reinterpret_cast<uint4 *>(smem + S::OFF_B + canon_off(n, c * S::EPC, S::SBO, S::ES)) = pack16<PREC>(v);
    }
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t a_base = smem_u32(smem), b_base = smem_u32(smem + S::OFF_B);
  constexpr uint32_t IDESC = instr_desc(PREC, 128, S::NP);
  const float *facn = reinterpret_cast<const float *>(a.fac[a.mode]);
  double err = 0;
  uint32_t phase = 0;
  bool timed_out = false, late = false;  // late: this thread's last MMA wait gave up
  typename S::Gram gram;
  if (KIND == 0) gram.init(lane);
  // a contiguous range of tiles per CTA, so a warp's running Gram sums follow a row across tiles
  const uint64_t ntiles = (a.nnz + kTcThreads - 1) / kTcThreads;
  const uint64_t per = (ntiles + nctas - 1) / nctas;
  const uint64_t tile_end = min(ntiles, (uint64_t)(cta + 1) * per);
  // inputs of one tile for this thread: its nonzero's row, value and the factor
  // rows (p, q form the Kronecker operand; e1 (D = 3) finishes the contraction).
  // Loaded in two stages a tile apart -- the coordinates two tiles ahead, the
  // factor rows one tile ahead -- so no gather waits on the load of its own index.
  struct TileCrd {
    uint32_t row, ip, iq, ie;
    float x;
  };
  struct TileIn {
    uint32_t row;
    float x;
    FRow<J, LDG> p, q, e1;
  };
  auto load_crd = [&](uint64_t tl, TileCrd &c) {
    const uint64_t b0 = tl * kTcThreads;
    const int n_valid = (int)min((uint64_t)kTcThreads, a.nnz - b0);
    const bool ok = tid < n_valid;
    const uint64_t g = ok ? b0 + tid : b0;
    c.row = ok ? a.coord[a.mode][g] : 0xFFFFFFFFu;
    c.x = ok ? reinterpret_cast<const float *>(a.val)[g] : 0.f;
    c.ip = a.coord[a.others[D - 2]][g];
    c.iq = a.coord[a.others[D - 1]][g];
    c.ie = D == 3 ? a.coord[a.others[0]][g] : 0u;
  };
  auto load_rows = [&](const TileCrd &c, TileIn &in) {
    in.row = c.row;
    in.x = c.x;
    in.p.load(reinterpret_cast<const float *>(a.fac[a.others[D - 2]]), c.ip);
    in.q.load(reinterpret_cast<const float *>(a.fac[a.others[D - 1]]), c.iq);
    if (D == 3) in.e1.load(reinterpret_cast<const float *>(a.fac[a.others[0]]), c.ie);
  };
  TileIn cur;
  TileCrd crd;  // coordinates of the tile after `cur`
  const uint64_t tile_begin = (uint64_t)cta * per;
  if (tile_begin < tile_end) {
    load_crd(tile_begin, crd);
    load_rows(crd, cur);
  }
  if (tile_begin + 1 < tile_end) load_crd(tile_begin + 1, crd);
  for (uint64_t tile = tile_begin; tile < tile_end; ++tile) {
    const uint64_t t0 = tile * kTcThreads;
    const int nv = (int)min((uint64_t)kTcThreads, a.nnz - t0);
    const bool valid = tid < nv;
    const uint64_t gi = valid ? t0 + tid : t0;
    const uint32_t row = cur.row;
    const float x = cur.x;
    const float *p = cur.p.v, *q = cur.q.v;
    // A row `tid`: the Kronecker product p (x) q, rounded to the MMA input type
#pragma unroll
    for (int c = 0; c < S::KP / S::EPC; ++c) {
      float v[8];
      if constexpr (J % 2 == 0) {  // packed FP32x2: k, k + 1 share p[k / J]
#pragma unroll
        for (int e = 0; e < S::EPC; e += 2) {
          const int k = c * S::EPC + e;
          float2 m = make_float2(0.f, 0.f);
          if (k < S::KD) m = __fmul2_rn(make_float2(p[k / J], p[k / J]), make_float2(q[k % J], q[k % J + 1]));
          v[e] = m.x, v[e + 1] = m.y;
        }
      } else {
#pragma unroll
        for (int e = 0; e < S::EPC; ++e) {
          const int k = c * S::EPC + e;
          v[e] = k < S::KD ? p[k / J] * q[k % J] : 0.f;
        }
      }
      *reinterpret_cast<uint4 *>(smem + canon_off(tid, c * S::EPC, S::SBO, S::ES)) = pack16<PREC>(v);
    }
    fence_proxy_async_smem();
    tc_fence_before();
    if (__syncthreads_or(late ? 1 : 0)) {  // the previous tile's wait gave up somewhere in the CTA
      timed_out = true;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int s = 0; s < S::KP / S::KSTEP; ++s)
        mma<PREC>(tmem, smem_desc(a_base + s * 256, 128, S::SBO), smem_desc(b_base + s * 256, 128, S::SBO), IDESC,
                  s > 0 ? 1u : 0u);
      mma_commit(bar);
    }
    // the next tile's loads overlap this tile's MMAs, epilogue and reduction
    TileIn nxt;
    if (tile + 1 < tile_end) load_rows(crd, nxt);
    if (tile + 2 < tile_end) load_crd(tile + 2, crd);
    uint32_t spins = 0;
    bool done = false;
    while (!(done = mbar_try_wait(bar, phase)) && ++spins < kWaitLimit) {
    }
    late = !done;  // voted on at the next barrier; until then the results are discarded anyway
    phase ^= 1u;
    tc_fence_after();
    // epilogue: delta from this thread's TMEM lane
    float delta[J];
#pragma unroll
    for (int j = 0; j < J; ++j) delta[j] = 0.f;
    {
      const float *e1 = cur.e1.v;
      float v[S::NP / 16][16];  // the whole lane of the accumulator: all loads, then one wait
#pragma unroll
      for (int c = 0; c < S::NP / 16; ++c)
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), v[c]);
      tmem_wait_ld();
      if constexpr (D == 3 && J % 2 == 0) {
        // packed FP32x2: columns (j_n, j_1), (j_n, j_1 + 1) against e1[j_1], e1[j_1 + 1]
        float2 acc[J];
#pragma unroll
        for (int j = 0; j < J; ++j) acc[j] = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < S::NP / 16; ++c) {
#pragma unroll
          for (int i = 0; i < 16; i += 2) {
            const int col = c * 16 + i;
            if (col < S::ND)
              acc[col / J] = __ffma2_rn(make_float2(e1[col % J], e1[col % J + 1]),
                                        make_float2(v[c][i], v[c][i + 1]), acc[col / J]);
          }
        }
#pragma unroll
        for (int j = 0; j < J; ++j) delta[j] = acc[j].x + acc[j].y;
      } else {
#pragma unroll
        for (int c = 0; c < S::NP / 16; ++c) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int col = c * 16 + i;
            if (col < S::ND) {
              if (D == 2)
                delta[col] = v[c][i];
              else
                delta[col / J] += e1[col % J] * v[c][i];
            }
          }
        }
      }
    }
    tc_fence_before();
    if (KIND == 0) {
      if constexpr (S::GRAM_MMA) {
        GramMma<J>::store_row(ts.dx, lane, delta, x);
      } else {
#pragma unroll
        for (int j = 0; j < J; ++j) ts.dx[lane * S::LDD + j] = delta[j];
        ts.dx[lane * S::LDD + J] = x;
#pragma unroll
        for (int c = J + 1; c < S::LDD; ++c) ts.dx[lane * S::LDD + c] = 0.f;  // the A tile left data there
      }
      ts.rows[tid] = row;
      __syncwarp();
      const int nw = max(0, min(32, nv - warp * 32));  // this warp's valid nonzeros
      if (a.dstore) {  // the warp's delta rows, contiguous in view order
        float *dst = reinterpret_cast<float *>(a.dstore) + (t0 + warp * 32) * J;
        for (int k = lane; k < nw * J; k += 32) dst[k] = ts.dx[tile_off<S>(k / J, k % J)];
      }
      if constexpr (S::GRAM_MMA)
        gram.run(ts.dx, ts.rows + warp * 32, nw, a.gram, S::E, lane);
      else
        gram.template run<S::LDD>(ts.dx, ts.rows + warp * 32, 0, nw, a.gram, S::E, lane);
      __syncwarp();  // the next A tile overwrites these rows
    } else if (KIND == 1) {
      if (valid) {
        float xh = 0.f;
#pragma unroll
        for (int j = 0; j < J; ++j) xh += delta[j] * __ldg(facn + (size_t)row * LDG + j);
        const float d = x - xh;
        err += (double)d * (double)d;
      }
    } else {
      if (valid) {
        float *out = reinterpret_cast<float *>(a.out) + (size_t)a.vperm[gi] * J;
#pragma unroll
        for (int j = 0; j < J; ++j) out[j] = delta[j];
      }
    }
    cur = nxt;
  }
  // the last tile's wait (a CTA that broke out of the loop agreed already)
  if (!timed_out && __syncthreads_or(late ? 1 : 0)) timed_out = true;
  if (timed_out) {
    if (tid == 0) atomicOr(a.status, 2);
    // the MMAs of the tile whose wait gave up may still run: wait for them (bounded) before freeing TMEM
    uint32_t spins = 0;
    while (!mbar_try_wait(bar, phase ^ 1u) && ++spins < kWaitLimit) {
    }
  }
  if (KIND == 0 && !timed_out) gram.flush(a.gram, S::E, lane);
  if (KIND == 1) {
    const double tot = block_sum(err);
    if (tid == 0) a.partial[cta] = tot;
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, S::NCOLS);
  }
}

template <int J, int D, int PREC, int KIND>
__global__ void __launch_bounds__(kTcThreads) k_mode_tc(ModeArgs a) {
  mode_tc_body<J, D, PREC, KIND>(a, blockIdx.x, gridDim.x);
}

// many tensors of one shape class in one launch (batches), as k_mode_spec_multi
template <int J, int D, int PREC, int KIND>
__global__ void __launch_bounds__(kTcThreads) k_mode_tc_multi(const __grid_constant__ MultiParams p) {
  __shared__ ModeArgs sa;
  uint32_t cta, nctas;
  const ModeArgs &a = multi_select(p, sa, cta, nctas);
  mode_tc_body<J, D, PREC, KIND>(a, cta, nctas);
}

struct TcLaunch {
  const void *fn = nullptr;
  const void *fn_multi = nullptr;  // the multi-tensor form (updates), for batches
  int smem = 0, ncols = 0;
};

template <int J, int D, int PREC, int KIND> TcLaunch tc_entry() {
  using S = TcShape<J, D, PREC>;
  TcLaunch L;
  L.fn = (const void *)k_mode_tc<J, D, PREC, KIND>;
  if constexpr (KIND == 0) L.fn_multi = (const void *)k_mode_tc_multi<J, D, PREC, KIND>;
  L.smem = S::SMEM;
  L.ncols = S::NCOLS;
  return L;
}

// (N, J) shapes with a tensor-core form
template <int PREC, int KIND> bool tc_find(TcLaunch &L, int N, int J) {
#define GTK_TC(NN, JJ)                             \
  if (N == NN && J == JJ) {                        \
    L = tc_entry<JJ, NN - 1, PREC, KIND>();        \
    return true;                                   \
  }
  GTK_TC(3, 4) GTK_TC(3, 8) GTK_TC(3, 10) GTK_TC(3, 12) GTK_TC(3, 16)
  GTK_TC(4, 4) GTK_TC(4, 8) GTK_TC(4, 10) GTK_TC(4, 12)
#undef GTK_TC
  return false;
}

template <int KIND> bool tc_choose(TcLaunch &L, int prec, int N, int J) {
  return prec == GTK_PREC_BF16 ? tc_find<GTK_PREC_BF16, KIND>(L, N, J) : tc_find<GTK_PREC_TF32, KIND>(L, N, J);
}

int tc_prepare_uncached(const TcLaunch &L, int num_sms, int *grid_cap, int *smem_out);

// cached per kernel: no CUDA call after the first launch of a kernel (launches
// recorded into a CUDA graph then issue no attribute calls)
int tc_prepare(const TcLaunch &L, int num_sms, int *grid_cap, int *smem_out) {
  struct Entry {
    const void *fn;
    int sms, cap, smem;
  };
  static std::vector<Entry> cache;
  for (const Entry &e : cache)
    if (e.fn == L.fn && e.sms == num_sms) {
      *grid_cap = e.cap;
      *smem_out = e.smem;
      return 0;
    }
  if (int rc = tc_prepare_uncached(L, num_sms, grid_cap, smem_out)) return rc;
  cache.push_back({L.fn, num_sms, *grid_cap, *smem_out});
  return 0;
}

int tc_prepare_uncached(const TcLaunch &L, int num_sms, int *grid_cap, int *smem_out) {
  // at most 512 / ncols CTAs may share an SM's TMEM: request enough shared
  // memory that no more than that many fit, so tcgen05.alloc never has to wait
  const int max_ctas = 512 / L.ncols;
  const int sm_bytes = 233472;  // 228 KB of shared memory per SM
  int smem = L.smem;
  if ((smem + 1024) * (max_ctas + 1) <= sm_bytes) smem = sm_bytes / (max_ctas + 1) - 1024 + 16;
  GTK_CUDA(cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  GTK_CUDA(cudaFuncSetAttribute(L.fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  cudaFuncAttributes fa;
  GTK_CUDA(cudaFuncGetAttributes(&fa, L.fn));
  // residency from the kernel's own limits (shared memory incl. the 1 KB the
  // driver reserves per CTA, registers, threads); the occupancy API has been
  // seen to under-report it for this kernel
  int per_sm = sm_bytes / (smem + (int)fa.sharedSizeBytes + 1024);
  const int regs = fa.numRegs > 0 ? fa.numRegs : 64;
  per_sm = std::min(per_sm, 65536 / (regs * kTcThreads));
  per_sm = std::min(per_sm, 2048 / kTcThreads);
  if (per_sm < 1) return fail(GTK_ERR_UNSUPPORTED, "tensor-core mode kernel does not fit on an SM");
  if (per_sm > max_ctas) return fail(GTK_ERR_UNSUPPORTED, "tensor-core kernel would oversubscribe TMEM");
  *grid_cap = per_sm * num_sms;
  *smem_out = smem;
  return 0;
}

}  // namespace

// The factor rows the tensor-core kernels gather for `mode` (FRow): the other
// modes' factors, or for ldf = 12 their gather copies, refreshed here (one launch
// on the handle's stream) from the factors as they stand.  FRow's 256-bit loads
// need both on 32-byte boundaries (device allocations are 256-byte aligned;
// checked, not assumed).
static int gather_sources(DevTensor &t, int mode, cudaStream_t s, bool refresh, const void *(&src)[kMaxOrder]) {
  const bool copy = t.ldf == 12;
  PadList L;
  memset(&L, 0, sizeof(L));
  L.first[0] = 0;
  for (int k = 0; k < t.N; ++k) {
    src[k] = t.fac[k];
    if (k == mode) continue;
    if (copy) {
      if (!t.gfac[k]) return fail(GTK_ERR_STATE, "tensor-core form without the factors' gather copies");
      src[k] = t.gfac[k];
      L.it[L.n] = {reinterpret_cast<const float *>(t.fac[k]), reinterpret_cast<float *>(t.gfac[k])};
      L.first[L.n + 1] = L.first[L.n] + t.rows[k];
      ++L.n;
    }
    if (reinterpret_cast<uintptr_t>(src[k]) % 32) return fail(GTK_ERR_STATE, "factor rows not on 32-byte boundaries");
  }
  if (refresh && L.n && L.first[L.n]) {
    const uint64_t blocks = std::min<uint64_t>((L.first[L.n] + 255) / 256, 4ull * t.num_sms);
    k_pad_rows<<<(unsigned)blocks, 256, 0, s>>>(L);
    GTK_CUDA(cudaGetLastError());
    t.launches += 1;
  }
  return 0;
}

int tc_gather_items(const DevTensor &t, int mode, std::vector<PadItem> *items, std::vector<uint64_t> *first) {
  if (t.ldf != 12) return 0;
  for (int k = 0; k < t.N; ++k) {
    if (k == mode) continue;
    if (!t.gfac[k]) return fail(GTK_ERR_STATE, "tensor-core form without the factors' gather copies");
    items->push_back({reinterpret_cast<const float *>(t.fac[k]), reinterpret_cast<float *>(t.gfac[k])});
    first->push_back(first->back() + t.rows[k]);
  }
  return 0;
}

// a handle's mode update as one entry of its class's multi-tensor launch (batches)
int tc_multi_desc(DevTensor &t, int mode, MultiDesc *d) {
  TcLaunch L;
  if (!tc_choose<0>(L, t.precision, t.N, t.J)) {
    if (ts_supported(t.N, t.J, t.dtype, t.precision)) return ts_multi_desc(t, mode, d);
    return GTK_ERR_UNSUPPORTED;
  }
  if (t.dtype != GTK_F32 || !L.fn_multi) return GTK_ERR_UNSUPPORTED;
  const void *src[kMaxOrder];
  if (int rc = gather_sources(t, mode, nullptr, false, src)) return rc;  // the batch refreshes the copies per level
  TcLaunch M = L;
  M.fn = L.fn_multi;  // attributes and residency of the multi-tensor kernel itself
  int cap = 0, smem = 0;
  if (int rc = tc_prepare(M, t.num_sms, &cap, &smem)) return rc;
  ModeArgs a;
  memset(&a, 0, sizeof(a));
  for (int k = 0; k < t.N; ++k) {
    a.coord[k] = t.vidx[mode][k];
    a.fac[k] = src[k];
  }
  a.val = t.vval[mode];
  a.corep = t.corep[mode];
  a.vperm = t.vperm[mode];
  a.gram = t.gram;
  a.partial = t.partial;
  a.status = t.status;
  a.nnz = t.nnz;
  a.N = t.N;
  a.J = t.J;
  a.ldf = t.ldf;
  a.mode = mode;
  a.E = pairs_for(t.J);
  a.ldd = ldd_for(t.J);
  int m = 0;
  for (int k = 0; k < t.N; ++k)
    if (k != mode) a.others[m++] = k;
  const uint64_t ntiles = (t.nnz + kTcThreads - 1) / kTcThreads;
  d->fn = L.fn_multi;
  d->threads = kTcThreads;
  d->smem = (size_t)smem;
  d->ctas = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(ntiles, update_grid_cap(t, (uint64_t)cap / t.num_sms)));
  d->with_image = false;
  d->image = nullptr;
  d->tmem = true;
  static_assert(sizeof(ModeArgs) <= kModeArgsBytes, "argument block");
  memcpy(d->args, &a, sizeof(a));
  return 0;
}

bool tc_supported(int N, int J, int dtype, int prec) {
  if (dtype != GTK_F32 || (prec != GTK_PREC_BF16 && prec != GTK_PREC_TF32)) return false;
  TcLaunch L;
  return tc_choose<0>(L, prec, N, J) || ts_supported(N, J, dtype, prec);
}

// kind 0 update (Gram/RHS into t.gram), 1 fit (partials), 2 delta (out)
int run_mode_tc(DevTensor &t, int mode, int kind, void *out, int *grid_used) {
  TcLaunch L;
  const bool ok = kind == 0   ? tc_choose<0>(L, t.precision, t.N, t.J)
                  : kind == 1 ? tc_choose<1>(L, t.precision, t.N, t.J)
                              : tc_choose<2>(L, t.precision, t.N, t.J);
  if (!ok && ts_supported(t.N, t.J, t.dtype, t.precision)) return run_mode_tcs(t, mode, kind, out, grid_used);
  if (!ok || t.dtype != GTK_F32) return fail(GTK_ERR_UNSUPPORTED, "no tensor-core form for this shape");
  const void *src[kMaxOrder];
  if (int rc = gather_sources(t, mode, t.stream, true, src)) return rc;
  int cap = 0, smem = 0;
  if (int rc = tc_prepare(L, t.num_sms, &cap, &smem)) return rc;
  ModeArgs a;
  memset(&a, 0, sizeof(a));
  const ViewRange vr = view_of(t, mode);
  for (int k = 0; k < t.N; ++k) {
    a.coord[k] = vr.coord[k];
    a.fac[k] = src[k];
  }
  a.val = vr.val;
  a.corep = t.corep[mode];
  a.vperm = t.vperm[mode];
  if (kind == 0)
    a.dstore = out;
  else
    a.out = out;
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
  const uint64_t ntiles = (a.nnz + kTcThreads - 1) / kTcThreads;
  uint64_t grid = std::min<uint64_t>(ntiles, kind == 0 ? update_grid_cap(t, (uint64_t)cap / t.num_sms) : (uint64_t)cap);
  if (kind == 1) grid = std::min<uint64_t>(grid, kTcFitGrid);
  if (grid < 1) grid = 1;
  void *args[] = {&a};
  GTK_CUDA(cudaLaunchKernel(L.fn, dim3((unsigned)grid), dim3(kTcThreads), args, (size_t)smem, t.stream));
  if (grid_used) *grid_used = (int)grid;
  return 0;
}

}  // namespace gtk
