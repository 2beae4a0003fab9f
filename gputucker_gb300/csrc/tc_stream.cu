// tc_stream.cu -- the tensor-core (BF16) form for shapes whose core is too large
// to sit in shared memory as one B operand: N = 5 (J in {4, 8, 12, 16}) and
// N = 4, J = 16.
//
// For mode n with other modes o_1 < ... < o_D (D = N-1 = 3 or 4), per nonzero t:
//   K_t[(j, l)]   = a_{o_{D-1}}[t, j] * a_{o_D}[t, l]                          (A row, SIMT)
//   T[t, c]       = sum_k K_t[k] * G_n[c, k],   c = (j_n, j_1[, j_2])           (tcgen05.mma)
//   delta_t[j_n]  = sum_{j_1} a_{o_1}[t, j_1] T[t, (j_n, j_1)]                    (D = 3)
//                 = sum_{j_1} a_{o_1}[t, j_1] sum_{j_2} a_{o_2}[t, j_2] T[t, (j_n, j_1, j_2)]   (D = 4)
// G_n as the B operand is J^(D-1) columns x J^2 (2 MB in BF16 at N = 5, J = 16).
// An image of it, each chunk of CW columns already in the canonical K-major
// no-swizzle layout, is built once per core upload; per tile of 128 nonzeros the
// chunks stream through two shared-memory buffers by bulk asynchronous copies
// (cp.async.bulk, completion on an mbarrier), and two TMEM accumulators of CW
// columns alternate: while chunk c's MMAs run, every thread reads chunk c-1 from
// TMEM and folds it into delta (the SIMT epilogue above).  One thread issues the
// copies and the MMAs.  Every wait is bounded: on timeout the CTA sets bit 1 of the
// status word, waits (bounded) for its copies and MMAs in flight, frees its TMEM
// and returns.
//
// delta then feeds the same row-segmented Gram/RHS reduction, delta store, fit
// and delta output as the other mode kernels.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"
#include "mode_common.cuh"
#include "tc_ptx.cuh"

namespace gtk {
namespace {

constexpr int kTsThreads = 128;  // thread t owns TMEM lane t = nonzero t of the tile
constexpr int kTsFitGrid = 1024;
constexpr uint32_t kTsWaitLimit = 1u << 24;

constexpr int cpow(int b, int e) { return e == 0 ? 1 : b * cpow(b, e - 1); }
constexpr int cgcd(int a, int b) { return b == 0 ? a : cgcd(b, a % b); }

template <int N, int J> struct TsShape {
  static constexpr int D = N - 1;
  static constexpr int KD = J * J;
  static constexpr int KP = (KD + 15) / 16 * 16;  // K of the MMA (BF16: 16 per instruction)
  static constexpr int C = cpow(J, D - 1);         // columns of G_n as B: (j_n, j_1[, j_2])
  static constexpr int R = cpow(J, D - 2);         // columns per j_n
  // chunk width: <= 128 columns, a multiple of 16 and of J, dividing C
  static constexpr int L = J * 16 / cgcd(J, 16);   // lcm(J, 16): one group of TMEM loads
  static constexpr int CW = (C <= 128) ? C : (128 / L) * L;
  static_assert(C % CW == 0 && CW % L == 0 && CW % 16 == 0, "chunking");
  static constexpr int NCH = C / CW;
  static constexpr int NCOLS = CW <= 32 ? 32 : CW <= 64 ? 64 : CW <= 128 ? 128 : 256;
  static constexpr int SBO = (KP / 8) * 128;  // bytes between 8-row groups (A and B alike)
  static constexpr int A_BYTES = kTsThreads * KP * 2;
  static constexpr int B_BYTES = CW * KP * 2;  // one chunk
  static constexpr int LDD = (J + 2) / 2 * 2;  // even (64-bit pair loads in GramBlk)
  static constexpr int E = (J + 1) * (J + 2) / 2 - 1;
  static constexpr int OFF_B = A_BYTES;
  static constexpr int OFF_OROW = OFF_B + 2 * B_BYTES;
  static constexpr int OFF_DX = OFF_OROW + (D == 4 ? J * kTsThreads * 4 : 0);
  static constexpr int OFF_ROWS = OFF_DX + (kTsThreads * LDD * 4 + 15) / 16 * 16;
  static constexpr int OFF_BAR = OFF_ROWS + (kTsThreads * 4 + 15) / 16 * 16;  // full[2], done[2]
  static constexpr int OFF_SLOT = OFF_BAR + 32;
  static constexpr int SMEM = OFF_SLOT + 16;
  static_assert(B_BYTES % 16 == 0 && OFF_B % 16 == 0 && OFF_OROW % 16 == 0, "16-byte bulk copies");
  static_assert(SMEM <= 227 * 1024, "shared memory");
  static_assert(2 * NCOLS <= 512, "TMEM");
};

// B image of mode n: chunk c, column r (< CW), k -> canonical offset; BF16 of
// G_n[c*CW + r][k], G_n[col][(j, l)] = corep[(col * J + j) * ldf + l]
template <int N, int J>
__global__ void k_build_bimg(const float *__restrict__ corep, int ldf, unsigned char *__restrict__ img) {
  using S = TsShape<N, J>;
  const int total = S::NCH * S::CW * (S::KP / 8);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int chunk = idx / (S::CW * (S::KP / 8));
    const int rem = idx % (S::CW * (S::KP / 8));
    const int r = rem / (S::KP / 8), kc = rem % (S::KP / 8);
    const int col = chunk * S::CW + r;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = kc * 8 + e;
      v[e] = k < S::KD ? corep[((size_t)col * J + k / J) * ldf + (k % J)] : 0.f;
    }
    *reinterpret_cast<uint4 *>(img + (size_t)chunk * S::B_BYTES + canon_off(r, kc * 8, S::SBO, 2)) =
        pack16<GTK_PREC_BF16>(v);
  }
}

__device__ __forceinline__ bool wait_bounded(uint64_t *bar, uint32_t parity) {
  uint32_t spins = 0;
  bool done = false;
  while (!(done = mbar_try_wait(bar, parity)) && ++spins < kTsWaitLimit) {
  }
  return done;
}

template <int N, int J, int KIND>
__device__ __forceinline__ void mode_tcs_body(const ModeArgs &a, const unsigned char *__restrict__ bimg, uint32_t cta,
                                              uint32_t nctas) {
  using S = TsShape<N, J>;
  constexpr int D = S::D;
  constexpr int LDG = (J + 3) / 4 * 4;  // factor row stride (floats)
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + S::OFF_BAR);
  uint64_t *done = full + 2;
  uint32_t *slot = reinterpret_cast<uint32_t *>(smem + S::OFF_SLOT);
  float *orow = reinterpret_cast<float *>(smem + S::OFF_OROW);
  const int tid = threadIdx.x, warp = tid >> 5;
  TileSmem<float> ts;
  ts.gp = nullptr;
  ts.arow = nullptr;
  ts.dx = reinterpret_cast<float *>(smem + S::OFF_DX);
  ts.rows = reinterpret_cast<uint32_t *>(smem + S::OFF_ROWS);
  ts.seg = nullptr;
  ts.pi = ts.pj = nullptr;

  if (warp == 0) {
    tmem_alloc(slot, 2 * S::NCOLS);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (int b = 0; b < 4; ++b) mbar_init(full + b, 1);
    fence_mbar_init();
  }
  for (int c = J + 1; c < S::LDD; ++c) ts.dx[tid * S::LDD + c] = 0.f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t a_base = smem_u32(smem), b_base = smem_u32(smem + S::OFF_B);
  constexpr uint32_t IDESC = instr_desc(GTK_PREC_BF16, 128, S::CW);
  const float *facn = reinterpret_cast<const float *>(a.fac[a.mode]);
  double err = 0;
  GramBlk<J> gram;
  if (KIND == 0) gram.init(tid & 31);

  const uint64_t ntiles = (a.nnz + kTsThreads - 1) / kTsThreads;
  const uint64_t per = (ntiles + nctas - 1) / nctas;
  const uint64_t tile_begin = (uint64_t)cta * per;
  const uint64_t tile_end = min(ntiles, tile_begin + per);
  const uint64_t total = tile_begin < tile_end ? (tile_end - tile_begin) * S::NCH : 0;
  // thread 0's record of what is in flight: the last chunk copied and the last MMA group
  int64_t last_copy = -1, last_mma = -1;
  auto issue_copy = [&](uint64_t q) {  // chunk q % NCH into buffer q & 1
    const int b = (int)(q & 1);
    mbar_expect_tx(full + b, S::B_BYTES);
    bulk_g2s(smem + S::OFF_B + b * S::B_BYTES, bimg + (size_t)(q % S::NCH) * S::B_BYTES, S::B_BYTES, full + b);
    last_copy = (int64_t)q;
  };
  if (tid == 0 && total) issue_copy(0);

  const float *fo1 = reinterpret_cast<const float *>(a.fac[a.others[0]]);
  const float *fo2 = reinterpret_cast<const float *>(a.fac[a.others[1]]);
  const float *fp = reinterpret_cast<const float *>(a.fac[a.others[D - 2]]);
  const float *fq = reinterpret_cast<const float *>(a.fac[a.others[D - 1]]);
  uint64_t q = 0;  // chunks consumed by this CTA
  bool timed_out = false;
  for (uint64_t tile = tile_begin; tile < tile_end && !timed_out; ++tile) {
    const uint64_t t0 = tile * kTsThreads;
    const int nv = (int)min((uint64_t)kTsThreads, a.nnz - t0);
    const bool valid = tid < nv;
    const uint64_t gi = valid ? t0 + tid : t0;
    const uint32_t row = valid ? a.coord[a.mode][gi] : 0xFFFFFFFFu;
    const float x = valid ? reinterpret_cast<const float *>(a.val)[gi] : 0.f;
    // the inner epilogue factor row (o_1 for D = 3, o_2 for D = 4); the outer one (D = 4) to shared memory
    float inner[LDG];
    {
      const float4 *fi = reinterpret_cast<const float4 *>((D == 3 ? fo1 : fo2) +
                                                          (size_t)a.coord[a.others[D == 3 ? 0 : 1]][gi] * LDG);
#pragma unroll
      for (int c = 0; c < LDG / 4; ++c) {
        const float4 u = __ldg(fi + c);
        inner[4 * c] = u.x, inner[4 * c + 1] = u.y, inner[4 * c + 2] = u.z, inner[4 * c + 3] = u.w;
      }
      if (D == 4) {
        const float *fr = fo1 + (size_t)a.coord[a.others[0]][gi] * LDG;
#pragma unroll
        for (int j = 0; j < J; ++j) orow[j * kTsThreads + tid] = __ldg(fr + j);
      }
    }
    // A row `tid`: the Kronecker product p (x) q in BF16
    {
      float p[LDG], qv[LDG];
      const float4 *pp = reinterpret_cast<const float4 *>(fp + (size_t)a.coord[a.others[D - 2]][gi] * LDG);
      const float4 *qq = reinterpret_cast<const float4 *>(fq + (size_t)a.coord[a.others[D - 1]][gi] * LDG);
#pragma unroll
      for (int c = 0; c < LDG / 4; ++c) {
        const float4 u = __ldg(pp + c), w = __ldg(qq + c);
        p[4 * c] = u.x, p[4 * c + 1] = u.y, p[4 * c + 2] = u.z, p[4 * c + 3] = u.w;
        qv[4 * c] = w.x, qv[4 * c + 1] = w.y, qv[4 * c + 2] = w.z, qv[4 * c + 3] = w.w;
      }
#pragma unroll
      for (int c = 0; c < S::KP / 8; ++c) {
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int k = c * 8 + e;
          v[e] = k < S::KD ? p[k / J] * qv[k % J] : 0.f;
        }
        *reinterpret_cast<uint4 *>(smem + canon_off(tid, c * 8, S::SBO, 2)) = pack16<GTK_PREC_BF16>(v);
      }
    }
#pragma unroll
    for (int j = 0; j < J; ++j) ts.dx[tid * S::LDD + j] = 0.f;
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
    // fold TMEM chunk c (buffer b) into delta
    auto epilogue = [&](int c, int b) {
      constexpr int G16 = S::L / 16, RG = S::L / J, NG = S::CW / S::L;
      float acc = 0.f;
      int jn_cur = (c * S::CW) / S::R;
#pragma unroll 1
      for (int g = 0; g < NG; ++g) {
        float v[G16][16];
#pragma unroll
        for (int h = 0; h < G16; ++h)
          tmem_ld16(tmem + lane_off + (uint32_t)(b * S::NCOLS + g * S::L + h * 16), v[h]);
        tmem_wait_ld();
#pragma unroll
        for (int k = 0; k < RG; ++k) {
          float s = 0.f;
#pragma unroll
          for (int o = 0; o < J; ++o) s += v[(k * J + o) / 16][(k * J + o) % 16] * inner[o];
          const int rho = (c * S::CW + g * S::L) / J + k;  // rest-row: J consecutive columns
          int jn;
          float w;
          if (D == 3) {
            jn = rho;
            w = 1.f;
          } else {
            jn = rho / J;
            w = orow[(rho % J) * kTsThreads + tid];
          }
          if (jn != jn_cur) {  // warp-uniform
            ts.dx[tid * S::LDD + jn_cur] += acc;
            acc = 0.f;
            jn_cur = jn;
          }
          acc += w * s;
        }
      }
      ts.dx[tid * S::LDD + jn_cur] += acc;
    };
    for (int c = 0; c < S::NCH; ++c, ++q) {
      bool bad = false;
      if (tid == 0) {
        const int b = (int)(q & 1);
        if (!wait_bounded(full + b, (uint32_t)((q >> 1) & 1))) {
          bad = true;
        } else {
          tc_fence_after();
#pragma unroll
          for (int s = 0; s < S::KP / 16; ++s)
            mma<GTK_PREC_BF16>(tmem + (uint32_t)(b * S::NCOLS), smem_desc(a_base + s * 256, 128, S::SBO),
                               smem_desc(b_base + b * S::B_BYTES + s * 256, 128, S::SBO), IDESC, s > 0 ? 1u : 0u);
          mma_commit(done + b);
          last_mma = (int64_t)q;
          // the next chunk goes into the other buffer once its last reader (MMA q-1) is done
          if (q + 1 < total) {
            if (q >= 1 && !wait_bounded(done + ((q - 1) & 1), (uint32_t)(((q - 1) >> 1) & 1)))
              bad = true;
            else
              issue_copy(q + 1);
          }
        }
      }
      __syncwarp();  // warp 0 reconverges before the warp-wide TMEM loads
      if (c >= 1) {
        const uint64_t p = q - 1;
        if (!wait_bounded(done + (p & 1), (uint32_t)((p >> 1) & 1))) {
          bad = true;
        } else {
          tc_fence_after();
          epilogue(c - 1, (int)(p & 1));
        }
      }
      tc_fence_before();
      if (__syncthreads_or(bad ? 1 : 0)) {
        timed_out = true;
        break;
      }
      tc_fence_after();
    }
    if (timed_out) break;
    {  // the last chunk of the tile
      const uint64_t p = q - 1;
      bool bad = false;
      if (!wait_bounded(done + (p & 1), (uint32_t)((p >> 1) & 1))) {
        bad = true;
      } else {
        tc_fence_after();
        epilogue(S::NCH - 1, (int)(p & 1));
      }
      tc_fence_before();
      if (__syncthreads_or(bad ? 1 : 0)) {
        timed_out = true;
        break;
      }
      tc_fence_after();
    }
    // delta_t is in ts.dx[tid][0, J)
    if (KIND == 0) {
      ts.dx[tid * S::LDD + J] = x;
      ts.rows[tid] = row;
      __syncthreads();
      if (a.dstore) {
        float *dst = reinterpret_cast<float *>(a.dstore) + t0 * J;
        for (int k = tid; k < nv * J; k += kTsThreads) dst[k] = ts.dx[(k / J) * S::LDD + (k % J)];
      }
      gram.template run<S::LDD>(ts.dx, ts.rows, warp * 32, min(warp * 32 + 32, nv), a.gram, S::E, tid & 31);
      __syncthreads();
    } else if (KIND == 1) {
      if (valid) {
        float xh = 0.f;
#pragma unroll
        for (int j = 0; j < J; ++j) xh += ts.dx[tid * S::LDD + j] * __ldg(facn + (size_t)row * LDG + j);
        const float d = x - xh;
        err += (double)d * (double)d;
      }
      __syncthreads();
    } else {
      if (valid) {
        float *out = reinterpret_cast<float *>(a.out) + (size_t)a.vperm[gi] * J;
#pragma unroll
        for (int j = 0; j < J; ++j) out[j] = ts.dx[tid * S::LDD + j];
      }
      __syncthreads();
    }
  }
  if (timed_out) {
    // report, then let the copies and MMAs this CTA started finish before its
    // shared memory and TMEM go away (bounded again)
    if (tid == 0) {
      atomicOr(a.status, 2);
      if (last_copy >= 0) wait_bounded(full + (last_copy & 1), (uint32_t)((last_copy >> 1) & 1));
      if (last_mma >= 0) wait_bounded(done + (last_mma & 1), (uint32_t)((last_mma >> 1) & 1));
    }
  } else {
    if (KIND == 0) gram.flush(a.gram, S::E, tid & 31);
    if (KIND == 1) {
      const double tot = block_sum(err);
      if (tid == 0) a.partial[cta] = tot;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * S::NCOLS);
  }
}

template <int N, int J, int KIND>
__global__ void __launch_bounds__(kTsThreads, 1) k_mode_tcs(ModeArgs a, const unsigned char *__restrict__ bimg) {
  mode_tcs_body<N, J, KIND>(a, bimg, blockIdx.x, gridDim.x);
}

// many tensors of one shape class in one launch (batches), as k_mode_spec_multi
template <int N, int J, int KIND>
__global__ void __launch_bounds__(kTsThreads, 1) k_mode_tcs_multi(const __grid_constant__ MultiParams p) {
  __shared__ ModeArgs sa;
  uint32_t cta, nctas;
  const unsigned char *img = nullptr;
  const ModeArgs &a = multi_select(p, sa, cta, nctas, &img);
  mode_tcs_body<N, J, KIND>(a, img, cta, nctas);
}

struct TsLaunch {
  const void *fn = nullptr;
  const void *fn_multi = nullptr;  // the multi-tensor form (updates), for batches
  void (*build)(const float *, int, unsigned char *, cudaStream_t) = nullptr;
  int smem = 0, ncols = 0;
  size_t img_bytes = 0;
};

template <int N, int J> void build_img(const float *corep, int ldf, unsigned char *img, cudaStream_t s) {
  using S = TsShape<N, J>;
  const int total = S::NCH * S::CW * (S::KP / 8);
  k_build_bimg<N, J><<<(total + 255) / 256, 256, 0, s>>>(corep, ldf, img);
}

template <int N, int J, int KIND> TsLaunch ts_entry() {
  using S = TsShape<N, J>;
  TsLaunch L;
  L.fn = (const void *)k_mode_tcs<N, J, KIND>;
  if constexpr (KIND == 0) L.fn_multi = (const void *)k_mode_tcs_multi<N, J, KIND>;
  L.build = build_img<N, J>;
  L.smem = S::SMEM;
  L.ncols = 2 * S::NCOLS;
  L.img_bytes = (size_t)S::NCH * S::B_BYTES;
  return L;
}

template <int KIND> bool ts_find(TsLaunch &L, int N, int J) {
#define GTK_TS(NN, JJ)                  \
  if (N == NN && J == JJ) {             \
    L = ts_entry<NN, JJ, KIND>();       \
    return true;                        \
  }
  GTK_TS(4, 16) GTK_TS(5, 4) GTK_TS(5, 8) GTK_TS(5, 12) GTK_TS(5, 16)
#undef GTK_TS
  return false;
}

bool ts_choose(TsLaunch &L, int kind, int N, int J) {
  return kind == 0 ? ts_find<0>(L, N, J) : kind == 1 ? ts_find<1>(L, N, J) : ts_find<2>(L, N, J);
}

// once per kernel: shared-memory attribute and residency (TMEM: 512 / ncols CTAs per SM
// at most, enforced by requesting enough shared memory)
int ts_prepare(const TsLaunch &L, int num_sms, int *grid_cap, int *smem_out) {
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
  const int max_ctas = 512 / L.ncols;
  const int sm_bytes = 233472;
  int smem = L.smem;
  if ((smem + 1024) * (max_ctas + 1) <= sm_bytes) smem = sm_bytes / (max_ctas + 1) - 1024 + 16;
  GTK_CUDA(cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  GTK_CUDA(cudaFuncSetAttribute(L.fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  cudaFuncAttributes fa;
  GTK_CUDA(cudaFuncGetAttributes(&fa, L.fn));
  int per_sm = sm_bytes / (smem + (int)fa.sharedSizeBytes + 1024);
  const int regs = fa.numRegs > 0 ? fa.numRegs : 64;
  per_sm = std::min(per_sm, 65536 / (regs * kTsThreads));
  per_sm = std::min(per_sm, 2048 / kTsThreads);
  if (per_sm < 1) return fail(GTK_ERR_UNSUPPORTED, "streamed tensor-core kernel does not fit on an SM");
  if (per_sm > max_ctas) return fail(GTK_ERR_UNSUPPORTED, "streamed tensor-core kernel would oversubscribe TMEM");
  *grid_cap = per_sm * num_sms;
  *smem_out = smem;
  cache.push_back({L.fn, num_sms, *grid_cap, smem});
  return 0;
}

}  // namespace

// a handle's mode update as one entry of its class's multi-tensor launch (batches)
int ts_multi_desc(DevTensor &t, int mode, MultiDesc *d) {
  TsLaunch L;
  if (t.dtype != GTK_F32 || t.precision != GTK_PREC_BF16 || !ts_choose(L, 0, t.N, t.J) || !L.fn_multi)
    return GTK_ERR_UNSUPPORTED;
  if (!t.bimg[mode]) return fail(GTK_ERR_STATE, "core image missing (set the precision after the core)");
  TsLaunch M = L;
  M.fn = L.fn_multi;
  int cap = 0, smem = 0;
  if (int rc = ts_prepare(M, t.num_sms, &cap, &smem)) return rc;
  ModeArgs a;
  memset(&a, 0, sizeof(a));
  for (int k = 0; k < t.N; ++k) {
    a.coord[k] = t.vidx[mode][k];
    a.fac[k] = t.fac[k];
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
  const uint64_t ntiles = (t.nnz + kTsThreads - 1) / kTsThreads;
  d->fn = L.fn_multi;
  d->threads = kTsThreads;
  d->smem = (size_t)smem;
  d->ctas = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(ntiles, update_grid_cap(t, (uint64_t)cap / t.num_sms)));
  d->with_image = true;
  d->image = t.bimg[mode];
  d->tmem = true;
  static_assert(sizeof(ModeArgs) <= kModeArgsBytes, "argument block");
  memcpy(d->args, &a, sizeof(a));
  return 0;
}

bool ts_supported(int N, int J, int dtype, int prec) {
  TsLaunch L;
  return dtype == GTK_F32 && prec == GTK_PREC_BF16 && ts_choose(L, 0, N, J);
}

// (Re)build the B images of every mode from the device core permutations.
int ts_build_images(DevTensor &t) {
  TsLaunch L;
  if (!ts_choose(L, 0, t.N, t.J)) return 0;
  for (int n = 0; n < t.N; ++n) {
    if (!t.bimg[n]) {
      if (int rc = dalloc(t, (void **)&t.bimg[n], L.img_bytes)) return rc;
    }
    L.build(reinterpret_cast<const float *>(t.corep[n]), t.ldf, t.bimg[n], t.stream);
    GTK_CUDA(cudaGetLastError());
  }
  GTK_CUDA(cudaStreamSynchronize(t.stream));
  return 0;
}

// kind 0 update, 1 fit (partials), 2 delta (out)
int run_mode_tcs(DevTensor &t, int mode, int kind, void *out, int *grid_used) {
  TsLaunch L;
  if (t.dtype != GTK_F32 || t.precision != GTK_PREC_BF16 || !ts_choose(L, kind, t.N, t.J))
    return fail(GTK_ERR_UNSUPPORTED, "no streamed tensor-core form for this shape and precision");
  if (!t.bimg[mode]) return fail(GTK_ERR_STATE, "core image missing (set the precision after the core)");
  int cap = 0, smem = 0;
  if (int rc = ts_prepare(L, t.num_sms, &cap, &smem)) return rc;
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
  const uint64_t ntiles = (a.nnz + kTsThreads - 1) / kTsThreads;
  uint64_t grid = std::min<uint64_t>(ntiles, kind == 0 ? update_grid_cap(t, (uint64_t)cap / t.num_sms) : (uint64_t)cap);
  if (kind == 1) grid = std::min<uint64_t>(grid, kTsFitGrid);
  if (grid < 1) grid = 1;
  const unsigned char *img = t.bimg[mode];
  void *args[] = {&a, &img};
  GTK_CUDA(cudaLaunchKernel(L.fn, dim3((unsigned)grid), dim3(kTsThreads), args, (size_t)smem, t.stream));
  if (grid_used) *grid_used = (int)grid;
  return 0;
}

}  // namespace gtk
