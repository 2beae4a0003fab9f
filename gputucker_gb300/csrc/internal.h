// internal.h -- shared declarations of the gputucker_gb300 library (not installed).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "gputucker_gb300.h"

// NVTX range around a host-side stage (create, mode update, fit, sweep, batch
// sweep, warm-start training, core update): a no-op unless a profiler is attached
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

namespace gtk {

constexpr int kMaxOrder = GTK_MAX_ORDER;
constexpr int kMaxRank = GTK_MAX_RANK;
// update-kernel variants (the autotuner's search space)
constexpr int kVarAuto = -1;    // specialised NPT = 2 (plain) / tensor cores (precision forms)
constexpr int kVarSpec2 = 0;    // specialised SIMT kernel, 2 nonzeros per thread
constexpr int kVarSpec1 = 1;    // specialised SIMT kernel, 1 nonzero per thread
constexpr int kVarGeneric = 2;  // runtime-(N, J) SIMT kernel
constexpr int kVarTc = 3;       // tcgen05 kernel (precision forms)
constexpr int kVarRefOrder = 4;  // generic kernel, delta in the reference's operation order
static_assert(kVarAuto == GTK_VARIANT_AUTO && kVarSpec2 == GTK_VARIANT_SIMT2 && kVarSpec1 == GTK_VARIANT_SIMT1 &&
                  kVarGeneric == GTK_VARIANT_GENERIC && kVarTc == GTK_VARIANT_TENSOR_CORE &&
                  kVarRefOrder == GTK_VARIANT_REFERENCE_ORDER,
              "variant codes of the C ABI");
constexpr int kFitSumSlot = 1024;  // partial[] index of a fit's error sum
// constants.hpp:18 declares kLambda as a double initialised from the float
// literal 0.0001f, so its value is float(1e-4) widened to double.
constexpr double kLambda = (double)0.0001f;

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

inline int ck(cudaError_t e, const char *what) { return e == cudaSuccess ? 0 : cuda_fail(e, what); }

#define GTK_CUDA(call)                                      \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return ::gtk::cuda_fail(e_, #call); \
  } while (0)

// glibc rand(): TYPE_3 additive feedback generator.  r[i] = r[i-31] + r[i-3]
// (mod 2^32) after a Lehmer (16807 mod 2^31-1, Schrage) seeding of 31 words and
// 310 discarded outputs; rand() returns r[i] >> 1.  srand(0) behaves as srand(1).
struct GlibcRand {
  uint32_t ring[31];
  uint64_t i = 0;
  explicit GlibcRand(uint32_t seed) { reseed(seed); }
  void reseed(uint32_t seed) {
    int32_t r[34];
    r[0] = (int32_t)(seed == 0 ? 1u : seed);
    for (int k = 1; k < 31; ++k) {
      long long w = r[k - 1];
      long long hi = w / 127773, lo = w % 127773;
      w = 16807 * lo - 2836 * hi;
      if (w < 0) w += 2147483647;
      r[k] = (int32_t)w;
    }
    for (int k = 31; k < 34; ++k) r[k] = r[k - 31];
    for (int k = 3; k < 34; ++k) ring[k % 31] = (uint32_t)r[k];
    i = 34;
    for (int k = 34; k < 344; ++k) step();
  }
  inline uint32_t step() {
    uint32_t v = ring[i % 31] + ring[(i - 3) % 31];
    ring[i % 31] = v;
    ++i;
    return v;
  }
  inline int next() { return (int)(step() >> 1); }
  // frand<T>(0, 1) of the reference (helper.hpp:99)
  template <class T> inline T frand01() { return (T(1) - T(0)) * (static_cast<T>(next()) / 2147483647) + T(0); }
  // advance by k draws without producing them (hostpart.cpp)
  void jump(uint64_t k);
};

}  // namespace gtk

// Host-side parsed tensor: one block of global 0-based coordinates.
// std::allocator whose value-less construct leaves the element uninitialised:
// resize() of a large host array costs no serial zeroing pass, and its pages are
// first touched by the threads that fill them
template <class T> struct NoInitAlloc : std::allocator<T> {
  template <class U> struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <class U> NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
  template <class U> void construct(U *p) noexcept { ::new ((void *)p) U; }
  template <class U, class... A> void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
};
template <class T> using HostVec = std::vector<T, NoInitAlloc<T>>;

struct gtk_coo {
  int N = 0;
  int dtype = GTK_F32;
  uint64_t nnz = 0;
  uint32_t dims[GTK_MAX_ORDER] = {};
  HostVec<uint32_t> idx[GTK_MAX_ORDER];
  HostVec<float> vf;
  HostVec<double> vd;
  uint64_t draws = 0;  // rand() draws consumed by lines without a value
  bool pinned = false;
  const void *values() const { return dtype == GTK_F32 ? (const void *)vf.data() : (const void *)vd.data(); }
};

namespace gtk {

// A contiguous range of a mode view that the mode kernels read in place of the
// resident view (the streamed layout's staging buffers)
struct ViewRange {
  const uint32_t *coord[kMaxOrder];
  const void *val;
  uint64_t nnz;
};

// The blocked arrays and mode views in host memory (the streamed layout), with
// the same definitions and layouts as the device arrays of DevTensor below;
// vval/blk_val hold value_t bytes.
struct HostPart {
  HostVec<uint64_t> blk_ptr;
  HostVec<uint32_t> blk_idx[kMaxOrder];
  HostVec<unsigned char> blk_val;
  HostVec<uint64_t> count[kMaxOrder];
  HostVec<uint32_t> where[kMaxOrder];
  HostVec<uint32_t> vidx[kMaxOrder][kMaxOrder];
  HostVec<unsigned char> vval[kMaxOrder];
  bool pinned = false;  // vidx/vval page-locked (cudaHostRegister)
};

// Device buffers of one resident tensor.  Layout in HBM:
//   blocked arrays (block-major, the reference's Block order):
//     blk_ptr[nblk+1] u64, blk_idx[n][nnz] u32 local coords, blk_val[nnz] V,
//     count[n][nblk*(bd_n+1)] u64, where[n][nnz] u32
//   mode-n views (stable sort by global row i_n of the block-major order, so a
//   row's nonzeros appear in (block_id, position) order, the order in which
//   ComputingBC visits them): vidx[n][k][nnz] u32 global coords, vval[n][nnz] V
//   factor n: rows_n = P_n*bd_n rows of ldf values (ldf = J rounded to 16 bytes)
//   core: J^N linear; corep[n]: the core with mode n moved to the front,
//   rows of J values padded to ldf, i.e. [J^(N-1)][ldf]
//   gram: rows_max x E doubles, E = (J+1)(J+2)/2 - 1 (upper triangle of the
//   Gram matrix then the right-hand side, see sweep.cu)
struct DevTensor {
  int dev = 0;
  cudaStream_t stream = nullptr;
  int dtype = GTK_F32;
  size_t vsize = 4;
  int N = 0, J = 0, ldf = 0, E = 0;
  uint64_t nnz = 0, nblk = 1;
  uint32_t dims[kMaxOrder] = {}, P[kMaxOrder] = {}, bd[kMaxOrder] = {};
  uint64_t rows[kMaxOrder] = {};
  uint64_t core_n = 1;
  double norm = 0;
  double norm_ref = 0;  // the reference's ||X||: value_t serial sum of x^2 in input order, sqrt in value_t
  bool norm_ref_ready = false;  // norm_ref is summed when the reference-order variant is first selected
  void *val_in = nullptr;       // the values in input order (the order of that sum)
  void *xfer = nullptr;         // [max rows][J] value_t: factors in the slab layout on their way to/from the host
  int precision = GTK_PREC_PLAIN;
  bool have_factors = false, have_core = false;

  std::vector<uint64_t> h_blk_ptr;  // host copy of blk_ptr
  uint64_t *blk_ptr = nullptr;
  uint32_t *blk_idx[kMaxOrder] = {};
  void *blk_val = nullptr;
  uint64_t *count[kMaxOrder] = {};
  uint32_t *where[kMaxOrder] = {};
  unsigned char *bimg[kMaxOrder] = {};  // streamed tensor-core form: core image per mode (tc_stream.cu)
  uint32_t *vidx[kMaxOrder][kMaxOrder] = {};
  void *vval[kMaxOrder] = {};
  uint32_t *vperm[kMaxOrder] = {};  // view position -> block-major position
  void *fac[kMaxOrder] = {};
  // f32 handles with ldf = 12 (J = 9..12): the factors again with 64-byte rows,
  // which the tensor-core kernels gather from (refreshed before each launch)
  void *gfac[kMaxOrder] = {};
  void *core = nullptr;
  void *corep[kMaxOrder] = {};
  double *gram = nullptr;
  double *partial = nullptr;  // fit partial sums
  int *status = nullptr;      // device status words (numeric flags)
  int num_sms = 0;
  uint64_t lu_fallbacks = 0;
  bool fit_from_store = false;  // dstore holds the delta of the last mode's update
  bool fit_from_gram = false;   // gram holds the last mode's Gram/RHS and fac[N-1] its solution
  bool dstore_failed = false;
  void *dstore = nullptr;       // [nnz][J] value_t, view order of the last mode
  uint32_t *fallback = nullptr; // rows re-solved by pivoted LU
  uint32_t *fallback64 = nullptr; // precision form: rows re-solved in FP64
  // [0] rows of the current mode listed for LU, [1] for FP64 Cholesky;
  // [2] FP64 and [3] LU rows since creation or gtk_solve_counters' last reset
  unsigned int *nfallback = nullptr;
  uint64_t launches = 0;        // kernels launched by the sweep entry points
  int variant = -1;             // update kernel: kVarAuto or one the autotuner picked
  int ctas_per_sm = 0;          // update kernels' grids: CTAs per SM (0: as many as fit)
  bool use_graph = false;       // gtk_sweep replays a captured CUDA graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  uint64_t graph_kernels = 0;  // sweeps in which some row needed the pivoted-LU fallback

  // profiling
  bool prof = false;
  double prof_ms[4] = {};
  uint64_t prof_n[4] = {};
  // gtk_create_blocks, CUDA events on the stream: host-to-device upload of the
  // COO, then the partition and segmenting kernels (ms)
  double create_upload_ms = 0, create_kernels_ms = 0;
  bool create_direct = false;  // the partition read the host COO in place (no upload)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, tev0 = nullptr, tev1 = nullptr;

  std::vector<std::pair<void *, size_t>> allocs;  // device blocks of the handle and their sizes
  uint64_t bytes = 0;

  // Streamed layout, for tensors whose resident layout does not fit the device
  // memory the handle may use: the blocked arrays and the mode views stay in host
  // memory (hp), and every pass over a mode view streams it through two device
  // staging buffers of `chunk` nonzeros -- copies on copy_stream, kernels on
  // stream, events hand each buffer back and forth.  Factors, core, Gram/RHS and
  // the fit's partial sums stay resident.
  bool streamed = false;
  std::unique_ptr<HostPart> hp;
  uint64_t chunk = 0;
  uint32_t *stage_idx[2][kMaxOrder] = {};
  void *stage_val[2] = {};
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t stage_ready[2] = {}, stage_free[2] = {};
  double stream_copy_bytes = 0;  // host-to-device bytes the streamed passes moved
  const ViewRange *range = nullptr;  // set around a launch: the kernels read this range, not the resident view
};

// the view a mode kernel reads: the resident view of `mode`, or t.range
inline ViewRange view_of(const DevTensor &t, int mode) {
  if (t.range) return *t.range;
  ViewRange r;
  for (int k = 0; k < kMaxOrder; ++k) r.coord[k] = t.vidx[mode][k];
  r.val = t.vval[mode];
  r.nnz = t.nnz;
  return r;
}

// device memory helpers (api.cpp)
int dalloc(DevTensor &t, void **p, size_t bytes);
// Process-wide cache of device blocks: a freed block is kept (up to half of its
// device's memory) and handed back to the next request of the same size on that
// device, so that repeated handles of one shape neither unmap nor map memory.
// dev_alloc: nullptr on failure (after clearing the cache and retrying once);
// dev_free: the work using p must have finished.
void *dev_alloc(int dev, size_t bytes);
void dev_free(int dev, void *p, size_t bytes);
uint64_t dev_cached_bytes(int dev);
void dev_cache_clear(int dev);  // dev < 0: every device
// cudaMalloc on the current device; when it fails, the blocks the cache holds
// for that device go back to the driver and the allocation is tried once more
// (so memory this process keeps cached never makes an allocation fail)
cudaError_t malloc_retry(void **p, size_t bytes);
template <class T> inline cudaError_t malloc_retry(T **p, size_t bytes) {
  return malloc_retry(reinterpret_cast<void **>(p), bytes);
}
// a device buffer freed (cudaFree) on every return path
struct DevBuf {
  void *p = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes) { return malloc_retry(&p, bytes); }
  template <class T> T *as() const { return static_cast<T *>(p); }
};

// ---- batches: kernels shared by many handles per launch (gtk_batch_sweep)
constexpr size_t kModeArgsBytes = 320;
// the grid cap of an update kernel that fits per_sm CTAs on an SM: the handle's
// CTAs per SM (gtk_set_ctas_per_sm, the autotuner's tile-shape choice) where set
inline uint64_t update_grid_cap(const DevTensor &t, uint64_t per_sm) {
  if (t.ctas_per_sm > 0 && (uint64_t)t.ctas_per_sm < per_sm) per_sm = (uint64_t)t.ctas_per_sm;
  return per_sm * (uint64_t)t.num_sms;
}

// Gather copies of FP32 factor rows of 12 floats (48 bytes, every other one off
// a 32-byte boundary) as 64-byte rows, which the tensor-core kernels read with
// one 256-bit load and one 64- or 128-bit load: two sector accesses per row
// instead of three 16-byte loads' three.
struct PadItem {
  const float *src;  // [rows][12]
  float *dst;        // [rows][16]
};
// the copies the tensor-core kernels of `mode` read (none unless ldf = 12),
// appended with the prefix of their row counts (tc_sweep.cu)
int tc_gather_items(const DevTensor &t, int mode, std::vector<PadItem> *items, std::vector<uint64_t> *first);

// The 31-value windows r[s - 31 .. s - 1] at the chunk starts s = c * len,
// c = 0 .. chunks-1, of the stream continuing from g (hostpart.cpp): chunk c's
// draws follow from out[31 c ..] by the recurrence alone
void glibc_chunk_states(const GlibcRand &g, uint64_t len, int chunks, uint32_t *out);
// coefficients of x^(j step) mod (x^31 - x^28 - 1), j = 0 .. count-1, 31 words
// each: applied to a chunk's start window they give the window j steps of
// `step` draws further on (the device splits each chunk by them)
void glibc_step_polys(uint64_t step, int count, uint32_t *out);
// the device generation's split: chunks of kFacChunk draws (start windows from
// the host), each cut into kFacSplit pieces of one thread each
constexpr uint64_t kFacChunk = 16384;
constexpr int kFacSplit = 16;
// the draws gtk_init_random places in the factors (tucker.cuh:84-97), generated on
// the device from chunk states of g, written into the zeroed factors (sweep.cu);
// afterwards g stands after the factors' draws
int factor_init_device(DevTensor &t, GlibcRand &g);

// One handle's mode update in the form its kernel class's multi-tensor kernel takes
struct MultiDesc {
  const void *fn = nullptr;              // k_mode_*_multi<...> of the class
  int threads = 0;
  size_t smem = 0;
  uint32_t ctas = 0;                     // this handle's share of the grid
  bool with_image = false;               // streamed-core tensor-core class: a core-image table too
  bool tmem = false;                     // the class allocates tensor memory (launched one class at a time)
  const unsigned char *image = nullptr;
  alignas(16) unsigned char args[kModeArgsBytes];  // the kernel's argument block for this handle
};
int tc_multi_desc(DevTensor &t, int mode, MultiDesc *d);  // tc_sweep.cu (defers to tc_stream.cu's classes)
int ts_multi_desc(DevTensor &t, int mode, MultiDesc *d);  // tc_stream.cu
// A sweep of many handles in few launches (sweep.cu): per mode index one kernel
// zeroing every handle's Gram/RHS, one multi-tensor update launch per kernel
// class (classes on side streams), one batched row solve and its FP64 and LU
// list passes; then one fit launch and one reduction that also gathers the
// status words.  fused_batch_build returns GTK_ERR_UNSUPPORTED when some handle
// has no multi-tensor form (the caller then launches per handle).
struct FusedBatch;
int fused_batch_build(const std::vector<DevTensor *> &ts, FusedBatch **out);
int fused_batch_enqueue(FusedBatch *fb, cudaStream_t s, double *err_out, int *status_out, uint64_t *kernels);
void fused_batch_free(FusedBatch *fb);

// partition.cu
int build_partition(DevTensor &t, const gtk_coo &coo);
// hostpart.cpp: the blocked arrays and mode views of the streamed layout, in t.hp
int build_host_partition(DevTensor &t, const gtk_coo &coo);
// GTK_ERR_UNSUPPORTED for a streamed handle: `what` needs the resident views
int need_resident(const DevTensor &t, const char *what);

// sweep.cu
int upload_core_perms(DevTensor &t, const void *core_host);
int run_update_mode(DevTensor &t, int mode);
int run_fit(DevTensor &t, double *fit);
int run_delta(DevTensor &t, int mode, void *d_delta_blockmajor);
int run_sweep(DevTensor &t, double *fit);
int run_fit_enqueue(DevTensor &t);
double fit_from_err(const DevTensor &t, double err);  // fit = 1 - sqrt(err) / ||X|| (the variant's formula)  // the fit kernels only; the sum lands in partial[kFitSumSlot]
int run_row_stats(DevTensor &t, int mode, uint32_t *max_count);
int ensure_dstore(DevTensor &t);
int ensure_norm_ref(DevTensor &t);  // the reference's value_t norm from val_in (host, serial)
int put_core(DevTensor &t, const void *core_host);  // core in linear order -> core, corep, images
int run_update_core(DevTensor &t, int cg_iters, int *iters_run, double *rel_residual);
int run_validate(DevTensor &t, uint64_t *violations);  // GTK_VALIDATE_CHECKS counters
int factor_to_host(const DevTensor &t, int n, void *slabs);    // device [rows][ldf] -> host [rows][J]
int factor_from_host(DevTensor &t, int n, const void *slabs);  // host [rows][J] -> device [rows][ldf]
void fit_invalidate(DevTensor &t);         // factors, core or kernel changed: the next fit recomputes
void fit_after_sweep(DevTensor &t);        // what a replayed sweep leaves for its fit
bool sweep_needs_dstore(const DevTensor &t);  // a sweep's fit (or its variant) reads the delta store
void drop_graph(DevTensor &t);
// tc_sweep.cu: the tensor-core (BF16 / TF32) form; kind 0 update, 1 fit, 2 delta
// tensor-core form exists for (N, J, value type, precision): tc_sweep.cu's kernels
// (core as one B operand) or tc_stream.cu's (core streamed, BF16)
bool tc_supported(int N, int J, int dtype, int prec);
int run_mode_tc(DevTensor &t, int mode, int kind, void *out, int *grid_used);
// tc_stream.cu
bool ts_supported(int N, int J, int dtype, int prec);
int ts_build_images(DevTensor &t);
int run_mode_tcs(DevTensor &t, int mode, int kind, void *out, int *grid_used);
// per-kernel CUDA-event timing on the handle's stream (kind 0 delta+gram, 1 solve, 2 fit)
int prof_begin(DevTensor &t, cudaEvent_t *a);
int prof_end(DevTensor &t, int kind, cudaEvent_t a);
int prof_resolve(DevTensor &t);

}  // namespace gtk

struct gtk_tensor : gtk::DevTensor {};
