// batch.cu -- many independent tensors per sweep, and the kernel autotuner.
//
// No reference counterpart (the reference decomposes one tensor per process).
//
// Batching: gtk_batch_sweep runs one ALS sweep of every tensor of the batch as
// ONE CUDA-graph launch.  The graph is captured on the second sweep (the first
// runs eagerly, so that every kernel's attributes and every buffer exist before
// capture): a fork event on the batch's stream, then each tensor's sweep (every
// mode's update kernels and the fit kernels) on the tensor's own stream, then a
// join, then one gather kernel that copies every tensor's error sum and status
// word into the batch's arrays (and clears the status words).  The tensors'
// chains are independent branches of the graph, so the GPU runs them
// concurrently -- small tensors, which alone cannot fill 152 SMs, fill it
// together -- and a sweep of the whole batch costs one graph launch and one
// device-to-host copy.  GTK_BATCH_FUSED=1 puts the fused sweep in the graph
// instead (sweep.cu, FusedBatch: per mode index one launch per kernel class for
// every handle of the class, batched row solves, one fit): 30x fewer launches,
// measured 8-30 % slower, since it waits for every handle at each mode.  Each tensor keeps its own kernels (chosen by order, rank
// and precision, or by the autotuner), its own buffers and its own results;
// factor and core contents may change between sweeps.  A change of a tensor's
// precision or kernel variant is seen at the next sweep, which captures anew.
//
// Autotuner: gtk_autotune times the update-kernel variants that apply to a
// tensor (specialised SIMT with 2 or 1 nonzeros per thread, tensor cores for the
// precision forms) on its mode-0 update, restores the factor it touched, keeps
// the fastest, and caches the choice by (order, rank, value type, precision,
// log2 of the mean row length, log2 of the longest row over the mean): tensors
// of the same shape class reuse it without timing.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"

struct gtk_batch {
  int dev = 0;
  int count = 0;
  std::vector<gtk_tensor *> ts;
  std::vector<std::tuple<int, int, int>> captured;  // (precision, variant, CTAs per SM) of each tensor in the graph
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  // device: count error-sum pointers, count status pointers; count doubles + count ints out
  void **d_tab = nullptr;
  void *d_out = nullptr;
  std::vector<unsigned char> h_out;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  uint64_t graph_kernels = 0;
  bool warmed = false;
  gtk::FusedBatch *fused = nullptr;  // the few-launch form of the sweep, when every handle has one
  uint64_t fused_kernels = 0;
  std::vector<std::pair<int, int>> fused_for;  // (precision, variant) of each handle the plan was built for
};

using namespace gtk;

namespace {

__global__ void k_batch_gather(const double *const *__restrict__ errp, int *const *__restrict__ statp, int count,
                               double *__restrict__ err, int *__restrict__ st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  err[i] = *errp[i];
  const int s = *statp[i];
  st[i] = s;
  if (s) *statp[i] = 0;
}

using TuneKey = std::tuple<int, int, int, int, int, int>;
std::mutex g_tune_mutex;
std::map<TuneKey, std::pair<int, int>> g_tune_cache;  // (variant, CTAs per SM)

int time_update(gtk_tensor *t, int variant, int ctas, void *save, size_t bytes, double *ms) {
  t->variant = variant;
  t->ctas_per_sm = ctas;
  // warm (the first launch of a kernel sets its attributes), then time two updates of mode 0
  if (int rc = run_update_mode(*t, 0)) return rc;
  GTK_CUDA(cudaMemcpyAsync(t->fac[0], save, bytes, cudaMemcpyDeviceToDevice, t->stream));
  cudaEvent_t a, b;
  GTK_CUDA(cudaEventCreate(&a));
  if (int rc = ck(cudaEventCreate(&b), "cudaEventCreate")) {
    cudaEventDestroy(a);
    return rc;
  }
  int rc = ck(cudaEventRecord(a, t->stream), "cudaEventRecord");
  for (int k = 0; k < 2 && !rc; ++k) {
    rc = run_update_mode(*t, 0);
    if (!rc) rc = ck(cudaMemcpyAsync(t->fac[0], save, bytes, cudaMemcpyDeviceToDevice, t->stream), "restore");
  }
  if (!rc) rc = ck(cudaEventRecord(b, t->stream), "cudaEventRecord");
  if (!rc) rc = ck(cudaEventSynchronize(b), "cudaEventSynchronize");
  float m = 0;
  if (!rc) rc = ck(cudaEventElapsedTime(&m, a, b), "cudaEventElapsedTime");
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = m;
  return rc;
}

double *out_err(gtk_batch *b) { return static_cast<double *>(b->d_out); }
int *out_status(gtk_batch *b) { return reinterpret_cast<int *>(out_err(b) + b->count); }

int batch_enqueue(gtk_batch *b) {
  if (b->fused) {
    uint64_t k = 0;
    if (int rc = fused_batch_enqueue(b->fused, b->stream, out_err(b), out_status(b), &k)) return rc;
    b->fused_kernels = k;
    return 0;
  }
  GTK_CUDA(cudaEventRecord(b->fork, b->stream));
  for (int i = 0; i < b->count; ++i) {
    gtk_tensor *t = b->ts[i];
    GTK_CUDA(cudaStreamWaitEvent(t->stream, b->fork, 0));
    for (int n = 0; n < t->N; ++n)
      if (int rc = run_update_mode(*t, n)) return rc;
    if (int rc = run_fit_enqueue(*t)) return rc;
    GTK_CUDA(cudaEventRecord(b->joins[i], t->stream));
    GTK_CUDA(cudaStreamWaitEvent(b->stream, b->joins[i], 0));
  }
  const double *const *errp = reinterpret_cast<const double *const *>(b->d_tab);
  int *const *statp = reinterpret_cast<int *const *>(b->d_tab + b->count);
  k_batch_gather<<<(b->count + 255) / 256, 256, 0, b->stream>>>(errp, statp, b->count, out_err(b), out_status(b));
  GTK_CUDA(cudaGetLastError());
  return 0;
}

void drop_batch_graph(gtk_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
  b->graph_kernels = 0;
  // the fused plan holds each handle's kernel choice: rebuilt (eagerly) at the next sweep
  if (b->fused) {
    cudaStreamSynchronize(b->stream);
    fused_batch_free(b->fused);
    b->fused = nullptr;
    b->warmed = false;
  }
}

int capture(gtk_batch *b) {
  std::vector<uint64_t> l0;
  std::vector<bool> prof;
  for (gtk_tensor *t : b->ts) {
    l0.push_back(t->launches);
    prof.push_back(t->prof);
    t->prof = false;  // no profiling events inside the graph
  }
  GTK_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = batch_enqueue(b);
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
  uint64_t kernels = b->fused ? b->fused_kernels : 1;  // fused: every kernel; else the gather kernel + the handles'
  for (int i = 0; i < b->count; ++i) {
    if (!b->fused) kernels += b->ts[i]->launches - l0[i];
    b->ts[i]->launches = l0[i];
    b->ts[i]->prof = prof[i];
  }
  if (rc || ec != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc ? rc : cuda_fail(ec, "cudaStreamEndCapture");
  }
  b->graph = g;
  const cudaError_t ei = cudaGraphInstantiate(&b->gexec, b->graph, 0);
  if (ei != cudaSuccess) {
    drop_batch_graph(b);
    return cuda_fail(ei, "cudaGraphInstantiate");
  }
  b->graph_kernels = kernels;
  b->captured.clear();
  for (gtk_tensor *t : b->ts) b->captured.emplace_back(t->precision, t->variant, t->ctas_per_sm);
  return 0;
}

}  // namespace

extern "C" {

int gtk_set_kernel_variant(gtk_tensor *t, int variant) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (variant < GTK_VARIANT_AUTO || variant > GTK_VARIANT_REFERENCE_ORDER) return fail(GTK_ERR_ARG, "unknown variant");
  if (variant == GTK_VARIANT_TENSOR_CORE && t->precision == GTK_PREC_PLAIN)
    return fail(GTK_ERR_UNSUPPORTED, "the tensor-core variant needs a precision form (gtk_set_precision)");
  if (variant == GTK_VARIANT_REFERENCE_ORDER) {
    if (int rc = need_resident(*t, "the reference-order variant")) return rc;
    if (int rc = ensure_norm_ref(*t)) return rc;
  }
  t->variant = variant;
  fit_invalidate(*t);
  drop_graph(*t);
  return 0;
}

int gtk_get_kernel_variant(const gtk_tensor *t, int *variant) {
  if (!t || !variant) return fail(GTK_ERR_ARG, "null argument");
  *variant = t->variant;
  return 0;
}

int gtk_set_ctas_per_sm(gtk_tensor *t, int ctas) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (ctas < 0) return fail(GTK_ERR_ARG, "CTAs per SM must be >= 0");
  t->ctas_per_sm = ctas;
  drop_graph(*t);
  return 0;
}

int gtk_get_ctas_per_sm(const gtk_tensor *t, int *ctas) {
  if (!t || !ctas) return fail(GTK_ERR_ARG, "null argument");
  *ctas = t->ctas_per_sm;
  return 0;
}

int gtk_autotune(gtk_tensor *t, int *variant) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (!t->have_factors || !t->have_core) return fail(GTK_ERR_STATE, "factors and core are not initialised");
  GTK_CUDA(cudaSetDevice(t->dev));
  try {
    uint32_t maxc = 0;
    if (int rc = run_row_stats(*t, 0, &maxc)) return rc;
    const double mean = (double)t->nnz / (double)std::max<uint64_t>(1, t->rows[0]);
    const int b_mean = (int)std::floor(std::log2(std::max(1.0, mean)));
    const int b_skew = (int)std::floor(std::log2(std::max(1.0, maxc / std::max(1.0, mean))));
    const TuneKey key{t->N, t->J, t->dtype, t->precision, b_mean, b_skew};
    int best = kVarAuto, best_ctas = 0;
    bool cached = false;
    {
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) {
        best = it->second.first;
        best_ctas = it->second.second;
        cached = true;
      }
    }
    if (!cached && t->nnz) {
      std::vector<int> cands;
      if (t->precision != GTK_PREC_PLAIN && tc_supported(t->N, t->J, t->dtype, t->precision)) cands.push_back(kVarTc);
      cands.push_back(kVarSpec2);
      cands.push_back(kVarSpec1);
      const size_t bytes = t->rows[0] * (size_t)t->ldf * t->vsize;
      void *save = nullptr;
      GTK_CUDA(malloc_retry(&save, bytes));
      int rc = ck(cudaMemcpyAsync(save, t->fac[0], bytes, cudaMemcpyDeviceToDevice, t->stream), "save");
      const bool prof = t->prof;
      t->prof = false;
      // tile shape: the grid at as many CTAs per SM as fit (0), and at 2 and 1 --
      // fewer, longer-lived CTAs (more tiles each, fewer contending for an SM's
      // shared memory, L1 and tensor pipe); values at or above what fits equal 0
      const int ctas_cands[] = {0, 2, 1};
      double best_ms = 1e300;
      for (int v : cands)
        for (int c : ctas_cands) {
          if (rc) break;
          double ms = 0;
          rc = time_update(t, v, c, save, bytes, &ms);
          if (!rc && ms < best_ms * 0.97) {  // a shape other than the first must win by 3 %
            best_ms = ms;
            best = v;
            best_ctas = c;
          }
        }
      t->prof = prof;
      const int rc2 = ck(cudaMemcpyAsync(t->fac[0], save, bytes, cudaMemcpyDeviceToDevice, t->stream), "restore");
      const int rc3 = ck(cudaStreamSynchronize(t->stream), "cudaStreamSynchronize");
      cudaFree(save);
      if (rc || rc2 || rc3) {
        t->variant = kVarAuto;
        t->ctas_per_sm = 0;
        drop_graph(*t);
        return rc ? rc : rc2 ? rc2 : rc3;
      }
      // the timed updates may have flagged singular rows on the restored factor's
      // behalf; the status word belongs to the caller's next real update
      GTK_CUDA(cudaMemset(t->status, 0, 4));
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      g_tune_cache[key] = {best, best_ctas};
    }
    t->variant = best;
    t->ctas_per_sm = best_ctas;
    fit_invalidate(*t);
    drop_graph(*t);
    if (variant) *variant = best;
    return 0;
  } catch (std::exception &e) {
    return fail(GTK_ERR_ARG, e.what());
  }
}

int gtk_batch_create(gtk_tensor *const *tensors, int count, gtk_batch **out) {
  if (!tensors || count < 1 || !out) return fail(GTK_ERR_ARG, "need at least one tensor");
  for (int i = 0; i < count; ++i) {
    if (!tensors[i] || tensors[i]->dev != tensors[0]->dev)
      return fail(GTK_ERR_ARG, "every tensor of a batch must exist and share one device");
    if (int rc = need_resident(*tensors[i], "a batch")) return rc;
    for (int k = 0; k < i; ++k)
      if (tensors[k] == tensors[i]) return fail(GTK_ERR_ARG, "a tensor appears twice in the batch");
  }
  gtk_batch *b = new gtk_batch();
  b->dev = tensors[0]->dev;
  b->count = count;
  b->ts.assign(tensors, tensors + count);
  auto bail = [&](int rc) {
    gtk_batch_destroy(b);
    return rc;
  };
  if (int rc = ck(cudaSetDevice(b->dev), "cudaSetDevice")) return bail(rc);
  if (int rc = ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate")) return bail(rc);
  if (int rc = ck(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate")) return bail(rc);
  b->joins.assign(count, nullptr);
  for (int i = 0; i < count; ++i)
    if (int rc = ck(cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming), "cudaEventCreate"))
      return bail(rc);
  std::vector<void *> tab(2 * (size_t)count);
  for (int i = 0; i < count; ++i) {
    tab[i] = b->ts[i]->partial + kFitSumSlot;
    tab[count + i] = b->ts[i]->status;
  }
  const size_t out_bytes = (size_t)count * (sizeof(double) + sizeof(int));
  if (int rc = ck(malloc_retry(&b->d_tab, tab.size() * sizeof(void *)), "cudaMalloc")) return bail(rc);
  if (int rc = ck(malloc_retry(&b->d_out, out_bytes), "cudaMalloc")) return bail(rc);
  if (int rc = ck(cudaMemcpy(b->d_tab, tab.data(), tab.size() * sizeof(void *), cudaMemcpyHostToDevice), "H2D"))
    return bail(rc);
  b->h_out.resize(out_bytes);
  *out = b;
  return 0;
}

int gtk_batch_sweep(gtk_batch *b, double *fits) {
  NvtxRange nvtx("gtk_batch_sweep");
  if (!b) return fail(GTK_ERR_ARG, "null batch");
  GTK_CUDA(cudaSetDevice(b->dev));
  for (gtk_tensor *t : b->ts)
    if (!t->have_factors || !t->have_core) return fail(GTK_ERR_STATE, "factors and core are not initialised");
  try {
    if (b->gexec) {
      for (int i = 0; i < b->count && b->gexec; ++i)
        if (b->captured[i] != std::make_tuple(b->ts[i]->precision, b->ts[i]->variant, b->ts[i]->ctas_per_sm))
          drop_batch_graph(b);
    }
    if (b->fused) {
      for (int i = 0; i < b->count && b->fused; ++i)
        if (b->fused_for[i] != std::make_pair(b->ts[i]->precision, b->ts[i]->variant)) drop_batch_graph(b);
    }
    if (!b->warmed) {
      for (gtk_tensor *t : b->ts)
        if (sweep_needs_dstore(*t))
          if (int rc = ensure_dstore(*t)) return rc;
      // GTK_BATCH_FUSED=1: the few-launch form where every handle has one; by
      // default one launch chain per handle (measured faster: the handles' chains
      // overlap freely, while the fused form waits for every handle at each mode)
      const char *fz = getenv("GTK_BATCH_FUSED");
      if (!b->fused && fz && *fz == '1') {
        std::vector<DevTensor *> ts(b->ts.begin(), b->ts.end());
        const int rc = fused_batch_build(ts, &b->fused);
        if (rc && rc != GTK_ERR_UNSUPPORTED) return rc;
        if (rc) set_error("");
        b->fused_for.clear();
        for (gtk_tensor *t : b->ts) b->fused_for.emplace_back(t->precision, t->variant);
      }
      if (int rc = batch_enqueue(b)) return rc;
      if (b->fused) b->graph_kernels = b->fused_kernels;  // the same launches the graph will hold
      b->warmed = true;
    } else {
      if (!b->gexec)
        if (int rc = capture(b)) return rc;
      GTK_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    }
    for (gtk_tensor *t : b->ts) fit_after_sweep(*t);
    GTK_CUDA(cudaMemcpyAsync(b->h_out.data(), b->d_out, b->h_out.size(), cudaMemcpyDeviceToHost, b->stream));
    GTK_CUDA(cudaStreamSynchronize(b->stream));
    const double *err = reinterpret_cast<const double *>(b->h_out.data());
    const int *st = reinterpret_cast<const int *>(err + b->count);
    int worst = 0;
    for (int i = 0; i < b->count; ++i) {
      gtk_tensor *t = b->ts[i];
      if (st[i] & 4) t->lu_fallbacks += 1;
      worst |= st[i];
      if (fits) fits[i] = fit_from_err(*t, err[i]);
    }
    if (worst & 2) return fail(GTK_ERR_CUDA, "a tensor-core kernel gave up waiting for its MMAs");
    if (worst & 1) return fail(GTK_ERR_NUMERIC, "a row system was singular (zero LU pivot)");
    return 0;
  } catch (std::exception &e) {
    return fail(GTK_ERR_ARG, e.what());
  }
}

int gtk_batch_kernels(const gtk_batch *b, uint64_t *kernels) {
  if (!b || !kernels) return fail(GTK_ERR_ARG, "null argument");
  *kernels = b->graph_kernels;
  return 0;
}

void gtk_batch_destroy(gtk_batch *b) {
  if (!b) return;
  cudaSetDevice(b->dev);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_batch_graph(b);
  if (b->fused) fused_batch_free(b->fused);
  for (cudaEvent_t e : b->joins)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->d_tab) cudaFree(b->d_tab);
  if (b->d_out) cudaFree(b->d_out);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // extern "C"
