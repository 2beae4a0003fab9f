// api.cpp -- the C ABI (include/gputucker_gb300.h): handle lifecycle, readback,
// initialisation and the sweep driver.  Returns status codes; never exits.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "internal.h"

namespace gtk {

int parse_buffer(const char *buf, size_t len, int N, int dtype, uint32_t seed, gtk_coo *out);
int parse_file(const char *path, int N, int dtype, uint32_t seed, gtk_coo *out);

namespace {
thread_local std::string g_err;
constexpr int kPartialDoubles = 2048;  // per-CTA partial sums (fit, norm) + their total

uint64_t memory_cap() {
  const char *s = getenv("GTK_DEVICE_MEMORY_CAP");
  if (!s || !*s) return 0;
  return strtoull(s, nullptr, 10);
}
}  // namespace

void set_error(const std::string &msg) { g_err = msg; }
int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear a non-sticky error so the context stays usable
  return e == cudaErrorMemoryAllocation ? GTK_ERR_OOM : GTK_ERR_CUDA;
}

// Device allocation owned by the handle; honours GTK_DEVICE_MEMORY_CAP (bytes).
// the reference's norm (tensor_manager.tpp:263-293: NormX += val * val in value_t,
// input order, sqrt in value_t), summed on the host from the input-order values
// the partition left on the device; only the reference-order variant uses it
int ensure_norm_ref(DevTensor &t) {
  if (t.norm_ref_ready) return 0;
  if (t.nnz && !t.val_in) return fail(GTK_ERR_STATE, "the input-order values are gone");
  std::vector<unsigned char> h(t.nnz * t.vsize);
  if (t.nnz) {
    GTK_CUDA(cudaMemcpyAsync(h.data(), t.val_in, h.size(), cudaMemcpyDeviceToHost, t.stream));
    GTK_CUDA(cudaStreamSynchronize(t.stream));
  }
  if (t.dtype == GTK_F32) {
    const float *v = reinterpret_cast<const float *>(h.data());
    float s = 0.f;
    for (uint64_t i = 0; i < t.nnz; ++i) s += v[i] * v[i];
    t.norm_ref = (double)std::sqrt(s);
  } else {
    const double *v = reinterpret_cast<const double *>(h.data());
    double s = 0.0;
    for (uint64_t i = 0; i < t.nnz; ++i) s += v[i] * v[i];
    t.norm_ref = std::sqrt(s);
  }
  t.norm_ref_ready = true;
  return 0;
}

namespace {
struct CachedBlock {
  int dev;
  size_t bytes;
  void *p;
};
std::mutex g_cache_mu;
std::vector<CachedBlock> g_cache;
uint64_t g_cache_cap[64] = {};  // half of each device's memory, read once

uint64_t cache_cap(int dev) {
  if (dev < 0 || dev >= 64) return 0;
  if (!g_cache_cap[dev]) {
    // the total memory of `dev` itself, whichever device is current
    int cur = -1;
    size_t f = 0, total = 0;
    const bool ok = cudaGetDevice(&cur) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess &&
                    cudaMemGetInfo(&f, &total) == cudaSuccess;
    if (cur >= 0) cudaSetDevice(cur);
    if (!ok) {
      cudaGetLastError();
      return 0;
    }
    g_cache_cap[dev] = total / 2;
  }
  return g_cache_cap[dev];
}
}  // namespace

void *dev_alloc(int dev, size_t bytes) {
  {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    for (size_t i = 0; i < g_cache.size(); ++i)
      if (g_cache[i].dev == dev && g_cache[i].bytes == bytes) {
        void *p = g_cache[i].p;
        g_cache.erase(g_cache.begin() + (long)i);
        return p;
      }
  }
  void *p = nullptr;
  if (cudaMalloc(&p, bytes) == cudaSuccess) return p;
  cudaGetLastError();
  dev_cache_clear(dev);  // memory held by the cache goes back to the driver, then once more
  if (cudaMalloc(&p, bytes) == cudaSuccess) return p;
  cudaGetLastError();
  return nullptr;
}

cudaError_t malloc_retry(void **p, size_t bytes) {
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaErrorMemoryAllocation) return e;
  cudaGetLastError();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return e;
  if (dev_cached_bytes(dev) == 0) return e;
  dev_cache_clear(dev);
  return cudaMalloc(p, bytes);
}

void dev_free(int dev, void *p, size_t bytes) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    uint64_t held = 0;
    for (const CachedBlock &b : g_cache)
      if (b.dev == dev) held += b.bytes;
    if (held + bytes <= cache_cap(dev)) {
      g_cache.push_back({dev, bytes, p});
      return;
    }
  }
  cudaFree(p);
}

uint64_t dev_cached_bytes(int dev) {
  std::lock_guard<std::mutex> lock(g_cache_mu);
  uint64_t held = 0;
  for (const CachedBlock &b : g_cache)
    if (b.dev == dev) held += b.bytes;
  return held;
}

void dev_cache_clear(int dev) {
  std::vector<CachedBlock> out;
  {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    for (size_t i = 0; i < g_cache.size();) {
      if (dev < 0 || g_cache[i].dev == dev) {
        out.push_back(g_cache[i]);
        g_cache.erase(g_cache.begin() + (long)i);
      } else {
        ++i;
      }
    }
  }
  int cur = 0;
  cudaGetDevice(&cur);
  for (const CachedBlock &b : out) {
    cudaSetDevice(b.dev);
    cudaFree(b.p);
  }
  cudaSetDevice(cur);
  cudaGetLastError();
}

int dalloc(DevTensor &t, void **p, size_t bytes) {
  if (bytes < 16) bytes = 16;
  bytes = (bytes + 255) / 256 * 256;
  uint64_t cap = memory_cap();
  if (cap && t.bytes + bytes > cap)
    return fail(GTK_ERR_OOM, "device memory cap (GTK_DEVICE_MEMORY_CAP) exceeded");
  *p = dev_alloc(t.dev, bytes);
  if (!*p) return fail(GTK_ERR_OOM, "device allocation of " + std::to_string(bytes) + " bytes failed");
  t.allocs.push_back({*p, bytes});
  t.bytes += bytes;
  return 0;
}

int need_resident(const DevTensor &t, const char *what) {
  if (!t.streamed) return 0;
  return fail(GTK_ERR_UNSUPPORTED, std::string(what) + " needs the device-resident layout; this handle streams its "
                                                        "views from host memory");
}

static void release(DevTensor &t) {
  if (t.dev >= 0) cudaSetDevice(t.dev);
  if (t.stream) cudaStreamSynchronize(t.stream);
  if (t.copy_stream) cudaStreamSynchronize(t.copy_stream);
  drop_graph(t);
  for (const auto &a : t.allocs) dev_free(t.dev, a.first, a.second);
  t.allocs.clear();
  if (t.tev0) cudaEventDestroy(t.tev0);
  if (t.tev1) cudaEventDestroy(t.tev1);
  for (int b = 0; b < 2; ++b) {
    if (t.stage_ready[b]) cudaEventDestroy(t.stage_ready[b]);
    if (t.stage_free[b]) cudaEventDestroy(t.stage_free[b]);
    t.stage_ready[b] = t.stage_free[b] = nullptr;
  }
  if (t.hp && t.hp->pinned) {
    for (int m = 0; m < t.N; ++m) {
      for (int k = 0; k < t.N; ++k)
        if (!t.hp->vidx[m][k].empty()) cudaHostUnregister(t.hp->vidx[m][k].data());
      if (!t.hp->vval[m].empty()) cudaHostUnregister(t.hp->vval[m].data());
    }
    t.hp->pinned = false;
  }
  if (t.copy_stream) cudaStreamDestroy(t.copy_stream);
  t.copy_stream = nullptr;
  if (t.stream) cudaStreamDestroy(t.stream);
  t.stream = nullptr;
}

namespace {
// device bytes of the resident layout (persistent arrays) and of the partition's
// temporaries, to decide between the resident and the streamed layout
void resident_bytes(const DevTensor &t, uint64_t *persist, uint64_t *temp) {
  const uint64_t n = t.nnz, vs = t.vsize, N = (uint64_t)t.N;
  uint64_t p = (t.nblk + 1) * 8 + n * vs * 2;  // blk_ptr, blk_val, val_in
  for (int k = 0; k < t.N; ++k)
    p += n * 4 * (3 + N) + n * vs + t.nblk * (uint64_t)(t.bd[k] + 1) * 8;  // blk_idx, where, vperm, views, count
  *persist = p;
  *temp = n * (4 * N + 4 * 8) + n * 64;  // uploaded coordinates, sort scratch, block-major copies, records
}
}  // namespace

// The streamed layout: the partition in host memory (hostpart.cpp), page-locked
// views where the host allows, and two device staging buffers of `chunk`
// nonzeros (GTK_STREAM_CHUNK nonzeros, else as many as fit a quarter of the
// memory the handle may still use, at most 2^26).
int setup_streamed(DevTensor &t, const gtk_coo &coo) {
  if (int rc = build_host_partition(t, coo)) return rc;
  HostPart &h = *t.hp;
  const uint64_t per = (uint64_t)t.N * 4 + t.vsize;  // staged bytes per nonzero
  uint64_t chunk = 0;
  if (const char *s = getenv("GTK_STREAM_CHUNK")) chunk = strtoull(s, nullptr, 10);
  if (!chunk) {
    const uint64_t cap = memory_cap();
    size_t fr = 0, tot = 0;
    GTK_CUDA(cudaMemGetInfo(&fr, &tot));
    uint64_t room = (uint64_t)fr + dev_cached_bytes(t.dev);
    if (cap) room = std::min<uint64_t>(room, cap > t.bytes ? cap - t.bytes : 0);
    chunk = room / 4 / per;
    chunk = std::min<uint64_t>(chunk, 1ull << 26);
  }
  chunk = std::max<uint64_t>(std::min<uint64_t>(chunk, t.nnz), 1);
  t.chunk = chunk;
  for (int b = 0; b < 2; ++b) {
    for (int k = 0; k < t.N; ++k)
      if (int rc = dalloc(t, (void **)&t.stage_idx[b][k], chunk * 4)) return rc;
    if (int rc = dalloc(t, &t.stage_val[b], chunk * t.vsize)) return rc;
    GTK_CUDA(cudaEventCreateWithFlags(&t.stage_ready[b], cudaEventDisableTiming));
    GTK_CUDA(cudaEventCreateWithFlags(&t.stage_free[b], cudaEventDisableTiming));
  }
  GTK_CUDA(cudaStreamCreateWithFlags(&t.copy_stream, cudaStreamNonBlocking));
  // page-locked views copy asynchronously; without registration (not allowed, or
  // out of lockable memory) the copies read pageable memory
  if (t.nnz) {
    bool ok = true;
    for (int m = 0; m < t.N && ok; ++m) {
      for (int k = 0; k < t.N && ok; ++k)
        ok = cudaHostRegister(h.vidx[m][k].data(), t.nnz * 4, cudaHostRegisterDefault) == cudaSuccess;
      if (ok) ok = cudaHostRegister(h.vval[m].data(), t.nnz * t.vsize, cudaHostRegisterDefault) == cudaSuccess;
      if (!ok) {
        cudaGetLastError();
        // undo this mode's partial registration and every earlier mode's
        for (int mm = 0; mm <= m; ++mm) {
          for (int k = 0; k < t.N; ++k) cudaHostUnregister(h.vidx[mm][k].data());
          cudaHostUnregister(h.vval[mm].data());
        }
        cudaGetLastError();
      }
    }
    h.pinned = ok;
  }
  return 0;
}

// slab layout [rows][J] <-> device [rows][ldf]
static int put_factor(DevTensor &t, int n, const void *slabs) {
  fit_invalidate(t);
  return factor_from_host(t, n, slabs);
}

static int get_factor(const DevTensor &t, int n, void *slabs) { return factor_to_host(t, n, slabs); }

int put_core(DevTensor &t, const void *core) {
  fit_invalidate(t);
  GTK_CUDA(cudaMemcpyAsync(t.core, core, t.core_n * t.vsize, cudaMemcpyHostToDevice, t.stream));
  if (int rc = upload_core_perms(t, core)) return rc;
  t.have_core = true;
  if (t.precision == GTK_PREC_BF16 && ts_supported(t.N, t.J, t.dtype, t.precision))
    if (int rc = ts_build_images(t)) return rc;
  return 0;
}

static int check_status(DevTensor &t) {
  int st = 0;
  GTK_CUDA(cudaMemcpyAsync(&st, t.status, 4, cudaMemcpyDeviceToHost, t.stream));
  GTK_CUDA(cudaStreamSynchronize(t.stream));
  if (st & 4) t.lu_fallbacks += 1;  // Cholesky gave way to pivoted LU somewhere: informational
  if (st) GTK_CUDA(cudaMemsetAsync(t.status, 0, 4, t.stream));
  if (st & 2) return fail(GTK_ERR_CUDA, "a tensor-core kernel gave up waiting for its MMAs");
  if (st & 1) return fail(GTK_ERR_NUMERIC, "a row system was singular (zero LU pivot)");
  return 0;
}

}  // namespace gtk

using namespace gtk;

#define GTK_GUARD_BEGIN try {
#define GTK_GUARD_END                                         \
  }                                                           \
  catch (std::bad_alloc &) {                                  \
    return fail(GTK_ERR_OOM, "host allocation failed");       \
  }                                                           \
  catch (std::exception & e) {                                \
    return fail(GTK_ERR_ARG, e.what());                       \
  }

static int set_dev(const gtk_tensor *t) {
  GTK_CUDA(cudaSetDevice(t->dev));
  return 0;
}

extern "C" {

const char *gtk_last_error(void) { return g_err.c_str(); }
int gtk_version(void) { return GTK_VERSION; }

int gtk_parse_buffer(const char *buf, size_t len, int order, int dtype, uint32_t rand_seed, gtk_coo **out) {
  if (!out || (!buf && len)) return fail(GTK_ERR_ARG, "null argument");
  GTK_GUARD_BEGIN
  gtk_coo *c = new gtk_coo();
  int rc = parse_buffer(buf, len, order, dtype, rand_seed, c);
  if (rc) {
    delete c;
    return rc;
  }
  *out = c;
  return 0;
  GTK_GUARD_END
}

int gtk_parse_file(const char *path, int order, int dtype, uint32_t rand_seed, gtk_coo **out) {
  if (!path || !out) return fail(GTK_ERR_ARG, "null argument");
  GTK_GUARD_BEGIN
  gtk_coo *c = new gtk_coo();
  int rc = parse_file(path, order, dtype, rand_seed, c);
  if (rc) {
    delete c;
    return rc;
  }
  *out = c;
  return 0;
  GTK_GUARD_END
}

int gtk_coo_from_arrays(int order, uint64_t nnz, const uint32_t *const *idx, const void *values, int dtype,
                        const uint32_t *dims, gtk_coo **out) {
  if (!out || (nnz && (!idx || !values))) return fail(GTK_ERR_ARG, "null argument");
  if (order < 1 || order > GTK_MAX_ORDER) return fail(GTK_ERR_ARG, "order must be 1..8");
  if (dtype != GTK_F32 && dtype != GTK_F64) return fail(GTK_ERR_ARG, "bad dtype");
  GTK_GUARD_BEGIN
  gtk_coo *c = new gtk_coo();
  c->N = order;
  c->dtype = dtype;
  c->nnz = nnz;
  for (int n = 0; n < order; ++n) {
    if (nnz && !idx[n]) {
      delete c;
      return fail(GTK_ERR_ARG, "null index array");
    }
    c->idx[n].assign(idx[n], idx[n] + nnz);
    uint32_t mx = 0;
    for (uint64_t k = 0; k < nnz; ++k) mx = std::max(mx, idx[n][k]);
    if (dims) {
      if (nnz && mx >= dims[n]) {
        delete c;
        return fail(GTK_ERR_ARG, "coordinate out of bounds");
      }
      c->dims[n] = dims[n];
    } else {
      c->dims[n] = nnz ? mx + 1 : 0;
    }
  }
  if (dtype == GTK_F32)
    c->vf.assign((const float *)values, (const float *)values + nnz);
  else
    c->vd.assign((const double *)values, (const double *)values + nnz);
  *out = c;
  return 0;
  GTK_GUARD_END
}

int gtk_coo_info(const gtk_coo *c, int *order, int *dtype, uint64_t *nnz, uint32_t *dims, uint64_t *draws) {
  if (!c) return fail(GTK_ERR_ARG, "null coo");
  if (order) *order = c->N;
  if (dtype) *dtype = c->dtype;
  if (nnz) *nnz = c->nnz;
  if (dims)
    for (int n = 0; n < c->N; ++n) dims[n] = c->dims[n];
  if (draws) *draws = c->draws;
  return 0;
}

int gtk_coo_export(const gtk_coo *c, uint32_t *const *idx, void *values) {
  if (!c) return fail(GTK_ERR_ARG, "null coo");
  if (idx)
    for (int n = 0; n < c->N; ++n)
      if (idx[n]) memcpy(idx[n], c->idx[n].data(), c->nnz * 4);
  if (values) memcpy(values, c->values(), c->nnz * (c->dtype == GTK_F32 ? 4 : 8));
  return 0;
}

int gtk_coo_pin(gtk_coo *c) {
  if (!c) return fail(GTK_ERR_ARG, "null coo");
  if (c->pinned || c->nnz == 0) return 0;
  for (int n = 0; n < c->N; ++n)
    GTK_CUDA(cudaHostRegister(c->idx[n].data(), c->nnz * 4, cudaHostRegisterDefault));
  GTK_CUDA(cudaHostRegister(const_cast<void *>(c->values()), c->nnz * (c->dtype == GTK_F32 ? 4 : 8),
                            cudaHostRegisterDefault));
  c->pinned = true;
  return 0;
}

void gtk_coo_free(gtk_coo *c) {
  if (!c) return;
  if (c->pinned) {
    for (int n = 0; n < c->N; ++n) cudaHostUnregister(c->idx[n].data());
    cudaHostUnregister(const_cast<void *>(c->values()));
  }
  delete c;
}

int gtk_create_blocks(const gtk_coo *coo, const uint32_t *P, int rank, int device, gtk_tensor **out) {
  NvtxRange nvtx("gtk_create_blocks");
  if (!coo || !P || !out) return fail(GTK_ERR_ARG, "null argument");
  if (rank < 1 || rank > GTK_MAX_RANK) return fail(GTK_ERR_ARG, "rank must be 1..64");
  const int N = coo->N;
  if (coo->nnz >= 0xFFFFFFFFull) return fail(GTK_ERR_UNSUPPORTED, "more than 2^32-2 nonzeros");
  uint64_t nblk = 1;
  uint32_t bd[GTK_MAX_ORDER];
  for (int n = 0; n < N; ++n) {
    if (P[n] == 0) return fail(GTK_ERR_ARG, "partition parameter must be >= 1");
    if (coo->dims[n] == 0) return fail(GTK_ERR_ARG, "empty tensor dimension");
    // tensor.tpp:199-213 / optimizer.tpp:360-376
    bd[n] = (uint32_t)(((uint64_t)coo->dims[n] + P[n] - 1) / P[n]);
    uint32_t check = (uint32_t)(((uint64_t)coo->dims[n] + bd[n] - 1) / bd[n]);
    if (check != P[n]) return fail(GTK_ERR_PARTITION, "Block dimension is larger than the tensor dimension.");
    nblk *= P[n];
    if (nblk > 0xFFFFFFFFull) return fail(GTK_ERR_UNSUPPORTED, "more than 2^32 blocks");
  }
  uint64_t core_n = 1;
  for (int n = 0; n < N; ++n) {
    core_n *= (uint64_t)rank;
    if (core_n > (1ull << 28)) return fail(GTK_ERR_UNSUPPORTED, "core tensor larger than 2^28 entries");
  }
  GTK_GUARD_BEGIN
  gtk_tensor *t = new gtk_tensor();
  t->dev = device;
  t->dtype = coo->dtype;
  t->vsize = coo->dtype == GTK_F32 ? 4 : 8;
  t->N = N;
  t->J = rank;
  const int w = (int)(16 / t->vsize);
  t->ldf = (rank + w - 1) / w * w;
  t->E = (rank + 1) * (rank + 2) / 2 - 1;
  t->nnz = coo->nnz;
  t->nblk = nblk;
  t->core_n = core_n;
  uint64_t max_rows = 0;
  for (int n = 0; n < N; ++n) {
    t->dims[n] = coo->dims[n];
    t->P[n] = P[n];
    t->bd[n] = bd[n];
    t->rows[n] = (uint64_t)P[n] * bd[n];
    max_rows = std::max(max_rows, t->rows[n]);
  }
  auto bail = [&](int rc) {
    release(*t);
    delete t;
    return rc;
  };
  if (int rc = ck(cudaSetDevice(device), "cudaSetDevice")) return bail(rc);
  int sms = 0;
  if (int rc = ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "device attribute"))
    return bail(rc);
  t->num_sms = sms;
  if (int rc = ck(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking), "cudaStreamCreate")) return bail(rc);
  const uint64_t nnz = t->nnz;
  const size_t vs = t->vsize;
  int rc = 0;
  auto A = [&](void **p, size_t b) {
    if (!rc) rc = dalloc(*t, p, b);
  };
  // the resident layout, or -- when it does not fit the memory the handle may
  // use (GTK_DEVICE_MEMORY_CAP, else the device's free memory) -- the streamed one
  {
    uint64_t persist = 0, temp = 0;
    resident_bytes(*t, &persist, &temp);
    const uint64_t cap = memory_cap();
    size_t fr = 0, tot = 0;
    if ((rc = ck(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo"))) return bail(rc);
    const uint64_t avail = (uint64_t)fr + dev_cached_bytes(device);
    t->streamed = (cap && persist > cap) || persist + temp > avail;
    const char *force = getenv("GTK_FORCE_STREAMED");
    if (force && *force == '1') t->streamed = true;
  }
  if (!t->streamed) {
    A((void **)&t->blk_ptr, (nblk + 1) * 8);
    A(&t->blk_val, nnz * vs);
  }
  for (int n = 0; n < N; ++n) {
    if (!t->streamed) {
      A((void **)&t->blk_idx[n], nnz * 4);
      A((void **)&t->count[n], nblk * (uint64_t)(bd[n] + 1) * 8);
      A((void **)&t->where[n], nnz * 4);
      A((void **)&t->vperm[n], nnz * 4);
      A(&t->vval[n], nnz * vs);
      for (int k = 0; k < N; ++k) A((void **)&t->vidx[n][k], nnz * 4);
    }
    A(&t->fac[n], t->rows[n] * t->ldf * vs);
    if (vs == 4 && t->ldf == 12) A(&t->gfac[n], t->rows[n] * 64);
    A(&t->corep[n], (core_n / rank) * t->ldf * vs);
  }
  A(&t->core, core_n * vs);
  A((void **)&t->gram, max_rows * (uint64_t)t->E * 8);
  A((void **)&t->partial, kPartialDoubles * 8);
  A((void **)&t->status, 16);
  A((void **)&t->fallback, max_rows * 4);
  A((void **)&t->fallback64, max_rows * 4);
  A((void **)&t->nfallback, 16);
  A(&t->xfer, max_rows * (uint64_t)rank * vs);
  if (rc) return bail(rc);
  for (int n = 0; n < N; ++n) {
    if ((rc = ck(cudaMemsetAsync(t->fac[n], 0, t->rows[n] * t->ldf * vs, t->stream), "memset"))) return bail(rc);
    if ((rc = ck(cudaMemsetAsync(t->corep[n], 0, (core_n / rank) * t->ldf * vs, t->stream), "memset"))) return bail(rc);
  }
  if ((rc = ck(cudaMemsetAsync(t->status, 0, 16, t->stream), "memset"))) return bail(rc);
  if ((rc = ck(cudaMemsetAsync(t->nfallback, 0, 16, t->stream), "memset"))) return bail(rc);
  if (t->streamed) {
    if ((rc = setup_streamed(*t, *coo))) return bail(rc);
  } else {
    rc = build_partition(*t, *coo);
  }
  if (rc) return bail(rc);
  *out = t;
  return 0;
  GTK_GUARD_END
}

int gtk_tensor_info_get(const gtk_tensor *t, gtk_tensor_info *info) {
  if (!t || !info) return fail(GTK_ERR_ARG, "null argument");
  memset(info, 0, sizeof(*info));
  info->order = t->N;
  info->rank = t->J;
  info->dtype = t->dtype;
  info->device = t->dev;
  info->nnz = t->nnz;
  info->block_count = t->nblk;
  for (int n = 0; n < t->N; ++n) {
    info->dims[n] = t->dims[n];
    info->partition_dims[n] = t->P[n];
    info->block_dims[n] = t->bd[n];
  }
  info->norm = t->norm;
  info->device_bytes = t->bytes;
  info->streamed = t->streamed ? 1 : 0;
  info->stream_chunk = t->chunk;
  info->host_direct = t->create_direct ? 1 : 0;
  return 0;
}

int gtk_block_info(const gtk_tensor *t, uint64_t b, uint32_t *coord, uint64_t *nnz) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (b >= t->nblk) return fail(GTK_ERR_ARG, "block id out of range");
  if (coord) {
    uint64_t r = b;
    for (int n = t->N - 1; n >= 0; --n) {
      coord[n] = (uint32_t)(r % t->P[n]);
      r /= t->P[n];
    }
  }
  if (nnz) *nnz = t->h_blk_ptr[b + 1] - t->h_blk_ptr[b];
  return 0;
}

int gtk_block_data(const gtk_tensor *t, uint64_t b, uint32_t *const *idx, void *values) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (b >= t->nblk) return fail(GTK_ERR_ARG, "block id out of range");
  if (int rc = set_dev(t)) return rc;
  const uint64_t s = t->h_blk_ptr[b], n = t->h_blk_ptr[b + 1] - s;
  if (t->streamed) {
    if (idx)
      for (int k = 0; k < t->N; ++k)
        if (idx[k] && n) memcpy(idx[k], t->hp->blk_idx[k].data() + s, n * 4);
    if (values && n) memcpy(values, t->hp->blk_val.data() + s * t->vsize, n * t->vsize);
    return 0;
  }
  if (idx)
    for (int k = 0; k < t->N; ++k)
      if (idx[k] && n) GTK_CUDA(cudaMemcpyAsync(idx[k], t->blk_idx[k] + s, n * 4, cudaMemcpyDeviceToHost, t->stream));
  if (values && n)
    GTK_CUDA(cudaMemcpyAsync(values, (const char *)t->blk_val + s * t->vsize, n * t->vsize, cudaMemcpyDeviceToHost,
                             t->stream));
  GTK_CUDA(cudaStreamSynchronize(t->stream));
  return 0;
}

int gtk_block_segments(const gtk_tensor *t, uint64_t b, int mode, uint64_t *count_nnz, uint32_t *where_nnz) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (b >= t->nblk || mode < 0 || mode >= t->N) return fail(GTK_ERR_ARG, "block or mode out of range");
  if (int rc = set_dev(t)) return rc;
  const uint64_t s = t->h_blk_ptr[b], n = t->h_blk_ptr[b + 1] - s;
  const uint64_t rows = (uint64_t)t->bd[mode] + 1;
  if (t->streamed) {
    if (count_nnz) memcpy(count_nnz, t->hp->count[mode].data() + b * rows, rows * 8);
    if (where_nnz && n) memcpy(where_nnz, t->hp->where[mode].data() + s, n * 4);
    return 0;
  }
  if (count_nnz)
    GTK_CUDA(cudaMemcpyAsync(count_nnz, t->count[mode] + b * rows, rows * 8, cudaMemcpyDeviceToHost, t->stream));
  if (where_nnz && n)
    GTK_CUDA(cudaMemcpyAsync(where_nnz, t->where[mode] + s, n * 4, cudaMemcpyDeviceToHost, t->stream));
  GTK_CUDA(cudaStreamSynchronize(t->stream));
  return 0;
}

void gtk_destroy(gtk_tensor *t) {
  if (!t) return;
  release(*t);
  delete t;
}

int gtk_init_random(gtk_tensor *t, uint32_t seed, uint64_t skip) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (int rc = set_dev(t)) return rc;
  GTK_GUARD_BEGIN
  GlibcRand g(seed);
  g.jump(skip);
  // tucker.cuh:84-97 (the factors, generated on the device), then
  // tucker.cuh:117-134: the core in linear order
  fit_invalidate(*t);
  if (int rc = factor_init_device(*t, g)) return rc;
  std::vector<unsigned char> core(t->core_n * t->vsize);
  for (uint64_t i = 0; i < t->core_n; ++i) {
    const double v = g.frand01<double>();
    if (t->dtype == GTK_F32)
      ((float *)core.data())[i] = (float)v;
    else
      ((double *)core.data())[i] = v;
  }
  if (int rc = put_core(*t, core.data())) return rc;
  t->have_factors = true;
  return 0;
  GTK_GUARD_END
}

int gtk_random_sequence(uint32_t rand_seed, uint64_t skip_draws, uint64_t n, double *out) {
  if (n && !out) return fail(GTK_ERR_ARG, "null output");
  GTK_GUARD_BEGIN
  GlibcRand g(rand_seed);
  g.jump(skip_draws);
  // by the split gtk_init_random's device generation uses: chunk start windows,
  // each chunk's pieces moved on from them by the step polynomials, each piece's
  // draws by the recurrence alone
  const uint64_t len = kFacChunk / kFacSplit;
  const int chunks = (int)std::max<uint64_t>(1, (n + kFacChunk - 1) / kFacChunk);
  std::vector<uint32_t> st((size_t)chunks * 31), pol((size_t)kFacSplit * 31);
  glibc_chunk_states(g, kFacChunk, chunks, st.data());
  glibc_step_polys(len, kFacSplit, pol.data());
  for (int c = 0; c < chunks; ++c)
    for (int piece = 0; piece < kFacSplit; ++piece) {
      const uint64_t b = (uint64_t)c * kFacChunk + (uint64_t)piece * len, e = std::min<uint64_t>(n, b + len);
      if (b >= e) break;
      uint32_t a[31], w[31];
      for (int j = 0; j < 31; ++j) a[j] = pol[31 * (size_t)piece + j];
      for (int m = 0; m < 31; ++m) {  // w[m] = (x^(piece len + m) mod p) . chunk window
        uint32_t v = 0;
        for (int j = 0; j < 31; ++j) v += a[j] * st[31 * (size_t)c + j];
        w[m] = v;
        const uint32_t top = a[30];
        for (int j = 30; j > 0; --j) a[j] = a[j - 1];
        a[0] = top;
        a[28] += top;
      }
      for (uint64_t d = b; d < e; ++d) {  // r[d] = r[d - 31] + r[d - 3]
        const int k = (int)((d - b) % 31);
        w[k] += w[(k + 28) % 31];
        out[d] = (double)(int)(w[k] >> 1) / 2147483647;
      }
    }
  return 0;
  GTK_GUARD_END
}

int gtk_set_factor(gtk_tensor *t, int mode, const void *slabs) {
  if (!t || !slabs) return fail(GTK_ERR_ARG, "null argument");
  if (mode < 0 || mode >= t->N) return fail(GTK_ERR_ARG, "mode out of range");
  if (int rc = set_dev(t)) return rc;
  if (int rc = put_factor(*t, mode, slabs)) return rc;
  t->have_factors = true;
  return 0;
}

int gtk_get_factor(const gtk_tensor *t, int mode, void *slabs) {
  if (!t || !slabs) return fail(GTK_ERR_ARG, "null argument");
  if (mode < 0 || mode >= t->N) return fail(GTK_ERR_ARG, "mode out of range");
  if (int rc = set_dev(t)) return rc;
  return get_factor(*t, mode, slabs);
}

int gtk_set_core(gtk_tensor *t, const void *core) {
  if (!t || !core) return fail(GTK_ERR_ARG, "null argument");
  if (int rc = set_dev(t)) return rc;
  GTK_GUARD_BEGIN
  return put_core(*t, core);
  GTK_GUARD_END
}

int gtk_get_core(const gtk_tensor *t, void *core) {
  if (!t || !core) return fail(GTK_ERR_ARG, "null argument");
  if (int rc = set_dev(t)) return rc;
  GTK_CUDA(cudaMemcpyAsync(core, t->core, t->core_n * t->vsize, cudaMemcpyDeviceToHost, t->stream));
  GTK_CUDA(cudaStreamSynchronize(t->stream));
  return 0;
}

int gtk_set_precision(gtk_tensor *t, int precision) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (precision != GTK_PREC_PLAIN && precision != GTK_PREC_BF16 && precision != GTK_PREC_TF32)
    return fail(GTK_ERR_ARG, "unknown precision");
  fit_invalidate(*t);
  drop_graph(*t);
  if (precision != GTK_PREC_PLAIN && !tc_supported(t->N, t->J, t->dtype, precision))
    return fail(GTK_ERR_UNSUPPORTED, "no tensor-core form for this order/rank/value type/precision (FP32; "
                                     "BF16 or TF32: N = 3, J in {4, 8, 10, 12, 16}; N = 4, J in {4, 8, 10, 12}; "
                                     "BF16 only: N = 4, J = 16; N = 5, J in {4, 8, 12, 16})");
  if (precision == GTK_PREC_BF16 && t->have_core && ts_supported(t->N, t->J, t->dtype, precision))
    if (int rc = ts_build_images(*t)) return rc;
  t->precision = precision;
  if (precision == GTK_PREC_PLAIN && t->variant == kVarTc) t->variant = kVarAuto;
  return 0;
}

static int ready(gtk_tensor *t) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (!t->have_factors || !t->have_core) return fail(GTK_ERR_STATE, "factors and core are not initialised");
  return set_dev(t);
}

int gtk_update_mode(gtk_tensor *t, int mode) {
  if (int rc = ready(t)) return rc;
  if (mode < 0 || mode >= t->N) return fail(GTK_ERR_ARG, "mode out of range");
  GTK_GUARD_BEGIN
  return run_update_mode(*t, mode);
  GTK_GUARD_END
}

int gtk_validate(gtk_tensor *t, uint64_t *violations) {
  if (!t || !violations) return fail(GTK_ERR_ARG, "null argument");
  if (int rc = need_resident(*t, "gtk_validate")) return rc;
  if (int rc = set_dev(t)) return rc;
  GTK_GUARD_BEGIN
  return run_validate(*t, violations);
  GTK_GUARD_END
}

int gtk_update_core(gtk_tensor *t, int cg_iters, int *iters_run, double *rel_residual) {
  if (int rc = ready(t)) return rc;
  if (int rc = need_resident(*t, "gtk_update_core")) return rc;
  if (cg_iters < 0) return fail(GTK_ERR_ARG, "negative iteration count");
  GTK_GUARD_BEGIN
  return run_update_core(*t, cg_iters, iters_run, rel_residual);
  GTK_GUARD_END
}

int gtk_update_factor_matrices(gtk_tensor *t) {
  if (int rc = ready(t)) return rc;
  GTK_GUARD_BEGIN
  for (int n = 0; n < t->N; ++n)
    if (int rc = run_update_mode(*t, n)) return rc;
  return 0;
  GTK_GUARD_END
}

int gtk_sweep(gtk_tensor *t, double *fit) {
  if (int rc = ready(t)) return rc;
  if (!fit) return fail(GTK_ERR_ARG, "null fit");
  GTK_GUARD_BEGIN
  if (int rc = run_sweep(*t, fit)) return rc;
  return check_status(*t);
  GTK_GUARD_END
}

int gtk_set_graph(gtk_tensor *t, int on) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (int rc = set_dev(t)) return rc;
  t->use_graph = on != 0;
  if (!t->use_graph) drop_graph(*t);
  return 0;
}

int gtk_reconstruction(gtk_tensor *t, double *fit) {
  if (int rc = ready(t)) return rc;
  if (!fit) return fail(GTK_ERR_ARG, "null fit");
  GTK_GUARD_BEGIN
  if (int rc = run_fit(*t, fit)) return rc;
  return check_status(*t);
  GTK_GUARD_END
}

int gtk_tucker_decomposition(gtk_tensor *t, int max_iters, double tol, double *fits, int *iters) {
  if (int rc = ready(t)) return rc;
  if (max_iters < 1) return fail(GTK_ERR_ARG, "max_iters must be >= 1");
  GTK_GUARD_BEGIN
  // tucker.cuh:166-187
  int it = 0;
  double p_fit = -1, fit = -1;
  int numeric = 0;
  while (true) {
    if (int rc = run_sweep(*t, &fit)) return rc;
    if (int rc = check_status(*t)) {  // a singular row is reported at the end; anything else ends the run
      if (rc != GTK_ERR_NUMERIC) return rc;
      numeric = rc;
    }
    if (fits) fits[it] = fit;
    ++it;
    if (it >= max_iters || (p_fit != -1 && std::fabs(p_fit - fit) <= tol)) break;
    p_fit = fit;
  }
  if (iters) *iters = it;
  if (numeric) return fail(GTK_ERR_NUMERIC, "a row solve met a non-positive pivot");
  return 0;
  GTK_GUARD_END
}

int gtk_compute_delta(gtk_tensor *t, int mode, void *delta) {
  if (int rc = ready(t)) return rc;
  if (int rc = need_resident(*t, "gtk_compute_delta")) return rc;
  if (mode < 0 || mode >= t->N || !delta) return fail(GTK_ERR_ARG, "bad mode or null output");
  GTK_GUARD_BEGIN
  const size_t bytes = t->nnz * (size_t)t->J * t->vsize;
  if (!bytes) return 0;
  DevBuf d;
  GTK_CUDA(d.alloc(bytes));
  int rc = run_delta(*t, mode, d.p);
  if (!rc) rc = ck(cudaMemcpyAsync(delta, d.p, bytes, cudaMemcpyDeviceToHost, t->stream), "delta readback");
  if (!rc) rc = ck(cudaStreamSynchronize(t->stream), "sync");
  return rc;
  GTK_GUARD_END
}

int gtk_solve_counters(gtk_tensor *t, uint64_t *fp64_rows, uint64_t *lu_rows, int reset) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (int rc = set_dev(t)) return rc;
  unsigned int c[4] = {0, 0, 0, 0};
  GTK_CUDA(cudaMemcpyAsync(c, t->nfallback, sizeof(c), cudaMemcpyDeviceToHost, t->stream));
  GTK_CUDA(cudaStreamSynchronize(t->stream));
  if (fp64_rows) *fp64_rows = c[2];
  if (lu_rows) *lu_rows = c[3];
  if (reset) {
    GTK_CUDA(cudaMemsetAsync(t->nfallback + 2, 0, 8, t->stream));
    GTK_CUDA(cudaStreamSynchronize(t->stream));
  }
  return 0;
}

int gtk_profile_enable(gtk_tensor *t, int on) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  t->prof = on != 0;
  return 0;
}

int gtk_profile_read(gtk_tensor *t, int kind, double *ms, uint64_t *launches) {
  if (!t || kind < 0 || kind > 6) return fail(GTK_ERR_ARG, "bad argument");
  if (kind == 4) {  // kernels launched by the sweep entry points since the last reset
    if (ms) *ms = 0;
    if (launches) *launches = t->launches;
    return 0;
  }
  if (kind >= 5) {  // phases of gtk_create_blocks
    if (ms) *ms = kind == 5 ? t->create_upload_ms : t->create_kernels_ms;
    if (launches) *launches = 0;
    return 0;
  }
  if (int rc = set_dev(t)) return rc;
  if (int rc = prof_resolve(*t)) return rc;
  double m = 0;
  uint64_t c = 0;
  if (kind == 3) {
    for (int k = 0; k < 3; ++k) {
      m += t->prof_ms[k];
      c += t->prof_n[k];
    }
  } else {
    m = t->prof_ms[kind];
    c = t->prof_n[kind];
  }
  if (ms) *ms = m;
  if (launches) *launches = c;
  return 0;
}

int gtk_profile_reset(gtk_tensor *t) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (int rc = prof_resolve(*t)) return rc;
  for (int k = 0; k < 4; ++k) {
    t->prof_ms[k] = 0;
    t->prof_n[k] = 0;
  }
  t->launches = 0;
  return 0;
}

int gtk_timer_begin(gtk_tensor *t) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (int rc = set_dev(t)) return rc;
  if (!t->tev0) GTK_CUDA(cudaEventCreate(&t->tev0));
  if (!t->tev1) GTK_CUDA(cudaEventCreate(&t->tev1));
  GTK_CUDA(cudaEventRecord(t->tev0, t->stream));
  return 0;
}

int gtk_timer_end(gtk_tensor *t, double *ms) {
  if (!t || !t->tev0) return fail(GTK_ERR_STATE, "timer not started");
  if (int rc = set_dev(t)) return rc;
  GTK_CUDA(cudaEventRecord(t->tev1, t->stream));
  GTK_CUDA(cudaEventSynchronize(t->tev1));
  float m = 0;
  GTK_CUDA(cudaEventElapsedTime(&m, t->tev0, t->tev1));
  if (ms) *ms = m;
  return 0;
}

int gtk_synchronize(gtk_tensor *t) {
  if (!t) return fail(GTK_ERR_ARG, "null tensor");
  if (int rc = set_dev(t)) return rc;
  GTK_CUDA(cudaStreamSynchronize(t->stream));
  return 0;
}

}  // extern "C"
