// plan.cpp -- the partition planner (P_n from tensor size and GPU memory), and
// the factor/core checkpoint (dump + resume).
//
// Planner: the reference's Optimizer::FindPartitionParms (optimizer.tpp:71-89)
// with _DeterminePartitionType (:95-121), _DimensionBasedPartitioning (:138-153),
// _AvailableNonzeroCountPerTask (:160-164), the size terms (:203-286),
// _NextPartitionAxis (:343-352) and _RefreshBlockDims (:360-376), restated with
// the reference's integer widths (32-bit dims x rank products, 64-bit counts,
// unsigned wrap where the reference wraps) so that the same inputs give the same
// partition.  Where _RefreshBlockDims throws (a P_n that leaves an empty last
// slab), this returns GTK_ERR_PARTITION.  "Nonzero-based" means the whole
// problem fits the GPUs' memory (P_n = 1); "dimension-based" grows P_n on the
// mode with the largest block until one block's data fits a quarter of a GPU's
// memory and there are at least 4 blocks per GPU.
//
// Checkpoint: no reference counterpart (the reference keeps nothing between
// runs).  A little-endian binary file:
//   "GTKCKPT1" | u32 version=1 | u32 order | u32 rank | u32 dtype |
//   u32 dims[order] | u32 P[order] | u32 block_dims[order] | u32 nfits |
//   f64 fits[nfits] | factor n = P_n*block_dims[n] x rank value_t, n = 0..order-1 |
//   core rank^order value_t (last mode fastest) | u64 FNV-1a of all bytes before.
// Saved to `path`.tmp and renamed, so a crash leaves the previous checkpoint.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "internal.h"

using namespace gtk;

namespace {

struct Planner {
  int N;
  const uint32_t *dims;
  uint64_t nnz;
  uint32_t J;
  uint64_t isz = 4, vsz;
  uint32_t P[kMaxOrder], bd[kMaxOrder];
  uint64_t nblk = 1, avg = 0;

  bool refresh() {  // _RefreshBlockDims
    nblk = 1;
    for (int n = 0; n < N; ++n) {
      bd[n] = (uint32_t)(dims[n] + P[n] - 1) / P[n];
      const uint32_t check = (uint32_t)(dims[n] + bd[n] - 1) / bd[n];
      if (check != P[n]) return false;
      nblk *= P[n];
    }
    avg = (nnz + nblk - 1) / nblk;
    return true;
  }
  uint64_t core() const {
    const uint64_t cn = (uint64_t)std::pow((double)J, (double)N);
    return cn * (N * isz + vsz);
  }
  uint64_t sub_tensor() const { return avg * (N * isz + vsz); }
  uint64_t sub_factors() const {
    uint64_t s = 0;
    for (int n = 0; n < N; ++n) s += (uint32_t)(bd[n] * J);  // 32-bit product, as index_t * unsigned
    return s * vsz;
  }
  uint64_t all_factors() const {
    uint64_t s = 0;
    for (int n = 0; n < N; ++n) s += (uint32_t)(dims[n] * J);
    return s * vsz;
  }
  uint64_t sub_delta() const { return avg * J * vsz; }
  uint64_t all_data() const { return sub_tensor() + core() + sub_factors() + sub_delta(); }  // GetAllDataSize
  int next_axis() const {  // first mode with the largest block
    int m = 0;
    for (int n = 1; n < N; ++n)
      if (bd[m] < bd[n]) m = n;
    return m;
  }
};

uint64_t fnv1a(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}
constexpr uint64_t kFnvBasis = 14695981039346656037ull;
constexpr char kMagic[8] = {'G', 'T', 'K', 'C', 'K', 'P', 'T', '1'};

struct Writer {
  FILE *f;
  uint64_t h = kFnvBasis;
  bool ok = true;
  void put(const void *p, size_t n) {
    if (!ok) return;
    ok = fwrite(p, 1, n, f) == n;
    h = fnv1a(h, p, n);
  }
  void u32(uint32_t v) { put(&v, 4); }
};

struct Reader {
  FILE *f;
  uint64_t h = kFnvBasis;
  bool ok = true;
  void get(void *p, size_t n) {
    if (!ok) return;
    ok = fread(p, 1, n, f) == n;
    if (ok) h = fnv1a(h, p, n);
  }
  uint32_t u32() {
    uint32_t v = 0;
    get(&v, 4);
    return v;
  }
};

struct Header {
  uint32_t order = 0, rank = 0, dtype = 0, nfits = 0;
  uint32_t dims[kMaxOrder] = {}, P[kMaxOrder] = {}, bd[kMaxOrder] = {};
};

int read_header(Reader &r, Header &h, const char *path) {
  char magic[8] = {};
  r.get(magic, 8);
  if (!r.ok || memcmp(magic, kMagic, 8) != 0) return fail(GTK_ERR_PARSE, std::string("not a checkpoint: ") + path);
  const uint32_t version = r.u32();
  if (!r.ok || version != 1) return fail(GTK_ERR_PARSE, "unsupported checkpoint version");
  h.order = r.u32();
  h.rank = r.u32();
  h.dtype = r.u32();
  if (!r.ok || h.order < 1 || h.order > (uint32_t)kMaxOrder || h.rank < 1 || h.rank > (uint32_t)kMaxRank ||
      (h.dtype != GTK_F32 && h.dtype != GTK_F64))
    return fail(GTK_ERR_PARSE, "corrupt checkpoint header");
  for (uint32_t n = 0; n < h.order; ++n) h.dims[n] = r.u32();
  for (uint32_t n = 0; n < h.order; ++n) h.P[n] = r.u32();
  for (uint32_t n = 0; n < h.order; ++n) h.bd[n] = r.u32();
  h.nfits = r.u32();
  if (!r.ok || h.nfits > (1u << 20)) return fail(GTK_ERR_PARSE, "corrupt checkpoint header");
  return 0;
}

}  // namespace

extern "C" {

int gtk_plan_partition(int order, const uint32_t *dims, uint64_t nnz, int rank, int dtype, int gpu_count,
                       uint64_t gpu_mem_bytes, gtk_plan *out) {
  if (order < 1 || order > kMaxOrder || !dims || !out) return fail(GTK_ERR_ARG, "bad order, dims or output");
  if (rank < 1 || rank > kMaxRank) return fail(GTK_ERR_ARG, "rank must be 1..64");
  if (dtype != GTK_F32 && dtype != GTK_F64) return fail(GTK_ERR_ARG, "dtype must be GTK_F32 or GTK_F64");
  if (gpu_count < 1 || gpu_count > 65535) return fail(GTK_ERR_ARG, "gpu_count must be 1..65535");
  for (int n = 0; n < order; ++n)
    if (dims[n] < 1) return fail(GTK_ERR_ARG, "every dim must be >= 1");
  Planner p;
  p.N = order;
  p.dims = dims;
  p.nnz = nnz;
  p.J = (uint32_t)rank;
  p.vsz = dtype == GTK_F64 ? 8 : 4;
  for (int n = 0; n < order; ++n) p.P[n] = 1;
  if (!p.refresh()) return fail(GTK_ERR_PARTITION, "partition leaves an empty slab");
  // _DeterminePartitionType
  const uint64_t total = (uint64_t)(uint16_t)gpu_count * gpu_mem_bytes;
  const uint64_t required = nnz * (order * p.isz + p.vsz) + (uint64_t)gpu_count * p.core() +
                            (uint64_t)gpu_count * p.all_factors() + nnz * p.J * p.vsz;
  int streams = 1;
  const bool dim_based = required > total;
  if (dim_based) {  // _DimensionBasedPartitioning
    streams = 4;
    const uint64_t buf = gpu_mem_bytes / (uint64_t)streams;
    const uint32_t total_streams = (uint32_t)gpu_count * (uint32_t)streams;
    do {
      const int axis = p.next_axis();
      p.P[axis]++;
      if (!p.refresh())
        return fail(GTK_ERR_PARTITION, "no partition fits: P_" + std::to_string(axis) + " = " +
                                             std::to_string(p.P[axis]) + " leaves an empty slab of dim " +
                                             std::to_string(dims[axis]) + " (the reference throws here)");
    } while (!(p.all_data() < buf && p.nblk >= total_streams));
  }
  // _AvailableNonzeroCountPerTask (unsigned wrap kept)
  const uint64_t buf = gpu_mem_bytes / (uint64_t)streams;
  const uint64_t avail_buf = buf - (p.core() + p.sub_factors());
  memset(out, 0, sizeof(*out));
  for (int n = 0; n < order; ++n) {
    out->partition_dims[n] = p.P[n];
    out->block_dims[n] = p.bd[n];
  }
  out->block_count = p.nblk;
  out->dimension_based = dim_based ? 1 : 0;
  out->streams = streams;
  out->avail_nnz_per_task = avail_buf / (order * p.isz + p.vsz + p.J * p.vsz);
  out->required_bytes = required;
  out->block_bytes = p.all_data();
  return 0;
}

int gtk_device_memory(int device, uint64_t *free_bytes, uint64_t *total_bytes) {
  if (!free_bytes || !total_bytes) return fail(GTK_ERR_ARG, "null output");
  int cur = 0;
  GTK_CUDA(cudaGetDevice(&cur));
  GTK_CUDA(cudaSetDevice(device));
  size_t f = 0, t = 0;
  const cudaError_t e = cudaMemGetInfo(&f, &t);
  cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
  *free_bytes = f + dev_cached_bytes(device);  // blocks the library keeps cached are free for its own use
  *total_bytes = t;
  return 0;
}

void gtk_release_cached_memory(void) { dev_cache_clear(-1); }

int gtk_checkpoint_save(gtk_tensor *t, const char *path, const double *fits, int nfits) {
  if (!t || !path || nfits < 0 || (nfits > 0 && !fits)) return fail(GTK_ERR_ARG, "bad argument");
  if (!t->have_factors || !t->have_core) return fail(GTK_ERR_STATE, "factors and core are not initialised");
  const std::string tmp = std::string(path) + ".tmp";
  FILE *f = fopen(tmp.c_str(), "wb");
  if (!f) return fail(GTK_ERR_IO, "cannot write " + tmp);
  Writer w{f};
  w.put(kMagic, 8);
  w.u32(1);
  w.u32((uint32_t)t->N);
  w.u32((uint32_t)t->J);
  w.u32((uint32_t)t->dtype);
  for (int n = 0; n < t->N; ++n) w.u32(t->dims[n]);
  for (int n = 0; n < t->N; ++n) w.u32(t->P[n]);
  for (int n = 0; n < t->N; ++n) w.u32(t->bd[n]);
  w.u32((uint32_t)nfits);
  if (nfits) w.put(fits, sizeof(double) * (size_t)nfits);
  int rc = 0;
  std::vector<unsigned char> buf;
  for (int n = 0; n < t->N && !rc && w.ok; ++n) {
    buf.resize(t->rows[n] * (size_t)t->J * t->vsize);
    rc = gtk_get_factor(t, n, buf.data());
    if (!rc) w.put(buf.data(), buf.size());
  }
  if (!rc && w.ok) {
    buf.resize(t->core_n * t->vsize);
    rc = gtk_get_core(t, buf.data());
    if (!rc) w.put(buf.data(), buf.size());
  }
  const uint64_t h = w.h;
  if (!rc && w.ok) w.ok = fwrite(&h, 8, 1, f) == 1;
  const bool closed = fclose(f) == 0;
  if (rc || !w.ok || !closed) {
    remove(tmp.c_str());
    return rc ? rc : fail(GTK_ERR_IO, "write failed: " + tmp);
  }
  if (rename(tmp.c_str(), path) != 0) {
    remove(tmp.c_str());
    return fail(GTK_ERR_IO, std::string("cannot rename to ") + path);
  }
  return 0;
}

int gtk_checkpoint_info(const char *path, int *order, int *rank, int *dtype, uint32_t *dims, uint32_t *partition_dims,
                        int *nfits) {
  if (!path) return fail(GTK_ERR_ARG, "null path");
  FILE *f = fopen(path, "rb");
  if (!f) return fail(GTK_ERR_IO, std::string("cannot open ") + path);
  Reader r{f};
  Header h;
  const int rc = read_header(r, h, path);
  fclose(f);
  if (rc) return rc;
  if (order) *order = (int)h.order;
  if (rank) *rank = (int)h.rank;
  if (dtype) *dtype = (int)h.dtype;
  for (uint32_t n = 0; n < h.order; ++n) {
    if (dims) dims[n] = h.dims[n];
    if (partition_dims) partition_dims[n] = h.P[n];
  }
  if (nfits) *nfits = (int)h.nfits;
  return 0;
}

int gtk_checkpoint_load(gtk_tensor *t, const char *path, double *fits, int fits_cap, int *nfits) {
  if (!t || !path || fits_cap < 0 || (fits_cap > 0 && !fits)) return fail(GTK_ERR_ARG, "bad argument");
  FILE *f = fopen(path, "rb");
  if (!f) return fail(GTK_ERR_IO, std::string("cannot open ") + path);
  Reader r{f};
  Header h;
  if (int rc = read_header(r, h, path)) {
    fclose(f);
    return rc;
  }
  bool same = h.order == (uint32_t)t->N && h.rank == (uint32_t)t->J && h.dtype == (uint32_t)t->dtype;
  for (uint32_t n = 0; same && n < h.order; ++n)
    same = h.dims[n] == t->dims[n] && h.P[n] == t->P[n] && h.bd[n] == t->bd[n];
  if (!same) {
    fclose(f);
    return fail(GTK_ERR_ARG, "checkpoint is for another tensor shape, rank, value type or partition");
  }
  std::vector<double> fv(h.nfits);
  if (h.nfits) r.get(fv.data(), 8 * (size_t)h.nfits);
  std::vector<std::vector<unsigned char>> fac(t->N);
  for (int n = 0; n < t->N && r.ok; ++n) {
    fac[n].resize(t->rows[n] * (size_t)t->J * t->vsize);
    r.get(fac[n].data(), fac[n].size());
  }
  std::vector<unsigned char> core(t->core_n * t->vsize);
  r.get(core.data(), core.size());
  const uint64_t want = r.h;
  uint64_t got = 0;
  const bool tail = r.ok && fread(&got, 8, 1, f) == 1;
  char extra;
  const bool at_end = tail && fread(&extra, 1, 1, f) == 0;
  fclose(f);
  if (!r.ok || !tail) return fail(GTK_ERR_PARSE, "truncated checkpoint");
  if (got != want || !at_end) return fail(GTK_ERR_PARSE, "checkpoint checksum mismatch (corrupt file)");
  for (int n = 0; n < t->N; ++n)
    if (int rc = gtk_set_factor(t, n, fac[n].data())) return rc;
  if (int rc = gtk_set_core(t, core.data())) return rc;
  const int k = std::min<int>((int)h.nfits, fits_cap);
  for (int i = 0; i < k; ++i) fits[i] = fv[(size_t)h.nfits - k + i];  // the most recent ones
  if (nfits) *nfits = (int)h.nfits;
  return 0;
}

}  // extern "C"
