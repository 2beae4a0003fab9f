// ref_driver.cu -- drives the GPUTucker reference's own host code, compiled in
// place from the reference sources (see oracle/Makefile), so that the CPU
// restatement in gtk_oracle.cpp can be pinned against it.
//
// TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ (git-ignored) in a
// container that has the reference sources; never shipped, never on the
// product path.
//
// Reference code used unmodified (paths inside the GPUTucker project):
//   ParseFromFile / _ReadData ...... include/gputucker/tensor_manager.tpp:19-191
//   CreateTensorBlocks ............. include/gputucker/tensor_manager.tpp:201-302
//   Block::AssignIndicesToEachMode . include/gputucker/block.tpp:115-186
//   ComputingBC .................... include/gputucker/update.cuh:35-101
//   frand .......................... include/gputucker/helper.hpp:99
//   Eigen::MatrixXd::inverse ....... lib/Eigen (vendored 3.3.91)
// Restated here because they live inside GPU-only or monolithic functions:
//   the init draw order (tucker.cuh:84-134), the delta kernel body
//   (delta.cuh:62-90), the row-solve loop (update.cuh:163-194) and the
//   reconstruction kernel body + error loop (reconstruction.cuh:58-81, 259-276).

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gputucker/block.hpp"
#include "gputucker/constants.hpp"
#include "gputucker/helper.hpp"
#include "gputucker/optimizer.hpp"
#include "gputucker/tensor.hpp"
#include "gputucker/tensor_manager.hpp"
#include "gputucker/update.cuh"

using namespace supertensor::gputucker;

namespace {

thread_local std::string g_err;

template <class V> struct Ref {
  using block_t = Block<uint32_t, V>;
  using tensor_t = Tensor<block_t>;
  tensor_t *src = nullptr;   // parsed tensor (1 block, global 0-based coords)
  tensor_t *dst = nullptr;   // blocked tensor
  int J = 0;
  V **fac[constants::kMaxOrder] = {};
  std::vector<V> core;
  std::vector<std::vector<uint32_t>> core_idx;
  uint64_t core_n = 1;
};

struct Handle {
  int dtype;
  Ref<float> f;
  Ref<double> d;
};

template <class V> int do_parse(Ref<V> &r, const char *path, int order) {
  try {
    r.src = new typename Ref<V>::tensor_t((unsigned short)order);
    ParseFromFile<typename Ref<V>::tensor_t>(std::string(path), &r.src);
  } catch (std::exception &e) {
    g_err = e.what();
    return 3;
  }
  return 0;
}

template <class V> int do_blocks(Ref<V> &r, const uint32_t *P, int J) {
  using tensor_t = typename Ref<V>::tensor_t;
  try {
    Optimizer<tensor_t> *opt = new Optimizer<tensor_t>();
    int N = r.src->order;
    opt->block_dims = allocate<uint32_t>(N);
    opt->partition_dims = allocate<uint32_t>(N);
    opt->block_count = 1;
    for (int n = 0; n < N; ++n) {
      opt->partition_dims[n] = P[n];
      opt->block_dims[n] = (r.src->dims[n] + P[n] - 1) / P[n];
      opt->block_count *= P[n];
    }
    r.dst = new tensor_t(r.src);
    CreateTensorBlocks<tensor_t, Optimizer<tensor_t>>(&r.src, &r.dst, opt);
  } catch (std::exception &e) {
    g_err = e.what();
    return 4;
  }
  r.J = J;
  int N = r.dst->order;
  for (int n = 0; n < N; ++n) {
    uint32_t P_n = r.dst->partition_dims[n];
    r.fac[n] = (V **)malloc(sizeof(V *) * P_n);
    for (uint32_t p = 0; p < P_n; ++p) r.fac[n][p] = (V *)calloc((size_t)r.dst->block_dims[n] * J, sizeof(V));
  }
  r.core_n = 1;
  for (int n = 0; n < N; ++n) r.core_n *= (uint64_t)J;
  r.core.assign(r.core_n, V(0));
  r.core_idx.assign(N, std::vector<uint32_t>(r.core_n));
  for (uint64_t i = 0; i < r.core_n; ++i) {
    uint64_t rem = i;
    for (int n = N - 1; n >= 0; --n) {
      r.core_idx[n][i] = (uint32_t)(rem % J);
      rem /= J;
    }
  }
  return 0;
}

// tucker.cuh:84-134 draw order, using the reference's frand
template <class V> void do_init(Ref<V> &r) {
  int N = r.dst->order, J = r.J;
  for (int axis = 0; axis < N; ++axis) {
    uint32_t rows = r.dst->block_dims[axis];
    for (uint32_t part = 0; part < r.dst->partition_dims[axis]; ++part) {
      if (part + 1 == r.dst->partition_dims[axis]) rows = r.dst->dims[axis] - part * r.dst->block_dims[axis];
      for (uint32_t row = 0; row < rows; ++row)
        for (int col = 0; col < J; ++col) r.fac[axis][part][row * J + col] = frand<double>(0, 1);
    }
  }
  for (uint64_t i = 0; i < r.core_n; ++i) r.core[i] = frand<double>(0, 1);
}

// delta.cuh:62-90 for every nonzero of every block
template <class V> void do_delta(Ref<V> &r, int mode, V **delta) {
  int N = r.dst->order, J = r.J;
  for (uint64_t b = 0; b < r.dst->block_count; ++b) {
    auto *blk = r.dst->blocks[b];
    uint32_t *coord = blk->get_block_coord();
#pragma omp parallel for
    for (long long t = 0; t < (long long)blk->nnz_count; ++t) {
      V tmp[64];
      for (int j = 0; j < J; ++j) tmp[j] = 0;
      for (uint64_t i = 0; i < r.core_n; ++i) {
        V beta = r.core[i];
        for (int n = 0; n < N; ++n)
          if (n != mode) beta *= r.fac[n][coord[n]][blk->indices[n][t] * J + r.core_idx[n][i]];
        tmp[r.core_idx[mode][i]] += beta;
      }
      for (int j = 0; j < J; ++j) delta[b][t * J + j] = tmp[j];
    }
  }
}

template <class V> void do_update(Ref<V> &r, int mode) {
  using tensor_t = typename Ref<V>::tensor_t;
  int J = r.J;
  uint64_t nb = r.dst->block_count;
  std::vector<V *> delta(nb);
  for (uint64_t b = 0; b < nb; ++b) delta[b] = (V *)malloc(sizeof(V) * (r.dst->blocks[b]->nnz_count * J + 1));
  do_delta(r, mode, delta.data());
  uint32_t maxp = 0, maxbd = 0;
  for (int n = 0; n < r.dst->order; ++n) {
    maxp = std::max(maxp, r.dst->partition_dims[n]);
    maxbd = std::max(maxbd, r.dst->block_dims[n]);
  }
  std::vector<double *> B(maxp), C(maxp);
  for (uint32_t p = 0; p < maxp; ++p) {
    B[p] = (double *)malloc(sizeof(double) * (size_t)maxbd * J * J);
    C[p] = (double *)malloc(sizeof(double) * (size_t)maxbd * J);
  }
  ComputingBC<tensor_t, double, V>(r.dst, delta.data(), B.data(), C.data(), mode, J);
  // update.cuh:163-194
  uint32_t rows = r.dst->block_dims[mode];
  for (uint32_t p = 0; p < r.dst->partition_dims[mode]; ++p) {
#pragma omp parallel for schedule(static)
    for (long long rr = 0; rr < (long long)rows; ++rr) {
      uint64_t row = (uint64_t)rr;
      Eigen::MatrixXd BB(J, J);
      for (int k = 0; k < J; ++k)
        for (int l = 0; l < J; ++l) BB(k, l) = B[p][row * J * J + k * J + l];
      Eigen::MatrixXd Binv = BB.inverse();
      for (int k = 0; k < J; ++k) {
        V res = 0;
        for (int l = 0; l < J; ++l) res += C[p][row * J + l] * Binv(l, k);
        r.fac[mode][p][row * J + k] = res;
      }
    }
  }
  for (uint32_t p = 0; p < maxp; ++p) { free(B[p]); free(C[p]); }
  for (uint64_t b = 0; b < nb; ++b) free(delta[b]);
}

// reconstruction.cuh:58-81 and 259-276 (value_t serial error, as the reference)
template <class V> double do_fit(Ref<V> &r, double *err_out) {
  int N = r.dst->order, J = r.J;
  V Error = 0;
  for (uint64_t b = 0; b < r.dst->block_count; ++b) {
    auto *blk = r.dst->blocks[b];
    uint32_t *coord = blk->get_block_coord();
    std::vector<V> xh(blk->nnz_count);
#pragma omp parallel for
    for (long long t = 0; t < (long long)blk->nnz_count; ++t) {
      V res = 0;
      for (uint64_t i = 0; i < r.core_n; ++i) {
        V tmp = r.core[i];
        for (int n = 0; n < N; ++n) tmp *= r.fac[n][coord[n]][blk->indices[n][t] * J + r.core_idx[n][i]];
        res += tmp;
      }
      xh[t] = res;
    }
    for (uint64_t t = 0; t < blk->nnz_count; ++t) {
      V e = blk->values[t] - xh[t];
      Error += e * e;
    }
  }
  if (err_out) *err_out = (double)Error;
  if (r.dst->norm == 0) return 1.0;
  return 1.0f - std::sqrt(Error) / r.dst->norm;
}

}  // namespace

#define REF_DISPATCH(h, expr)                              \
  do {                                                     \
    if ((h)->dtype == 0) { auto &r = (h)->f; expr; }       \
    else { auto &r = (h)->d; expr; }                       \
  } while (0)

namespace {

// Optimizer::FindPartitionParms (optimizer.tpp:71-89) on a tensor that has only
// order, dims and nnz_count set -- all the planner reads.
template <class V>
int do_plan(int order, const uint32_t *dims, uint64_t nnz, int J, int gpus, uint64_t mem, uint32_t *P, uint32_t *bd,
            uint64_t *info) {
  using tensor_t = typename Ref<V>::tensor_t;
  try {
    tensor_t *t = new tensor_t((unsigned short)order);
    for (int n = 0; n < order; ++n) t->dims[n] = dims[n];
    t->nnz_count = nnz;
    Optimizer<tensor_t> *opt = new Optimizer<tensor_t>();
    opt->Initialize((unsigned short)gpus, (unsigned)J, mem, t);
    uint32_t *pd = opt->FindPartitionParms();
    for (int n = 0; n < order; ++n) {
      P[n] = pd[n];
      bd[n] = opt->block_dims[n];
    }
    info[0] = opt->block_count;
    info[1] = opt->partition_type == enums::PartitionTypes::kDimensionPartition ? 1 : 0;
    info[2] = (uint64_t)opt->cuda_stream_count;
    info[3] = opt->avail_nnz_count_per_task;
  } catch (std::exception &e) {
    g_err = e.what();
    return 3;
  }
  return 0;
}

}  // namespace

extern "C" {

int ref_plan(int order, const uint32_t *dims, uint64_t nnz, int J, int dtype, int gpus, uint64_t mem, uint32_t *P,
             uint32_t *bd, uint64_t *info) {
  return dtype == 1 ? do_plan<double>(order, dims, nnz, J, gpus, mem, P, bd, info)
                    : do_plan<float>(order, dims, nnz, J, gpus, mem, P, bd, info);
}

const char *ref_last_error(void) { return g_err.c_str(); }

// srand(seed) then ParseFromFile; returns handle or NULL
void *ref_parse_file(const char *path, int order, int dtype, unsigned seed, int *status) {
  srand(seed);
  Handle *h = new Handle();
  h->dtype = dtype;
  int rc;
  REF_DISPATCH(h, rc = do_parse(r, path, order));
  *status = rc;
  if (rc) { delete h; return nullptr; }
  return h;
}

void ref_parsed(void *hp, uint64_t *nnz, uint32_t *dims, uint32_t *const *idx, void *vals) {
  Handle *h = (Handle *)hp;
  REF_DISPATCH(h, {
    *nnz = r.src->nnz_count;
    for (int n = 0; n < r.src->order; ++n) dims[n] = r.src->dims[n];
    if (idx) {
      for (int n = 0; n < r.src->order; ++n) memcpy(idx[n], r.src->blocks[0]->indices[n], sizeof(uint32_t) * r.src->nnz_count);
      memcpy(vals, r.src->blocks[0]->values, sizeof(r.src->blocks[0]->values[0]) * r.src->nnz_count);
    }
  });
}

int ref_blocks(void *hp, const uint32_t *P, int J) {
  Handle *h = (Handle *)hp;
  int rc;
  REF_DISPATCH(h, rc = do_blocks(r, P, J));
  return rc;
}

void ref_info(void *hp, uint32_t *bd, uint64_t *nblk, double *norm) {
  Handle *h = (Handle *)hp;
  REF_DISPATCH(h, {
    for (int n = 0; n < r.dst->order; ++n) bd[n] = r.dst->block_dims[n];
    *nblk = r.dst->block_count;
    *norm = (double)r.dst->norm;
  });
}

// same layout as ora_partition
void ref_partition(void *hp, uint64_t *blk_ptr, uint32_t *blk_coord, uint32_t *const *idx, void *vals,
                   uint64_t *const *count, uint32_t *const *where) {
  Handle *h = (Handle *)hp;
  REF_DISPATCH(h, {
    int N = r.dst->order;
    uint64_t off = 0;
    for (uint64_t b = 0; b < r.dst->block_count; ++b) {
      auto *blk = r.dst->blocks[b];
      blk_ptr[b] = off;
      for (int n = 0; n < N; ++n) blk_coord[b * N + n] = blk->get_block_coord()[n];
      for (int n = 0; n < N; ++n) {
        memcpy(idx[n] + off, blk->indices[n], sizeof(uint32_t) * blk->nnz_count);
        memcpy(where[n] + off, blk->where_nnz[n], sizeof(uint32_t) * blk->nnz_count);
        uint64_t rows = r.dst->block_dims[n];
        memcpy(count[n] + b * (rows + 1), blk->count_nnz[n], sizeof(uint64_t) * (rows + 1));
      }
      memcpy((char *)vals + off * sizeof(blk->values[0]), blk->values, sizeof(blk->values[0]) * blk->nnz_count);
      off += blk->nnz_count;
    }
    blk_ptr[r.dst->block_count] = off;
  });
}

// srand(seed), discard `skip` draws, then the reference init order
void ref_init_random(void *hp, unsigned seed, uint64_t skip) {
  Handle *h = (Handle *)hp;
  srand(seed);
  for (uint64_t k = 0; k < skip; ++k) (void)rand();
  REF_DISPATCH(h, do_init(r));
}

void ref_get_factor(void *hp, int n, void *out) {
  Handle *h = (Handle *)hp;
  REF_DISPATCH(h, {
    size_t slab = (size_t)r.dst->block_dims[n] * r.J;
    for (uint32_t p = 0; p < r.dst->partition_dims[n]; ++p)
      memcpy((char *)out + p * slab * sizeof(r.fac[n][p][0]), r.fac[n][p], slab * sizeof(r.fac[n][p][0]));
  });
}

void ref_get_core(void *hp, void *out) {
  Handle *h = (Handle *)hp;
  REF_DISPATCH(h, memcpy(out, r.core.data(), r.core.size() * sizeof(r.core[0])));
}

void ref_delta(void *hp, int mode, void *out) {
  Handle *h = (Handle *)hp;
  REF_DISPATCH(h, {
    using V = typename std::remove_reference<decltype(r.core[0])>::type;
    std::vector<V *> d(r.dst->block_count);
    uint64_t off = 0;
    for (uint64_t b = 0; b < r.dst->block_count; ++b) {
      d[b] = (V *)out + off * r.J;
      off += r.dst->blocks[b]->nnz_count;
    }
    do_delta(r, mode, d.data());
  });
}

void ref_update_mode(void *hp, int mode) {
  Handle *h = (Handle *)hp;
  REF_DISPATCH(h, do_update(r, mode));
}

double ref_fit(void *hp, double *err) {
  Handle *h = (Handle *)hp;
  double f;
  REF_DISPATCH(h, f = do_fit(r, err));
  return f;
}

}  // extern "C"
