// gtk_oracle.cpp -- CPU restatement of GPUTucker's sparse Tucker ALS path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
// library in gputucker_gb300/: only tests/, __graft_entry__.smoke() and the
// CPU-baseline / reference legs of bench.py load it.  Nothing in the product
// path links or calls it.
//
// Every stage restates the reference's algorithm with its summation order
// (citations are paths inside the GPUTucker project):
//   * glibc rand() replay ...... helper.hpp:99 (frand), tucker.cuh:84-134 (draw order)
//   * text parser .............. tensor_manager.tpp:46-191
//   * block partition + norm ... tensor_manager.tpp:201-302, tensor.tpp:157-213, block.tpp:100-108
//   * per-mode segmenting ...... block.tpp:115-186
//   * delta formula ............ delta.cuh:62-90
//   * B/C accumulation ......... update.cuh:35-101
//   * row solve ................ update.cuh:163-194 (Eigen PartialPivLU inverse, restated)
//   * reconstruction / fit ..... reconstruction.cuh:58-81, 259-276
//
// value_t is float (the reference's FP32 instantiation) or double (main.cu:25,
// the FP64 oracle); B and C are always double (tucker.cuh:140).
// Pinned against the reference's own host code compiled from its sources
// (oracle/Makefile -> oracle/_ref) by tests/test_oracle_pin.py, and against
// the committed fixtures in tests/golden/.

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kMaxOrder = 8;          // constants.hpp:16
constexpr double kLambda = 0.0001f;   // constants.hpp:18 (a float literal widened to double)
constexpr double kRandMax = 2147483647.0;

thread_local std::string g_err;

// glibc rand(): the TYPE_3 additive-feedback generator (r[i] = r[i-31] + r[i-3],
// output r[i] >> 1 after discarding 310 warm-up words), seeded by the
// Lehmer/Schrage recurrence 16807 mod 2^31-1.  The reference never seeds it,
// which is srand(1); srand(0) is the same stream.
struct GlibcRand {
  uint32_t ring[31];
  uint64_t i;
  explicit GlibcRand(uint32_t seed) { reseed(seed); }
  void reseed(uint32_t seed) {
    int32_t r[34];
    r[0] = (int32_t)(seed == 0 ? 1u : seed);
    for (int k = 1; k < 31; ++k) {
      long word = r[k - 1];
      long hi = word / 127773, lo = word % 127773;
      word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      r[k] = (int32_t)word;
    }
    for (int k = 31; k < 34; ++k) r[k] = r[k - 31];
    for (int k = 3; k < 34; ++k) ring[k % 31] = (uint32_t)r[k];
    i = 34;
    for (int k = 34; k < 344; ++k) step();
  }
  uint32_t step() {
    uint32_t v = ring[i % 31] + ring[(i - 3) % 31];
    ring[i % 31] = v;
    ++i;
    return v;
  }
  int next() { return (int)(step() >> 1); }
};

// frand<T>(0,1) = (1 - 0) * (T(rand()) / RAND_MAX) + 0   (helper.hpp:99)
template <class T> T frand01(GlibcRand &g) {
  return (T(1) - T(0)) * (static_cast<T>(g.next()) / RAND_MAX) + T(0);
}

template <class V> struct Ora {
  int N = 0, J = 0;
  uint64_t nnz = 0, nblk = 1;
  uint32_t dims[kMaxOrder] = {}, P[kMaxOrder] = {}, bd[kMaxOrder] = {};
  std::vector<uint64_t> blk_ptr;                  // block b occupies [blk_ptr[b], blk_ptr[b+1])
  std::vector<uint32_t> blk_coord;                // [nblk][N]
  std::vector<std::vector<uint32_t>> idx;         // [N][nnz] block-local coords, block-major
  std::vector<V> val;                             // [nnz]
  std::vector<std::vector<uint64_t>> count_nnz;   // [N][nblk*(bd+1)]
  std::vector<std::vector<uint32_t>> where_nnz;   // [N][nnz] position inside the block
  V norm_ref = 0;                                 // value_t serial sum (tensor_manager.tpp:263-293)
  double norm64 = 0;                              // same sum in double
  std::vector<std::vector<V>> fac;                // [N][P*bd*J] slabs concatenated
  std::vector<V> core;                            // [J^N] linear, last mode fastest
  uint64_t core_n = 1;
  std::vector<std::vector<uint32_t>> core_idx;    // [N][J^N]

  uint32_t gidx(int n, uint64_t b, uint64_t t) const {
    return blk_coord[b * N + n] * bd[n] + idx[n][t];
  }
};

// tensor.tpp:157-174 (block id -> block coordinate, last mode fastest)
static void block_coord_of(uint64_t b, int N, const uint32_t *P, uint32_t *c) {
  for (int n = N - 1; n >= 0; --n) {
    c[n] = (uint32_t)(b % P[n]);
    b /= P[n];
  }
}

template <class V>
int build(Ora<V> &o, int N, uint64_t nnz, const uint32_t *const *gi, const V *vals, const uint32_t *dims,
          const uint32_t *P, int J) {
  if (N < 1 || N > kMaxOrder || J < 1) { g_err = "bad order/rank"; return 1; }
  o.N = N; o.J = J; o.nnz = nnz; o.nblk = 1;
  for (int n = 0; n < N; ++n) {
    if (P[n] == 0 || dims[n] == 0) { g_err = "zero dim or partition"; return 1; }
    o.dims[n] = dims[n];
    o.P[n] = P[n];
    // tensor.tpp:203-209 / optimizer.tpp:367-371
    o.bd[n] = (dims[n] + P[n] - 1) / P[n];
    uint32_t check = (dims[n] + o.bd[n] - 1) / o.bd[n];
    if (check != P[n]) { g_err = "Block dimension is larger than the tensor dimension."; return 4; }
    o.nblk *= P[n];
  }
  // histogram (tensor_manager.tpp:224-258)
  std::vector<uint64_t> bid(nnz), hist(o.nblk, 0);
  for (uint64_t t = 0; t < nnz; ++t) {
    uint64_t b = 0, mult = 1;
    for (int it = 0; it < N; ++it) {
      int n = N - it - 1;
      if (gi[n][t] >= dims[n]) { g_err = "coordinate out of bounds"; return 1; }
      b += (uint64_t)(gi[n][t] / o.bd[n]) * mult;
      mult *= P[n];
    }
    bid[t] = b;
    ++hist[b];
  }
  o.blk_ptr.assign(o.nblk + 1, 0);
  for (uint64_t b = 0; b < o.nblk; ++b) o.blk_ptr[b + 1] = o.blk_ptr[b] + hist[b];
  o.blk_coord.assign(o.nblk * N, 0);
  for (uint64_t b = 0; b < o.nblk; ++b) block_coord_of(b, N, P, &o.blk_coord[b * N]);
  // serial insert in file order (tensor_manager.tpp:267-290, block.tpp:100-108):
  // position in block = nnz_count - remaining, i.e. arrival order.
  o.idx.assign(N, std::vector<uint32_t>(nnz));
  o.val.assign(nnz, V(0));
  std::vector<uint64_t> fill(o.blk_ptr.begin(), o.blk_ptr.end() - 1);
  V normx = 0;
  double norm64 = 0;
  for (uint64_t t = 0; t < nnz; ++t) {
    uint64_t b = bid[t], p = fill[b]++;
    for (int n = 0; n < N; ++n) o.idx[n][p] = gi[n][t] - o.blk_coord[b * N + n] * o.bd[n];
    V v = vals[t];
    o.val[p] = v;
    normx += v * v;
    norm64 += (double)v * (double)v;
  }
  o.norm_ref = std::sqrt(normx);
  o.norm64 = std::sqrt(norm64);
  // per-mode segmenting (block.tpp:115-186): CSR row pointer + stable counting sort
  o.count_nnz.assign(N, std::vector<uint64_t>());
  o.where_nnz.assign(N, std::vector<uint32_t>(nnz));
  for (int n = 0; n < N; ++n) {
    uint64_t rows = o.bd[n];
    o.count_nnz[n].assign(o.nblk * (rows + 1), 0);
#pragma omp parallel for schedule(dynamic)
    for (long long bb = 0; bb < (long long)o.nblk; ++bb) {
      uint64_t b = (uint64_t)bb;
      uint64_t *cnt = &o.count_nnz[n][b * (rows + 1)];
      uint64_t s = o.blk_ptr[b], e = o.blk_ptr[b + 1];
      std::vector<uint64_t> tmp(rows + 1, 0);
      for (uint64_t t = s; t < e; ++t) ++cnt[o.idx[n][t]];
      uint32_t now = 0;  // index_t accumulator in the reference
      for (uint64_t r = 0; r < rows; ++r) {
        uint64_t k = cnt[r];
        cnt[r] = now;
        tmp[r] = now;
        now += (uint32_t)k;
      }
      cnt[rows] = now;
      for (uint64_t t = s; t < e; ++t) {
        uint32_t k = o.idx[n][t];
        o.where_nnz[n][s + tmp[k]] = (uint32_t)(t - s);
        ++tmp[k];
      }
    }
  }
  // core index table (tucker.cuh:118-134)
  o.core_n = 1;
  for (int n = 0; n < N; ++n) o.core_n *= (uint64_t)J;
  o.core_idx.assign(N, std::vector<uint32_t>(o.core_n));
  for (uint64_t i = 0; i < o.core_n; ++i) {
    uint64_t r = i;
    for (int n = N - 1; n >= 0; --n) {
      o.core_idx[n][i] = (uint32_t)(r % J);
      r /= J;
    }
  }
  o.fac.assign(N, std::vector<V>());
  for (int n = 0; n < N; ++n) o.fac[n].assign((uint64_t)o.P[n] * o.bd[n] * J, V(0));
  o.core.assign(o.core_n, V(0));
  return 0;
}

// tucker.cuh:84-134: mode 0..N-1, slab 0..P-1, real rows only, col; then the core
template <class V> void init_random(Ora<V> &o, uint32_t seed, uint64_t skip) {
  GlibcRand g(seed);
  for (uint64_t k = 0; k < skip; ++k) g.next();
  for (int n = 0; n < o.N; ++n) {
    std::fill(o.fac[n].begin(), o.fac[n].end(), V(0));
    for (uint32_t p = 0; p < o.P[n]; ++p) {
      uint32_t rows = o.bd[n];
      if (p + 1 == o.P[n]) rows = o.dims[n] - p * o.bd[n];
      for (uint32_t r = 0; r < rows; ++r)
        for (int c = 0; c < o.J; ++c)
          o.fac[n][((uint64_t)p * o.bd[n] + r) * o.J + c] = (V)frand01<double>(g);
    }
  }
  for (uint64_t i = 0; i < o.core_n; ++i) o.core[i] = (V)frand01<double>(g);
}

// delta.cuh:62-90 for one nonzero (block b, block-major position t)
template <class V> void delta_one(const Ora<V> &o, int mode, uint64_t b, uint64_t t, V *out) {
  const int N = o.N, J = o.J;
  V tmp[64];
  for (int r = 0; r < J; ++r) tmp[r] = V(0);
  uint64_t row[kMaxOrder];
  for (int n = 0; n < N; ++n) row[n] = (uint64_t)o.gidx(n, b, t) * J;
  for (uint64_t i = 0; i < o.core_n; ++i) {
    V beta = o.core[i];
    for (int n = 0; n < N; ++n)
      if (n != mode) beta *= o.fac[n][row[n] + o.core_idx[n][i]];
    tmp[o.core_idx[mode][i]] += beta;
  }
  for (int r = 0; r < J; ++r) out[r] = tmp[r];
}

template <class V> void compute_delta(const Ora<V> &o, int mode, V *delta /* [nnz][J] block-major */) {
  for (uint64_t b = 0; b < o.nblk; ++b) {
    long long s = (long long)o.blk_ptr[b], e = (long long)o.blk_ptr[b + 1];
#pragma omp parallel for schedule(static)
    for (long long t = s; t < e; ++t) delta_one(o, mode, b, (uint64_t)t, delta + (uint64_t)t * o.J);
  }
}

// Eigen::PartialPivLU(...).inverse() restated: LU with row pivoting, then solve A X = I.
static bool inverse_pplu(int J, const double *A, double *inv) {
  std::vector<double> lu(A, A + (size_t)J * J);
  std::vector<int> perm(J);
  for (int i = 0; i < J; ++i) perm[i] = i;
  for (int k = 0; k < J; ++k) {
    int piv = k;
    double best = std::fabs(lu[(size_t)k * J + k]);
    for (int i = k + 1; i < J; ++i) {
      double v = std::fabs(lu[(size_t)i * J + k]);
      if (v > best) { best = v; piv = i; }
    }
    if (piv != k) {
      for (int c = 0; c < J; ++c) std::swap(lu[(size_t)k * J + c], lu[(size_t)piv * J + c]);
      std::swap(perm[k], perm[piv]);
    }
    double d = lu[(size_t)k * J + k];
    if (d == 0.0) continue;
    for (int i = k + 1; i < J; ++i) {
      double f = lu[(size_t)i * J + k] /= d;
      for (int c = k + 1; c < J; ++c) lu[(size_t)i * J + c] -= f * lu[(size_t)k * J + c];
    }
  }
  for (int col = 0; col < J; ++col) {
    std::vector<double> y(J);
    for (int i = 0; i < J; ++i) {
      double s = (perm[i] == col) ? 1.0 : 0.0;
      for (int c = 0; c < i; ++c) s -= lu[(size_t)i * J + c] * y[c];
      y[i] = s;
    }
    for (int i = J - 1; i >= 0; --i) {
      double s = y[i];
      for (int c = i + 1; c < J; ++c) s -= lu[(size_t)i * J + c] * y[c];
      y[i] = s / lu[(size_t)i * J + i];
    }
    for (int i = 0; i < J; ++i) inv[(size_t)i * J + col] = y[i];
  }
  return true;
}

// update.cuh:128-199 for one mode: delta, ComputingBC, row solve
template <class V> void update_mode(Ora<V> &o, int mode) {
  const int J = o.J;
  const uint64_t rows = o.bd[mode];
  std::vector<V> delta(o.nnz * (uint64_t)J);
  compute_delta(o, mode, delta.data());
  // ComputingBC (update.cuh:52-100)
  const uint32_t P = o.P[mode];
  std::vector<std::vector<double>> B(P, std::vector<double>(rows * J * J)), C(P, std::vector<double>(rows * J));
  for (uint32_t p = 0; p < P; ++p) {
    for (uint64_t r = 0; r < rows; ++r) {
      for (int k = 0; k < J; ++k) {
        for (int l = 0; l < J; ++l) B[p][r * J * J + k * J + l] = (k == l) ? kLambda : 0.0;
        C[p][r * J + k] = 0.0;
      }
    }
  }
  for (uint64_t b = 0; b < o.nblk; ++b) {
    uint32_t part = o.blk_coord[b * o.N + mode];
    const uint64_t *cnt = &o.count_nnz[mode][b * (rows + 1)];
    const uint64_t s = o.blk_ptr[b];
#pragma omp parallel for schedule(dynamic)
    for (long long rr = 0; rr < (long long)rows; ++rr) {
      uint64_t r = (uint64_t)rr;
      uint64_t n_in = cnt[r + 1] - cnt[r];
      uint64_t wp = cnt[r];
      for (uint64_t kk = 0; kk < n_in; ++kk) {
        uint64_t pos = o.where_nnz[mode][s + wp + kk];
        V x = o.val[s + pos];
        const V *d = &delta[(s + pos) * J];
        double *Br = &B[part][r * J * J];
        double *Cr = &C[part][r * J];
        for (int i = 0; i < J; ++i) {
          V c = d[i];
          for (int j = 0; j < J; ++j) Br[i * J + j] += c * d[j];
          Cr[i] += c * x;
        }
      }
    }
  }
  // row solve (update.cuh:163-194): a = C^T * inverse(B), accumulated in value_t
  for (uint32_t p = 0; p < P; ++p) {
#pragma omp parallel for schedule(static)
    for (long long rr = 0; rr < (long long)rows; ++rr) {
      uint64_t r = (uint64_t)rr;
      std::vector<double> inv((size_t)J * J);
      inverse_pplu(J, &B[p][r * J * J], inv.data());
      for (int k = 0; k < J; ++k) {
        V res = 0;
        for (int l = 0; l < J; ++l) res += C[p][r * J + l] * inv[(size_t)l * J + k];
        o.fac[mode][((uint64_t)p * rows + r) * J + k] = res;
      }
    }
  }
}

// reconstruction.cuh:58-81 (x_hat), 259-276 (error, fit)
template <class V> void fit(const Ora<V> &o, double *fit_ref, double *fit64, double *err_ref, double *err64) {
  std::vector<V> xh(o.nnz);
  const int N = o.N, J = o.J;
  for (uint64_t b = 0; b < o.nblk; ++b) {
    long long s = (long long)o.blk_ptr[b], e = (long long)o.blk_ptr[b + 1];
#pragma omp parallel for schedule(static)
    for (long long tt = s; tt < e; ++tt) {
      uint64_t t = (uint64_t)tt;
      uint64_t row[kMaxOrder];
      for (int n = 0; n < N; ++n) row[n] = (uint64_t)o.gidx(n, b, t) * J;
      V res = 0;
      for (uint64_t i = 0; i < o.core_n; ++i) {
        V tmp = o.core[i];
        for (int n = 0; n < N; ++n) tmp *= o.fac[n][row[n] + o.core_idx[n][i]];
        res += tmp;
      }
      xh[t] = res;
    }
  }
  V err = 0;
  double e64 = 0;
  for (uint64_t t = 0; t < o.nnz; ++t) {
    V d = o.val[t] - xh[t];
    err += d * d;
    e64 += (double)d * (double)d;
  }
  if (err_ref) *err_ref = (double)err;
  if (err64) *err64 = e64;
  if (fit_ref) *fit_ref = (o.norm_ref == 0) ? 1.0 : (double)(1.0f - std::sqrt(err) / o.norm_ref);
  if (fit64) *fit64 = (o.norm64 == 0) ? 1.0 : 1.0 - std::sqrt(e64) / o.norm64;
}

struct Handle {
  int dtype;  // 0 float, 1 double
  Ora<float> f;
  Ora<double> d;
};

}  // namespace

extern "C" {

const char *ora_last_error(void) { return g_err.c_str(); }

int ora_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void ora_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// glibc rand() replay: n draws after `skip` draws from srand(seed)
void ora_rand(uint32_t seed, uint64_t skip, uint64_t n, int32_t *out) {
  GlibcRand g(seed);
  for (uint64_t k = 0; k < skip; ++k) g.next();
  for (uint64_t k = 0; k < n; ++k) out[k] = g.next();
}

// Text parser restated serially in file order (tensor_manager.tpp:46-191).
// Pass 1 (idx == NULL): returns nnz and dims.  Pass 2: fills idx[N][nnz] (0-based),
// vals (dtype), and *draws = rand() draws consumed for missing values.
// Returns 0, or 3 on a parse error (index 0: the reference throws; fewer than N
// index tokens: the reference reads uninitialised memory).
int ora_parse(const char *buf, uint64_t len, int N, int dtype, uint32_t seed, uint64_t *nnz_out, uint32_t *dims,
              uint32_t *const *idx, void *vals, uint64_t *draws) {
  GlibcRand g(seed);
  uint64_t line = 0, ndraw = 0;
  for (int n = 0; n < N; ++n) dims[n] = 0;
  uint64_t start = 0;
  std::vector<char> tok;
  for (uint64_t p = 0; p < len; ++p) {
    if (buf[p] != '\n') continue;
    // tokenize [start, p)
    std::string s(buf + start, buf + p);
    start = p + 1;
    const char *delim = " \t";
    char *save = nullptr;
    char *rest = &s[0];
    int n = 0;
    char *t = nullptr;
    uint32_t ci[kMaxOrder];
    while ((t = strtok_r(rest, delim, &save)) && n < N) {
      rest = nullptr;
      unsigned long long v = strtoull(t, nullptr, 10);
      uint32_t iv = (uint32_t)v;
      if (iv < 1) { g_err = "We note that input tensors must follow base-1 indexing"; return 3; }
      ci[n] = iv;
      ++n;
    }
    if (n < N) { g_err = "line with fewer indices than the order"; return 3; }
    double dv = 0;
    float fv = 0;
    if (t != nullptr) {  // std::stod, then narrowed to value_t
      dv = strtod(t, nullptr);
      fv = (float)dv;
    } else {             // frand<value_t>(0, 1): one draw
      if (dtype == 0) fv = frand01<float>(g); else dv = frand01<double>(g);
      ++ndraw;
    }
    for (int m = 0; m < N; ++m) {
      if (ci[m] > dims[m]) dims[m] = ci[m];
      if (idx) idx[m][line] = ci[m] - 1;
    }
    if (vals) {
      if (dtype == 0) ((float *)vals)[line] = fv; else ((double *)vals)[line] = dv;
    }
    ++line;
  }
  *nnz_out = line;
  if (draws) *draws = ndraw;
  return 0;
}

// Build the blocked tensor (partition + segmenting).  idx: [N] pointers to 0-based u32 coords.
void *ora_create(int dtype, int N, uint64_t nnz, const uint32_t *const *idx, const void *vals, const uint32_t *dims,
                 const uint32_t *P, int J, int *status) {
  Handle *h = new Handle();
  h->dtype = dtype;
  int rc = (dtype == 0) ? build(h->f, N, nnz, idx, (const float *)vals, dims, P, J)
                        : build(h->d, N, nnz, idx, (const double *)vals, dims, P, J);
  *status = rc;
  if (rc) { delete h; return nullptr; }
  return h;
}

void ora_destroy(void *hp) { delete (Handle *)hp; }

#define ORA_DISPATCH(h, expr)           \
  do {                                  \
    if ((h)->dtype == 0) { auto &o = (h)->f; expr; } \
    else { auto &o = (h)->d; expr; }    \
  } while (0)

// info: block_dims[N], P-derived counts; norms
void ora_info(void *hp, uint32_t *bd, uint64_t *nblk, double *norm_ref, double *norm64) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, {
    for (int n = 0; n < o.N; ++n) bd[n] = o.bd[n];
    *nblk = o.nblk;
    *norm_ref = (double)o.norm_ref;
    *norm64 = o.norm64;
  });
}

// partition readback: blk_ptr[nblk+1], blk_coord[nblk*N], idx[N][nnz], vals, count[N][nblk*(bd+1)], where[N][nnz]
void ora_partition(void *hp, uint64_t *blk_ptr, uint32_t *blk_coord, uint32_t *const *idx, void *vals,
                   uint64_t *const *count, uint32_t *const *where) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, {
    std::copy(o.blk_ptr.begin(), o.blk_ptr.end(), blk_ptr);
    std::copy(o.blk_coord.begin(), o.blk_coord.end(), blk_coord);
    for (int n = 0; n < o.N; ++n) {
      std::copy(o.idx[n].begin(), o.idx[n].end(), idx[n]);
      std::copy(o.count_nnz[n].begin(), o.count_nnz[n].end(), count[n]);
      std::copy(o.where_nnz[n].begin(), o.where_nnz[n].end(), where[n]);
    }
    std::copy(o.val.begin(), o.val.end(), (decltype(o.val.data()))vals);
  });
}

void ora_init_random(void *hp, uint32_t seed, uint64_t skip) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, init_random(o, seed, skip));
}

// factor in slab layout [P*bd][J]; core [J^N]
void ora_get_factor(void *hp, int n, void *out) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, std::copy(o.fac[n].begin(), o.fac[n].end(), (decltype(o.fac[n].data()))out));
}
void ora_set_factor(void *hp, int n, const void *in) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, {
    auto p = (decltype(o.fac[n].data()))in;
    std::copy(p, p + o.fac[n].size(), o.fac[n].begin());
  });
}
void ora_get_core(void *hp, void *out) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, std::copy(o.core.begin(), o.core.end(), (decltype(o.core.data()))out));
}
void ora_set_core(void *hp, const void *in) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, {
    auto p = (decltype(o.core.data()))in;
    std::copy(p, p + o.core.size(), o.core.begin());
  });
}

// delta for every nonzero, block-major order [nnz][J] (the reference's per-block delta buffers concatenated)
void ora_delta(void *hp, int mode, void *out) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, compute_delta(o, mode, (decltype(o.val.data()))out));
}

void ora_update_mode(void *hp, int mode) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, update_mode(o, mode));
}

// one sweep = UpdateFactorMatrices (modes 0..N-1) then Reconstruction
void ora_sweep(void *hp, double *fit_ref, double *fit64) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, {
    for (int n = 0; n < o.N; ++n) update_mode(o, n);
    fit(o, fit_ref, fit64, nullptr, nullptr);
  });
}

void ora_fit(void *hp, double *fit_ref, double *fit64, double *err_ref, double *err64) {
  Handle *h = (Handle *)hp;
  ORA_DISPATCH(h, fit(o, fit_ref, fit64, err_ref, err64));
}

}  // extern "C"
