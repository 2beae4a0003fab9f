// gen.cpp -- seeded synthetic sparse tensors and the reference's text writer.
//
// Coordinates: each mode's index is uniform, or Zipf(s) over ranks 1..I mapped
// through a seeded random permutation of the axis (power-law slice sizes).
// Coordinates are distinct: candidates are drawn in a fixed order (chunks of
// 2^20 samples, each chunk with its own seeded stream, so the result does not
// depend on the thread count), duplicates keep their first occurrence, and the
// first `nnz` distinct candidates in draw order are the tensor.
// Values: uniform [0,1), lognormal(0,1) divided by the largest drawn value, or
// a planted Tucker model (core and nonnegative factors uniform [0,1) from the
// seed) plus Gaussian noise.
// Writer: the reference's text format -- 1-based indices and the value,
// tab-separated, '\n' after every line (tensor_manager.tpp:88-155).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace gtk {
namespace {

constexpr uint64_t kChunk = 1ull << 20;

inline uint64_t splitmix(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Xoshiro {  // xoshiro256**
  uint64_t s[4];
  explicit Xoshiro(uint64_t seed) {
    for (auto &v : s) v = splitmix(seed);
  }
  static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  inline uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  inline float uniformf() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
  inline double normal() {
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

// threads for `tasks` independent work items (chunks or buckets)
unsigned threads_for(uint64_t tasks) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  nt = std::min<unsigned>(nt, 64);
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(nt, tasks));
}

template <class F> void parallel_for(uint64_t n, F f) {
  unsigned nt = threads_for(n);
  std::atomic<uint64_t> next{0};
  auto body = [&]() {
    for (;;) {
      uint64_t c = next.fetch_add(1);
      if (c >= n) break;
      f(c);
    }
  };
  std::vector<std::thread> th;
  for (unsigned i = 1; i < nt; ++i) th.emplace_back(body);
  body();
  for (auto &t : th) t.join();
}

struct Axis {
  std::vector<double> cdf;      // Zipf CDF over ranks, empty for uniform
  std::vector<uint32_t> perm;   // rank -> index
  uint32_t dim;
  inline uint32_t draw(Xoshiro &r) const {
    if (cdf.empty()) return (uint32_t)(((unsigned __int128)r.next() * dim) >> 64);
    double u = r.uniform();
    size_t k = (size_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
    if (k >= cdf.size()) k = cdf.size() - 1;
    return perm[k];
  }
};

inline uint64_t tuple_hash(const uint32_t *const *idx, int N, uint64_t t) {
  uint64_t h = 0x243F6A8885A308D3ull;
  for (int n = 0; n < N; ++n) {
    h ^= idx[n][t] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xFF51AFD7ED558CCDull;
  }
  return h ^ (h >> 33);
}

}  // namespace

int generate(int N, const uint32_t *dims, uint64_t nnz, int index_dist, double zipf_s, int value_dist, int dtype,
             uint64_t seed, const double *noise_sigma, int planted_rank, gtk_coo *out) {
  if (N < 1 || N > kMaxOrder) return fail(GTK_ERR_ARG, "order must be 1..8");
  double space = 1;
  for (int n = 0; n < N; ++n) {
    if (dims[n] == 0) return fail(GTK_ERR_ARG, "zero dimension");
    space *= dims[n];
  }
  if ((double)nnz > 0.5 * space) return fail(GTK_ERR_ARG, "nnz must be at most half the coordinate space");
  if (nnz >= 0xFFFFFFFFull) return fail(GTK_ERR_UNSUPPORTED, "too many nonzeros");
  uint64_t sseed = seed * 0x9E3779B97F4A7C15ull + 12345;
  std::vector<Axis> axes(N);
  for (int n = 0; n < N; ++n) {
    Axis &a = axes[n];
    a.dim = dims[n];
    if (index_dist == GTK_GEN_ZIPF) {
      a.cdf.resize(dims[n]);
      double s = 0;
      for (uint32_t r = 0; r < dims[n]; ++r) {
        s += std::pow((double)(r + 1), -zipf_s);
        a.cdf[r] = s;
      }
      for (auto &c : a.cdf) c /= s;
      a.perm.resize(dims[n]);
      for (uint32_t r = 0; r < dims[n]; ++r) a.perm[r] = r;
      Xoshiro pr(splitmix(sseed) ^ (uint64_t)n);
      for (uint32_t r = dims[n] - 1; r > 0; --r) {
        uint32_t j = (uint32_t)(((unsigned __int128)pr.next() * (r + 1)) >> 64);
        std::swap(a.perm[r], a.perm[j]);
      }
    } else if (index_dist != GTK_GEN_UNIFORM) {
      return fail(GTK_ERR_ARG, "unknown index distribution");
    }
  }
  const uint64_t cseed = splitmix(sseed);
  // candidates, grown until enough distinct ones exist
  uint64_t M = nnz + nnz / 4 + 1024;
  std::vector<std::vector<uint32_t>> cand(N);
  std::vector<unsigned char> keep;
  uint64_t have_chunks = 0, distinct = 0;
  for (int attempt = 0; attempt < 12; ++attempt) {
    const uint64_t chunks = (M + kChunk - 1) / kChunk;
    const uint64_t total = chunks * kChunk;
    for (int n = 0; n < N; ++n) cand[n].resize(total);
    parallel_for(chunks - have_chunks, [&](uint64_t c0) {
      const uint64_t c = have_chunks + c0;
      Xoshiro r(cseed ^ (c * 0xD1B54A32D192ED03ull));
      for (uint64_t k = 0; k < kChunk; ++k)
        for (int n = 0; n < N; ++n) cand[n][c * kChunk + k] = axes[n].draw(r);
    });
    have_chunks = chunks;
    // dedup: bucket by hash, sort each bucket by (tuple, draw index), keep the first
    const uint32_t B = 4096;
    std::vector<const uint32_t *> ip(N);
    for (int n = 0; n < N; ++n) ip[n] = cand[n].data();
    std::vector<uint32_t> bucket_of(total);
    const uint64_t nchunk = (total + kChunk - 1) / kChunk;
    std::vector<uint64_t> hist(nchunk * B, 0);  // [chunk][bucket]
    parallel_for(nchunk, [&](uint64_t c) {
      uint64_t *h = &hist[c * B];
      const uint64_t e = std::min(total, (c + 1) * kChunk);
      for (uint64_t t = c * kChunk; t < e; ++t) {
        const uint32_t b = (uint32_t)(tuple_hash(ip.data(), N, t) % B);
        bucket_of[t] = b;
        ++h[b];
      }
    });
    // slot of (bucket, chunk): buckets in order, chunks in order inside a bucket
    std::vector<uint64_t> start(B + 1, 0), base(nchunk * B);
    {
      uint64_t pos = 0;
      for (uint32_t b = 0; b < B; ++b) {
        start[b] = pos;
        for (uint64_t c = 0; c < nchunk; ++c) {
          base[c * B + b] = pos;
          pos += hist[c * B + b];
        }
      }
      start[B] = pos;
    }
    std::vector<uint32_t> order(total);
    parallel_for(nchunk, [&](uint64_t c) {
      uint64_t *bp = &base[c * B];
      const uint64_t e = std::min(total, (c + 1) * kChunk);
      for (uint64_t t = c * kChunk; t < e; ++t) order[bp[bucket_of[t]]++] = (uint32_t)t;
    });
    keep.assign(total, 0);
    parallel_for(B, [&](uint64_t b) {
      uint32_t *s = order.data() + start[b], *e = order.data() + start[b + 1];
      std::sort(s, e, [&](uint32_t x, uint32_t y) {
        for (int n = 0; n < N; ++n)
          if (ip[n][x] != ip[n][y]) return ip[n][x] < ip[n][y];
        return x < y;
      });
      for (uint32_t *p = s; p < e; ++p) {
        bool first = (p == s);
        if (!first) {
          for (int n = 0; n < N; ++n)
            if (ip[n][*p] != ip[n][*(p - 1)]) {
              first = true;
              break;
            }
        }
        if (first) keep[*p] = 1;
      }
    });
    distinct = 0;
    {
      std::vector<uint64_t> part(nchunk, 0);
      parallel_for(nchunk, [&](uint64_t c) {
        const uint64_t e = std::min(total, (c + 1) * kChunk);
        uint64_t k = 0;
        for (uint64_t t = c * kChunk; t < e; ++t) k += keep[t];
        part[c] = k;
      });
      for (uint64_t k : part) distinct += k;
    }
    if (distinct >= nnz) break;
    M = total + (total - distinct) * 2 + (nnz - distinct) * 2;
  }
  if (distinct < nnz) return fail(GTK_ERR_ARG, "could not draw enough distinct coordinates");
  out->N = N;
  out->dtype = dtype;
  out->nnz = nnz;
  for (int n = 0; n < N; ++n) out->idx[n].resize(nnz);
  {
    // the first nnz kept candidates, in draw order; chunk offsets make it parallel
    const uint64_t total = keep.size(), nchunk = (total + kChunk - 1) / kChunk;
    std::vector<uint64_t> off(nchunk + 1, 0);
    parallel_for(nchunk, [&](uint64_t c) {
      uint64_t k = 0;
      const uint64_t e = std::min(total, (c + 1) * kChunk);
      for (uint64_t t = c * kChunk; t < e; ++t) k += keep[t];
      off[c + 1] = k;
    });
    for (uint64_t c = 0; c < nchunk; ++c) off[c + 1] += off[c];
    parallel_for(nchunk, [&](uint64_t c) {
      uint64_t k = off[c];
      const uint64_t e = std::min(total, (c + 1) * kChunk);
      for (uint64_t t = c * kChunk; t < e && k < nnz; ++t) {
        if (!keep[t]) continue;
        for (int n = 0; n < N; ++n) out->idx[n][k] = cand[n][t];
        ++k;
      }
    });
  }
  cand.clear();
  for (int n = 0; n < N; ++n) {
    const uint64_t nchunk = (nnz + kChunk - 1) / kChunk;
    std::vector<uint32_t> mx(nchunk + 1, 0);
    parallel_for(nchunk, [&](uint64_t c) {
      const uint64_t e = std::min(nnz, (c + 1) * kChunk);
      uint32_t m = 0;
      for (uint64_t k = c * kChunk; k < e; ++k) m = std::max(m, out->idx[n][k]);
      mx[c] = m;
    });
    uint32_t m = 0;
    for (uint32_t x : mx) m = std::max(m, x);
    out->dims[n] = nnz ? m + 1 : 0;
  }
  // values
  const uint64_t vseed = splitmix(sseed);
  HostVec<double> v(nnz);
  if (value_dist == GTK_VAL_PLANTED) {
    const int R = planted_rank;
    if (R < 1 || R > GTK_MAX_RANK) return fail(GTK_ERR_ARG, "planted rank must be 1..64");
    Xoshiro pr(vseed ^ 0x5151);
    std::vector<std::vector<double>> F(N);
    for (int n = 0; n < N; ++n) {
      F[n].resize((size_t)dims[n] * R);
      for (auto &x : F[n]) x = pr.uniform();
    }
    uint64_t cn = 1;
    for (int n = 0; n < N; ++n) cn *= (uint64_t)R;
    std::vector<double> G(cn);
    for (auto &x : G) x = pr.uniform();
    const double sigma = noise_sigma ? *noise_sigma : 0.0;
    parallel_for((nnz + kChunk - 1) / kChunk, [&](uint64_t c) {
      Xoshiro r(vseed ^ (c * 0xA24BAED4963EE407ull));
      const uint64_t e = std::min(nnz, (c + 1) * kChunk);
      for (uint64_t t = c * kChunk; t < e; ++t) {
        double s = 0;
        for (uint64_t i = 0; i < cn; ++i) {
          uint64_t rem = i;
          double p = G[i];
          for (int n = N - 1; n >= 0; --n) {
            p *= F[n][(size_t)out->idx[n][t] * R + rem % R];
            rem /= R;
          }
          s += p;
        }
        v[t] = s + sigma * r.normal();
      }
    });
  } else {
    parallel_for((nnz + kChunk - 1) / kChunk, [&](uint64_t c) {
      Xoshiro r(vseed ^ (c * 0xA24BAED4963EE407ull));
      const uint64_t e = std::min(nnz, (c + 1) * kChunk);
      for (uint64_t t = c * kChunk; t < e; ++t) {
        if (value_dist == GTK_VAL_LOGNORMAL)
          v[t] = std::exp(r.normal());
        else
          v[t] = dtype == GTK_F32 ? (double)r.uniformf() : r.uniform();
      }
    });
    if (value_dist == GTK_VAL_LOGNORMAL) {
      double mx = 0;
      for (double x : v) mx = std::max(mx, x);
      if (mx > 0)
        for (double &x : v) x /= mx;
    } else if (value_dist != GTK_VAL_UNIFORM) {
      return fail(GTK_ERR_ARG, "unknown value distribution");
    }
  }
  if (dtype == GTK_F32) {
    out->vf.resize(nnz);
    parallel_for((nnz + kChunk - 1) / kChunk, [&](uint64_t c) {
      const uint64_t e = std::min(nnz, (c + 1) * kChunk);
      for (uint64_t t = c * kChunk; t < e; ++t) out->vf[t] = (float)v[t];
    });
  } else {
    out->vd = std::move(v);
  }
  out->draws = 0;
  return 0;
}

int write_text(const gtk_coo &c, const char *path) {
  FILE *f = fopen(path, "wb");
  if (!f) return fail(GTK_ERR_IO, std::string("cannot open \"") + path + "\" for writing");
  const uint64_t per = 1 << 16;
  const uint64_t chunks = (c.nnz + per - 1) / per;
  std::vector<std::string> bufs(chunks);
  parallel_for(chunks, [&](uint64_t k) {
    std::string &s = bufs[k];
    char line[512];
    const uint64_t e = std::min(c.nnz, (k + 1) * per);
    for (uint64_t t = k * per; t < e; ++t) {
      int o = 0;
      for (int n = 0; n < c.N; ++n) o += snprintf(line + o, sizeof line - o, "%u\t", c.idx[n][t] + 1);
      if (c.dtype == GTK_F32)
        o += snprintf(line + o, sizeof line - o, "%.9g\n", (double)c.vf[t]);
      else
        o += snprintf(line + o, sizeof line - o, "%.17g\n", c.vd[t]);
      s.append(line, (size_t)o);
    }
  });
  for (auto &s : bufs)
    if (fwrite(s.data(), 1, s.size(), f) != s.size()) {
      fclose(f);
      return fail(GTK_ERR_IO, "short write");
    }
  if (fclose(f) != 0) return fail(GTK_ERR_IO, "close failed");
  return 0;
}

}  // namespace gtk

extern "C" {

int gtk_generate(int order, const uint32_t *dims, uint64_t nnz, int index_dist, double zipf_s, int value_dist,
                 int dtype, uint64_t seed, gtk_coo **out) {
  if (!dims || !out) return gtk::fail(GTK_ERR_ARG, "null argument");
  if (dtype != GTK_F32 && dtype != GTK_F64) return gtk::fail(GTK_ERR_ARG, "bad dtype");
  try {
    gtk_coo *c = new gtk_coo();
    int rc = gtk::generate(order, dims, nnz, index_dist, zipf_s, value_dist, dtype, seed, nullptr, 0, c);
    if (rc) {
      delete c;
      return rc;
    }
    *out = c;
    return 0;
  } catch (std::bad_alloc &) {
    return gtk::fail(GTK_ERR_OOM, "host allocation failed");
  }
}

int gtk_generate_planted(int order, const uint32_t *dims, uint64_t nnz, int planted_rank, double noise_sigma,
                         int dtype, uint64_t seed, gtk_coo **out) {
  if (!dims || !out) return gtk::fail(GTK_ERR_ARG, "null argument");
  if (dtype != GTK_F32 && dtype != GTK_F64) return gtk::fail(GTK_ERR_ARG, "bad dtype");
  try {
    gtk_coo *c = new gtk_coo();
    int rc = gtk::generate(order, dims, nnz, GTK_GEN_UNIFORM, 0.0, GTK_VAL_PLANTED, dtype, seed, &noise_sigma,
                           planted_rank, c);
    if (rc) {
      delete c;
      return rc;
    }
    *out = c;
    return 0;
  } catch (std::bad_alloc &) {
    return gtk::fail(GTK_ERR_OOM, "host allocation failed");
  }
}

int gtk_write_text(const gtk_coo *coo, const char *path) {
  if (!coo || !path) return gtk::fail(GTK_ERR_ARG, "null argument");
  try {
    return gtk::write_text(*coo, path);
  } catch (std::bad_alloc &) {
    return gtk::fail(GTK_ERR_OOM, "host allocation failed");
  }
}

}  // extern "C"
