// hostpart.cpp -- the blocked layout and the mode views built in host memory, for
// the streamed layout (tensors whose resident layout exceeds the device memory
// the handle may use).  The arrays have the definitions and layouts that
// partition.cu gives the device arrays, so readback and parity are the same:
//   * block id of a nonzero: sum_n (i_n / bd_n) * prod_{m>n} P_m (the last mode
//     fastest, tensor_manager.tpp:229-246); block-major order keeps input order
//     inside a block (the reference's stable insert, :267-290); block-local
//     coordinates i_n - (i_n / bd_n) * bd_n;
//   * count_nnz / where_nnz of every block and mode (block.tpp:115-186): a
//     counting sort of the block's positions by local row, stable;
//   * mode view m: the block-major order stably sorted by global row i_m.
// All sorts are stable LSD radix sorts over every host thread.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "internal.h"

namespace gtk {

unsigned host_threads(uint64_t work) {
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min<unsigned>(nt, 64));
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(nt, work / (1 << 16) + 1));
}

// glibc's random() (TYPE_3, the generator behind the reference's rand()) is the
// linear recurrence r[n] = r[n-3] + r[n-31] mod 2^32 from its 34th value on, with
// characteristic polynomial p(x) = x^31 - x^28 - 1.  For any such sequence
// r[m + k] = sum_j a_j r[m + j] where x^k mod p(x) = sum_j a_j x^j (p is monic,
// so the reduction is exact over the integers mod 2^32).  The 31 values after a
// jump of k are therefore dot products of x^(k+j) mod p, j = 0..30, with the
// current 31-value window: bit-exact, O(31^2 log k) work.
namespace {
struct Poly31 {
  uint32_t c[31];
};
Poly31 poly_mul(const Poly31 &a, const Poly31 &b) {
  uint32_t t[61] = {};
  for (int i = 0; i < 31; ++i)
    for (int j = 0; j < 31; ++j) t[i + j] += a.c[i] * b.c[j];
  for (int d = 60; d >= 31; --d) {  // x^d = x^(d-3) + x^(d-31) mod p
    t[d - 3] += t[d];
    t[d - 31] += t[d];
  }
  Poly31 r;
  for (int i = 0; i < 31; ++i) r.c[i] = t[i];
  return r;
}
Poly31 poly_shift(const Poly31 &a) {  // x * a mod p
  Poly31 r;
  const uint32_t top = a.c[30];
  r.c[0] = top;  // x^31 = x^28 + 1
  for (int i = 1; i < 31; ++i) r.c[i] = a.c[i - 1];
  r.c[28] += top;
  return r;
}
Poly31 poly_xpow(uint64_t k) {
  Poly31 r = {}, b = {};
  r.c[0] = 1;
  b.c[1] = 1;
  for (; k; k >>= 1) {
    if (k & 1) r = poly_mul(r, b);
    b = poly_mul(b, b);
  }
  return r;
}
}  // namespace

void GlibcRand::jump(uint64_t k) {
  if (k < 512) {
    for (uint64_t s = 0; s < k; ++s) step();
    return;
  }
  uint32_t w[31];  // r[i - 31 + j]
  for (int j = 0; j < 31; ++j) w[j] = ring[(i + j) % 31];
  Poly31 a = poly_xpow(k);
  uint32_t nw[31];
  for (int j = 0; j < 31; ++j) {
    uint32_t v = 0;
    for (int m = 0; m < 31; ++m) v += a.c[m] * w[m];
    nw[j] = v;
    a = poly_shift(a);
  }
  i += k;
  for (int j = 0; j < 31; ++j) ring[(i + j) % 31] = nw[j];
}

void glibc_step_polys(uint64_t step, int count, uint32_t *out) {
  Poly31 a = {};
  a.c[0] = 1;  // x^0
  const Poly31 s = poly_xpow(step);
  for (int j = 0; j < count; ++j) {
    for (int m = 0; m < 31; ++m) out[31 * j + m] = a.c[m];
    a = poly_mul(a, s);
  }
}

void glibc_chunk_states(const GlibcRand &g, uint64_t len, int chunks, uint32_t *out) {
  uint32_t w[31];  // r[s - 31 + j], s the current chunk start
  for (int j = 0; j < 31; ++j) w[j] = g.ring[(g.i + j) % 31];
  if (chunks <= 0) return;
  Poly31 a0 = poly_xpow(len);
  for (int c = 0; c < chunks; ++c) {
    for (int j = 0; j < 31; ++j) out[31 * c + j] = w[j];
    if (c + 1 == chunks) break;
    Poly31 a = a0;
    uint32_t nw[31];
    for (int j = 0; j < 31; ++j) {
      uint32_t v = 0;
      for (int m = 0; m < 31; ++m) v += a.c[m] * w[m];
      nw[j] = v;
      a = poly_shift(a);
    }
    for (int j = 0; j < 31; ++j) w[j] = nw[j];
  }
}

namespace {

template <class F> void par(unsigned nt, F f) {
  std::vector<std::thread> th;
  for (unsigned c = 1; c < nt; ++c) th.emplace_back(f, c);
  f(0u);
  for (auto &x : th) x.join();
}

inline void range_of(uint64_t n, unsigned nt, unsigned c, uint64_t &lo, uint64_t &hi) {
  lo = n / nt * c;
  hi = c + 1 == nt ? n : n / nt * (c + 1);
}

int bits_for(uint64_t maxkey) {
  int b = 0;
  while (b < 64 && (maxkey >> b)) ++b;
  return b;
}

// stable LSD radix sort of (key, val) by the low `bits` bits of key, 11-bit digits
void radix_sort_host(HostVec<uint64_t> &key, HostVec<uint32_t> &val, int bits) {
  const uint64_t n = key.size();
  if (n < 2 || bits == 0) return;
  constexpr int D = 11;
  constexpr uint32_t R = 1u << D;
  HostVec<uint64_t> k2(n);
  HostVec<uint32_t> v2(n);
  const unsigned nt = host_threads(n);
  std::vector<uint64_t> hist((size_t)nt * R);
  for (int shift = 0; shift < bits; shift += D) {
    par(nt, [&](unsigned c) {
      uint64_t lo, hi;
      range_of(n, nt, c, lo, hi);
      uint64_t *h = hist.data() + (size_t)c * R;
      std::fill(h, h + R, 0);
      for (uint64_t i = lo; i < hi; ++i) ++h[(key[i] >> shift) & (R - 1)];
    });
    uint64_t s = 0;
    for (uint32_t d = 0; d < R; ++d)
      for (unsigned c = 0; c < nt; ++c) {
        const uint64_t x = hist[(size_t)c * R + d];
        hist[(size_t)c * R + d] = s;
        s += x;
      }
    par(nt, [&](unsigned c) {
      uint64_t lo, hi;
      range_of(n, nt, c, lo, hi);
      uint64_t *h = hist.data() + (size_t)c * R;
      for (uint64_t i = lo; i < hi; ++i) {
        const uint64_t p = h[(key[i] >> shift) & (R - 1)]++;
        k2[p] = key[i];
        v2[p] = val[i];
      }
    });
    key.swap(k2);
    val.swap(v2);
  }
}

}  // namespace

int build_host_partition(DevTensor &t, const gtk_coo &coo) {
  NvtxRange nvtx("host partition");
  const uint64_t n = t.nnz;
  const int N = t.N;
  const size_t vs = t.vsize;
  t.hp.reset(new HostPart());
  HostPart &h = *t.hp;
  const unsigned nt = host_threads(n);
  uint64_t stride[kMaxOrder];
  {
    uint64_t s = 1;
    for (int k = N - 1; k >= 0; --k) {
      stride[k] = s;
      s *= t.P[k];
    }
  }
  // block ids, then the stable sort into blocks
  HostVec<uint64_t> key(n);
  HostVec<uint32_t> perm(n);
  par(nt, [&](unsigned c) {
    uint64_t lo, hi;
    range_of(n, nt, c, lo, hi);
    for (uint64_t i = lo; i < hi; ++i) {
      uint64_t b = 0;
      for (int k = 0; k < N; ++k) b += (uint64_t)(coo.idx[k][i] / t.bd[k]) * stride[k];
      key[i] = b;
      perm[i] = (uint32_t)i;
    }
  });
  radix_sort_host(key, perm, bits_for(t.nblk - 1));
  h.blk_ptr.assign(t.nblk + 1, 0);
  for (uint64_t j = 0; j < n; ++j) ++h.blk_ptr[key[j] + 1];
  for (uint64_t b = 0; b < t.nblk; ++b) h.blk_ptr[b + 1] += h.blk_ptr[b];
  // block-major arrays: local coordinates, values, and (temporarily) global coordinates
  HostVec<uint32_t> gblk[kMaxOrder];
  for (int k = 0; k < N; ++k) {
    gblk[k].resize(n);
    h.blk_idx[k].resize(n);
  }
  h.blk_val.resize(n * vs);
  const unsigned char *vin = static_cast<const unsigned char *>(coo.values());
  par(nt, [&](unsigned c) {
    uint64_t lo, hi;
    range_of(n, nt, c, lo, hi);
    for (uint64_t j = lo; j < hi; ++j) {
      const uint32_t p = perm[j];
      for (int k = 0; k < N; ++k) {
        const uint32_t g = coo.idx[k][p];
        gblk[k][j] = g;
        h.blk_idx[k][j] = g - (g / t.bd[k]) * t.bd[k];
      }
      memcpy(h.blk_val.data() + j * vs, vin + (size_t)p * vs, vs);
    }
  });
  // ||X|| in FP64: per-thread partial sums over fixed ranges, added in thread order
  {
    std::vector<double> part(nt, 0.0);
    par(nt, [&](unsigned c) {
      uint64_t lo, hi;
      range_of(n, nt, c, lo, hi);
      double s = 0;
      for (uint64_t j = lo; j < hi; ++j) {
        const double v = t.dtype == GTK_F32 ? (double)reinterpret_cast<const float *>(h.blk_val.data())[j]
                                            : reinterpret_cast<const double *>(h.blk_val.data())[j];
        s += v * v;
      }
      part[c] = s;
    });
    double ss = 0;
    for (double x : part) ss += x;
    t.norm = std::sqrt(ss);
  }
  for (int m = 0; m < N; ++m) {
    // count_nnz and where_nnz: a counting sort of each block's positions by local row
    const uint64_t rows = (uint64_t)t.bd[m] + 1;
    h.count[m].assign(t.nblk * rows, 0);
    h.where[m].resize(n);
    const unsigned ntb = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(nt, t.nblk));
    par(ntb, [&](unsigned c) {
      for (uint64_t b = c; b < t.nblk; b += ntb) {
        uint64_t *cnt = h.count[m].data() + b * rows;
        const uint64_t s = h.blk_ptr[b], e = h.blk_ptr[b + 1];
        for (uint64_t j = s; j < e; ++j) ++cnt[h.blk_idx[m][j] + 1];
        for (uint64_t r = 0; r + 1 < rows; ++r) cnt[r + 1] += cnt[r];
        std::vector<uint64_t> next(cnt, cnt + rows - 1);
        for (uint64_t j = s; j < e; ++j) h.where[m][s + next[h.blk_idx[m][j]]++] = (uint32_t)(j - s);
      }
    });
    // the mode view: block-major positions stably sorted by global row
    par(nt, [&](unsigned c) {
      uint64_t lo, hi;
      range_of(n, nt, c, lo, hi);
      for (uint64_t j = lo; j < hi; ++j) {
        key[j] = gblk[m][j];
        perm[j] = (uint32_t)j;
      }
    });
    radix_sort_host(key, perm, bits_for(t.dims[m] ? t.dims[m] - 1 : 0));
    for (int k = 0; k < N; ++k) h.vidx[m][k].resize(n);
    h.vval[m].resize(n * vs);
    par(nt, [&](unsigned c) {
      uint64_t lo, hi;
      range_of(n, nt, c, lo, hi);
      for (uint64_t j = lo; j < hi; ++j) {
        const uint32_t p = perm[j];
        for (int k = 0; k < N; ++k) h.vidx[m][k][j] = gblk[k][p];
        memcpy(h.vval[m].data() + j * vs, h.blk_val.data() + (size_t)p * vs, vs);
      }
    });
  }
  t.h_blk_ptr.assign(h.blk_ptr.begin(), h.blk_ptr.end());
  return 0;
}

}  // namespace gtk
