// parse.cpp -- the reference's tensor text format, parsed with all host threads.
//
// Semantics of _ReadData (tensor_manager.tpp:46-191):
//   * one nonzero per '\n'; bytes after the last '\n' are ignored (the reference
//     counts newlines, :88-94);
//   * tokens are maximal runs of characters other than ' ' and '\t' (strtok_r
//     with " \t", :134); the first N tokens are indices read with strtoull and
//     narrowed to uint32 (:135), stored minus one (:143); an index that is 0
//     after narrowing is an error (:166-169);
//   * the next token is the value, std::stod narrowed to value_t (:150-151); a
//     line without one gets frand<value_t>(0,1) (:152-155) -- drawn here in file
//     order (the reference draws in OpenMP thread order, which equals file order
//     with one thread);
//   * dims[n] = the largest index seen (:164-176).
// Where the reference is undefined this parser reports GTK_ERR_PARSE instead: a
// line with fewer than N index tokens (the reference reads uninitialised
// memory; this includes empty lines, which the reference merges with the next
// line) and a value token strtod cannot read (std::stod throws).

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace gtk {
namespace {

inline bool is_delim(char c) { return c == ' ' || c == '\t'; }

// strtoull(token, NULL, 10) narrowed to uint32; fast path for plain digit runs
inline uint32_t parse_index(const char *s, const char *e) {
  size_t n = (size_t)(e - s);
  if (n > 0 && n <= 19) {
    uint64_t v = 0;
    bool ok = true;
    for (const char *p = s; p < e; ++p) {
      unsigned d = (unsigned)(*p - '0');
      if (d > 9) {
        ok = false;
        break;
      }
      v = v * 10 + d;
    }
    if (ok) return (uint32_t)v;
  }
  std::string tok(s, e);
  return (uint32_t)strtoull(tok.c_str(), nullptr, 10);
}

// 10^0 .. 10^22: every one exactly representable in double
constexpr double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                               1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// The value token as strtod reads it, for the common decimal forms
// [+-]digits[.digits][(e|E)[+-]digits] spanning the whole token.  Clinger's fast
// path (W. D. Clinger, "How to read floating point numbers accurately", PLDI
// 1990): with the significant digits m < 2^53 and the decimal exponent
// |q| <= 22, m and 10^|q| are exact doubles, so one IEEE multiply or divide
// gives the correctly rounded value -- the double strtod returns.  Anything else
// (more digits, larger exponents, hex, inf/nan, trailing characters) returns
// false and goes to strtod.
inline bool parse_value_fast(const char *s, const char *e, double &out) {
  const char *p = s;
  bool neg = false;
  if (p < e && (*p == '+' || *p == '-')) {
    neg = *p == '-';
    ++p;
  }
  uint64_t m = 0;
  int sig = 0, q = 0;
  bool digits = false;
  for (; p < e && (unsigned)(*p - '0') <= 9u; ++p) {
    digits = true;
    if (m || *p != '0') {
      if (++sig > 19) return false;
      m = m * 10 + (unsigned)(*p - '0');
    }
  }
  if (p < e && *p == '.') {
    for (++p; p < e && (unsigned)(*p - '0') <= 9u; ++p) {
      digits = true;
      --q;
      if (m || *p != '0') {
        if (++sig > 19) return false;
        m = m * 10 + (unsigned)(*p - '0');
      }
    }
  }
  if (!digits) return false;
  if (p < e && (*p == 'e' || *p == 'E')) {
    ++p;
    bool eneg = false;
    if (p < e && (*p == '+' || *p == '-')) {
      eneg = *p == '-';
      ++p;
    }
    if (p >= e) return false;
    int x = 0;
    for (; p < e && (unsigned)(*p - '0') <= 9u; ++p) {
      if (x > 10000) return false;
      x = x * 10 + (*p - '0');
    }
    q += eneg ? -x : x;
  }
  if (p != e) return false;
  if (m == 0) {
    out = neg ? -0.0 : 0.0;
    return true;
  }
  if (m > (1ull << 53) || q < -22 || q > 22) return false;
  const double v = q < 0 ? (double)m / kPow10[-q] : (double)m * kPow10[q];
  out = neg ? -v : v;
  return true;
}

struct Chunk {
  size_t begin = 0, end = 0;  // byte range, whole lines
  uint64_t lines = 0, first_line = 0;
  uint32_t maxd[kMaxOrder] = {};
  uint64_t err_line = UINT64_MAX;
  int err_code = 0;
  std::string err_msg;
  std::vector<uint64_t> missing;  // lines without a value, in file order
};

}  // namespace

int parse_buffer(const char *buf, size_t len, int N, int dtype, uint32_t seed, gtk_coo *out) {
  if (N < 1 || N > kMaxOrder) return fail(GTK_ERR_ARG, "order must be 1..8");
  if (dtype != GTK_F32 && dtype != GTK_F64) return fail(GTK_ERR_ARG, "dtype must be GTK_F32 or GTK_F64");
  // ignore bytes after the last newline
  size_t eff = 0;
  for (size_t p = len; p > 0; --p)
    if (buf[p - 1] == '\n') {
      eff = p;
      break;
    }
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  nt = std::min<unsigned>(nt, 64);
  nt = (unsigned)std::min<size_t>(nt, eff / (1 << 20) + 1);
  std::vector<Chunk> ch(nt);
  // chunk boundaries at line starts
  size_t prev = 0;
  for (unsigned c = 0; c < nt; ++c) {
    size_t target = (c + 1 == nt) ? eff : (eff / nt) * (c + 1);
    if (target < prev) target = prev;
    while (target < eff && target > 0 && buf[target - 1] != '\n') ++target;
    ch[c].begin = prev;
    ch[c].end = target;
    prev = target;
  }
  auto count = [&](unsigned c) {
    uint64_t n = 0;
    const char *p = buf + ch[c].begin, *e = buf + ch[c].end;
    while (p < e) {
      const void *q = memchr(p, '\n', (size_t)(e - p));
      if (!q) break;
      ++n;
      p = (const char *)q + 1;
    }
    ch[c].lines = n;
  };
  {
    std::vector<std::thread> th;
    for (unsigned c = 1; c < nt; ++c) th.emplace_back(count, c);
    count(0);
    for (auto &x : th) x.join();
  }
  uint64_t nnz = 0;
  for (auto &c : ch) {
    c.first_line = nnz;
    nnz += c.lines;
  }
  out->N = N;
  out->dtype = dtype;
  out->nnz = nnz;
  // uninitialised: every entry is written below by the thread that parses its line
  for (int n = 0; n < N; ++n) out->idx[n].resize(nnz);
  if (dtype == GTK_F32)
    out->vf.resize(nnz);
  else
    out->vd.resize(nnz);

  auto work = [&](unsigned c) {
    Chunk &k = ch[c];
    const char *p = buf + k.begin, *e = buf + k.end;
    uint64_t line = k.first_line;
    std::string vtok;
    while (p < e) {
      // One pass over the common line: N plain digit indices (>= 1, at most 19
      // digits), each followed by a space or tab, then a value token that the
      // exact decimal path reads.  The chunk holds whole lines, so every scan
      // stops at the line's '\n'.  Any other line goes to the general code below,
      // which gives the same results (and the errors) for everything.
      {
        const char *s = p;
        uint32_t iv[kMaxOrder];
        bool ok = true;
        for (int n = 0; n < N && ok; ++n) {
          while (*s == ' ' || *s == '\t') ++s;
          const char *d0 = s;
          uint64_t v = 0;
          for (unsigned d; (d = (unsigned)(*s - '0')) <= 9u; ++s) v = v * 10 + d;
          const size_t len = (size_t)(s - d0);
          iv[n] = (uint32_t)v;  // strtoull's value narrowed to uint32, as parse_index
          ok = len > 0 && len <= 19 && iv[n] >= 1 && (*s == ' ' || *s == '\t');
        }
        if (ok) {
          while (*s == ' ' || *s == '\t') ++s;
          const char *vs = s;
          while (*s != '\n' && *s != ' ' && *s != '\t') ++s;
          double d = 0;
          ok = s > vs && parse_value_fast(vs, s, d);
          if (ok) {
            const char *nl = *s == '\n' ? s : (const char *)memchr(s, '\n', (size_t)(e - s));
            for (int n = 0; n < N; ++n) {
              out->idx[n][line] = iv[n] - 1;
              if (iv[n] > k.maxd[n]) k.maxd[n] = iv[n];
            }
            if (dtype == GTK_F32)
              out->vf[line] = (float)d;
            else
              out->vd[line] = d;
            ++line;
            p = nl + 1;
            continue;
          }
        }
      }
      const char *nl = (const char *)memchr(p, '\n', (size_t)(e - p));
      if (!nl) break;
      const char *s = p;
      int n = 0;
      const char *vs = nullptr, *ve = nullptr;
      while (s < nl) {
        while (s < nl && is_delim(*s)) ++s;
        if (s >= nl) break;
        const char *te = s;
        while (te < nl && !is_delim(*te)) ++te;
        if (n < N) {
          uint32_t v = parse_index(s, te);
          if (v < 1) {
            if (line < k.err_line) {
              k.err_line = line;
              k.err_code = GTK_ERR_PARSE;
              k.err_msg = "input tensors must follow base-1 indexing";
            }
            out->idx[n][line] = 0;
          } else {
            out->idx[n][line] = v - 1;
            if (v > k.maxd[n]) k.maxd[n] = v;
          }
          ++n;
        } else {
          vs = s;
          ve = te;
          break;
        }
        s = te;
      }
      if (n < N) {
        if (line < k.err_line) {
          k.err_line = line;
          k.err_code = GTK_ERR_PARSE;
          k.err_msg = "line has fewer indices than the tensor order";
        }
      } else if (vs) {
        double d = 0;
        if (!parse_value_fast(vs, ve, d)) {
          vtok.assign(vs, ve);
          char *endp = nullptr;
          d = strtod(vtok.c_str(), &endp);
          if (endp == vtok.c_str() && line < k.err_line) {
            k.err_line = line;
            k.err_code = GTK_ERR_PARSE;
            k.err_msg = "value token is not a number";
          }
        }
        if (dtype == GTK_F32)
          out->vf[line] = (float)d;  // std::stod, then narrowed to value_t
        else
          out->vd[line] = d;
      } else {
        k.missing.push_back(line);
      }
      ++line;
      p = nl + 1;
    }
  };
  {
    std::vector<std::thread> th;
    for (unsigned c = 1; c < nt; ++c) th.emplace_back(work, c);
    work(0);
    for (auto &x : th) x.join();
  }
  for (auto &c : ch) {
    if (c.err_code) {
      char b[64];
      snprintf(b, sizeof b, " (line %llu)", (unsigned long long)(c.err_line + 1));
      return fail(c.err_code, c.err_msg + b);
    }
  }
  for (int n = 0; n < N; ++n) {
    out->dims[n] = 0;
    for (auto &c : ch) out->dims[n] = std::max(out->dims[n], c.maxd[n]);
  }
  // values of lines without one, in file order (chunks are in file order)
  GlibcRand g(seed);
  uint64_t draws = 0;
  for (const Chunk &c : ch)
    for (uint64_t l : c.missing) {
      if (dtype == GTK_F32)
        out->vf[l] = g.frand01<float>();
      else
        out->vd[l] = g.frand01<double>();
      ++draws;
    }
  out->draws = draws;
  return 0;
}

int parse_file(const char *path, int N, int dtype, uint32_t seed, gtk_coo *out) {
  const int fd = open(path, O_RDONLY);
  if (fd < 0) return fail(GTK_ERR_IO, std::string("cannot open file \"") + path + "\" for reading");
  struct stat st;
  if (fstat(fd, &st) != 0) {
    close(fd);
    return fail(GTK_ERR_IO, std::string("cannot stat \"") + path + "\"");
  }
  const size_t size = st.st_size > 0 ? (size_t)st.st_size : 0;
  HostVec<char> data(size);  // uninitialised; each reader thread touches its own pages
  // the file in slices read by all host threads at once (pread: no shared offset)
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min<unsigned>(nt, 64));
  nt = (unsigned)std::min<size_t>(nt, size / (8 << 20) + 1);
  std::vector<int> ok(nt, 1);
  auto rd = [&](unsigned c) {
    size_t off = size / nt * c;
    const size_t end = c + 1 == nt ? size : size / nt * (c + 1);
    while (off < end) {
      const ssize_t r = pread(fd, data.data() + off, end - off, (off_t)off);
      if (r <= 0) {
        if (r < 0 && errno == EINTR) continue;
        ok[c] = 0;
        return;
      }
      off += (size_t)r;
    }
  };
  {
    std::vector<std::thread> th;
    for (unsigned c = 1; c < nt; ++c) th.emplace_back(rd, c);
    rd(0);
    for (auto &x : th) x.join();
  }
  close(fd);
  for (int v : ok)
    if (!v) return fail(GTK_ERR_IO, std::string("short read on \"") + path + "\"");
  return parse_buffer(data.data(), data.size(), N, dtype, seed, out);
}

}  // namespace gtk
