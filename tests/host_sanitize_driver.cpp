// Host-only entry points of the library under AddressSanitizer and
// UndefinedBehaviorSanitizer (tests/test_host_sanitizers.py builds the library
// and this driver with -fsanitize=address,undefined; no GPU is touched).
// Exercises the parser on well-formed and malformed text, the generator, the text
// writer (round trip through the parser), the partition planner and the
// checkpoint and warm-start model readers on damaged files.  Exit status 0 when every call
// returned what it should; the sanitizers abort on any memory or UB error.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gputucker_gb300.h"

static int failures = 0;
#define EXPECT(cond)                                                    \
  do {                                                                  \
    if (!(cond)) {                                                      \
      fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                       \
    }                                                                   \
  } while (0)

static int parse_text(const std::string &text, int order, int dtype, gtk_coo **out) {
  return gtk_parse_buffer(text.data(), text.size(), order, dtype, 1, out);
}

int main(int argc, char **argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";
  // parser: value-less lines, spaces and tabs, CRLF-free input, trailing text without '\n'
  {
    gtk_coo *c = nullptr;
    EXPECT(parse_text("1\t2\t3\t0.5\n4 5 6 1.25\n2\t2\t2\n7\t1\t1\t-3e-2\n9\t9\t9\t1", 3, GTK_F64, &c) == 0);
    int order = 0, dtype = -1;
    uint64_t nnz = 0, draws = 0;
    uint32_t dims[GTK_MAX_ORDER] = {};
    EXPECT(gtk_coo_info(c, &order, &dtype, &nnz, dims, &draws) == 0);
    EXPECT(order == 3 && nnz == 4 && draws == 1 && dims[0] == 7 && dims[1] == 5 && dims[2] == 6);
    std::vector<uint32_t> i0(nnz), i1(nnz), i2(nnz);
    std::vector<double> v(nnz);
    uint32_t *idx[3] = {i0.data(), i1.data(), i2.data()};
    EXPECT(gtk_coo_export(c, idx, v.data()) == 0);
    EXPECT(i0[0] == 0 && i1[1] == 4 && v[1] == 1.25);
    gtk_coo_free(c);
  }
  // malformed: 0-based index, too few indices, bad number, empty input, huge order
  {
    gtk_coo *c = nullptr;
    EXPECT(parse_text("0\t1\t1\t1.0\n", 3, GTK_F32, &c) == GTK_ERR_PARSE);
    EXPECT(parse_text("1\t1\n", 3, GTK_F32, &c) == GTK_ERR_PARSE);
    EXPECT(parse_text("1\t1\t1\tabc\n", 3, GTK_F32, &c) == GTK_ERR_PARSE);
    EXPECT(parse_text("\n", 3, GTK_F32, &c) == GTK_ERR_PARSE);
    EXPECT(parse_text("", 3, GTK_F32, &c) != 0 || (c != nullptr && (gtk_coo_free(c), true)));
    c = nullptr;
    EXPECT(parse_text("1\t1\t1\t1.0\n", 9, GTK_F32, &c) == GTK_ERR_ARG);
    EXPECT(gtk_parse_file((dir + "/does_not_exist.tns").c_str(), 3, GTK_F32, 1, &c) == GTK_ERR_IO);
  }
  // generator -> text writer -> parser round trip, every distribution
  const int dists[][2] = {{GTK_GEN_UNIFORM, GTK_VAL_UNIFORM}, {GTK_GEN_ZIPF, GTK_VAL_UNIFORM},
                          {GTK_GEN_ZIPF, GTK_VAL_LOGNORMAL}};
  for (const auto &d : dists) {
    const uint32_t dims[4] = {50, 60, 70, 80};
    gtk_coo *g = nullptr;
    EXPECT(gtk_generate(4, dims, 5000, d[0], 1.1, d[1], GTK_F64, 7, &g) == 0);
    const std::string path = dir + "/roundtrip.tns";
    EXPECT(gtk_write_text(g, path.c_str()) == 0);
    gtk_coo *r = nullptr;
    EXPECT(gtk_parse_file(path.c_str(), 4, GTK_F64, 1, &r) == 0);
    uint64_t n1 = 0, n2 = 0;
    int o = 0, dt = 0;
    uint32_t d1[GTK_MAX_ORDER] = {}, d2[GTK_MAX_ORDER] = {};
    uint64_t dr = 0;
    EXPECT(gtk_coo_info(g, &o, &dt, &n1, d1, &dr) == 0);
    EXPECT(gtk_coo_info(r, &o, &dt, &n2, d2, &dr) == 0);
    EXPECT(n1 == n2 && n1 == 5000);
    gtk_coo_free(g);
    gtk_coo_free(r);
  }
  {
    const uint32_t dims[3] = {40, 40, 40};
    gtk_coo *g = nullptr;
    EXPECT(gtk_generate_planted(3, dims, 3000, 4, 0.01, GTK_F32, 3, &g) == 0);
    gtk_coo_free(g);
  }
  // planner: small and large problems, one and several GPUs, invalid arguments
  {
    gtk_plan p;
    const uint32_t small[3] = {1000, 1000, 1000};
    const uint32_t big[4] = {100000, 100000, 100000, 100000};
    EXPECT(gtk_plan_partition(3, small, 1000000, 10, GTK_F64, 1, 80ull << 30, &p) == 0);
    EXPECT(p.block_count >= 1);
    EXPECT(gtk_plan_partition(4, big, 100000000, 10, GTK_F32, 1, 1ull << 30, &p) == 0);
    EXPECT(p.block_count >= 1);
    EXPECT(gtk_plan_partition(4, big, 100000000, 10, GTK_F32, 4, 16ull << 30, &p) == 0);
    EXPECT(gtk_plan_partition(0, small, 10, 10, GTK_F32, 1, 1ull << 30, &p) != 0);
  }
  // checkpoint header reader on missing, empty, truncated and garbage files
  {
    int order, rank, dtype, nfits;
    uint32_t dims[GTK_MAX_ORDER], parts[GTK_MAX_ORDER];
    EXPECT(gtk_checkpoint_info((dir + "/none.ckpt").c_str(), &order, &rank, &dtype, dims, parts, &nfits) != 0);
    const std::string bad = dir + "/bad.ckpt";
    for (size_t len : {0, 3, 8, 40, 200}) {
      FILE *f = fopen(bad.c_str(), "wb");
      std::vector<unsigned char> junk(len);
      for (size_t k = 0; k < len; ++k) junk[k] = (unsigned char)(k * 131 + 7);
      if (len >= 8) memcpy(junk.data(), "GTKCKPT1", 8);
      if (len) fwrite(junk.data(), 1, len, f);
      fclose(f);
      EXPECT(gtk_checkpoint_info(bad.c_str(), &order, &rank, &dtype, dims, parts, &nfits) != 0);
    }
  }
  // warm-start model reader on missing, truncated and garbage files (rejected
  // before any device is touched)
  {
    gtk_ws *m = nullptr;
    EXPECT(gtk_ws_load((dir + "/none.ws").c_str(), 0, &m) == GTK_ERR_IO);
    const std::string bad = dir + "/bad.ws";
    for (size_t len : {0, 7, 8, 32, 40, 400}) {
      FILE *f = fopen(bad.c_str(), "wb");
      std::vector<unsigned char> junk(len);
      for (size_t k = 0; k < len; ++k) junk[k] = (unsigned char)(k * 37 + 11);
      if (len >= 8) memcpy(junk.data(), "GTKWS001", 8);
      if (len) fwrite(junk.data(), 1, len, f);
      fclose(f);
      EXPECT(gtk_ws_load(bad.c_str(), 0, &m) == GTK_ERR_PARSE);
    }
  }
  if (failures) fprintf(stderr, "%d expectation(s) failed\n", failures);
  printf("host sanitizer driver: %s\n", failures ? "FAILED" : "ok");
  return failures ? 1 : 0;
}
