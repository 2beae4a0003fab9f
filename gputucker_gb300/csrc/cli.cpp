// cli.cpp -- the gputucker_gb300 command line, a drop-in for GPUTucker's main.cu.
//
// Options of the reference (cmdline_opts.cpp:27-32): -i/--input (required, a
// regular file), -o/--order (required), -r/--rank (default 10), -g/--gpus
// (default 1; this build runs one GPU).  Added: -p/--partition P_1,..,P_N
// (the reference derives P_n from free GPU memory), --iters (default 3 =
// kMaxIteration, constants.hpp:17), --tol (default 1e-4 = kLambda, the
// reference's stopping threshold, tucker.cuh:183), --seed (glibc srand seed,
// default 1 = the reference's unseeded rand()), --dtype f32|f64 (main.cu:25
// uses double), --device, --write-factors PREFIX (factor n in the slab layout,
// one text row per factor row), --checkpoint PATH (factors, core and fits saved
// after every sweep), --resume PATH (start from a saved checkpoint: its factors
// and core, sweep count and last fit), --core-update K (after each sweep's factor
// updates, K conjugate-gradient steps of the least-squares core; the reference
// never updates the core, so this changes results), --precision plain|bf16|tf32
// (the tensor-core form of the delta contraction and Gram/RHS, FP32 values only;
// default plain, the reference's arithmetic), --init-model PATH (a learned warm
// start saved by gtk_ws_save: its predicted factor rows replace the random ones,
// the core stays the random draw).  Without -p the partition comes from the
// planner (gtk_plan_partition) with the device's free memory, as the
// reference's TuckerDecomposition does (tucker.cuh:49-55).

#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gputucker_gb300.h"

static void usage() {
  printf(
      "Program Options:\n"
      "  -h [ --help ]          Display help menu.\n"
      "  -i [ --input ] arg     Input tensor path\n"
      "  -o [ --order ] arg     Order\n"
      "  -r [ --rank ] arg (=10)  Rank\n"
      "  -g [ --gpus ] arg (=1)   The number of GPUs (this build: 1)\n"
      "  -p [ --partition ] P1,..,PN (=planned)  Partition parameters\n"
      "  --iters arg (=3)       Maximum ALS sweeps\n"
      "  --tol arg (=1e-4)      Stop when |fit - previous fit| <= tol\n"
      "  --seed arg (=1)        glibc srand() seed of the initialisation\n"
      "  --dtype f32|f64 (=f64) Value type\n"
      "  --device arg (=0)      CUDA device\n"
      "  --write-factors PREFIX Write PREFIX<n>.txt per factor\n"
      "  --checkpoint PATH      Save factors, core and fits after every sweep\n"
      "  --resume PATH          Continue from a checkpoint\n"
      "  --precision plain|bf16|tf32 (=plain)  Tensor-core form (needs --dtype f32)\n"
      "  --init-model PATH      Initial factors from a saved warm-start model\n"
      "  --core-update K (=0)   K CG steps of the least-squares core after each sweep's\n"
      "                         factor updates (not in the reference: changes results)\n");
}

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

#define CHECK(x)                                                             \
  do {                                                                       \
    int rc_ = (x);                                                           \
    if (rc_) {                                                               \
      fprintf(stderr, "[ERROR] %s failed (%d): %s\n", #x, rc_, gtk_last_error()); \
      return 1;                                                              \
    }                                                                        \
  } while (0)

int main(int argc, char **argv) {
  std::string input, prefix, parts, ckpt, resume, init_model;
  int order = -1, rank = 10, gpus = 1, iters = 3, dtype = GTK_F64, device = 0, core_update = 0,
      precision = GTK_PREC_PLAIN;
  double tol = 1e-4;
  unsigned seed = 1;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto val = [&](const char *name) -> const char * {
      if (i + 1 >= argc) {
        fprintf(stderr, "[ERROR] Parsing error : option '%s' requires an argument\n", name);
        exit(2);
      }
      return argv[++i];
    };
    if (a == "-h" || a == "--help") {
      usage();
      return 0;
    } else if (a == "-i" || a == "--input") {
      input = val("input");
    } else if (a == "-o" || a == "--order") {
      order = atoi(val("order"));
    } else if (a == "-r" || a == "--rank") {
      rank = atoi(val("rank"));
    } else if (a == "-g" || a == "--gpus") {
      gpus = atoi(val("gpus"));
    } else if (a == "-p" || a == "--partition") {
      parts = val("partition");
    } else if (a == "--iters") {
      iters = atoi(val("iters"));
    } else if (a == "--tol") {
      tol = atof(val("tol"));
    } else if (a == "--seed") {
      seed = (unsigned)strtoul(val("seed"), nullptr, 10);
    } else if (a == "--dtype") {
      std::string d = val("dtype");
      if (d == "f32") dtype = GTK_F32;
      else if (d == "f64") dtype = GTK_F64;
      else {
        fprintf(stderr, "[ERROR] --dtype must be f32 or f64\n");
        return 2;
      }
    } else if (a == "--device") {
      device = atoi(val("device"));
    } else if (a == "--write-factors") {
      prefix = val("write-factors");
    } else if (a == "--checkpoint") {
      ckpt = val("checkpoint");
    } else if (a == "--resume") {
      resume = val("resume");
    } else if (a == "--core-update") {
      core_update = atoi(val("core-update"));
    } else if (a == "--init-model") {
      init_model = val("init-model");
    } else if (a == "--precision") {
      const std::string pr = val("precision");
      if (pr == "plain") precision = GTK_PREC_PLAIN;
      else if (pr == "bf16") precision = GTK_PREC_BF16;
      else if (pr == "tf32") precision = GTK_PREC_TF32;
      else {
        fprintf(stderr, "[ERROR] --precision must be plain, bf16 or tf32\n");
        return 2;
      }
    } else {
      fprintf(stderr, "[ERROR] Parsing error : unrecognised option '%s'\n", a.c_str());
      usage();
      return 2;
    }
  }
  if (input.empty()) {
    printf("[ERROR] Input file must be specified!!!\n");
    usage();
    return 2;
  }
  struct stat st;
  if (stat(input.c_str(), &st) != 0 || !S_ISREG(st.st_mode)) {
    printf("[ERROR] Input file provided does not exist [%s]\n", input.c_str());
    return 2;
  }
  if (order < 1) {
    printf("[ERROR] Tensor order must be specified!!!\n");
    usage();
    return 2;
  }
  if (gpus != 1) {
    printf("[ERROR] this build runs on one GPU (-g 1); got -g %d\n", gpus);
    return 2;
  }
  std::vector<uint32_t> P(order, 1);
  if (!parts.empty()) {
    size_t pos = 0;
    for (int n = 0; n < order; ++n) {
      size_t e = parts.find(',', pos);
      std::string tok = parts.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
      if (tok.empty()) {
        printf("[ERROR] -p needs %d comma-separated values\n", order);
        return 2;
      }
      P[n] = (uint32_t)strtoul(tok.c_str(), nullptr, 10);
      if (e == std::string::npos) {
        if (n != order - 1) {
          printf("[ERROR] -p needs %d comma-separated values\n", order);
          return 2;
        }
        break;
      }
      pos = e + 1;
    }
  }
  printf("%s\n", input.c_str());
  printf("Values are %s type.\n", dtype == GTK_F64 ? "double" : "float");
  double t0 = now();
  gtk_coo *coo = nullptr;
  CHECK(gtk_parse_file(input.c_str(), order, dtype, seed, &coo));
  uint64_t nnz = 0, draws = 0;
  std::vector<uint32_t> dims(order);
  CHECK(gtk_coo_info(coo, nullptr, nullptr, &nnz, dims.data(), &draws));
  printf("Parse time : %lf\n", now() - t0);
  for (int n = 0; n < order; ++n) printf("Max. dim[%d] = %u\n", n, dims[n]);
  printf("# nnzs: %llu\n", (unsigned long long)nnz);
  if (parts.empty()) {
    uint64_t free_b = 0, total_b = 0;
    CHECK(gtk_device_memory(device, &free_b, &total_b));
    gtk_plan plan;
    CHECK(gtk_plan_partition(order, dims.data(), nnz, rank, dtype, 1, free_b, &plan));
    for (int n = 0; n < order; ++n) P[n] = plan.partition_dims[n];
    printf("Partitioning Type: %s\n", plan.dimension_based ? "Dimension-based" : "Nonzero-based");
  }
  t0 = now();
  gtk_tensor *t = nullptr;
  CHECK(gtk_create_blocks(coo, P.data(), rank, device, &t));
  gtk_coo_free(coo);
  gtk_tensor_info info;
  CHECK(gtk_tensor_info_get(t, &info));
  printf("Blocking time : %lf\n", now() - t0);
  for (int n = 0; n < order; ++n) printf("Partition dim[%d] = %u\tBlock dim[%d] = %u\n", n, P[n], n, info.block_dims[n]);
  printf("# blocks: %llu\n", (unsigned long long)info.block_count);
  CHECK(gtk_init_random(t, seed, draws));
  if (!init_model.empty()) {
    gtk_ws *m = nullptr;
    CHECK(gtk_ws_load(init_model.c_str(), device, &m));
    const int rc = gtk_ws_apply(m, t);
    gtk_ws_destroy(m);
    CHECK(rc);
    printf("Initial factors from %s\n", init_model.c_str());
  }
  if (precision != GTK_PREC_PLAIN) CHECK(gtk_set_precision(t, precision));
  double p_fit = -1, fit = -1;
  int it = 0;
  std::vector<double> fits;
  if (!resume.empty()) {
    std::vector<double> saved(4096);
    int nsaved = 0;
    CHECK(gtk_checkpoint_load(t, resume.c_str(), saved.data(), (int)saved.size(), &nsaved));
    const int k = nsaved < (int)saved.size() ? nsaved : (int)saved.size();
    fits.assign(saved.begin(), saved.begin() + k);
    it = nsaved;
    if (k > 0) p_fit = fits.back();
    printf("Resumed from %s after %d sweeps (fit %lf)\n", resume.c_str(), it, p_fit);
  }
  const int it0 = it;
  double avg = now();
  while (it < iters) {
    double itertime = now(), step = itertime;
    CHECK(gtk_update_factor_matrices(t));
    CHECK(gtk_synchronize(t));
    printf("Factor Time : %lf\n", now() - step);
    if (core_update > 0) {
      step = now();
      int steps = 0;
      double res = 0;
      CHECK(gtk_update_core(t, core_update, &steps, &res));
      printf("Core Time : %lf (%d CG steps, relative residual %.3g)\n", now() - step, steps, res);
    }
    step = now();
    CHECK(gtk_reconstruction(t, &fit));
    printf("Recon Time : %lf\n\n", now() - step);
    ++it;
    fits.push_back(fit);
    if (!ckpt.empty()) CHECK(gtk_checkpoint_save(t, ckpt.c_str(), fits.data(), (int)fits.size()));
    printf("iter %d\t Fit: %.10g\n", it, fit);
    printf("iter%d :      Fit : %lf\tElapsed Time : %lf\n\n", it, fit, now() - itertime);
    if (it >= iters || (p_fit != -1 && (p_fit - fit > 0 ? p_fit - fit : fit - p_fit) <= tol)) break;
    p_fit = fit;
  }
  printf("Average sweep time : %lf\n", (now() - avg) / (it - it0 > 0 ? it - it0 : 1));
  if (!prefix.empty()) {
    for (int n = 0; n < order; ++n) {
      const size_t rows = (size_t)P[n] * info.block_dims[n];
      std::vector<double> fd(rows * rank);
      std::vector<float> ff(rows * rank);
      CHECK(gtk_get_factor(t, n, dtype == GTK_F64 ? (void *)fd.data() : (void *)ff.data()));
      std::string path = prefix + std::to_string(n) + ".txt";
      FILE *f = fopen(path.c_str(), "w");
      if (!f) {
        fprintf(stderr, "[ERROR] cannot write %s\n", path.c_str());
        return 1;
      }
      for (size_t r = 0; r < dims[n]; ++r) {
        for (int c = 0; c < rank; ++c)
          fprintf(f, c + 1 < rank ? "%.17g\t" : "%.17g\n", dtype == GTK_F64 ? fd[r * rank + c] : (double)ff[r * rank + c]);
      }
      fclose(f);
    }
  }
  gtk_destroy(t);
  printf("DONE\n");
  return 0;
}
