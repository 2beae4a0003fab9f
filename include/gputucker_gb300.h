/*
 * gputucker_gb300.h -- C ABI of the GB300-native sparse Tucker ALS library.
 *
 * This is the drop-in boundary for GPUTucker's factor-update path.  Each entry
 * point names the reference interface it replaces (paths inside the GPUTucker
 * project).  The reference is header-only C++ templates without a C ABI; its
 * state travels as raw pointers (Tensor<Block<uint32_t,V>>*, V*** factor slabs,
 * double** B/C scratch).  Here that state lives behind an opaque handle in the
 * GPU's HBM and crosses the boundary only as plain host arrays in the
 * reference's own layouts:
 *
 *   coordinates ... 0-based uint32, one array per mode (Block::indices, block.hpp:171)
 *   values ........ float or double (value_t; main.cu:25 uses double)
 *   factor n ...... slabs concatenated: [P_n][block_dims[n]][J] row-major, the
 *                   reference's factor_matrices[n][part][row*J+col] (tucker.cuh:71-81)
 *   core .......... J^N values in linear order, last mode fastest (tucker.cuh:117-134)
 *   count_nnz ..... per block and mode, block_dims[n]+1 uint64 (block.hpp:174)
 *   where_nnz ..... per block and mode, nnz uint32 positions (block.hpp:173)
 *
 * Every function returns GTK_OK (0) or a GTK_ERR_* status and never exits the
 * process or throws (the reference calls exit(1) on CUDA errors,
 * cuda_helper.cpp:102-109, and throws std::runtime_error on bad input).
 * gtk_last_error() returns the message of the calling thread's last failure.
 * A handle is single-threaded: do not call into one handle from two threads at
 * once.  All work of a handle runs on its own CUDA stream on one GPU.
 */
#ifndef GPUTUCKER_GB300_H_
#define GPUTUCKER_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GTK_VERSION 1

/* status codes */
#define GTK_OK 0
#define GTK_ERR_ARG 1         /* invalid argument (null pointer, order > 8, rank out of range ...) */
#define GTK_ERR_IO 2          /* file cannot be opened or read */
#define GTK_ERR_PARSE 3       /* malformed text: 0-based index, too few indices, bad number */
#define GTK_ERR_PARTITION 4   /* infeasible P_n: ceil(dims/ceil(dims/P_n)) != P_n (tensor.tpp:199-213) */
#define GTK_ERR_CUDA 5        /* CUDA runtime error (message in gtk_last_error) */
#define GTK_ERR_OOM 6         /* device allocation failed or exceeds the handle's memory cap */
#define GTK_ERR_STATE 7       /* call out of order (e.g. a sweep before the factors exist) */
#define GTK_ERR_UNSUPPORTED 8 /* shape or option not supported by this build */
#define GTK_ERR_NUMERIC 9     /* a row solve met a non-positive pivot (reported, factor row still written) */

/* value types (the reference's value_t) */
#define GTK_F32 0
#define GTK_F64 1

/* arithmetic forms of the sweep */
#define GTK_PREC_PLAIN 0      /* value_t SIMT arithmetic, FP64 Gram/solve: the reference's method */
#define GTK_PREC_BF16 1       /* delta contraction on tcgen05 tensor cores in BF16, FP32 accumulate */
#define GTK_PREC_TF32 2       /* delta contraction on tcgen05 tensor cores in TF32, FP32 accumulate */

#define GTK_MAX_ORDER 8       /* constants.hpp:16 kMaxOrder */
#define GTK_MAX_RANK 64       /* the reference's delta kernel caps J at 50 (delta.cuh:63) */

typedef struct gtk_coo gtk_coo;       /* a parsed tensor on the host (one block, global coords) */
typedef struct gtk_tensor gtk_tensor; /* a blocked tensor + factors + core resident on one GPU */

typedef struct gtk_tensor_info {
  int order;                          /* N */
  int rank;                           /* J */
  int dtype;                          /* GTK_F32 / GTK_F64 */
  int device;                         /* CUDA ordinal */
  uint64_t nnz;
  uint64_t block_count;               /* prod P_n */
  uint32_t dims[GTK_MAX_ORDER];       /* max 1-based index per mode (tensor_manager.tpp:164-176) */
  uint32_t partition_dims[GTK_MAX_ORDER];
  uint32_t block_dims[GTK_MAX_ORDER]; /* ceil(dims/P_n) */
  double norm;                        /* ||X||, summed in FP64 (the reference sums in value_t) */
  uint64_t device_bytes;              /* HBM held by the handle */
  uint32_t streamed;                  /* 1: the streamed layout (views in host memory, see gtk_create_blocks) */
  uint64_t stream_chunk;              /* nonzeros per device staging buffer of the streamed layout */
  uint32_t host_direct;               /* 1: gtk_create_blocks read the host COO in place (no upload copy) */
} gtk_tensor_info;

/* ---- errors / version ------------------------------------------------- */
const char *gtk_last_error(void);
int gtk_version(void);

/* ---- parsing: replaces ParseFromFile / _ReadData (tensor_manager.tpp:19-191) ----
 * Tab- or space-separated, 1-based indices then a value, one nonzero per '\n';
 * text after the last '\n' is ignored; dims = the largest index seen per mode.
 * A line without a value draws frand<value_t>(0,1) from the glibc rand() stream
 * seeded by `rand_seed` (the reference's unseeded rand() is seed 1), in file
 * order; gtk_coo_info reports how many draws the parse consumed so that
 * gtk_init_random can continue the same stream. */
int gtk_parse_file(const char *path, int order, int dtype, uint32_t rand_seed, gtk_coo **out);
int gtk_parse_buffer(const char *buf, size_t len, int order, int dtype, uint32_t rand_seed, gtk_coo **out);
/* A COO from arrays: idx[n] -> nnz 0-based uint32 coords; values of dtype.
 * dims may be NULL (then dims = max index + 1 per mode, as the parser does). */
int gtk_coo_from_arrays(int order, uint64_t nnz, const uint32_t *const *idx, const void *values, int dtype,
                        const uint32_t *dims, gtk_coo **out);
int gtk_coo_info(const gtk_coo *coo, int *order, int *dtype, uint64_t *nnz, uint32_t *dims, uint64_t *rand_draws);
/* copies the parsed coordinates (0-based) and values out */
int gtk_coo_export(const gtk_coo *coo, uint32_t *const *idx, void *values);
/* page-locks the COO's host arrays (cudaHostRegister) so gtk_create_blocks
 * uploads them at full link speed; undone by gtk_coo_free */
int gtk_coo_pin(gtk_coo *coo);
void gtk_coo_free(gtk_coo *coo);

/* ---- blocking: replaces CreateTensorBlocks (tensor_manager.tpp:201-302) +
 *      Tensor::AssignIndicesOfEachBlock (tensor.tpp:139-147, block.tpp:115-186).
 * Reads the COO into HBM -- in place from host memory where the device reaches
 * pageable host memory (Grace: NVLink-C2C address translation; GTK_HOST_DIRECT=0
 * uploads a copy instead), else by an upload -- and, on the GPU, assigns block
 * ids (last mode fastest),
 * stable-sorts nonzeros into blocks in input order, stores block-local coords,
 * builds the per-mode count_nnz / where_nnz of every block (bit-exact with the
 * reference) and the per-mode row-sorted views the sweep runs on.
 * P_n are given explicitly (the reference picks them from free GPU memory,
 * optimizer.tpp:95-153; all-ones is its choice whenever the tensor fits).
 * device: CUDA ordinal.  rank: J, 1..GTK_MAX_RANK. */
int gtk_create_blocks(const gtk_coo *coo, const uint32_t *partition_dims, int rank, int device, gtk_tensor **out);
int gtk_tensor_info_get(const gtk_tensor *t, gtk_tensor_info *info);
/* Layouts.  The resident layout keeps the blocked arrays, count_nnz/where_nnz
 * and one row-sorted view per mode in HBM (about (N+1)(N+3)*4 + 3*value bytes
 * per nonzero).  When that does not fit the device memory the handle may use
 * (GTK_DEVICE_MEMORY_CAP bytes if set, else the device's free memory), or when
 * GTK_FORCE_STREAMED=1, gtk_create_blocks builds the streamed layout instead --
 * the reference's host<->device block pipeline for tensors beyond HBM
 * (delta.cuh:141-213, reconstruction.cuh:132-202): the partition and the views
 * are built in host memory (page-locked where the host allows) and every mode
 * update streams its view through two device staging buffers of
 * GTK_STREAM_CHUNK nonzeros (default: a quarter of the memory left, at most
 * 2^26), copies overlapping the fused kernels on a second stream.  Factors,
 * core and Gram/RHS stay resident; the fit comes from the last mode's Gram/RHS.
 * Results equal the resident layout's up to the order of FP64 atomic adds.  Not
 * available on a streamed handle (GTK_ERR_UNSUPPORTED): the reference-order
 * variant, gtk_compute_delta, gtk_update_core, gtk_validate, the warm start,
 * batches; gtk_set_graph is accepted but sweeps run eagerly. */

/* block coordinate (N values) and nnz of one block */
int gtk_block_info(const gtk_tensor *t, uint64_t block_id, uint32_t *coord, uint64_t *nnz);
/* block-local coords (idx[n] -> nnz of the block) and values of one block, in the block's order */
int gtk_block_data(const gtk_tensor *t, uint64_t block_id, uint32_t *const *idx, void *values);
/* count_nnz (block_dims[mode]+1 uint64) and where_nnz (nnz uint32) of one block and mode */
int gtk_block_segments(const gtk_tensor *t, uint64_t block_id, int mode, uint64_t *count_nnz, uint32_t *where_nnz);
void gtk_destroy(gtk_tensor *t);

/* ---- factors and core: replaces the init in TuckerDecomposition (tucker.cuh:71-134) ----
 * Draws frand<double>(0,1) from the glibc rand() stream of `rand_seed` after
 * skipping `skip_draws` draws: factor 0..N-1, slab 0..P_n-1, the real rows of the
 * slab, column 0..J-1, then the J^N core entries in linear order.  Padding rows
 * of the last slab are 0. */
int gtk_init_random(gtk_tensor *t, uint32_t rand_seed, uint64_t skip_draws);
/* The draws gtk_init_random places, in that order: n values of frand<double>(0,1)
 * from the glibc rand() stream of `rand_seed` after `skip_draws` draws.
 * gtk_init_random generates the factors' draws on the device, in chunks whose
 * start states come from jumps in the generator's linear recurrence
 * (r[k] = r[k-3] + r[k-31] mod 2^32); this function runs the same chunks on the
 * host (no device). */
int gtk_random_sequence(uint32_t rand_seed, uint64_t skip_draws, uint64_t n, double *out);
/* slab layout [P_n * block_dims[n]][J], element type = dtype */
int gtk_set_factor(gtk_tensor *t, int mode, const void *slabs);
int gtk_get_factor(const gtk_tensor *t, int mode, void *slabs);
/* J^N values, linear order */
int gtk_set_core(gtk_tensor *t, const void *core);
int gtk_get_core(const gtk_tensor *t, void *core);

/* ---- the ALS sweep ---------------------------------------------------- */
/* GTK_PREC_PLAIN (default), GTK_PREC_BF16 or GTK_PREC_TF32 */
int gtk_set_precision(gtk_tensor *t, int precision);
/* one mode update: delta, Gram/RHS (B = lambda*I + sum delta delta^T, C = sum x*delta)
 * and the J x J row solves a = C^T B^-1, all on the GPU (update.cuh:128-199 for one mode) */
int gtk_update_mode(gtk_tensor *t, int mode);
/* No reference counterpart (GPUTucker never updates the core; off unless called,
 * and it changes results).  With the factors fixed, G minimises
 * sum_t (x_t - <G, a_0[i_0] (x) ... (x) a_{N-1}[i_{N-1}]>)^2 + lambda ||G||^2
 * (lambda = (double)0.0001f): up to cg_iters conjugate-gradient steps on its normal
 * equations from the current core, each one pass of the plain delta kernels and
 * one accumulation of sum_t y_t phi_t over the nonzeros.  At most 65536 core
 * entries (rank^order).  *iters_run receives the steps taken (they stop early at
 * a relative residual of 1e-14) and *rel_residual |b - H g| / |b| of the normal
 * equations (either may be NULL).  On an error the core is put back. */
int gtk_update_core(gtk_tensor *t, int cg_iters, int *iters_run, double *rel_residual);
/* No reference counterpart.  Consistency checks of a handle's device arrays,
 * one pass over each (no trap, no stop): violations[c] counts, for c =
 *   0 block-local coordinates >= block_dims[n], 1 view coordinates >= dims[k],
 *   2 view entries out of row order, 3 view permutation entries >= nnz,
 *   4 where_nnz entries >= their block's size, 5 count_nnz row pointers that
 *   decrease, do not start at 0 or do not end at the block's size, 6 non-finite
 *   factor or core entries, 7 block pointers that decrease, do not end at nnz or
 *   differ from the host copy.  All zero for a handle built by gtk_create_blocks. */
#define GTK_VALIDATE_CHECKS 8
int gtk_validate(gtk_tensor *t, uint64_t *violations);
/* replaces UpdateFactorMatrices (update.cuh:128-199): modes 0..N-1 in order */
int gtk_update_factor_matrices(gtk_tensor *t);
/* replaces Reconstruction (reconstruction.cuh:228-277): fit = 1 - sqrt(sum (x - x_hat)^2) / ||X||,
 * with the error summed in FP64.  Right after an update of the last mode the error
 * comes from that update: in the plain form from its stored delta, in the
 * tensor-core forms from its Gram/RHS (err = ||X||^2 - sum_i (2 a_i.c_i -
 * a_i^T G_i a_i), within ~1e-7 of the direct sum at fit 0.5); otherwise (factors
 * or core set since) delta is recomputed per nonzero. */
int gtk_reconstruction(gtk_tensor *t, double *fit);
/* replaces the loop of TuckerDecomposition (tucker.cuh:166-187): up to max_iters sweeps
 * (each UpdateFactorMatrices then Reconstruction), stopping early when
 * |fit - previous fit| <= tol (the reference: 3 sweeps, tol = lambda = 1e-4).
 * fits[i] receives the fit of sweep i (array of max_iters), *iters the sweeps run. */
int gtk_tucker_decomposition(gtk_tensor *t, int max_iters, double tol, double *fits, int *iters);
/* one sweep: gtk_update_factor_matrices then gtk_reconstruction */
int gtk_sweep(gtk_tensor *t, double *fit);
/* No reference counterpart.  on != 0: gtk_sweep (and gtk_tucker_decomposition)
 * capture the device work of a sweep -- every mode's kernels and the fit
 * kernels -- into a CUDA graph on first use and replay it afterwards; changing
 * the precision drops the graph.  Factor and core contents may change freely
 * between replays (the graph holds the handle's buffers, not their values). */
int gtk_set_graph(gtk_tensor *t, int on);
/* the delta of every nonzero for `mode` with the current factors, [nnz][J] in
 * block-major order (the reference's per-block delta buffers concatenated,
 * delta.cuh:206).  A parity hook: the sweep itself never writes delta to HBM. */
int gtk_compute_delta(gtk_tensor *t, int mode, void *delta);

/* ---- partition planner --------------------------------------------------
 * Replaces Optimizer::FindPartitionParms (optimizer.tpp:71-89), which
 * TuckerDecomposition calls with the GPU memory it could allocate
 * (tucker.cuh:49-55): same inputs, same P_n.  If the whole problem (tensor,
 * delta, core and factors per GPU) fits gpu_count * gpu_mem_bytes the plan is
 * "nonzero-based": P_n = 1.  Otherwise ("dimension-based") P_n grows on the mode
 * with the largest block until one block's data fits a quarter of one GPU's
 * memory and there are at least 4 blocks per GPU.  GTK_ERR_PARTITION where the
 * reference throws (a P_n that would leave an empty last slab).
 * gtk_device_memory reports cudaMemGetInfo of a device, the figure to plan with. */
typedef struct gtk_plan {
  uint32_t partition_dims[GTK_MAX_ORDER]; /* P_n */
  uint32_t block_dims[GTK_MAX_ORDER];     /* ceil(dims[n] / P_n) */
  uint64_t block_count;
  int dimension_based;         /* 0: nonzero-based (fits), 1: dimension-based */
  int streams;                 /* CUDA streams per GPU the reference would run: 1 or 4 */
  uint64_t avail_nnz_per_task; /* the reference's per-task nonzero budget */
  uint64_t required_bytes;     /* whole-problem bytes the decision compares with the GPUs' memory */
  uint64_t block_bytes;        /* one block's data (GetAllDataSize) under the plan */
} gtk_plan;
int gtk_plan_partition(int order, const uint32_t *dims, uint64_t nnz, int rank, int dtype, int gpu_count,
                       uint64_t gpu_mem_bytes, gtk_plan *out);
int gtk_device_memory(int device, uint64_t *free_bytes, uint64_t *total_bytes);
/* No reference counterpart.  Device blocks freed by gtk_destroy and by the
 * partition's temporaries stay cached in the process (up to half of each
 * device's memory) and serve the next requests of the same size, so repeated
 * handles of one shape neither unmap nor map memory; gtk_device_memory counts
 * them as free, an allocation that fails clears the cache and retries, and this
 * call returns every cached block to the driver. */
void gtk_release_cached_memory(void);

/* ---- checkpoint ---------------------------------------------------------
 * No reference counterpart.  gtk_checkpoint_save writes the factors, the core
 * and an optional fit history (fits[0..nfits)) of a handle to `path` (binary,
 * FNV-1a checksum, written to path.tmp then renamed).  gtk_checkpoint_load
 * restores them into a handle of the same shape, rank, value type and partition
 * (else GTK_ERR_ARG; a damaged file is GTK_ERR_PARSE) and returns the last
 * min(nfits, fits_cap) fits; sweeps then continue where the saved run stopped.
 * gtk_checkpoint_info reads the header only (no device needed). */
int gtk_checkpoint_save(gtk_tensor *t, const char *path, const double *fits, int nfits);
int gtk_checkpoint_load(gtk_tensor *t, const char *path, double *fits, int fits_cap, int *nfits);
int gtk_checkpoint_info(const char *path, int *order, int *rank, int *dtype, uint32_t *dims, uint32_t *partition_dims,
                        int *nfits);

/* ---- kernel variants, autotuner, batches -------------------------------
 * No reference counterpart.  The update kernel of a handle is one of:
 * GTK_VARIANT_SIMT2 / SIMT1 (specialised SIMT kernels, 2 or 1 nonzeros per
 * thread; shapes without a specialisation run GENERIC), GTK_VARIANT_GENERIC
 * (runtime order and rank), GTK_VARIANT_TENSOR_CORE (tcgen05; needs a precision
 * form), GTK_VARIANT_REFERENCE_ORDER (delta of the update, the fit and
 * gtk_compute_delta in the reference's operation order, computing_delta_kernel,
 * delta.cuh:62-90: core entries in linear order, products left to right, each
 * rounded -- FP32 delta bit-identical to the reference's; slow, for parity;
 * selecting it first sums the reference's serial value_t norm on the host).
 * GTK_VARIANT_AUTO: tensor cores for the precision forms, SIMT2 otherwise.  gtk_set_kernel_variant forces one; gtk_autotune times the variants
 * that apply on the handle's mode-0 update (factor 0 restored afterwards), each
 * at three tile shapes -- grids of as many CTAs per SM as fit, of 2 and of 1
 * (fewer CTAs, each sweeping more tiles of 128 / 256 / 512 nonzeros) -- keeps
 * the fastest pair (another than the first must win by 3 %) and caches it per
 * (order, rank, value type, precision, log2 mean row length, log2 longest/mean
 * row length) for the process, so later handles of the same class skip the
 * timing.  gtk_set_ctas_per_sm sets the tile shape directly (0: as many CTAs
 * per SM as fit, the default; a value above that means the same). */
#define GTK_VARIANT_AUTO (-1)
#define GTK_VARIANT_SIMT2 0
#define GTK_VARIANT_SIMT1 1
#define GTK_VARIANT_GENERIC 2
#define GTK_VARIANT_TENSOR_CORE 3
#define GTK_VARIANT_REFERENCE_ORDER 4
int gtk_set_kernel_variant(gtk_tensor *t, int variant);
int gtk_get_kernel_variant(const gtk_tensor *t, int *variant);
int gtk_autotune(gtk_tensor *t, int *variant);
int gtk_set_ctas_per_sm(gtk_tensor *t, int ctas);
int gtk_get_ctas_per_sm(const gtk_tensor *t, int *ctas);
/* A batch of handles on one device swept together: gtk_batch_sweep runs one
 * sweep (gtk_sweep) of every handle -- the first eagerly, later ones as one
 * replayed CUDA graph whose per-handle branches run concurrently -- and writes
 * fits[i] for handle i.  Handles keep their own state and may also be used on
 * their own between batch sweeps (not concurrently with one); a change of a
 * handle's precision or variant recaptures the graph.  Destroy the batch before
 * its handles.  gtk_batch_kernels: kernels in one replay of the graph (0 before
 * the first capture).  With GTK_BATCH_FUSED=1 in the environment when the batch
 * first sweeps, the graph holds the fused sweep instead: per mode index one
 * kernel zeroing every handle's Gram/RHS, one update launch per kernel class
 * for every handle of that class, the row solves batched per (rank, path), one
 * fit launch and one reduction (FP32 handles of rank <= 24 without the
 * reference-order variant; others fall back to per-handle launches). */
typedef struct gtk_batch gtk_batch;
int gtk_batch_create(gtk_tensor *const *tensors, int count, gtk_batch **out);
int gtk_batch_sweep(gtk_batch *b, double *fits);
int gtk_batch_kernels(const gtk_batch *b, uint64_t *kernels);
void gtk_batch_destroy(gtk_batch *b);

/* ---- learned warm start -------------------------------------------------
 * No reference counterpart (the reference starts from uniform [0,1) draws,
 * tucker.cuh:84-97, which stay the fallback).  A small MLP (two hidden ReLU
 * layers of `hidden` units) maps per-row statistics of a tensor to initial
 * factor rows.  Features of row i of mode n (F = 4 + 6(order-1) + order floats):
 * log(1+c_i), mean and std of the row's values; for each other mode m, over the
 * row's nonzeros: mean and std of the co-indexed row's mean value mu_m, mean of
 * lc_m = log(1 + its nonzero count), and the cross moments E[x mu_m],
 * E[x mu_m^2], E[x lc_m]; E[x prod_m mu_m]; one-hot of n.  Training and
 * inference run in the library's CUDA kernels (FP32, Adam).
 *   gtk_ws_add_example: the handle's current factors (converged by the plain
 *     method) become training targets for the features of its non-empty rows;
 *   gtk_ws_train: `steps` Adam steps on random batches of the examples (the
 *     feature standardisation is fixed from the examples at the first call);
 *   gtk_ws_apply: writes predicted factor rows into every mode of a handle whose
 *     core is set (gtk_init_random first: its core is kept, its factors replaced;
 *     padding rows 0);
 *   gtk_ws_loss_grad / gtk_ws_predict: one forward (+ backward) pass on host
 *     arrays of already standardised features (gradient checks, inspection);
 *     grad receives the flat parameter gradient in gtk_ws_get_params order:
 *     W1 [hidden x F], b1, W2 [hidden x hidden], b2, W3 [rank x hidden], b3. */
typedef struct gtk_ws gtk_ws;
int gtk_ws_create(int order, int rank, int hidden, uint64_t seed, int device, gtk_ws **out);
void gtk_ws_destroy(gtk_ws *m);
int gtk_ws_info(const gtk_ws *m, int *features, uint64_t *params, uint64_t *examples);
/* a trained model to / from a file (order, rank, width, weights, feature
 * standardisation; FNV-1a checksum; written to path.tmp then renamed).
 * gtk_ws_load creates the model on `device`; a damaged file is GTK_ERR_PARSE. */
int gtk_ws_save(const gtk_ws *m, const char *path);
int gtk_ws_load(const char *path, int device, gtk_ws **out);
int gtk_ws_get_params(const gtk_ws *m, float *params, float *feat_mean, float *feat_std);
int gtk_ws_set_params(gtk_ws *m, const float *params, const float *feat_mean, const float *feat_std);
int gtk_ws_features(gtk_tensor *t, int mode, float *out);  /* raw features, rows of mode x F, host */
int gtk_ws_add_example(gtk_ws *m, gtk_tensor *t);
int gtk_ws_train(gtk_ws *m, int steps, int batch, float lr, double *final_loss);
int gtk_ws_apply(gtk_ws *m, gtk_tensor *t);
int gtk_ws_loss_grad(gtk_ws *m, const float *x, const float *target, int batch, double *loss, float *grad);
int gtk_ws_predict(gtk_ws *m, const float *x, int batch, float *y);

/* ---- no device allocation ----------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory where they run -- latency-critical loops that must not touch the
 * allocator (cudaMalloc/cudaFree synchronise the device and take milliseconds),
 * hosts whose device memory belongs to another runtime's pool or is capped by
 * it: the sum of squared reconstruction errors sum_t (x_t - x_hat_t)^2
 * of caller-owned device data, written to d_err (one double in device memory)
 * by kernels enqueued on `stream` (a cudaStream_t; NULL = the legacy default
 * stream).  FP32 data: d_idx[n] -> nnz 0-based coordinates of mode n, d_vals ->
 * nnz values, d_factors[n] -> (largest index of mode n + 1) x rank row-major,
 * d_core -> rank^order values, last mode fastest (the arrays are device
 * pointers; the two pointer tables are host arrays).  fit = 1 - sqrt(err)/||X||.
 * Allocates nothing: the kernels' scratch is a fixed device array of
 * 8 KB + 4 MB inside the library, held on every GPU that loads it, so
 * rank^(order-1) * round_up(rank, 4) must not exceed 2^20 (else
 * GTK_ERR_UNSUPPORTED).  The first call on a device looks the array up; make it
 * before any stream capture starts.  Calls whose kernels overlap on the GPU
 * share the array and race: serialise them. */
int gtk_reconstruction_error_noalloc(int order, int rank, uint64_t nnz, const uint32_t *const *d_idx,
                                     const float *d_vals, const float *const *d_factors, const float *d_core,
                                     double *d_err, void *stream);

/* ---- data on either side of the path ----------------------------------
 * No reference counterpart: the reference only reads files it did not make.
 * gtk_generate draws `nnz` distinct coordinates (each mode uniform, or
 * Zipf(zipf_s) over a seeded permutation of the axis) and values (uniform
 * [0,1), or lognormal(0,1) scaled by its maximum to [0,1]); dims of the result
 * are the largest index drawn + 1, as the parser would report.  Deterministic
 * in `seed` whatever the host thread count.  gtk_generate_planted draws uniform
 * coordinates and values of a planted Tucker model (core and nonnegative
 * factors uniform [0,1) of rank planted_rank) plus N(0, noise_sigma^2).
 * gtk_write_text writes the reference's text format (1-based, tab-separated). */
#define GTK_GEN_UNIFORM 0
#define GTK_GEN_ZIPF 1
#define GTK_VAL_UNIFORM 0
#define GTK_VAL_LOGNORMAL 1
#define GTK_VAL_PLANTED 2
int gtk_generate(int order, const uint32_t *dims, uint64_t nnz, int index_dist, double zipf_s, int value_dist,
                 int dtype, uint64_t seed, gtk_coo **out);
int gtk_generate_planted(int order, const uint32_t *dims, uint64_t nnz, int planted_rank, double noise_sigma,
                         int dtype, uint64_t seed, gtk_coo **out);
int gtk_write_text(const gtk_coo *coo, const char *path);

/* ---- row-solve statistics ---------------------------------------------
 * No reference counterpart (the reference inverts every B by LU in FP64,
 * update.cuh:163-194).  Rows solved by a fallback since the handle was created
 * or the counters were last reset: fp64_rows -- rows of the precision forms
 * whose 1-norm condition estimate ||B||_1 est(||B^-1||_1) (Hager/Higham, from
 * the FP32 Cholesky factor) exceeded 1e5, or whose FP32 Cholesky met a
 * non-positive pivot, and were re-solved by FP64 Cholesky; lu_rows --
 * rows whose FP64 Cholesky met a non-positive pivot and were solved by LU with
 * partial pivoting.  reset != 0 zeroes both after reading. */
int gtk_solve_counters(gtk_tensor *t, uint64_t *fp64_rows, uint64_t *lu_rows, int reset);

/* ---- timing ----------------------------------------------------------- */
/* Per-kernel device time accumulated with CUDA events on the handle's stream
 * while enabled.  kind: 0 delta+gram, 1 solve, 2 fit, 3 whole sweeps replayed
 * from a graph (gtk_set_graph); kind 4 reads the number of kernels the sweep
 * entry points launched (ms = 0).  Kinds 5 and 6 read the phases of the
 * handle's gtk_create_blocks, always recorded: 5 the host-to-device upload of
 * the COO, 6 the partition and segmenting kernels (launches = 0). */
int gtk_profile_enable(gtk_tensor *t, int on);
int gtk_profile_read(gtk_tensor *t, int kind, double *ms, uint64_t *launches);
int gtk_profile_reset(gtk_tensor *t);
/* events on the handle's stream: begin records, end records + waits and returns ms */
int gtk_timer_begin(gtk_tensor *t);
int gtk_timer_end(gtk_tensor *t, double *ms);
int gtk_synchronize(gtk_tensor *t);

#ifdef __cplusplus
}
#endif

#endif /* GPUTUCKER_GB300_H_ */
