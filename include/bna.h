/*
 * bna.h — C ABI of the GB300-native voxel-network builder.
 *
 * The path: BOLD time series -> z-score -> Pearson correlation as tiled GEMM
 * -> threshold (r value, |r| value or exact density) -> CSR
 * (row_ptr / col_idx / val) -> eigenvector centrality by power iteration.
 *
 * Reference (BNAPlatform, "W/" = BNAPlatform-weighted-win64-cuda7.0-20160331/src,
 * "U/" = BNAPlatform-win64-cuda7.0-20160115/src).  The reference has no plugin
 * or FFI layer; its boundary is a set of in-process C++ functions plus the
 * .csr / _ec.nm file formats.  Each entry point below names the reference
 * function(s) whose behaviour it reproduces.
 *
 * Conventions
 *  - Every call returns a bna_status (0 = success).  The reference returned 1
 *    on success from CorMat_gpu (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:161);
 *    that convention is not kept.
 *  - Plain pointers and sizes only.  "_dev" pointers are device memory of the
 *    context's device; "_host" pointers are host memory.  `stream` is a
 *    cudaStream_t passed as void* (NULL = legacy default stream).
 *  - One context per host thread at a time; contexts are independent.
 */
#ifndef BNA_H
#define BNA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bna_status {
  BNA_OK = 0,
  BNA_BAD_ARG = 1,
  BNA_OOM = 2,                /* device allocation failed */
  BNA_NNZ_OVERFLOW_INT32 = 3, /* edge count exceeds the int32 .csr format */
  BNA_NOT_CONVERGED = 4,      /* power iteration reached max_iter; outputs are still written */
  BNA_TIMEOUT = 5,
  BNA_CUDA_ERROR = 6,
  BNA_NO_DEVICE = 7,
  BNA_IO_ERROR = 8,
  BNA_CORRUPT_FILE = 9,       /* .csr lengths inconsistent (W/CUEC/weighted-net.cu:283) */
  BNA_INTERNAL = 10,          /* an internal consistency check failed */
  BNA_UNSUPPORTED = 11,
  BNA_SCRATCH_LIMIT = 12,     /* problem larger than bna_ec_noalloc's fixed scratch */
  BNA_CAPACITY = 13,          /* caller's output buffers too small (required size reported) */
  BNA_OVER_BUDGET = 14        /* request needs more device memory than the server's budget */
} bna_status;

/* Threshold rules.  r below is the reference's value after post_block
 * (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:869-884): a correlation outside
 * [-1, 1] (or NaN from a zero-variance voxel) becomes 0, except in
 * BNA_THR_R_EPS, which compares the unclamped value.  The diagonal is never
 * an edge. */
typedef enum bna_thr_mode {
  BNA_THR_R_GT = 0,   /* r >  tau : FormFullGraph, CorMat.cpp:696 (CUCorMat "r" mode) */
  BNA_THR_R_GE = 1,   /* r >= tau */
  BNA_THR_ABS_GT = 2, /* |r| > tau: FormFullGraph, U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp:198 */
  BNA_THR_ABS_GE = 3, /* |r| >= tau */
  BNA_THR_DENSITY = 4, /* value = sparsity s in percent: exactly k = Clength/2 undirected edges,
                         Clength = floor(2*M1*s/100) rounded up to even (CorMat.cpp:327-328);
                         tau = the k-th largest r; ties at tau kept in row-major (i<j) scan
                         order (FormFullGraph_s, CorMat.cpp:743-822) */
  BNA_THR_R_EPS = 5   /* tau - 1e-6 < r <= 1 + 1e-6, both sides in double (r and tau as float,
                         ep = 1e-6 a double): the 2mm and chunk GPU builders' rule,
                         W/CuCorMat-2mm/CorMat-2mm.cu:13,140,156 and
                         "CuCorMat-2mm - spa - GPUhisto-10n6 -chunk"/step2-dense2csr.cu:17,52.
                         r is the reference CPU value without post_block's clamp (a
                         zero-variance voxel's NaN never passes; 1 < r <= 1 + 8 ulp does).
                         Single-subject and batch builds; not the averaging or
                         re-thresholding entry points */
} bna_thr_mode;

/* Arithmetic of the correlation tiles.  Whatever the form, every pair whose
 * approximate r lies within `delta` of tau (or of +-1) is recomputed exactly
 * as the reference CPU path does (float products, double accumulation in
 * time order, CorMat.cpp:955-964), so the edge set equals the reference's. */
typedef enum bna_precision {
  BNA_PREC_FP32 = 0,   /* plain FP32 CUDA-core GEMM */
  BNA_PREC_BF16X3 = 1, /* split BF16 (hi*hi + hi*lo + lo*hi) on tcgen05 tensor cores, FP32 accumulate */
  BNA_PREC_TF32 = 2,   /* TF32 on tcgen05 tensor cores, FP32 accumulate */
  BNA_PREC_AUTO = 3    /* the tensor-core form bna_autotune picked for the size (tuned on
                          first use of a size bucket) */
} bna_precision;

typedef struct bna_csr {
  int32_t n;        /* vertices (voxels) */
  int64_t nnz;      /* directed entries = 2 x undirected edges */
  int32_t* row_ptr; /* n + 1 */
  int32_t* col_idx; /* nnz, ascending within each row */
  float* val;       /* nnz, r of each edge; NULL for a binary graph */
} bna_csr;

typedef struct bna_corr_opts {
  int32_t mode;      /* bna_thr_mode */
  int32_t precision; /* bna_precision */
  double value;      /* tau (compared as float, like the reference's real__t), or density percent */
  int32_t weighted;  /* 1: fill val; 0: binary graph (val = NULL) */
  double delta;      /* recompute band half-width; <= 0 selects the precision's bound */
  int32_t reserved[8];
} bna_corr_opts;

typedef struct bna_corr_stats {
  double tau;              /* threshold applied (density mode: the selected k-th largest r) */
  double delta;            /* recompute band half-width used */
  int64_t nnz;             /* directed entries */
  int64_t band_candidates; /* pairs recomputed exactly */
  int64_t band_edges;      /* recomputed pairs that became edges */
  int64_t band_1e6;        /* recomputed pairs with |r - tau| <= 1e-6 */
  int64_t ties_dropped;    /* density mode: pairs equal to tau left out to hit the exact count */
  float ms_zscore, ms_count, ms_recompute, ms_scan, ms_fill, ms_total; /* device time per stage */
  int32_t passes;          /* GEMM passes run */
  int32_t kernel_launches; /* kernels this call launched */
  int32_t precision;       /* the form that ran (BNA_PREC_AUTO resolved) */
  int32_t tile_band;       /* tensor-core forms: row blocks per band of the tile order */
  int32_t reserved[4];
} bna_corr_stats;

typedef struct bna_ctx bna_ctx;

const char* bna_status_string(int32_t status);
const char* bna_version(void);

/* Context on one CUDA device.  Owns a grow-only device arena reused across
 * calls (no allocation in steady state). */
int32_t bna_ctx_create(int32_t device, bna_ctx** out);
int32_t bna_ctx_destroy(bna_ctx* ctx);
const char* bna_ctx_last_error(const bna_ctx* ctx);
/* Release the arena's device memory (the context stays usable). */
int32_t bna_ctx_trim(bna_ctx* ctx);
/* Bytes currently held by the arena. */
int64_t bna_ctx_arena_bytes(const bna_ctx* ctx);

/* Context options (bna_ctx_set_option).  No reference counterpart: the
 * reference runs one subject per process.
 *   BNA_OPT_TILES_PER_LAUNCH: split each tensor-core correlation pass into
 *     launches of at most this many 128 x 256 tiles (0 = one launch), so that
 *     work of other streams - other requests of a server - can be scheduled
 *     between them; with it set, the exact-value passes also leave half of
 *     every SM to other work;
 *   BNA_OPT_MAX_NNZ: bna_corr_csr returns BNA_CAPACITY (stats->nnz = the
 *     required size) instead of building a CSR with more entries (0 = no
 *     limit);
 *   BNA_OPT_EC_ITERS_PER_LAUNCH: power iterations per centrality launch or
 *     graph replay, rounded up to even for replays (0 = automatic: the whole
 *     iteration for small graphs and 32 per replay for larger ones; with a
 *     launch gate, about a millisecond of iterations);
 *   BNA_OPT_TILE_BAND: row blocks (of 128 voxels) per band of the tensor-core
 *     tile order (0 = the default, 32): a persistent launch takes the tiles of
 *     a band column by column, so each column block is read from HBM once per
 *     band; the result does not depend on it. */
typedef enum bna_option {
  BNA_OPT_TILES_PER_LAUNCH = 0,
  BNA_OPT_MAX_NNZ = 1,
  BNA_OPT_EC_ITERS_PER_LAUNCH = 2,
  BNA_OPT_TILE_BAND = 3
} bna_option;
int32_t bna_ctx_set_option(bna_ctx* ctx, int32_t option, int64_t value);

/* Launch gate (no reference counterpart).  Long passes call gate(user,
 * stream, phase, done) on the calling thread between their launches: before
 * each correlation launch after the first (BNA_PHASE_CORR, done = tiles
 * launched), before each fill chunk after the first (BNA_PHASE_FILL, done =
 * row blocks filled) and before each centrality launch or graph replay after
 * the first (BNA_PHASE_EC, done = iterations completed).  With a gate set,
 * the fill runs in row-block chunks and a centrality launch or replay holds
 * about a millisecond of iterations.  The gate may block, e.g. to keep a large
 * request from queueing work while a smaller one runs (the server's use).
 * NULL removes it.  BNA_PHASE_UPLOAD (done = bytes uploaded) is the server's
 * own call before each chunk of a request's series upload. */
typedef enum bna_phase {
  BNA_PHASE_CORR = 0,
  BNA_PHASE_FILL = 1,
  BNA_PHASE_EC = 2,
  BNA_PHASE_UPLOAD = 3
} bna_phase;
typedef void (*bna_gate_fn)(void* user, void* stream, int32_t phase, int64_t done);
int32_t bna_ctx_set_gate(bna_ctx* ctx, bna_gate_fn gate, void* user);

/* Autotuner (no reference counterpart).  The shapes it searches: the two
 * tensor-core forms differ in their tile shape along K (64 BF16 values x 3
 * products vs 32 TF32 values x 1 per 128-byte stage row of a 128 x 256 tile,
 * 2 vs 4 pipeline stages) and in the width of the exact-recompute band; the
 * tile band (BNA_OPT_TILE_BAND: 16, 32 or 64 row blocks listed column by
 * column) sets how much of the operands a persistent launch re-reads from
 * HBM.  Which shape builds a CSR fastest depends on N, T and the rule.
 * bna_autotune_shape times the six on a seeded synthetic subject of size
 * N x T under `opts` (rule and value), remembers the fastest for the size
 * bucket (half-octaves of N and T) and rule kind, and returns its form and
 * band; BNA_PREC_AUTO calls resolve through these choices (form and band).
 * With the environment variable BNA_TUNE_CACHE set, choices are read from and
 * appended to that file, one line per bucket: key form band N T and the six
 * times (form-major: split-BF16 at bands 16, 32, 64, then TF32).  ms_out
 * (optional, 6 floats): those times.  bna_autotune is the same search with
 * ms_out holding the best time of each form (2 floats). */
int32_t bna_autotune_shape(bna_ctx* ctx, int32_t N, int32_t T, const bna_corr_opts* opts,
                           int32_t* precision_out, int32_t* band_out, float* ms_out);
int32_t bna_autotune(bna_ctx* ctx, int32_t N, int32_t T, const bna_corr_opts* opts,
                     int32_t* precision_out, float* ms_out);

/* Z-score, the prologue of CorMat_gpu / CorMat_cpu (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:24-52,
 * CorMat.cpp:923-951): per voxel mean and centred L2 norm in double, summed in time
 * order, z = (x - mean) / norm rounded to float.  bold_dev is time-major [T][N];
 * z_dev is voxel-major [N][ldz] (ldz >= T; columns T..ldz-1 are zeroed).  The
 * result is bit-identical to the reference's host loop. */
int32_t bna_zscore(bna_ctx* ctx, const float* bold_dev, int32_t N, int32_t T, float* z_dev,
                   int32_t ldz, void* stream);

/* Correlation -> thresholded CSR on the device.  Replaces the chain
 * CorMat_gpu (CorMat.cu:17) -> post_block (CorMat.cpp:824) -> FormFullGraph /
 * FormFullGraph_s (CorMat.cpp:683 / :743) -> FormCSRGraph (CorMat.cpp:889),
 * without materialising the N x N matrix.  bold_dev is time-major [T][N].
 * On success *out_dev points at device buffers owned by the context, valid
 * until the next bna_corr_csr / bna_ctx_trim / bna_ctx_destroy on it.
 * row_ptr and col_idx equal the reference's output on the same input. */
int32_t bna_corr_csr(bna_ctx* ctx, const float* bold_dev, int32_t N, int32_t T,
                     const bna_corr_opts* opts, bna_csr* out_dev, bna_corr_stats* stats,
                     void* stream);

/* Host-buffer form of bna_corr_csr: bold_host is time-major [T][N]; the CSR is
 * returned in host memory allocated by the library (release it with
 * bna_csr_free_host).  Host<->device copies happen inside the call. */
int32_t bna_corr_csr_host(bna_ctx* ctx, const float* bold_host, int32_t N, int32_t T,
                          const bna_corr_opts* opts, bna_csr* out_host, bna_corr_stats* stats);
void bna_csr_free_host(bna_csr* csr);

/* Host-buffer form with caller-owned outputs, like FormCSRGraph's R, C, V
 * (CorMat.cpp:889, caller-allocated after FormFullGraph returned Clength).
 * row_ptr_host has N+1 entries; col_idx_host and val_host (NULL for a binary
 * graph) have room for `cap` entries.  Pinned buffers make the copies fast.
 * *nnz_out receives the edge count; if it exceeds cap, only row_ptr is
 * written and BNA_CAPACITY is returned so the caller can grow and retry. */
int32_t bna_corr_csr_host_into(bna_ctx* ctx, const float* bold_host, int32_t N, int32_t T,
                               const bna_corr_opts* opts, int32_t* row_ptr_host,
                               int32_t* col_idx_host, float* val_host, int64_t cap,
                               int64_t* nnz_out, bna_corr_stats* stats);

/* A batch of subjects (voxel counts and series lengths may differ), each
 * built like bna_corr_csr with the same options; with a tensor-core form the
 * count passes of all subjects run as one persistent launch over their
 * concatenated tiles, and the other stages of all subjects are queued with
 * one host synchronisation per stage.  No reference counterpart (the
 * reference runs subjects one after another, CorMat.cpp:196-416).
 * out_dev[k] / stats[k] (stats may be NULL) describe subject k; its CSR
 * stays valid until the next batch call on this context (a context keeps one
 * subject context per batch position). */
int32_t bna_corr_csr_batch(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev,
                           const int32_t* N, const int32_t* T, const bna_corr_opts* opts,
                           bna_csr* out_dev, bna_corr_stats* stats, void* stream);

/* Multi-subject average, the reference's to_average modes (y / b with f or n,
 * W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:418-670): every subject's r (post_block:
 * only values in [-1, 1] count; with fisher = 1 its Fisher z, fishertrans
 * :36-42) is added in subject order into one matrix, divided by nsub (then
 * inv_fishertrans :44-50), and thresholded like one subject's matrix (opts:
 * any rule, a tensor-core form).  bold_dev[k] is subject k's time-major
 * [T[k]][N] series (same voxels for all subjects).  Device memory: the packed
 * averaged matrix (N(N-1)/2 floats) and every subject's z-scores. */
int32_t bna_corr_csr_avg(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev, int32_t N,
                         const int32_t* T, int32_t fisher, const bna_corr_opts* opts,
                         bna_csr* out_dev, bna_corr_stats* stats, void* stream);

/* The packed correlation matrix itself, the reference's .cormat content
 * (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:301-310: r of every pair i < j,
 * row-major, after post_block): approximate values of the chosen tensor-core
 * form (within its error bound of the reference's r).  With nsub > 1 the
 * multi-subject average of bna_corr_csr_avg.  packed_dev holds N(N-1)/2
 * floats of device memory. */
int32_t bna_corr_packed(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev, int32_t N,
                        const int32_t* T, int32_t fisher, int32_t precision, float* packed_dev,
                        void* stream);

/* NIfTI-1 ingest (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:141-242).  Mask:
 * datatype 2 or 16, a voxel is kept when mask >= cut; sel_out (total bytes,
 * NULL to query the sizes) marks the kept voxels.  Series: float or double
 * samples (bitpix 32 / 64) gathered for the kept voxels into bold_out, the
 * time-major [T][N] layout (NULL: only *T_out is set).  BNA_CORRUPT_FILE for
 * other types or short files. */
int32_t bna_nifti_mask(const char* path, double cut, int32_t dims_out[3], int64_t* total_out,
                       int32_t* n_out, uint8_t* sel_out);
int32_t bna_nifti_bold(const char* path, const uint8_t* sel, int64_t total, int32_t N,
                       float* bold_out, int32_t* T_out);

/* Several thresholds from one correlation pass (the reference thresholds one
 * correlation matrix once per value of its threshold list,
 * W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:105-111, 318-341).  in_dev must be the
 * weighted CSR of this context's last bna_corr_csr (an r or |r| rule); the
 * result is the CSR of the same kind of rule at tau >= the built threshold,
 * equal to what bna_corr_csr would build at tau.  Entries within the
 * recompute band of tau get their exact reference value.  out_dev lives in
 * the context's arena until the next call; band_1e6 (optional) counts the
 * entries with |r - tau| <= 1e-6. */
int32_t bna_csr_rethreshold(bna_ctx* ctx, const bna_csr* in_dev, int32_t mode, double tau,
                            bna_csr* out_dev, int64_t* band_1e6, void* stream);

/* Approximate correlation values of one BM x BN tile (rows I*128.., columns
 * J*128.. of the z-scored matrix), written row-major to out_dev (128 x 128
 * floats), for measuring max |r - r_fp64| of a precision form.  z_dev as
 * produced by bna_zscore with ldz = bna_zscore_ld(T). */
int32_t bna_corr_tile_values(bna_ctx* ctx, const float* bold_dev, int32_t N, int32_t T,
                             int32_t precision, int32_t I, int32_t J, float* out_dev, void* stream);
int32_t bna_zscore_ld(int32_t T);

/* Eigenvector centrality by power iteration, Lead_Vector_GPU
 * (W/CUEC/weighted-net.cu:55-221): u0[i] = i; loop { u0 = u; lambda = ||u||;
 * u = A (u / lambda); e1 = ||u - u0||; e2 = ||u + u0|| } until e1 <= eps or
 * e2 <= eps or max_iter iterations.  ec = the last u (not unit-norm), lambda =
 * the norm used in the last iteration.  Values are read as float and
 * promoted to double (weighted-net.cu:295-297); a NULL val means every entry
 * is 1 (U/CUEC/CUEC/CUEC_unweighted.cu:47-52).  Only the first 2*floor(nnz/2)
 * entries are used (weighted-net.cu:61).  Each row sum runs in float-float
 * (about 48 significant bits); vectors, norms and the stop test are FP64.
 * Returns BNA_NOT_CONVERGED (outputs still written) at max_iter. */
int32_t bna_ec(bna_ctx* ctx, const bna_csr* csr_dev, int32_t max_iter, double eps, double* ec_dev,
               double* lambda, int32_t* iters, void* stream);

/* Eigenvector centrality without any allocation.  No counterpart in the
 * reference: for callers that cannot allocate device memory when they need
 * the result (a process whose device memory is held by its own pool, an
 * embedder that forbids allocation after load).  Same kernels and results as
 * bna_ec, but the working vectors and iteration state live in a fixed
 * __device__ array of the library (about 8 MB, kept by every GPU that loads
 * the library until exit), so the call allocates nothing; no context is
 * needed.  Call it from ordinary host code, not from a stream callback or a
 * cudaLaunchHostFunc function: it issues CUDA calls (launches, copies, a
 * stream synchronisation), which CUDA forbids there.  Limit: n <= 262,144
 * vertices, else BNA_SCRATCH_LIMIT.  All calls share that array: calls that
 * overlap on a GPU race, so serialise them.  The first call on a device (and
 * the first after a cudaDeviceReset) looks up the array's address; make it
 * before any stream capture.  Synchronous: returns after ec_dev is written. */
int32_t bna_ec_noalloc(const bna_csr* csr_dev, int32_t max_iter, double eps, double* ec_dev,
                       double* lambda, int32_t* iters, void* stream);

/* Host-buffer form with the reference's signature shape:
 * double Lead_Vector_GPU(int* R, int* C, double* V, long N, double* ec).
 * V may be NULL (binary graph).  ec_host has N doubles. */
int32_t bna_lead_vector(bna_ctx* ctx, const int32_t* R, const int32_t* C, const double* V,
                        int64_t N, double* ec_host, double* lambda, int32_t* iters);

/* Degree of every vertex of a device CSR (the reference's Degree tool,
 * W/Degree/Degree/Degree.cpp:80-84): the float sum of each row's values in
 * column order (bit-identical to the reference's loop); the row length for a
 * binary CSR (val NULL).  deg_dev: n floats of device memory; asynchronous
 * on `stream`, on the current device. */
int32_t bna_degree(const bna_csr* csr_dev, float* deg_dev, void* stream);

/* Newman spectral modularity of the binary graph of a device CSR (the
 * reference's modularity tool, U/Newman_Modularity_CPU/Modularity_CPU/
 * Modularity_CPU.cpp: Partition :173-240, Sub_Partition :250-300,
 * Lead_Vector :315-377): round by round, the nodes of one module are split
 * by the sign of the leading eigenvector of their generalised modularity
 * matrix when its eigenvalue exceeds lambda_min (<= 0: the tool's 0.001) and
 * both sides hold more than one node.  labels_dev (n int32, device): module
 * of every vertex, 1-based, numbered in the order the modules stopped
 * dividing; *modules: their count; *q: the modularity Q (NaN without edges,
 * where the reference divides by zero).  Column order within rows is free.
 * log (optional, host, log_cap entries): one record per round that held
 * nodes, in the reference's round order — what its _modu.txt log prints
 * (Modularity_CPU.cpp:196-203, 268-283, 362-363); *log_n (optional): the
 * number of such rounds, also when it exceeds log_cap. */
typedef struct bna_mod_round {
  int32_t round;       /* the label being divided (Partition's Round) */
  int32_t nodes;       /* its node count (NumG) */
  int32_t iters[2];    /* power steps of Lead_Vector: first call, retry with
                          beta = -lambda (0 when lambda >= 0) */
  double residual[2];  /* min(err1, err2) when each call stopped */
  double lambda;       /* the eigenvalue the division test uses */
  int32_t divided;     /* 1: split in two (lambda > lambda_min, both sides > 1 node) */
  int32_t reserved;
} bna_mod_round;
int32_t bna_modularity(bna_ctx* ctx, const bna_csr* csr_dev, double lambda_min,
                       int32_t* labels_dev, int32_t* modules, double* q, bna_mod_round* log,
                       int32_t log_cap, int32_t* log_n, void* stream);
/* _modu.nm file (Modularity_CPU.cpp:122-131): int32 N; float labels[N]. */
int32_t bna_modu_write(const char* path, const int32_t* labels_host, int32_t N);

/* .csr file (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:353-360 writer,
 * W/CUEC/weighted-net.cu:275-287 reader): int32 Rlength=N+1; int32 R[N+1];
 * int32 Clength; int32 C[Clength]; then, for a weighted graph, int32 Vlength;
 * float V[Vlength].  Host buffers; bna_csr_read allocates (bna_csr_free_host). */
int32_t bna_csr_write(const char* path, const bna_csr* csr_host);
int32_t bna_csr_read(const char* path, bna_csr* csr_host_out);
/* _ec.nm file (weighted-net.cu:309-318): int32 N; float ec[N]. */
int32_t bna_ec_write(const char* path, const double* ec_host, int32_t N);

/* Serving engine.  No reference counterpart (the reference builds one
 * subject per process run).  A server owns `slots` workers on one GPU, each
 * with its own context and CUDA streams.  Submitted requests wait in arrival
 * order and are admitted as soon as a slot is free and their device-memory
 * estimate (bna_request_bytes) fits the HBM budget next to the memory the
 * other slots hold (continuous batching: requests that arrive while others
 * run join them on the device; their kernels overlap).  A request larger than
 * the whole budget is refused at submission (BNA_OVER_BUDGET).  Each request
 * runs bna_corr_csr and, if ec_max_iter > 0, bna_ec on the resulting CSR;
 * its results go to the caller's host buffers, like bna_corr_csr_host_into.
 * Requests with less work run on higher-priority streams, and correlation
 * passes are split into bounded launches, so a small request does not wait
 * for a large one to finish.  Results do not depend on what else runs. */
typedef struct bna_server bna_server;
typedef struct bna_request {
  const float* bold_host; /* time-major [T][N]; must stay valid until the reply.  A
                             page-locked buffer (cudaHostAlloc / cudaMallocHost) is read
                             by the SMs at full link speed whatever else runs; a pageable
                             one goes through the copy engine */
  int32_t N, T;
  bna_corr_opts opts;
  int32_t ec_max_iter;    /* 0: no centrality */
  double ec_eps;
  int32_t* row_ptr_host;  /* N + 1, or NULL: the CSR is not copied back (only consumed
                             on the device by the centrality) */
  int32_t* col_idx_host;  /* cap */
  float* val_host;        /* cap, or NULL (binary graph or values not wanted) */
  int64_t cap;            /* largest CSR (entries) the request may build: the size of the
                             caller's buffers; also bounds its device memory */
  double* ec_host;        /* N, or NULL */
  int64_t tag;            /* caller's value, returned in the reply */
} bna_request;
typedef struct bna_reply {
  int32_t status;         /* bna_status of the request (BNA_CAPACITY: nnz > cap) */
  int32_t slot;           /* worker that ran it */
  int64_t tag;
  int64_t nnz;            /* directed entries (the required cap on BNA_CAPACITY) */
  double lambda;          /* centrality eigenvalue (0 without centrality) */
  int32_t ec_iters;
  int32_t ec_converged;
  double t_submit, t_start, t_done; /* seconds since the server was created */
  double t_corr;          /* the CSR was built (seconds since the server was created) */
  bna_corr_stats stats;
} bna_reply;
int32_t bna_server_create(int32_t device, int32_t slots, int64_t hbm_budget_bytes,
                          bna_server** out);
/* Queue a request; *ticket identifies it for bna_server_wait. */
int32_t bna_server_submit(bna_server* srv, const bna_request* req, int64_t* ticket);
/* Block until the request is done (timeout_s < 0: no limit); fills *reply
 * and forgets the ticket.  BNA_TIMEOUT if it is still running at the limit. */
int32_t bna_server_wait(bna_server* srv, int64_t ticket, double timeout_s, bna_reply* reply);
/* Device bytes the server's slots hold right now. */
int64_t bna_server_device_bytes(const bna_server* srv);
/* Finish the queued requests and release everything. */
int32_t bna_server_destroy(bna_server* srv);
/* Directed entries of the CSR the density rule (BNA_THR_DENSITY) builds for
 * N voxels at `percent`: Clength of W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:327-328
 * (the reference's float x double arithmetic, rounded up to even). */
int64_t bna_density_nnz(int32_t N, double percent);
/* Upper estimate of the device memory one request needs (admission rule). */
int64_t bna_request_bytes(int32_t N, int32_t T, const bna_corr_opts* opts, int64_t cap,
                          int32_t with_ec);

/* Deterministic synthetic BOLD (factor model), float32 time-major [T][N]. */
typedef enum bna_synth_kind { BNA_SYNTH_IID = 0, BNA_SYNTH_BLOCKNET = 1 } bna_synth_kind;
typedef struct bna_synth_params {
  int32_t N, T, K;
  int32_t kind;      /* bna_synth_kind */
  uint64_t seed;
  double phi;        /* AR(1) coefficient of the factors */
  double load_sd;    /* loading sd (IID) or network loading scale (BLOCKNET) */
  double jitter_sd;  /* BLOCKNET: per-voxel loading sd */
  int32_t block;     /* BLOCKNET: voxels per contiguous block */
  int32_t n_net;     /* BLOCKNET: networks; block b belongs to network b mod n_net */
} bna_synth_params;
int bna_synth_bold(const bna_synth_params* p, float* out_host, int n_threads);

#ifdef __cplusplus
}
#endif
#endif /* BNA_H */
