// Host side of the C ABI, shared by its translation units: the launchers of
// the kernels, the context (its device arena, options and cached state) and
// the helpers the entry points share.  api.cu holds the context, the arena and
// the single-subject correlation -> CSR flow; tune.cu the autotuner;
// average.cu the multi-subject average; batch.cu batches; graph.cu the
// consumers of a CSR (re-thresholding, centrality, modularity).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace bna {
size_t zscore_scratch_bytes(int n_pad);
cudaError_t launch_zscore(const float* bold, int N, int T, int n_pad, float* z, int ldz,
                          uint16_t* zhi, uint16_t* zlo, int ldb, uint8_t* bad, void* scratch,
                          cudaStream_t stream);
cudaError_t launch_corr_simt(const CorrArgs& a, int pass, cudaStream_t stream);
cudaError_t launch_corr_simt_dump(const CorrArgs& a, int I, int J, float* out,
                                  cudaStream_t stream);
cudaError_t launch_recompute(const CorrArgs& a, int grid, cudaStream_t stream);
cudaError_t launch_exact_pairs(const CorrArgs& a, const uint2* pairs, int n, float* out,
                               cudaStream_t stream);
cudaError_t launch_csr_scan(int32_t* seg, int nb, int n_pad, int n, long long* rowlen,
                            long long* pre, long long* bsum, long long* total, int32_t* row_ptr,
                            uint32_t* err, cudaStream_t stream);
size_t ec_state_bytes();
size_t mod_group_bytes();
size_t mod_assign_bytes();
int mod_parts_per_block();
int mod_level_grid(int sms, size_t smem);
int mod_stage_max();
int mod_smem_max();
void mod_group_set(void* rec, int label, int row_off, int rows, int blk0, int nblk, long long kg);
void mod_group_get(const void* rec, int* err, int iters[2], double resid[2], double* lambda,
                   long long* subp, long long* subn, int* fbuf);
void mod_assign_set(void* rec, int row_off, int rows, int fbuf, int base, double w);
cudaError_t launch_mod_build(int nrows, const int32_t* rows, const int32_t* rp,
                             const int32_t* ci, const int32_t* label, const int32_t* loc,
                             int32_t* cnt, int32_t* lrp, int32_t* lci, int sms, cudaStream_t s);
cudaError_t launch_mod_level(int n, long long M, const int32_t* rp, const int32_t* label,
                             const int32_t* rows, const int32_t* lrp, const int32_t* lci,
                             void* groups, const int32_t* blk_grp, double* vd, float2* vf,
                             float2* rs, double* y, double* parts, int nrows, int stage_max,
                             int stage_bytes, int ecap, int e16, size_t smem, int grid,
                             int max_iter, double eps, cudaStream_t s);
cudaError_t launch_mod_assign(int nrows, const int32_t* rows, const void* as, int nas,
                              const double* vd, int32_t* label, cudaStream_t s);
cudaError_t launch_mod_q(int n, const int32_t* rp, const int32_t* ci, const int32_t* label,
                         unsigned long long* kmod, unsigned long long* same, int sms,
                         cudaStream_t s);
cudaError_t launch_mod_map(int n, const int32_t* label, const int32_t* adj, int32_t* out,
                           int sms, cudaStream_t s);
cudaError_t launch_ec_init(int n, double* u, float2* uf, double* parts, void* st, int grid,
                           int max_iter, cudaStream_t stream);
cudaError_t launch_ec_iter(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, const double* u,
                           const float2* uf, double* un, float2* unf, double* parts, void* st,
                           int grid, int max_iter, double eps, cudaStream_t stream);
cudaError_t launch_ec_iter_sparse(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, const double* u,
                           const float2* uf, double* un, float2* unf, double* parts, void* st,
                           int grid, int max_iter, double eps, cudaStream_t stream);
void ec_state_read(const void* host_copy, double* lam2, double* lambda_used, double* e1,
                   double* e2, int* iter, int* done);
int ec_state_err(const void* host_copy);
int ec_coop_grid(int n, int sms);
int ec_chunk_count(int n);
cudaError_t launch_ec_chunk_prep(int n, const int32_t* rp, const int32_t* ci, long long nnz_used,
                                 unsigned long long* info, int* csplit, int grid, int* rowsplit,
                                 cudaStream_t stream);
cudaError_t prepare_ec_chunk();
cudaError_t launch_ec_chunk(int n, const int32_t* rp, const int32_t* ci, const float* val,
                            const double* vald, long long nnz_used, const double* u,
                            const float2* uf, double* un, float2* unf, double* parts, void* st,
                            int grid, int max_iter, double eps, const int* rowsplit,
                            const int* csplit, float2* part, cudaStream_t stream);
cudaError_t launch_ec_coop(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, double* u, float2* uf,
                           double* parts, void* st, int grid, int it_end, int max_iter,
                           double eps, cudaStream_t stream);
void tc_tile_list(int nb, int band, std::vector<int2>& out);
long long tc_tile_count(int nb);
cudaError_t launch_tile_lists(int nb, int band, int2* tiles, long long n_smp, int s, int2* smp,
                              cudaStream_t st);
cudaError_t launch_block_bad(const uint8_t* bad, int nb, uint8_t* blockbad, cudaStream_t st);
// sched: the launch's tile counters (two, zero; the launch leaves them zero)
cudaError_t launch_corr_tc(const CorrArgs& a, int pass, int form, const int2* tiles, int ntiles,
                           const uint8_t* blockbad, float* dump, int dump_half, int grid,
                           unsigned int* sched, cudaStream_t st, const AvgPass* avg = nullptr);
cudaError_t launch_seal_candidates(const CorrArgs& a, int nwarps, cudaStream_t st);
size_t tc_subj_bytes();
bool tc_subj_fill(void* host, int s, const CorrArgs& a, const uint8_t* blockbad, int form);
cudaError_t prepare_corr_tc_multi(int form, bool dens, bool absm);
cudaError_t launch_corr_tc_multi(const CorrArgs& batch, const void* subj_dev, const int4* tiles4,
                                 int ntiles, int form, bool dens, bool absm, int grid,
                                 unsigned int* sched, cudaStream_t st);
cudaError_t launch_rowlen_scan(const long long* rowlen, int n, long long* pre, long long* bsum,
                               long long* total, int32_t* row_ptr, uint32_t* err,
                               cudaStream_t stream);
cudaError_t launch_rethr_count(const CorrArgs& a, const int32_t* rp, const int32_t* ci,
                               const float* val, const Threshold& th, uint8_t* keep, float* valx,
                               long long* rowlen, unsigned long long* band, int sms,
                               cudaStream_t st);
cudaError_t launch_rethr_fill(int n, const int32_t* rp, const int32_t* ci, const float* valx,
                              const uint8_t* keep, const int32_t* rp2, int32_t* ci2, float* val2,
                              long long nnz2, uint32_t* err, int sms, cudaStream_t st);
cudaError_t launch_corr_packed(const CorrArgs& a, int pass, cudaStream_t stream);
cudaError_t launch_avg_finalize(float* packed, long long m, int S, int fisher, int sms,
                                cudaStream_t st);
cudaError_t launch_avg_exact(const CorrArgs& a, const void* subj, int S, int fisher, float* out,
                             int sms, cudaStream_t st);
size_t avg_subj_bytes();
void avg_subj_fill(void* host, int s, const float* z, const uint8_t* bad, int ldz, int T);
size_t dens_state_bytes();
size_t dens_ties_cap();
void dens_state_read(const void* host, int* err, float* tau, long long* n_exact,
                     long long* n_ties, int* n_drop);
cudaError_t dens_set(void* state, long long k, float delta, double A, double B, cudaStream_t st);
cudaError_t launch_density_select(const CorrArgs& a, void* state, unsigned int* hist,
                                  uint8_t* cls, int* eidx, float* exact, float* slot_val,
                                  unsigned long long* ties, unsigned long long* drop, int sms,
                                  cudaStream_t st);
cudaError_t launch_csr_fill(const CorrArgs& a, int sms, int* dense_list, unsigned int* dense_count,
                            cudaStream_t stream);
cudaError_t launch_csr_fill_dense(const CorrArgs& a, int sms, int* dense_list,
                                  unsigned int* dense_count, cudaStream_t stream);
cudaError_t launch_csr_fill_rows(const CorrArgs& a, int sms, int I0, int I1, cudaStream_t stream);
cudaError_t launch_collect_candidates(const CorrArgs& a, int sms, cudaStream_t stream);
cudaError_t launch_cand_values(const CorrArgs& a, float* vals, int grid, cudaStream_t stream);
}  // namespace bna

namespace bna {


enum Slot {
  S_BOLD, S_Z, S_ZHI, S_ZLO, S_BAD, S_SEG, S_ROWLEN, S_PRE, S_BSUM, S_ROWPTR, S_COL, S_VAL,
  S_CAND, S_HKEYS, S_HVAL, S_HEDGE, S_STATUS, S_DROP, S_EC_U, S_EC_PARTS, S_EC_STATE,
  S_EC_R, S_EC_C, S_EC_V, S_EC_VD, S_DUMP, S_TILES, S_BLOCKBAD, S_DUMPTILE, S_ELIST, S_ETAB, S_HIST, S_CANDVAL,
  S_DENSE, S_WSTATE, S_VSTAT,
  S_TILES_SMP, S_DSTATE, S_DHIST, S_DCLS, S_DEIDX, S_DEXACT, S_CANDAPX, S_DTIES,
  S_RT_KEEP, S_RT_VALX, S_RT_ROWPTR, S_RT_COL, S_RT_VAL,
  S_AVG_Z, S_AVG_BAD, S_AVG_PACKED, S_AVG_UNC, S_AVG_BADZ, S_AVG_SUBJ,
  S_BATCH_SUBJ, S_BATCH_TILES,
  S_MOD_LABEL, S_MOD_ROWS, S_MOD_LOC, S_MOD_CNT, S_MOD_LRP, S_MOD_LCI, S_MOD_VD, S_MOD_VF,
  S_MOD_RS, S_MOD_Y, S_MOD_PARTS, S_MOD_GROUPS, S_MOD_BLKGRP, S_MOD_ASSIGN, S_MOD_KMOD,
  S_MOD_ADJ, S_EC_SPLIT, S_EC_PART, S_EC_ROWS, S_EC_FLAG, S_TCSCHED, S_COUNT
};

// Small device block the host reads once per pass.
struct DevStatus {
  unsigned long long cand_count;
  uint32_t err;
  uint32_t dense;  // dense sub-tiles queued by the fill pass
  unsigned long long stats[4];
  long long total;
  unsigned long long epool;  // edge-list entries handed out by the count pass
};

struct EcGraph {
  cudaGraphExec_t exec = nullptr;
  int iters = 0;  // iterations per replay
  bool chunked = false;  // the column-chunked kernel
  // the CSR, the iterate, the state block, and the chunked kernel's buffers
  const void* key[9] = {};
  int n = -1, grid = 0, max_iter = 0;
  long long nnz_used = -1;
  double eps = 0;
};

constexpr int kGraphIters = 32;
// Density rule: the histogram that locates the k-th value runs on about this
// many tiles (every s-th tile) when the problem has at least 4x as many.
constexpr int kSampleTiles = 2048;
// Row blocks per band of the tensor-core tile list (BNA_OPT_TILE_BAND): 64
// keeps a band's row operands (T = 1200: 64 x 0.6 MB) and the column pairs in
// flight in L2 and reads every column pair from DRAM once per band (measured
// on the 180k x 1200 network: count pass 76.6 ms with a row-major list,
// 61.4 / 59.4 / 72.1 ms with bands of 32 / 64 / 128).
constexpr int kDefaultBand = 64;
// Autotuner shapes: operand forms x tile bands.
struct TuneChoice {
  int prec = BNA_PREC_BF16X3;
  int band = 0;  // 0: the context's band
};
constexpr int kTuneForms[2] = {BNA_PREC_BF16X3, BNA_PREC_TF32};
constexpr int kTuneBandCount = 3;
constexpr int kTuneBands[kTuneBandCount] = {16, 32, 64};
constexpr int kTuneShapes = 2 * kTuneBandCount;
// Row-block chunks of the fill pass when the CSR goes to host buffers: chunk
// c's rows are copied out while chunk c + 1 is filled.
constexpr int kFillChunks = 8;


}  // namespace bna

using namespace bna;

struct bna_ctx {
  int device = 0;
  int sms = 0;
  cudaStream_t own_stream = nullptr;
  void* ptr[S_COUNT] = {};
  size_t cap[S_COUNT] = {};
  void* pinned = nullptr;  // small pinned host buffer for status readback
  cudaEvent_t ev[8] = {};
  std::string last_error;
  long long cand_cap = 1 << 20;
  long long elist_cap = 1LL << 23;  // edge-list pool entries (grows on demand)
  EcGraph ecg;
  int tiles_nb = -1;  // block count the uploaded tensor-core tile list was built for
  int tiles_band = 0; // and its band height (row blocks listed column by column together)
  int band = kDefaultBand;  // BNA_OPT_TILE_BAND
  int band_now = kDefaultBand;  // the band of the current call (the autotuner's for AUTO)
  int ntiles = 0;
  int ntiles_smp = 0;  // sampled tile list (density histogram), same block count
  int tiles_per_launch = 0;  // BNA_OPT_TILES_PER_LAUNCH
  int klaunch = 0;           // kernels launched by the current bna_corr_csr call
  // layout and rule of the last bna_corr_csr (its z-scores stay in the arena):
  // what bna_csr_rethreshold recomputes exact values from
  CorrArgs last{};
  bool last_ok = false;
  // multi-subject average in progress (bna_corr_csr_avg): subject table on the
  // device, count, Fisher flag
  struct Avg {
    const void* subj;
    int S;
    int fisher;
  };
  const Avg* avg = nullptr;
  // batches: one context per subject (their arenas), the host staging of the
  // density histograms, and the cached multi-subject tile list
  std::vector<bna_ctx*> kids;
  unsigned int* hist_host = nullptr;
  size_t hist_host_cap = 0;
  std::vector<int> batch_nb;
  int batch_band = 0;
  int batch_ntiles = 0;
  // autotuner choices: bucket key -> precision
  std::map<long long, TuneChoice> tune;
  bool tune_loaded = false;
  cudaStream_t cur = nullptr;  // stream of the call in progress (arena growth is ordered on it)
  long long max_nnz = 0;     // BNA_OPT_MAX_NNZ
  // host destination of the CSR (bna_corr_csr_host_into): row_ptr is copied
  // with the scan's status, and the fill pass runs in row-block chunks whose
  // entries are copied out on copy_stream while the next chunk fills
  struct Sink {
    int32_t* row_ptr;
    int32_t* col;
    float* val;
    long long cap;
    bool done;  // the CSR has been copied (row_ptr, col, val)
  };
  Sink* sink = nullptr;
  cudaStream_t copy_stream = nullptr;
  int ec_seg = 0;               // BNA_OPT_EC_ITERS_PER_LAUNCH
  bna_gate_fn gate = nullptr;  // bna_ctx_set_gate
  void* gate_user = nullptr;
  cudaEvent_t chunk_ev[kFillChunks + 1] = {};
};

namespace bna {

int32_t fail(bna_ctx* c, int32_t st, const char* fmt, ...);
cudaMemPool_t lib_pool(int device);
int32_t ensure(bna_ctx* ctx, Slot s, size_t bytes, void** out);
inline int round_up(int x, int m) { return (x + m - 1) / m * m; }
double default_delta(int precision, int T);
unsigned long long next_pow2(unsigned long long x);
inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
// Every entry point starts here: device current, and the call's stream
// recorded for stream-ordered arena growth.
int32_t set_device(bna_ctx* ctx, cudaStream_t st = nullptr);
// Z-score into the arena; fills layout fields of `a`.
int32_t run_zscore(bna_ctx* ctx, const float* bold, int N, int T, bool need_bf16, CorrArgs& a,
                   cudaStream_t st);
// Tensor-core preparation: per-block NaN flags and the upper-triangle tile list.
int32_t tc_prepare(bna_ctx* ctx, const CorrArgs& a, cudaStream_t st);
long long elist_chunk(const bna_ctx* ctx, const CorrArgs& a);
void window_from_hist(const unsigned int* hh, long long k_dens, bool sampled, int N,
                      double delta, double* winA, double* winB, Threshold* th);
// The caller's launch gate (bna_ctx_set_gate), if any.
inline void gate(bna_ctx* ctx, cudaStream_t st, int phase, long long done) {
  if (ctx->gate) ctx->gate(ctx->gate_user, st, phase, done);
}
// Blocks of the exact-value passes (warp per candidate, grid-stride): eight
// per SM fill every SM; a context that interleaves its launches with other
// work (BNA_OPT_TILES_PER_LAUNCH set: a server slot) takes half, so a
// smaller request's kernels find room beside a long exact-value pass.
inline int band_grid(const bna_ctx* ctx) {
  return ctx->tiles_per_launch > 0 ? ctx->sms * 4 : ctx->sms * 8;
}
// pass 0: count (+ edge lists); pass 3: density histogram (sampled: on the
// sampled tile list, tensor-core forms)
int32_t corr_pass(bna_ctx* ctx, const CorrArgs& a, int precision, int pass, cudaStream_t st,
                  bool sampled = false);
// Free the arena on `st` (to_driver: the pool's cached memory too).
void arena_release(bna_ctx* ctx, cudaStream_t st, bool to_driver);
// Everything after the z-scores of a single build.
int32_t corr_csr_core(bna_ctx* ctx, CorrArgs& a, int32_t N, int32_t T, const bna_corr_opts* opts,
                      int prec, double delta, bna_csr* out_dev, bna_corr_stats* stats,
                      cudaStream_t st);
// Known threshold rules and the float the kernels compare tau against.
inline bool mode_known(int m) { return m >= BNA_THR_R_GT && m <= BNA_THR_R_EPS; }
float rule_tau(const bna_corr_opts* o);
// Autotuner bucket and the precision / band of a call (tune.cu).
long long tune_key(int N, int T, int mode);
int32_t resolve_precision(bna_ctx* ctx, int N, int T, const bna_corr_opts* opts, int* prec);

}  // namespace bna

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, BNA_CUDA_ERROR, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                   \
  } while (0)

#define ENSURE(slot, bytes, ptrvar)                                          \
  do {                                                                       \
    void* p_ = nullptr;                                                      \
    int32_t st_ = ensure(ctx, slot, (size_t)(bytes), &p_);                   \
    if (st_ != BNA_OK) return st_;                                           \
    ptrvar = reinterpret_cast<decltype(ptrvar)>(p_);                         \
  } while (0)
