// C ABI of the voxel-network builder: context, device arena and the host
// orchestration of the correlation -> CSR passes and the power iteration.
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
void ec_state_read(const void* host_copy, double* lam2, double* lambda_used, double* e1,
                   double* e2, int* iter, int* done);
int ec_state_err(const void* host_copy);
int ec_coop_grid(int n, int sms);
cudaError_t launch_ec_coop(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, double* u, float2* uf,
                           double* parts, void* st, int grid, int it_end, int max_iter,
                           double eps, cudaStream_t stream);
void tc_tile_list(int nb, int band, std::vector<int2>& out);
long long tc_tile_count(int nb);
cudaError_t launch_tile_lists(int nb, int band, int2* tiles, long long n_smp, int s, int2* smp,
                              cudaStream_t st);
cudaError_t launch_block_bad(const uint8_t* bad, int nb, uint8_t* blockbad, cudaStream_t st);
cudaError_t launch_corr_tc(const CorrArgs& a, int pass, int form, const int2* tiles, int ntiles,
                           const uint8_t* blockbad, float* dump, int dump_half, int grid,
                           cudaStream_t st, const AvgPass* avg = nullptr);
cudaError_t launch_seal_candidates(const CorrArgs& a, int nwarps, cudaStream_t st);
size_t tc_subj_bytes();
bool tc_subj_fill(void* host, int s, const CorrArgs& a, const uint8_t* blockbad, int form);
cudaError_t prepare_corr_tc_multi(int form, bool dens, bool absm);
cudaError_t launch_corr_tc_multi(const CorrArgs& batch, const void* subj_dev, const int4* tiles4,
                                 int ntiles, int form, bool dens, bool absm, int grid,
                                 cudaStream_t st);
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

using namespace bna;

namespace {

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
  S_MOD_ADJ, S_COUNT
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
  const void* key[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
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

}  // namespace

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

namespace {

int32_t fail(bna_ctx* c, int32_t st, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->last_error = buf;
  }
  return st;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, BNA_CUDA_ERROR, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                   \
  } while (0)

}  // namespace

namespace bna {

// The library's device memory pool, one per device: freed arena blocks stay
// cached in it (release threshold: no limit) instead of going back to the
// driver at every synchronisation, so an arena that grows again (a server
// slot taking a larger request) reuses memory instead of mapping new memory;
// bna_ctx_trim hands the cached memory back.
cudaMemPool_t lib_pool(int device) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(device);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  uint64_t keep = ~0ull;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  pools[device] = pool;
  return pool;
}

}  // namespace bna

namespace {

int32_t ensure(bna_ctx* ctx, Slot s, size_t bytes, void** out) {
  if (bytes == 0) bytes = 16;
  if (ctx->cap[s] < bytes) {
    // stream-ordered on the call's stream: growing one context's arena does
    // not wait for the work other contexts have on the device
    if (ctx->ptr[s]) {
      cudaError_t e = cudaFreeAsync(ctx->ptr[s], ctx->cur);
      ctx->ptr[s] = nullptr;
      ctx->cap[s] = 0;
      if (e != cudaSuccess)
        return fail(ctx, BNA_CUDA_ERROR, "cudaFreeAsync: %s", cudaGetErrorString(e));
    }
    const size_t want = bytes + bytes / 8;  // headroom so small growth does not reallocate
    cudaMemPool_t pool = lib_pool(ctx->device);
    if (!pool) return fail(ctx, BNA_CUDA_ERROR, "no device memory pool");
    cudaError_t e = cudaMallocFromPoolAsync(&ctx->ptr[s], want, pool, ctx->cur);
    if (e != cudaSuccess) {
      cudaGetLastError();
      cudaStreamSynchronize(ctx->cur);
      cudaMemPoolTrimTo(pool, 0);  // cached blocks of other sizes go back first
      e = cudaMallocFromPoolAsync(&ctx->ptr[s], bytes, pool, ctx->cur);
      if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->ptr[s] = nullptr;
        return fail(ctx, BNA_OOM, "cudaMalloc(%zu bytes) failed", bytes);
      }
      ctx->cap[s] = bytes;
    } else {
      ctx->cap[s] = want;
    }
  }
  *out = ctx->ptr[s];
  return BNA_OK;
}

#define ENSURE(slot, bytes, ptrvar)                                          \
  do {                                                                       \
    void* p_ = nullptr;                                                      \
    int32_t st_ = ensure(ctx, slot, (size_t)(bytes), &p_);                   \
    if (st_ != BNA_OK) return st_;                                           \
    ptrvar = reinterpret_cast<decltype(ptrvar)>(p_);                         \
  } while (0)

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

double default_delta(int precision, int T) {
  const double u24 = std::ldexp(1.0, -24), u23 = std::ldexp(1.0, -23);
  switch (precision) {
    case BNA_PREC_BF16X3: return std::ldexp(1.0, -14) + 2.0 * (T + 8) * u23;
    case BNA_PREC_TF32: return std::ldexp(1.0, -9) + 2.0 * (T + 8) * u23;
    default: return 2.0 * (T + 8) * u24;
  }
}

unsigned long long next_pow2(unsigned long long x) {
  unsigned long long p = 1;
  while (p < x) p <<= 1;
  return p;
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Every entry point starts here: device current, and the call's stream
// recorded for stream-ordered arena growth.
int32_t set_device(bna_ctx* ctx, cudaStream_t st = nullptr) {
  CK(cudaSetDevice(ctx->device));
  ctx->cur = st;
  return BNA_OK;
}

// Z-score into the arena; fills layout fields of `a`.
int32_t run_zscore(bna_ctx* ctx, const float* bold, int N, int T, bool need_bf16, CorrArgs& a,
                   cudaStream_t st) {
  a.n = N;
  a.T = T;
  a.n_pad = round_up(N, kBlk);
  a.nb = a.n_pad / kBlk;
  a.ldz = round_up(T, 32);
  a.ldb = round_up(T, 64);
  float* z;
  uint8_t* bad;
  ENSURE(S_Z, (size_t)a.n_pad * a.ldz * sizeof(float), z);
  ENSURE(S_BAD, (size_t)a.n_pad, bad);
  uint16_t *zhi = nullptr, *zlo = nullptr;
  if (need_bf16) {
    ENSURE(S_ZHI, (size_t)a.n_pad * a.ldb * 2, zhi);
    ENSURE(S_ZLO, (size_t)a.n_pad * a.ldb * 2, zlo);
  }
  void* vstat;
  ENSURE(S_VSTAT, zscore_scratch_bytes(a.n_pad), vstat);
  CK(launch_zscore(bold, N, T, a.n_pad, z, a.ldz, zhi, zlo, a.ldb, bad, vstat, st));
  ctx->klaunch += 2;
  a.z = z;
  a.zhi = zhi;
  a.zlo = zlo;
  a.bad = bad;
  return BNA_OK;
}

// Tensor-core preparation: per-block NaN flags and the upper-triangle tile list.
int32_t tc_prepare(bna_ctx* ctx, const CorrArgs& a, cudaStream_t st) {
  uint8_t* bb;
  ENSURE(S_BLOCKBAD, (size_t)a.nb, bb);
  CK(launch_block_bad(a.bad, a.nb, bb, st));
  ctx->klaunch += 1;
  if (ctx->tiles_nb != a.nb || ctx->tiles_band != ctx->band_now) {
    // built on the device in stream order: no host wait for the work ahead
    const long long nt = tc_tile_count(a.nb);
    // every s-th tile: the sample the density histogram may be taken on
    const int s = (int)std::max<long long>(1, nt / kSampleTiles);
    const long long nsmp = (nt + s - 1) / s;
    int2 *d, *ds;
    ENSURE(S_TILES, (size_t)nt * sizeof(int2), d);
    ENSURE(S_TILES_SMP, (size_t)nsmp * sizeof(int2), ds);
    CK(launch_tile_lists(a.nb, ctx->band_now, d, nsmp, s, ds, st));
    ctx->klaunch += 2;
    ctx->tiles_nb = a.nb;
    ctx->tiles_band = ctx->band_now;
    ctx->ntiles = (int)nt;
    ctx->ntiles_smp = (int)nsmp;
  }
  return BNA_OK;
}

// Edge-list chunk per warp: small problems (few tiles per warp) take small
// chunks so the pool's minimum size stays modest.
long long elist_chunk(const bna_ctx* ctx, const CorrArgs& a) {
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  return nst < (long long)ctx->sms * 8 * 16 ? kElistChunkMin : kElistChunk;
}

// Density rule: the window [A, B] that holds the k-th largest exact r, from
// the histogram of r~ (2048 bins over [-1, 1) plus the specials bin); from a
// sample of the tiles the expected count gets a margin for the sampling
// spread.  Sets the count pass threshold: every pair whose exact r can lie in
// [A, B] becomes a candidate.
void window_from_hist(const unsigned int* hh, long long k_dens, bool sampled, int N,
                      double delta, double* winA, double* winB, Threshold* th) {
  const long long specials = hh[kHistBins];
  // exact counts: the k-th largest r~ lies in bins b2..b1
  double want_hi = (double)k_dens, want_lo = (double)(k_dens - specials);
  if (sampled) {
    double ns = 0;
    for (int b = 0; b <= kHistBins; ++b) ns += hh[b];
    const double M1 = (double)N * (N - 1) / 2;
    const double e = (double)k_dens / M1 * ns;
    const double m = 16.0 * std::sqrt(e) + 256.0;
    want_hi = e + m;
    want_lo = e - m - (double)specials;
  }
  long long cum = 0;
  int b1 = 0, b2 = 0;
  bool f1 = false, f2 = false;
  for (int b = kHistBins - 1; b >= 0; --b) {
    cum += hh[b];
    if (!f2 && (double)cum >= want_lo) { b2 = b; f2 = true; }
    if (!f1 && (double)cum >= want_hi) { b1 = b; f1 = true; }
  }
  if (!f2 || want_lo <= 0) b2 = kHistBins - 1;
  const double w = 2.0 / kHistBins;
  *winA = (b1 * w - 1.0) - delta;        // tau* >= A
  *winB = ((b2 + 1) * w - 1.0) + delta;  // tau* <= B
  th->mode = BNA_THR_R_GE;
  th->tau = (float)(0.5 * (*winA + *winB));
  th->delta = (float)((0.5 * (*winB - *winA) + delta) * (1.0 + 1e-6) + 1e-7);
}

// pass 0: count (+ edge lists); pass 3: density histogram (sampled: on the
// sampled tile list, tensor-core forms)
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

int32_t corr_pass(bna_ctx* ctx, const CorrArgs& a, int precision, int pass, cudaStream_t st,
                  bool sampled = false) {
  if (ctx->avg) {  // the averaged matrix is the source
    CK(launch_corr_packed(a, pass, st));
    ctx->klaunch += 1;
    return BNA_OK;
  }
  switch (precision) {
    case BNA_PREC_FP32:
      CK(launch_corr_simt(a, pass, st));
      ctx->klaunch += 1;
      return BNA_OK;
    case BNA_PREC_BF16X3:
    case BNA_PREC_TF32: {
      const int2* tiles = reinterpret_cast<const int2*>(ctx->ptr[sampled ? S_TILES_SMP : S_TILES]);
      const int nt = sampled ? ctx->ntiles_smp : ctx->ntiles;
      const int per = ctx->tiles_per_launch > 0 ? ctx->tiles_per_launch : nt;
      for (int t0 = 0; t0 < nt; t0 += per, ++ctx->klaunch) {
        if (t0 > 0) gate(ctx, st, BNA_PHASE_CORR, t0);
        CK(launch_corr_tc(a, pass, precision == BNA_PREC_BF16X3 ? 0 : 1, tiles + t0,
                          std::min(per, nt - t0),
                          reinterpret_cast<const uint8_t*>(ctx->ptr[S_BLOCKBAD]), nullptr, 0,
                          ctx->sms, st));
      }
      return BNA_OK;
    }
    default:
      return fail(ctx, BNA_UNSUPPORTED, "precision %d is not built in this library", precision);
  }
}

}  // namespace

extern "C" {

const char* bna_version(void) { return "bna-gb300 0.1"; }

const char* bna_status_string(int32_t s) {
  switch (s) {
    case BNA_OK: return "ok";
    case BNA_BAD_ARG: return "bad argument";
    case BNA_OOM: return "out of device memory";
    case BNA_NNZ_OVERFLOW_INT32: return "edge count exceeds the int32 CSR format";
    case BNA_NOT_CONVERGED: return "power iteration did not converge";
    case BNA_TIMEOUT: return "timeout";
    case BNA_CUDA_ERROR: return "CUDA error";
    case BNA_NO_DEVICE: return "no CUDA device";
    case BNA_IO_ERROR: return "I/O error";
    case BNA_CORRUPT_FILE: return "corrupt file";
    case BNA_INTERNAL: return "internal consistency check failed";
    case BNA_UNSUPPORTED: return "unsupported";
    case BNA_SCRATCH_LIMIT: return "problem exceeds the fixed scratch of the no-allocation entry point";
    case BNA_CAPACITY: return "output buffers too small";
    case BNA_OVER_BUDGET: return "request exceeds the server's device-memory budget";
    default: return "unknown status";
  }
}

int32_t bna_ctx_create(int32_t device, bna_ctx** out) {
  if (!out) return BNA_BAD_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return BNA_NO_DEVICE;
  }
  if (device < 0 || device >= n) return BNA_BAD_ARG;
  bna_ctx* ctx = new bna_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaMallocHost(&ctx->pinned, 4096) != cudaSuccess) {
    delete ctx;
    return BNA_CUDA_ERROR;
  }
  for (auto& e : ctx->ev) {
    if (cudaEventCreate(&e) != cudaSuccess) {
      delete ctx;
      return BNA_CUDA_ERROR;
    }
  }
  *out = ctx;
  return BNA_OK;
}

int64_t bna_density_nnz(int32_t N, double percent) {
  if (N < 1 || !(percent >= 0.0 && percent <= 100.0)) return -1;
  const long long M1 = (long long)N * (N - 1) / 2;
  long long clen = (long long)((double)((float)(2 * M1) * (float)percent) / 100.0);
  return clen + clen % 2;
}

int64_t bna_request_bytes(int32_t N, int32_t T, const bna_corr_opts* opts, int64_t cap,
                          int32_t with_ec) {
  if (N < 1 || T < 1 || !opts || cap < 0) return -1;
  // the arena slots bna_corr_csr / bna_ec size (run_zscore, the count pass
  // buffers, the CSR), plus the request's own BOLD and centrality buffers
  const long long n_pad = round_up(N, kBlk), nb = n_pad / kBlk;
  const long long ldz = round_up(T, 32), ldb = round_up(T, 64);
  const long long nst = nb * (nb + 1) / 2;
  const long long ntiles = nb * (nb / 2 + 1);
  const bool density = opts->mode == BNA_THR_DENSITY;
  long long nnz = cap;
  if (density) nnz = std::min<long long>(nnz, bna_density_nnz(N, opts->value));
  const int sms = 160;  // upper bound of this GPU family's SM count, for the pool minimum
  const long long chunk = nst < (long long)sms * 8 * 16 ? kElistChunkMin : kElistChunk;
  const long long elist = std::max<long long>((long long)sms * 8 * 2 * chunk, nnz / 2 + nnz / 8);
  const long long cand = 1LL << 20;
  long long b = 0;
  b += (long long)N * T * 4;                                   // BOLD
  b += n_pad * ldz * 4 + n_pad;                                // z, bad
  if (opts->precision == BNA_PREC_BF16X3 || opts->precision == BNA_PREC_AUTO)
    b += n_pad * ldb * 4;  // z hi / lo
  b += nb * n_pad * 4 + 2 * n_pad * 8 + 4096 * 8;              // seg, row lengths, block sums
  b += nst * 64 + nst * 4 + ntiles * 8 + nb;                   // etab, dense list, tiles, flags
  b += elist * 8;                                              // edge lists
  b += cand * 8 + 2 * cand * 13 + (density ? cand * 4 : 0);    // candidates, hash, values
  b += (long long)(N + 1) * 4 + nnz * (opts->weighted ? 8 : 4);  // CSR
  if (with_ec) b += (long long)N * (2 * 16 + 8) + 64 * 1024;     // iterates, output, partials
  return b;
}

int32_t bna_ctx_set_gate(bna_ctx* ctx, bna_gate_fn fn, void* user) {
  if (!ctx) return BNA_BAD_ARG;
  ctx->gate = fn;
  ctx->gate_user = fn ? user : nullptr;
  return BNA_OK;
}

int32_t bna_ctx_set_option(bna_ctx* ctx, int32_t option, int64_t value) {
  if (!ctx || value < 0) return fail(ctx, BNA_BAD_ARG, "bna_ctx_set_option: bad arguments");
  switch (option) {
    case BNA_OPT_TILES_PER_LAUNCH:
      if (value > 0x7fffffff) return fail(ctx, BNA_BAD_ARG, "tiles per launch too large");
      ctx->tiles_per_launch = (int)value;
      return BNA_OK;
    case BNA_OPT_MAX_NNZ: ctx->max_nnz = value; return BNA_OK;
    case BNA_OPT_EC_ITERS_PER_LAUNCH:
      if (value > 1000000) return fail(ctx, BNA_BAD_ARG, "iterations per launch too large");
      ctx->ec_seg = (int)value;
      return BNA_OK;
    case BNA_OPT_TILE_BAND:
      if (value > 4096) return fail(ctx, BNA_BAD_ARG, "band of %lld row blocks too large",
                                    (long long)value);
      ctx->band = value > 0 ? (int)value : kDefaultBand;
      return BNA_OK;
    default: return fail(ctx, BNA_BAD_ARG, "unknown option %d", option);
  }
}

}  // extern "C"

// Free the arena on `st` (into the library's pool; with to_driver, the
// pool's cached memory then goes back to the driver); the caller guarantees
// that no work using the arena is pending on any other stream.
static void arena_release(bna_ctx* ctx, cudaStream_t st, bool to_driver) {
  for (int s = 0; s < S_COUNT; ++s) {
    if (ctx->ptr[s]) cudaFreeAsync(ctx->ptr[s], st);
    ctx->ptr[s] = nullptr;
    ctx->cap[s] = 0;
  }
  cudaStreamSynchronize(st);
  if (to_driver)
    if (cudaMemPool_t pool = lib_pool(ctx->device)) cudaMemPoolTrimTo(pool, 0);
  ctx->tiles_nb = -1;  // the tile list lived in the arena
  ctx->last_ok = false;
  if (ctx->ecg.exec) cudaGraphExecDestroy(ctx->ecg.exec);
  ctx->ecg = EcGraph();
}

// Trim of a context whose every call has been synchronised (a server slot
// between requests): no device-wide wait, and the memory stays cached in the
// library's pool for the request that needs it.
int32_t bna_ctx_trim_idle(bna_ctx* ctx) {
  if (!ctx) return BNA_BAD_ARG;
  cudaSetDevice(ctx->device);
  arena_release(ctx, ctx->cur, false);
  return BNA_OK;
}

extern "C" {

int32_t bna_ctx_trim(bna_ctx* ctx) {
  if (!ctx) return BNA_BAD_ARG;
  cudaSetDevice(ctx->device);
  // the arena is stream-ordered memory: wait for every user, then free it
  cudaDeviceSynchronize();
  arena_release(ctx, nullptr, true);
  return BNA_OK;
}

int64_t bna_ctx_arena_bytes(const bna_ctx* ctx) {
  if (!ctx) return 0;
  int64_t t = 0;
  for (int s = 0; s < S_COUNT; ++s) t += (int64_t)ctx->cap[s];
  return t;
}

int32_t bna_ctx_destroy(bna_ctx* ctx) {
  if (!ctx) return BNA_BAD_ARG;
  for (bna_ctx* k : ctx->kids) bna_ctx_destroy(k);
  ctx->kids.clear();
  if (ctx->hist_host) cudaFreeHost(ctx->hist_host);
  bna_ctx_trim(ctx);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : ctx->chunk_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  delete ctx;
  return BNA_OK;
}

const char* bna_ctx_last_error(const bna_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int32_t bna_zscore_ld(int32_t T) { return round_up(T, 32); }

int32_t bna_zscore(bna_ctx* ctx, const float* bold_dev, int32_t N, int32_t T, float* z_dev,
                   int32_t ldz, void* stream) {
  if (!ctx || !bold_dev || !z_dev || N <= 0 || T <= 0 || ldz < T || ldz % 32 != 0)
    return fail(ctx, BNA_BAD_ARG, "bna_zscore: bad arguments");
  int32_t s = set_device(ctx, as_stream(stream));
  ctx->last_ok = false;  // the arena's z-scores may be rewritten
  if (s) return s;
  const int n_pad = round_up(N, kBlk);
  uint8_t* bad;
  ENSURE(S_BAD, (size_t)n_pad, bad);
  void* vstat;
  ENSURE(S_VSTAT, zscore_scratch_bytes(n_pad), vstat);
  // The kernel writes n_pad rows; the caller's buffer holds N rows, so stage
  // through the arena when N is not a multiple of the block.
  if (n_pad == N) {
    CK(launch_zscore(bold_dev, N, T, n_pad, z_dev, ldz, nullptr, nullptr, 0, bad, vstat,
                     as_stream(stream)));
  } else {
    float* z;
    ENSURE(S_Z, (size_t)n_pad * ldz * sizeof(float), z);
    CK(launch_zscore(bold_dev, N, T, n_pad, z, ldz, nullptr, nullptr, 0, bad, vstat,
                     as_stream(stream)));
    CK(cudaMemcpyAsync(z_dev, z, (size_t)N * ldz * sizeof(float), cudaMemcpyDeviceToDevice,
                       as_stream(stream)));
  }
  return BNA_OK;
}

static int32_t corr_csr_core(bna_ctx* ctx, CorrArgs& a, int32_t N, int32_t T,
                             const bna_corr_opts* opts, int prec, double delta, bna_csr* out_dev,
                             bna_corr_stats* stats, cudaStream_t st);

// Known threshold rules, and the float the kernels compare against: tau as
// the reference's float, or for the 2mm tools' rule (r > tau - 1e-6 in
// double) the smallest float above tau - 1e-6.
static bool mode_known(int m) { return m >= BNA_THR_R_GT && m <= BNA_THR_R_EPS; }
static float rule_tau(const bna_corr_opts* o) {
  const float t = (float)o->value;
  if (o->mode != BNA_THR_R_EPS) return t;
  const double lo = (double)t - 1e-6;
  float f = (float)lo;
  if ((double)f <= lo) f = std::nextafter(f, INFINITY);
  return f;
}

// Autotuner bucket: half-octaves of N and T, and the rule kind.
static long long tune_key(int N, int T, int mode) {
  const int nb = (int)std::floor(2.0 * std::log2((double)std::max(N, 2)));
  const int tb = (int)std::floor(2.0 * std::log2((double)std::max(T, 2)));
  return ((long long)nb << 24) | ((long long)tb << 8) | (mode == BNA_THR_DENSITY ? 1 : 0);
}

static bool band_ok(int b) { return b >= 1 && b <= 4096; }

// Cache lines: key precision band [N T times...]; a line without a valid band
// keeps the default band.
static void tune_load(bna_ctx* ctx) {
  if (ctx->tune_loaded) return;
  ctx->tune_loaded = true;
  const char* path = std::getenv("BNA_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  char line[512];
  while (std::fgets(line, sizeof line, f)) {
    long long key;
    int prec, band = 0;
    const int n = std::sscanf(line, "%lld %d %d", &key, &prec, &band);
    if (n < 2 || (prec != BNA_PREC_BF16X3 && prec != BNA_PREC_TF32)) continue;
    ctx->tune[key] = TuneChoice{prec, n == 3 && band_ok(band) ? band : 0};
  }
  std::fclose(f);
}

// The precision and tile band of a call: the caller's, or for BNA_PREC_AUTO
// the autotuner's choice for the size bucket (tuned now if not known yet).
static int32_t resolve_precision(bna_ctx* ctx, int N, int T, const bna_corr_opts* opts,
                                 int* prec) {
  *prec = opts->precision;
  ctx->band_now = ctx->band;
  if (opts->precision != BNA_PREC_AUTO) return BNA_OK;
  tune_load(ctx);
  auto it = ctx->tune.find(tune_key(N, T, opts->mode));
  if (it == ctx->tune.end()) {
    int32_t best = BNA_PREC_BF16X3, band = 0;
    const int32_t s = bna_autotune_shape(ctx, N, T, opts, &best, &band, nullptr);
    if (s) return s;
    it = ctx->tune.find(tune_key(N, T, opts->mode));
    if (it == ctx->tune.end()) return fail(ctx, BNA_INTERNAL, "autotuner kept no choice");
  }
  *prec = it->second.prec;
  ctx->band_now = it->second.band > 0 ? it->second.band : ctx->band;
  return BNA_OK;
}

int32_t bna_autotune_shape(bna_ctx* ctx, int32_t N, int32_t T, const bna_corr_opts* opts,
                           int32_t* precision_out, int32_t* band_out, float* ms_out) {
  if (!ctx || N < 2 || T < 2 || !opts || !precision_out || !band_out)
    return fail(ctx, BNA_BAD_ARG, "bna_autotune: bad arguments");
  if (!mode_known(opts->mode))
    return fail(ctx, BNA_BAD_ARG, "bna_autotune: unknown threshold mode %d", opts->mode);
  tune_load(ctx);
  int32_t s = set_device(ctx);
  if (s) return s;
  // a seeded synthetic subject of this size (the factor model of the workloads)
  std::vector<float> h((size_t)N * T);
  bna_synth_params sp{};
  sp.N = N;
  sp.T = T;
  sp.K = 40;
  sp.kind = BNA_SYNTH_IID;
  sp.seed = 0x5eedULL;
  sp.phi = 0.7;
  sp.load_sd = 0.3;
  if (bna_synth_bold(&sp, h.data(), 0) != 0) return fail(ctx, BNA_INTERNAL, "synthetic subject");
  float* bold = nullptr;
  CK(cudaMalloc(&bold, h.size() * sizeof(float)));
  cudaError_t ce = cudaMemcpy(bold, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) {
    cudaFree(bold);
    return fail(ctx, BNA_CUDA_ERROR, "bna_autotune: %s", cudaGetErrorString(ce));
  }
  // the shapes: operand form (K depth per stage, ring stages, recompute band)
  // x tile band (row blocks listed column by column)
  float ms[kTuneShapes];
  for (int k = 0; k < kTuneShapes; ++k) ms[k] = INFINITY;
  const int saved_band = ctx->band;
  for (int k = 0; k < kTuneShapes && s == BNA_OK; ++k) {
    bna_corr_opts o = *opts;
    o.precision = kTuneForms[k / kTuneBandCount];
    ctx->band = kTuneBands[k % kTuneBandCount];
    for (int rep = 0; rep < 3 && s == BNA_OK; ++rep) {  // first run warms up
      bna_csr c{};
      bna_corr_stats st{};
      s = bna_corr_csr(ctx, bold, N, T, &o, &c, &st, nullptr);
      if (s == BNA_OK && rep > 0) ms[k] = std::min(ms[k], st.ms_total);
    }
  }
  ctx->band = saved_band;
  cudaFree(bold);
  if (s) return s;
  int bk = 0;
  for (int k = 1; k < kTuneShapes; ++k)
    if (ms[k] < ms[bk]) bk = k;
  const TuneChoice best{kTuneForms[bk / kTuneBandCount], kTuneBands[bk % kTuneBandCount]};
  const long long key = tune_key(N, T, opts->mode);
  ctx->tune[key] = best;
  const char* path = std::getenv("BNA_TUNE_CACHE");
  if (path && *path) {
    if (FILE* f = std::fopen(path, "a")) {
      std::fprintf(f, "%lld %d %d %d %d", key, best.prec, best.band, N, T);
      for (int k = 0; k < kTuneShapes; ++k) std::fprintf(f, " %.4f", ms[k]);
      std::fprintf(f, "\n");
      std::fclose(f);
    }
  }
  *precision_out = best.prec;
  *band_out = best.band;
  if (ms_out)
    for (int k = 0; k < kTuneShapes; ++k) ms_out[k] = ms[k];
  return BNA_OK;
}

int32_t bna_autotune(bna_ctx* ctx, int32_t N, int32_t T, const bna_corr_opts* opts,
                     int32_t* precision_out, float* ms_out) {
  int32_t band = 0;
  float ms[kTuneShapes];
  const int32_t s = bna_autotune_shape(ctx, N, T, opts, precision_out, &band, ms);
  if (s == BNA_OK && ms_out)
    for (int f = 0; f < 2; ++f) {  // the best time of each form
      ms_out[f] = INFINITY;
      for (int b = 0; b < kTuneBandCount; ++b)
        ms_out[f] = std::min(ms_out[f], ms[f * kTuneBandCount + b]);
    }
  return s;
}

int32_t bna_corr_csr(bna_ctx* ctx, const float* bold_dev, int32_t N, int32_t T,
                     const bna_corr_opts* opts, bna_csr* out_dev, bna_corr_stats* stats,
                     void* stream) {
  if (!ctx || !bold_dev || !opts || !out_dev || N < 1 || T < 1)
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr: bad arguments");
  if (!mode_known(opts->mode))
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr: unknown threshold mode %d", opts->mode);
  if (opts->precision < BNA_PREC_FP32 || opts->precision > BNA_PREC_AUTO)
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr: unknown precision %d", opts->precision);
  const bool density = opts->mode == BNA_THR_DENSITY;
  if (density && !(opts->value >= 0.0 && opts->value <= 100.0))
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr: density %g%% outside [0, 100]", opts->value);
  int prec = opts->precision;
  int32_t s = resolve_precision(ctx, N, T, opts, &prec);
  if (s) return s;
  s = set_device(ctx, as_stream(stream));
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  ctx->klaunch = 0;
  ctx->last_ok = false;  // the arena is about to be rewritten
  CorrArgs a{};
  CK(cudaEventRecord(ctx->ev[0], st));
  s = run_zscore(ctx, bold_dev, N, T, prec == BNA_PREC_BF16X3, a, st);
  if (s) return s;
  if (prec != BNA_PREC_FP32) {
    s = tc_prepare(ctx, a, st);
    if (s) return s;
  }
  CK(cudaEventRecord(ctx->ev[1], st));
  const double delta = opts->delta > 0 ? opts->delta : default_delta(prec, T);
  return corr_csr_core(ctx, a, N, T, opts, prec, delta, out_dev, stats, st);
}

// Everything after the z-scores: count pass(es), candidates, density rule,
// scan, fill.  With ctx->avg set (multi-subject average) the count pass reads
// the averaged matrix and candidates get their exact averaged value.
static int32_t corr_csr_core(bna_ctx* ctx, CorrArgs& a, int32_t N, int32_t T,
                             const bna_corr_opts* opts, int prec, double delta, bna_csr* out_dev,
                             bna_corr_stats* stats, cudaStream_t st) {
  const bool density = opts->mode == BNA_THR_DENSITY;
  int32_t s = BNA_OK;
  a.weighted = opts->weighted ? 1 : 0;

  ENSURE(S_SEG, (size_t)a.nb * a.n_pad * sizeof(int32_t), a.seg);
  long long *rowlen, *pre, *bsum;
  ENSURE(S_ROWLEN, (size_t)a.n_pad * 8, rowlen);
  ENSURE(S_PRE, (size_t)a.n_pad * 8, pre);
  ENSURE(S_BSUM, (size_t)4096 * 8, bsum);
  int32_t* row_ptr;
  ENSURE(S_ROWPTR, (size_t)(N + 1) * 4, row_ptr);
  DevStatus* ds;
  ENSURE(S_STATUS, sizeof(DevStatus), ds);
  a.err = &ds->err;
  a.cand_count = &ds->cand_count;
  a.stats = ds->stats;
  a.drop_keys = nullptr;
  a.n_drop = 0;
  a.cand_val = nullptr;
  DevStatus* hs = reinterpret_cast<DevStatus*>(ctx->pinned);
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  ENSURE(S_ETAB, (size_t)nst * 4 * sizeof(longlong2), a.etab);
  a.epool = &ds->epool;

  // ---- threshold of the count pass
  long long k_dens = 0;  // density: exact undirected edge count (CorMat.cpp:327-329)
  if (density) k_dens = bna_density_nnz(N, opts->value) / 2;
  const bool tc = prec != BNA_PREC_FP32 && !ctx->avg;
  // density with a tensor-core form: the k-th value is selected on the device;
  // its window comes first from a histogram of sampled tiles, and from the
  // full histogram if the sample's window missed
  bool sampled = density && k_dens > 0 && tc && ctx->ntiles >= 4 * kSampleTiles;
  bool dev_sel = density && k_dens > 0 && tc;
  double winA = 0, winB = 0;
  int passes = 0;
  float* cvals = nullptr;
  long long ties_dropped = 0;
  int dens_err = 0;
  for (int wtry = 0;; ++wtry) {
    if (!density) {
      a.th.mode = opts->mode;
      a.th.tau = rule_tau(opts);
      a.th.delta = (float)delta;
    } else if (k_dens == 0) {
      a.th.mode = BNA_THR_R_GT;  // no edge at all
      a.th.tau = 2.0f;
      a.th.delta = (float)delta;
    } else {
      // histogram pass: locate the bin(s) that can hold the k-th largest r
      unsigned int* hist;
      ENSURE(S_HIST, (kHistBins + 1) * sizeof(unsigned int), hist);
      CK(cudaMemsetAsync(hist, 0, (kHistBins + 1) * sizeof(unsigned int), st));
      a.hist = hist;
      a.cand_apx = nullptr;
      a.th.mode = BNA_THR_R_GE;
      a.th.tau = 0.0f;
      a.th.delta = (float)delta;
      s = corr_pass(ctx, a, prec, 3, st, sampled);
      if (s) return s;
      ++passes;
      std::vector<unsigned int> hh(kHistBins + 1);
      CK(cudaMemcpyAsync(hh.data(), hist, hh.size() * sizeof(unsigned int),
                         cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      window_from_hist(hh.data(), k_dens, sampled, N, delta, &winA, &winB, &a.th);
    }
    const Threshold count_th = a.th;

    for (int attempt = 0;; ++attempt) {
      a.cand_cap = ctx->cand_cap;
      // the pool hands out one chunk per warp at a time: room for two per warp
      a.echunk = elist_chunk(ctx, a);
      const long long min_pool = (long long)ctx->sms * 8 * 2 * a.echunk;
      if (ctx->elist_cap < min_pool) ctx->elist_cap = min_pool;
      a.ecap = ctx->elist_cap;
      const unsigned long long hcap = next_pow2((unsigned long long)a.cand_cap * 2);
      a.hmask = hcap - 1;
      ENSURE(S_CAND, (size_t)a.cand_cap * sizeof(uint2), a.cand);
      ENSURE(S_HKEYS, hcap * 8, a.hkeys);
      ENSURE(S_HVAL, hcap * 4, a.hval);
      ENSURE(S_HEDGE, hcap, a.hedge);
      ENSURE(S_ELIST, (size_t)a.ecap * sizeof(uint2), a.elist);
      if ((density && k_dens > 0) || ctx->avg)
        ENSURE(S_CANDVAL, (size_t)a.cand_cap * sizeof(float), cvals);
      a.cand_apx = nullptr;
      if (dev_sel) ENSURE(S_CANDAPX, (size_t)a.cand_cap * sizeof(float), a.cand_apx);
      CK(cudaMemsetAsync(ds, 0, sizeof(DevStatus), st));
      CK(cudaMemsetAsync(a.hkeys, 0xff, hcap * 8, st));
      const int nwarps = ctx->sms * 8;  // epilogue warps of the tensor-core pass
      ENSURE(S_WSTATE, (size_t)nwarps * 4 * sizeof(long long), a.wstate);
      CK(cudaMemsetAsync(a.wstate, 0, (size_t)nwarps * 4 * sizeof(long long), st));
      a.th = count_th;
      s = corr_pass(ctx, a, prec, 0, st);
      if (s) return s;
      if (tc) CK(launch_seal_candidates(a, nwarps, st));
      ctx->klaunch += 1;  // seal or collect
      ++passes;
      CK(cudaEventRecord(ctx->ev[2], st));
      // the tensor-core count pass lists its candidates itself
      if (!tc) CK(launch_collect_candidates(a, ctx->sms, st));
      if (dev_sel) {
        void* dstate;
        unsigned int* dhist;
        uint8_t* dcls;
        int* deidx;
        float* dexact;
        unsigned long long* dties;
        ENSURE(S_DSTATE, dens_state_bytes(), dstate);
        ENSURE(S_DHIST, 2048 * sizeof(unsigned int), dhist);
        ENSURE(S_DCLS, (size_t)a.cand_cap, dcls);
        ENSURE(S_DEIDX, (size_t)a.cand_cap * sizeof(int), deidx);
        ENSURE(S_DEXACT, (size_t)a.cand_cap * sizeof(float), dexact);
        ENSURE(S_DTIES, 2 * dens_ties_cap() * sizeof(unsigned long long), dties);
        CK(dens_set(dstate, k_dens, (float)delta, winA, winB, st));
        CK(cudaMemsetAsync(dhist, 0, 2048 * sizeof(unsigned int), st));
        CK(launch_density_select(a, dstate, dhist, dcls, deidx, dexact, cvals, dties,
                                 dties + dens_ties_cap(), ctx->sms, st));
        ctx->klaunch += 18 + 4;  // selection and decision, scan
        CK(cudaEventRecord(ctx->ev[3], st));
        CK(launch_csr_scan(a.seg, a.nb, a.n_pad, N, rowlen, pre, bsum, &ds->total, row_ptr,
                           a.err, st));
        CK(cudaMemcpyAsync(static_cast<char*>(ctx->pinned) + 2048, dstate, dens_state_bytes(),
                           cudaMemcpyDeviceToHost, st));
      } else if (density && k_dens > 0) {
        if (ctx->avg)
          CK(launch_avg_exact(a, ctx->avg->subj, ctx->avg->S, ctx->avg->fisher, cvals, ctx->sms,
                              st));
        else
          CK(launch_cand_values(a, cvals, band_grid(ctx), st));
        ctx->klaunch += 1;
      } else {
        if (ctx->avg) {  // exact averaged values, then the decisions on them
          CK(launch_avg_exact(a, ctx->avg->subj, ctx->avg->S, ctx->avg->fisher, cvals, ctx->sms,
                              st));
          a.cand_val = cvals;
          ctx->klaunch += 1;
        }
        CK(launch_recompute(a, band_grid(ctx), st));
        ctx->klaunch += 1 + 4;  // recompute, scan
        CK(cudaEventRecord(ctx->ev[3], st));
        CK(launch_csr_scan(a.seg, a.nb, a.n_pad, N, rowlen, pre, bsum, &ds->total, row_ptr,
                           a.err, st));
      }
      CK(cudaEventRecord(ctx->ev[4], st));
      if (ctx->sink)
        CK(cudaMemcpyAsync(ctx->sink->row_ptr, row_ptr, (size_t)(N + 1) * 4,
                           cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(hs, ds, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      bool again = false;
      if ((hs->err & (ERR_BAND_OVERFLOW | ERR_HASH_FULL)) && attempt < 3) {
        ctx->cand_cap = (long long)(hs->cand_count * 3 / 2) + 1024;
        again = true;
      }
      if ((hs->err & ERR_ELIST) && attempt < 3) {
        ctx->elist_cap = (long long)(hs->epool + hs->epool / 4) + a.echunk;
        again = true;
      }
      if (!again) break;
    }
    if (hs->err & ERR_TIMEOUT) return fail(ctx, BNA_TIMEOUT, "count pass: a bounded wait expired");
    if (hs->err & ERR_BAND_OVERFLOW)
      return fail(ctx, BNA_INTERNAL, "candidate list overflow (%llu candidates)", hs->cand_count);
    if (hs->err & ERR_ELIST)
      return fail(ctx, BNA_INTERNAL, "edge-list pool overflow (%llu entries)", hs->epool);
    if (hs->err & ERR_HASH_FULL) return fail(ctx, BNA_INTERNAL, "candidate hash full");
    if (dev_sel) {
      float tau_d = 0;
      long long n_exact = 0, n_ties = 0;
      int n_drop = 0;
      dens_state_read(static_cast<char*>(ctx->pinned) + 2048, &dens_err, &tau_d, &n_exact,
                      &n_ties, &n_drop);
      if (dens_err == 1 && sampled) {  // the sampled window missed: full histogram
        sampled = false;
        continue;
      }
      if (dens_err == 0) {
        a.th.mode = BNA_THR_DENSITY;
        a.th.tau = tau_d;
        ties_dropped = n_drop;
        if (hs->total != 2 * k_dens)
          return fail(ctx, BNA_INTERNAL, "density: %lld entries instead of %lld", hs->total,
                      2 * k_dens);
      } else {
        // ties beyond the device sort (or an inconsistency): the host selection
        dev_sel = false;
        CK(launch_cand_values(a, cvals, band_grid(ctx), st));
        ctx->klaunch += 1;
      }
    }
    break;
  }
  if (density && k_dens > 0 && !dev_sel) {
    // FormFullGraph_s (CorMat.cpp:770-808): tau* = the k-th largest r; every
    // larger pair is an edge; of the pairs equal to tau*, the first ones in
    // row-major (i < j) order are kept up to k edges.  Every pair that can be
    // tau* or a tie is a candidate with its exact value here.
    // candidate slots (the tensor-core pass leaves unused slots marked kCandNone)
    const long long slots = std::min<long long>((long long)hs->cand_count, a.cand_cap);
    const long long definite = (long long)hs->stats[2];
    std::vector<float> v(slots);
    std::vector<uint2> keys(slots);
    CK(cudaMemcpyAsync(v.data(), cvals, slots * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(keys.data(), a.cand, slots * sizeof(uint2), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    long long n = 0;
    for (long long c = 0; c < slots; ++c)
      if (keys[c].x != kCandNone) {
        v[n] = v[c];
        keys[n] = keys[c];
        ++n;
      }
    v.resize(n);
    keys.resize(n);
    const long long need = k_dens - definite;
    if (need < 1 || need > n)
      return fail(ctx, BNA_INTERNAL, "density window missed the k-th value (k %lld, definite %lld, "
                  "candidates %lld)", k_dens, definite, n);
    std::vector<float> w(v);
    std::nth_element(w.begin(), w.begin() + (need - 1), w.end(), std::greater<float>());
    const float tau_star = w[need - 1];
    long long greater = definite;
    std::vector<unsigned long long> ties;
    for (long long c = 0; c < n; ++c) {
      if (v[c] > tau_star) ++greater;
      else if (v[c] == tau_star)
        ties.push_back(((unsigned long long)keys[c].x << 32) | keys[c].y);
    }
    const long long keep = k_dens - greater;
    if (keep < 0 || (double)tau_star < winA || (double)tau_star > winB)
      return fail(ctx, BNA_INTERNAL, "density: the k-th value lies outside its window");
    std::sort(ties.begin(), ties.end());
    std::vector<unsigned long long> drop(ties.begin() + std::min<long long>(keep, ties.size()),
                                         ties.end());
    std::sort(drop.begin(), drop.end());
    ties_dropped = (long long)drop.size();
    unsigned long long* dk = nullptr;
    ENSURE(S_DROP, std::max<size_t>(drop.size(), 1) * 8, dk);
    if (!drop.empty())
      CK(cudaMemcpyAsync(dk, drop.data(), drop.size() * 8, cudaMemcpyHostToDevice, st));
    a.drop_keys = dk;
    a.n_drop = (int)drop.size();
    a.th.mode = BNA_THR_DENSITY;
    a.th.tau = tau_star;
    a.cand_val = cvals;
    CK(launch_recompute(a, band_grid(ctx), st));
    ctx->klaunch += 1 + 4;  // decide, scan
    CK(cudaEventRecord(ctx->ev[3], st));
    CK(launch_csr_scan(a.seg, a.nb, a.n_pad, N, rowlen, pre, bsum, &ds->total, row_ptr, a.err,
                       st));
    CK(cudaEventRecord(ctx->ev[4], st));
    if (ctx->sink)
      CK(cudaMemcpyAsync(ctx->sink->row_ptr, row_ptr, (size_t)(N + 1) * 4,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hs, ds, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hs->err & ERR_HASH_FULL) return fail(ctx, BNA_INTERNAL, "candidate hash full");
    if (hs->total != 2 * k_dens)
      return fail(ctx, BNA_INTERNAL, "density: %lld entries instead of %lld", hs->total,
                  2 * k_dens);
  }
  if (hs->err & ERR_NNZ_INT32 || hs->total > 0x7fffffffLL)
    return fail(ctx, BNA_NNZ_OVERFLOW_INT32, "nnz %lld exceeds int32", hs->total);
  const long long nnz = hs->total;
  if (ctx->max_nnz > 0 && nnz > ctx->max_nnz) {
    if (stats) {
      std::memset(stats, 0, sizeof *stats);
      stats->nnz = nnz;
      stats->tau = (double)a.th.tau;
      stats->delta = delta;
    }
    return fail(ctx, BNA_CAPACITY, "CSR needs %lld entries, limit %lld", nnz, ctx->max_nnz);
  }
  const unsigned long long cand_count = hs->stats[3];  // candidates (not slots)
  const unsigned long long band_edges = hs->stats[0], band_1e6 = hs->stats[1];
  int32_t* col;
  ENSURE(S_COL, (size_t)std::max(nnz, 1LL) * 4, col);
  float* val = nullptr;
  if (a.weighted) ENSURE(S_VAL, (size_t)std::max(nnz, 1LL) * 4, val);
  a.row_ptr = row_ptr;
  a.col_idx = col;
  a.val = val;
  a.nnz = nnz;
  int* dense_list;
  ENSURE(S_DENSE, (size_t)nst * sizeof(int), dense_list);
  int fill_launches = 3;
  bna_ctx::Sink* sink = ctx->sink;
  if (sink && nnz <= sink->cap && (nnz == 0 || sink->col) && sink->row_ptr[N] == nnz) {
    // chunked fill, each chunk's entries copied out while the next fills
    if (!ctx->copy_stream) {
      CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
      for (auto& e : ctx->chunk_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    CK(launch_csr_fill_dense(a, ctx->sms, dense_list, &ds->dense, st));
    const int nch = std::min(kFillChunks, a.nb);
    for (int c = 0; c < nch; ++c) {
      const int I0 = (int)((long long)c * a.nb / nch), I1 = (int)((long long)(c + 1) * a.nb / nch);
      CK(launch_csr_fill_rows(a, ctx->sms, I0, I1, st));
      CK(cudaEventRecord(ctx->chunk_ev[c], st));
      CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->chunk_ev[c], 0));
      const long long e0 = sink->row_ptr[std::min(I0 * kBlk, N)];
      const long long e1 = sink->row_ptr[std::min(I1 * kBlk, N)];
      if (e1 > e0) {
        CK(cudaMemcpyAsync(sink->col + e0, col + e0, (size_t)(e1 - e0) * 4,
                           cudaMemcpyDeviceToHost, ctx->copy_stream));
        if (val && sink->val)
          CK(cudaMemcpyAsync(sink->val + e0, val + e0, (size_t)(e1 - e0) * 4,
                             cudaMemcpyDeviceToHost, ctx->copy_stream));
      }
    }
    CK(cudaEventRecord(ctx->chunk_ev[nch], ctx->copy_stream));
    CK(cudaStreamWaitEvent(st, ctx->chunk_ev[nch], 0));
    sink->done = true;
    fill_launches = 2 + nch;
  } else if (ctx->gate) {
    // row-block chunks with the gate between them
    CK(launch_csr_fill_dense(a, ctx->sms, dense_list, &ds->dense, st));
    const int nch = std::min(kFillChunks, a.nb);
    for (int c = 0; c < nch; ++c) {
      if (c > 0) gate(ctx, st, BNA_PHASE_FILL, (long long)c * a.nb / nch);
      CK(launch_csr_fill_rows(a, ctx->sms, (int)((long long)c * a.nb / nch),
                              (int)((long long)(c + 1) * a.nb / nch), st));
    }
    fill_launches = 2 + nch;
  } else {
    CK(launch_csr_fill(a, ctx->sms, dense_list, &ds->dense, st));
  }
  CK(cudaEventRecord(ctx->ev[5], st));
  CK(cudaMemcpyAsync(hs, ds, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (hs->err & ERR_HASH_MISS) return fail(ctx, BNA_INTERNAL, "fill pass missed a candidate");
  if (hs->err & ERR_RANGE) return fail(ctx, BNA_INTERNAL, "fill pass position out of range");
  out_dev->n = N;
  out_dev->nnz = nnz;
  out_dev->row_ptr = row_ptr;
  out_dev->col_idx = col;
  out_dev->val = val;
  ctx->last = a;
  ctx->last.th.delta = (float)delta;
  ctx->last_ok = !density && a.weighted && !ctx->avg;
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->tau = density && k_dens == 0 ? INFINITY : (double)a.th.tau;
    stats->delta = delta;
    stats->nnz = nnz;
    stats->band_candidates = (int64_t)cand_count;
    stats->band_edges = (int64_t)band_edges;
    stats->band_1e6 = (int64_t)band_1e6;
    stats->ties_dropped = ties_dropped;
    stats->passes = passes + (density && k_dens > 0 ? 1 : 0);
    stats->kernel_launches = ctx->klaunch + fill_launches;
    stats->precision = prec;
    stats->tile_band = prec != BNA_PREC_FP32 ? ctx->band_now : 0;
    cudaEventElapsedTime(&stats->ms_zscore, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&stats->ms_count, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&stats->ms_recompute, ctx->ev[2], ctx->ev[3]);
    cudaEventElapsedTime(&stats->ms_scan, ctx->ev[3], ctx->ev[4]);
    cudaEventElapsedTime(&stats->ms_fill, ctx->ev[4], ctx->ev[5]);
    cudaEventElapsedTime(&stats->ms_total, ctx->ev[0], ctx->ev[5]);
  }
  return BNA_OK;
}

int32_t bna_corr_csr_host(bna_ctx* ctx, const float* bold_host, int32_t N, int32_t T,
                          const bna_corr_opts* opts, bna_csr* out_host, bna_corr_stats* stats) {
  if (!ctx || !bold_host || !out_host || N < 1 || T < 1)
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_host: bad arguments");
  int32_t s = set_device(ctx);
  if (s) return s;
  float* bold;
  ENSURE(S_BOLD, (size_t)N * T * sizeof(float), bold);
  CK(cudaMemcpyAsync(bold, bold_host, (size_t)N * T * sizeof(float), cudaMemcpyHostToDevice,
                     nullptr));
  bna_csr d{};
  s = bna_corr_csr(ctx, bold, N, T, opts, &d, stats, nullptr);
  if (s) return s;
  out_host->n = N;
  out_host->nnz = d.nnz;
  out_host->row_ptr = (int32_t*)std::malloc((size_t)(N + 1) * 4);
  out_host->col_idx = (int32_t*)std::malloc((size_t)std::max<int64_t>(d.nnz, 1) * 4);
  out_host->val = d.val ? (float*)std::malloc((size_t)std::max<int64_t>(d.nnz, 1) * 4) : nullptr;
  if (!out_host->row_ptr || !out_host->col_idx || (d.val && !out_host->val)) {
    bna_csr_free_host(out_host);
    return fail(ctx, BNA_OOM, "host allocation failed");
  }
  CK(cudaMemcpyAsync(out_host->row_ptr, d.row_ptr, (size_t)(N + 1) * 4, cudaMemcpyDeviceToHost,
                     nullptr));
  if (d.nnz > 0) {
    CK(cudaMemcpyAsync(out_host->col_idx, d.col_idx, (size_t)d.nnz * 4, cudaMemcpyDeviceToHost,
                       nullptr));
    if (d.val)
      CK(cudaMemcpyAsync(out_host->val, d.val, (size_t)d.nnz * 4, cudaMemcpyDeviceToHost,
                         nullptr));
  }
  CK(cudaStreamSynchronize(nullptr));
  return BNA_OK;
}

int32_t bna_corr_csr_host_into(bna_ctx* ctx, const float* bold_host, int32_t N, int32_t T,
                               const bna_corr_opts* opts, int32_t* row_ptr_host,
                               int32_t* col_idx_host, float* val_host, int64_t cap,
                               int64_t* nnz_out, bna_corr_stats* stats) {
  if (!ctx || !bold_host || !opts || !row_ptr_host || N < 1 || T < 1 || cap < 0)
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_host_into: bad arguments");
  int32_t s = set_device(ctx);
  if (s) return s;
  float* bold;
  ENSURE(S_BOLD, (size_t)N * T * sizeof(float), bold);
  CK(cudaMemcpyAsync(bold, bold_host, (size_t)N * T * sizeof(float), cudaMemcpyHostToDevice,
                     nullptr));
  bna_csr d{};
  bna_ctx::Sink sink{row_ptr_host, col_idx_host, val_host, cap, false};
  ctx->sink = &sink;
  s = bna_corr_csr(ctx, bold, N, T, opts, &d, stats, nullptr);
  ctx->sink = nullptr;
  if (s) return s;
  if (nnz_out) *nnz_out = d.nnz;
  if (sink.done) return BNA_OK;  // copied chunk by chunk behind the fill pass
  CK(cudaMemcpyAsync(row_ptr_host, d.row_ptr, (size_t)(N + 1) * 4, cudaMemcpyDeviceToHost,
                     nullptr));
  if (d.nnz > cap) {
    CK(cudaStreamSynchronize(nullptr));
    return fail(ctx, BNA_CAPACITY, "%lld entries do not fit the %lld given", (long long)d.nnz,
                (long long)cap);
  }
  if (d.nnz > 0) {
    if (!col_idx_host) return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_host_into: col_idx is NULL");
    CK(cudaMemcpyAsync(col_idx_host, d.col_idx, (size_t)d.nnz * 4, cudaMemcpyDeviceToHost,
                       nullptr));
    if (d.val && val_host)
      CK(cudaMemcpyAsync(val_host, d.val, (size_t)d.nnz * 4, cudaMemcpyDeviceToHost, nullptr));
  }
  CK(cudaStreamSynchronize(nullptr));
  return BNA_OK;
}

void bna_csr_free_host(bna_csr* c) {
  if (!c) return;
  std::free(c->row_ptr);
  std::free(c->col_idx);
  std::free(c->val);
  c->row_ptr = nullptr;
  c->col_idx = nullptr;
  c->val = nullptr;
}

int32_t bna_corr_tile_values(bna_ctx* ctx, const float* bold_dev, int32_t N, int32_t T,
                             int32_t precision, int32_t I, int32_t J, float* out_dev,
                             void* stream) {
  if (!ctx || !bold_dev || !out_dev || N < 1 || T < 1)
    return fail(ctx, BNA_BAD_ARG, "bna_corr_tile_values: bad arguments");
  int32_t s = set_device(ctx, as_stream(stream));
  ctx->last_ok = false;  // the z-scores are rewritten
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  CorrArgs a{};
  s = run_zscore(ctx, bold_dev, N, T, precision == BNA_PREC_BF16X3, a, st);
  if (s) return s;
  if (I < 0 || J < 0 || I >= a.nb || J >= a.nb)
    return fail(ctx, BNA_BAD_ARG, "tile (%d, %d) outside the %d-block grid", I, J, a.nb);
  switch (precision) {
    case BNA_PREC_FP32: CK(launch_corr_simt_dump(a, I, J, out_dev, st)); break;
    case BNA_PREC_BF16X3:
    case BNA_PREC_TF32: {
      uint8_t* bb;
      ENSURE(S_BLOCKBAD, (size_t)a.nb, bb);
      CK(launch_block_bad(a.bad, a.nb, bb, st));
      int2* d;
      ENSURE(S_DUMPTILE, sizeof(int2), d);
      const int2 t = make_int2(I, J / 2);
      CK(cudaMemcpyAsync(d, &t, sizeof t, cudaMemcpyHostToDevice, st));
      CK(launch_corr_tc(a, 2, precision == BNA_PREC_BF16X3 ? 0 : 1, d, 1, bb, out_dev, J % 2, 1,
                        st));
      CK(cudaStreamSynchronize(st));
      break;
    }
    default: return fail(ctx, BNA_UNSUPPORTED, "precision %d is not built", precision);
  }
  return BNA_OK;
}

// The multi-subject sums: every subject's z-scores (kept in the arena for the
// exact recompute; their table goes to subj_dev) and pass 4 over all tiles,
// into packed / unc (zeroed here), then the division / inverse transform.
static int32_t avg_accumulate(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev,
                              int32_t N, const int32_t* T, int fisher, int prec, double delta_opt,
                              float* packed, uint32_t* unc, void** subj_dev_out, double* dsum,
                              cudaStream_t st) {
  const int n_pad = round_up(N, kBlk), nb = n_pad / kBlk;
  const long long M1 = (long long)N * (N - 1) / 2;
  size_t zoff_total = 0;
  int ldb_max = 0;
  std::vector<size_t> zoff(nsub);
  for (int k = 0; k < nsub; ++k) {
    zoff[k] = zoff_total;
    zoff_total += (size_t)n_pad * round_up(T[k], 32);
    ldb_max = std::max(ldb_max, round_up(T[k], 64));
  }
  float* zall;
  uint8_t* badall;
  void* subj_dev;
  void* vstat;
  uint16_t *zhi = nullptr, *zlo = nullptr;
  ENSURE(S_AVG_Z, zoff_total * sizeof(float), zall);
  ENSURE(S_AVG_BAD, (size_t)nsub * n_pad, badall);
  ENSURE(S_AVG_SUBJ, (size_t)nsub * avg_subj_bytes(), subj_dev);
  ENSURE(S_VSTAT, zscore_scratch_bytes(n_pad), vstat);
  if (prec == BNA_PREC_BF16X3) {
    ENSURE(S_ZHI, (size_t)n_pad * ldb_max * 2, zhi);
    ENSURE(S_ZLO, (size_t)n_pad * ldb_max * 2, zlo);
  }
  CK(cudaMemsetAsync(packed, 0, (size_t)M1 * sizeof(float), st));
  CK(cudaMemsetAsync(unc, 0, (size_t)((M1 + 31) / 32) * sizeof(uint32_t), st));
  std::vector<char> subj_host((size_t)nsub * avg_subj_bytes());
  *dsum = 0;
  for (int k = 0; k < nsub; ++k) {
    // subject k: z-scores, then its values added into the sums in file order
    CorrArgs as{};
    as.n = N;
    as.n_pad = n_pad;
    as.nb = nb;
    as.T = T[k];
    as.ldz = round_up(T[k], 32);
    as.ldb = round_up(T[k], 64);
    as.z = zall + zoff[k];
    as.zhi = zhi;
    as.zlo = zlo;
    as.bad = badall + (size_t)k * n_pad;
    CK(launch_zscore(bold_dev[k], N, T[k], n_pad, const_cast<float*>(as.z), as.ldz, zhi, zlo,
                     as.ldb, const_cast<uint8_t*>(as.bad), vstat, st));
    ctx->klaunch += 2;
    int32_t s = tc_prepare(ctx, as, st);
    if (s) return s;
    const double dk = delta_opt > 0 ? delta_opt : default_delta(prec, T[k]);
    *dsum += dk;
    as.th.mode = BNA_THR_R_GE;
    as.th.tau = 2.0f;
    as.th.delta = (float)dk;
    AvgPass ap{packed, unc, fisher ? 1 : 0, fisher ? 0.9f : (float)(1.0 - dk)};
    const int2* tiles = reinterpret_cast<const int2*>(ctx->ptr[S_TILES]);
    const int per = ctx->tiles_per_launch > 0 ? ctx->tiles_per_launch : ctx->ntiles;
    for (int t0 = 0; t0 < ctx->ntiles; t0 += per, ++ctx->klaunch)
      CK(launch_corr_tc(as, 4, prec == BNA_PREC_BF16X3 ? 0 : 1, tiles + t0,
                        std::min(per, ctx->ntiles - t0),
                        reinterpret_cast<const uint8_t*>(ctx->ptr[S_BLOCKBAD]), nullptr, 0,
                        ctx->sms, st, &ap));
    avg_subj_fill(subj_host.data(), k, as.z, as.bad, as.ldz, T[k]);
  }
  CK(cudaMemcpyAsync(subj_dev, subj_host.data(), subj_host.size(), cudaMemcpyHostToDevice, st));
  CK(launch_avg_finalize(packed, M1, nsub, fisher ? 1 : 0, ctx->sms, st));
  ctx->klaunch += 1;
  CK(cudaStreamSynchronize(st));  // subj_host is released at return
  *subj_dev_out = subj_dev;
  return BNA_OK;
}

static int32_t avg_check(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev, int32_t N,
                         const int32_t* T, int prec) {
  if (!ctx || nsub < 1 || !bold_dev || !T || N < 2)
    return fail(ctx, BNA_BAD_ARG, "multi-subject call: bad arguments");
  for (int k = 0; k < nsub; ++k)
    if (!bold_dev[k] || T[k] < 1)
      return fail(ctx, BNA_BAD_ARG, "subject %d: bad arguments", k);
  if (prec != BNA_PREC_BF16X3 && prec != BNA_PREC_TF32)
    return fail(ctx, BNA_UNSUPPORTED, "multi-subject call: a tensor-core form is required");
  return BNA_OK;
}

int32_t bna_corr_csr_avg(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev, int32_t N,
                         const int32_t* T, int32_t fisher, const bna_corr_opts* opts,
                         bna_csr* out_dev, bna_corr_stats* stats, void* stream) {
  if (!opts || !out_dev || !T || nsub < 1)
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_avg: bad arguments");
  int prec_r = opts->precision;
  int32_t s = resolve_precision(ctx, N, T[0], opts, &prec_r);
  if (s) return s;
  bna_corr_opts opts_r = *opts;
  opts_r.precision = prec_r;
  opts = &opts_r;
  s = avg_check(ctx, nsub, bold_dev, N, T, opts->precision);
  if (s) return s;
  if (!mode_known(opts->mode) ||
      (opts->mode == BNA_THR_DENSITY && !(opts->value >= 0.0 && opts->value <= 100.0)))
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_avg: bad threshold rule");
  if (opts->mode == BNA_THR_R_EPS)
    return fail(ctx, BNA_UNSUPPORTED, "bna_corr_csr_avg: the 2mm tools' rule has no average");
  const int prec = opts->precision;
  s = set_device(ctx, as_stream(stream));
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  ctx->klaunch = 0;
  ctx->last_ok = false;
  const int n_pad = round_up(N, kBlk), nb = n_pad / kBlk;
  const long long M1 = (long long)N * (N - 1) / 2;
  float* packed;
  uint32_t* unc;
  uint8_t* badz;
  ENSURE(S_AVG_PACKED, (size_t)M1 * sizeof(float), packed);
  ENSURE(S_AVG_UNC, (size_t)((M1 + 31) / 32) * sizeof(uint32_t), unc);
  ENSURE(S_AVG_BADZ, (size_t)n_pad, badz);
  CK(cudaMemsetAsync(badz, 0, (size_t)n_pad, st));
  CK(cudaEventRecord(ctx->ev[0], st));
  void* subj_dev = nullptr;
  double dsum = 0;
  s = avg_accumulate(ctx, nsub, bold_dev, N, T, fisher, prec, opts->delta, packed, unc,
                     &subj_dev, &dsum, st);
  if (s) return s;
  CK(cudaEventRecord(ctx->ev[1], st));
  // bound of |average~ - average| (per-subject bounds, the float sums and
  // division; with Fisher z the transform's slope below |r| = 0.91, larger
  // |r~| being uncertain pairs that are always recomputed)
  const double dmean = dsum / nsub;
  const double u24 = std::ldexp(1.0, -24);
  const double davg = fisher ? 6.0 * dmean + 4e-6 + (nsub + 2) * 4.0 * u24
                             : dmean + (nsub + 1) * u24 + 4.0 * u24;
  CorrArgs a{};
  a.n = N;
  a.n_pad = n_pad;
  a.nb = nb;
  a.T = 1;
  a.ldz = 32;
  a.bad = badz;
  a.avg_packed = packed;
  a.avg_unc = unc;
  const bna_ctx::Avg ac{subj_dev, nsub, fisher ? 1 : 0};
  ctx->avg = &ac;
  s = corr_csr_core(ctx, a, N, 1, opts, prec, davg, out_dev, stats, st);
  ctx->avg = nullptr;
  return s;
}

int32_t bna_corr_packed(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev, int32_t N,
                        const int32_t* T, int32_t fisher, int32_t precision, float* packed_dev,
                        void* stream) {
  int32_t s = avg_check(ctx, nsub, bold_dev, N, T, precision);
  if (s) return s;
  if (!packed_dev) return fail(ctx, BNA_BAD_ARG, "bna_corr_packed: packed_dev is NULL");
  s = set_device(ctx, as_stream(stream));
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  ctx->klaunch = 0;
  ctx->last_ok = false;
  const long long M1 = (long long)N * (N - 1) / 2;
  uint32_t* unc;
  ENSURE(S_AVG_UNC, (size_t)((M1 + 31) / 32) * sizeof(uint32_t), unc);
  void* subj_dev = nullptr;
  double dsum = 0;
  return avg_accumulate(ctx, nsub, bold_dev, N, T, fisher, precision, 0.0, packed_dev, unc,
                        &subj_dev, &dsum, st);
}

// ---------------------------------------------------------------- batches

namespace {

// One subject of a batch (its arguments live in its own context's arena).
struct BatchSubj {
  CorrArgs a{};
  int N = 0, T = 0;
  double delta = 0, winA = 0, winB = 0;
  long long k_dens = 0;
  bool sampled = false;
  bool fallback = false;
  DevStatus* ds = nullptr;
  long long *rowlen = nullptr, *pre = nullptr, *bsum = nullptr;
  int32_t* row_ptr = nullptr;
  float* cvals = nullptr;
  void* dstate = nullptr;
  unsigned int *dhist = nullptr;
  uint8_t* dcls = nullptr;
  int* deidx = nullptr;
  float* dexact = nullptr;
  unsigned long long* dties = nullptr;
  long long nnz = 0;
};

// z-scores, buffers and (density) the histogram pass of one subject.
int32_t batch_prep(bna_ctx* ctx, BatchSubj& b, const float* bold, const bna_corr_opts* opts,
                   int prec, unsigned int* hist_host, cudaStream_t st) {
  int32_t s = set_device(ctx, st);
  if (s) return s;
  ctx->klaunch = 0;
  ctx->last_ok = false;
  CorrArgs& a = b.a;
  a = CorrArgs{};
  s = run_zscore(ctx, bold, b.N, b.T, prec == BNA_PREC_BF16X3, a, st);
  if (s) return s;
  s = tc_prepare(ctx, a, st);
  if (s) return s;
  b.delta = opts->delta > 0 ? opts->delta : default_delta(prec, b.T);
  a.weighted = opts->weighted ? 1 : 0;
  ENSURE(S_SEG, (size_t)a.nb * a.n_pad * sizeof(int32_t), a.seg);
  ENSURE(S_ROWLEN, (size_t)a.n_pad * 8, b.rowlen);
  ENSURE(S_PRE, (size_t)a.n_pad * 8, b.pre);
  ENSURE(S_BSUM, (size_t)4096 * 8, b.bsum);
  ENSURE(S_ROWPTR, (size_t)(b.N + 1) * 4, b.row_ptr);
  ENSURE(S_STATUS, sizeof(DevStatus), b.ds);
  a.err = &b.ds->err;
  a.cand_count = &b.ds->cand_count;
  a.stats = b.ds->stats;
  a.epool = &b.ds->epool;
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  ENSURE(S_ETAB, (size_t)nst * 4 * sizeof(longlong2), a.etab);
  const bool density = opts->mode == BNA_THR_DENSITY;
  b.k_dens = density ? bna_density_nnz(b.N, opts->value) / 2 : 0;
  if (!density) {
    a.th.mode = opts->mode;
    a.th.tau = rule_tau(opts);
    a.th.delta = (float)b.delta;
  } else if (b.k_dens == 0) {
    a.th.mode = BNA_THR_R_GT;
    a.th.tau = 2.0f;
    a.th.delta = (float)b.delta;
  } else {
    unsigned int* hist;
    ENSURE(S_HIST, (kHistBins + 1) * sizeof(unsigned int), hist);
    CK(cudaMemsetAsync(hist, 0, (kHistBins + 1) * sizeof(unsigned int), st));
    a.hist = hist;
    a.th.mode = BNA_THR_R_GE;
    a.th.tau = 0.0f;
    a.th.delta = (float)b.delta;
    b.sampled = ctx->ntiles >= 4 * kSampleTiles;
    s = corr_pass(ctx, a, prec, 3, st, b.sampled);
    if (s) return s;
    CK(cudaMemcpyAsync(hist_host, hist, (kHistBins + 1) * sizeof(unsigned int),
                       cudaMemcpyDeviceToHost, st));
  }
  return BNA_OK;
}

// Count pass buffers of one subject (cleared for the pass).
int32_t batch_buffers(bna_ctx* ctx, BatchSubj& b, bool dev_sel, cudaStream_t st) {
  CorrArgs& a = b.a;
  a.cand_cap = ctx->cand_cap;
  a.echunk = elist_chunk(ctx, a);
  const long long min_pool = (long long)ctx->sms * 8 * 2 * a.echunk;
  if (ctx->elist_cap < min_pool) ctx->elist_cap = min_pool;
  a.ecap = ctx->elist_cap;
  const unsigned long long hcap = next_pow2((unsigned long long)a.cand_cap * 2);
  a.hmask = hcap - 1;
  ENSURE(S_CAND, (size_t)a.cand_cap * sizeof(uint2), a.cand);
  ENSURE(S_HKEYS, hcap * 8, a.hkeys);
  ENSURE(S_HVAL, hcap * 4, a.hval);
  ENSURE(S_HEDGE, hcap, a.hedge);
  ENSURE(S_ELIST, (size_t)a.ecap * sizeof(uint2), a.elist);
  ENSURE(S_CANDVAL, (size_t)a.cand_cap * sizeof(float), b.cvals);
  a.cand_apx = nullptr;
  if (dev_sel) {
    ENSURE(S_CANDAPX, (size_t)a.cand_cap * sizeof(float), a.cand_apx);
    ENSURE(S_DSTATE, dens_state_bytes(), b.dstate);
    ENSURE(S_DHIST, 2048 * sizeof(unsigned int), b.dhist);
    ENSURE(S_DCLS, (size_t)a.cand_cap, b.dcls);
    ENSURE(S_DEIDX, (size_t)a.cand_cap * sizeof(int), b.deidx);
    ENSURE(S_DEXACT, (size_t)a.cand_cap * sizeof(float), b.dexact);
    ENSURE(S_DTIES, 2 * dens_ties_cap() * sizeof(unsigned long long), b.dties);
  }
  const int nwarps = ctx->sms * 8;
  ENSURE(S_WSTATE, (size_t)nwarps * 4 * sizeof(long long), a.wstate);
  CK(cudaMemsetAsync(b.ds, 0, sizeof(DevStatus), st));
  CK(cudaMemsetAsync(a.hkeys, 0xff, hcap * 8, st));
  CK(cudaMemsetAsync(a.wstate, 0, (size_t)nwarps * 4 * sizeof(long long), st));
  return BNA_OK;
}

// After the count pass: candidates, density selection or recompute, scan.
int32_t batch_after(bna_ctx* ctx, BatchSubj& b, bool dev_sel, cudaStream_t st) {
  CorrArgs& a = b.a;
  CK(launch_seal_candidates(a, ctx->sms * 8, st));
  if (dev_sel) {
    CK(dens_set(b.dstate, b.k_dens, (float)b.delta, b.winA, b.winB, st));
    CK(cudaMemsetAsync(b.dhist, 0, 2048 * sizeof(unsigned int), st));
    CK(launch_density_select(a, b.dstate, b.dhist, b.dcls, b.deidx, b.dexact, b.cvals, b.dties,
                             b.dties + dens_ties_cap(), ctx->sms, st));
    CK(cudaMemcpyAsync(static_cast<char*>(ctx->pinned) + 2048, b.dstate, dens_state_bytes(),
                       cudaMemcpyDeviceToHost, st));
  } else {
    CK(launch_recompute(a, band_grid(ctx), st));
  }
  CK(launch_csr_scan(a.seg, a.nb, a.n_pad, b.N, b.rowlen, b.pre, b.bsum, &b.ds->total, b.row_ptr,
                     a.err, st));
  CK(cudaMemcpyAsync(ctx->pinned, b.ds, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
  return BNA_OK;
}

// CSR arrays and the fill pass of one subject.
int32_t batch_fill(bna_ctx* ctx, BatchSubj& b, cudaStream_t st) {
  CorrArgs& a = b.a;
  int32_t* col;
  ENSURE(S_COL, (size_t)std::max(b.nnz, 1LL) * 4, col);
  float* val = nullptr;
  if (a.weighted) ENSURE(S_VAL, (size_t)std::max(b.nnz, 1LL) * 4, val);
  a.row_ptr = b.row_ptr;
  a.col_idx = col;
  a.val = val;
  a.nnz = b.nnz;
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  int* dense_list;
  ENSURE(S_DENSE, (size_t)nst * sizeof(int), dense_list);
  CK(launch_csr_fill(a, ctx->sms, dense_list, &b.ds->dense, st));
  CK(cudaMemcpyAsync(ctx->pinned, b.ds, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
  return BNA_OK;
}

}  // namespace

int32_t bna_corr_csr_batch(bna_ctx* ctx, int32_t nsub, const float* const* bold_dev,
                           const int32_t* N, const int32_t* T, const bna_corr_opts* opts,
                           bna_csr* out_dev, bna_corr_stats* stats, void* stream) {
  if (!ctx || nsub < 1 || !bold_dev || !N || !T || !opts || !out_dev)
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_batch: bad arguments");
  for (int k = 0; k < nsub; ++k)
    if (!bold_dev[k] || N[k] < 1 || T[k] < 1)
      return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_batch: subject %d: bad arguments", k);
  if (!mode_known(opts->mode) ||
      opts->precision < BNA_PREC_FP32 || opts->precision > BNA_PREC_AUTO ||
      (opts->mode == BNA_THR_DENSITY && !(opts->value >= 0.0 && opts->value <= 100.0)))
    return fail(ctx, BNA_BAD_ARG, "bna_corr_csr_batch: bad options");
  // one form for the batch: the autotuner's choice for its largest subject
  int kmax = 0;
  for (int k = 1; k < nsub; ++k)
    if ((double)N[k] * N[k] * T[k] > (double)N[kmax] * N[kmax] * T[kmax]) kmax = k;
  int prec_r = opts->precision;
  int32_t s = resolve_precision(ctx, N[kmax], T[kmax], opts, &prec_r);
  if (s) return s;
  bna_corr_opts opts_r = *opts;
  opts_r.precision = prec_r;
  opts = &opts_r;
  s = set_device(ctx, as_stream(stream));
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  while ((int)ctx->kids.size() < nsub) {
    bna_ctx* k = nullptr;
    s = bna_ctx_create(ctx->device, &k);
    if (s) return fail(ctx, s, "bna_corr_csr_batch: context for a subject");
    ctx->kids.push_back(k);
  }
  const int prec = opts->precision;
  auto single = [&](int k) -> int32_t {  // the one-subject path (retries, fallbacks)
    bna_ctx* kid = ctx->kids[k];
    kid->tiles_per_launch = ctx->tiles_per_launch;
    kid->band = kid->band_now = ctx->band_now;
    const int32_t r = bna_corr_csr(kid, bold_dev[k], N[k], T[k], opts, &out_dev[k],
                                   stats ? &stats[k] : nullptr, stream);
    if (r) return fail(ctx, r, "subject %d: %s", k, kid->last_error.c_str());
    return BNA_OK;
  };
  if (prec == BNA_PREC_FP32) {  // the plain form has no multi-subject pass
    for (int k = 0; k < nsub; ++k)
      if ((s = single(k))) return s;
    return BNA_OK;
  }
  const bool density = opts->mode == BNA_THR_DENSITY;
  const bool absm = opts->mode == BNA_THR_ABS_GT || opts->mode == BNA_THR_ABS_GE;
  CK(cudaEventRecord(ctx->ev[0], st));
  // ---- z-scores, buffers, density histograms (one synchronisation)
  const size_t hbins = kHistBins + 1;
  if (density && ctx->hist_host_cap < hbins * nsub) {
    if (ctx->hist_host) cudaFreeHost(ctx->hist_host);
    ctx->hist_host = nullptr;
    ctx->hist_host_cap = 0;
    CK(cudaMallocHost(&ctx->hist_host, hbins * nsub * sizeof(unsigned int)));
    ctx->hist_host_cap = hbins * nsub;
  }
  std::vector<BatchSubj> bs(nsub);
  for (int k = 0; k < nsub; ++k) {
    bs[k].N = N[k];
    bs[k].T = T[k];
    s = batch_prep(ctx->kids[k], bs[k], bold_dev[k], opts, prec,
                   density ? ctx->hist_host + hbins * k : nullptr, st);
    if (s) return fail(ctx, s, "subject %d: %s", k, ctx->kids[k]->last_error.c_str());
  }
  CK(cudaStreamSynchronize(st));
  for (int k = 0; k < nsub; ++k)
    if (density && bs[k].k_dens > 0)
      window_from_hist(ctx->hist_host + hbins * k, bs[k].k_dens, bs[k].sampled, N[k],
                       bs[k].delta, &bs[k].winA, &bs[k].winB, &bs[k].a.th);
  // ---- one persistent count pass over the tiles of every subject
  const bool dev_sel = density;
  std::vector<char> table((size_t)nsub * tc_subj_bytes());
  for (int k = 0; k < nsub; ++k) {
    bna_ctx* kid = ctx->kids[k];
    s = batch_buffers(kid, bs[k], dev_sel, st);  // the density count pass lists r~ for all
    if (s) return fail(ctx, s, "subject %d: %s", k, kid->last_error.c_str());
    if (!tc_subj_fill(table.data(), k, bs[k].a,
                      reinterpret_cast<const uint8_t*>(kid->ptr[S_BLOCKBAD]),
                      prec == BNA_PREC_BF16X3 ? 0 : 1))
      return fail(ctx, BNA_INTERNAL, "subject %d: operand map", k);
  }
  std::vector<int> nbs(nsub);
  for (int k = 0; k < nsub; ++k) nbs[k] = bs[k].a.nb;
  if (nbs != ctx->batch_nb || ctx->batch_band != ctx->band_now) {
    std::vector<int4> t4;
    for (int k = 0; k < nsub; ++k) {
      std::vector<int2> t;
      tc_tile_list(nbs[k], ctx->band_now, t);
      for (const int2& x : t) t4.push_back(make_int4(x.x, x.y, k, 0));
    }
    int4* d;
    ENSURE(S_BATCH_TILES, t4.size() * sizeof(int4), d);
    CK(cudaMemcpyAsync(d, t4.data(), t4.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    ctx->batch_nb = nbs;
    ctx->batch_band = ctx->band_now;
    ctx->batch_ntiles = (int)t4.size();
  }
  void* table_dev;
  ENSURE(S_BATCH_SUBJ, table.size(), table_dev);
  CK(cudaMemcpyAsync(table_dev, table.data(), table.size(), cudaMemcpyHostToDevice, st));
  DevStatus* bst;
  ENSURE(S_STATUS, sizeof(DevStatus), bst);
  CK(cudaMemsetAsync(bst, 0, sizeof(DevStatus), st));
  CorrArgs batch{};
  batch.err = &bst->err;
  const int4* tiles4 = reinterpret_cast<const int4*>(ctx->ptr[S_BATCH_TILES]);
  const int per = ctx->tiles_per_launch > 0 ? ctx->tiles_per_launch : ctx->batch_ntiles;
  const int form = prec == BNA_PREC_BF16X3 ? 0 : 1;
  int launches = 0;
  // the persistent count pass over every subject's tiles, replayed from a
  // captured CUDA graph (one launch, or the chunks a launch gate asks for)
  CK(prepare_corr_tc_multi(form, dev_sel, absm));  // its attributes: outside the capture
  struct ExecGuard {  // released once its launch is over, on every return path
    cudaGraphExec_t e = nullptr;
    cudaStream_t s = nullptr;
    ~ExecGuard() {
      if (e) {
        cudaStreamSynchronize(s);
        cudaGraphExecDestroy(e);
      }
    }
  } guard;
  guard.s = st;
  cudaGraphExec_t& count_exec = guard.e;
  {
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    for (int t0 = 0; ce == cudaSuccess && t0 < ctx->batch_ntiles; t0 += per, ++launches)
      ce = launch_corr_tc_multi(batch, table_dev, tiles4 + t0,
                                std::min(per, ctx->batch_ntiles - t0), form, dev_sel, absm,
                                ctx->sms, cap);
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(cap, &graph);
    if (ce == cudaSuccess) ce = ee;
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&count_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    CK(ce);
  }
  CK(cudaGraphLaunch(count_exec, st));
  CK(cudaEventRecord(ctx->ev[2], st));
  // ---- candidates, selection / recompute, scans (one synchronisation)
  for (int k = 0; k < nsub; ++k) {
    s = batch_after(ctx->kids[k], bs[k], dev_sel && bs[k].k_dens > 0, st);
    if (s) return fail(ctx, s, "subject %d: %s", k, ctx->kids[k]->last_error.c_str());
  }
  CK(cudaMemcpyAsync(ctx->pinned, bst, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
  const cudaError_t se = cudaStreamSynchronize(st);
  cudaGraphExecDestroy(count_exec);  // its launch has completed
  count_exec = nullptr;
  CK(se);
  if (reinterpret_cast<DevStatus*>(ctx->pinned)->err & ERR_TIMEOUT)
    return fail(ctx, BNA_TIMEOUT, "batch count pass: a bounded wait expired");
  for (int k = 0; k < nsub; ++k) {
    bna_ctx* kid = ctx->kids[k];
    const DevStatus* hs = reinterpret_cast<const DevStatus*>(kid->pinned);
    BatchSubj& b = bs[k];
    bool bad = (hs->err & (ERR_BAND_OVERFLOW | ERR_HASH_FULL | ERR_ELIST | ERR_TIMEOUT)) != 0;
    if (hs->err & (ERR_BAND_OVERFLOW | ERR_HASH_FULL))
      kid->cand_cap = (long long)(hs->cand_count * 3 / 2) + 1024;
    if (hs->err & ERR_ELIST)
      kid->elist_cap = (long long)(hs->epool + hs->epool / 4) + b.a.echunk;
    if (!bad && dev_sel && b.k_dens > 0) {
      int derr = 0, n_drop = 0;
      float tau = 0;
      long long ne = 0, nt = 0;
      dens_state_read(static_cast<char*>(kid->pinned) + 2048, &derr, &tau, &ne, &nt, &n_drop);
      bad = derr != 0 || hs->total != 2 * b.k_dens;
      b.a.th.mode = BNA_THR_DENSITY;
      b.a.th.tau = tau;
    }
    if (!bad && (hs->err & ERR_NNZ_INT32 || hs->total > 0x7fffffffLL)) bad = true;
    if (!bad && kid->max_nnz > 0 && hs->total > kid->max_nnz) bad = true;
    b.fallback = bad;
    b.nnz = hs->total;
    if (stats && !bad) {
      bna_corr_stats& o = stats[k];
      std::memset(&o, 0, sizeof o);
      o.tau = density && b.k_dens == 0 ? INFINITY : (double)b.a.th.tau;
      o.delta = b.delta;
      o.nnz = b.nnz;
      o.band_candidates = (int64_t)hs->stats[3];
      o.band_edges = (int64_t)hs->stats[0];
      o.band_1e6 = (int64_t)hs->stats[1];
      o.passes = 1 + (density && b.k_dens > 0 ? 1 : 0);
      o.precision = prec;
      o.tile_band = ctx->band_now;
    }
  }
  // ---- fill (one synchronisation)
  for (int k = 0; k < nsub; ++k) {
    if (bs[k].fallback) continue;
    s = batch_fill(ctx->kids[k], bs[k], st);
    if (s) return fail(ctx, s, "subject %d: %s", k, ctx->kids[k]->last_error.c_str());
  }
  CK(cudaEventRecord(ctx->ev[5], st));
  CK(cudaStreamSynchronize(st));
  float ms_total = 0, ms_count = 0;
  cudaEventElapsedTime(&ms_total, ctx->ev[0], ctx->ev[5]);
  cudaEventElapsedTime(&ms_count, ctx->ev[0], ctx->ev[2]);
  for (int k = 0; k < nsub; ++k) {
    BatchSubj& b = bs[k];
    if (!b.fallback) {
      const DevStatus* hs = reinterpret_cast<const DevStatus*>(ctx->kids[k]->pinned);
      if (hs->err & (ERR_HASH_MISS | ERR_RANGE)) b.fallback = true;
    }
    if (b.fallback) {
      if ((s = single(k))) return s;
      continue;
    }
    out_dev[k].n = N[k];
    out_dev[k].nnz = b.nnz;
    out_dev[k].row_ptr = b.row_ptr;
    out_dev[k].col_idx = b.a.col_idx;
    out_dev[k].val = b.a.val;
    if (stats) {
      stats[k].ms_total = ms_total;  // the whole batch
      stats[k].ms_count = ms_count;
      stats[k].kernel_launches = ctx->kids[k]->klaunch + (k == 0 ? launches : 0) +
                                 (dev_sel ? 1 + 18 + 4 : 1 + 1 + 4) + 2;
    }
  }
  return BNA_OK;
}

int32_t bna_csr_rethreshold(bna_ctx* ctx, const bna_csr* in_dev, int32_t mode, double tau,
                            bna_csr* out_dev, int64_t* band_1e6, void* stream) {
  if (!ctx || !in_dev || !out_dev || !in_dev->row_ptr || (in_dev->nnz > 0 && !in_dev->val))
    return fail(ctx, BNA_BAD_ARG, "bna_csr_rethreshold: bad arguments (a weighted CSR is needed)");
  if (!ctx->last_ok || in_dev->n != ctx->last.n)
    return fail(ctx, BNA_BAD_ARG, "bna_csr_rethreshold: the CSR must come from this context's "
                "last bna_corr_csr (threshold rule, weighted)");
  const int m0 = ctx->last.th.mode;
  const bool abs0 = m0 == BNA_THR_ABS_GT || m0 == BNA_THR_ABS_GE;
  const bool abs1 = mode == BNA_THR_ABS_GT || mode == BNA_THR_ABS_GE;
  if (mode < BNA_THR_R_GT || mode > BNA_THR_ABS_GE || abs0 != abs1 ||
      (float)tau < ctx->last.th.tau)
    return fail(ctx, BNA_BAD_ARG, "bna_csr_rethreshold: the rule must be of the same kind and "
                "tau not below the built one");
  int32_t s = set_device(ctx, as_stream(stream));
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  const int N = in_dev->n;
  const long long nnz_in = in_dev->nnz;
  CorrArgs a = ctx->last;
  Threshold th{mode, (float)tau, ctx->last.th.delta};
  uint8_t* keep;
  float* valx;
  long long *rowlen, *pre, *bsum;
  int32_t* rp2;
  DevStatus* ds;
  ENSURE(S_RT_KEEP, (size_t)std::max(nnz_in, 1LL), keep);
  ENSURE(S_RT_VALX, (size_t)std::max(nnz_in, 1LL) * 4, valx);
  ENSURE(S_ROWLEN, (size_t)round_up(N, kBlk) * 8, rowlen);
  ENSURE(S_PRE, (size_t)round_up(N, kBlk) * 8, pre);
  ENSURE(S_BSUM, (size_t)4096 * 8, bsum);
  ENSURE(S_RT_ROWPTR, (size_t)(N + 1) * 4, rp2);
  ENSURE(S_STATUS, sizeof(DevStatus), ds);
  CK(cudaMemsetAsync(ds, 0, sizeof(DevStatus), st));
  CK(launch_rethr_count(a, in_dev->row_ptr, in_dev->col_idx, in_dev->val, th, keep, valx, rowlen,
                        &ds->stats[1], ctx->sms, st));
  CK(launch_rowlen_scan(rowlen, N, pre, bsum, &ds->total, rp2, &ds->err, st));
  DevStatus* hs = reinterpret_cast<DevStatus*>(ctx->pinned);
  CK(cudaMemcpyAsync(hs, ds, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const long long nnz = hs->total;
  int32_t* ci2;
  float* va2;
  ENSURE(S_RT_COL, (size_t)std::max(nnz, 1LL) * 4, ci2);
  ENSURE(S_RT_VAL, (size_t)std::max(nnz, 1LL) * 4, va2);
  CK(launch_rethr_fill(N, in_dev->row_ptr, in_dev->col_idx, valx, keep, rp2, ci2, va2, nnz,
                       &ds->err, ctx->sms, st));
  CK(cudaMemcpyAsync(hs, ds, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (hs->err & ERR_RANGE) return fail(ctx, BNA_INTERNAL, "rethreshold: position out of range");
  out_dev->n = N;
  out_dev->nnz = nnz;
  out_dev->row_ptr = rp2;
  out_dev->col_idx = ci2;
  out_dev->val = va2;
  if (band_1e6) *band_1e6 = (int64_t)hs->stats[1];
  return BNA_OK;
}

// ---------------------------------------------------------------- centrality

static int32_t ec_run(bna_ctx* ctx, int n, const int32_t* rp, const int32_t* ci, const float* val,
                      const double* vald, long long nnz, int max_iter, double eps, double* ec_dev,
                      double* lambda, int32_t* iters, cudaStream_t st) {
  const long long nnz_used = 2 * (nnz / 2);  // weighted-net.cu:61
  double *u, *parts;
  void* state;
  // two double iterates, then their two (hi, lo) float copies
  ENSURE(S_EC_U, (size_t)2 * n * (sizeof(double) + sizeof(float2)), u);
  float2* uf = reinterpret_cast<float2*>(u + (size_t)2 * n);
  const int grid = std::max(1, ctx->sms * 4);
  ENSURE(S_EC_PARTS, (size_t)grid * 6 * sizeof(double), parts);
  ENSURE(S_EC_STATE, ec_state_bytes(), state);
  CK(cudaMemsetAsync(state, 0, ec_state_bytes(), st));
  CK(launch_ec_init(n, u, uf, parts, state, grid, max_iter, st));
  // the whole iteration as one cooperative persistent launch
  const int cgrid = ec_coop_grid(n, ctx->sms);
  if (cgrid > 0) {
    // one launch; with a launch gate, segments of about a millisecond of
    // iterations (each resumes from the state block) with the gate between
    int seg = std::max(max_iter, 1);
    if (ctx->ec_seg > 0) {
      seg = ctx->ec_seg;
    } else if (ctx->gate) {
      const double iter_us = std::max(10.0, (8.0 * (double)nnz_used + 16.0 * n) / 2.0e6);
      seg = (int)std::max(2.0, 1000.0 / iter_us);
    }
    double lam2 = 0, lam = 0, e1 = 0, e2 = 0;
    int it = 0, done = 0;
    for (long long it_end = std::min(seg, max_iter);; it_end += seg) {
      if (it > 0) gate(ctx, st, BNA_PHASE_EC, it);
      CK(launch_ec_coop(n, rp, ci, val, vald, nnz_used, u, uf, parts, state, cgrid,
                        (int)std::min<long long>(it_end, max_iter), max_iter, eps, st));
      CK(cudaMemcpyAsync(ctx->pinned, state, ec_state_bytes(), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (ec_state_err(ctx->pinned))
        return fail(ctx, BNA_TIMEOUT, "centrality: a bounded grid barrier expired");
      ec_state_read(ctx->pinned, &lam2, &lam, &e1, &e2, &it, &done);
      if (done || it >= max_iter) break;
    }
    CK(cudaMemcpyAsync(ec_dev, u + (size_t)(it & 1) * n, (size_t)n * sizeof(double),
                       cudaMemcpyDeviceToDevice, st));
    if (lambda) *lambda = lam;
    if (iters) *iters = it;
    return (e1 <= eps || e2 <= eps) ? BNA_OK : BNA_NOT_CONVERGED;
  }
  // otherwise: a captured graph of per-iteration launches, kGraphIters of
  // them (with a launch gate: about a millisecond of iterations, estimated
  // from the CSR bytes an iteration streams at ~2 TB/s, so the gate runs
  // that often)
  int giters = kGraphIters;
  if (ctx->ec_seg > 0) {
    giters = std::min(ctx->ec_seg + (ctx->ec_seg & 1), 1 << 12);
  } else if (ctx->gate) {
    const double iter_us = (8.0 * (double)nnz_used + 16.0 * n) / 2.0e6;
    giters = (int)std::max(1.0, std::min((double)kGraphIters, 1000.0 / std::max(iter_us, 1.0)));
    // even: iteration it of a replay reads buffer it & 1, so every replay
    // must end on the buffer the next one starts from
    giters = std::max(2, giters & ~1);
  }
  EcGraph& g = ctx->ecg;
  const void* key[6] = {rp, ci, val, vald, u, state};
  bool same = g.exec && g.n == n && g.grid == grid && g.max_iter == max_iter && g.eps == eps &&
              g.nnz_used == nnz_used && g.iters == giters;
  for (int k = 0; k < 6 && same; ++k) same = (g.key[k] == key[k]);
  if (!same) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = EcGraph();
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < giters; ++it) {
      const size_t cur = (size_t)(it & 1) * n, nxt = (size_t)((it + 1) & 1) * n;
      launch_ec_iter(n, rp, ci, val, vald, nnz_used, u + cur, uf + cur, u + nxt, uf + nxt, parts,
                     state, grid, max_iter, eps, cap);
    }
    cudaGraph_t graph;
    cudaError_t ce = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    CK(ce);
    ce = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ce);
    for (int k = 0; k < 6; ++k) g.key[k] = key[k];
    g.n = n;
    g.grid = grid;
    g.max_iter = max_iter;
    g.eps = eps;
    g.nnz_used = nnz_used;
    g.iters = giters;
  }
  double lam2 = 0, lam = 0, e1 = 0, e2 = 0;
  int it = 0, done = 0;
  for (int launched = 0; launched < max_iter; launched += giters) {
    if (launched > 0) gate(ctx, st, BNA_PHASE_EC, it);
    CK(cudaGraphLaunch(g.exec, st));
    CK(cudaMemcpyAsync(ctx->pinned, state, ec_state_bytes(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ec_state_read(ctx->pinned, &lam2, &lam, &e1, &e2, &it, &done);
    if (done) break;
  }
  if (max_iter <= 0) {
    CK(cudaMemcpyAsync(ctx->pinned, state, ec_state_bytes(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ec_state_read(ctx->pinned, &lam2, &lam, &e1, &e2, &it, &done);
  }
  // iterate k writes buffer (k+1)&1, so the last iterate sits in buffer it&1
  CK(cudaMemcpyAsync(ec_dev, u + (size_t)(it & 1) * n, (size_t)n * sizeof(double),
                     cudaMemcpyDeviceToDevice, st));
  if (lambda) *lambda = lam;
  if (iters) *iters = it;
  const bool converged = (e1 <= eps || e2 <= eps);
  return converged ? BNA_OK : BNA_NOT_CONVERGED;
}

// ---------------------------------------------------------------- modularity

// Partition (Modularity_CPU.cpp:173-240) as a breadth-first walk of the
// division tree: the rounds of one level are the labels created by the
// previous level, [lo, maxres]; they run together in one cooperative launch
// (several when the level holds more groups than fit), then the host takes
// their decisions in round order — numbering the children as the sequential
// loop does — and a kernel writes the children's labels.
int32_t bna_modularity(bna_ctx* ctx, const bna_csr* csr, double lambda_min, int32_t* labels_dev,
                       int32_t* modules, double* q, bna_mod_round* log, int32_t log_cap,
                       int32_t* log_n, void* stream) {
  if (!ctx || !csr || !labels_dev || !modules || !q || csr->n < 1 || !csr->row_ptr ||
      (csr->nnz > 0 && !csr->col_idx) || (log_cap > 0 && !log) || log_cap < 0)
    return fail(ctx, BNA_BAD_ARG, "bna_modularity: bad arguments");
  if (log_n) *log_n = 0;
  int32_t s = set_device(ctx, as_stream(stream));
  if (s) return s;
  cudaStream_t st = as_stream(stream);
  const int n = csr->n;
  const int32_t* rp = csr->row_ptr;
  const int32_t* ci = csr->col_idx;
  const double lam_min = lambda_min > 0 ? lambda_min : 0.001;  // Modularity_CPU.cpp:19
  std::vector<int32_t> R((size_t)n + 1);
  CK(cudaMemcpyAsync(R.data(), rp, R.size() * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const long long M = ((long long)R[n] - R[0]) / 2;  // (:175)
  if (M == 0) {  // no edge: one module; the reference's Q is 0 / 0
    std::vector<int32_t> ones(n, 1);
    CK(cudaMemcpyAsync(labels_dev, ones.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    *modules = 1;
    *q = std::nan("");
    return BNA_OK;
  }
  const int sms = ctx->sms;
  const int stage_max = mod_stage_max();
  const int grid0 = mod_level_grid(sms, 0);                          // most blocks
  const int grid_lo = mod_level_grid(sms, (size_t)stage_max * 8);  // fewest blocks
  if (grid0 < 1 || grid_lo < 1)
    return fail(ctx, BNA_CUDA_ERROR, "bna_modularity: no resident block fits");
  const size_t gbytes = mod_group_bytes(), abytes = mod_assign_bytes();
  const long long nnz = (long long)R[n] - R[0];
  int32_t *label, *rows, *loc, *cnt, *lrp, *lci, *blkgrp, *adj_dev;
  double *vd, *y, *parts;
  float2 *vf, *rs;
  void *groups, *assign;
  unsigned long long* kmod;
  ENSURE(S_MOD_LABEL, (size_t)n * 4, label);
  ENSURE(S_MOD_ROWS, (size_t)n * 4, rows);
  ENSURE(S_MOD_LOC, (size_t)n * 4, loc);
  ENSURE(S_MOD_CNT, (size_t)n * 4, cnt);
  ENSURE(S_MOD_LRP, (size_t)(n + 1) * 4, lrp);
  ENSURE(S_MOD_LCI, (size_t)std::max(nnz, 1LL) * 4, lci);
  ENSURE(S_MOD_VD, (size_t)2 * n * 8, vd);
  ENSURE(S_MOD_VF, (size_t)2 * n * 8, vf);
  ENSURE(S_MOD_RS, (size_t)n * 8, rs);
  ENSURE(S_MOD_Y, (size_t)2 * n * 8, y);
  ENSURE(S_MOD_PARTS, (size_t)grid0 * mod_parts_per_block() * 8, parts);
  ENSURE(S_MOD_BLKGRP, (size_t)grid0 * 4, blkgrp);
  ENSURE(S_MOD_GROUPS, (size_t)grid0 * gbytes, groups);  // at most one group per block
  ENSURE(S_MOD_ASSIGN, (size_t)(n / 2 + 1) * abytes, assign);
  ENSURE(S_MOD_KMOD, (size_t)(2 * n + 2) * 8 + 8, kmod);  // labels run up to 2 (n - 1)
  ENSURE(S_MOD_ADJ, (size_t)(2 * n + 2) * 4, adj_dev);
  CK(cudaMemsetAsync(label, 0, (size_t)n * 4, st));
  std::vector<int32_t> lab_h((size_t)n, 0), rows_h, loc_h((size_t)n, 0), lrp_h, blk_h;
  std::vector<int32_t> adj((size_t)2 * n + 2, 0);
  std::vector<char> grp_h, asg_h;
  std::vector<bna_mod_round> recs;
  std::vector<int> gcount, goff;
  int lo = 0, maxres = 0, index = 1, mods = 1;
  int32_t nrec = 0;
  while (lo <= maxres) {
    const int hi = maxres, nlab = hi - lo + 1;
    // the level's groups: nodes by label, ascending (counting sort on the host)
    gcount.assign((size_t)nlab + 1, 0);
    for (int i = 0; i < n; ++i)
      if (lab_h[i] >= lo && lab_h[i] <= hi) ++gcount[lab_h[i] - lo + 1];
    goff.assign((size_t)nlab + 1, 0);
    for (int k = 0; k < nlab; ++k) goff[k + 1] = goff[k] + gcount[k + 1];
    const int nrows = goff[nlab];
    rows_h.resize((size_t)nrows);
    {
      std::vector<int> fill(goff.begin(), goff.end() - 1);
      for (int i = 0; i < n; ++i)
        if (lab_h[i] >= lo && lab_h[i] <= hi) {
          const int k = lab_h[i] - lo;
          loc_h[i] = fill[k] - goff[k];
          rows_h[fill[k]++] = i;
        }
    }
    std::vector<int> live;  // non-empty labels of the level, ascending
    for (int k = 0; k < nlab; ++k)
      if (goff[k + 1] > goff[k]) live.push_back(k);
    if (live.empty()) {
      lo = hi + 1;
      continue;
    }
    // the level's induced subgraph (edges inside a group, group-local columns)
    CK(cudaMemcpyAsync(rows, rows_h.data(), (size_t)nrows * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(loc, loc_h.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
    CK(launch_mod_build(nrows, rows, rp, ci, label, loc, cnt, lrp, lci, sms, st));
    lrp_h.resize((size_t)nrows + 1);
    CK(cudaMemcpyAsync(lrp_h.data(), lrp, lrp_h.size() * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    recs.assign(live.size(), bna_mod_round{});
    std::vector<int> fb(live.size());
    std::vector<long long> sp(live.size()), sn(live.size());
    // launches of at most grid_lo groups; blocks shared out by each group's
    // work per step (positions + in-group edges)
    for (size_t c0 = 0; c0 < live.size(); c0 += (size_t)grid_lo) {
      const size_t c1 = std::min(live.size(), c0 + (size_t)grid_lo);
      const int ng = (int)(c1 - c0);
      int stage_rows = 0;
      bool e16 = true;
      for (int k = 0; k < ng; ++k) {
        const int gk = live[c0 + k], nr = goff[gk + 1] - goff[gk];
        if (nr <= stage_max) stage_rows = std::max(stage_rows, nr);
        e16 = e16 && nr <= 65536;
      }
      const int stage_bytes = (stage_rows * 8 + 15) / 16 * 16;
      std::vector<double> work((size_t)ng);
      double wsum = 0;
      for (int k = 0; k < ng; ++k) {
        const int gk = live[c0 + k];
        work[k] = (double)(goff[gk + 1] - goff[gk]) * 8.0 +
                  (double)(lrp_h[goff[gk + 1]] - lrp_h[goff[gk]]);
        wsum += work[k];
      }
      // blocks per group for a grid of gm blocks, and the largest column slice
      // of a block (the kernel's split: equal shares of positions + edges)
      std::vector<int> nbk((size_t)ng);
      auto share_out = [&](int gm) -> long long {
        long long emax = 0;
        for (int k = 0; k < ng; ++k) {
          const int gk = live[c0 + k], off = goff[gk], nr = goff[gk + 1] - goff[gk];
          // a share of the grid by work, but no block with less than ~32 entries
          // per thread: more blocks than that only lengthen the group's barriers
          const int nb = std::min(1 + (int)((double)(gm - ng) * work[k] / wsum),
                                  1 + (int)(work[k] / 32768.0));
          nbk[k] = nb;
          const long long e0 = lrp_h[off], W = (long long)nr + (lrp_h[off + nr] - e0);
          int prev = off;
          for (int b = 1; b <= nb; ++b) {
            int p;
            if (b == nb) {
              p = off + nr;
            } else {
              const long long t = W * b / nb;
              int l = 0, h = nr;
              while (l < h) {
                const int mid = (l + h) >> 1;
                if ((long long)mid + (lrp_h[off + mid] - e0) >= t) h = mid;
                else l = mid + 1;
              }
              p = off + l;
            }
            emax = std::max(emax, (long long)lrp_h[p] - lrp_h[prev]);
            prev = p;
          }
        }
        return emax;
      };
      // the most blocks per SM whose shared memory holds the iterate stage and
      // every block's column slice; else column slices stay in global memory
      size_t smem = 0;
      int ecap = 0, grid_max = 0;
      const int esz = e16 ? 2 : 4;
      for (int bps = 4; bps >= 1 && !ecap; --bps) {
        int dyn = std::min(mod_smem_max(), (228 * 1024) / bps - 17 * 1024) / 1024 * 1024;
        int gm = 0;
        for (int tries = 0; tries < 8 && dyn >= stage_bytes; ++tries, dyn -= 1024) {
          gm = mod_level_grid(sms, (size_t)dyn);
          if (gm >= bps * sms) break;
        }
        if (gm < bps * sms || dyn < stage_bytes) continue;
        gm = bps * sms;
        if (gm < ng) continue;
        const long long emax = share_out(gm);
        if ((long long)stage_bytes + emax * esz <= dyn) {
          smem = (size_t)stage_bytes + (size_t)emax * esz;
          ecap = (int)std::max(emax, 1LL);
          grid_max = gm;
        }
      }
      if (!ecap) {
        smem = (size_t)stage_bytes;
        grid_max = std::max(ng, mod_level_grid(sms, smem));
        share_out(grid_max);
      }
      grp_h.assign((size_t)ng * gbytes, 0);
      blk_h.clear();
      for (int k = 0; k < ng; ++k) {
        const int gk = live[c0 + k];
        const int nb = nbk[k];
        long long kg = 0;
        for (int q2 = goff[gk]; q2 < goff[gk + 1]; ++q2)
          kg += R[rows_h[q2] + 1] - R[rows_h[q2]];
        mod_group_set(grp_h.data() + (size_t)k * gbytes, lo + gk, goff[gk],
                      goff[gk + 1] - goff[gk], (int)blk_h.size(), nb, kg);
        for (int b = 0; b < nb; ++b) blk_h.push_back(k);
      }
      const int grid = (int)blk_h.size();  // <= grid_max: every block resident
      CK(cudaMemcpyAsync(groups, grp_h.data(), grp_h.size(), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(blkgrp, blk_h.data(), (size_t)grid * 4, cudaMemcpyHostToDevice, st));
      CK(launch_mod_level(n, M, rp, label, rows, lrp, lci, groups, blkgrp, vd, vf, rs, y, parts,
                          nrows, stage_rows, stage_bytes, ecap, e16 ? 1 : 0, smem, grid, 10000,
                          1e-6, st));
      CK(cudaMemcpyAsync(grp_h.data(), groups, grp_h.size(), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int k = 0; k < ng; ++k) {
        const int gk = live[c0 + k];
        bna_mod_round& e = recs[c0 + k];
        int err = 0;
        mod_group_get(grp_h.data() + (size_t)k * gbytes, &err, e.iters, e.residual, &e.lambda,
                      &sp[c0 + k], &sn[c0 + k], &fb[c0 + k]);
        if (err) return fail(ctx, BNA_TIMEOUT, "bna_modularity: a group barrier wait expired");
        e.round = lo + gk;
        e.nodes = goff[gk + 1] - goff[gk];
      }
    }
    // decisions in round order (:204-211, :283-292)
    int nas = 0;
    asg_h.resize(live.size() * abytes);
    for (size_t k = 0; k < live.size(); ++k) {
      bna_mod_round& e = recs[k];
      const bool issub = e.lambda > lam_min && sp[k] > 1 && sn[k] > 1;
      e.divided = issub ? 1 : 0;
      if (issub) {
        const int gk = live[k];
        mod_assign_set(asg_h.data() + (size_t)nas * abytes, goff[gk], goff[gk + 1] - goff[gk],
                       fb[k], maxres, (double)(sp[k] - sn[k]) + 0.5);
        ++nas;
        maxres += 2;
        ++mods;
      } else {
        adj[e.round] = index++;
      }
      if (nrec < log_cap) log[nrec] = e;
      ++nrec;
    }
    if (nas) {
      CK(cudaMemcpyAsync(assign, asg_h.data(), (size_t)nas * abytes, cudaMemcpyHostToDevice, st));
      CK(launch_mod_assign(nrows, rows, assign, nas, vd, label, st));
      CK(cudaMemcpyAsync(lab_h.data(), label, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
    }
    lo = hi + 1;
  }
  // Q (:215-224) from integer counts: same-module entries and module degree sums
  unsigned long long* same_dev = kmod + (size_t)2 * n + 2;
  CK(cudaMemsetAsync(kmod, 0, (size_t)(2 * n + 3) * 8, st));
  CK(launch_mod_q(n, rp, ci, label, kmod, same_dev, sms, st));
  std::vector<unsigned long long> kh((size_t)maxres + 2);
  CK(cudaMemcpyAsync(kh.data(), kmod, (size_t)(maxres + 1) * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&kh[maxres + 1], same_dev, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(adj_dev, adj.data(), (size_t)(maxres + 1) * 4, cudaMemcpyHostToDevice, st));
  CK(launch_mod_map(n, label, adj_dev, labels_dev, sms, st));
  CK(cudaStreamSynchronize(st));
  double qq = (double)kh[maxres + 1];
  for (int k = 0; k <= maxres; ++k) qq -= (double)kh[k] * (double)kh[k] / 2 / (double)M;
  qq /= 2 * (double)M;
  *modules = mods;
  *q = qq;
  if (log_n) *log_n = nrec;
  ctx->klaunch = 0;
  return BNA_OK;
}

int32_t bna_ec(bna_ctx* ctx, const bna_csr* csr, int32_t max_iter, double eps, double* ec_dev,
               double* lambda, int32_t* iters, void* stream) {
  if (!ctx || !csr || !ec_dev || csr->n < 1 || !csr->row_ptr || (csr->nnz > 0 && !csr->col_idx))
    return fail(ctx, BNA_BAD_ARG, "bna_ec: bad arguments");
  int32_t s = set_device(ctx, as_stream(stream));
  if (s) return s;
  return ec_run(ctx, csr->n, csr->row_ptr, csr->col_idx, csr->val, nullptr, csr->nnz, max_iter,
                eps, ec_dev, lambda, iters, as_stream(stream));
}

int32_t bna_lead_vector(bna_ctx* ctx, const int32_t* R, const int32_t* C, const double* V,
                        int64_t N, double* ec_host, double* lambda, int32_t* iters) {
  if (!ctx || !R || !ec_host || N < 1 || N > 0x7fffffffLL)
    return fail(ctx, BNA_BAD_ARG, "bna_lead_vector: bad arguments");
  int32_t s = set_device(ctx);
  if (s) return s;
  const long long nnz = R[N];
  if (nnz < 0) return fail(ctx, BNA_BAD_ARG, "bna_lead_vector: negative R[N]");
  if (nnz > 0 && !C) return fail(ctx, BNA_BAD_ARG, "bna_lead_vector: C is NULL");
  int32_t *dr, *dc;
  double* dv = nullptr;
  double* dec;
  ENSURE(S_EC_R, (size_t)(N + 1) * 4, dr);
  ENSURE(S_EC_C, (size_t)std::max(nnz, 1LL) * 4, dc);
  if (V) ENSURE(S_EC_VD, (size_t)std::max(nnz, 1LL) * 8, dv);
  ENSURE(S_DUMP, (size_t)N * 8, dec);
  CK(cudaMemcpyAsync(dr, R, (size_t)(N + 1) * 4, cudaMemcpyHostToDevice, nullptr));
  if (nnz > 0) {
    CK(cudaMemcpyAsync(dc, C, (size_t)nnz * 4, cudaMemcpyHostToDevice, nullptr));
    if (V) CK(cudaMemcpyAsync(dv, V, (size_t)nnz * 8, cudaMemcpyHostToDevice, nullptr));
  }
  s = ec_run(ctx, (int)N, dr, dc, nullptr, dv, nnz, 10000, 1e-6, dec, lambda, iters, nullptr);
  if (s != BNA_OK && s != BNA_NOT_CONVERGED) return s;
  CK(cudaMemcpyAsync(ec_host, dec, (size_t)N * 8, cudaMemcpyDeviceToHost, nullptr));
  CK(cudaStreamSynchronize(nullptr));
  return s;
}

}  // extern "C"
