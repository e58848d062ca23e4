// C ABI of the voxel-network builder: the context and its device arena, its
// options, the z-score entry point and the single-subject correlation -> CSR
// flow (z-scores, count pass, candidates, density rule, scans, fill), with
// device or host buffers.
#include "ctx.cuh"

namespace bna {

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

}  // namespace bna

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

namespace bna {

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



// Every entry point starts here: device current, and the call's stream
// recorded for stream-ordered arena growth.
int32_t set_device(bna_ctx* ctx, cudaStream_t st) {
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


int32_t corr_pass(bna_ctx* ctx, const CorrArgs& a, int precision, int pass, cudaStream_t st,
                  bool sampled) {
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
      unsigned int* sched;
      ENSURE(S_TCSCHED, 2 * sizeof(unsigned int), sched);
      CK(cudaMemsetAsync(sched, 0, 2 * sizeof(unsigned int), st));
      for (int t0 = 0; t0 < nt; t0 += per, ++ctx->klaunch) {
        if (t0 > 0) gate(ctx, st, BNA_PHASE_CORR, t0);
        CK(launch_corr_tc(a, pass, precision == BNA_PREC_BF16X3 ? 0 : 1, tiles + t0,
                          std::min(per, nt - t0),
                          reinterpret_cast<const uint8_t*>(ctx->ptr[S_BLOCKBAD]), nullptr, 0,
                          ctx->sms, sched, st));
      }
      return BNA_OK;
    }
    default:
      return fail(ctx, BNA_UNSUPPORTED, "precision %d is not built in this library", precision);
  }
}

}  // namespace bna


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


// Free the arena on `st` (into the library's pool; with to_driver, the
// pool's cached memory then goes back to the driver); the caller guarantees
// that no work using the arena is pending on any other stream.
void bna::arena_release(bna_ctx* ctx, cudaStream_t st, bool to_driver) {
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


// Known threshold rules, and the float the kernels compare against: tau as
// the reference's float, or for the 2mm tools' rule (r > tau - 1e-6 in
// double) the smallest float above tau - 1e-6.
float bna::rule_tau(const bna_corr_opts* o) {
  const float t = (float)o->value;
  if (o->mode != BNA_THR_R_EPS) return t;
  const double lo = (double)t - 1e-6;
  float f = (float)lo;
  if ((double)f <= lo) f = std::nextafter(f, INFINITY);
  return f;
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
int32_t bna::corr_csr_core(bna_ctx* ctx, CorrArgs& a, int32_t N, int32_t T,
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
      unsigned int* sched;
      ENSURE(S_TCSCHED, 2 * sizeof(unsigned int), sched);
      CK(cudaMemsetAsync(sched, 0, 2 * sizeof(unsigned int), st));
      CK(launch_corr_tc(a, 2, precision == BNA_PREC_BF16X3 ? 0 : 1, d, 1, bb, out_dev, J % 2, 1,
                        sched, st));
      CK(cudaStreamSynchronize(st));
      break;
    }
    default: return fail(ctx, BNA_UNSUPPORTED, "precision %d is not built", precision);
  }
  return BNA_OK;
}

