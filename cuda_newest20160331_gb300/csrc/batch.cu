// Batches: several subjects' count passes in one persistent tensor-core
// launch replayed from a captured CUDA graph, then each subject's selection,
// recompute, scans and fill.
#include "ctx.cuh"

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
  // the launches' tile counters (each launch leaves them zero)
  unsigned int* sched;
  ENSURE(S_TCSCHED, 2 * sizeof(unsigned int), sched);
  CK(cudaMemsetAsync(sched, 0, 2 * sizeof(unsigned int), st));
  {
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    for (int t0 = 0; ce == cudaSuccess && t0 < ctx->batch_ntiles; t0 += per, ++launches)
      ce = launch_corr_tc_multi(batch, table_dev, tiles4 + t0,
                                std::min(per, ctx->batch_ntiles - t0), form, dev_sel, absm,
                                ctx->sms, sched, cap);
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

