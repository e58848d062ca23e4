// Multi-subject average with optional Fisher z (the reference's to_average
// modes, W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:418-670) and the packed
// correlation matrix (.cormat) entry point.
#include "ctx.cuh"

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
    unsigned int* sched;
    ENSURE(S_TCSCHED, 2 * sizeof(unsigned int), sched);
    CK(cudaMemsetAsync(sched, 0, 2 * sizeof(unsigned int), st));
    for (int t0 = 0; t0 < ctx->ntiles; t0 += per, ++ctx->klaunch)
      CK(launch_corr_tc(as, 4, prec == BNA_PREC_BF16X3 ? 0 : 1, tiles + t0,
                        std::min(per, ctx->ntiles - t0),
                        reinterpret_cast<const uint8_t*>(ctx->ptr[S_BLOCKBAD]), nullptr, 0,
                        ctx->sms, sched, st, &ap));
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

