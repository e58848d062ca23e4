// Autotuner of the tensor-core shapes (operand form x tile band) and the
// resolution of BNA_PREC_AUTO calls through its choices.
#include "ctx.cuh"

// Autotuner bucket: half-octaves of N and T, and the rule kind.
long long bna::tune_key(int N, int T, int mode) {
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
int32_t bna::resolve_precision(bna_ctx* ctx, int N, int T, const bna_corr_opts* opts,
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

