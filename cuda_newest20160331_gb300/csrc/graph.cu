// Consumers of a device CSR: re-thresholding (several thresholds from one
// pass), eigenvector centrality (Lead_Vector_GPU) and Newman modularity.
#include "ctx.cuh"

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

// The column-chunked kernel serves graphs of at most kEcChunkMax chunks whose
// gathers fall in a sector of their own for at least kEcChunkFresh of the
// entries (measured: a random-like 45k graph, 98 % such entries, 93 -> 73 us
// per iteration; a block-network 40k graph, 43 %, 33 us with the
// per-iteration kernel and 93 us chunked).
constexpr int kEcChunkMax = 4;
constexpr double kEcChunkFresh = 0.6;
// ... and at least this many entries per row on average: every block stages
// the whole iterate each iteration, which a sparse graph's few gathers do not
// repay (graphs of a few hundred edges on 50,665 and 94,939 vertices took 33
// and 55 us per iteration chunked, one on 168,220 vertices 33 us unchunked)
constexpr long long kEcChunkMinDeg = 8;
// Graphs of at most this many entries per row on average (those whose
// centrality converges slowly or never) sum their rows a thread per row.
constexpr long long kEcSparseDeg = 2;

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
  // the column-chunked kernel (iterate staged in shared memory) for graphs
  // of up to kEcChunkMax chunks whose rows have ascending columns and whose
  // gathers have little locality (most entries in a sector of their own:
  // clustered graphs hit L1 with the per-iteration kernel and run faster there)
  const int nch = ec_chunk_count(n);
  bool chunked = nch >= 1 && nch <= kEcChunkMax && nnz_used > 0 &&
                 nnz_used >= kEcChunkMinDeg * (long long)n;
  const bool sparse = nnz_used <= kEcSparseDeg * (long long)n;
  int* csplit = nullptr;
  int* rowsplit = nullptr;
  float2* part = nullptr;
  const int cgrid_rows = ctx->sms;
  if (chunked) {
    unsigned long long* info;
    ENSURE(S_EC_SPLIT, (size_t)std::max(nch - 1, 1) * n * sizeof(int), csplit);
    ENSURE(S_EC_PART, (size_t)n * sizeof(float2), part);
    ENSURE(S_EC_ROWS, (size_t)(cgrid_rows + 1) * sizeof(int), rowsplit);
    ENSURE(S_EC_FLAG, 2 * sizeof(unsigned long long), info);
    CK(launch_ec_chunk_prep(n, rp, ci, nnz_used, info, csplit, cgrid_rows, rowsplit, st));
    CK(cudaMemcpyAsync(ctx->pinned, info, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                       st));
    CK(cudaStreamSynchronize(st));
    const unsigned long long* h = static_cast<const unsigned long long*>(ctx->pinned);
    chunked = h[0] == 0 && (double)h[1] >= kEcChunkFresh * (double)nnz_used;
    if (chunked) CK(prepare_ec_chunk());
  }
  EcGraph& g = ctx->ecg;
  const void* key[9] = {rp, ci, val, vald, u, state, csplit, rowsplit, part};
  bool same = g.exec && g.n == n && g.grid == grid && g.max_iter == max_iter && g.eps == eps &&
              g.nnz_used == nnz_used && g.iters == giters && g.chunked == chunked;
  for (int k = 0; k < 9 && same; ++k) same = (g.key[k] == key[k]);
  if (!same) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = EcGraph();
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < giters; ++it) {
      const size_t cur = (size_t)(it & 1) * n, nxt = (size_t)((it + 1) & 1) * n;
      if (chunked)
        launch_ec_chunk(n, rp, ci, val, vald, nnz_used, u + cur, uf + cur, u + nxt, uf + nxt,
                        parts, state, cgrid_rows, max_iter, eps, rowsplit, csplit, part, cap);
      else if (sparse)
        launch_ec_iter_sparse(n, rp, ci, val, vald, nnz_used, u + cur, uf + cur, u + nxt,
                              uf + nxt, parts, state, grid, max_iter, eps, cap);
      else
        launch_ec_iter(n, rp, ci, val, vald, nnz_used, u + cur, uf + cur, u + nxt, uf + nxt,
                       parts, state, grid, max_iter, eps, cap);
    }
    cudaGraph_t graph;
    cudaError_t ce = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    CK(ce);
    ce = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ce);
    for (int k = 0; k < 9; ++k) g.key[k] = key[k];
    g.n = n;
    g.grid = grid;
    g.max_iter = max_iter;
    g.eps = eps;
    g.nnz_used = nnz_used;
    g.iters = giters;
    g.chunked = chunked;
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

