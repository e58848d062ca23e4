/*
 * ORACLE — test infrastructure only.  Nothing in the product links or calls
 * this file; tests/, the smoke check and bench.py's CPU-baseline leg use it
 * as the checker.
 *
 * A plain-C restatement of the reference's CPU arithmetic for the
 * correlation -> CSR -> eigenvector-centrality path ("W/" =
 * BNAPlatform-weighted-win64-cuda7.0-20160331/src):
 *   orc_zscore          CorMat_cpu normalisation   W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:923-951
 *                       (identical to CorMat_gpu's  W/CorMat/CUCorMat/CUCorMat/CorMat.cu:24-52)
 *   orc_cormat_packed   CorMat_cpu cross terms     CorMat.cpp:955-965, packed i<j row-major,
 *                       then post_block's clamp    CorMat.cpp:883 (outside [-1,1] or NaN -> 0)
 *   orc_threshold_csr   FormFullGraph + FormCSRGraph  CorMat.cpp:683-703, 889-918 (r rules),
 *                       |r| rule of U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp:198
 *   orc_density         FormFullGraph_s + select   CorMat.cpp:705-822, 327-329
 *   orc_ec              Lead_Vector_GPU            W/CUEC/weighted-net.cu:55-221 (FP64)
 *   orc_avg_accumulate  multi-subject average      CorMat.cpp:847-883 (post_block with
 *   orc_avg_finalize                               accumulation, fishertrans :36-42),
 *                                                  :652-666 (division, inv_fishertrans :44-50)
 *   orc_cormat_mt_f32   CorMat_cpu_MT/Cross_term   U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp:283-383
 *                       (float accumulation; used as the multi-core CPU baseline)
 *   orc_mt_prepare,     the same tool with its graph  CorMat_CPU.cpp:190-226, 283-383 (CSR
 *   orc_mt_rows_csr     steps on a row sample      values as W's CorMat.cpp:889-918): the
 *                                                  timed CPU baseline, CSR assembly included
 *   orc_synth_bold      the workloads' seeded factor-model input (no reference counterpart),
 *                       so the CPU baseline needs nothing from the product library
 * Built with -ffp-contract=off so every operation rounds like the reference's
 * scalar code.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

enum { R_GT = 0, R_GE = 1, ABS_GT = 2, ABS_GE = 3, R_EPS = 5 };

/* z[i*T + t] (voxel-major) from bold[t*N + i] (time-major). */
void orc_zscore(const float* bold, int N, int T, float* z) {
  for (int i = 0; i < N; ++i) {
    double sum1 = 0, sum2 = 0;
    for (int l = 0; l < T; ++l) sum1 += bold[(size_t)l * N + i];
    sum1 /= T;
    for (int l = 0; l < T; ++l) {
      const double d = bold[(size_t)l * N + i] - sum1;
      sum2 += d * d;
    }
    sum2 = sqrt(sum2);
    for (int l = 0; l < T; ++l) z[(size_t)i * T + l] = (float)((bold[(size_t)l * N + i] - sum1) / sum2);
  }
}

/* The reference value of one pair: float products, double accumulation in
 * time order, rounded to float (NaN for a zero-variance voxel); orc_pair_r
 * then applies post_block's clamp. */
float orc_pair_r_raw(const float* z, int T, int i, int j) {
  const float* a = z + (size_t)i * T;
  const float* b = z + (size_t)j * T;
  double s = 0;
  for (int l = 0; l < T; ++l) {
    const float p = a[l] * b[l];
    s += p;
  }
  return (float)s;
}

float orc_pair_r(const float* z, int T, int i, int j) {
  const float r = orc_pair_r_raw(z, T, i, j);
  return (r >= -1.0f && r <= 1.0f) ? r : 0.0f;
}

static int64_t packed_index(int64_t N, int64_t i, int64_t j) { /* i < j, CorMat.cpp:905 */
  return i * N - (1 + i) * i / 2 + j - (i + 1);
}

struct pk_job { const float* z; int N, T, tid, nth, raw; float* out; };

static void* pk_worker(void* p) {
  struct pk_job* jb = (struct pk_job*)p;
  for (int i = jb->tid; i < jb->N; i += jb->nth)
    for (int j = i + 1; j < jb->N; ++j)
      jb->out[packed_index(jb->N, i, j)] =
          jb->raw ? orc_pair_r_raw(jb->z, jb->T, i, j) : orc_pair_r(jb->z, jb->T, i, j);
  return NULL;
}

/* packed[M1], M1 = N(N-1)/2, row-major over i < j; raw: without
 * post_block's clamp (the values the 2mm tools' rule compares). */
void orc_cormat_packed2(const float* z, int N, int T, float* packed, int nthreads, int raw) {
  if (nthreads < 1) nthreads = 1;
  pthread_t th[256];
  struct pk_job jobs[256];
  if (nthreads > 256) nthreads = 256;
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = (struct pk_job){z, N, T, t, nthreads, raw, packed};
    if (t > 0) pthread_create(&th[t], NULL, pk_worker, &jobs[t]);
  }
  pk_worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
}

void orc_cormat_packed(const float* z, int N, int T, float* packed, int nthreads) {
  orc_cormat_packed2(z, N, T, packed, nthreads, 0);
}

/* R_EPS: the 2mm / chunk GPU tools' rule, CorMat-2mm.cu:140,156 and
 * step2-dense2csr.cu:52, on the raw value: out > (r_thresh - ep) &&
 * out <= (1 + ep) with ep the double 1e-6 (CorMat-2mm.cu:13), so both
 * comparisons run in double. */
static int is_edge(float r, int mode, float tau) {
  switch (mode) {
    case R_EPS: return (double)r > (double)tau - 1e-6 && (double)r <= 1.0 + 1e-6;
    case R_GT: return r > tau;
    case ABS_GT: return fabsf(r) > tau;
    case ABS_GE: return fabsf(r) >= tau;
    default: return r >= tau;
  }
}

/* Key of a pair for the density tie list. */
static uint64_t pkey(int i, int j) { return ((uint64_t)(uint32_t)i << 32) | (uint32_t)j; }

static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : x > y;
}

static int in_sorted(const uint64_t* k, int64_t n, uint64_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t m = (lo + hi) / 2;
    if (k[m] < key) lo = m + 1; else hi = m;
  }
  return lo < n && k[lo] == key;
}

/* CSR of the thresholded graph straight from the packed triangle: row i lists
 * columns j < i then j > i, ascending, as FormCSRGraph's row-major scan of the
 * symmetric bool matrix does.  R has N+1 entries; C / V may be NULL (count
 * only).  drop (sorted keys, may be NULL) removes listed pairs (density ties).
 * Returns nnz (directed). */
int64_t orc_threshold_csr(const float* packed, int N, int mode, float tau, const uint64_t* drop,
                          int64_t ndrop, int32_t* R, int32_t* C, float* V) {
  int64_t nnz = 0;
  if (R) R[0] = 0;
  for (int i = 0; i < N; ++i) {
    for (int j = 0; j < N; ++j) {
      if (j == i) continue;
      const int a = i < j ? i : j, b = i < j ? j : i;
      const float r = packed[packed_index(N, a, b)];
      if (!is_edge(r, mode, tau)) continue;
      if (drop && r == tau && in_sorted(drop, ndrop, pkey(a, b))) continue;
      if (C) C[nnz] = j;
      if (V) V[nnz] = r;
      ++nnz;
    }
    if (R) R[i + 1] = (int32_t)nnz;
  }
  return nnz;
}

/* Density rule of FormFullGraph_s.  k = orc_density_k (CorMat.cpp:327-329);
 * tau = k-th largest packed value; edges r >= tau
 * in row-major (i<j) scan order, where once the count exceeds k the most
 * recent tie is removed (:797-808) — i.e. the earliest (k - #greater) ties in
 * scan order are kept.  Writes the sorted keys of the dropped ties to
 * drop_out (capacity drop_cap) and returns tau; *k_out = k, *ndrop_out = the
 * number of dropped ties (-1 if drop_cap was too small). */
/* Edge count of the density rule as CorMat.cpp:327-328 computes it:
 * Clength = (long long) 2*M1*s/100.0 with s a float (parsed by atof into
 * real__t): the product 2*M1*s is formed in float, then divided in double. */
int64_t orc_density_k(int N, double s_percent) {
  const int64_t M1 = (int64_t)N * (N - 1) / 2;
  const float s = (float)s_percent;
  const float prod = (float)(2 * M1) * s;
  int64_t clen = (int64_t)((double)prod / 100.0);
  clen += clen % 2;
  return clen / 2;
}

float orc_density(const float* packed, int N, double s_percent, int64_t* k_out,
                  uint64_t* drop_out, int64_t drop_cap, int64_t* ndrop_out) {
  const int64_t M1 = (int64_t)N * (N - 1) / 2;
  const int64_t k = orc_density_k(N, s_percent);
  *k_out = k;
  if (k <= 0) {
    *ndrop_out = 0;
    return INFINITY;
  }
  float* cp = (float*)malloc(sizeof(float) * (size_t)M1);
  memcpy(cp, packed, sizeof(float) * (size_t)M1);
  /* k-th largest by quickselect on a copy (the value is order-independent) */
  int64_t lo = 0, hi = M1 - 1;
  const int64_t want = k - 1;
  while (lo < hi) {
    const float pv = cp[lo + (hi - lo) / 2];
    int64_t a = lo, b = hi;
    while (a <= b) {
      while (cp[a] > pv) ++a;
      while (cp[b] < pv) --b;
      if (a <= b) {
        const float t = cp[a]; cp[a] = cp[b]; cp[b] = t;
        ++a; --b;
      }
    }
    if (want <= b) hi = b;
    else if (want >= a) lo = a;
    else break;
  }
  const float tau = cp[want];
  free(cp);
  int64_t greater = 0;
  for (int64_t q = 0; q < M1; ++q) greater += packed[q] > tau;
  int64_t keep = k - greater, nd = 0, idx = 0;
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j, ++idx) {
      if (packed[idx] != tau) continue;
      if (keep > 0) { --keep; continue; }
      if (nd < drop_cap) drop_out[nd] = pkey(i, j);
      ++nd;
    }
  if (nd > drop_cap) { *ndrop_out = -1; return tau; }
  qsort(drop_out, (size_t)nd, sizeof(uint64_t), cmp_u64);
  *ndrop_out = nd;
  return tau;
}

/* Power iteration of Lead_Vector_GPU.  V may be NULL (every entry 1).
 * Returns the iteration count; ec = last u, *lambda = norm used last. */
int orc_ec(const int32_t* R, const int32_t* C, const double* V, int N, int max_iter, double eps,
           double* ec, double* lambda, double* e1_out, double* e2_out) {
  const int64_t nnz_used = 2 * (int64_t)(R[N] / 2);
  double* u = (double*)malloc(sizeof(double) * (size_t)N);
  double* u0 = (double*)malloc(sizeof(double) * (size_t)N);
  double* y = (double*)malloc(sizeof(double) * (size_t)N);
  for (int i = 0; i < N; ++i) u[i] = i;
  double e1 = 1, e2 = 1, vnorm = 0;
  int iter = 0;
  while (e1 > eps && e2 > eps && iter < max_iter) {
    memcpy(u0, u, sizeof(double) * (size_t)N);
    double s = 0;
    for (int i = 0; i < N; ++i) s += u[i] * u[i];
    vnorm = sqrt(s);
    const double inv = 1.0 / vnorm;
    for (int i = 0; i < N; ++i) u[i] = u[i] * inv;
    for (int i = 0; i < N; ++i) {
      double acc = 0;
      int64_t e = R[i + 1] < nnz_used ? R[i + 1] : nnz_used;
      for (int64_t q = R[i]; q < e; ++q) acc += (V ? V[q] : 1.0) * u[C[q]];
      y[i] = acc;
    }
    memcpy(u, y, sizeof(double) * (size_t)N);
    double d1 = 0, d2 = 0;
    for (int i = 0; i < N; ++i) {
      const double a = u[i] - u0[i], b = u[i] + u0[i];
      d1 += a * a;
      d2 += b * b;
    }
    e1 = sqrt(d1);
    e2 = sqrt(d2);
    ++iter;
  }
  memcpy(ec, u, sizeof(double) * (size_t)N);
  *lambda = vnorm;
  if (e1_out) *e1_out = e1;
  if (e2_out) *e2_out = e2;
  free(u); free(u0); free(y);
  return iter;
}

/* CorMat_cpu_MT arithmetic (old CPU tool): rows centred in float,
 * m2 = sqrt(sum x^2 - (sum x)^2 / L) from double sums, float-accumulated
 * cross products, r = sum3 / m2_i / m2_j (0 if a moment is 0).  Rows
 * [row0, row1) against all j > i; values into packed (full M1 layout). */
struct mt_job { const float* bt; const float* m2; int N, L, row0, row1, tid, nth; float* out; };

static void* mt_worker(void* p) {
  struct mt_job* jb = (struct mt_job*)p;
  for (int i = jb->row0; i < jb->row1; ++i)
    for (int j = i + 1 + jb->tid; j < jb->N; j += jb->nth) {
      float s3 = 0;
      for (int l = 0; l < jb->L; ++l) s3 += jb->bt[(size_t)i * jb->L + l] * jb->bt[(size_t)j * jb->L + l];
      float r = s3 / jb->m2[i] / jb->m2[j];
      if (jb->m2[i] == 0 || jb->m2[j] == 0) r = 0;
      jb->out[packed_index(jb->N, i, j)] = r;
    }
  return NULL;
}

void orc_cormat_mt_f32(const float* bold, int N, int L, int row0, int row1, float* packed,
                       int nthreads) {
  float* bt = (float*)malloc(sizeof(float) * (size_t)N * L);
  float* m2 = (float*)malloc(sizeof(float) * (size_t)N);
  for (int l = 0; l < L; ++l)
    for (int i = 0; i < N; ++i) bt[(size_t)i * L + l] = bold[(size_t)l * N + i];
  for (int i = 0; i < N; ++i) {
    double s1 = 0, s2 = 0;
    float* row = bt + (size_t)i * L;
    for (int l = 0; l < L; ++l) {
      s1 += row[l];
      s2 += row[l] * row[l];
    }
    m2[i] = (float)sqrt(s2 - s1 * s1 / L);
    s1 /= L;
    for (int l = 0; l < L; ++l) row[l] -= (float)s1;
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  struct mt_job jobs[256];
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = (struct mt_job){bt, m2, N, L, row0, row1, t, nthreads, packed};
    if (t > 0) pthread_create(&th[t], NULL, mt_worker, &jobs[t]);
  }
  mt_worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(bt);
  free(m2);
}

/* Rows [row0, row1) of the thresholded CSR, straight from z (no packed
 * triangle): the full-size parity check of a row slice.  R_local has
 * row1-row0+1 entries (R_local[0] = 0); C / V may be NULL to count.
 * Rows are split across threads; each row's columns are ascending. */
struct rows_job {
  const float* z; int N, T, mode; float tau; int row0, row1, tid, nth;
  int64_t* cnt; int32_t* R; int32_t* C; float* V;
};

static void* rows_worker(void* p) {
  struct rows_job* jb = (struct rows_job*)p;
  for (int i = jb->row0 + jb->tid; i < jb->row1; i += jb->nth) {
    int64_t c = 0;
    int64_t base = jb->R ? jb->R[i - jb->row0] : 0;
    for (int j = 0; j < jb->N; ++j) {
      if (j == i) continue;
      const int lo = i < j ? i : j, hi = i < j ? j : i;
      const float r = jb->mode == R_EPS ? orc_pair_r_raw(jb->z, jb->T, lo, hi)
                                        : orc_pair_r(jb->z, jb->T, lo, hi);
      if (!is_edge(r, jb->mode, jb->tau)) continue;
      if (jb->C) jb->C[base + c] = j;
      if (jb->V) jb->V[base + c] = r;
      ++c;
    }
    if (jb->cnt) jb->cnt[i - jb->row0] = c;
  }
  return NULL;
}

int64_t orc_rows_csr(const float* z, int N, int T, int mode, float tau, int row0, int row1,
                     int32_t* R_local, int32_t* C, float* V, int nthreads) {
  const int nr = row1 - row0;
  int64_t* cnt = (int64_t*)calloc((size_t)nr + 1, sizeof(int64_t));
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  struct rows_job jobs[256];
  for (int pass = 0; pass < (C ? 2 : 1); ++pass) {
    for (int t = 0; t < nthreads; ++t) {
      jobs[t] = (struct rows_job){z, N, T, mode, tau, row0, row1, t, nthreads,
                                  pass == 0 ? cnt : NULL, pass == 0 ? NULL : R_local,
                                  pass == 0 ? NULL : C, pass == 0 ? NULL : V};
      if (t > 0) pthread_create(&th[t], NULL, rows_worker, &jobs[t]);
    }
    rows_worker(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    if (pass == 0) {
      int64_t s = 0;
      for (int q = 0; q < nr; ++q) {
        if (R_local) R_local[q] = (int32_t)s;
        s += cnt[q];
      }
      if (R_local) R_local[nr] = (int32_t)s;
    }
  }
  int64_t total = 0;
  for (int q = 0; q < nr; ++q) total += cnt[q];
  free(cnt);
  return total;
}

/* CPU baseline: the reference's multi-threaded correlation tool
 * (CorMat_cpu_MT / Cross_term, U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp:283-383:
 * float-centred rows, float-accumulated cross terms, r = sum3 / m2_i / m2_j,
 * j strided by thread id) over rows [row0, row1) against every j > i, with
 * its threshold rule |r| > tau (CorMat_CPU.cpp:198) counted in place instead
 * of stored (so a bounded row sample needs no N x N buffer).  Returns the
 * number of undirected edges. */
struct mtc_job { const float* bt; const float* m2; int N, L, row0, row1, tid, nth; float tau; int64_t cnt; };

static void* mtc_worker(void* p) {
  struct mtc_job* jb = (struct mtc_job*)p;
  int64_t c = 0;
  for (int i = jb->row0; i < jb->row1; ++i)
    for (int j = i + 1 + jb->tid; j < jb->N; j += jb->nth) {
      float s3 = 0;
      for (int l = 0; l < jb->L; ++l) s3 += jb->bt[(size_t)i * jb->L + l] * jb->bt[(size_t)j * jb->L + l];
      float r = s3 / jb->m2[i] / jb->m2[j];
      if (jb->m2[i] == 0 || jb->m2[j] == 0) r = 0;
      c += fabsf(r) > jb->tau;
    }
  jb->cnt = c;
  return NULL;
}

int64_t orc_rows_mt_f32_count(const float* bold, int N, int L, int row0, int row1, float tau,
                              int nthreads) {
  float* bt = (float*)malloc(sizeof(float) * (size_t)N * L);
  float* m2 = (float*)malloc(sizeof(float) * (size_t)N);
  for (int l = 0; l < L; ++l)
    for (int i = 0; i < N; ++i) bt[(size_t)i * L + l] = bold[(size_t)l * N + i];
  for (int i = 0; i < N; ++i) {
    double s1 = 0, s2 = 0;
    float* row = bt + (size_t)i * L;
    for (int l = 0; l < L; ++l) {
      s1 += row[l];
      s2 += row[l] * row[l];
    }
    m2[i] = (float)sqrt(s2 - s1 * s1 / L);
    s1 /= L;
    for (int l = 0; l < L; ++l) row[l] -= (float)s1;
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  struct mtc_job jobs[256];
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = (struct mtc_job){bt, m2, N, L, row0, row1, t, nthreads, tau, 0};
    if (t > 0) pthread_create(&th[t], NULL, mtc_worker, &jobs[t]);
  }
  mtc_worker(&jobs[0]);
  int64_t total = jobs[0].cnt;
  for (int t = 1; t < nthreads; ++t) {
    pthread_join(th[t], NULL);
    total += jobs[t].cnt;
  }
  free(bt);
  free(m2);
  return total;
}

/* fishertrans / inv_fishertrans (CorMat.cpp:36-50) in the reference's float
 * arithmetic: log and exp of a float argument are the float functions there
 * (C++ overloads), logf / expf here. */
static float orc_fisher_z(float r) {
  if (r == 1.0f) r = (float)((double)r - 1e-6);
  return (float)(0.5 * (double)logf((1.0f + r) / (1.0f - r)));
}
static float orc_fisher_r(float z) {
  float r = expf(2.0f * z);
  return (r - 1.0f) / (r + 1.0f);
}

/* One subject's post_block'd packed r (values outside [-1, 1] already 0,
 * which adds nothing) added into acc in float: post_block's accumulation. */
void orc_avg_accumulate(const float* packed_r, long long m, int fisher, float* acc) {
  for (long long i = 0; i < m; ++i) {
    const float r = packed_r[i];
    if (r >= -1.0f && r <= 1.0f) acc[i] += fisher ? orc_fisher_z(r) : r;
  }
}

/* acc / nsub, then inv_fishertrans when fisher (CorMat.cpp:652-666). */
void orc_avg_finalize(float* acc, long long m, int nsub, int fisher) {
  for (long long i = 0; i < m; ++i) {
    acc[i] /= (float)nsub;
    if (fisher) acc[i] = orc_fisher_r(acc[i]);
  }
}

/* ---- Newman spectral modularity (unweighted), restating the reference CPU
 * tool U/Newman_Modularity_CPU/Modularity_CPU/Modularity_CPU.cpp (the
 * 20160115 tree): Partition (:186-240), Sub_Partition (:252-300),
 * Lead_Vector (:315-377), VectorNorm (:383-389).  The graph is the binary
 * CSR (R, C); M = R[N] / 2.  Labels out: 1-based module per node, in the
 * order the rounds stopped dividing.  Returns the number of modules. */
static double mod_norm(const double* x, const unsigned char* g, int N) {
  double s = 0;
  for (int i = 0; i < N; ++i) s += g[i] ? x[i] * x[i] : 0;
  return sqrt(s);
}

static double mod_lead_vector(const int32_t* R, const int32_t* C, int N, long long M,
                              const double* sumbg, const unsigned char* g, double beta, double* v,
                              double* v0, double* verr, int* iters) {
  for (int i = 0; i < N; ++i) v[i] = g[i] ? (double)i : 0;  /* :322-324 */
  double err1 = 1, err2 = 1, vnorm = 0;
  int it = 0;
  while (err1 > 1e-6 && err2 > 1e-6 && it < 10000) {
    for (int i = 0; i < N; ++i) v0[i] = g[i] ? v[i] : 0;
    double vk = 0;
    for (int i = 0; i < N; ++i) vk += g[i] ? v0[i] * (double)(R[i + 1] - R[i]) : 0;
    for (int i = 0; i < N; ++i) {
      if (!g[i]) continue;
      double t = 0;
      for (int32_t j = R[i]; j < R[i + 1]; ++j) t += g[C[j]] ? v0[C[j]] : 0;
      t -= vk / 2 / (double)M * (double)(R[i + 1] - R[i]) + (sumbg[i] - beta) * v0[i];
      v[i] = t;
    }
    vnorm = mod_norm(v, g, N);
    for (int i = 0; i < N; ++i) v[i] = g[i] ? (v[i] / vnorm) : 0;
    for (int i = 0; i < N; ++i) verr[i] = g[i] ? (v[i] - v0[i]) : 0;
    err1 = mod_norm(verr, g, N);
    for (int i = 0; i < N; ++i) verr[i] = v[i] + v0[i];
    err2 = mod_norm(verr, g, N);
    ++it;
  }
  *iters = it;
  int mi = 0; /* :370-374 */
  v[0] = g[0] ? v[0] : 0;
  for (int i = 0; i < N; ++i)
    if (g[i] && fabs(v[i]) > fabs(v[mi])) mi = i;
  return (v[mi] * v0[mi] > 0) ? vnorm : -vnorm;
}

/* log (optional, 6 doubles per round that held nodes, at most 2N + 2 rounds):
 * round, nodes, iterations of the first and of the retried Lead_Vector call
 * (0: none), lambda, divided. */
int orc_modularity(const int32_t* R, const int32_t* C, int N, double lambda_min, int32_t* labels,
                   double* q_out, int* rounds_out, double* log, int* log_n) {
  const long long M = (R[N] - R[0]) / 2;
  if (log_n) *log_n = 0;
  if (M == 0) { /* no edge: the reference divides by M = 0; one module, Q undefined */
    for (int i = 0; i < N; ++i) labels[i] = 1;
    *q_out = NAN;
    if (rounds_out) *rounds_out = 1;
    return 1;
  }
  int* res = (int*)calloc((size_t)N, sizeof(int));
  int* adj = (int*)malloc(sizeof(int) * (size_t)(2 * N + 2));
  unsigned char* g = (unsigned char*)malloc((size_t)N);
  double* v = (double*)malloc(sizeof(double) * (size_t)N);
  double* v0 = (double*)malloc(sizeof(double) * (size_t)N);
  double* verr = (double*)malloc(sizeof(double) * (size_t)N);
  double* sumbg = (double*)malloc(sizeof(double) * (size_t)N);
  int round = 0, max_result = 0, index = 1, modules = 1;
  while (round <= max_result) {
    int numg = 0;
    for (int i = 0; i < N; ++i) {
      g[i] = res[i] == round;
      numg += g[i];
    }
    if (numg) {
      /* Sub_Partition: sumBG in integer arithmetic (:258-266) */
      long long kg = 0;
      for (int j = 0; j < N; ++j) kg += (long long)(R[j + 1] - R[j]) * g[j];
      for (int i = 0; i < N; ++i) {
        if (!g[i]) continue;
        long long in = 0;
        for (int32_t j = R[i]; j < R[i + 1]; ++j) in += g[C[j]];
        sumbg[i] = (double)(in - (long long)(R[i + 1] - R[i]) * kg / 2 / M);
      }
      int it = 0, it2 = 0;
      double lambda = mod_lead_vector(R, C, N, M, sumbg, g, 0.0, v, v0, verr, &it);
      if (lambda < 0) lambda += mod_lead_vector(R, C, N, M, sumbg, g, -lambda, v, v0, verr, &it2);
      long long subn = 0, subp = 0;
      for (int i = 0; i < N; ++i) {
        subp += g[i] && v[i] > 0;
        subn += g[i] && v[i] <= 0;
      }
      const int issub = lambda > lambda_min && subp > 1 && subn > 1;
      if (log && log_n) {
        double* e = log + 6 * (size_t)(*log_n)++;
        e[0] = round;
        e[1] = numg;
        e[2] = it;
        e[3] = it2;
        e[4] = lambda;
        e[5] = issub;
      }
      if (issub) {
        for (int i = 0; i < N; ++i)
          if (g[i]) res[i] = max_result + 1 + (v[i] * ((double)(subp - subn) + 0.5) <= 0);
        max_result += 2;
      } else {
        adj[round] = index++;
      }
      modules += issub;
    }
    ++round;
  }
  /* Q (:215-224) */
  double q = 0;
  for (int i = 0; i < N; ++i)
    for (int32_t j = R[i]; j < R[i + 1]; ++j) q += 1.0 * (res[i] == res[C[j]]);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      q -= 1.0 * (res[i] == res[j]) * (R[i + 1] - R[i]) * (R[j + 1] - R[j]) / 2 / M;
  q /= 2 * M;
  for (int i = 0; i < N; ++i) labels[i] = adj[res[i]];
  *q_out = q;
  if (rounds_out) *rounds_out = round;
  free(res);
  free(adj);
  free(g);
  free(v);
  free(v0);
  free(verr);
  free(sumbg);
  return modules;
}

/* ---- synthetic input, restated for the reference arm ---------------------
 * The seeded factor-model generator of the workloads, restated here so the
 * reference's CPU path can be fed without loading the product library:
 *   x_i(t) = sum_k L_ik f_k(t) + eps_i(t), f_k AR(1) with coefficient phi and
 *   unit stationary variance (innovation sqrt(1 - phi^2), 100 burn-in steps),
 *   eps ~ N(0, 1); kind 0: L_ik = load_sd * N(0,1); kind 1 (block network):
 *   voxel i is in block i / block, network (block mod n_net), L_ik =
 *   load_sd * g[net][k] + jitter_sd * N(0,1).
 * Random numbers: a counter hash (murmur3's 64-bit finaliser over the seed,
 * stream, index and draw) mapped to (0, 1); normals by Marsaglia's polar
 * method; ln by the atanh series of the mantissa (no libm), so every host
 * gives the same bits.  Output float32 time-major [T][N]. */
static uint64_t syn_mix(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

static double syn_u01(uint64_t seed, uint64_t stream, uint64_t idx, uint64_t draw) {
  uint64_t h = syn_mix((seed * 0x9E3779B97F4A7C15ULL) ^ (stream * 0xD1B54A32D192ED03ULL));
  h = syn_mix(h ^ (idx * 0x8CB92BA72F3D8DD7ULL));
  h = syn_mix(h ^ (draw * 0xABC98388FB8FAC03ULL + 0x632BE59BD9B4E019ULL));
  return (double)(h >> 11) * 0x1.0p-53 + 0x1.0p-54;
}

static double syn_ln(double x) {
  uint64_t bits;
  memcpy(&bits, &x, 8);
  int ex = (int)((bits >> 52) & 0x7ff) - 1023;
  bits = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
  double m;
  memcpy(&m, &bits, 8);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    ex += 1;
  }
  const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
  double acc = 1.0 / 25.0;
  for (int k = 11; k >= 0; --k) acc = acc * s2 + 1.0 / (double)(2 * k + 1);
  return (double)ex * 0x1.62e42fefa39efp-1 + 2.0 * s * acc;
}

static double syn_normal(uint64_t seed, uint64_t stream, uint64_t idx) {
  for (uint64_t d = 0;; d += 2) {
    const double a = 2.0 * syn_u01(seed, stream, idx, d) - 1.0;
    const double b = 2.0 * syn_u01(seed, stream, idx, d + 1) - 1.0;
    const double q = a * a + b * b;
    if (q > 0.0 && q < 1.0) return a * sqrt(-2.0 * syn_ln(q) / q);
  }
}

struct syn_job {
  int N, T, K, kind, block, n_net, tid, nth;
  uint64_t seed;
  double load_sd, jitter_sd;
  const double* f; const double* g;
  float* out;
};

static void* syn_worker(void* p) {
  struct syn_job* jb = (struct syn_job*)p;
  const int K = jb->K, T = jb->T, N = jb->N;
  double* L = (double*)malloc(sizeof(double) * (size_t)256 * (K > 0 ? K : 1));
  for (int c = jb->tid; c * 256 < N; c += jb->nth) {
    const int i0 = c * 256, i1 = i0 + 256 < N ? i0 + 256 : N;
    for (int i = i0; i < i1; ++i)
      for (int k = 0; k < K; ++k) {
        const double h = syn_normal(jb->seed, 2, (uint64_t)i * K + k);
        L[(size_t)(i - i0) * K + k] =
            jb->kind == 1 ? jb->load_sd * jb->g[(size_t)((i / jb->block) % jb->n_net) * K + k] +
                                jb->jitter_sd * h
                          : jb->load_sd * h;
      }
    for (int t = 0; t < T; ++t)
      for (int i = i0; i < i1; ++i) {
        double x = 0.0;
        for (int k = 0; k < K; ++k) x = x + L[(size_t)(i - i0) * K + k] * jb->f[(size_t)k * T + t];
        x = x + syn_normal(jb->seed, 4, (uint64_t)i * T + t);
        jb->out[(size_t)t * N + i] = (float)x;
      }
  }
  free(L);
  return NULL;
}

int orc_synth_bold(int N, int T, int K, int kind, uint64_t seed, double phi, double load_sd,
                   double jitter_sd, int block, int n_net, float* out, int nthreads) {
  if (N <= 0 || T <= 0 || K < 0 || (kind == 1 && (block <= 0 || n_net <= 0))) return -1;
  const int burn = 100;
  const double innov = sqrt(1.0 - phi * phi);
  double* f = (double*)malloc(sizeof(double) * ((size_t)K * T + 1));
  for (int k = 0; k < K; ++k) {
    double v = 0.0;
    for (int t = 0; t < burn + T; ++t) {
      v = phi * v + innov * syn_normal(seed, 1, (uint64_t)k * (burn + T) + t);
      if (t >= burn) f[(size_t)k * T + (t - burn)] = v;
    }
  }
  double* g = NULL;
  if (kind == 1) {
    g = (double*)malloc(sizeof(double) * ((size_t)n_net * K + 1));
    for (int n = 0; n < n_net; ++n)
      for (int k = 0; k < K; ++k) g[(size_t)n * K + k] = syn_normal(seed, 3, (uint64_t)n * K + k);
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  struct syn_job jobs[256];
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = (struct syn_job){N, T, K, kind, block, n_net, t, nthreads, seed, load_sd, jitter_sd,
                               f, g, out};
    if (t > 0) pthread_create(&th[t], NULL, syn_worker, &jobs[t]);
  }
  syn_worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(f);
  free(g);
  return 0;
}

/* ---- the reference's CPU tool on a row sample, CSR included --------------
 * U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp runs CorMat_cpu_MT (:283-337:
 * transpose, float-centred rows, m2 = sqrt(sum x^2 - (sum x)^2 / L) from
 * double sums), Cross_term (:340-383: float-accumulated cross terms,
 * r = sum3 / m2_i / m2_j, 0 when a moment is 0, j strided by thread id) into
 * the packed triangle, then FormFullGraph (:190-206: the N x N bool matrix,
 * cleared, both (i,j) and (j,i) set per edge) and FormCSRGraph (:209-226: a
 * row-major scan of that matrix); the weighted tree's FormCSRGraph also
 * copies each edge's r (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:889-918).
 *
 * orc_mt_prepare is the one-time part (transpose, moments, centring).
 * orc_mt_rows_csr runs the per-pair part for the pairs (i, j > i) of a set
 * of sample rows S (ascending): cross terms on `nthreads` threads as
 * Cross_term does, then, single-threaded as in the reference, the graph and
 * CSR steps restricted to the sample: the bool rows of S (full width N) and,
 * for rows outside S, their bool columns at S, cleared and set like
 * FormFullGraph, then scanned row by row like FormCSRGraph.  R has N + 1
 * entries; C / V (cap entries, V may be NULL) receive the sample's directed
 * entries in CSR order.  Returns nnz, or -nnz - 1 when nnz > cap (C / V
 * untouched past cap).  secs (optional) gets the seconds of the three steps. */
void orc_mt_prepare(const float* bold, int N, int L, float* bt, float* m2) {
  /* the transpose in 64 x 64 blocks (a copy: the order does not change a value) */
  for (int l0 = 0; l0 < L; l0 += 64)
    for (int i0 = 0; i0 < N; i0 += 64)
      for (int i = i0; i < i0 + 64 && i < N; ++i)
        for (int l = l0; l < l0 + 64 && l < L; ++l) bt[(size_t)i * L + l] = bold[(size_t)l * N + i];
  for (int i = 0; i < N; ++i) {
    double s1 = 0, s2 = 0;
    float* row = bt + (size_t)i * L;
    for (int l = 0; l < L; ++l) {
      s1 += row[l];
      s2 += row[l] * row[l];
    }
    m2[i] = (float)sqrt(s2 - s1 * s1 / L);
    s1 /= L;
    for (int l = 0; l < L; ++l) row[l] -= (float)s1;
  }
}

struct mts_job {
  const float* bt; const float* m2; const int32_t* S; int ns, N, L, tid, nth;
  const int64_t* off; float* out;
};

static void* mts_worker(void* p) {
  struct mts_job* jb = (struct mts_job*)p;
  for (int s = 0; s < jb->ns; ++s) {
    const int i = jb->S[s];
    float* o = jb->out + jb->off[s];
    for (int j = i + 1 + jb->tid; j < jb->N; j += jb->nth) {
      float s3 = 0;
      for (int l = 0; l < jb->L; ++l) s3 += jb->bt[(size_t)i * jb->L + l] * jb->bt[(size_t)j * jb->L + l];
      float r = s3 / jb->m2[i] / jb->m2[j];
      if (jb->m2[i] == 0 || jb->m2[j] == 0) r = 0;
      o[j - i - 1] = r;
    }
  }
  return NULL;
}

static double orc_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int64_t orc_mt_rows_csr(const float* bt, const float* m2, int N, int L, const int32_t* S, int ns,
                        int mode, float tau, int nthreads, int32_t* R, int32_t* C, float* V,
                        int64_t cap, double* secs) {
  const double t0 = orc_now();
  int64_t* off = (int64_t*)malloc(sizeof(int64_t) * ((size_t)ns + 1));
  int32_t* pos = (int32_t*)malloc(sizeof(int32_t) * (size_t)N); /* row -> sample slot or -1 */
  off[0] = 0;
  for (int s = 0; s < ns; ++s) off[s + 1] = off[s] + (N - 1 - S[s]);
  for (int i = 0; i < N; ++i) pos[i] = -1;
  for (int s = 0; s < ns; ++s) pos[S[s]] = s;
  float* rs = (float*)malloc(sizeof(float) * ((size_t)off[ns] + 1));
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  struct mts_job jobs[256];
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = (struct mts_job){bt, m2, S, ns, N, L, t, nthreads, off, rs};
    if (t > 0) pthread_create(&th[t], NULL, mts_worker, &jobs[t]);
  }
  mts_worker(&jobs[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  const double t1 = orc_now();
  /* FormFullGraph on the sample: rows of S at full width, other rows' columns at S */
  unsigned char* rows = (unsigned char*)malloc((size_t)ns * N);
  unsigned char* cols = (unsigned char*)malloc((size_t)N * ns);
  memset(rows, 0, (size_t)ns * N);
  memset(cols, 0, (size_t)N * ns);
  for (int s = 0; s < ns; ++s) {
    const int i = S[s];
    const float* o = rs + off[s];
    for (int j = i + 1; j < N; ++j) {
      if (!is_edge(o[j - i - 1], mode, tau)) continue;
      rows[(size_t)s * N + j] = 1;
      if (pos[j] >= 0) rows[(size_t)pos[j] * N + i] = 1;
      else cols[(size_t)j * ns + s] = 1;
    }
  }
  const double t2 = orc_now();
  /* FormCSRGraph: row-major scan; a value is the pair's r from the sample */
  int64_t nnz = 0;
  R[0] = 0;
  for (int i = 0; i < N; ++i) {
    if (pos[i] >= 0) {
      const unsigned char* a = rows + (size_t)pos[i] * N;
      for (int j = 0; j < N; ++j) {
        if (!a[j]) continue;
        if (nnz < cap) {
          C[nnz] = j;
          if (V) V[nnz] = i < j ? rs[off[pos[i]] + (j - i - 1)] : rs[off[pos[j]] + (i - j - 1)];
        }
        ++nnz;
      }
    } else {
      const unsigned char* a = cols + (size_t)i * ns;
      for (int s = 0; s < ns; ++s) {
        if (!a[s]) continue;
        if (nnz < cap) {
          C[nnz] = S[s];
          if (V) V[nnz] = rs[off[s] + (i - S[s] - 1)];
        }
        ++nnz;
      }
    }
    R[i + 1] = (int32_t)nnz;
  }
  const double t3 = orc_now();
  if (secs) {
    secs[0] = t1 - t0;
    secs[1] = t2 - t1;
    secs[2] = t3 - t2;
  }
  free(rows);
  free(cols);
  free(rs);
  free(pos);
  free(off);
  return nnz <= cap ? nnz : -nnz - 1;
}
