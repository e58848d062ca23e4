// Eigenvector centrality by power iteration on the device-resident CSR.
//
// Reference: Lead_Vector_GPU (W/CUEC/weighted-net.cu:55-221), whose loop
// (:154-189) per iteration does u0 = u; lambda = ||u||; u = u / lambda;
// u = A u (cusparseDcsrmv); e1 = ||u - u0||; e2 = ||u + u0|| with three
// blocking host reductions.  Here one kernel does a whole iteration:
//   lambda = sqrt(sum u^2)   (sum produced by the previous iteration)
//   y_i    = (sum_k val_k * u[col_k]) / lambda
//   partial sums of y^2, (y - u)^2, (y + u)^2 per block
// and the last block to finish reduces the partials in a fixed order, so the
// iteration is deterministic.  A device flag stops later launches once
// e1 <= eps or e2 <= eps (no host round trip per iteration); the host replays
// a captured CUDA graph of 32 iterations and reads the flag between graphs.
//
// Normally the whole power iteration is one cooperative, persistent launch
// (ec_coop_kernel): blocks meet at a grid barrier once per iteration and
// every block then reduces the block partials in the same fixed order, so no
// launch, tail or host round trip separates the iterations; graphs with many
// iterations (a graph that never meets the stop test runs the reference's
// 10,000) cost microseconds per iteration.  The per-iteration kernel above
// remains for the no-allocation entry point.
//
// The SpMV runs in float-float ("double-float") arithmetic instead of FP64,
// whose rate on this GPU is ~1/70 of FP32: the iterate is kept twice, as
// double (norms, convergence test, output) and as a (hi, lo) float pair for
// the gather; each product val * (hi + lo) is split exactly with an FMA
// (TwoProduct, Dekker 1971 / Ogita-Rump-Oishi 2005) and summed with Knuth's
// TwoSum, so a row sum carries about 48 significant bits (relative error
// ~2^-38 for rows of ~1000 entries), far inside the 1e-5 tolerance against
// the FP64 reference.  Row results, norms and the stop test stay in FP64.
#include <cmath>

#include "common.cuh"

namespace bna {

struct EcState {
  double lam2;        // sum of squares of the current iterate
  double lambda_used; // lambda of the last completed iteration (the returned eigenvalue)
  double e1, e2;
  int iter;           // completed iterations
  int done;
  unsigned int counter;
  int err;                // bounded grid barrier expired (persistent kernel)
  unsigned int bar_count, bar_gen;  // grid barrier of the persistent kernel
  double tot[5];          // persistent kernel: lam2, e1, e2, lambda, 1/lambda published by
                          // the last block to reach the barrier
};

constexpr int kEcThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Fixed-order reduction of `parts` (nparts x 3) by one block; results to out[3].
__device__ __forceinline__ void reduce_partials(const double* parts, int nparts, double* out) {
  __shared__ double red[kEcThreads][3];
  double s0 = 0, s1 = 0, s2 = 0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
    s0 += parts[b * 3 + 0];
    s1 += parts[b * 3 + 1];
    s2 += parts[b * 3 + 2];
  }
  red[threadIdx.x][0] = s0;
  red[threadIdx.x][1] = s1;
  red[threadIdx.x][2] = s2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[threadIdx.x][0] += red[threadIdx.x + w][0];
      red[threadIdx.x][1] += red[threadIdx.x + w][1];
      red[threadIdx.x][2] += red[threadIdx.x + w][2];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = red[0][0];
    out[1] = red[0][1];
    out[2] = red[0][2];
  }
}

__device__ __forceinline__ bool last_block_arrives(EcState* st) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(&st->counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// (hi, lo) float pair of a double: hi = RN(x), lo = RN(x - hi).
__device__ __forceinline__ float2 split_df(double x) {
  const float hi = __double2float_rn(x);
  return make_float2(hi, __double2float_rn(x - (double)hi));
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__global__ __launch_bounds__(kEcThreads) void ec_init_kernel(int n, double* u, float2* uf,
                                                             double* parts, EcState* st,
                                                             int max_iter) {
  __shared__ double ws[kEcThreads / 32];
  double s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = (double)i;  // init_AD, weighted-net.cu:38-43
    u[i] = v;
    uf[i] = split_df(v);
    s += v * v;
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < kEcThreads / 32; ++w) t += ws[w];
    parts[blockIdx.x * 3 + 0] = t;
    parts[blockIdx.x * 3 + 1] = 0;
    parts[blockIdx.x * 3 + 2] = 0;
  }
  if (last_block_arrives(st)) {
    __shared__ double tot[3];
    reduce_partials(parts, gridDim.x, tot);
    if (threadIdx.x == 0) {
      st->lam2 = tot[0];
      st->lambda_used = 0;
      st->e1 = 1;
      st->e2 = 1;
      st->iter = 0;
      st->done = (max_iter <= 0) ? 1 : 0;
      st->counter = 0;
    }
  }
}

// One nonzero: (sh, sl) += v * (x.hi + x.lo), v given as (vh, vl) (vl = 0 for float values).
template <int VK>
__device__ __forceinline__ void df_accum(float& sh, float& sl, float vh, float vl, float2 x) {
  float p, pe;
  if (VK == 0) {  // binary graph: v = 1
    p = x.x;
    pe = x.y;
  } else {
    p = __fmul_rn(vh, x.x);
    pe = __fmaf_rn(vh, x.x, -p);  // exact low part of vh * x.hi
    pe = __fmaf_rn(vh, x.y, pe);
    if (VK == 2) pe = __fmaf_rn(vl, x.x, pe);
  }
  float s, e;
  two_sum(sh, p, s, e);
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(e, pe));
}

// One warp, one row: (sh, sl) += sum over entries [b, e) of val * x[col], eight
// entries per lane in flight per round (predicated, so a row costs
// ceil((e - b) / 256) memory round trips).  l2_only: read x through L2 only
// (the persistent kernel, whose iterate other blocks rewrite in the same launch).
template <int VK>
__device__ __forceinline__ void ec_row_accum(const int32_t* __restrict__ ci,
                                             const float* __restrict__ val,
                                             const double* __restrict__ vald,
                                             const float2* uf, long long b, long long e,
                                             int lane, float& sh, float& sl, bool l2_only) {
  for (long long k0 = b; k0 < e; k0 += 256) {
    int c[8];
    float vh[8], vl[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const long long k = k0 + lane + 32 * m;
      const bool ok = k < e;
      c[m] = ok ? __ldg(ci + k) : -1;
      vh[m] = 1.0f;
      vl[m] = 0.0f;
      if (VK == 1) vh[m] = ok ? __ldg(val + k) : 0.0f;
      if (VK == 2) {
        const float2 d = split_df(ok ? __ldg(vald + k) : 0.0);
        vh[m] = d.x;
        vl[m] = d.y;
      }
    }
    float2 x[8];
#pragma unroll
    for (int m = 0; m < 8; ++m)
      x[m] = c[m] < 0 ? make_float2(0.0f, 0.0f) : (l2_only ? __ldcg(uf + c[m]) : uf[c[m]]);
#pragma unroll
    for (int m = 0; m < 8; ++m) df_accum<VK>(sh, sl, vh[m], vl[m], x[m]);
  }
}

// Rounds per batch: round k of a block covers rows blockIdx.x * 8 + k * (all
// warps) .. + 7, one per warp (the interleaving spreads dense row ranges over
// every block); the batch's float-float row sums wait in shared memory for the
// thread-per-row FP64 epilogue, one thread per row.
constexpr int kEcRounds = kEcThreads / (kEcThreads / 32);

// One iteration's work of this block: warp per row for the float-float sums,
// then one thread per row for the FP64 epilogue (y = sum / lambda, the
// iterate copies, the partial sums of y^2, (y - u)^2, (y + u)^2).  The FP64
// pipe of this GPU is narrow and a warp instruction costs it the same with
// one lane as with 32, so the FP64 work runs on full warps instead of on
// lane 0 of every row's warp.
template <int VK>
__device__ __forceinline__ void ec_block_rows(int n, const int32_t* __restrict__ rp,
                                              const int32_t* __restrict__ ci,
                                              const float* __restrict__ val,
                                              const double* __restrict__ vald, long long nnz_used,
                                              const double* uc, const float2* ufc, double* un,
                                              float2* unf, double inv, bool l2_only, double& a0,
                                              double& a1, double& a2) {
  constexpr int kW = kEcThreads / 32;
  __shared__ float2 rs[kEcThreads];
  __shared__ bool rempty[kEcThreads];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = gridDim.x * kW;
  for (long long base = (long long)blockIdx.x * kW; base < n; base += (long long)kEcRounds * nw) {
    for (int k = 0; k < kEcRounds; ++k) {
      const long long row = base + (long long)k * nw + warp;
      if (row >= n) break;  // later rounds of this warp are past n too
      long long b = __ldg(rp + row), e = __ldg(rp + row + 1);
      if (e > nnz_used) e = nnz_used;
      float sh = 0.0f, sl = 0.0f;
      ec_row_accum<VK>(ci, val, vald, ufc, b, e, lane, sh, sl, l2_only);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, sh, o);
        const float ol = __shfl_xor_sync(0xffffffffu, sl, o);
        float s2, e2;
        two_sum(sh, oh, s2, e2);
        sh = s2;
        sl = __fadd_rn(sl, __fadd_rn(ol, e2));
      }
      if (lane == 0) {
        rs[k * kW + warp] = make_float2(sh, sl);
        rempty[k * kW + warp] = e <= b;
      }
    }
    __syncthreads();
    {
      const int k = threadIdx.x / kW, w = threadIdx.x % kW;
      const long long row = base + (long long)k * nw + w;
      if (row < n) {
        // y = A (u / lambda) as the reference orders it (weighted-net.cu:160-167):
        // a row without entries gives 0 even when 1 / lambda is infinite (an
        // all-zero iterate), where sum * (1 / lambda) would give 0 * inf = NaN
        const float2 sm = rs[threadIdx.x];
        const double y = rempty[threadIdx.x] ? 0.0 : ((double)sm.x + (double)sm.y) * inv;
        const double old = l2_only ? __ldcg(uc + row) : uc[row];
        un[row] = y;
        unf[row] = split_df(y);
        a0 += y * y;
        const double d = y - old, p = y + old;
        a1 += d * d;
        a2 += p * p;
      }
    }
    __syncthreads();
  }
}

// The same iteration's work for a sparse graph (average degree <= 2, the
// graphs whose centrality converges slowly or never): one thread per row
// (the epilogue's row), its few entries summed in order in float-float, so a
// warp does not walk ~20 nearly empty rows one after another; a row of more
// than kEcSparseRow entries is summed by the whole warp as above.
constexpr int kEcSparseRow = 32;

template <int VK>
__device__ __forceinline__ void ec_block_rows_sparse(int n, const int32_t* __restrict__ rp,
                                                     const int32_t* __restrict__ ci,
                                                     const float* __restrict__ val,
                                                     const double* __restrict__ vald,
                                                     long long nnz_used, const double* uc,
                                                     const float2* ufc, double* un, float2* unf,
                                                     double inv, double& a0, double& a1,
                                                     double& a2) {
  constexpr int kW = kEcThreads / 32;
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * kW;
  const int k = threadIdx.x / kW, w = threadIdx.x % kW;
  for (long long base = (long long)blockIdx.x * kW; base < n; base += (long long)kEcRounds * nw) {
    const long long row = base + (long long)k * nw + w;
    long long b = 0, e = 0;
    if (row < n) {
      b = __ldg(rp + row);
      e = __ldg(rp + row + 1);
      if (e > nnz_used) e = nnz_used;
      if (b > e) b = e;
    }
    float sh = 0.0f, sl = 0.0f;
    const bool wide = e - b > kEcSparseRow;
    if (!wide) {
#pragma unroll 4
      for (long long q = b; q < e; ++q) {
        float vh = 1.0f, vl = 0.0f;
        if (VK == 1) vh = __ldg(val + q);
        if (VK == 2) {
          const float2 d = split_df(__ldg(vald + q));
          vh = d.x;
          vl = d.y;
        }
        df_accum<VK>(sh, sl, vh, vl, ufc[__ldg(ci + q)]);
      }
    }
    // wide rows: the warp sums each of them together (every lane takes part)
    for (unsigned m = __ballot_sync(0xffffffffu, wide); m; m &= m - 1) {
      const int src = __ffs(m) - 1;
      const long long wb = __shfl_sync(0xffffffffu, b, src), we = __shfl_sync(0xffffffffu, e, src);
      float wh = 0.0f, wl = 0.0f;
      ec_row_accum<VK>(ci, val, vald, ufc, wb, we, lane, wh, wl, false);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, wh, o);
        const float ol = __shfl_xor_sync(0xffffffffu, wl, o);
        float s2, e2;
        two_sum(wh, oh, s2, e2);
        wh = s2;
        wl = __fadd_rn(wl, __fadd_rn(ol, e2));
      }
      if (lane == src) {
        sh = wh;
        sl = wl;
      }
    }
    if (row < n) {
      // as ec_block_rows: a row without entries gives 0 (weighted-net.cu:160-167)
      const double y = e <= b ? 0.0 : ((double)sh + (double)sl) * inv;
      const double old = uc[row];
      un[row] = y;
      unf[row] = split_df(y);
      a0 += y * y;
      const double d = y - old, p = y + old;
      a1 += d * d;
      a2 += p * p;
    }
  }
}

// Block sums of the three partials (warp butterflies over the first aw warps,
// then a butterfly over the warps' sums in warp 0) into parts[blockIdx.x * 3 ..].
__device__ __forceinline__ void ec_block_partials(double a0, double a1, double a2, int aw,
                                                  double* parts) {
  __shared__ double ws[kEcThreads / 32][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < aw) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
      ws[warp][0] = a0;
      ws[warp][1] = a1;
      ws[warp][2] = a2;
    }
  }
  __syncthreads();
  if (warp == 0) {  // the warps' sums by a butterfly (a dependent FP64 add costs ~0.3 us here)
    double t0 = lane < aw ? ws[lane][0] : 0.0;
    double t1 = lane < aw ? ws[lane][1] : 0.0;
    double t2 = lane < aw ? ws[lane][2] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      t0 += __shfl_xor_sync(0xffffffffu, t0, o);
      t1 += __shfl_xor_sync(0xffffffffu, t1, o);
      t2 += __shfl_xor_sync(0xffffffffu, t2, o);
    }
    if (lane == 0) {
      parts[blockIdx.x * 3 + 0] = t0;
      parts[blockIdx.x * 3 + 1] = t1;
      parts[blockIdx.x * 3 + 2] = t2;
    }
  }
}

// VK: 0 binary (val NULL), 1 float values, 2 double values (split into a float pair).
// SPARSE: rows by ec_block_rows_sparse.
template <int VK, bool SPARSE = false>
__global__ __launch_bounds__(kEcThreads, 4) void ec_iter_kernel(
    int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
    const float* __restrict__ val, const double* __restrict__ vald, long long nnz_used,
    const double* __restrict__ u, const float2* __restrict__ uf, double* __restrict__ un,
    float2* __restrict__ unf, double* parts, EcState* st, int max_iter, double eps) {
  if (st->done || st->iter >= max_iter) return;
  // lambda and its reciprocal once per block (FP64 sqrt and division are
  // long instruction sequences on this GPU), shared through shared memory
  __shared__ double lam_s[2];
  if (threadIdx.x == 0) {  // 1 / lambda and lambda from one reciprocal square root
    const double l2 = st->lam2;
    lam_s[1] = rsqrt(l2);
    lam_s[0] = l2 == 0.0 ? 0.0 : l2 * lam_s[1];  // sqrt(0) = 0, 1 / 0 = inf
  }
  __syncthreads();
  const double lam = lam_s[0];
  const double inv = lam_s[1];
  double a0 = 0, a1 = 0, a2 = 0;
  if (SPARSE)
    ec_block_rows_sparse<VK>(n, rp, ci, val, vald, nnz_used, u, uf, un, unf, inv, a0, a1, a2);
  else
    ec_block_rows<VK>(n, rp, ci, val, vald, nnz_used, u, uf, un, unf, inv, false, a0, a1, a2);
  ec_block_partials(a0, a1, a2, kEcThreads / 32, parts);
  if (last_block_arrives(st)) {
    __shared__ double tot[3];
    reduce_partials(parts, gridDim.x, tot);
    if (threadIdx.x == 0) {
      st->lambda_used = lam;
      st->lam2 = tot[0];
      st->e1 = sqrt(tot[1]);
      st->e2 = sqrt(tot[2]);
      st->iter += 1;
      if (st->e1 <= eps || st->e2 <= eps) st->done = 1;
      st->counter = 0;
    }
  }
}

// ---- column-chunked form -------------------------------------------------------
//
// For graphs whose iterate does not stay in L1 (random graphs of tens of
// thousands of vertices), the (hi, lo) iterate gathers of ec_iter_kernel miss
// L1 and pull a 32-byte L2 sector per 8-byte entry.  Here one 1024-thread block
// per SM stages the iterate in shared memory a chunk of kEcChunkCols columns
// at a time and gathers from there; each row's entries are split at the chunk
// boundaries once per CSR (columns ascending within a row), and a row's
// partial sum is carried from chunk to chunk in float-float.  Rows go to blocks
// in contiguous ranges balanced by entries (plus a per-row weight); the FP64
// epilogue, the block partials and the last-block reduction follow
// ec_iter_kernel's, in a fixed order.
constexpr int kEcChunkThreads = 1024;
constexpr int kEcChunkCols = 24576;  // 192 KB of (hi, lo) pairs
constexpr int kEcChunkRowsSmem = 3072;  // 24 KB of row sums beside them
constexpr int kEcRowWeight = 32;     // entries a row costs in the block split

// One warp, one row: eight entries per lane in flight per round of 256.
template <int VK>
__device__ __forceinline__ void ec_row_accum_smem(const int32_t* __restrict__ ci,
                                                  const float* __restrict__ val,
                                                  const double* __restrict__ vald,
                                                  const float2* xs, int c0, long long b,
                                                  long long e, int lane, float& sh, float& sl) {
  for (long long k0 = b; k0 < e; k0 += 256) {
    int c[8];
    float vh[8], vl[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const long long k = k0 + lane + 32 * m;
      const bool ok = k < e;
      c[m] = ok ? __ldg(ci + k) - c0 : -1;
      vh[m] = 1.0f;
      vl[m] = 0.0f;
      if (VK == 1) vh[m] = ok ? __ldg(val + k) : 0.0f;
      if (VK == 2) {
        const float2 d = split_df(ok ? __ldg(vald + k) : 0.0);
        vh[m] = d.x;
        vl[m] = d.y;
      }
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const float2 x = c[m] < 0 ? make_float2(0.0f, 0.0f) : xs[c[m]];
      df_accum<VK>(sh, sl, vh[m], vl[m], x);
    }
  }
}

template <int VK>
__global__ __launch_bounds__(kEcChunkThreads, 1) void ec_chunk_kernel(
    int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
    const float* __restrict__ val, const double* __restrict__ vald, long long nnz_used,
    const double* __restrict__ u, const float2* __restrict__ uf, double* __restrict__ un,
    float2* __restrict__ unf, double* parts, EcState* st, int max_iter, double eps,
    const int* __restrict__ rowsplit, const int* __restrict__ csplit, int nch,
    float2* __restrict__ part) {
  extern __shared__ __align__(16) float2 xs[];
  if (st->done || st->iter >= max_iter) return;
  __shared__ double lam_s[2];
  if (threadIdx.x == 0) {
    const double l2 = st->lam2;
    lam_s[1] = rsqrt(l2);
    lam_s[0] = l2 == 0.0 ? 0.0 : l2 * lam_s[1];
  }
  constexpr int kW = kEcChunkThreads / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = rowsplit[blockIdx.x], r1 = rowsplit[blockIdx.x + 1];
  // the block's row sums between chunks: shared memory when they fit
  float2* ps = xs + kEcChunkCols;
  const bool in_smem = r1 - r0 <= kEcChunkRowsSmem;
  for (int c = 0; c < nch; ++c) {
    const int c0 = c * kEcChunkCols;
    const int cn = min(kEcChunkCols, n - c0);
    __syncthreads();  // the previous chunk's readers are done
    // two pairs per 16-byte load when the chunk starts on a 16-byte boundary
    // (the second iterate buffer starts at uf + n: 8-byte aligned for odd n)
    if ((reinterpret_cast<uintptr_t>(uf + c0) & 15u) == 0) {
      const float4* src4 = reinterpret_cast<const float4*>(uf + c0);
      float4* dst4 = reinterpret_cast<float4*>(xs);
      for (int k = threadIdx.x; k < cn / 2; k += kEcChunkThreads) dst4[k] = src4[k];
      if ((cn & 1) && threadIdx.x == 0) xs[cn - 1] = uf[c0 + cn - 1];
    } else {
      for (int k = threadIdx.x; k < cn; k += kEcChunkThreads) xs[k] = uf[c0 + k];
    }
    __syncthreads();
    for (int row = r0 + warp; row < r1; row += kW) {
      long long b = c == 0 ? __ldg(rp + row) : __ldg(csplit + (size_t)(c - 1) * n + row);
      long long e = c == nch - 1 ? __ldg(rp + row + 1) : __ldg(csplit + (size_t)c * n + row);
      if (e > nnz_used) e = nnz_used;
      if (b >= e && c > 0) continue;  // nothing of this row in this chunk
      float sh = 0.0f, sl = 0.0f;
      if (b < e) ec_row_accum_smem<VK>(ci, val, vald, xs, c0, b, e, lane, sh, sl);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, sh, o);
        const float ol = __shfl_xor_sync(0xffffffffu, sl, o);
        float s2, e2;
        two_sum(sh, oh, s2, e2);
        sh = s2;
        sl = __fadd_rn(sl, __fadd_rn(ol, e2));
      }
      if (lane == 0) {
        float2* pr = in_smem ? &ps[row - r0] : &part[row];
        if (c > 0) {  // add to the row's sum of the earlier chunks
          const float2 p = *pr;
          float s2, e2;
          two_sum(p.x, sh, s2, e2);
          sh = s2;
          sl = __fadd_rn(__fadd_rn(p.y, sl), e2);
        }
        *pr = make_float2(sh, sl);
      }
    }
  }
  __syncthreads();  // every row's sum is in ps[] / part[]
  const double lam = lam_s[0], inv = lam_s[1];
  double a0 = 0, a1 = 0, a2 = 0;
  for (int row = r0 + (int)threadIdx.x; row < r1; row += kEcChunkThreads) {
    long long b = __ldg(rp + row), e = __ldg(rp + row + 1);
    if (e > nnz_used) e = nnz_used;
    const float2 sm = in_smem ? ps[row - r0] : part[row];
    // a row without entries gives 0 even when 1 / lambda is infinite
    const double y = e <= b ? 0.0 : ((double)sm.x + (double)sm.y) * inv;
    const double old = u[row];
    un[row] = y;
    unf[row] = split_df(y);
    a0 += y * y;
    const double d = y - old, p = y + old;
    a1 += d * d;
    a2 += p * p;
  }
  // block partials: warp butterflies, then the warps' sums by warp 0
  __shared__ double ws[kW][3];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
  }
  if (lane == 0) {
    ws[warp][0] = a0;
    ws[warp][1] = a1;
    ws[warp][2] = a2;
  }
  __syncthreads();
  if (warp == 0) {
    double t0 = ws[lane][0], t1 = ws[lane][1], t2 = ws[lane][2];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      t0 += __shfl_xor_sync(0xffffffffu, t0, o);
      t1 += __shfl_xor_sync(0xffffffffu, t1, o);
      t2 += __shfl_xor_sync(0xffffffffu, t2, o);
    }
    if (lane == 0) {
      parts[blockIdx.x * 3 + 0] = t0;
      parts[blockIdx.x * 3 + 1] = t1;
      parts[blockIdx.x * 3 + 2] = t2;
    }
  }
  // the last block to finish reduces the blocks' partials (warp 0: strided
  // sums per lane, then a butterfly; a fixed order)
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(&st->counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (warp == 0) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int b = lane; b < (int)gridDim.x; b += 32) {
      t0 += __ldcg(parts + b * 3 + 0);
      t1 += __ldcg(parts + b * 3 + 1);
      t2 += __ldcg(parts + b * 3 + 2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      t0 += __shfl_xor_sync(0xffffffffu, t0, o);
      t1 += __shfl_xor_sync(0xffffffffu, t1, o);
      t2 += __shfl_xor_sync(0xffffffffu, t2, o);
    }
    if (lane == 0) {
      st->lambda_used = lam;
      st->lam2 = t0;
      st->e1 = sqrt(t1);
      st->e2 = sqrt(t2);
      st->iter += 1;
      if (st->e1 <= eps || st->e2 <= eps) st->done = 1;
      st->counter = 0;
    }
  }
}

// Columns ascending within every row and inside [0, n) (the chunked form
// needs both: its gathers index the staged chunk): info[0] = 1 if some row
// breaks either; and the gathers' locality: info[1] = the
// entries whose iterate pair lies in another 32-byte sector than the row's
// previous entry's (about every entry for a graph without column locality).
// Warp per row.
__global__ void ec_sorted_kernel(int n, const int32_t* __restrict__ rp,
                                 const int32_t* __restrict__ ci, long long nnz_used,
                                 unsigned long long* info) {
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  unsigned long long fresh = 0;
  bool bad = false;
  for (long long row = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); row < n;
       row += nw) {
    long long b = rp[row], e = rp[row + 1];
    if (e > nnz_used) e = nnz_used;
    for (long long k = b + lane; k < e; k += 32) {
      const int cur = ci[k];
      const int prev = k > b ? ci[k - 1] : -8;
      bad |= (k > b && cur <= prev) || cur < 0 || cur >= n;
      fresh += (cur >> 2) != (prev >> 2);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) fresh += __shfl_xor_sync(0xffffffffu, fresh, o);
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    if (bad) atomicOr(info, 1ull);
    if (fresh) atomicAdd(info + 1, fresh);
  }
}

// Chunk boundaries of every row: csplit[(c - 1) * n + row] = the first entry
// of the row with a column >= c * kEcChunkCols (binary search), c = 1..nch-1;
// and the block ranges: rowsplit[b] = the first row r with rp[r] + w r >=
// b (nnz_used + w n) / G.
__global__ void ec_split_kernel(int n, const int32_t* __restrict__ rp,
                                const int32_t* __restrict__ ci, long long nnz_used, int nch,
                                int* csplit, int G, int* rowsplit) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    const int row = (int)t;
    long long b = rp[row], e = rp[row + 1];
    if (e > nnz_used) e = nnz_used;
    if (b > e) b = e;
    for (int c = 1; c < nch; ++c) {
      const int col = c * kEcChunkCols;
      long long lo = b, hi = e;
      while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (ci[mid] < col) lo = mid + 1; else hi = mid;
      }
      csplit[(size_t)(c - 1) * n + row] = (int)lo;
    }
  }
  if (t <= G) {
    const double total = (double)nnz_used + (double)kEcRowWeight * n;
    const double want = total * (double)t / (double)G;
    int lo = 0, hi = n;
    while (lo < hi) {  // first r with min(rp[r], nnz_used) + w r >= want
      const int mid = (lo + hi) >> 1;
      const double f = (double)min((long long)rp[mid], nnz_used) + (double)kEcRowWeight * mid;
      if (f < want) lo = mid + 1; else hi = mid;
    }
    rowsplit[t] = t == G ? n : lo;
  }
}

// ---- persistent form ----------------------------------------------------------

// Grid barrier for a cooperative launch (all blocks co-resident).  Bounded:
// a wait longer than limit_ns gives up and returns false.
__device__ __forceinline__ bool grid_barrier(EcState* st, uint64_t limit_ns) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &st->bar_gen;
    const unsigned int g = *gen;  // the generation cannot advance before this block arrives
    __threadfence();
    int ok = 1;
    if (atomicAdd(&st->bar_count, 1u) == gridDim.x - 1) {
      st->bar_count = 0;
      __threadfence();
      atomicAdd(&st->bar_gen, 1u);
    } else {
      uint64_t t0;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      while (*gen == g) {
        uint64_t t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > limit_ns) {
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Grid barrier of the persistent kernel that also reduces the iteration's
// block partials pp (grid x 3): the last block to arrive sums them in a fixed
// order (thread-strided sums, then a shared-memory tree: the order of the
// per-iteration kernel's reduce_partials), publishes lam2, e1, e2 and the next
// iteration's lambda and 1/lambda in st->tot, and releases the others — each
// partial is read once, not once per block.  Bounded like grid_barrier.
__device__ __forceinline__ bool grid_sync_reduce(EcState* st, const double* pp,
                                                 uint64_t limit_ns) {
  __shared__ int last_s, ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &st->bar_gen;
    const unsigned int g = *gen;  // the generation cannot advance before this block arrives
    __threadfence();
    const bool last = atomicAdd(&st->bar_count, 1u) == gridDim.x - 1;
    last_s = last ? 1 : 0;
    ok_s = 1;
    if (!last) {
      uint64_t t0;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      while (*gen == g) {
        uint64_t t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > limit_ns) {
          ok_s = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  if (last_s) {
    __shared__ double red[kEcThreads][3];
    double s0 = 0, s1 = 0, s2 = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
      s0 += __ldcg(pp + b * 3 + 0);
      s1 += __ldcg(pp + b * 3 + 1);
      s2 += __ldcg(pp + b * 3 + 2);
    }
    red[threadIdx.x][0] = s0;
    red[threadIdx.x][1] = s1;
    red[threadIdx.x][2] = s2;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) {
        red[threadIdx.x][0] += red[threadIdx.x + w][0];
        red[threadIdx.x][1] += red[threadIdx.x + w][1];
        red[threadIdx.x][2] += red[threadIdx.x + w][2];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double r0 = red[0][0], inv = rsqrt(r0);
      st->tot[0] = r0;
      st->tot[1] = sqrt(red[0][1]);
      st->tot[2] = sqrt(red[0][2]);
      st->tot[3] = r0 == 0.0 ? 0.0 : r0 * inv;
      st->tot[4] = inv;
      st->bar_count = 0;
      __threadfence();
      atomicAdd(&st->bar_gen, 1u);
    }
    __syncthreads();
    return true;
  }
  if (!ok_s && threadIdx.x == 0) atomicOr(&st->err, 1);
  return ok_s != 0;
}

template <int VK>
__global__ __launch_bounds__(kEcThreads, 4) void ec_coop_kernel(
    int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
    const float* __restrict__ val, const double* __restrict__ vald, long long nnz_used,
    double* u, float2* uf, double* parts, EcState* st, int it_end, int max_iter, double eps) {
  // resume from the state block (ec_init_kernel's, or the previous segment's)
  double lam2 = st->lam2, lam_used = st->lambda_used, e1 = st->e1, e2 = st->e2;
  int it = st->iter;
  if (st->done) it_end = it;
  if (it_end > max_iter) it_end = max_iter;
  // lambda and its reciprocal for the first iteration (FP64 sqrt and division
  // are long instruction sequences on this GPU: one thread computes them)
  __shared__ double lam_s[2];
  if (threadIdx.x == 0) {
    lam_s[1] = rsqrt(lam2);
    lam_s[0] = lam2 == 0.0 ? 0.0 : lam2 * lam_s[1];
  }
  __syncthreads();
  double lam = lam_s[0], inv = lam_s[1];
  while (it < it_end) {
    const size_t cur = (size_t)(it & 1) * n, nxt = (size_t)((it + 1) & 1) * n;
    // the iterate was written by other blocks: read it from L2 (__ldcg), not L1
    double a0 = 0, a1 = 0, a2 = 0;
    ec_block_rows<VK>(n, rp, ci, val, vald, nnz_used, u + cur, uf + cur, u + nxt, uf + nxt, inv,
                      true, a0, a1, a2);
    double* pp = parts + (size_t)(it & 1) * gridDim.x * 3;
    ec_block_partials(a0, a1, a2, kEcThreads / 32, pp);
    if (!grid_sync_reduce(st, pp, 2000000000ull)) return;
    // the totals: published by the last block (L2 reads; the same bits everywhere)
    lam_used = lam;
    lam2 = __ldcg(&st->tot[0]);
    e1 = __ldcg(&st->tot[1]);
    e2 = __ldcg(&st->tot[2]);
    lam = __ldcg(&st->tot[3]);
    inv = __ldcg(&st->tot[4]);
    ++it;
    if (e1 <= eps || e2 <= eps) break;
  }
  // every block has read the state above before the first grid barrier; with
  // no iteration run, block 0 writes back what it read
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->lambda_used = lam_used;
    st->lam2 = lam2;
    st->e1 = e1;
    st->e2 = e2;
    st->iter = it;
    st->done = (e1 <= eps || e2 <= eps || it >= max_iter) ? 1 : 0;
  }
}

// The persistent kernel serves small graphs only (n <= kEcCoopMaxN), with at
// most one block per SM, so a long iteration (a graph that never meets the
// stop test runs 10,000 of them) occupies a small share of the GPU.  Larger
// graphs use per-iteration launches: their gathers then hit in L1, which the
// persistent kernel must bypass.  Returns 0 for "use per-iteration launches".
constexpr int kEcCoopMaxN = 16384;
int ec_coop_grid(int n, int sms) {
  if (n > kEcCoopMaxN) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ec_coop_kernel<1>, kEcThreads, 0) !=
          cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return 0;
  }
  const int want = (n + 8 * (kEcThreads / 32) - 1) / (8 * (kEcThreads / 32));
  return want < sms ? (want < 1 ? 1 : want) : sms;
}

// The power iteration from the state block's iteration up to it_end (the
// whole of it with it_end = max_iter): parts holds 2 * grid * 3 doubles.
cudaError_t launch_ec_coop(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, double* u, float2* uf,
                           double* parts, void* st, int grid, int it_end, int max_iter,
                           double eps, cudaStream_t stream) {
  EcState* s = (EcState*)st;
  void* args[] = {&n,     &rp, &ci, &val, &vald,   &nnz_used, &u,
                  &uf,    &parts, &s, &it_end, &max_iter, &eps};
  const void* fn = val    ? (const void*)ec_coop_kernel<1>
                   : vald ? (const void*)ec_coop_kernel<2>
                          : (const void*)ec_coop_kernel<0>;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kEcThreads), args, 0, stream);
}

size_t ec_state_bytes() { return sizeof(EcState); }

int ec_chunk_count(int n) { return (n + kEcChunkCols - 1) / kEcChunkCols; }

// The chunked form's preparation: rows sorted and gather locality (info, read
// by the caller), chunk splits and block ranges.  csplit: (nch - 1) x n ints; rowsplit:
// grid + 1 ints.
cudaError_t launch_ec_chunk_prep(int n, const int32_t* rp, const int32_t* ci, long long nnz_used,
                                 unsigned long long* info, int* csplit, int grid, int* rowsplit,
                                 cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(info, 0, 2 * sizeof(unsigned long long), stream);
  if (e != cudaSuccess) return e;
  const int blocks = (n + 7) / 8 < 4096 ? (n + 7) / 8 : 4096;
  ec_sorted_kernel<<<blocks > 0 ? blocks : 1, 256, 0, stream>>>(n, rp, ci, nnz_used, info);
  const long long cnt = (long long)n > grid + 1 ? n : grid + 1;
  ec_split_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, stream>>>(
      n, rp, ci, nnz_used, ec_chunk_count(n), csplit, grid, rowsplit);
  return cudaGetLastError();
}

// Shared-memory limit of the chunked kernels (set outside any capture).
cudaError_t prepare_ec_chunk() {
  const int smem = (kEcChunkCols + kEcChunkRowsSmem) * (int)sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(ec_chunk_kernel<0>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(ec_chunk_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(ec_chunk_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
  return e;
}

cudaError_t launch_ec_chunk(int n, const int32_t* rp, const int32_t* ci, const float* val,
                            const double* vald, long long nnz_used, const double* u,
                            const float2* uf, double* un, float2* unf, double* parts, void* st,
                            int grid, int max_iter, double eps, const int* rowsplit,
                            const int* csplit, float2* part, cudaStream_t stream) {
  const int nch = ec_chunk_count(n);
  const size_t smem = (size_t)(kEcChunkCols + kEcChunkRowsSmem) * sizeof(float2);
  if (val)
    ec_chunk_kernel<1><<<grid, kEcChunkThreads, smem, stream>>>(
        n, rp, ci, val, vald, nnz_used, u, uf, un, unf, parts, (EcState*)st, max_iter, eps,
        rowsplit, csplit, nch, part);
  else if (vald)
    ec_chunk_kernel<2><<<grid, kEcChunkThreads, smem, stream>>>(
        n, rp, ci, val, vald, nnz_used, u, uf, un, unf, parts, (EcState*)st, max_iter, eps,
        rowsplit, csplit, nch, part);
  else
    ec_chunk_kernel<0><<<grid, kEcChunkThreads, smem, stream>>>(
        n, rp, ci, val, vald, nnz_used, u, uf, un, unf, parts, (EcState*)st, max_iter, eps,
        rowsplit, csplit, nch, part);
  return cudaGetLastError();
}

cudaError_t launch_ec_init(int n, double* u, float2* uf, double* parts, void* st, int grid,
                           int max_iter, cudaStream_t stream) {
  ec_init_kernel<<<grid, kEcThreads, 0, stream>>>(n, u, uf, parts, (EcState*)st, max_iter);
  return cudaGetLastError();
}

cudaError_t launch_ec_iter(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, const double* u,
                           const float2* uf, double* un, float2* unf, double* parts, void* st,
                           int grid, int max_iter, double eps, cudaStream_t stream) {
  if (val)
    ec_iter_kernel<1><<<grid, kEcThreads, 0, stream>>>(n, rp, ci, val, vald, nnz_used, u, uf, un,
                                                       unf, parts, (EcState*)st, max_iter, eps);
  else if (vald)
    ec_iter_kernel<2><<<grid, kEcThreads, 0, stream>>>(n, rp, ci, val, vald, nnz_used, u, uf, un,
                                                       unf, parts, (EcState*)st, max_iter, eps);
  else
    ec_iter_kernel<0><<<grid, kEcThreads, 0, stream>>>(n, rp, ci, val, vald, nnz_used, u, uf, un,
                                                       unf, parts, (EcState*)st, max_iter, eps);
  return cudaGetLastError();
}

// launch_ec_iter for a graph of average degree <= 2 (rows by thread).
cudaError_t launch_ec_iter_sparse(int n, const int32_t* rp, const int32_t* ci, const float* val,
                                  const double* vald, long long nnz_used, const double* u,
                                  const float2* uf, double* un, float2* unf, double* parts,
                                  void* st, int grid, int max_iter, double eps,
                                  cudaStream_t stream) {
  if (val)
    ec_iter_kernel<1, true><<<grid, kEcThreads, 0, stream>>>(
        n, rp, ci, val, vald, nnz_used, u, uf, un, unf, parts, (EcState*)st, max_iter, eps);
  else if (vald)
    ec_iter_kernel<2, true><<<grid, kEcThreads, 0, stream>>>(
        n, rp, ci, val, vald, nnz_used, u, uf, un, unf, parts, (EcState*)st, max_iter, eps);
  else
    ec_iter_kernel<0, true><<<grid, kEcThreads, 0, stream>>>(
        n, rp, ci, val, vald, nnz_used, u, uf, un, unf, parts, (EcState*)st, max_iter, eps);
  return cudaGetLastError();
}

// Host view of the state block (same layout as EcState).
int ec_state_err(const void* host_copy) { return ((const EcState*)host_copy)->err; }

void ec_state_read(const void* host_copy, double* lam2, double* lambda_used, double* e1,
                   double* e2, int* iter, int* done) {
  const EcState* s = (const EcState*)host_copy;
  *lam2 = s->lam2;
  *lambda_used = s->lambda_used;
  *e1 = s->e1;
  *e2 = s->e2;
  *iter = s->iter;
  *done = s->done;
}

}  // namespace bna
