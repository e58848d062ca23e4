// Newman spectral modularity on the device-resident CSR (binary graph).
//
// Reference: the unweighted Newman modularity tool,
// U/Newman_Modularity_CPU/Modularity_CPU/Modularity_CPU.cpp — Partition
// (:173-240) divides the network round by round: round r takes the nodes
// labelled r (mask G), Sub_Partition (:250-300) builds the integer diagonal
// term sumBG[i] = |adj(i) ∩ G| - floor(k_i * K_G / 2 / M) and Lead_Vector
// (:315-377) finds the leading eigenvector of the generalised modularity
// matrix B_G - beta*I by power iteration (v_0[i] = i on G; per step
// y = A_G v0 - (v0.k / 2 / M) k - (sumBG - beta) v0, v = y / |y|, stop when
// |v - v0| or |v + v0| <= 1e-6 or after 10,000 steps; eigenvalue = +-|y| by
// the sign of v*v0 at the first largest |v|).  A negative eigenvalue is
// retried with beta = -lambda; the round divides when lambda > LAMBDA and
// both signs hold more than one node.  Q (:215-224) is computed at the end.
//
// Rounds are the nodes of a binary division tree visited breadth first, so
// the groups of one tree level depend on nothing but their own nodes: here
// every level is one cooperative, persistent launch (mod_level_kernel) in
// which each group owns a contiguous range of blocks and runs its whole
// Sub_Partition — sumBG, Lead_Vector, the retry, the sign rule and the sizes
// of the two sides — with barriers among its own blocks only (bounded waits).
// The host then takes the decisions in round order, which numbers the
// children exactly as the sequential loop does.
//
// Arithmetic: GB300's FP64 rate is ~1/64 of its FP32 rate and a dependent
// FP64 operation takes ~0.3 us, so a power step runs in float-float
// ("double-float": TwoSum, FMA TwoProduct) on the iterate kept as a (hi, lo)
// float pair: about 44-48 significant bits per operation, the same order as
// the reference's sequential FP64 sums.  The SpMV, the correction term, the
// normalisation, the norms, the stop test and the reductions (fixed order,
// so a run is deterministic) all use it; the final iterate is widened to
// double for the sign rule and the division.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace bna {

// One group (round) of a tree level.  Host-written: label .. kg; device-
// written: the rest.
struct ModGroup {
  int label;     // the round number (Result value) of the group
  int row_off;   // its nodes: rows[row_off, row_off + rows), ascending
  int rows;
  int blk0;      // its blocks: [blk0, blk0 + nblk) of the launch
  int nblk;
  int err;       // a bounded barrier wait expired
  long long kg;  // K_G = sum of the degrees of its nodes
  int iters[2];
  double resid[2];
  double lambda;
  long long subp, subn;
  int fbuf;      // buffer (0/1) of the final eigenvector iterate
  unsigned int bar_count, bar_gen;
  unsigned int arrive;  // blocks' arrivals at the summing barriers of this launch
};

constexpr int kModThreads = 1024;
constexpr int kModWarps = kModThreads / 32;
// Partial sums per block: slots 0-3 and 4-7 hold the sums of the summing
// barriers (start vector; a power step's |y|^2, y.k and the two norms) of
// even and odd barrier number, 8-11 the eigenvalue sign and side sizes.
constexpr int kModParts = 12;
// Groups of at most this many nodes keep their iterate ((hi, lo) floats) in
// shared memory during the gathers: 96 KB.
constexpr int kModStageMax = 12288;
// Dynamic shared memory a block may ask for (iterate stage + column slice).
constexpr int kModSmemMax = 200 * 1024;

// (hi, lo) float pair of a double: hi = RN(x), lo = RN(x - hi).
__device__ __forceinline__ float2 mod_split(double x) {
  const float hi = __double2float_rn(x);
  return make_float2(hi, __double2float_rn(x - (double)hi));
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void mod_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Float-float ("double-float") arithmetic for the per-node work of a power
// step: (hi, lo) pairs with |lo| <= ulp(hi) / 2, about 2^-44 relative per
// operation (Dekker 1971; TwoProduct by FMA).  The FP64 latency of this GPU
// (~0.3 us per dependent operation) made the FP64 form of these chains the
// largest part of a step.
__device__ __forceinline__ float2 ff_norm(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  float s, e;
  mod_two_sum(a.x, b.x, s, e);
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  return ff_norm(s, e);
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ float2 ff_mulf(float2 a, float f) {  // f exact in float
  const float p = __fmul_rn(a.x, f);
  float e = __fmaf_rn(a.x, f, -p);
  e = __fmaf_rn(a.y, f, e);
  return ff_norm(p, e);
}
__device__ __forceinline__ double ff_to_d(float2 a) { return (double)a.x + (double)a.y; }
// An integer of at most 2^48 in magnitude, exactly.
__device__ __forceinline__ float2 ff_from_ll(long long x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (long long)h));
}

// Float-float comparison a > b (both normalised).
__device__ __forceinline__ bool ff_gt(float2 a, float2 b) {
  return a.x > b.x || (a.x == b.x && a.y > b.y);
}

// 1 / sqrt(y) in float-float: rsqrtf's estimate r0 and one Newton step
// r1 = r0 + r0 (1 - y r0^2) / 2 (the correction is ~2^-22 relative, so float
// precision suffices for it).  y = 0 gives (inf, 0).
__device__ __forceinline__ float2 ff_rsqrt(float2 y) {
  const float r0 = rsqrtf(y.x);
  if (y.x == 0.0f || !isfinite(r0)) return make_float2(r0, 0.0f);
  const float2 t = ff_mulf(ff_mulf(y, r0), r0);            // y r0^2 ~ 1
  const float2 e = ff_add(make_float2(1.0f, 0.0f), ff_neg(t));  // 1 - y r0^2
  float h, l;
  mod_two_sum(r0, __fmul_rn(__fmul_rn(r0, e.x), 0.5f), h, l);
  return make_float2(h, l);
}

__device__ __forceinline__ float2 ff_shfl_xor(float2 a, int o) {
  return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}

// Block sum of W float-float values per thread (warp butterflies, then a
// butterfly over the warps' sums: a fixed order) into partial slots
// k0 .. k0 + W - 1 of this block and into tot for every thread.  Only the
// first `aw` warps can hold non-zero values; with one such warp the second
// butterfly is skipped.
template <int W>
__device__ __forceinline__ void block_partials_ff(float2 (&a)[W], float2* parts, int k0, int aw,
                                                  float2 (&tot)[W]) {
  __shared__ float2 wsf[kModWarps][W];
  __shared__ float2 btf[W];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < aw) {
#pragma unroll
    for (int w = 0; w < W; ++w)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a[w] = ff_add(a[w], ff_shfl_xor(a[w], o));
    if (lane == 0)
#pragma unroll
      for (int w = 0; w < W; ++w) wsf[warp][w] = a[w];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int w = 0; w < W; ++w) {
      float2 t = lane < aw ? wsf[lane][w] : make_float2(0.0f, 0.0f);
      if (aw > 1)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = ff_add(t, ff_shfl_xor(t, o));
      if (lane == 0) {
        parts[(size_t)blockIdx.x * kModParts + k0 + w] = t;
        btf[w] = t;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int w = 0; w < W; ++w) tot[w] = btf[w];
}

// Barrier among the nb blocks of one group (all co-resident: cooperative
// launch).  Bounded: a wait longer than limit_ns raises g->err and returns false.
__device__ __forceinline__ bool group_barrier(ModGroup* g, int nb, uint64_t limit_ns) {
  __shared__ int ok_s;
  __syncthreads();
  if (nb == 1) return true;  // a group of one block: its own barrier suffices
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &g->bar_gen;
    const unsigned int g0 = *gen;  // cannot advance before this block arrives
    __threadfence();
    int ok = 1;
    if (atomicAdd(&g->bar_count, 1u) == (unsigned int)nb - 1) {
      g->bar_count = 0;
      __threadfence();
      atomicAdd(&g->bar_gen, 1u);
    } else {
      uint64_t t0;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      while (*gen == g0) {
        uint64_t t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > limit_ns) {
          ok = 0;
          atomicExch(&g->err, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Warps holding thread-per-position work for `cnt` positions.
__device__ __forceinline__ int active_warps(int cnt) {
  const int w = (cnt + 31) >> 5;
  return w < kModWarps ? w : kModWarps;
}

// Sum over the group's blocks [b0, b0 + nb) of float-float partial
// k0 .. k0 + W - 1 in a fixed order (thread-strided sums, warp butterflies, a
// butterfly over the warps' sums when more than one warp holds values), so
// the result does not depend on timing.  Every thread gets the totals.
template <int W>
__device__ __forceinline__ void group_reduce(const float2* parts, int b0, int nb, int k0,
                                             float2 (&out)[W]) {
  __shared__ float2 ws[kModWarps][W];
  __shared__ float2 tot[W];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 s[W];
#pragma unroll
  for (int w = 0; w < W; ++w) s[w] = make_float2(0.0f, 0.0f);
  for (int b = threadIdx.x; b < nb; b += kModThreads)
#pragma unroll
    for (int w = 0; w < W; ++w)
      s[w] = ff_add(s[w], __ldcg(parts + (size_t)(b0 + b) * kModParts + k0 + w));
  const int aw = active_warps(nb);
  if (warp < aw) {
#pragma unroll
    for (int w = 0; w < W; ++w)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s[w] = ff_add(s[w], ff_shfl_xor(s[w], o));
    if (lane == 0)
#pragma unroll
      for (int w = 0; w < W; ++w) ws[warp][w] = s[w];
  }
  __syncthreads();
  if (warp == 0)
#pragma unroll
    for (int w = 0; w < W; ++w) {
      float2 t = lane < aw ? ws[lane][w] : make_float2(0.0f, 0.0f);
      if (aw > 1)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = ff_add(t, ff_shfl_xor(t, o));
      if (lane == 0) tot[w] = t;
    }
  __syncthreads();
#pragma unroll
  for (int w = 0; w < W; ++w) out[w] = tot[w];
  __syncthreads();
}

// Induced subgraph of a tree level, built before its launch: positions p of
// the level's node list (groups contiguous, nodes ascending within a group);
// lrp / lci = the CSR of the edges whose ends share a group, columns as
// group-local indices (position - the group's first position), in the
// original column order.

// Edges of each position's node that stay inside its group (warp per position).
__global__ void mod_count_kernel(int nrows, const int32_t* __restrict__ rows,
                                 const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                 const int32_t* __restrict__ label, int32_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  for (int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); p < nrows;
       p += gridDim.x * (blockDim.x >> 5)) {
    const int i = rows[p], r = label[i];
    const int kb = rp[i], ke = rp[i + 1];
    int in = 0;
    for (int k = kb + lane; k < ke; k += 32) in += __ldg(label + __ldg(ci + k)) == r;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) in += __shfl_xor_sync(0xffffffffu, in, o);
    if (lane == 0) cnt[p] = in;
  }
}

// Exclusive scan of cnt[0, m) into out[0, m] by one block of 1024 threads
// (int64 running sums; the totals fit int32 since they are CSR entries).
__global__ __launch_bounds__(1024) void mod_scan_kernel(int m, const int32_t* __restrict__ cnt,
                                                        int32_t* __restrict__ out) {
  __shared__ long long tot[1024];
  const int per = (m + 1023) / 1024;
  const int b = threadIdx.x * per, e = min(m, b + per);
  long long s = 0;
  for (int k = b; k < e; ++k) s += cnt[k];
  tot[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan of the thread sums
    const long long v = threadIdx.x >= (unsigned)o ? tot[threadIdx.x - o] : 0;
    __syncthreads();
    tot[threadIdx.x] += v;
    __syncthreads();
  }
  long long run = threadIdx.x ? tot[threadIdx.x - 1] : 0;
  for (int k = b; k < e; ++k) {
    out[k] = (int32_t)run;
    run += cnt[k];
  }
  if (threadIdx.x == 1023) out[m] = (int32_t)tot[1023];
}

// Group-local columns of the in-group edges, original order (warp per
// position; ballot + prefix popcount place each lane's entry).
__global__ void mod_fill_kernel(int nrows, const int32_t* __restrict__ rows,
                                const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                const int32_t* __restrict__ label, const int32_t* __restrict__ loc,
                                const int32_t* __restrict__ lrp, int32_t* __restrict__ lci) {
  const int lane = threadIdx.x & 31;
  for (int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); p < nrows;
       p += gridDim.x * (blockDim.x >> 5)) {
    const int i = rows[p], r = label[i];
    const int kb = rp[i], ke = rp[i + 1];
    int pos = lrp[p];
    const int end = lrp[p + 1];
    for (int k0 = kb; k0 < ke; k0 += 32) {
      const int k = k0 + lane;
      const int j = k < ke ? __ldg(ci + k) : -1;
      const bool in = j >= 0 && __ldg(label + j) == r;
      const unsigned bal = __ballot_sync(0xffffffffu, in);
      const int at = pos + __popc(bal & ((1u << lane) - 1u));
      if (in && at < end) lci[at] = loc[j];
      pos += __popc(bal);
    }
  }
}

// Summing barrier number `epoch` (1, 2, ... in every block of the group, in
// the same sequence): the block's W float-float values go to its partial
// slots of the barrier's parity, the block counts its arrival, waits for the
// group's nb * epoch arrivals (bounded: a longer wait than limit_ns raises
// g->err and returns false) and then sums every block's partials itself in
// the group's fixed order, so all blocks hold the same totals.  Two slot sets
// suffice: a block can rewrite a set only after every block has arrived at
// the barrier in between, that is, after every block has read the set.
template <int W>
__device__ __forceinline__ bool group_sums(float2 (&a)[W], ModGroup* g, int nb, int b0, int aw,
                                           float2* parts, unsigned int& epoch, uint64_t limit_ns,
                                           float2 (&out)[W]) {
  __shared__ int ok_s;
  ++epoch;
  const int k0 = (int)(epoch & 1u) * 4;
  block_partials_ff<W>(a, parts, k0, aw, out);  // ends with __syncthreads
  if (nb == 1) return true;  // a group of one block takes its own totals
  if (threadIdx.x == 0) {
    const unsigned int target = (unsigned int)nb * epoch;
    __threadfence();  // the block's partials before its arrival
    int ok = 1;
    if (atomicAdd(&g->arrive, 1u) + 1u < target) {
      volatile unsigned int* c = &g->arrive;
      uint64_t t0;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      while (*c < target) {
        uint64_t t1;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        if (t1 - t0 > limit_ns) {
          ok = 0;
          atomicExch(&g->err, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  if (!ok_s) return false;
  group_reduce<W>(parts, b0, nb, k0, out);
  return true;
}

struct ModArgs {
  int n;
  long long M;
  const int32_t* rp;       // the graph's row pointers (degrees)
  const int32_t* label;
  const int32_t* rows;     // level positions -> nodes
  const int32_t* lrp;      // induced CSR of the level (positions)
  const int32_t* lci;      // group-local columns
  ModGroup* groups;
  const int32_t* blk_grp;  // group index of every block
  double* vd;              // [2][nrows] by position: the final and previous iterates in double;
                           // during the steps, the iterate of nodes without edges
  float2* vf;              // [2][nrows] iterate (hi, lo), by position
  float2* rs;              // [nrows] float-float row sums of a step
  double* y;               // [2][nrows] unnormalised iterates (hi, lo floats)
  double* parts;           // [grid][kModParts]
  int nrows;
  int stage_max;           // groups of at most this many nodes gather from shared memory
  int stage_bytes;         // offset of the column slice in dynamic shared memory
  int ecap;                // column-slice capacity (entries) in shared memory, 0: none
  int e16;                 // slice entries are 16-bit (every group below 65,536 nodes)
  int max_iter;
  double eps;
  uint64_t limit_ns;
};

// Column (group-local index) of in-group edge e: from the block's slice in
// shared memory (s16 / s32, first edge eb0) when it was loaded there.
__device__ __forceinline__ int edge_col(const ModArgs& a, const uint16_t* s16, const int32_t* s32,
                                        int eb0, int e) {
  return s16 ? (int)s16[e - eb0] : s32 ? s32[e - eb0] : __ldg(a.lci + e);
}

// One Lead_Vector call (Modularity_CPU.cpp:315-377) of group g with the
// given beta, run by the group's blocks; this block owns positions [p0, p1).
// Returns false when a barrier wait expired.  On return: *lambda,
// iterations, residual, final buffer (the final and the previous iterate
// in vd, double), the sizes of the two signs.
__device__ bool lead_vector(const ModArgs& a, ModGroup* g, int r, int b0, int nb, int p0, int p1,
                            long long kg, double beta, float2* stage, const uint16_t* s16,
                            const int32_t* s32, double* lambda, int* iters, double* resid,
                            int* fbuf, long long* subp, long long* subn, unsigned int& epoch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int off = g->row_off, nr = g->rows;
  const double Md = (double)a.M;
  const bool staged = stage != nullptr;
  const int eb0 = __ldg(a.lrp + p0);
  // v = (G ? i : 0) (:322-324); v.k for the first step
  float2 p1s[1] = {make_float2(0.0f, 0.0f)};
  // a single-block group keeps its staged iterate current itself (no reload per step)
  const bool self_stage = staged && nb == 1;
  float2* const yb = reinterpret_cast<float2*>(a.y);  // [2][nrows] unnormalised iterates y_s
  for (int p = p0 + (int)threadIdx.x; p < p1; p += kModThreads) {
    const int i = a.rows[p];
    const float2 x = ff_from_ll(i);
    a.vf[p] = x;
    a.vd[p] = (double)i;  // the double iterate of a node without edges
    yb[p] = x;  // y_0 = x_0 with 1 / |y_0| taken as 1
    if (self_stage) stage[p - off] = x;
    p1s[0] = ff_add(p1s[0], ff_mulf(ff_from_ll(i), (float)(a.rp[i + 1] - a.rp[i])));
  }
  const int aw = active_warps(p1 - p0);
  // per-step scalars, computed by one thread, and every sum of a step in
  // float-float: a dependent FP64 operation costs ~0.3 us on this GPU and
  // these chains sit between the group barriers
  __shared__ float2 scal_ff[3];
  const float2 nbeta = mod_split(-beta);
  // v_k / 2 / M as v_k * (0.5 / M); the stop test on squared norms (no
  // square root per step)
  const float2 half_inv_m = mod_split(0.5 / Md);
  const float2 eps2 = mod_split(a.eps * a.eps);
  float2* parts2 = reinterpret_cast<float2*>(a.parts);
  // a group of one block takes its own totals: no global barrier, no L2 round trip
  float2 t1[1];
  if (!group_sums<1>(p1s, g, nb, b0, aw, parts2, epoch, a.limit_ns, t1)) return false;
  // Power steps (:327-366) with one group barrier each.  Step s gathers the
  // unnormalised y_{s-1} (published before the previous barrier) and scales
  // the row sums by 1 / |y_{s-1}|, since A (y / |y|) = (A y) / |y|; it forms
  // x_{s-1} = y_{s-1} / |y_{s-1}| for its own positions, y_s, and the sums
  // |y_s|^2, y_s.k, |x_{s-1} -+ x_{s-2}|^2 in one reduction.  So the stop test
  // of iteration s - 1 (:358-361: the norms computed directly, as there) is
  // read one step later, and the step that revealed it is discarded.
  float2 inv = make_float2(1.0f, 0.0f);            // 1 / |y_{s-1}|
  float2 c = ff_mul(t1[0], half_inv_m);            // v_k / 2 / M of x_{s-1}
  float2 vn = make_float2(0.0f, 0.0f);             // |y_{s-1}|: the eigenvalue estimate
  float2 err1 = make_float2(1.0f, 0.0f), err2 = err1;  // of iteration s - 1
  int it = 0;  // iterations done: x_it is the current iterate
  for (int s = 1; a.max_iter > 0; ++s) {
    const size_t yprv = (size_t)((s - 1) & 1) * a.nrows, ycur = (size_t)(s & 1) * a.nrows;
    const size_t xcur = (size_t)((s - 1) & 1) * a.nrows, xold = (size_t)(s & 1) * a.nrows;
    const float2* ypc = yb + yprv + off;  // y_{s-1} of the group, group-local index
    if (staged && !self_stage) {
      for (int q = threadIdx.x; q < nr; q += kModThreads) stage[q] = __ldcg(ypc + q);
      __syncthreads();
    }
    // A_G y_{s-1} over the in-group edges (:342-343), float-float: warp per position
    for (int p = p0 + warp; p < p1; p += kModWarps) {
      const int eb = __ldg(a.lrp + p), ee = __ldg(a.lrp + p + 1);
      float sh = 0.0f, sl = 0.0f;
      for (int e0 = eb; e0 < ee; e0 += 128) {
        float2 x[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const int e = e0 + lane + 32 * m;
          const int q = e < ee ? edge_col(a, s16, s32, eb0, e) : -1;
          x[m] = q < 0 ? make_float2(0.0f, 0.0f) : (staged ? stage[q] : __ldcg(ypc + q));
        }
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          float t, e;
          mod_two_sum(sh, x[m].x, t, e);
          sh = t;
          sl = __fadd_rn(sl, __fadd_rn(e, x[m].y));
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, sh, o);
        const float ol = __shfl_xor_sync(0xffffffffu, sl, o);
        float t, e;
        mod_two_sum(sh, oh, t, e);
        sh = t;
        sl = __fadd_rn(sl, __fadd_rn(ol, e));
      }
      if (lane == 0) a.rs[p] = make_float2(sh, sl);
    }
    __syncthreads();
    // thread per position: x_{s-1} = y_{s-1} / |y_{s-1}| (:349-351), its
    // distances to x_{s-2} (:352-357), and y_s = A_G x_{s-1} - (v_k / 2 / M k
    // + (sumBG - beta) x_{s-1}) (:344); sumBG = |adj(i) ∩ G| - k K_G / 2 / M
    // in integers (:258-266)
    float2 pe[4] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f),
                    make_float2(0.0f, 0.0f)};
    for (int p = p0 + (int)threadIdx.x; p < p1; p += kModThreads) {
      const int i = a.rows[p];
      const long long k = a.rp[i + 1] - a.rp[i];
      if (k == 0) {
        // A node without edges: y = beta x (no gather term, sumBG = 0), so
        // under beta > 0 its entry shrinks by a factor per step and can fall
        // far below float's range while staying positive in the reference's
        // doubles (and so counted on the positive side).  Its iterate stays
        // in double (vd, by the parity of the float-float buffers).
        double xd = a.vd[p];  // x_0 = i
        if (s > 1) {
          const double xo = a.vd[xold + p];
          xd = __dmul_rn(__dmul_rn(beta, xo), ff_to_d(inv));
          a.vd[xcur + p] = xd;
          const double d = __dsub_rn(xd, xo), u = __dadd_rn(xd, xo);
          pe[2] = ff_add(pe[2], mod_split(__dmul_rn(d, d)));
          pe[3] = ff_add(pe[3], mod_split(__dmul_rn(u, u)));
        }
        const double yd = __dmul_rn(beta, xd);
        const float2 y = mod_split(yd);
        yb[ycur + p] = y;
        if (self_stage) stage[p - off] = y;
        pe[0] = ff_add(pe[0], mod_split(__dmul_rn(yd, yd)));
        continue;
      }
      const float2 x = s == 1 ? a.vf[p] : ff_mul(yb[yprv + p], inv);
      if (s > 1) {
        const float2 old = a.vf[xold + p];
        a.vf[xcur + p] = x;
        const float2 d = ff_add(x, ff_neg(old)), u = ff_add(x, old);
        pe[2] = ff_add(pe[2], ff_mul(d, d));
        pe[3] = ff_add(pe[3], ff_mul(u, u));
      }
      const float2 sbg =
          ff_from_ll((long long)(a.lrp[p + 1] - a.lrp[p]) - k * kg / 2 / a.M);
      const float2 corr = ff_add(ff_mulf(c, (float)k), ff_mul(ff_add(sbg, nbeta), x));
      const float2 y = ff_add(ff_mul(a.rs[p], inv), ff_neg(corr));
      yb[ycur + p] = y;
      if (self_stage) stage[p - off] = y;  // the gathers of this step are over
      pe[0] = ff_add(pe[0], ff_mul(y, y));
      pe[1] = ff_add(pe[1], ff_mulf(y, (float)k));
    }
    float2 te[4];
    if (!group_sums<4>(pe, g, nb, b0, aw, parts2, epoch, a.limit_ns, te)) return false;
    it = s - 1;
    if (s > 1) {
      err1 = te[2];
      err2 = te[3];
      if (!(ff_gt(err1, eps2) && ff_gt(err2, eps2) && it < a.max_iter)) break;
    }
    // VectorNorm (:383-389), its reciprocal and v_k / 2 / M of x_s, one thread
    if (threadIdx.x == 0) {
      const float2 r = ff_rsqrt(te[0]);
      scal_ff[0] = r;
      scal_ff[1] = te[0].x == 0.0f ? make_float2(0.0f, 0.0f) : ff_mul(te[0], r);  // sqrt(0) = 0
      scal_ff[2] = ff_mul(ff_mul(te[1], r), half_inv_m);
    }
    __syncthreads();
    inv = scal_ff[0];
    vn = scal_ff[1];
    c = scal_ff[2];
  }
  // eigenvalue sign (:369-375): the first node of G with the largest |v|
  // (node 0 when none exceeds |v[0]|, v[0] taken as 0 off G); side sizes (:276-281)
  const size_t fin = (size_t)(it & 1) * a.nrows, prv = (size_t)((it + 1) & 1) * a.nrows;
  for (int p = p0 + (int)threadIdx.x; p < p1; p += kModThreads) {
    const int i = a.rows[p];
    if (a.rp[i + 1] == a.rp[i]) continue;  // kept in double during the steps
    a.vd[fin + p] = ff_to_d(a.vf[fin + p]);
    a.vd[prv + p] = ff_to_d(a.vf[prv + p]);
  }
  double best = 0.0;
  int bq = 0x7fffffff;  // position of the maximum (positions ascend with node index)
  long long sp = 0, sn = 0;
  for (int p = p0 + (int)threadIdx.x; p < p1; p += kModThreads) {
    const double v = a.vd[fin + p];
    const double av = fabs(v);
    if (av > best) {  // ascending positions per thread: the first maximum is kept
      best = av;
      bq = p;
    }
    sp += v > 0;
    sn += v <= 0;
  }
  // warp butterflies (largest |v|, then the smaller position), warps in order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oq = __shfl_xor_sync(0xffffffffu, bq, o);
    if (ob > best || (ob == best && oq < bq)) {
      best = ob;
      bq = oq;
    }
    sp += __shfl_xor_sync(0xffffffffu, sp, o);
    sn += __shfl_xor_sync(0xffffffffu, sn, o);
  }
  __shared__ double sb[kModWarps];
  __shared__ int si[kModWarps];
  __shared__ long long sps[kModWarps], sns[kModWarps];
  if (lane == 0) {
    sb[warp] = best;
    si[warp] = bq;
    sps[warp] = sp;
    sns[warp] = sn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kModWarps; ++w) {
      if (sb[w] > sb[0] || (sb[w] == sb[0] && si[w] < si[0])) {
        sb[0] = sb[w];
        si[0] = si[w];
      }
      sps[0] += sps[w];
      sns[0] += sns[w];
    }
    double* pp = a.parts + (size_t)blockIdx.x * kModParts;
    pp[8] = sb[0];
    pp[9] = (double)si[0];
    pp[10] = (double)sps[0];  // counts < 2^53: exact in a double
    pp[11] = (double)sns[0];
  }
  if (!group_barrier(g, nb, a.limit_ns)) return false;
  double gb = 0.0;
  int gq = 0x7fffffff;
  long long gp = 0, gn = 0;
  for (int b = 0; b < nb; ++b) {  // fixed order, every block alike
    const double* pp = a.parts + (size_t)(b0 + b) * kModParts;
    const double ob = __ldcg(pp + 8);
    const int oi = (int)__ldcg(pp + 9);
    if (ob > gb || (ob == gb && oi < gq)) {
      gb = ob;
      gq = oi;
    }
    gp += (long long)__ldcg(pp + 10);
    gn += (long long)__ldcg(pp + 11);
  }
  double prod = 0.0;
  if (gb > 0.0) {
    prod = __ldcg(a.vd + fin + gq) * __ldcg(a.vd + prv + gq);
  } else if (__ldg(a.label) == r) {  // max_index stays 0, node 0 in G: its position is off
    prod = __ldcg(a.vd + fin + off) * __ldcg(a.vd + prv + off);
  }
  const double vnd = ff_to_d(vn);
  *lambda = prod > 0 ? vnd : -vnd;
  *iters = it;
  const double e1 = ff_to_d(err1), e2 = ff_to_d(err2);
  *resid = sqrt(e1 < e2 ? e1 : e2);
  *fbuf = it & 1;
  *subp = gp;
  *subn = gn;
  // the next call rewrites the iterate: wait until every block has read it
  return group_barrier(g, nb, a.limit_ns);
}

// One tree level: every group's Sub_Partition (Modularity_CPU.cpp:250-285)
// up to the division test, which the host takes in round order.
__global__ __launch_bounds__(kModThreads, 1) void mod_level_kernel(ModArgs a) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  const int gidx = a.blk_grp[blockIdx.x];
  ModGroup* g = a.groups + gidx;
  const int r = g->label, b0 = g->blk0, nb = g->nblk, lb = blockIdx.x - b0;
  const int off = g->row_off, nr = g->rows;
  const long long kg = g->kg;
  // this block's positions: an equal share of (positions + in-group edges)
  __shared__ int range_s[2];
  if (threadIdx.x < 2) {
    const long long e0 = a.lrp[off];
    const long long W = (long long)nr + (a.lrp[off + nr] - e0);
    const long long t = W * (lb + (int)threadIdx.x) / nb;
    int lo = 0, hi = nr;  // first q with q + lrp[off + q] - e0 >= t
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if ((long long)mid + (a.lrp[off + mid] - e0) >= t) hi = mid;
      else lo = mid + 1;
    }
    range_s[threadIdx.x] = off + lo;
  }
  __syncthreads();
  const int p0 = range_s[0], p1 = lb == nb - 1 ? off + nr : range_s[1];
  float2* stage = (nr <= a.stage_max) ? reinterpret_cast<float2*>(dyn_smem) : nullptr;
  // the block's in-group columns, kept in shared memory for the whole launch
  // when they fit (every power step reads them)
  const int eb0 = a.lrp[p0], ne = a.lrp[p1] - eb0;
  uint16_t* s16 = nullptr;
  int32_t* s32 = nullptr;
  if (ne <= a.ecap) {
    if (a.e16) {
      s16 = reinterpret_cast<uint16_t*>(dyn_smem + a.stage_bytes);
      for (int e = threadIdx.x; e < ne; e += kModThreads) s16[e] = (uint16_t)__ldg(a.lci + eb0 + e);
    } else {
      s32 = reinterpret_cast<int32_t*>(dyn_smem + a.stage_bytes);
      for (int e = threadIdx.x; e < ne; e += kModThreads) s32[e] = __ldg(a.lci + eb0 + e);
    }
  }
  __syncthreads();
  double lambda = 0, l2 = 0, res = 0;
  int its = 0, fb = 0;
  long long sp = 0, sn = 0;
  unsigned int epoch = 0;  // summing barriers passed (the same count in every block of the group)
  if (!lead_vector(a, g, r, b0, nb, p0, p1, kg, 0.0, stage, s16, s32, &lambda, &its, &res, &fb,
                   &sp, &sn, epoch))
    return;
  if (lb == 0 && threadIdx.x == 0) {
    g->iters[0] = its;
    g->resid[0] = res;
    g->iters[1] = 0;
    g->resid[1] = 0;
  }
  if (lambda < 0) {  // the leading eigenvalue of B - lambda I (:271-272)
    if (!lead_vector(a, g, r, b0, nb, p0, p1, kg, -lambda, stage, s16, s32, &l2, &its, &res, &fb,
                     &sp, &sn, epoch))
      return;
    lambda += l2;
    if (lb == 0 && threadIdx.x == 0) {
      g->iters[1] = its;
      g->resid[1] = res;
    }
  }
  if (lb == 0 && threadIdx.x == 0) {
    g->lambda = lambda;
    g->subp = sp;
    g->subn = sn;
    g->fbuf = fb;
  }
}

// A division (:285-287): the group's nodes go to base + 1 or base + 2 by the
// sign of v * (subP - subN + 0.5).
struct ModAssign {
  int row_off, rows, fbuf, base;
  double w;
};

__global__ void mod_assign_kernel(int nrows, const int32_t* __restrict__ rows,
                                  const ModAssign* __restrict__ as, int nas,
                                  const double* __restrict__ vd, int32_t* __restrict__ label) {
  for (int k = blockIdx.y; k < nas; k += gridDim.y) {
    const ModAssign s = as[k];
    const double* v = vd + (size_t)s.fbuf * nrows;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < s.rows; q += gridDim.x * blockDim.x) {
      const int p = s.row_off + q;
      label[rows[p]] = s.base + 1 + (v[p] * s.w <= 0 ? 1 : 0);
    }
  }
}

// Q's counts: directed entries inside a module (warp per row) and the degree
// sum of every module (labels < nlab), both integer.
__global__ void mod_q_kernel(int n, const int32_t* __restrict__ rp,
                             const int32_t* __restrict__ ci, const int32_t* __restrict__ label,
                             unsigned long long* __restrict__ kmod,
                             unsigned long long* __restrict__ same_out) {
  const int lane = threadIdx.x & 31;
  long long same = 0;
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n;
       i += gridDim.x * (blockDim.x >> 5)) {
    const int b = rp[i], e = rp[i + 1];
    const int li = label[i];
    for (int k = b + lane; k < e; k += 32) same += label[ci[k]] == li;
    if (lane == 0) atomicAdd(&kmod[li], (unsigned long long)(e - b));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) same += __shfl_xor_sync(0xffffffffu, same, o);
  if (lane == 0 && same) atomicAdd(same_out, (unsigned long long)same);
}

// Final labels: the consecutive module numbers of the rounds that stopped.
__global__ void mod_map_kernel(int n, const int32_t* __restrict__ label,
                               const int32_t* __restrict__ adj, int32_t* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = adj[label[i]];
}

// ---- host side -----------------------------------------------------------------

size_t mod_group_bytes() { return sizeof(ModGroup); }
size_t mod_assign_bytes() { return sizeof(ModAssign); }
int mod_parts_per_block() { return kModParts; }

// Blocks of mod_level_kernel that fit on the device at once (cooperative
// launch) with `smem` bytes of staged iterate per block.
int mod_level_grid(int sms, size_t smem) {
  if (cudaFuncSetAttribute(mod_level_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kModSmemMax) != cudaSuccess) {  // per device: set every call
    cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mod_level_kernel, kModThreads,
                                                    smem) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return 0;
  }
  return per_sm * sms;
}

int mod_stage_max() { return kModStageMax; }
int mod_smem_max() { return kModSmemMax; }

// Host view of a group record: host-written fields in, results out.
void mod_group_set(void* rec, int label, int row_off, int rows, int blk0, int nblk, long long kg) {
  ModGroup g{};
  g.label = label;
  g.row_off = row_off;
  g.rows = rows;
  g.blk0 = blk0;
  g.nblk = nblk;
  g.kg = kg;
  *(ModGroup*)rec = g;
}

void mod_group_get(const void* rec, int* err, int iters[2], double resid[2], double* lambda,
                   long long* subp, long long* subn, int* fbuf) {
  const ModGroup* g = (const ModGroup*)rec;
  *err = g->err;
  iters[0] = g->iters[0];
  iters[1] = g->iters[1];
  resid[0] = g->resid[0];
  resid[1] = g->resid[1];
  *lambda = g->lambda;
  *subp = g->subp;
  *subn = g->subn;
  *fbuf = g->fbuf;
}

void mod_assign_set(void* rec, int row_off, int rows, int fbuf, int base, double w) {
  ModAssign s{row_off, rows, fbuf, base, w};
  *(ModAssign*)rec = s;
}

cudaError_t launch_mod_build(int nrows, const int32_t* rows, const int32_t* rp,
                             const int32_t* ci, const int32_t* label, const int32_t* loc,
                             int32_t* cnt, int32_t* lrp, int32_t* lci, int sms, cudaStream_t s) {
  const int grid = (int)std::min<long long>(((long long)nrows + 7) / 8, (long long)sms * 16);
  mod_count_kernel<<<grid, 256, 0, s>>>(nrows, rows, rp, ci, label, cnt);
  mod_scan_kernel<<<1, 1024, 0, s>>>(nrows, cnt, lrp);
  mod_fill_kernel<<<grid, 256, 0, s>>>(nrows, rows, rp, ci, label, loc, lrp, lci);
  return cudaGetLastError();
}

cudaError_t launch_mod_level(int n, long long M, const int32_t* rp, const int32_t* label,
                             const int32_t* rows, const int32_t* lrp, const int32_t* lci,
                             void* groups, const int32_t* blk_grp, double* vd, float2* vf,
                             float2* rs, double* y, double* parts, int nrows, int stage_max,
                             int stage_bytes, int ecap, int e16, size_t smem, int grid,
                             int max_iter, double eps, cudaStream_t s) {
  ModArgs a{n,        M,           rp,   label, rows,  lrp,      lci,
            (ModGroup*)groups, blk_grp, vd, vf, rs,    y,        parts,
            nrows,    stage_max,   stage_bytes, ecap, e16, max_iter, eps,
            2000000000ull};
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)mod_level_kernel, dim3(grid), dim3(kModThreads),
                                     args, smem, s);
}

cudaError_t launch_mod_assign(int nrows, const int32_t* rows, const void* as, int nas,
                              const double* vd, int32_t* label, cudaStream_t s) {
  if (nas <= 0) return cudaSuccess;
  const int gy = nas < 65535 ? nas : 65535;
  mod_assign_kernel<<<dim3(8, gy), 256, 0, s>>>(nrows, rows, (const ModAssign*)as, nas, vd,
                                                label);
  return cudaGetLastError();
}

static int mod_grid(int n, int per_block, int sms) {
  const long long want = ((long long)n + per_block - 1) / per_block;
  const long long cap = (long long)sms * 8;
  return (int)(want < 1 ? 1 : want < cap ? want : cap);
}

cudaError_t launch_mod_q(int n, const int32_t* rp, const int32_t* ci, const int32_t* label,
                         unsigned long long* kmod, unsigned long long* same, int sms,
                         cudaStream_t s) {
  mod_q_kernel<<<mod_grid(n, 8, sms), 256, 0, s>>>(n, rp, ci, label, kmod, same);
  return cudaGetLastError();
}

cudaError_t launch_mod_map(int n, const int32_t* label, const int32_t* adj, int32_t* out,
                           int sms, cudaStream_t s) {
  mod_map_kernel<<<mod_grid(n, 256, sms), 256, 0, s>>>(n, label, adj, out);
  return cudaGetLastError();
}

}  // namespace bna
