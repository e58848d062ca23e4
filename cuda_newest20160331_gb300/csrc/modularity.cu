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
// the sign of v*v0 at the largest |v|).  A negative eigenvalue is retried
// with beta = -lambda; the round divides when lambda > LAMBDA and both signs
// hold more than one node.  Q (:215-224) is computed at the end.
//
// Here one round's steps are kernels: the mask and K_G, the integer sumBG,
// then per power step a warp-per-row SpMV (FP64; the correction term with
// the reference's operation order, no contraction) and an elementwise
// normalisation with fixed-order reductions of |y|^2, |v -+ v0|^2 and v.k;
// the steps are replayed from a CUDA graph and stop on a device flag.  The
// decisions (divide or not, new labels) are the reference's.
#include "common.cuh"

namespace bna {

struct ModState {
  double vk;     // sum over G of v0_i k_i for the next step
  double y2;     // |y|^2 of the current step
  double vnorm;  // |y| of the last completed step
  double err1, err2;
  double beta;
  double eps;
  double lambda;  // +-vnorm by the sign rule
  long long numg, kg;
  long long subp, subn;
  long long same;  // directed entries whose ends share a label (Q)
  int iter, done, max_iter;
  int maxi;
  unsigned int counter;
};

constexpr int kModThreads = 256;

__device__ __forceinline__ bool mod_last_block(ModState* st) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(&st->counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// Fixed-order sum of nparts x W partials by one block (all threads call).
template <int W>
__device__ __forceinline__ void mod_reduce(const double* parts, int nparts, double* out) {
  __shared__ double red[kModThreads][W];
  double s[W];
#pragma unroll
  for (int w = 0; w < W; ++w) s[w] = 0;
  for (int b = threadIdx.x; b < nparts; b += kModThreads)
#pragma unroll
    for (int w = 0; w < W; ++w) s[w] += parts[b * W + w];
#pragma unroll
  for (int w = 0; w < W; ++w) red[threadIdx.x][w] = s[w];
  __syncthreads();
  for (int h = kModThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
#pragma unroll
      for (int w = 0; w < W; ++w) red[threadIdx.x][w] += red[threadIdx.x + h][w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int w = 0; w < W; ++w) out[w] = red[0][w];
  __syncthreads();
}

template <int W>
__device__ __forceinline__ void mod_block_partials(double (&a)[W], double* parts) {
  __shared__ double ws[kModThreads / 32][W];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < W; ++w)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a[w] += __shfl_xor_sync(0xffffffffu, a[w], o);
  if (lane == 0)
#pragma unroll
    for (int w = 0; w < W; ++w) ws[warp][w] = a[w];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int w = 0; w < W; ++w) {
      double t = 0;
      for (int k = 0; k < kModThreads / 32; ++k) t += ws[k][w];
      parts[blockIdx.x * W + w] = t;
    }
}

// Round setup: G = (label == round), |G| and K_G = sum of degrees over G
// (integer atomics: exact in any order).  st->numg / kg zeroed by the host.
__global__ void mod_round_kernel(int n, const int32_t* __restrict__ label, int round,
                                 const int32_t* __restrict__ rp, uint8_t* __restrict__ g,
                                 ModState* st) {
  long long cnt = 0, deg = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool in = label[i] == round;
    g[i] = in ? 1 : 0;
    if (in) {
      ++cnt;
      deg += rp[i + 1] - rp[i];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    deg += __shfl_xor_sync(0xffffffffu, deg, o);
  }
  if ((threadIdx.x & 31) == 0 && cnt) {
    atomicAdd((unsigned long long*)&st->numg, (unsigned long long)cnt);
    atomicAdd((unsigned long long*)&st->kg, (unsigned long long)deg);
  }
}

// sumBG[i] = |adj(i) ∩ G| - k_i * K_G / 2 / M in integer arithmetic
// (Modularity_CPU.cpp:258-266), warp per row of G.
__global__ void mod_sumbg_kernel(int n, const int32_t* __restrict__ rp,
                                 const int32_t* __restrict__ ci, const uint8_t* __restrict__ g,
                                 long long M, const ModState* st, double* __restrict__ sumbg) {
  const int lane = threadIdx.x & 31;
  const long long kg = st->kg;
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n;
       i += gridDim.x * (blockDim.x >> 5)) {
    if (!g[i]) continue;
    const int b = rp[i], e = rp[i + 1];
    int in = 0;
    for (int k = b + lane; k < e; k += 32) in += g[ci[k]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) in += __shfl_xor_sync(0xffffffffu, in, o);
    if (lane == 0) sumbg[i] = (double)((long long)in - (long long)(e - b) * kg / 2 / M);
  }
}

// Start of a power iteration: v = (G ? i : 0), v.k, counters.
__global__ __launch_bounds__(kModThreads) void mod_init_kernel(
    int n, const uint8_t* __restrict__ g, const int32_t* __restrict__ rp, double* __restrict__ v,
    double* parts, ModState* st, double beta, int max_iter, double eps) {
  double a[1] = {0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double x = g[i] ? (double)i : 0.0;
    v[i] = x;
    if (g[i]) a[0] += x * (double)(rp[i + 1] - rp[i]);
  }
  mod_block_partials<1>(a, parts);
  if (mod_last_block(st)) {
    __shared__ double tot[1];
    mod_reduce<1>(parts, gridDim.x, tot);
    if (threadIdx.x == 0) {
      st->vk = tot[0];
      st->beta = beta;
      st->eps = eps;
      st->max_iter = max_iter;
      st->iter = 0;
      st->err1 = st->err2 = 1.0;
      st->vnorm = 0.0;
      st->done = max_iter <= 0 ? 1 : 0;
      st->counter = 0;
    }
  }
}

// One power step, part 1: y = A_G v0 - (vk / 2 / M * k + (sumBG - beta) * v0)
// on G (v0 is zero off G, so the gather needs no mask), |y|^2.
__global__ __launch_bounds__(kModThreads) void mod_spmv_kernel(
    int n, long long M, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
    const uint8_t* __restrict__ g, const double* __restrict__ sumbg,
    const double* __restrict__ v0, double* __restrict__ y, double* parts, ModState* st) {
  if (st->done) return;
  const double vk = st->vk, beta = st->beta;
  const double c = __ddiv_rn(__ddiv_rn(vk, 2.0), (double)M);  // vk / 2 / M
  const int lane = threadIdx.x & 31;
  double a[1] = {0};
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n;
       i += gridDim.x * (blockDim.x >> 5)) {
    if (!g[i]) continue;
    const int b = rp[i], e = rp[i + 1];
    double t = 0;
    for (int k0 = b; k0 < e; k0 += 128) {
      double x[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int k = k0 + lane + 32 * m;
        x[m] = k < e ? v0[__ldg(ci + k)] : 0.0;
      }
#pragma unroll
      for (int m = 0; m < 4; ++m) t = __dadd_rn(t, x[m]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = __dadd_rn(t, __shfl_xor_sync(0xffffffffu, t, o));
    if (lane == 0) {
      const double corr = __dadd_rn(__dmul_rn(c, (double)(e - b)),
                                    __dmul_rn(__dsub_rn(sumbg[i], beta), v0[i]));
      t = __dsub_rn(t, corr);
      y[i] = t;
      a[0] = __dadd_rn(a[0], __dmul_rn(t, t));
    }
  }
  mod_block_partials<1>(a, parts);
  if (mod_last_block(st)) {
    __shared__ double tot[1];
    mod_reduce<1>(parts, gridDim.x, tot);
    if (threadIdx.x == 0) {
      st->y2 = tot[0];
      st->counter = 0;
    }
  }
}

// One power step, part 2: v = y / |y| on G, |v - v0|, |v + v0|, v.k, stop test.
__global__ __launch_bounds__(kModThreads) void mod_norm_kernel(
    int n, const int32_t* __restrict__ rp, const uint8_t* __restrict__ g,
    const double* __restrict__ y, const double* __restrict__ v0, double* __restrict__ v,
    double* parts, ModState* st) {
  if (st->done) return;
  __shared__ double nrm;
  if (threadIdx.x == 0) nrm = sqrt(st->y2);
  __syncthreads();
  const double vn = nrm;
  double a[3] = {0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double old = v0[i];
    const double x = g[i] ? __ddiv_rn(y[i], vn) : 0.0;
    v[i] = x;
    const double d = __dsub_rn(x, old), s = __dadd_rn(x, old);
    a[0] = __dadd_rn(a[0], __dmul_rn(d, d));
    a[1] = __dadd_rn(a[1], __dmul_rn(s, s));
    if (g[i]) a[2] = __dadd_rn(a[2], __dmul_rn(x, (double)(rp[i + 1] - rp[i])));
  }
  mod_block_partials<3>(a, parts);
  if (mod_last_block(st)) {
    __shared__ double tot[3];
    mod_reduce<3>(parts, gridDim.x, tot);
    if (threadIdx.x == 0) {
      st->vnorm = vn;
      st->err1 = sqrt(tot[0]);
      st->err2 = sqrt(tot[1]);
      st->vk = tot[2];
      st->iter += 1;
      if (!(st->err1 > st->eps && st->err2 > st->eps && st->iter < st->max_iter)) st->done = 1;
      st->counter = 0;
    }
  }
}

// After a power iteration (one block): the first node of G with the largest
// |v| (node 0 when that is 0), the sign rule for lambda, and the sizes of the
// two signs.
__global__ __launch_bounds__(1024) void mod_final_kernel(int n, const uint8_t* __restrict__ g,
                                                         const double* __restrict__ v,
                                                         const double* __restrict__ v0,
                                                         ModState* st) {
  __shared__ double bv[1024];
  __shared__ int bi[1024];
  __shared__ long long bp[1024], bn[1024];
  double best = 0.0;
  int idx = 0;
  long long p = 0, q = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (!g[i]) continue;
    const double a = fabs(v[i]);
    if (a > best) {  // ascending i per thread: the first maximum is kept
      best = a;
      idx = i;
    }
    p += v[i] > 0;
    q += v[i] <= 0;
  }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = idx;
  bp[threadIdx.x] = p;
  bn[threadIdx.x] = q;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      const double ov = bv[threadIdx.x + h];
      const int oi = bi[threadIdx.x + h];
      if (ov > bv[threadIdx.x] || (ov == bv[threadIdx.x] && ov > 0 && oi < bi[threadIdx.x])) {
        bv[threadIdx.x] = ov;
        bi[threadIdx.x] = oi;
      }
      bp[threadIdx.x] += bp[threadIdx.x + h];
      bn[threadIdx.x] += bn[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int mi = bv[0] > 0 ? bi[0] : 0;
    st->maxi = mi;
    st->lambda = (v[mi] * v0[mi] > 0) ? st->vnorm : -st->vnorm;
    st->subp = bp[0];
    st->subn = bn[0];
  }
}

// A successful division: G's nodes go to maxres + 1 or maxres + 2 by sign.
__global__ void mod_assign_kernel(int n, const uint8_t* __restrict__ g,
                                  const double* __restrict__ v, int maxres, long long subp,
                                  long long subn, int32_t* __restrict__ label) {
  const double w = (double)(subp - subn) + 0.5;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (g[i]) label[i] = maxres + 1 + (v[i] * w <= 0 ? 1 : 0);
}

// Q's counts: directed entries inside a module (warp per row) and the degree
// sum of every module (labels < nlab), both integer.
__global__ void mod_q_kernel(int n, const int32_t* __restrict__ rp,
                             const int32_t* __restrict__ ci, const int32_t* __restrict__ label,
                             long long* __restrict__ kmod, ModState* st) {
  const int lane = threadIdx.x & 31;
  long long same = 0;
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n;
       i += gridDim.x * (blockDim.x >> 5)) {
    const int b = rp[i], e = rp[i + 1];
    const int li = label[i];
    for (int k = b + lane; k < e; k += 32) same += label[ci[k]] == li;
    if (lane == 0) atomicAdd((unsigned long long*)&kmod[li], (unsigned long long)(e - b));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) same += __shfl_xor_sync(0xffffffffu, same, o);
  if (lane == 0 && same) atomicAdd((unsigned long long*)&st->same, (unsigned long long)same);
}

// Final labels: the consecutive module numbers of the rounds that stopped.
__global__ void mod_map_kernel(int n, const int32_t* __restrict__ label,
                               const int32_t* __restrict__ adj, int32_t* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = adj[label[i]];
}

// ---- launchers ------------------------------------------------------------------

size_t mod_state_bytes() { return sizeof(ModState); }

void mod_state_read(const void* h, long long* numg, long long* kg, int* iter, int* done,
                    double* lambda, long long* subp, long long* subn, long long* same) {
  const ModState* s = (const ModState*)h;
  if (numg) *numg = s->numg;
  if (kg) *kg = s->kg;
  if (iter) *iter = s->iter;
  if (done) *done = s->done;
  if (lambda) *lambda = s->lambda;
  if (subp) *subp = s->subp;
  if (subn) *subn = s->subn;
  if (same) *same = s->same;
}

static int mod_grid(int n, int per_block, int sms) {
  const long long want = ((long long)n + per_block - 1) / per_block;
  const long long cap = (long long)sms * 8;
  return (int)(want < 1 ? 1 : want < cap ? want : cap);
}

cudaError_t launch_mod_round(int n, const int32_t* label, int round, const int32_t* rp,
                             uint8_t* g, void* st, int sms, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(st, 0, sizeof(ModState), s);
  if (e != cudaSuccess) return e;
  mod_round_kernel<<<mod_grid(n, 256, sms), 256, 0, s>>>(n, label, round, rp, g, (ModState*)st);
  return cudaGetLastError();
}

cudaError_t launch_mod_sumbg(int n, const int32_t* rp, const int32_t* ci, const uint8_t* g,
                             long long M, const void* st, double* sumbg, int sms, cudaStream_t s) {
  mod_sumbg_kernel<<<mod_grid(n, 8, sms), 256, 0, s>>>(n, rp, ci, g, M, (const ModState*)st,
                                                       sumbg);
  return cudaGetLastError();
}

int mod_grid_blocks(int sms) { return sms * 4; }

cudaError_t launch_mod_init(int n, const uint8_t* g, const int32_t* rp, double* v, double* parts,
                            void* st, double beta, int max_iter, double eps, int sms,
                            cudaStream_t s) {
  mod_init_kernel<<<mod_grid_blocks(sms), kModThreads, 0, s>>>(n, g, rp, v, parts, (ModState*)st,
                                                               beta, max_iter, eps);
  return cudaGetLastError();
}

cudaError_t launch_mod_step(int n, long long M, const int32_t* rp, const int32_t* ci,
                            const uint8_t* g, const double* sumbg, const double* v0, double* y,
                            double* v, double* parts, void* st, int sms, cudaStream_t s) {
  const int grid = mod_grid_blocks(sms);
  mod_spmv_kernel<<<grid, kModThreads, 0, s>>>(n, M, rp, ci, g, sumbg, v0, y, parts,
                                               (ModState*)st);
  mod_norm_kernel<<<grid, kModThreads, 0, s>>>(n, rp, g, y, v0, v, parts, (ModState*)st);
  return cudaGetLastError();
}

cudaError_t launch_mod_final(int n, const uint8_t* g, const double* v, const double* v0, void* st,
                             cudaStream_t s) {
  mod_final_kernel<<<1, 1024, 0, s>>>(n, g, v, v0, (ModState*)st);
  return cudaGetLastError();
}

cudaError_t launch_mod_assign(int n, const uint8_t* g, const double* v, int maxres,
                              long long subp, long long subn, int32_t* label, int sms,
                              cudaStream_t s) {
  mod_assign_kernel<<<mod_grid(n, 256, sms), 256, 0, s>>>(n, g, v, maxres, subp, subn, label);
  return cudaGetLastError();
}

cudaError_t launch_mod_q(int n, const int32_t* rp, const int32_t* ci, const int32_t* label,
                         long long* kmod, void* st, int sms, cudaStream_t s) {
  mod_q_kernel<<<mod_grid(n, 8, sms), 256, 0, s>>>(n, rp, ci, label, kmod, (ModState*)st);
  return cudaGetLastError();
}

cudaError_t launch_mod_map(int n, const int32_t* label, const int32_t* adj, int32_t* out,
                           int sms, cudaStream_t s) {
  mod_map_kernel<<<mod_grid(n, 256, sms), 256, 0, s>>>(n, label, adj, out);
  return cudaGetLastError();
}

}  // namespace bna
