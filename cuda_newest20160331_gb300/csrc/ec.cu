// Eigenvector centrality by power iteration on the device-resident CSR.
//
// Reference: Lead_Vector_GPU (W/CUEC/weighted-net.cu:55-221), whose loop
// (:154-189) per iteration does u0 = u; lambda = ||u||; u = u / lambda;
// u = A u (cusparseDcsrmv); e1 = ||u - u0||; e2 = ||u + u0|| with three
// blocking host reductions.  Here one kernel does a whole iteration:
//   lambda = sqrt(sum u^2)   (sum produced by the previous iteration)
//   y_i    = (sum_k val_k * u[col_k]) / lambda      (FP64, val read as float)
//   partial sums of y^2, (y - u)^2, (y + u)^2 per block
// and the last block to finish reduces the partials in a fixed order, so the
// iteration is deterministic.  A device flag stops later launches once
// e1 <= eps or e2 <= eps (no host round trip per iteration); the host replays
// a captured CUDA graph of 32 iterations and reads the flag between graphs.
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
  int pad;
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

__global__ __launch_bounds__(kEcThreads) void ec_init_kernel(int n, double* u, double* parts,
                                                             EcState* st, int max_iter) {
  __shared__ double ws[kEcThreads / 32];
  double s = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = (double)i;  // init_AD, weighted-net.cu:38-43
    u[i] = v;
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

__global__ __launch_bounds__(kEcThreads, 4) void ec_iter_kernel(
    int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
    const float* __restrict__ val, const double* __restrict__ vald, long long nnz_used,
    const double* __restrict__ u,
    double* __restrict__ un, double* parts, EcState* st, int max_iter, double eps) {
  if (st->done || st->iter >= max_iter) return;
  const double lam = sqrt(st->lam2);
  const double inv = 1.0 / lam;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = gridDim.x * (kEcThreads / 32);
  double a0 = 0, a1 = 0, a2 = 0;
  for (int row = blockIdx.x * (kEcThreads / 32) + warp; row < n; row += nwarps) {
    long long b = rp[row], e = rp[row + 1];
    if (e > nnz_used) e = nnz_used;
    double s = 0;
    if (val) {
      for (long long k = b + lane; k < e; k += 32) s += (double)__ldg(val + k) * u[__ldg(ci + k)];
    } else if (vald) {
      for (long long k = b + lane; k < e; k += 32) s += __ldg(vald + k) * u[__ldg(ci + k)];
    } else {
      for (long long k = b + lane; k < e; k += 32) s += u[__ldg(ci + k)];
    }
    s = warp_sum(s);
    if (lane == 0) {
      const double y = s * inv;
      const double old = u[row];
      un[row] = y;
      a0 += y * y;
      const double d = y - old, p = y + old;
      a1 += d * d;
      a2 += p * p;
    }
  }
  __shared__ double ws[kEcThreads / 32][3];
  if (lane == 0) {
    ws[warp][0] = a0;
    ws[warp][1] = a1;
    ws[warp][2] = a2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int w = 0; w < kEcThreads / 32; ++w) {
      t0 += ws[w][0];
      t1 += ws[w][1];
      t2 += ws[w][2];
    }
    parts[blockIdx.x * 3 + 0] = t0;
    parts[blockIdx.x * 3 + 1] = t1;
    parts[blockIdx.x * 3 + 2] = t2;
  }
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

size_t ec_state_bytes() { return sizeof(EcState); }

cudaError_t launch_ec_init(int n, double* u, double* parts, void* st, int grid, int max_iter,
                           cudaStream_t stream) {
  ec_init_kernel<<<grid, kEcThreads, 0, stream>>>(n, u, parts, (EcState*)st, max_iter);
  return cudaGetLastError();
}

cudaError_t launch_ec_iter(int n, const int32_t* rp, const int32_t* ci, const float* val,
                           const double* vald, long long nnz_used, const double* u, double* un,
                           double* parts, void* st, int grid, int max_iter, double eps,
                           cudaStream_t stream) {
  ec_iter_kernel<<<grid, kEcThreads, 0, stream>>>(n, rp, ci, val, vald, nnz_used, u, un, parts,
                                                  (EcState*)st, max_iter, eps);
  return cudaGetLastError();
}

// Host view of the state block (same layout as EcState).
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
