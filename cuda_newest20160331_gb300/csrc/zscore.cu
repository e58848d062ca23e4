// Z-score kernel: the prologue of the reference's CorMat_gpu / CorMat_cpu
// (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:24-52, CorMat.cpp:923-951).
//
// Per voxel i (reference arithmetic, reproduced bit for bit):
//   mean = (sum_t double(x_t)) / T          sequential double adds in time order
//   norm = sqrt(sum_t (double(x_t) - mean)^2)  (L2 norm of the centred row, not sigma)
//   z_t  = float((double(x_t) - mean) / norm)
// so that z_i . z_j is the Pearson r.
//
// A block owns V voxels (V = 128 when the V x T series fit in shared memory,
// fewer for long series).  It reads BOLD[t][v0 .. v0+V) once from HBM with
// coalesced loads into shared memory; one thread per voxel then runs the two
// sequential FP64 sums in the reference's order from shared memory; finally
// the block writes the voxel-major rows (z FP32, BF16 hi = bf16(z),
// lo = bf16(z - hi)) with one warp per voxel row, 32 consecutive t per store.
//
// The division is done as q = (x - mean) * RN(1/norm), within 3 double ulps
// of the correctly rounded quotient; q rounds to the same float as the
// quotient unless it lies within 8 double ulps of a float rounding midpoint
// (or in the float subnormal range), and exactly those elements redo the
// IEEE division.  bad[i] = 1 when the voxel's z contains a NaN (zero variance).
#include <cuda_bf16.h>

#include "common.cuh"

namespace bna {

constexpr int kZThreads = 128;
constexpr size_t kZSmemMax = 160 * 1024;

__device__ __forceinline__ float zdiv(double d, double nrm, double inv) {
  double qq = __dmul_rn(d, inv);
  const unsigned long long bits = (unsigned long long)__double_as_longlong(qq);
  const int low = (int)(bits & 0x1FFFFFFFull);  // bits below float precision
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (abs(low - 0x10000000) <= 8 || ex < 1023 - 120) qq = __ddiv_rn(d, nrm);
  return __double2float_rn(qq);
}

// s[t * (V+1) + v]: BOLD value of voxel v0+v at time t.
__global__ __launch_bounds__(kZThreads) void zscore_kernel(const float* __restrict__ bold, int N,
                                                           int T, int n_pad, int V,
                                                           float* __restrict__ z, int ldz,
                                                           uint16_t* __restrict__ zhi,
                                                           uint16_t* __restrict__ zlo, int ldb,
                                                           uint8_t* __restrict__ bad) {
  extern __shared__ float zs[];
  const int ld = V + 1;
  float* s = zs;
  double* st_mean = reinterpret_cast<double*>(zs + (((size_t)T * ld + 1) & ~(size_t)1));
  double* st_nrm = st_mean + V;
  double* st_inv = st_nrm + V;
  const int v0 = blockIdx.x * V;
  const int nv = min(V, max(0, N - v0));  // voxels of this block that exist
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // 1. coalesced load of the block's series
  for (int idx = threadIdx.x; idx < T * V; idx += kZThreads) {
    const int t = idx / V, v = idx - t * V;
    s[t * ld + v] = (v < nv) ? __ldg(bold + (size_t)t * N + v0 + v) : 0.0f;
  }
  __syncthreads();

  // 2. the reference's sequential sums, one thread per voxel
  for (int v = threadIdx.x; v < V; v += kZThreads) {
    double mean = 0.0, nrm = 1.0, inv = 1.0;
    if (v < nv) {
      double s1 = 0.0;
      for (int t = 0; t < T; ++t) s1 = __dadd_rn(s1, (double)s[t * ld + v]);
      mean = __ddiv_rn(s1, (double)T);
      double s2 = 0.0;
      for (int t = 0; t < T; ++t) {
        const double d = __dsub_rn((double)s[t * ld + v], mean);
        s2 = __dadd_rn(s2, __dmul_rn(d, d));
      }
      nrm = __dsqrt_rn(s2);
      inv = __drcp_rn(nrm);
    }
    st_mean[v] = mean;
    st_nrm[v] = nrm;
    st_inv[v] = inv;
  }
  __syncthreads();

  // 3. voxel-major rows, one warp per voxel
  const int tmax = ldz > ldb ? ldz : ldb;
  for (int v = warp; v < V; v += kZThreads / 32) {
    const size_t gi = (size_t)v0 + v;
    if (gi >= (size_t)n_pad) break;
    const double mean = st_mean[v], nrm = st_nrm[v], inv = st_inv[v];
    bool nan_seen = false;
    for (int t = lane; t < tmax; t += 32) {
      float zz = 0.0f;
      if (v < nv && t < T) {
        zz = zdiv(__dsub_rn((double)s[t * ld + v], mean), nrm, inv);
        nan_seen |= (zz != zz);
      }
      if (t < ldz) z[gi * ldz + t] = zz;
      if (zhi != nullptr && t < ldb) {
        const __nv_bfloat16 h = __float2bfloat16_rn(zz);
        const __nv_bfloat16 l = __float2bfloat16_rn(zz - __bfloat162float(h));
        zhi[gi * ldb + t] = __bfloat16_as_ushort(h);
        zlo[gi * ldb + t] = __bfloat16_as_ushort(l);
      }
    }
    nan_seen = __any_sync(0xffffffffu, nan_seen);
    if (lane == 0) bad[gi] = nan_seen ? 1 : 0;
  }
}

static size_t zscore_smem(int T, int V);

// Voxels per block: the largest of 128, 96, 64, 32, 16, 8 whose series fit in
// kZSmemMax (8 for very long series).
static int zscore_block_voxels(int T) {
  const int cand[6] = {128, 96, 64, 32, 16, 8};
  for (int c = 0; c < 5; ++c)
    if (zscore_smem(T, cand[c]) <= kZSmemMax) return cand[c];
  return 8;
}

static size_t zscore_smem(int T, int V) {
  return (((size_t)T * (V + 1) + 1) & ~(size_t)1) * 4 + (size_t)V * 24;
}

cudaError_t launch_zscore(const float* bold, int N, int T, int n_pad, float* z, int ldz,
                          uint16_t* zhi, uint16_t* zlo, int ldb, uint8_t* bad,
                          cudaStream_t stream) {
  if (n_pad % 128 != 0 || ldz % 32 != 0 || (zhi && ldb % 32 != 0)) return cudaErrorInvalidValue;
  const int V = zscore_block_voxels(T);
  const size_t smem = zscore_smem(T, V);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;  // T beyond ~6,000 volumes
  cudaError_t e = cudaFuncSetAttribute(zscore_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  zscore_kernel<<<(n_pad + V - 1) / V, kZThreads, smem, stream>>>(bold, N, T, n_pad, V, z, ldz, zhi, zlo,
                                                        zhi ? ldb : 0, bad);
  return cudaGetLastError();
}

}  // namespace bna
