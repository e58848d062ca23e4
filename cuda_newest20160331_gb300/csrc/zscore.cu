// Z-score kernel: the prologue of the reference's CorMat_gpu / CorMat_cpu
// (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:24-52, CorMat.cpp:923-951).
//
// Per voxel i (reference arithmetic, reproduced bit for bit):
//   mean = (sum_t double(x_t)) / T          sequential double adds in time order
//   norm = sqrt(sum_t (double(x_t) - mean)^2)  (L2 norm of the centred row, not sigma)
//   z_t  = float((double(x_t) - mean) / norm)
// so that z_i . z_j is the Pearson r.  One thread walks one voxel's series in
// time order (the reference's order, so the double sums are identical); the
// reads BOLD[t][i .. i+127] of a block are coalesced because the input is
// time-major.  The voxel-major output is transposed through shared memory in
// 32-step chunks so the writes are coalesced too.
//
// Outputs: z [n_pad][ldz] FP32 (columns >= T and rows >= N are zero),
// optional BF16 hi/lo split [n_pad][ldb] (hi = bf16(z), lo = bf16(z - hi)),
// and bad[i] = 1 when the voxel's z contains a NaN (zero-variance voxel).
#include <cuda_bf16.h>

#include "common.cuh"

namespace bna {

__global__ __launch_bounds__(128) void zscore_kernel(const float* __restrict__ bold, int N, int T,
                                                     int n_pad, float* __restrict__ z, int ldz,
                                                     uint16_t* __restrict__ zhi,
                                                     uint16_t* __restrict__ zlo, int ldb,
                                                     uint8_t* __restrict__ bad) {
  __shared__ float tile[128][33];
  const int v0 = blockIdx.x * 128;
  const int i = v0 + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool valid = i < N;
  double mean = 0.0, nrm = 1.0;
  if (valid) {
    double s1 = 0.0;
    for (int t = 0; t < T; ++t) s1 = __dadd_rn(s1, (double)__ldg(bold + (size_t)t * N + i));
    mean = __ddiv_rn(s1, (double)T);
    double s2 = 0.0;
    for (int t = 0; t < T; ++t) {
      const double d = __dsub_rn((double)__ldg(bold + (size_t)t * N + i), mean);
      s2 = __dadd_rn(s2, __dmul_rn(d, d));
    }
    nrm = __dsqrt_rn(s2);
  }
  bool nan_seen = false;
  const int tmax = ldz > ldb ? ldz : ldb;
  for (int t0 = 0; t0 < tmax; t0 += 32) {
#pragma unroll 4
    for (int k = 0; k < 32; ++k) {
      const int t = t0 + k;
      float zz = 0.0f;
      if (valid && t < T) {
        const double d = __dsub_rn((double)__ldg(bold + (size_t)t * N + i), mean);
        zz = __double2float_rn(__ddiv_rn(d, nrm));
        nan_seen |= (zz != zz);
      }
      tile[threadIdx.x][k] = zz;
    }
    __syncthreads();
    for (int r = 0; r < 32; ++r) {
      const int vl = warp * 32 + r;
      const size_t gi = (size_t)v0 + vl;
      const float zz = tile[vl][lane];
      const int t = t0 + lane;
      if (t < ldz) z[gi * ldz + t] = zz;
      if (zhi != nullptr && t < ldb) {
        const __nv_bfloat16 h = __float2bfloat16_rn(zz);
        const __nv_bfloat16 l = __float2bfloat16_rn(zz - __bfloat162float(h));
        zhi[gi * ldb + t] = __bfloat16_as_ushort(h);
        zlo[gi * ldb + t] = __bfloat16_as_ushort(l);
      }
    }
    __syncthreads();
  }
  if (i < n_pad) bad[i] = nan_seen ? 1 : 0;
}

cudaError_t launch_zscore(const float* bold, int N, int T, int n_pad, float* z, int ldz,
                          uint16_t* zhi, uint16_t* zlo, int ldb, uint8_t* bad,
                          cudaStream_t stream) {
  if (n_pad % 128 != 0 || ldz % 32 != 0 || (zhi && ldb % 32 != 0)) return cudaErrorInvalidValue;
  zscore_kernel<<<n_pad / 128, 128, 0, stream>>>(bold, N, T, n_pad, z, ldz, zhi, zlo,
                                                 zhi ? ldb : 0, bad);
  return cudaGetLastError();
}

}  // namespace bna
