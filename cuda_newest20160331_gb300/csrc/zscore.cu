// Z-score kernel: the prologue of the reference's CorMat_gpu / CorMat_cpu
// (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:24-52, CorMat.cpp:923-951).
//
// Per voxel i (reference arithmetic, reproduced bit for bit):
//   mean = (sum_t double(x_t)) / T          sequential double adds in time order
//   norm = sqrt(sum_t (double(x_t) - mean)^2)  (L2 norm of the centred row, not sigma)
//   z_t  = float((double(x_t) - mean) / norm)
// so that z_i . z_j is the Pearson r.
//
// FP64 throughput on this GPU is ~1/70 of FP32, so the kernel keeps only the
// double operations whose rounding matters and does the rest exactly with
// integer arithmetic:
//   * the time-order double sum of floats equals their exact sum whenever
//     sum |x_t| < 2^53 units of the smallest ulp among the x_t (every partial
//     sum is then representable); it is accumulated exactly in int64 fixed
//     point, with the sequential double sum as fallback otherwise;
//   * float -> double conversions are exact bit manipulations;
//   * z = RN_float(d * RN(1/norm)): the double product is within 3 double ulps
//     of the correctly rounded quotient d / norm, so it rounds to the same
//     float unless it lies within 8 double ulps of a float rounding midpoint
//     (or in the float subnormal range) — exactly those elements redo the IEEE
//     division; the float rounding itself is done on the bits.
//   The centred sum of squares keeps its sequential double adds.
//
// Layout: one thread per voxel, 64 voxels per block; every pass reads the
// time-major input coalesced (a warp reads 128 consecutive bytes per time
// step, several steps in flight).  Pass 1 finds the smallest ulp exponent and
// the exact int64 sum together (the accumulator is rescaled when a smaller
// exponent appears); pass 2 runs the sequential centred sum of squares;
// pass 3 writes the voxel-major rows (z FP32, BF16 hi = bf16(z),
// lo = bf16(z - hi)) through a 32-step shared-memory transpose so each warp
// store covers 32 consecutive t of one voxel.  bad[i] = 1 when z has a NaN.
#include <cuda_bf16.h>

#include "common.cuh"

namespace bna {

constexpr int kZV = 64;  // voxels per block = threads per block

// Exact float -> double on the bits (normal floats); other classes by the cvt.
__device__ __forceinline__ double f2d_exact(float x) {
  const uint32_t b = __float_as_uint(x);
  const uint32_t e8 = (b >> 23) & 0xFFu;
  if (e8 == 0u || e8 == 0xFFu) return (double)x;
  const unsigned long long d = ((unsigned long long)(b >> 31) << 63) |
                               ((unsigned long long)(e8 + 896u) << 52) |
                               ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}

// z = RN_float(d / nrm) (with nrm's reciprocal inv), reference rounding.
__device__ __forceinline__ float zdiv(double d, double nrm, double inv) {
  const double qq = __dmul_rn(d, inv);
  const unsigned long long bits = (unsigned long long)__double_as_longlong(qq);
  const uint32_t low = (uint32_t)(bits & 0x1FFFFFFFull);  // bits below float precision
  const uint32_t ex = (uint32_t)((bits >> 52) & 0x7FFu);
  const int dist = (int)low - 0x10000000;
  if ((dist <= 8 && dist >= -8) || ex < 1023u - 120u || ex == 0x7FFu)
    return __double2float_rn(__ddiv_rn(d, nrm));
  // round to nearest on the bits: truncate, add one ulp above the midpoint
  uint32_t f = (uint32_t)((bits >> 63) << 31) | ((ex - 896u) << 23) |
               (uint32_t)((bits >> 29) & 0x7FFFFFull);
  f += (low > 0x10000000u) ? 1u : 0u;  // carries into the exponent correctly
  return __uint_as_float(f);
}

__global__ __launch_bounds__(kZV) void zscore_kernel(const float* __restrict__ bold, int N, int T,
                                                    int n_pad, float* __restrict__ z, int ldz,
                                                    uint16_t* __restrict__ zhi,
                                                    uint16_t* __restrict__ zlo, int ldb,
                                                    uint8_t* __restrict__ bad) {
  __shared__ float tile[32][kZV + 1];  // tile[tt][v]: z of voxel v0+v at time t0+tt
  const int v = threadIdx.x, lane = v & 31, warp = v >> 5;
  const int v0 = blockIdx.x * kZV;
  const int gv = v0 + v;
  const bool live = gv < N;
  const float* col = bold + (live ? gv : 0);  // x_t = col[t * N]

  double mean = 0.0, nrm = 1.0, inv = 1.0;
  if (live) {
    // 1. exact sum: int64 fixed point in units of 2^e0, e0 = smallest ulp
    //    exponent so far (the accumulator is shifted when e0 drops); exact
    //    while every value is normal and sum |x| < 2^53 units of the final e0
    constexpr int kNone = 1 << 20;
    int e0 = kNone;
    long long acc = 0, mag = 0;
    bool exact = true;
#pragma unroll 8
    for (int t = 0; t < T; ++t) {
      const uint32_t b = __float_as_uint(__ldg(col + (size_t)t * N));
      const int e8 = (int)((b >> 23) & 0xFFu);
      const uint32_t mant = b & 0x7FFFFFu;
      if (e8 == 0xFF || (e8 == 0 && mant)) exact = false;  // inf / nan / subnormal
      if (e8 == 0 || !exact) continue;
      const int ue = e8 - 150;  // value = (mant | 2^23) * 2^ue
      if (ue < e0) {
        if (e0 != kNone) {
          const int sh = e0 - ue;
          if (sh >= 53 || (mag >> (53 - sh)) != 0) {
            exact = false;
            continue;
          }
          acc <<= sh;
          mag <<= sh;
        }
        e0 = ue;
      }
      const int sh = ue - e0;
      if (sh > 29) {
        exact = false;
        continue;
      }
      const long long m = (long long)(mant | 0x800000u) << sh;
      mag += m;
      if (mag >= (1LL << 53)) exact = false;
      acc += (b >> 31) ? -m : m;
    }
    double s1;
    if (exact) {
      // exact integer -> double (|acc| < 2^53), then the exact power-of-two scale
      s1 = (e0 == kNone) ? 0.0 : __dmul_rn(__ll2double_rn(acc), ldexp(1.0, e0));
    } else {
      s1 = 0.0;
      for (int t = 0; t < T; ++t) s1 = __dadd_rn(s1, (double)__ldg(col + (size_t)t * N));
    }
    mean = __ddiv_rn(s1, (double)T);
    // 2. centred sum of squares, sequential double adds in time order
    double s2 = 0.0;
#pragma unroll 8
    for (int t = 0; t < T; ++t) {
      const double dd = __dsub_rn(f2d_exact(__ldg(col + (size_t)t * N)), mean);
      s2 = __dadd_rn(s2, __dmul_rn(dd, dd));
    }
    nrm = __dsqrt_rn(s2);
    inv = __drcp_rn(nrm);
  }

  // 3. voxel-major rows, 32 steps at a time through the transpose tile
  const int tmax = ldz > ldb ? ldz : ldb;
  bool nan_seen = false;
  for (int t0 = 0; t0 < tmax; t0 += 32) {
#pragma unroll 8
    for (int tt = 0; tt < 32; ++tt) {
      const int t = t0 + tt;
      float zz = 0.0f;
      if (live && t < T) {
        zz = zdiv(__dsub_rn(f2d_exact(__ldg(col + (size_t)t * N)), mean), nrm, inv);
        nan_seen |= (zz != zz);
      }
      tile[tt][v] = zz;
    }
    __syncthreads();
    // warp w writes voxels w, w+2, ...: lane = time step within the chunk
    for (int vv = warp; vv < kZV; vv += kZV / 32) {
      const size_t gi = (size_t)v0 + vv;
      const int t = t0 + lane;
      const float zz = tile[lane][vv];
      if (t < ldz) z[gi * ldz + t] = zz;
      if (zhi != nullptr && t < ldb) {
        const __nv_bfloat16 hh = __float2bfloat16_rn(zz);
        const __nv_bfloat16 ll = __float2bfloat16_rn(zz - __bfloat162float(hh));
        zhi[gi * ldb + t] = __bfloat16_as_ushort(hh);
        zlo[gi * ldb + t] = __bfloat16_as_ushort(ll);
      }
    }
    __syncthreads();
  }
  if (gv < n_pad) bad[gv] = nan_seen ? 1 : 0;
}

cudaError_t launch_zscore(const float* bold, int N, int T, int n_pad, float* z, int ldz,
                          uint16_t* zhi, uint16_t* zlo, int ldb, uint8_t* bad,
                          cudaStream_t stream) {
  if (n_pad % kZV != 0 || ldz % 32 != 0 || (zhi && ldb % 32 != 0)) return cudaErrorInvalidValue;
  const int grid = n_pad / kZV;
  zscore_kernel<<<grid, kZV, 0, stream>>>(bold, N, T, n_pad, z, ldz, zhi, zlo, zhi ? ldb : 0, bad);
  return cudaGetLastError();
}

}  // namespace bna
