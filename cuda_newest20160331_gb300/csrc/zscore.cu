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
// Layout: a block owns 32 voxels; one warp runs their sums, one thread per
// voxel.  Short series (T <= 360) are read once, coalesced, into shared
// memory; longer ones are read coalesced from global memory in each pass.
// The block writes the voxel-major rows (z FP32, BF16 hi = bf16(z),
// lo = bf16(z - hi)) 32 consecutive t per warp store.  bad[i] = 1 when z has
// a NaN.
#include <cuda_bf16.h>

#include "common.cuh"

namespace bna {

constexpr int kZThreads = 128;
constexpr int kZV = 32;  // voxels per block

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

// s[t * (kZV+1) + v]: BOLD value of voxel v0+v at time t.
template <bool RESIDENT>
__global__ __launch_bounds__(kZThreads) void zscore_kernel(const float* __restrict__ bold, int N,
                                                           int T, int n_pad,
                                                           float* __restrict__ z, int ldz,
                                                           uint16_t* __restrict__ zhi,
                                                           uint16_t* __restrict__ zlo, int ldb,
                                                           uint8_t* __restrict__ bad) {
  extern __shared__ float zs[];
  constexpr int ld = kZV + 1;
  const int rows = RESIDENT ? T : 32;  // series in smem, or one 32-step chunk
  float* s = zs;
  double* st_mean = reinterpret_cast<double*>(zs + (((size_t)rows * ld + 1) & ~(size_t)1));
  double* st_nrm = st_mean + kZV;
  double* st_inv = st_nrm + kZV;
  const int v0 = blockIdx.x * kZV;
  const int nv = min(kZV, max(0, N - v0));  // voxels of this block that exist
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // BOLD value of voxel v0+v at time t (shared-memory copy or coalesced global read)
  auto X = [&](int t, int v) -> float {
    return RESIDENT ? s[t * ld + v] : __ldg(bold + (size_t)t * N + v0 + v);
  };

  // 1. coalesced load of the block's series (one 128-byte row per time step)
  if (RESIDENT) {
    for (int idx = threadIdx.x; idx < T * kZV; idx += kZThreads) {
      const int t = idx >> 5, v = idx & 31;
      s[t * ld + v] = (v < nv) ? __ldg(bold + (size_t)t * N + v0 + v) : 0.0f;
    }
    __syncthreads();
  }

  // 2. mean and centred norm, one thread per voxel
  if (warp == 0) {
    const int v = lane;
    double mean = 0.0, nrm = 1.0, inv = 1.0;
    if (v < nv) {
      // smallest ulp exponent among the finite non-zero values
      int emin = 1 << 20;
      bool special = false;
      for (int t = 0; t < T; ++t) {
        const uint32_t b = __float_as_uint(X(t, v));
        const int e8 = (int)((b >> 23) & 0xFFu);
        if (e8 == 0xFF || (e8 == 0 && (b & 0x7FFFFFu))) special = true;  // inf/nan/subnormal
        if (e8 != 0) emin = min(emin, e8 - 150);  // ulp exponent: value = m * 2^(e8-150)
      }
      double s1;
      bool exact = !special;
      long long acc = 0;
      if (exact && emin != (1 << 20)) {
        // sum |x| in units of 2^emin must stay below 2^53
        long long mag = 0;
        for (int t = 0; t < T && exact; ++t) {
          const uint32_t b = __float_as_uint(X(t, v));
          const int e8 = (int)((b >> 23) & 0xFFu);
          if (e8 == 0) continue;
          const int sh = e8 - 150 - emin;
          if (sh > 29) {
            exact = false;
            break;
          }
          const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u) << sh;
          mag += m;
          if (mag >= (1LL << 53)) exact = false;
          acc += (b >> 31) ? -m : m;
        }
      }
      if (exact) {
        // exact integer -> double (|acc| < 2^53), then the exact power-of-two scale
        s1 = (emin == (1 << 20)) ? 0.0 : __dmul_rn(__ll2double_rn(acc), ldexp(1.0, emin));
      } else {
        s1 = 0.0;
        for (int t = 0; t < T; ++t) s1 = __dadd_rn(s1, (double)X(t, v));
      }
      mean = __ddiv_rn(s1, (double)T);
      double s2 = 0.0;
      for (int t = 0; t < T; ++t) {
        const double dd = __dsub_rn(f2d_exact(X(t, v)), mean);
        s2 = __dadd_rn(s2, __dmul_rn(dd, dd));
      }
      nrm = __dsqrt_rn(s2);
      inv = __drcp_rn(nrm);
    }
    st_mean[v] = mean;
    st_nrm[v] = nrm;
    st_inv[v] = inv;
  }
  __syncthreads();

  // 3. voxel-major rows
  const int tmax = ldz > ldb ? ldz : ldb;
  auto emit = [&](size_t gi, int t, float zz) {
    if (t < ldz) z[gi * ldz + t] = zz;
    if (zhi != nullptr && t < ldb) {
      const __nv_bfloat16 hh = __float2bfloat16_rn(zz);
      const __nv_bfloat16 ll = __float2bfloat16_rn(zz - __bfloat162float(hh));
      zhi[gi * ldb + t] = __bfloat16_as_ushort(hh);
      zlo[gi * ldb + t] = __bfloat16_as_ushort(ll);
    }
  };
  if (RESIDENT) {
    // one warp per voxel row, 32 consecutive t per store
    for (int v = warp; v < kZV; v += kZThreads / 32) {
      const size_t gi = (size_t)v0 + v;
      if (gi >= (size_t)n_pad) break;
      const double mean = st_mean[v], nrm = st_nrm[v], inv = st_inv[v];
      bool nan_seen = false;
      for (int t = lane; t < tmax; t += 32) {
        float zz = 0.0f;
        if (v < nv && t < T) {
          zz = zdiv(__dsub_rn(f2d_exact(s[t * ld + v]), mean), nrm, inv);
          nan_seen |= (zz != zz);
        }
        emit(gi, t, zz);
      }
      nan_seen = __any_sync(0xffffffffu, nan_seen);
      if (lane == 0) bad[gi] = nan_seen ? 1 : 0;
    }
  } else {
    // 32-step chunks: compute z[t][v] into the smem tile (coalesced reads),
    // then write each voxel's 32 values with one warp store
    __shared__ int nan_flag[kZV];
    if (threadIdx.x < kZV) nan_flag[threadIdx.x] = 0;
    for (int t0 = 0; t0 < tmax; t0 += 32) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < 32 * kZV; idx += kZThreads) {
        const int tt = idx >> 5, v = idx & 31, t = t0 + tt;
        float zz = 0.0f;
        if (v < nv && t < T) {
          zz = zdiv(__dsub_rn(f2d_exact(__ldg(bold + (size_t)t * N + v0 + v)), st_mean[v]),
                    st_nrm[v], st_inv[v]);
          if (zz != zz) nan_flag[v] = 1;
        }
        s[tt * ld + v] = zz;
      }
      __syncthreads();
      for (int v = warp; v < kZV; v += kZThreads / 32) {
        const size_t gi = (size_t)v0 + v;
        if (gi < (size_t)n_pad) emit(gi, t0 + lane, s[lane * ld + v]);
      }
    }
    __syncthreads();
    if (threadIdx.x < kZV && (size_t)v0 + threadIdx.x < (size_t)n_pad)
      bad[v0 + threadIdx.x] = nan_flag[threadIdx.x] ? 1 : 0;
  }
}

static size_t zscore_smem(int rows) {
  return (((size_t)rows * (kZV + 1) + 1) & ~(size_t)1) * 4 + (size_t)kZV * 24;
}

// Series up to this length stay in shared memory (about 48 KB per block, so
// several blocks - and their FP64 chains - share an SM); longer ones stream.
constexpr int kZResidentMaxT = 360;

cudaError_t launch_zscore(const float* bold, int N, int T, int n_pad, float* z, int ldz,
                          uint16_t* zhi, uint16_t* zlo, int ldb, uint8_t* bad,
                          cudaStream_t stream) {
  if (n_pad % 128 != 0 || ldz % 32 != 0 || (zhi && ldb % 32 != 0)) return cudaErrorInvalidValue;
  const bool resident = T <= kZResidentMaxT;
  const size_t smem = zscore_smem(resident ? T : 32);
  const int grid = n_pad / kZV;
  const int ldbv = zhi ? ldb : 0;
  cudaError_t e;
  if (resident) {
    e = cudaFuncSetAttribute(zscore_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    zscore_kernel<true><<<grid, kZThreads, smem, stream>>>(bold, N, T, n_pad, z, ldz, zhi, zlo,
                                                           ldbv, bad);
  } else {
    zscore_kernel<false><<<grid, kZThreads, smem, stream>>>(bold, N, T, n_pad, z, ldz, zhi, zlo,
                                                            ldbv, bad);
  }
  return cudaGetLastError();
}

}  // namespace bna
