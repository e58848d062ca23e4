// Z-score kernel: the prologue of the reference's CorMat_gpu / CorMat_cpu
// (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:24-52, CorMat.cpp:923-951).
//
// Per voxel i (reference arithmetic, reproduced bit for bit):
//   mean = (sum_t double(x_t)) / T          sequential double adds in time order
//   norm = sqrt(sum_t (double(x_t) - mean)^2)  (L2 norm of the centred row, not sigma)
//   z_t  = float((double(x_t) - mean) / norm)
// so that z_i . z_j is the Pearson r.
//
// FP64 throughput on this GPU is ~1/70 of FP32, so the double operations
// are limited to those whose rounding matters:
//   * the time-order double sum of floats equals their exact sum whenever
//     sum |x_t| < 2^53 units of the smallest ulp among the x_t (every partial
//     sum is then representable); it is accumulated exactly in int64 fixed
//     point, with the sequential double sum as fallback otherwise;
//   * float -> double conversions are exact bit manipulations;
//   * the centred sum of squares keeps its sequential double adds;
//   * z itself is computed in float-float arithmetic (TwoSum / FMA-based
//     TwoProduct, Knuth and Dekker): q' ~ (x - mean) / norm with a rigorous
//     error bound B; whenever [q' - B, q' + B] holds no float rounding
//     midpoint, RN_float of the reference's double quotient is the float part
//     of q'.  The few elements that fail the test (about 2^-19 of them) take
//     the exact double path: z = RN_float(d * RN(1/norm)), which rounds like
//     the correctly rounded quotient unless it lies within 8 double ulps of a
//     float rounding midpoint (or in the float subnormal range), where the
//     IEEE division is redone; the float rounding is done on the bits.
//
// Two kernels:
//   zscore_stats_kernel  one thread per voxel: pass 1 finds the smallest ulp
//                        exponent and the exact int64 sum together (the
//                        accumulator is rescaled when a smaller exponent
//                        appears); pass 2 runs the sequential centred sum of
//                        squares.  Reads are coalesced (a warp reads 128
//                        consecutive bytes per time step).
//   zscore_emit_kernel   one element per thread-step over 32 voxels x 32
//                        steps tiles: reads coalesced along voxels, computes
//                        z, and writes the voxel-major rows (z FP32, BF16
//                        hi = bf16(z), lo = bf16(z - hi)) through a shared-
//                        memory transpose.  bad[i] = 1 when z has a NaN.
#include <cuda_bf16.h>

#include "common.cuh"

namespace bna {

constexpr int kZStatThreads = 128;
constexpr int kZEmitT = 256;  // time steps per emit block (8 chunks of 32)

// Per-voxel statistics handed from the stats kernel to the emit kernel.
struct VoxStat {
  double mean, nrm, inv;  // reference mean, norm and RN(1 / norm)
  float m0, m1, m2;       // mean = m0 + m1 + m2 exactly (float split)
  float ih, il;           // inv ~ ih + il (relative error <= 2^-48)
  int fast;               // the float-float path applies to this voxel
};

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

__global__ __launch_bounds__(kZStatThreads) void zscore_stats_kernel(
    const float* __restrict__ bold, int N, int T, int n_pad, VoxStat* __restrict__ vs,
    uint8_t* __restrict__ bad) {
  const int gv = blockIdx.x * kZStatThreads + threadIdx.x;
  if (gv >= n_pad) return;
  VoxStat o;
  o.mean = 0.0;
  o.nrm = 1.0;
  o.inv = 1.0;
  o.m0 = o.m1 = o.m2 = 0.0f;
  o.ih = 1.0f;
  o.il = 0.0f;
  o.fast = 1;
  if (gv < N) {
    const float* col = bold + gv;  // x_t = col[t * N]
    // 1. exact sum: int64 fixed point in units of 2^e0, e0 = smallest ulp
    //    exponent so far (the accumulator is shifted when e0 drops); exact
    //    while every value is normal and sum |x| < 2^53 units of the final e0
    constexpr int kNone = 1 << 20;
    constexpr int kPf = 16;  // loads in flight per thread
    int e0 = kNone;
    long long acc = 0, mag = 0;
    bool exact = true;
    for (int t0 = 0; t0 < T; t0 += kPf) {
      float xs[kPf];
#pragma unroll
      for (int k = 0; k < kPf; ++k) xs[k] = (t0 + k < T) ? __ldg(col + (size_t)(t0 + k) * N) : 0.0f;
#pragma unroll
      for (int k = 0; k < kPf; ++k) {
        const uint32_t b = __float_as_uint(xs[k]);  // padding zeros add nothing
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
    }
    double s1;
    if (exact) {
      // exact integer -> double (|acc| < 2^53), then the exact power-of-two scale
      s1 = (e0 == kNone) ? 0.0 : __dmul_rn(__ll2double_rn(acc), ldexp(1.0, e0));
    } else {
      s1 = 0.0;
      for (int t = 0; t < T; ++t) s1 = __dadd_rn(s1, (double)__ldg(col + (size_t)t * N));
    }
    const double mean = __ddiv_rn(s1, (double)T);
    // 2. centred sum of squares, sequential double adds in time order
    double s2 = 0.0;
    for (int t0 = 0; t0 < T; t0 += kPf) {
      float xs[kPf];
#pragma unroll
      for (int k = 0; k < kPf; ++k) xs[k] = (t0 + k < T) ? __ldg(col + (size_t)(t0 + k) * N) : 0.0f;
#pragma unroll
      for (int k = 0; k < kPf; ++k) {
        if (t0 + k < T) {
          const double dd = __dsub_rn(f2d_exact(xs[k]), mean);
          s2 = __dadd_rn(s2, __dmul_rn(dd, dd));
        }
      }
    }
    o.mean = mean;
    o.nrm = __dsqrt_rn(s2);
    o.inv = __drcp_rn(o.nrm);
    // float splits for the emit kernel's float-float path
    o.m0 = __double2float_rn(mean);
    const double r1 = __dsub_rn(mean, (double)o.m0);
    o.m1 = __double2float_rn(r1);
    o.m2 = __double2float_rn(__dsub_rn(r1, (double)o.m1));
    o.ih = __double2float_rn(o.inv);
    o.il = __double2float_rn(__dsub_rn(o.inv, (double)o.ih));
    const double back = __dadd_rn(__dadd_rn((double)o.m0, (double)o.m1), (double)o.m2);
    const float aih = fabsf(o.ih);
    o.fast = (back == mean) && isfinite(mean) && o.nrm > 0.0 && isfinite(o.nrm) &&
             aih >= 1.0e-30f && aih <= 1.0e30f && (fabsf(o.m0) <= 1.0e30f) &&
             (o.m0 == 0.0f || fabsf(o.m0) >= 1.0e-30f);
  }
  vs[gv] = o;
  bad[gv] = 0;
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void zs_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// The reference's z of one element: the float-float path when it is provably
// right, else the exact double path.
__device__ __forceinline__ float z_of(float x, const VoxStat& v) {
  if (v.fast && isfinite(x)) {
    // d = x - mean as (dh, dl): x - m0 exactly (TwoSum), then the small terms
    float s, e;
    zs_two_sum(x, -v.m0, s, e);
    const float t = __fsub_rn(__fsub_rn(e, v.m1), v.m2);
    float dh, dl;
    zs_two_sum(s, t, dh, dl);
    // q' = (dh + dl) * (ih + il): exact head product, FMA-accumulated tail
    const float ph = __fmul_rn(dh, v.ih);
    float pe = __fmaf_rn(dh, v.ih, -ph);
    pe = __fmaf_rn(dh, v.il, pe);
    pe = __fmaf_rn(dl, v.ih, pe);
    const float qh = __fadd_rn(ph, pe);
    const float ql = __fsub_rn(pe, __fsub_rn(qh, ph));
    // error bound of q' against the reference's double quotient: relative
    // terms (inv split, dropped dl*il, tail roundings, the reference's two
    // roundings) below 2^-44 |q|, plus the error of d, below
    // 2^-46 (|x| + |mean|), times inv
    const uint32_t qb = __float_as_uint(qh);
    const uint32_t e8 = (qb >> 23) & 0xFFu;
    if (e8 >= 25u && e8 <= 253u && (qb & 0x7FFFFFu) != 0u) {
      const float half_ulp = __uint_as_float((e8 - 24u) << 23);
      const float bound = fabsf(qh) * 5.6843419e-14f /* 2^-44 */ +
                          (fabsf(x) + fabsf(v.m0)) * fabsf(v.ih) * 2.8421709e-14f /* 2^-45 */;
      if (half_ulp - fabsf(ql) > bound) return qh;
    }
  }
  return zdiv(__dsub_rn(f2d_exact(x), v.mean), v.nrm, v.inv);
}

__global__ __launch_bounds__(256) void zscore_emit_kernel(
    const float* __restrict__ bold, int N, int T, const VoxStat* __restrict__ vs,
    float* __restrict__ z, int ldz, uint16_t* __restrict__ zhi, uint16_t* __restrict__ zlo,
    int ldb, uint8_t* __restrict__ bad) {
  __shared__ float tile[32][33];  // tile[tt][v]: z of voxel v0+v at time t0+tt
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int v0 = blockIdx.x * 32;
  const int gv = v0 + lane;
  const bool live = gv < N;
  const VoxStat st = vs[gv];  // gv < n_pad: the grid covers n_pad / 32 groups
  const int tmax = ldz > ldb ? ldz : ldb;
  const int tb = blockIdx.y * kZEmitT;
  bool nan_seen = false;
  for (int t0 = tb; t0 < tb + kZEmitT && t0 < tmax; t0 += 32) {
    float xs[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int t = t0 + warp + 8 * k;
      xs[k] = (live && t < T) ? __ldg(bold + (size_t)t * N + gv) : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int tt = warp + 8 * k, t = t0 + tt;
      float zz = 0.0f;
      if (live && t < T) {
        zz = z_of(xs[k], st);
        nan_seen |= (zz != zz);
      }
      tile[tt][lane] = zz;
    }
    __syncthreads();
    // warp w writes voxels w, w+8, w+16, w+24; lane = time step in the chunk
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int vv = warp + 8 * k;
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
  if (nan_seen) bad[gv] = 1;
}

size_t zscore_scratch_bytes(int n_pad) { return (size_t)n_pad * sizeof(VoxStat); }

// scratch: zscore_scratch_bytes(n_pad) bytes of device memory.
cudaError_t launch_zscore(const float* bold, int N, int T, int n_pad, float* z, int ldz,
                          uint16_t* zhi, uint16_t* zlo, int ldb, uint8_t* bad, void* scratch,
                          cudaStream_t stream) {
  if (n_pad % 128 != 0 || ldz % 32 != 0 || (zhi && ldb % 32 != 0) || !scratch)
    return cudaErrorInvalidValue;
  VoxStat* vs = static_cast<VoxStat*>(scratch);
  zscore_stats_kernel<<<n_pad / kZStatThreads, kZStatThreads, 0, stream>>>(bold, N, T, n_pad, vs,
                                                                           bad);
  const int ldbv = zhi ? ldb : 0;
  const int tmax = ldz > ldbv ? ldz : ldbv;
  const dim3 grid(n_pad / 32, (tmax + kZEmitT - 1) / kZEmitT);
  zscore_emit_kernel<<<grid, 256, 0, stream>>>(bold, N, T, vs, z, ldz, zhi, zlo, ldbv, bad);
  return cudaGetLastError();
}

}  // namespace bna
