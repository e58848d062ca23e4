// Exact reference value of one pair (shared by the recompute and the
// density selection kernels).
#pragma once
#include "common.cuh"

namespace bna {

// The reference value of a pair: float(sum_t double(float(z_it * z_jt))), the
// double sum in time order (CorMat.cpp:955-964).  That sequential sum equals
// the exact sum of the float products whenever every product is a normal
// float and sum |p_t| < 2^53 units of the smallest ulp among them (each
// partial sum is then representable).  A warp evaluates one pair: lanes take
// t = lane, lane+32, ..., the exact sum is an int64 fixed-point reduction
// across the warp, and only when the condition fails does lane 0 run the
// sequential double adds.  Returns the raw value (NaN for a voxel with a NaN
// z-score); exact_r_warp_z gives it after post_block's clamp.
__device__ __forceinline__ float exact_r_warp_raw(const float* z, const uint8_t* bad, int ldz,
                                                  int T, int i, int j, int lane) {
  if (bad[i] | bad[j]) return __int_as_float(0x7fc00000);  // NaN
  const float* zi = z + (size_t)i * ldz;
  const float* zj = z + (size_t)j * ldz;
  int emin = 1 << 20;
  bool special = false;
  for (int t = lane; t < T; t += 32) {
    const uint32_t b = __float_as_uint(__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
    const int e8 = (int)((b >> 23) & 0xFFu);
    special |= (e8 == 0xFF) || (e8 == 0 && (b & 0x7FFFFFu));
    if (e8 != 0) emin = min(emin, e8 - 150);
  }
  emin = __reduce_min_sync(0xffffffffu, emin);
  special = __any_sync(0xffffffffu, special);
  bool exact = !special;
  long long acc = 0, mag = 0;
  if (exact && emin != (1 << 20)) {
    for (int t = lane; t < T; t += 32) {
      const uint32_t b = __float_as_uint(__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
      const int e8 = (int)((b >> 23) & 0xFFu);
      if (e8 == 0) continue;
      const int sh = e8 - 150 - emin;
      if (sh > 29) {
        exact = false;
        continue;
      }
      const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u) << sh;
      mag += m;
      acc += (b >> 31) ? -m : m;
    }
    exact = __all_sync(0xffffffffu, exact);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
      mag += __shfl_xor_sync(0xffffffffu, mag, o);
    }
    exact = exact && mag < (1LL << 53);
  }
  float r = 0.0f;
  if (lane == 0) {
    if (exact) {
      r = (emin == (1 << 20)) ? 0.0f
                              : __double2float_rn(__dmul_rn(__ll2double_rn(acc), ldexp(1.0, emin)));
    } else {
      double s = 0.0;
      for (int t = 0; t < T; ++t)
        s = __dadd_rn(s, (double)__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
      r = __double2float_rn(s);
    }
  }
  return __shfl_sync(0xffffffffu, r, 0);
}

__device__ __forceinline__ float exact_r_warp_z(const float* z, const uint8_t* bad, int ldz,
                                                int T, int i, int j, int lane) {
  return post_block(exact_r_warp_raw(z, bad, ldz, T, i, j, lane));
}

__device__ __forceinline__ float exact_r_warp(const CorrArgs& a, int i, int j, int lane) {
  return exact_r_warp_z(a.z, a.bad, a.ldz, a.T, i, j, lane);
}

// The value a rule decides on: post_block's, or the raw one for BNA_THR_R_EPS.
__device__ __forceinline__ float exact_r_rule(const CorrArgs& a, int i, int j, int lane) {
  const float raw = exact_r_warp_raw(a.z, a.bad, a.ldz, a.T, i, j, lane);
  return a.th.mode == BNA_THR_R_EPS ? raw : post_block(raw);
}

// Binary search in ascending keys[0..n).
__device__ __forceinline__ bool in_sorted(const unsigned long long* keys, int n,
                                          unsigned long long k) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (keys[mid] < k)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < n && keys[lo] == k;
}

}  // namespace bna
