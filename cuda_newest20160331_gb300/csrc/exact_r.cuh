// Exact reference value of one pair (shared by the recompute and the
// density selection kernels).
#pragma once
#include "common.cuh"

namespace bna {

// Warp sum of 128-bit integers (two's complement, so signed sums too); every
// lane gets the total.
__device__ __forceinline__ unsigned __int128 warp_sum_u128(unsigned __int128 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long lo = __shfl_xor_sync(0xffffffffu, (unsigned long long)v, o);
    const unsigned long long hi = __shfl_xor_sync(0xffffffffu, (unsigned long long)(v >> 64), o);
    v += ((unsigned __int128)hi << 64) | lo;
  }
  return v;
}

__device__ __forceinline__ double u128_to_double(unsigned __int128 v) {
  return __dadd_rn(__dmul_rn((double)(unsigned long long)(v >> 64), 0x1p64),
                   (double)(unsigned long long)v);
}

// The float nearest to S = acc * 2^emin (acc exact, two's complement), and
// whether it is also the float nearest to every value within B of S, where
// B = (T + 1) 2^-51 mag 2^emin bounds the difference between S and the
// reference's sequential double sum of the same products (each of its T
// additions rounds by at most 2^-53 of a partial sum, and every partial sum
// is at most mag 2^emin = sum |p_t|; the bound carries a factor of 4 of
// margin): then the reference's float is this float.  False (sequential sum
// needed) when a float rounding midpoint lies within B of S, when S is 0, or
// when the result would leave float's normal range.
__device__ __forceinline__ bool round_sum_u128(unsigned __int128 acc, unsigned __int128 mag,
                                               int emin, int T, float* out) {
  const bool neg = (unsigned long long)(acc >> 127) != 0ull;
  const unsigned __int128 a = neg ? (~acc + 1) : acc;
  if (a == 0) return false;
  const unsigned long long ahi = (unsigned long long)(a >> 64);
  const int e = ahi ? 127 - __clzll((long long)ahi) : 63 - __clzll((long long)(unsigned long long)a);
  int eres = e + emin;  // weight of the leading bit: 2^eres
  uint32_t q24;
  double dist;  // distance from S to the nearest rounding midpoint, in units of 2^emin
  if (e >= 24) {
    const int sft = e - 23;
    const unsigned __int128 q = a >> sft;
    const unsigned __int128 rem = a - (q << sft);
    const unsigned __int128 half = (unsigned __int128)1 << (sft - 1);
    const unsigned __int128 dmid = rem > half ? rem - half : half - rem;
    // the midpoint below q: half a spacing lower, a quarter if q is a power of two
    const unsigned __int128 dlow = rem + ((unsigned long long)q == (1ull << 23) ? half >> 1 : half);
    dist = u128_to_double(dmid < dlow ? dmid : dlow);
    const bool up = rem > half || (rem == half && ((unsigned long long)q & 1ull));
    q24 = (uint32_t)(unsigned long long)q + (up ? 1u : 0u);
    if (q24 == (1u << 24)) {
      q24 = 1u << 23;
      ++eres;
    }
  } else {
    // at most 24 significant bits: S is a float; midpoints half a spacing away
    q24 = (uint32_t)(unsigned long long)a << (23 - e);
    dist = ldexp(1.0, e - 24 - (q24 == (1u << 23) ? 1 : 0));
  }
  if (eres < -125 || eres > 126) return false;
  const double bound = __dmul_rn(__dmul_rn((double)(T + 1), 0x1p-51), u128_to_double(mag));
  if (!(__dmul_rn(dist, 0.999) > bound)) return false;
  *out = __uint_as_float((neg ? 0x80000000u : 0u) | ((uint32_t)(eres + 127) << 23) |
                         (q24 & 0x7FFFFFu));
  return true;
}

// The reference value of a pair: float(sum_t double(float(z_it * z_jt))), the
// double sum in time order (CorMat.cpp:955-964).  A warp evaluates one pair:
// lanes take t = lane, lane+32, ...; the products are summed exactly in
// fixed point at the scale of the smallest one.  (1) When every product is
// normal, the int64 sum cannot overflow and sum |p_t| < 2^53 units of the
// smallest ulp, every partial sum of the sequential double loop is
// representable, so that loop equals the exact sum: an int64 reduction.
// (2) Otherwise (up to about 2^90 of spread) the exact sum is taken in
// 128-bit fixed point and its float is the reference's unless a rounding
// midpoint lies within the loop's rounding bound (round_sum_u128).  (3) Only
// then, or with subnormal or non-finite products, does lane 0 run the
// sequential double adds.  Returns the raw value (NaN for a voxel with a NaN
// z-score); exact_r_warp_z gives it after post_block's clamp.
__device__ __forceinline__ float exact_r_warp_raw(const float* z, const uint8_t* bad, int ldz,
                                                  int T, int i, int j, int lane) {
  if (bad[i] | bad[j]) return __int_as_float(0x7fc00000);  // NaN
  const float* zi = z + (size_t)i * ldz;
  const float* zj = z + (size_t)j * ldz;
  int emin = 1 << 20, emax = -(1 << 20);
  bool special = false;
#pragma unroll 4
  for (int t = lane; t < T; t += 32) {
    const uint32_t b = __float_as_uint(__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
    const int e8 = (int)((b >> 23) & 0xFFu);
    special |= (e8 == 0xFF) || (e8 == 0 && (b & 0x7FFFFFu));
    if (e8 != 0) {
      emin = min(emin, e8 - 150);
      emax = max(emax, e8 - 150);
    }
  }
  emin = __reduce_min_sync(0xffffffffu, emin);
  emax = __reduce_max_sync(0xffffffffu, emax);
  special = __any_sync(0xffffffffu, special);
  bool done = false;
  float r = 0.0f;
  if (!special && emin == (1 << 20)) {  // every product is zero
    done = true;
  } else if (!special && (emax - emin) + 24 + (32 - __clz(T)) <= 62) {  // no int64 overflow
    long long acc = 0, mag = 0;
    for (int t = lane; t < T; t += 32) {
      const uint32_t b = __float_as_uint(__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
      const int e8 = (int)((b >> 23) & 0xFFu);
      if (e8 == 0) continue;
      const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u) << (e8 - 150 - emin);
      mag += m;
      acc += (b >> 31) ? -m : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
      mag += __shfl_xor_sync(0xffffffffu, mag, o);
    }
    if (mag < (1LL << 53)) {
      r = __double2float_rn(__dmul_rn(__ll2double_rn(acc), ldexp(1.0, emin)));
      done = true;
    }
  }
  // (2): 24-bit mantissas shifted by up to emax - emin, T of them, below 2^127
  if (!done && !special && (emax - emin) + 24 + (32 - __clz(T)) <= 126) {
    unsigned __int128 acc = 0, mag = 0;
    for (int t = lane; t < T; t += 32) {
      const uint32_t b = __float_as_uint(__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
      const int e8 = (int)((b >> 23) & 0xFFu);
      if (e8 == 0) continue;
      const unsigned __int128 m = (unsigned __int128)((b & 0x7FFFFFu) | 0x800000u)
                                  << (e8 - 150 - emin);
      mag += m;
      acc += (b >> 31) ? (~m + 1) : m;
    }
    acc = warp_sum_u128(acc);
    mag = warp_sum_u128(mag);
    int ok = 0;
    if (lane == 0) ok = round_sum_u128(acc, mag, emin, T, &r) ? 1 : 0;
    done = __shfl_sync(0xffffffffu, ok, 0) != 0;
  }
  if (!done && lane == 0) {
    double s = 0.0;
    for (int t = 0; t < T; ++t)
      s = __dadd_rn(s, (double)__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
    r = __double2float_rn(s);
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
