// Several thresholds from one correlation pass: the reference's CUCorMat
// takes a list of thresholds on its command line and thresholds the same
// correlation matrix once per value (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:
// 105-111, 318-341).  Here the CSR of the lowest threshold tau0 (built by
// bna_corr_csr) already holds every pair of any higher threshold tau of the
// same rule, each with a value within delta of the reference's r (exactly r
// where the band recomputed it).  The CSR for tau keeps, row by row and in
// order, the entries that pass tau: decided on the stored value when it is
// more than delta from tau (and from +-1, where post_block clamps), otherwise
// on the exact reference value, recomputed here from the same z-scores.
#include "common.cuh"
#include "exact_r.cuh"

namespace bna {

// Warp per row: keep flag of every entry, the value to store (exact where it
// was recomputed), the row's kept count.
__global__ void rethr_count_kernel(CorrArgs a, const int32_t* __restrict__ rp,
                                   const int32_t* __restrict__ ci, const float* __restrict__ val,
                                   Threshold th, uint8_t* keep, float* valx, long long* rowlen,
                                   unsigned long long* band) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  const bool absm = th.mode == BNA_THR_ABS_GT || th.mode == BNA_THR_ABS_GE;
  const float lim = 1.0f - th.delta;
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < a.n; i += nw) {
    const long long b = rp[i], e = rp[i + 1];
    long long kept = 0;
    for (long long e0 = b; e0 < e; e0 += 32) {
      const long long k = e0 + lane;
      const bool in = k < e;
      float v = in ? val[k] : 0.0f;
      const float x = absm ? fabsf(v) : v;
      const bool need = in && (fabsf(x - th.tau) <= th.delta || fabsf(v) >= lim);
      bool kp = in && !need && edge_exact(v, th);
      uint32_t m = __ballot_sync(0xffffffffu, need);
      while (m) {  // exact values, one pair per warp pass
        const int l = __ffs(m) - 1;
        m &= m - 1;
        const int j = __shfl_sync(0xffffffffu, in ? ci[k] : 0, l);
        const float r = exact_r_warp(a, i < j ? i : j, i < j ? j : i, lane);
        if (lane == l) {
          v = r;
          kp = edge_exact(r, th);
          if (fabsf((absm ? fabsf(r) : r) - th.tau) <= 1e-6f) atomicAdd(band, 1ull);
        }
      }
      if (in) {
        keep[k] = kp ? 1 : 0;
        valx[k] = v;
      }
      kept += __popc(__ballot_sync(0xffffffffu, kp));
    }
    if (lane == 0) rowlen[i] = kept;
  }
}

// Warp per row: copy the kept entries in order.
__global__ void rethr_fill_kernel(int n, const int32_t* __restrict__ rp,
                                  const int32_t* __restrict__ ci, const float* __restrict__ valx,
                                  const uint8_t* __restrict__ keep, const int32_t* __restrict__ rp2,
                                  int32_t* ci2, float* val2, long long nnz2, uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += nw) {
    const long long b = rp[i], e = rp[i + 1];
    long long pos = rp2[i];
    for (long long e0 = b; e0 < e; e0 += 32) {
      const long long k = e0 + lane;
      const bool kp = k < e && keep[k];
      const uint32_t m = __ballot_sync(0xffffffffu, kp);
      if (kp) {
        const long long p = pos + __popc(m & ((1u << lane) - 1u));
        if (p < nnz2) {
          ci2[p] = ci[k];
          if (val2) val2[p] = valx[k];
        } else {
          atomicOr(err, ERR_RANGE);
        }
      }
      pos += __popc(m);
    }
  }
}

cudaError_t launch_rethr_count(const CorrArgs& a, const int32_t* rp, const int32_t* ci,
                               const float* val, const Threshold& th, uint8_t* keep, float* valx,
                               long long* rowlen, unsigned long long* band, int sms,
                               cudaStream_t st) {
  rethr_count_kernel<<<sms * 8, 256, 0, st>>>(a, rp, ci, val, th, keep, valx, rowlen, band);
  return cudaGetLastError();
}

cudaError_t launch_rethr_fill(int n, const int32_t* rp, const int32_t* ci, const float* valx,
                              const uint8_t* keep, const int32_t* rp2, int32_t* ci2, float* val2,
                              long long nnz2, uint32_t* err, int sms, cudaStream_t st) {
  rethr_fill_kernel<<<sms * 8, 256, 0, st>>>(n, rp, ci, valx, keep, rp2, ci2, val2, nnz2, err);
  return cudaGetLastError();
}

}  // namespace bna
