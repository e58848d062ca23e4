// Multi-subject averaging with optional Fisher z: the reference's
// to_average modes y/b (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:418-670).
//
// The reference accumulates, in file order, each subject's correlation into
// one packed float matrix (post_block with its fishtran flag, :847-883: r is
// added - or fishertrans(r) - only when -1 <= r <= 1), divides by the number
// of subjects (and applies inv_fishertrans), then thresholds the result like
// a single subject's matrix.  Here the accumulation is the tensor-core pass 4
// (approximate r~ of every pair, corr_tc.cu), these kernels finish the
// average, and the count pass reads the averaged values instead of a GEMM.
// Pairs whose average lies near the threshold (or where some subject's r~ is
// near +-1, where post_block's rule or the Fisher transform is sensitive) get
// their exact average: every subject's reference r (float products, time-
// order double sum), the same float accumulation, division and transforms.
#include "common.cuh"
#include "exact_r.cuh"

namespace bna {

struct SubjZ {
  const float* z;
  const uint8_t* bad;
  int ldz, T;
};

__global__ void avg_finalize_kernel(float* packed, long long m, int S, int fisher) {
  const float fs = (float)S;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x) {
    float v = __fdiv_rn(packed[i], fs);
    if (fisher) v = fisher_r(v);
    packed[i] = v;
  }
}

// Exact averaged value of every candidate slot (warp per candidate).
__global__ void avg_exact_kernel(CorrArgs a, const SubjZ* __restrict__ subj, int S, int fisher,
                                 float* out) {
  const unsigned long long cnt = *a.cand_count;
  const long long n = (long long)cnt < a.cand_cap ? (long long)cnt : a.cand_cap;
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long c = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); c < n;
       c += nw) {
    const uint2 p = a.cand[c];
    if (p.x == kCandNone) continue;
    float acc = 0.0f;
    for (int s = 0; s < S; ++s) {
      // post_block'd reference value: outside [-1, 1] (or NaN) it is 0, which
      // adds nothing, as the reference's skipped addition
      const float r = exact_r_warp_z(subj[s].z, subj[s].bad, subj[s].ldz, subj[s].T, (int)p.x,
                                     (int)p.y, lane);
      acc = __fadd_rn(acc, fisher ? fisher_z(r) : r);
    }
    float v = __fdiv_rn(acc, (float)S);
    if (fisher) v = fisher_r(v);
    if (lane == 0) out[c] = v;
  }
}

cudaError_t launch_avg_finalize(float* packed, long long m, int S, int fisher, int sms,
                                cudaStream_t st) {
  avg_finalize_kernel<<<sms * 8, 256, 0, st>>>(packed, m, S, fisher);
  return cudaGetLastError();
}

cudaError_t launch_avg_exact(const CorrArgs& a, const void* subj, int S, int fisher, float* out,
                             int sms, cudaStream_t st) {
  // an odd grid: candidate slots come in 256-slot chunks filled from the front
  avg_exact_kernel<<<sms * 8 - 1, 256, 0, st>>>(a, static_cast<const SubjZ*>(subj), S, fisher,
                                                 out);
  return cudaGetLastError();
}

size_t avg_subj_bytes() { return sizeof(SubjZ); }

void avg_subj_fill(void* host, int s, const float* z, const uint8_t* bad, int ldz, int T) {
  SubjZ* h = static_cast<SubjZ*>(host);
  h[s].z = z;
  h[s].bad = bad;
  h[s].ldz = ldz;
  h[s].T = T;
}

}  // namespace bna
