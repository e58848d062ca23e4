// Degree of every vertex of a device CSR: the reference's Degree tool
// (W/Degree/Degree/Degree.cpp:80-84), Degree[k] = the float sum of the row's
// values in column order; for a binary graph (no values) the row length.
// One warp per row: the values are loaded coalesced, 32 at a time, and lane 0
// adds them in order, so the float result equals the reference's.
#include <cuda_runtime.h>

#include <cstdint>

#include "bna.h"

namespace {

__global__ void degree_kernel(int n, const int32_t* __restrict__ rp,
                              const float* __restrict__ val, float* deg) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n; k += nw) {
    const int b = rp[k], e = rp[k + 1];
    if (!val) {
      if (lane == 0) deg[k] = (float)(e - b);
      continue;
    }
    float s = 0.0f;
    for (int e0 = b; e0 < e; e0 += 32) {
      const float v = e0 + lane < e ? __ldg(val + e0 + lane) : 0.0f;
      const int m = e - e0 < 32 ? e - e0 : 32;
      for (int q = 0; q < m; ++q) s = __fadd_rn(s, __shfl_sync(0xffffffffu, v, q));
    }
    if (lane == 0) deg[k] = s;
  }
}

}  // namespace

extern "C" int32_t bna_degree(const bna_csr* csr_dev, float* deg_dev, void* stream) {
  if (!csr_dev || !deg_dev || csr_dev->n < 1 || !csr_dev->row_ptr) return BNA_BAD_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return BNA_CUDA_ERROR;
  }
  degree_kernel<<<sms * 8, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      csr_dev->n, csr_dev->row_ptr, csr_dev->nnz > 0 ? csr_dev->val : nullptr, deg_dev);
  return cudaGetLastError() == cudaSuccess ? BNA_OK : BNA_CUDA_ERROR;
}
