// Host -> device copy by the SMs: a kernel reads the caller's page-locked,
// device-mapped host buffer directly and writes device memory.
//
// No reference counterpart (the reference copies with cudaMemcpy).  The
// serving engine uploads each request's series this way: on this system a
// copy-engine upload ran at ~210 GB/s alone but at a few GB/s while several
// requests' kernels and transfers shared the device, and a small request's
// upload then waited behind a large one's in the copy engine's queue; the
// SM-driven copy ran at the same ~210 GB/s alone and unchanged beside a
// running correlation pass.
#include <cstdint>

#include "common.cuh"

namespace bna {

// Each thread keeps four independent 16-byte loads of host memory in flight
// before it stores them: the link's latency grows when the host is busy, and
// one load per thread then left the copy latency-bound (measured: a copy with
// one load in flight fell to ~50 GB/s while this form held ~205 GB/s).
__global__ void copy_from_host_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                      size_t n16, const uint8_t* __restrict__ src_tail,
                                      uint8_t* __restrict__ dst_tail, int tail) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
  if (blockIdx.x == 0 && (int)threadIdx.x < tail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

// Copies `bytes` from host buffer `src` to device buffer `dst` on `stream`
// with a kernel when `src` is page-locked and mapped into the device's
// address space and both pointers are 16-byte aligned; returns
// cudaErrorInvalidValue (nothing launched) otherwise, and the caller copies
// with cudaMemcpyAsync.
cudaError_t copy_from_host(const void* src, void* dst, size_t bytes, int sms,
                           cudaStream_t stream) {
  if (bytes == 0) return cudaSuccess;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, src) != cudaSuccess) {
    cudaGetLastError();
    return cudaErrorInvalidValue;
  }
  const void* dsrc = at.devicePointer;
  if (at.type != cudaMemoryTypeHost || dsrc == nullptr || ((uintptr_t)dsrc & 15) ||
      ((uintptr_t)dst & 15))
    return cudaErrorInvalidValue;
  const size_t n16 = bytes / 16;
  const int tail = (int)(bytes - n16 * 16);
  const long long want = ((long long)n16 + 1023) / 1024;  // 4 x 16 B per thread
  const int grid = (int)(want < 1 ? 1 : (want < (long long)sms * 4 ? want : (long long)sms * 4));
  copy_from_host_kernel<<<grid, 256, 0, stream>>>(
      static_cast<const uint4*>(dsrc), static_cast<uint4*>(dst), n16,
      static_cast<const uint8_t*>(dsrc) + n16 * 16, static_cast<uint8_t*>(dst) + n16 * 16, tail);
  return cudaGetLastError();
}

}  // namespace bna
