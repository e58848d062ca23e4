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
//
// The copy runs on a few SMs only (kUploadBlocks blocks of 1024 threads):
// 16 such blocks already reach the link's ~211 GB/s, and a copy spread over
// every SM kept a high-priority kernel of another stream from finishing until
// the whole copy had drained (measured: a 0.1 ms kernel took 3.9 ms beside an
// 808 MB copy of 608 blocks of 256 threads, 0.12-0.17 ms beside one of 32
// blocks of 1024): each SM's load path stays full of host loads, whose
// latency is the link's, for the length of the copy.
#include <algorithm>
#include <cstdint>

#include "common.cuh"

namespace bna {

constexpr int kUploadThreads = 1024;
constexpr int kUploadBlocks = 32;
constexpr size_t kChunk16 = 1024;  // 16 KB: one warp's contiguous piece

// Each warp copies 16 KB chunks (chunk w, w + warps, ...), every lane keeping
// four independent 16-byte loads of host memory in flight before it stores
// them: the link's latency grows when the host is busy, and one load per
// thread then left the copy latency-bound (measured: a copy with one load in
// flight fell to ~50 GB/s while this form held ~205 GB/s).  Chunks per warp
// rather than one sweep over the buffer put about a quarter as many distinct
// 64 KB host pages in flight as warps (a sweep: one per 64 KB of loads in
// flight), for the times when a host page's first access is slow (uploads
// then ran at 6-8 GB/s as a sweep, 10-25 GB/s in chunks; 300 serving requests
// on one machine: per-request slowdown p99 2.1 and 3.1 in chunks, 5.0 as a
// sweep between them).
// With `blocks` set (diagnostics), each block records its start and end time
// (global timer, ns) and its SM: blocks[3 b + 0..2].
__global__ __launch_bounds__(kUploadThreads) void copy_from_host_kernel(
    const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16,
    const uint8_t* __restrict__ src_tail, uint8_t* __restrict__ dst_tail, int tail,
    unsigned long long* blocks) {
  if (blocks && threadIdx.x == 0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    blocks[3 * blockIdx.x] = t;
  }
  const int lane = threadIdx.x & 31;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  const size_t nchunks = (n16 + kChunk16 - 1) / kChunk16;
  for (size_t c = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nchunks;
       c += nwarps) {
    const size_t end = c * kChunk16 + kChunk16 < n16 ? c * kChunk16 + kChunk16 : n16;
    size_t i = c * kChunk16 + lane;
    for (; i + 96 < end; i += 128) {
      const uint4 a = src[i], b = src[i + 32], d = src[i + 64], e = src[i + 96];
      dst[i] = a;
      dst[i + 32] = b;
      dst[i + 64] = d;
      dst[i + 96] = e;
    }
    for (; i < end; i += 32) dst[i] = src[i];
  }
  if (blockIdx.x == 0 && (int)threadIdx.x < tail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
  if (blocks) {
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t;
      unsigned int sm;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
      blocks[3 * blockIdx.x + 1] = t;
      blocks[3 * blockIdx.x + 2] = sm;
    }
  }
}

// Copies `bytes` from host buffer `src` to device buffer `dst` on `stream`
// with a kernel when `src` is page-locked and mapped into the device's
// address space and both pointers are 16-byte aligned; returns
// cudaErrorInvalidValue (nothing launched) otherwise, and the caller copies
// with cudaMemcpyAsync.  `blocks` (optional, device memory of 3 x
// upload_max_blocks() values) receives each block's times and SM; *grid_out
// the number of blocks.
int upload_max_blocks() { return kUploadBlocks; }

cudaError_t copy_from_host(const void* src, void* dst, size_t bytes, int sms,
                           cudaStream_t stream, unsigned long long* blocks, int* grid_out) {
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
  // a warp per 16 KB chunk; at most kUploadBlocks blocks (and a quarter of
  // the SMs)
  const long long chunks = (long long)((n16 + kChunk16 - 1) / kChunk16);
  const long long want = (chunks + kUploadThreads / 32 - 1) / (kUploadThreads / 32);
  const long long most = std::max(1, std::min(kUploadBlocks, sms / 4));
  const int grid = (int)std::max(1LL, std::min(want, most));
  copy_from_host_kernel<<<grid, kUploadThreads, 0, stream>>>(
      static_cast<const uint4*>(dsrc), static_cast<uint4*>(dst), n16,
      static_cast<const uint8_t*>(dsrc) + n16 * 16, static_cast<uint8_t*>(dst) + n16 * 16, tail,
      blocks);
  if (grid_out) *grid_out = grid;
  return cudaGetLastError();
}

}  // namespace bna
