// Near-threshold recompute and CSR offset scans.
//
// Recompute: every candidate pair (|r_approx - tau| <= delta, or |r_approx|
// near 1) is evaluated with the reference CPU arithmetic of CorMat_cpu
// (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:955-964): float products of the
// float z-scores, accumulated in double in time order, rounded to float;
// then post_block's clamp (CorMat.cpp:883; not for the 2mm tools' rule,
// BNA_THR_R_EPS) and the exact threshold rule.
// Sequential per pair, so the value is bit-identical to the reference's.
//
// Scan: seg[b][i] (edges of row i in column block b) becomes the exclusive
// prefix along b, and row_ptr = exclusive prefix of the row totals
// (FormCSRGraph's R, CorMat.cpp:889-918).
#include "common.cuh"
#include "exact_r.cuh"

namespace bna {

// One pair on one thread, sequential double adds (diagnostics only).
__device__ __forceinline__ float exact_r(const CorrArgs& a, int i, int j) {
  if (a.bad[i] | a.bad[j]) return 0.0f;
  const float* zi = a.z + (size_t)i * a.ldz;
  const float* zj = a.z + (size_t)j * a.ldz;
  double s = 0.0;
  for (int t = 0; t < a.T; ++t) s = __dadd_rn(s, (double)__fmul_rn(__ldg(zi + t), __ldg(zj + t)));
  return post_block(__double2float_rn(s));
}


// Exact values of the candidates only (density mode: the threshold is
// selected from them before any decision is made).
__global__ void cand_values_kernel(CorrArgs a, float* vals) {
  const unsigned long long cnt = *a.cand_count;
  const long long n = (long long)cnt < a.cand_cap ? (long long)cnt : a.cand_cap;
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long c = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); c < n;
       c += nwarps) {
    const uint2 p = a.cand[c];
    if (p.x == kCandNone) continue;  // unused slot of a count-pass chunk
    const float r = exact_r_warp(a, (int)p.x, (int)p.y, lane);
    if (lane == 0) vals[c] = r;
  }
}

// Decide every candidate on its exact value (computed here, or given in
// a.cand_val), add the edges to the counts and store value + decision in the
// hash the fill pass reads.
__global__ void recompute_kernel(CorrArgs a) {
  const unsigned long long cnt = *a.cand_count;
  const long long n = (long long)cnt < a.cand_cap ? (long long)cnt : a.cand_cap;
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long c = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); c < n;
       c += nwarps) {
    const uint2 p = a.cand[c];
    if (p.x == kCandNone) continue;  // unused slot of a count-pass chunk
    const int i = (int)p.x, j = (int)p.y;
    const float r = a.cand_val ? a.cand_val[c] : exact_r_rule(a, i, j, lane);
    if (lane != 0) continue;
    const unsigned long long key = pair_key(i, j);
    bool e = edge_exact(r, a.th);
    if (e && a.th.mode == BNA_THR_DENSITY && r == a.th.tau && a.n_drop > 0 &&
        in_sorted(a.drop_keys, a.n_drop, key))
      e = false;
    if (e) {
      atomicAdd(&a.seg[(size_t)(j / kBlk) * a.n_pad + i], 1);
      atomicAdd(&a.seg[(size_t)(i / kBlk) * a.n_pad + j], 1);
      atomicAdd(&a.stats[0], 1ull);
    }
    const bool absm = (a.th.mode == BNA_THR_ABS_GT || a.th.mode == BNA_THR_ABS_GE);
    if (fabsf((absm ? fabsf(r) : r) - a.th.tau) <= 1e-6f) atomicAdd(&a.stats[1], 1ull);
    unsigned long long h = hash64(key) & a.hmask;
    bool stored = false;
    for (unsigned long long probe = 0; probe <= a.hmask; ++probe) {
      const unsigned long long prev = atomicCAS(&a.hkeys[h], ~0ull, key);
      if (prev == ~0ull || prev == key) {
        a.hval[h] = r;
        a.hedge[h] = e ? 1 : 0;
        stored = true;
        break;
      }
      h = (h + 1) & a.hmask;
    }
    if (!stored) atomicOr(a.err, ERR_HASH_FULL);
  }
}

// Gather the candidates flagged in the sub-tiles' edge lists into the
// candidate list (warp per sub-tile, one atomic per warp and round).  Used
// after the plain FP32 count pass; the tensor-core pass lists its candidates
// itself.
__global__ void collect_candidates_kernel(CorrArgs a, long long nst) {
  const int wpb = blockDim.x >> 5;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t below = (1u << lane) - 1u;
  for (long long st = (long long)blockIdx.x * wpb + w; st < nst; st += (long long)gridDim.x * wpb) {
    long long s0 = 0, c0 = 0;
    if (lane < 4) {
      const longlong2 e = a.etab[st * 4 + lane];
      s0 = e.x;
      c0 = e.y;
    }
    long long start[4], cnt[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      start[q] = __shfl_sync(0xffffffffu, s0, q);
      cnt[q] = __shfl_sync(0xffffffffu, c0, q);
    }
    bool inside = true;  // ranges written while the pool overflowed are not read
#pragma unroll
    for (int q = 0; q < 4; ++q)
      inside &= cnt[q] >= 0 && start[q] >= 0 && start[q] + cnt[q] <= a.ecap;
    if (!inside) {
      if (lane == 0) atomicOr(a.err, ERR_ELIST);
      continue;
    }
    const long long E = cnt[0] + cnt[1] + cnt[2] + cnt[3];
    if (E == 0) continue;
    int I, J;
    tile_coords(st, a.nb, I, J);
    const long long p1 = cnt[0], p2 = p1 + cnt[1], p3 = p2 + cnt[2];
    for (long long e0 = 0; e0 < E; e0 += 32) {
      const long long e = e0 + lane;
      bool flag = false;
      uint32_t key = 0;
      if (e < E) {
        const int q = e < p1 ? 0 : e < p2 ? 1 : e < p3 ? 2 : 3;
        const long long off = e - (q == 0 ? 0 : q == 1 ? p1 : q == 2 ? p2 : p3);
        const long long s = q == 0 ? start[0] : q == 1 ? start[1] : q == 2 ? start[2] : start[3];
        key = a.elist[s + off].x;
        flag = ((key >> 14) & 1u) != 0u;
      }
      const uint32_t bal = __ballot_sync(0xffffffffu, flag);
      // definite (unflagged) entries of this round, for the density selection
      const int nvalid = (int)((E - e0) < 32 ? (E - e0) : 32);
      if (lane == 0 && nvalid - __popc(bal) > 0)
        atomicAdd(&a.stats[2], (unsigned long long)(nvalid - __popc(bal)));
      if (!bal) continue;
      if (lane == 0) atomicAdd(&a.stats[3], (unsigned long long)__popc(bal));
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(a.cand_count, (unsigned long long)__popc(bal));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (flag) {
        const unsigned long long slot = base + __popc(bal & below);
        if ((long long)slot < a.cand_cap)
          a.cand[slot] = make_uint2((unsigned)(I * 128 + (key & 127)),
                                    (unsigned)(J * 128 + ((key >> 7) & 127)));
        else
          atomicOr(a.err, ERR_BAND_OVERFLOW);
      }
    }
  }
}

// Exact values of arbitrary pairs (diagnostics: max |r - r_ref| of a form).
__global__ void exact_pairs_kernel(CorrArgs a, const uint2* pairs, int n, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) out[c] = exact_r(a, (int)pairs[c].x, (int)pairs[c].y);
}

// seg[b][i] -> exclusive prefix over b; rowlen[i] = row total.  Loads are
// issued 16 at a time so each thread keeps 16 requests in flight.
__global__ void seg_scan_rows_kernel(int32_t* seg, int nb, int n_pad, int n, long long* rowlen) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  long long acc = 0;
  int b = 0;
  for (; b + 16 <= nb; b += 16) {
    int c[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) c[u] = seg[(size_t)(b + u) * n_pad + i];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      seg[(size_t)(b + u) * n_pad + i] = (int)acc;
      acc += c[u];
    }
  }
  for (; b < nb; ++b) {
    int32_t* p = seg + (size_t)b * n_pad + i;
    const int c = *p;
    *p = (int)acc;
    acc += c;
  }
  if (i < n) rowlen[i] = acc;
}

// Block-local exclusive scan of 4096 int64 values (1024 threads x 4).
__global__ __launch_bounds__(1024) void scan_block_kernel(const long long* in, int n, long long* out,
                                                          long long* bsum) {
  __shared__ long long wsum[32];
  const int base = blockIdx.x * 4096 + threadIdx.x * 4;
  long long v[4];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    long long w = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  long long run = x - s + (warp > 0 ? wsum[warp - 1] : 0);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 1023) bsum[blockIdx.x] = run;
}

__global__ __launch_bounds__(1024) void scan_sums_kernel(long long* bsum, int nblk,
                                                         long long* total) {
  __shared__ long long wsum[32];
  const int base = threadIdx.x * 4;
  long long v[4];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = (base + k < nblk) ? bsum[base + k] : 0;
    s += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    long long w = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  long long run = x - s + (warp > 0 ? wsum[warp - 1] : 0);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (base + k < nblk) bsum[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 1023) *total = run;
}

__global__ void scan_finish_kernel(const long long* pre, const long long* bsum, int n,
                                   const long long* total, int32_t* row_ptr, uint32_t* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const long long v = pre[i] + bsum[i / 4096];
    row_ptr[i] = (int32_t)v;
    if (v > 0x7fffffffLL) atomicOr(err, ERR_NNZ_INT32);
  } else if (i == n) {
    const long long v = *total;
    row_ptr[n] = (int32_t)v;
    if (v > 0x7fffffffLL) atomicOr(err, ERR_NNZ_INT32);
  }
}

// Candidate slots come in 256-slot chunks filled from the front; a warp count
// that is a multiple of 256 would give every warp the same offset in each
// chunk (and the filled offsets to a few warps): the grid is made odd.
static int odd_grid(int grid) { return grid > 1 ? (grid | 1) - 2 * ((grid & 1) == 0) : 1; }

cudaError_t launch_recompute(const CorrArgs& a, int grid, cudaStream_t stream) {
  recompute_kernel<<<odd_grid(grid), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cand_values(const CorrArgs& a, float* vals, int grid, cudaStream_t stream) {
  cand_values_kernel<<<odd_grid(grid), 256, 0, stream>>>(a, vals);
  return cudaGetLastError();
}

cudaError_t launch_collect_candidates(const CorrArgs& a, int sms, cudaStream_t stream) {
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  const long long want = (nst + 7) / 8;
  const int grid = (int)(want < (long long)sms * 8 ? want : (long long)sms * 8);
  if (grid <= 0) return cudaSuccess;
  collect_candidates_kernel<<<grid, 256, 0, stream>>>(a, nst);
  return cudaGetLastError();
}

cudaError_t launch_exact_pairs(const CorrArgs& a, const uint2* pairs, int n, float* out,
                               cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  exact_pairs_kernel<<<(n + 127) / 128, 128, 0, stream>>>(a, pairs, n, out);
  return cudaGetLastError();
}

// rowlen/pre: n int64; bsum: ceil(n/4096) int64 (<= 4096 blocks); total: 1 int64.
cudaError_t launch_csr_scan(int32_t* seg, int nb, int n_pad, int n, long long* rowlen,
                            long long* pre, long long* bsum, long long* total, int32_t* row_ptr,
                            uint32_t* err, cudaStream_t stream) {
  const int nblk = (n + 4095) / 4096;
  if (nblk > 4096) return cudaErrorInvalidValue;
  seg_scan_rows_kernel<<<(n_pad + 127) / 128, 128, 0, stream>>>(seg, nb, n_pad, n, rowlen);
  scan_block_kernel<<<nblk, 1024, 0, stream>>>(rowlen, n, pre, bsum);
  scan_sums_kernel<<<1, 1024, 0, stream>>>(bsum, nblk, total);
  scan_finish_kernel<<<(n + 1 + 255) / 256, 256, 0, stream>>>(pre, bsum, n, total, row_ptr, err);
  return cudaGetLastError();
}

// Exclusive prefix of given row lengths -> row_ptr (no seg step).
cudaError_t launch_rowlen_scan(const long long* rowlen, int n, long long* pre, long long* bsum,
                               long long* total, int32_t* row_ptr, uint32_t* err,
                               cudaStream_t stream) {
  const int nblk = (n + 4095) / 4096;
  if (nblk > 4096) return cudaErrorInvalidValue;
  scan_block_kernel<<<nblk, 1024, 0, stream>>>(rowlen, n, pre, bsum);
  scan_sums_kernel<<<1, 1024, 0, stream>>>(bsum, nblk, total);
  scan_finish_kernel<<<(n + 1 + 255) / 256, 256, 0, stream>>>(pre, bsum, n, total, row_ptr, err);
  return cudaGetLastError();
}

}  // namespace bna
