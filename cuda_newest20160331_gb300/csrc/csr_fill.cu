// Fill pass: place every listed edge into the CSR.
//
// Reference: FormCSRGraph (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:889-918) —
// rows in order, columns ascending, both (i, j) and (j, i) of each pair,
// V[e] = r of the pair.  Here the count pass has left, per 128 x 128
// sub-tile (I, J), I <= J, a compact list of its edges (value) and of its
// near-threshold candidates (resolved by the recompute pass into a hash).
// One warp handles one sub-tile:
//   1. mark every edge in the sub-tile's row and column bitmasks (smem);
//   2. bases: row i of block I starts its block-J segment at
//      row_ptr[i] + seg[J][i] (+ the count of its column-direction entries
//      on a diagonal sub-tile); column j of block J starts at
//      row_ptr[j] + seg[I][j];
//   3. each edge goes to base + (number of set bits before it) in its row
//      mask and in its column mask.
// Positions are range-checked (ERR_RANGE) so an inconsistent count cannot
// write outside the CSR.
#include "common.cuh"

namespace bna {

constexpr int kFillWarps = 8;

__device__ __forceinline__ int popc_before4(const uint32_t* m, int pos) {
  const int w = pos >> 5;
  int c = __popc(m[w] & ((1u << (pos & 31)) - 1u));
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (k < w) c += __popc(m[k]);
  return c;
}

__global__ __launch_bounds__(kFillWarps * 32) void csr_fill_kernel(CorrArgs a, long long nst) {
  __shared__ uint32_t rmask[kFillWarps][128][4];
  __shared__ uint32_t cmask[kFillWarps][128][4];
  __shared__ int rbase[kFillWarps][128];
  __shared__ int cbase[kFillWarps][128];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t(*rm)[4] = rmask[w];
  uint32_t(*cm)[4] = cmask[w];
  for (long long st = (long long)blockIdx.x * kFillWarps + w; st < nst;
       st += (long long)gridDim.x * kFillWarps) {
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
    const bool diag = (I == J);
    for (int idx = lane; idx < 512; idx += 32) {
      rm[idx >> 2][idx & 3] = 0u;
      cm[idx >> 2][idx & 3] = 0u;
    }
    __syncwarp();
    const long long p1 = cnt[0], p2 = p1 + cnt[1], p3 = p2 + cnt[2];
    auto entry = [&](long long e) {
      const int q = e < p1 ? 0 : e < p2 ? 1 : e < p3 ? 2 : 3;
      const long long off = e - (q == 0 ? 0 : q == 1 ? p1 : q == 2 ? p2 : p3);
      const long long s = q == 0 ? start[0] : q == 1 ? start[1] : q == 2 ? start[2] : start[3];
      return a.elist[s + off];
    };
    // 1. bitmasks (candidates resolved through the recompute hash)
    for (long long e = lane; e < E; e += 32) {
      const uint2 en = entry(e);
      const int il = en.x & 127, jl = (en.x >> 7) & 127;
      bool edge = true;
      if ((en.x >> 14) & 1u) {
        float v;
        hash_lookup(a, pair_key(I * 128 + il, J * 128 + jl), v, edge);
      }
      if (edge) {
        atomicOr(&rm[il][jl >> 5], 1u << (jl & 31));
        atomicOr(&cm[jl][il >> 5], 1u << (il & 31));
      }
    }
    __syncwarp();
    // 2. segment bases of the 128 rows and 128 columns
    for (int r = lane; r < 128; r += 32) {
      const int gi = I * 128 + r, gj = J * 128 + r;
      int b = 0;
      if (gi < a.n) {
        b = a.row_ptr[gi] + a.seg[(size_t)J * a.n_pad + gi];
        if (diag) b += __popc(cm[r][0]) + __popc(cm[r][1]) + __popc(cm[r][2]) + __popc(cm[r][3]);
      }
      rbase[w][r] = b;
      cbase[w][r] = (gj < a.n) ? a.row_ptr[gj] + a.seg[(size_t)I * a.n_pad + gj] : 0;
    }
    __syncwarp();
    // 3. place both directions
    for (long long e = lane; e < E; e += 32) {
      const uint2 en = entry(e);
      const int il = en.x & 127, jl = (en.x >> 7) & 127;
      const int gi = I * 128 + il, gj = J * 128 + jl;
      float v = __uint_as_float(en.y);
      bool edge = true;
      if ((en.x >> 14) & 1u) hash_lookup(a, pair_key(gi, gj), v, edge);
      if (!edge) continue;
      put_edge(a, (long long)rbase[w][il] + popc_before4(rm[il], jl), gj, v);
      put_edge(a, (long long)cbase[w][jl] + popc_before4(cm[jl], il), gi, v);
    }
    __syncwarp();
  }
}

cudaError_t launch_csr_fill(const CorrArgs& a, int sms, cudaStream_t stream) {
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  const long long want = (nst + kFillWarps - 1) / kFillWarps;
  const int grid = (int)(want < (long long)sms * 4 ? want : (long long)sms * 4);
  if (grid <= 0) return cudaSuccess;
  csr_fill_kernel<<<grid, kFillWarps * 32, 0, stream>>>(a, nst);
  return cudaGetLastError();
}

}  // namespace bna
