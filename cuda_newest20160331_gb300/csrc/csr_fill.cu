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
// Sub-tiles with more than kFillDenseE edge-list entries (the dense blocks of
// networked data) are queued instead and placed by csr_fill_dense_kernel, one
// block per sub-tile: the entries' values are staged in a 128 x 128 shared-
// memory matrix, and each row run and each column run of the sub-tile is then
// written by one warp as consecutive CSR positions (coalesced stores instead
// of one scattered 4-byte store per column-direction entry).
// Positions are range-checked (ERR_RANGE) so an inconsistent count cannot
// write outside the CSR.
#include "common.cuh"

namespace bna {

constexpr int kFillWarps = 8;
constexpr long long kFillDenseE = 1024;  // entries above which a sub-tile takes the dense path

__device__ __forceinline__ int popc_before4(const uint32_t* m, int pos) {
  const int w = pos >> 5;
  int c = __popc(m[w] & ((1u << (pos & 31)) - 1u));
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (k < w) c += __popc(m[k]);
  return c;
}

__global__ __launch_bounds__(kFillWarps * 32) void csr_fill_kernel(CorrArgs a, long long nst,
                                                                   int* dense_list,
                                                                   unsigned int* dense_count) {
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
    if (E > kFillDenseE) {  // dense sub-tile: queued for csr_fill_dense_kernel
      if (lane == 0) dense_list[atomicAdd(dense_count, 1u)] = (int)st;
      continue;
    }
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

// Dense sub-tiles, one block (8 warps) per sub-tile.
struct DenseSmem {
  float val[128][129];  // val[il][jl] of the listed edges (padded: column reads conflict-free)
  uint32_t rm[128][4], cm[128][4];
  int rbase[128], cbase[128];
  long long start[4], cnt[4];
};

__global__ __launch_bounds__(256) void csr_fill_dense_kernel(CorrArgs a, const int* dense_list,
                                                             const unsigned int* dense_count) {
  extern __shared__ __align__(16) uint8_t fill_smem[];
  DenseSmem& S = *reinterpret_cast<DenseSmem*>(fill_smem);
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const uint32_t below = (1u << lane) - 1u;
  const unsigned int n = *dense_count;
  for (unsigned int idx = blockIdx.x; idx < n; idx += gridDim.x) {
    const long long st = dense_list[idx];
    if (tid < 4) {
      const longlong2 e = a.etab[st * 4 + tid];
      S.start[tid] = e.x;
      S.cnt[tid] = e.y;
    }
    for (int k = tid; k < 512; k += 256) {
      (&S.rm[0][0])[k] = 0u;
      (&S.cm[0][0])[k] = 0u;
    }
    __syncthreads();
    int I, J;
    tile_coords(st, a.nb, I, J);
    const bool diag = (I == J);
    // 1. bitmasks and values (ranges were checked by csr_fill_kernel)
    const long long p1 = S.cnt[0], p2 = p1 + S.cnt[1], p3 = p2 + S.cnt[2], E = p3 + S.cnt[3];
    for (long long e = tid; e < E; e += 256) {
      const int q = e < p1 ? 0 : e < p2 ? 1 : e < p3 ? 2 : 3;
      const long long off = e - (q == 0 ? 0 : q == 1 ? p1 : q == 2 ? p2 : p3);
      const uint2 en = a.elist[S.start[q] + off];
      const int il = en.x & 127, jl = (en.x >> 7) & 127;
      float v = __uint_as_float(en.y);
      bool edge = true;
      if ((en.x >> 14) & 1u) hash_lookup(a, pair_key(I * 128 + il, J * 128 + jl), v, edge);
      if (edge) {
        S.val[il][jl] = v;
        atomicOr(&S.rm[il][jl >> 5], 1u << (jl & 31));
        atomicOr(&S.cm[jl][il >> 5], 1u << (il & 31));
      }
    }
    __syncthreads();
    // 2. segment bases (as in csr_fill_kernel)
    if (tid < 128) {
      const int r = tid, gi = I * 128 + r;
      int b = 0;
      if (gi < a.n) {
        b = a.row_ptr[gi] + a.seg[(size_t)J * a.n_pad + gi];
        if (diag)
          b += __popc(S.cm[r][0]) + __popc(S.cm[r][1]) + __popc(S.cm[r][2]) + __popc(S.cm[r][3]);
      }
      S.rbase[r] = b;
    } else {
      const int r = tid - 128, gj = J * 128 + r;
      S.cbase[r] = (gj < a.n) ? a.row_ptr[gj] + a.seg[(size_t)I * a.n_pad + gj] : 0;
    }
    __syncthreads();
    // 3. row runs (row il of block I, columns of block J) and column runs (row
    //    jl of block J, columns of block I), one warp per run, lane = bit
    for (int r = w; r < 256; r += 8) {
      const bool rows = r < 128;
      const int x = rows ? r : r - 128;
      const uint32_t* m = rows ? S.rm[x] : S.cm[x];
      long long pos = rows ? S.rbase[x] : S.cbase[x];
      const int colbase = rows ? J * 128 : I * 128;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t bits = m[q];
        if ((bits >> lane) & 1u) {
          const int y = q * 32 + lane;
          put_edge(a, pos + __popc(bits & below), colbase + y, rows ? S.val[x][y] : S.val[y][x]);
        }
        pos += __popc(bits);
      }
    }
    __syncthreads();
  }
}

cudaError_t launch_csr_fill(const CorrArgs& a, int sms, int* dense_list, unsigned int* dense_count,
                            cudaStream_t stream) {
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  const long long want = (nst + kFillWarps - 1) / kFillWarps;
  const int grid = (int)(want < (long long)sms * 4 ? want : (long long)sms * 4);
  if (grid <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(dense_count, 0, sizeof(unsigned int), stream);
  if (e != cudaSuccess) return e;
  csr_fill_kernel<<<grid, kFillWarps * 32, 0, stream>>>(a, nst, dense_list, dense_count);
  e = cudaFuncSetAttribute(csr_fill_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(DenseSmem));
  if (e != cudaSuccess) return e;
  csr_fill_dense_kernel<<<sms * 3, 256, sizeof(DenseSmem), stream>>>(a, dense_list, dense_count);
  return cudaGetLastError();
}

}  // namespace bna
