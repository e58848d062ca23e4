// Plain FP32 correlation -> CSR on CUDA cores (the "plain form").
//
// Reference: the tile loop of CorMat_gpu (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:87-154,
// cublasSgemm at :94) followed by post_block / FormFullGraph / FormCSRGraph
// (CorMat.cpp:824-918).  Here each CTA computes one 128 x 128 tile (I, J),
// I <= J, of Z Z^T in FP32 and thresholds it in registers; the N x N matrix
// never exists.
//
// The tile epilogue is shared by two launches over the same tiles:
//   count pass: per tile, count edges per row (seg[J][i]) and per column
//               (seg[I][j]); near-threshold pairs go to the candidate list;
//   fill pass : recompute the identical tile, place every edge at
//               row_ptr[row] + seg[block][row] + its rank in the tile's
//               row (or column) bitmask, writing both (i, j) and (j, i).
// A pair is evaluated once (diagonal tiles keep il < jl), so the CSR is
// symmetric by construction.
#include "common.cuh"

namespace bna {

constexpr int SB = 128;  // tile edge
constexpr int SK = 16;   // K (time) chunk per stage
constexpr int SPAD = 4;

__device__ __forceinline__ int popc_before(const uint32_t* m, int pos) {
  int c = 0;
  const int w = pos >> 5;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (k < w) c += __popc(m[k]);
  const uint32_t part = m[w] & ((1u << (pos & 31)) - 1u);
  return c + __popc(part);
}

// PASS 0 = count, 1 = fill, 2 = dump approximate values of one tile.
template <int PASS>
__global__ __launch_bounds__(256, 2) void corr_simt_kernel(CorrArgs a, int nt, int dumpI,
                                                           int dumpJ, float* dump) {
  __shared__ __align__(16) float As[2][SK][SB + SPAD];
  __shared__ __align__(16) float Bs[2][SK][SB + SPAD];
  __shared__ uint32_t rowmask[SB][4];
  __shared__ uint32_t colmask[SB][4];
  __shared__ int rowbase[SB];
  __shared__ int colbase[SB];

  int I, J;
  if (PASS == 2) {
    I = dumpI;
    J = dumpJ;
  } else {
    tile_coords(blockIdx.x, nt, I, J);
  }
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const float* Ag = a.z + (size_t)I * SB * a.ldz;
  const float* Bg = a.z + (size_t)J * SB * a.ldz;
  const int lr = tid >> 2, lk = (tid & 3) * 4;

  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

  const int kt = (a.T + SK - 1) / SK;
  float4 ra0, ra1, rb0, rb1;
  auto gload = [&](int k0) {
    ra0 = __ldg(reinterpret_cast<const float4*>(Ag + (size_t)lr * a.ldz + k0 + lk));
    ra1 = __ldg(reinterpret_cast<const float4*>(Ag + (size_t)(lr + 64) * a.ldz + k0 + lk));
    rb0 = __ldg(reinterpret_cast<const float4*>(Bg + (size_t)lr * a.ldz + k0 + lk));
    rb1 = __ldg(reinterpret_cast<const float4*>(Bg + (size_t)(lr + 64) * a.ldz + k0 + lk));
  };
  auto sstore = [&](int b) {
    As[b][lk + 0][lr] = ra0.x; As[b][lk + 1][lr] = ra0.y;
    As[b][lk + 2][lr] = ra0.z; As[b][lk + 3][lr] = ra0.w;
    As[b][lk + 0][lr + 64] = ra1.x; As[b][lk + 1][lr + 64] = ra1.y;
    As[b][lk + 2][lr + 64] = ra1.z; As[b][lk + 3][lr + 64] = ra1.w;
    Bs[b][lk + 0][lr] = rb0.x; Bs[b][lk + 1][lr] = rb0.y;
    Bs[b][lk + 2][lr] = rb0.z; Bs[b][lk + 3][lr] = rb0.w;
    Bs[b][lk + 0][lr + 64] = rb1.x; Bs[b][lk + 1][lr + 64] = rb1.y;
    Bs[b][lk + 2][lr + 64] = rb1.z; Bs[b][lk + 3][lr + 64] = rb1.w;
  };

  gload(0);
  sstore(0);
  __syncthreads();
  for (int kk = 0; kk < kt; ++kk) {
    const int b = kk & 1;
    if (kk + 1 < kt) gload((kk + 1) * SK);
#pragma unroll
    for (int k = 0; k < SK; ++k) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[b][k][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[b][k][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[b][k][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[b][k][64 + tx * 4]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    if (kk + 1 < kt) sstore(b ^ 1);
    __syncthreads();
  }

  if (PASS == 2) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int il = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
        const int jl = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
        dump[il * SB + jl] = acc[i][j];
      }
    return;
  }

  // ---- fused threshold epilogue ----
  if (tid < SB) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      rowmask[tid][k] = 0u;
      colmask[tid][k] = 0u;
    }
  }
  __syncthreads();
  const bool diag = (I == J);
  const int i0 = I * SB, j0 = J * SB;
  uint32_t badr = 0, badc = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int il = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
    const int jl = (i < 4) ? tx * 4 + i : 64 + tx * 4 + (i - 4);
    badr |= (uint32_t)a.bad[i0 + il] << i;
    badc |= (uint32_t)a.bad[j0 + jl] << i;
  }
  const float zero_is_edge = edge_exact(0.0f, a.th) ? 1.f : 0.f;
  unsigned long long emask = 0ull;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int il = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int jl = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
      const int gi = i0 + il, gj = j0 + jl;
      if (gj >= a.n || (diag && jl <= il)) continue;
      float r = acc[i][j];
      int c;
      if (((badr >> i) | (badc >> j)) & 1u) {
        r = 0.f;
        c = zero_is_edge != 0.f ? CLS_EDGE : CLS_NO;
      } else {
        c = classify(r, a.th);
      }
      if (c == CLS_BAND) {
        if (PASS == 0) {
          push_candidate(a, gi, gj);
          continue;
        }
        bool e;
        hash_lookup(a, pair_key(gi, gj), r, e);
        c = e ? CLS_EDGE : CLS_NO;
      }
      if (c == CLS_EDGE) {
        emask |= 1ull << (i * 8 + j);
        acc[i][j] = r;
        atomicOr(&rowmask[il][jl >> 5], 1u << (jl & 31));
        atomicOr(&colmask[jl][il >> 5], 1u << (il & 31));
      }
    }
  }
  __syncthreads();

  if (PASS == 0) {
    if (tid < SB) {
      const int rc = __popc(rowmask[tid][0]) + __popc(rowmask[tid][1]) +
                     __popc(rowmask[tid][2]) + __popc(rowmask[tid][3]);
      const int cc = __popc(colmask[tid][0]) + __popc(colmask[tid][1]) +
                     __popc(colmask[tid][2]) + __popc(colmask[tid][3]);
      if (diag) {
        a.seg[(size_t)I * a.n_pad + i0 + tid] = rc + cc;
      } else {
        a.seg[(size_t)J * a.n_pad + i0 + tid] = rc;
        a.seg[(size_t)I * a.n_pad + j0 + tid] = cc;
      }
    }
    return;
  }

  // fill pass
  if (tid < SB) {
    const int gi = i0 + tid, gj = j0 + tid;
    int cdiag = 0;
    if (diag)
      cdiag = __popc(colmask[tid][0]) + __popc(colmask[tid][1]) + __popc(colmask[tid][2]) +
              __popc(colmask[tid][3]);
    rowbase[tid] = (gi < a.n) ? a.row_ptr[gi] + a.seg[(size_t)J * a.n_pad + gi] + cdiag : 0;
    colbase[tid] = (gj < a.n) ? a.row_ptr[gj] + a.seg[(size_t)I * a.n_pad + gj] : 0;
  }
  __syncthreads();
  while (emask) {
    const int bit = __ffsll((long long)emask) - 1;
    emask &= emask - 1;
    const int i = bit >> 3, j = bit & 7;
    const int il = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
    const int jl = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
    float v = 0.f;
    // runtime index into the register tile: resolved through a small switch
#pragma unroll
    for (int ii = 0; ii < 8; ++ii)
#pragma unroll
      for (int jj = 0; jj < 8; ++jj)
        if (ii == i && jj == j) v = acc[ii][jj];
    const int pr = rowbase[il] + popc_before(rowmask[il], jl);
    const int pc = colbase[jl] + popc_before(colmask[jl], il);
    put_edge(a, pr, j0 + jl, v);
    put_edge(a, pc, i0 + il, v);
  }
}

cudaError_t launch_corr_simt(const CorrArgs& a, int pass, cudaStream_t stream) {
  const int nt = a.nb;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  if (tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  if (pass == 0)
    corr_simt_kernel<0><<<(unsigned)tiles, 256, 0, stream>>>(a, nt, 0, 0, nullptr);
  else
    corr_simt_kernel<1><<<(unsigned)tiles, 256, 0, stream>>>(a, nt, 0, 0, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_corr_simt_dump(const CorrArgs& a, int I, int J, float* out,
                                  cudaStream_t stream) {
  corr_simt_kernel<2><<<1, 256, 0, stream>>>(a, a.nb, I, J, out);
  return cudaGetLastError();
}

}  // namespace bna
