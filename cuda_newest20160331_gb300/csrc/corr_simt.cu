// Plain FP32 correlation -> CSR on CUDA cores (the "plain form").
//
// Reference: the tile loop of CorMat_gpu (W/CorMat/CUCorMat/CUCorMat/CorMat.cu:87-154,
// cublasSgemm at :94) followed by post_block / FormFullGraph / FormCSRGraph
// (CorMat.cpp:824-918).  Here each CTA computes one 128 x 128 tile (I, J),
// I <= J, of Z Z^T in FP32 and thresholds it in registers; the N x N matrix
// never exists.
//
// The tile epilogue (count pass) counts edges per row (seg[J][i]) and per
// column (seg[I][j]), sends near-threshold pairs to the candidate list, and
// appends the tile's edges with their values to its edge list (one pool
// allocation per tile, slots by a block prefix scan).  The fill pass
// (csr_fill.cu) places every listed edge at row_ptr[row] + seg[block][row] +
// its rank in the tile's row (or column) bitmask, writing (i, j) and (j, i).
// A pair is evaluated once (diagonal tiles keep il < jl), so the CSR is
// symmetric by construction.
#include "common.cuh"

namespace bna {

constexpr int SB = 128;  // tile edge
constexpr int SK = 16;   // K (time) chunk per stage
constexpr int SPAD = 4;

// PASS 0 = count (+ edge list), 2 = dump approximate values of one tile,
// 3 = density histogram.  PACKED: the tile's values come from the averaged
// packed matrix (multi-subject average) instead of the GEMM.
template <int PASS, bool PACKED = false>
__global__ __launch_bounds__(256, 2) void corr_simt_kernel(CorrArgs a, int nt, int dumpI,
                                                           int dumpJ, float* dump) {
  __shared__ __align__(16) float As[2][SK][SB + SPAD];
  __shared__ __align__(16) float Bs[2][SK][SB + SPAD];
  __shared__ uint32_t rowmask[SB][4];
  __shared__ uint32_t colmask[SB][4];
  __shared__ int wsum[8];
  __shared__ long long tbase;

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

  if (PACKED) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int gi = I * SB + ((i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4));
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int gj = J * SB + ((j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4));
        acc[i][j] = (gi < gj && gj < a.n) ? a.avg_packed[packed_index(gi, gj, a.n)] : 0.f;
      }
    }
  }
  const int kt = PACKED ? 0 : (a.T + SK - 1) / SK;
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

  if (!PACKED) {
    gload(0);
    sstore(0);
  }
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
  if (PASS == 3) {
    // density histogram of the approximate values in shared memory (the
    // operand tiles are free now), merged into the global one
    unsigned int* h = reinterpret_cast<unsigned int*>(&As[0][0][0]);
    for (int b = tid; b <= kHistBins; b += 256) h[b] = 0u;
    __syncthreads();
    const bool diag = (I == J);
    const float lim = 1.0f - a.th.delta;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int il = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
      const bool rb = a.bad[I * SB + il] != 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int jl = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
        const int gj = J * SB + jl;
        if (gj >= a.n || (diag && jl <= il)) continue;
        const bool badk = rb || a.bad[gj];
        const float r = badk ? 0.0f : acc[i][j];
        atomicAdd(&h[(!badk && !(fabsf(r) < lim)) ? kHistBins : hist_bin(r)], 1u);
      }
    }
    __syncthreads();
    for (int b = tid; b <= kHistBins; b += 256)
      if (h[b]) atomicAdd(&a.hist[b], h[b]);
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
  unsigned long long emask = 0ull, cmask = 0ull;  // edges, near-threshold candidates
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int il = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int jl = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
      const int gi = i0 + il, gj = j0 + jl;
      if (gj >= a.n || (diag && jl <= il)) continue;
      int c;
      if (((badr >> i) | (badc >> j)) & 1u) {
        acc[i][j] = 0.f;  // NaN voxel: the exact value is 0 (post_block)
        const float x = 0.0f - a.th.tau;
        c = x > a.th.delta ? CLS_EDGE : (x < -a.th.delta ? CLS_NO : CLS_BAND);
        if (a.th.mode == BNA_THR_R_EPS) c = CLS_NO;  // NaN is never an edge there
      } else if (PACKED && ((a.avg_unc[packed_index(gi, gj, a.n) >> 5] >>
                              (packed_index(gi, gj, a.n) & 31)) & 1u)) {
        c = CLS_BAND;  // some subject's value may be clamped by post_block
      } else {
        c = classify(acc[i][j], a.th);
      }
      if (c == CLS_BAND) {
        cmask |= 1ull << (i * 8 + j);  // flagged; collected after the pass
      } else if (c == CLS_EDGE) {
        emask |= 1ull << (i * 8 + j);
        atomicOr(&rowmask[il][jl >> 5], 1u << (jl & 31));
        atomicOr(&colmask[jl][il >> 5], 1u << (il & 31));
      }
    }
  }
  // edge list of the tile: block prefix scan of the per-thread entry counts,
  // one pool allocation per tile
  const unsigned long long ent = emask | cmask;
  const int ne = __popcll(ent);
  const int lane = tid & 31, warp = tid >> 5;
  int incl = ne;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int w = 0; w < 8; ++w) {
      const int c = wsum[w];
      wsum[w] = run;
      run += c;
    }
    const unsigned long long base = run ? atomicAdd(a.epool, (unsigned long long)run) : 0ull;
    tbase = (long long)base;
    const bool fits = !run || (long long)(base + run) <= a.ecap;
    if (!fits) atomicOr(a.err, ERR_ELIST);
    const long long st = subtile_index(I, J, a.nb);
    a.etab[st * 4 + 0] = fits ? make_longlong2((long long)base, run) : make_longlong2(0, 0);
    a.etab[st * 4 + 1] = make_longlong2(0, 0);
    a.etab[st * 4 + 2] = make_longlong2(0, 0);
    a.etab[st * 4 + 3] = make_longlong2(0, 0);
  }
  __syncthreads();
  if (ent && tbase + wsum[warp] + incl <= a.ecap) {
    uint2* dst = a.elist + tbase + wsum[warp] + (incl - ne);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int il = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int jl = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
        const int b = i * 8 + j;
        if ((ent >> b) & 1ull) {
          const uint32_t cf = (uint32_t)((cmask >> b) & 1ull);
          *dst++ = make_uint2(elist_key(il, jl, cf), cf ? 0u : __float_as_uint(acc[i][j]));
        }
      }
    }
  }
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
}

cudaError_t launch_corr_simt(const CorrArgs& a, int pass, cudaStream_t stream) {
  const int nt = a.nb;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  if (tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  if (pass == 0)
    corr_simt_kernel<0><<<(unsigned)tiles, 256, 0, stream>>>(a, nt, 0, 0, nullptr);
  else if (pass == 3)
    corr_simt_kernel<3><<<(unsigned)tiles, 256, 0, stream>>>(a, nt, 0, 0, nullptr);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// Count pass / density histogram over the averaged packed matrix.
cudaError_t launch_corr_packed(const CorrArgs& a, int pass, cudaStream_t stream) {
  const int nt = a.nb;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  if (tiles > 0x7fffffffLL || !a.avg_packed || !a.avg_unc) return cudaErrorInvalidValue;
  if (pass == 0)
    corr_simt_kernel<0, true><<<(unsigned)tiles, 256, 0, stream>>>(a, nt, 0, 0, nullptr);
  else if (pass == 3)
    corr_simt_kernel<3, true><<<(unsigned)tiles, 256, 0, stream>>>(a, nt, 0, 0, nullptr);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_corr_simt_dump(const CorrArgs& a, int I, int J, float* out,
                                  cudaStream_t stream) {
  corr_simt_kernel<2><<<1, 256, 0, stream>>>(a, a.nb, I, J, out);
  return cudaGetLastError();
}

}  // namespace bna
