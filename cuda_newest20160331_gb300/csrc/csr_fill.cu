// Fill pass: place every listed edge into the CSR.
//
// Reference: FormCSRGraph (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:889-918) —
// rows in order, columns ascending, both (i, j) and (j, i) of each pair,
// V[e] = r of the pair.  Here the count pass has left, per 128 x 128
// sub-tile (I, J), I <= J, a compact list of its edges (value) and of its
// near-threshold candidates (resolved by the recompute pass into a hash).
// One warp handles one sub-tile for the 128 rows of one row block: the
// direct entries of sub-tile (I, J), J >= I, or the transposed entries of
// sub-tile (J, I), J <= I, for the rows of block I:
//   1. mark the entries in per-row bitmasks (smem);
//   2. bases: row i of block I starts its block-J segment at
//      row_ptr[i] + seg[J][i] (+ the count of its transposed entries on a
//      diagonal sub-tile, whose columns come first);
//   3. each entry goes to base + (number of set bits before it) in its row.
// Each sub-tile is read twice (once per direction) so that each CTA writes
// contiguous stretches of the CSR rows.
// Sub-tiles with more than kFillDenseE edge-list entries (the dense blocks of
// networked data) are listed first (csr_dense_list_kernel, which also checks
// every sub-tile's ranges) and placed by csr_fill_dense_kernel, one block per
// sub-tile, before the row-block pass, which skips them: the entries' values are staged in a 128 x 128 shared-
// memory matrix, and each row run and each column run of the sub-tile is then
// written by one warp as consecutive CSR positions (coalesced stores instead
// of one scattered 4-byte store per column-direction entry).
// Positions are range-checked (ERR_RANGE) so an inconsistent count cannot
// write outside the CSR.
#include "common.cuh"

namespace bna {

constexpr int kFillWarps = 8;
constexpr long long kFillDenseE = 1024;  // entries above which a sub-tile takes the dense path
constexpr int kFillDenseLoads = 8;       // edge-list loads in flight per thread (dense path)

// Asynchronous global -> shared copies (no registers held while in flight).
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// put_edge for positions in 32 bits (a CSR's row offsets are int32)
__device__ __forceinline__ void put_edge32(const CorrArgs& a, int pos, int col, float v) {
  if ((unsigned long long)(unsigned)pos >= (unsigned long long)a.nnz) {
    atomicOr(a.err, ERR_RANGE);
    return;
  }
  a.col_idx[pos] = col;
  if (a.weighted) a.val[pos] = v;
}

// popc_before4 of a 16-byte-aligned row of four mask words, read in one load
__device__ __forceinline__ int popc_before4v(const uint32_t* m, int pos) {
  const uint4 v = *reinterpret_cast<const uint4*>(m);
  const int w = pos >> 5;
  const uint32_t low = (1u << (pos & 31)) - 1u;
  return __popc(w == 0 ? v.x & low : v.x) + (w >= 1 ? __popc(w == 1 ? v.y & low : v.y) : 0) +
         (w >= 2 ? __popc(w == 2 ? v.z & low : v.z) : 0) + (w == 3 ? __popc(v.w & low) : 0);
}

__device__ __forceinline__ int popc_before4(const uint32_t* m, int pos) {
  const int w = pos >> 5;
  int c = __popc(m[w] & ((1u << (pos & 31)) - 1u));
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (k < w) c += __popc(m[k]);
  return c;
}

// Row-block order: CTA (I, part) handles the rows of 128-row block I and the
// column blocks of one contiguous range `part`, its warps taking J = j0 + w,
// j0 + w + 8, ... in turn.  Sub-tile (I, J), J > I, gives the rows of I their
// entries (direct); sub-tile (J, I), J < I, gives them its column entries
// (transposed); the diagonal sub-tile both.  Each CSR row is thus written by
// `parts` CTAs, each filling one contiguous stretch of it segment after
// segment while it runs, so partial sectors are completed in L2 instead of
// being read back and written piecemeal.  A lane keeps its first kFillKeep
// entries, candidates resolved, in registers for the placing pass.
// Sub-tiles above kFillDenseE entries are queued (once) for
// csr_fill_dense_kernel.  The block's row starts are read once into shared
// memory, and each warp's loads run ahead of its work by asynchronous copies
// into shared memory: while it places a sub-tile's entries, the next
// sub-tile's segment offsets and first kFillStage entries and the ranges of
// the one after that are in flight (the entries' load latency was the
// kernel's main stall).
constexpr int kFillKeep = 8;
constexpr int kFillStage = 128;  // entries staged per warp ahead of use

__global__ __launch_bounds__(kFillWarps * 32, 4) void csr_fill_rows_kernel(CorrArgs a, int I0,
                                                                           int parts) {
  __shared__ __align__(16) uint32_t rmask[kFillWarps][128][4];  // direct: row il's columns jl
  __shared__ __align__(16) uint32_t tmask[kFillWarps][128][4];  // transposed: row jl's columns il
  __shared__ int dbase[kFillWarps][128];
  __shared__ int tbase[kFillWarps][128];
  __shared__ int rp_s[128];                        // row_ptr of the block's rows (0 past the end)
  __shared__ int nsg[kFillWarps][128];             // staged: rows' block-J segment offsets
  __shared__ longlong2 netab[kFillWarps][2][4];    // staged: quadrant ranges (two sub-tiles)
  __shared__ uint2 ent[kFillWarps][kFillStage];    // staged: first entries (raw)
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Ir = blockIdx.x / parts, part = blockIdx.x - Ir * parts;
  const int I = I0 + Ir;
  const int per = (a.nb + parts - 1) / parts;
  const int j0 = part * per, j1 = min(a.nb, j0 + per);
  if (threadIdx.x < 128) {
    const int gi = I * 128 + (int)threadIdx.x;
    rp_s[threadIdx.x] = gi < a.n ? a.row_ptr[gi] : 0;
  }
  __syncthreads();
  uint32_t(*rm)[4] = rmask[w];
  uint32_t(*tm)[4] = tmask[w];
  // a sub-tile's four quadrant ranges (lanes 0-3)
  auto fetch_ranges = [&](int J, int slot) {
    const long long st = subtile_index(min(I, J), max(I, J), a.nb);
    if (lane < 4) cp_async16(&netab[w][slot][lane], a.etab + st * 4 + lane);
  };
  // its rows' segment offsets (rows past the last real one read the padding,
  // never used) and, when the fill places it here, its first entries; its
  // ranges are in netab[w][slot]
  auto fetch_rest = [&](int J, int slot) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      cp_async4(&nsg[w][lane + 32 * k], a.seg + (size_t)J * a.n_pad + I * 128 + lane + 32 * k);
    long long s[4], c[4];
    bool inside = true;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const longlong2 r = netab[w][slot][q];
      s[q] = r.x;
      c[q] = r.y;
      inside &= c[q] >= 0 && s[q] >= 0 && s[q] + c[q] <= a.ecap;
    }
    const long long E = c[0] + c[1] + c[2] + c[3];
    if (!inside || E > kFillDenseE) return;
    const long long p1 = c[0], p2 = p1 + c[1], p3 = p2 + c[2];
#pragma unroll
    for (int k = 0; k < kFillStage / 32; ++k) {
      const long long e = lane + 32 * k;
      if (e < E) {
        const long long at = e < p1 ? s[0] + e : e < p2 ? s[1] + (e - p1)
                             : e < p3 ? s[2] + (e - p2) : s[3] + (e - p3);
        cp_async8(&ent[w][e], a.elist + at);
      }
    }
  };
  int v = 0;  // this warp's sub-tile count (range slot v & 1)
  if (j0 + w < j1) {
    fetch_ranges(j0 + w, 0);
    cp_async_commit();
    cp_async_wait_all();
    __syncwarp();
    fetch_rest(j0 + w, 0);
    if (j0 + w + kFillWarps < j1) fetch_ranges(j0 + w + kFillWarps, 1);
    cp_async_commit();
  }
  for (int J = j0 + w; J < j1; J += kFillWarps, ++v) {
    const int slot = v & 1;
    const int lo = min(I, J), hi = max(I, J);
    cp_async_wait_all();
    __syncwarp();
    long long s0 = 0, c0 = 0;
    if (lane < 4) {
      s0 = netab[w][slot][lane].x;
      c0 = netab[w][slot][lane].y;
    }
    // rows lane + 32k: start of their block-J segment (the transposed
    // entries' base; the previous sub-tile's placing is over)
#pragma unroll
    for (int k = 0; k < 4; ++k) tbase[w][lane + 32 * k] = rp_s[lane + 32 * k] + nsg[w][lane + 32 * k];
    // entry e of quadrant q is elist[b[q] + e] for p[q] <= e < p[q + 1]
    long long b[4], E = 0;
    int p1 = 0, p2 = 0, p3 = 0;  // a sub-tile placed here has at most kFillDenseE entries
    bool inside = true;  // ranges written while the pool overflowed are not read
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long st = __shfl_sync(0xffffffffu, s0, q);
      const long long ct = __shfl_sync(0xffffffffu, c0, q);
      inside &= ct >= 0 && st >= 0 && st + ct <= a.ecap;
      b[q] = st - E;
      E += ct;
      if (q == 0) p1 = (int)E;
      if (q == 1) p2 = (int)E;
      if (q == 2) p3 = (int)E;
    }
    const bool use = inside && E != 0 && E <= kFillDenseE;  // else flagged / the dense pass's
    const int Ei = use ? (int)E : 0;
    auto load = [&](int e) {
      return a.elist[e + (e < p1 ? b[0] : e < p2 ? b[1] : e < p3 ? b[2] : b[3])];
    };
    // candidate bit resolved: bit 15 set = not an edge, .y = the value to store
    auto resolve = [&](uint2 en) {
      if ((en.x >> 14) & 1u) {
        float val = 0.0f;
        bool edge = false;
        hash_lookup(a, pair_key(lo * 128 + (en.x & 127), hi * 128 + ((en.x >> 7) & 127)), val,
                    edge);
        en.y = __float_as_uint(val);
        if (!edge) en.x |= 1u << 15;
      }
      return en;
    };
    const int kmax = min((Ei + 31) / 32, kFillKeep);
    uint2 keep[kFillKeep];
#pragma unroll
    for (int k = 0; k < kFillKeep; ++k) {
      const int e = lane + 32 * k;
      keep[k] = make_uint2(1u << 15, 0u);
      if (k < kmax && e < Ei) keep[k] = k < kFillStage / 32 ? ent[w][e] : load(e);
    }
    __syncwarp();  // the staged data read by every lane before the next copies land
    if (J + kFillWarps < j1) {
      fetch_rest(J + kFillWarps, slot ^ 1);
      if (J + 2 * kFillWarps < j1) fetch_ranges(J + 2 * kFillWarps, slot);
    }
    cp_async_commit();
    if (!use) continue;
#pragma unroll
    for (int k = 0; k < kFillKeep; ++k)
      if (k < kmax) keep[k] = resolve(keep[k]);
    const bool diag = I == J, trans = J < I;
    // the masks this sub-tile uses: direct (rows of I), transposed (rows of
    // J as columns of I), both on the diagonal
    const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
    if (!trans)
#pragma unroll
      for (int k = 0; k < 4; ++k) reinterpret_cast<uint4*>(rm)[lane + 32 * k] = zero4;
    if (trans || diag)
#pragma unroll
      for (int k = 0; k < 4; ++k) reinterpret_cast<uint4*>(tm)[lane + 32 * k] = zero4;
    __syncwarp();
    // 1. masks
    auto mark = [&](uint2 en) {
      if ((en.x >> 15) & 1u) return;
      const int il = en.x & 127, jl = (en.x >> 7) & 127;
      if (!trans) atomicOr(&rm[il][jl >> 5], 1u << (jl & 31));
      if (trans || diag) atomicOr(&tm[jl][il >> 5], 1u << (il & 31));
    };
#pragma unroll
    for (int k = 0; k < kFillKeep; ++k)
      if (k < kmax) mark(keep[k]);
    for (int e = lane + 32 * kFillKeep; e < Ei; e += 32) mark(resolve(load(e)));
    __syncwarp();
    // 2. segment bases of the block's rows for column block J (on the
    // diagonal the transposed entries, columns < the row, come first)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int r = lane + 32 * k;
      if (diag) {
        const uint4 c = *reinterpret_cast<const uint4*>(tm[r]);
        dbase[w][r] = tbase[w][r] + __popc(c.x) + __popc(c.y) + __popc(c.z) + __popc(c.w);
      } else {
        dbase[w][r] = tbase[w][r];
      }
    }
    __syncwarp();
    // 3. place this block's entries: direct (row il) and transposed (row jl)
    auto place = [&](uint2 en) {
      if ((en.x >> 15) & 1u) return;
      const int il = en.x & 127, jl = (en.x >> 7) & 127;
      const float val = __uint_as_float(en.y);
      if (!trans) put_edge32(a, dbase[w][il] + popc_before4v(rm[il], jl), hi * 128 + jl, val);
      if (trans || diag) put_edge32(a, tbase[w][jl] + popc_before4v(tm[jl], il), lo * 128 + il, val);
    };
#pragma unroll
    for (int k = 0; k < kFillKeep; ++k)
      if (k < kmax) place(keep[k]);
    for (int e = lane + 32 * kFillKeep; e < Ei; e += 32) place(resolve(load(e)));
    __syncwarp();
  }
  cp_async_wait_all();  // nothing in flight into shared memory at exit
}

// The dense sub-tiles' list (and the check of every sub-tile's ranges),
// one thread per sub-tile.
__global__ __launch_bounds__(256) void csr_dense_list_kernel(CorrArgs a, long long nst,
                                                             int* dense_list,
                                                             unsigned int* dense_count) {
  const long long st = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (st >= nst) return;
  long long E = 0;
  bool inside = true;  // ranges written while the pool overflowed are not read
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const longlong2 e = a.etab[st * 4 + q];
    inside &= e.y >= 0 && e.x >= 0 && e.x + e.y <= a.ecap;
    E += e.y;
  }
  if (!inside)
    atomicOr(a.err, ERR_ELIST);
  else if (E > kFillDenseE)
    dense_list[atomicAdd(dense_count, 1u)] = (int)st;
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
    // 1. bitmasks and values (ranges were checked by csr_dense_list_kernel)
    const long long p1 = S.cnt[0], p2 = p1 + S.cnt[1], p3 = p2 + S.cnt[2], E = p3 + S.cnt[3];
    const long long s0 = S.start[0], s1 = S.start[1] - p1, s2 = S.start[2] - p2,
                    s3 = S.start[3] - p3;  // entry e of quadrant q is elist[s_q + e]
    // kFillDenseLoads independent loads per thread in flight before any is used
    for (long long e0 = tid; e0 < E; e0 += 256 * kFillDenseLoads) {
      uint2 en[kFillDenseLoads];
#pragma unroll
      for (int u = 0; u < kFillDenseLoads; ++u) {
        const long long e = e0 + 256 * u;
        en[u] = make_uint2(0u, 0u);
        if (e < E) en[u] = a.elist[(e < p1 ? s0 : e < p2 ? s1 : e < p3 ? s2 : s3) + e];
      }
#pragma unroll
      for (int u = 0; u < kFillDenseLoads; ++u) {
        if (e0 + 256 * u >= E) break;
        const int il = en[u].x & 127, jl = (en[u].x >> 7) & 127;
        float v = __uint_as_float(en[u].y);
        bool edge = true;
        if ((en[u].x >> 14) & 1u) hash_lookup(a, pair_key(I * 128 + il, J * 128 + jl), v, edge);
        if (edge) {
          S.val[il][jl] = v;
          atomicOr(&S.rm[il][jl >> 5], 1u << (jl & 31));
          atomicOr(&S.cm[jl][il >> 5], 1u << (il & 31));
        }
      }
    }
    __syncthreads();
    // 2. segment bases (as in csr_fill_rows_kernel)
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

cudaError_t launch_csr_fill_dense(const CorrArgs& a, int sms, int* dense_list,
                                  unsigned int* dense_count, cudaStream_t stream) {
  if (a.nb <= 0) return cudaSuccess;
  const long long nst = (long long)a.nb * (a.nb + 1) / 2;
  cudaError_t e = cudaMemsetAsync(dense_count, 0, sizeof(unsigned int), stream);
  if (e != cudaSuccess) return e;
  csr_dense_list_kernel<<<(unsigned)((nst + 255) / 256), 256, 0, stream>>>(a, nst, dense_list,
                                                                         dense_count);
  e = cudaFuncSetAttribute(csr_fill_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sizeof(DenseSmem));
  if (e != cudaSuccess) return e;
  csr_fill_dense_kernel<<<sms * 3, 256, sizeof(DenseSmem), stream>>>(a, dense_list, dense_count);
  return cudaGetLastError();
}

cudaError_t launch_csr_fill_rows(const CorrArgs& a, int sms, int I0, int I1,
                                 cudaStream_t stream) {
  if (I1 <= I0) return cudaSuccess;
  const int rows = I1 - I0;
  // split the column blocks so that about 8 CTAs per SM take part
  int parts = (sms * 8 + rows - 1) / rows;
  if (parts > (a.nb + 7) / 8) parts = (a.nb + 7) / 8;
  if (parts < 1) parts = 1;
  csr_fill_rows_kernel<<<rows * parts, kFillWarps * 32, 0, stream>>>(a, I0, parts);
  return cudaGetLastError();
}

cudaError_t launch_csr_fill(const CorrArgs& a, int sms, int* dense_list, unsigned int* dense_count,
                            cudaStream_t stream) {
  cudaError_t e = launch_csr_fill_dense(a, sms, dense_list, dense_count, stream);
  if (e != cudaSuccess) return e;
  return launch_csr_fill_rows(a, sms, 0, a.nb, stream);
}

}  // namespace bna
