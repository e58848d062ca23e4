// Shared device-side definitions of the voxel-network builder.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bna.h"

namespace bna {

// Square block of the voxel index space used for the CSR bookkeeping:
// seg[b][i] counts (then offsets) the edges of row i whose column lies in
// block b.  Every correlation tile covers whole 128-blocks.
constexpr int kBlk = 128;

// Error bits raised by kernels into CorrArgs::err (host reads them once per call).
enum : uint32_t {
  ERR_BAND_OVERFLOW = 1u,   // candidate list full
  ERR_HASH_MISS = 2u,       // fill pass met a candidate the recompute pass never stored
  ERR_HASH_FULL = 4u,
  ERR_NNZ_INT32 = 8u,
  ERR_TIES = 16u,           // density: tie bookkeeping inconsistent
  ERR_TIMEOUT = 32u,        // a bounded wait in a tensor-core kernel expired
  ERR_RANGE = 64u,          // a fill-pass position fell outside the CSR (write skipped)
  ERR_ELIST = 128u,         // edge-list pool too small (entries not written; pass is rerun)
};

// Edge-list pool: the tensor-core count pass allocates it in chunks of
// echunk entries per warp (one atomic per chunk; kElistChunkMin for small
// problems, kElistChunk otherwise) and never writes past ecap.  A chunk must
// hold a warp's worst case for one tile (32 rows x 128 columns).
constexpr long long kElistChunk = 16384;
constexpr long long kElistChunkMin = 4096;
// Candidate list: the tensor-core count pass writes its near-threshold pairs
// itself, in warp-private chunks of kCandChunk slots; slots a warp leaves
// unused hold (kCandNone, kCandNone) and are skipped by the consumers.
constexpr long long kCandChunk = 256;
constexpr uint32_t kCandNone = 0xFFFFFFFFu;

// Density mode: histogram of the approximate r over [-1, 1) in kHistBins
// bins (bin = floor((r + 1) * kHistBins / 2)); entry kHistBins counts the
// pairs near +-1 whose clamped value is not known yet.
constexpr int kHistBins = 2048;
__device__ __forceinline__ int hist_bin(float r) {
  int b = (int)floorf((r + 1.0f) * (0.5f * kHistBins));
  return b < 0 ? 0 : (b >= kHistBins ? kHistBins - 1 : b);
}

// Outcome of classifying one approximate correlation.
enum : int { CLS_NO = 0, CLS_EDGE = 1, CLS_BAND = 2 };

struct Threshold {
  int mode;      // bna_thr_mode (density runs as R_GE on tau = r_k plus the tie list)
  float tau;
  float delta;   // band half-width in r units (includes rounding margin)
};

// Fisher transform of the reference, fishertrans (W/CorMat/CUCorMat/CUCorMat/
// CorMat.cpp:36-42), in its float arithmetic: r == 1 is moved to float(1 - 1e-6),
// z = 0.5 log((1 + r) / (1 - r)).
__device__ __forceinline__ float fisher_z(float r) {
  if (r == 1.0f) r = 0.99999899f;  // float(1.0 - 1e-6)
  return 0.5f * logf(__fdiv_rn(__fadd_rn(1.0f, r), __fsub_rn(1.0f, r)));
}

// Its inverse, inv_fishertrans (CorMat.cpp:44-50): r = (e^(2z) - 1) / (e^(2z) + 1).
__device__ __forceinline__ float fisher_r(float z) {
  const float e = expf(__fmul_rn(2.0f, z));
  return __fdiv_rn(__fsub_rn(e, 1.0f), __fadd_rn(e, 1.0f));
}

// Multi-subject average pass (tensor-core pass 4) buffers.
struct AvgPass {
  float* packed;       // [n(n-1)/2] running sums, upper triangle row-major
  uint32_t* uncertain; // one bit per pair
  int fisher;
  float unc_lim;
};

// 1 + 1e-6 as the 2mm tools compare it, (double)r <= 1.0 + 1e-6: the largest
// float not above it is 1 + 8 * 2^-23.
constexpr float kEpsHi = 1.00000095367431640625f;

// Exact decision on the reference's value r (after post_block clamping; the
// raw value in BNA_THR_R_EPS, whose th.tau is the smallest float above
// tau - 1e-6 in double, so r >= th.tau is the tools' r > tau - ep).
__device__ __forceinline__ bool edge_exact(float r, const Threshold& th) {
  switch (th.mode) {
    case BNA_THR_R_GT: return r > th.tau;
    case BNA_THR_R_EPS: return r >= th.tau && r <= kEpsHi;
    case BNA_THR_ABS_GT: return fabsf(r) > th.tau;
    case BNA_THR_ABS_GE: return fabsf(r) >= th.tau;
    default: return r >= th.tau;  // R_GE and DENSITY
  }
}

// post_block (CorMat.cpp:869-884): values outside [-1, 1], and NaN, become 0.
__device__ __forceinline__ float post_block(float r) {
  return (r >= -1.0f && r <= 1.0f) ? r : 0.0f;
}

// Classify an approximate correlation whose error vs the reference value is
// at most th.delta.  A value is decided directly only when the whole
// interval [r - delta, r + delta] lies inside (-1, 1) and on one side of tau.
__device__ __forceinline__ int classify(float r, const Threshold& th) {
  const float a = fabsf(r);
  if (!(a < 1.0f - th.delta)) return CLS_BAND;  // near +-1, or NaN
  const bool absm = (th.mode == BNA_THR_ABS_GT || th.mode == BNA_THR_ABS_GE);
  const float x = absm ? a : r;
  const float d = x - th.tau;
  if (d > th.delta) return CLS_EDGE;
  if (d < -th.delta) return CLS_NO;
  return CLS_BAND;
}

// Pointers and sizes shared by the correlation passes.
struct CorrArgs {
  const float* z;            // voxel-major [n_pad][ldz], FP32 z-scores (exact recompute source)
  const uint16_t* zhi;       // voxel-major [n_pad][ldb] BF16 hi parts (tensor-core forms)
  const uint16_t* zlo;       // BF16 lo parts
  const uint8_t* bad;        // [n_pad] 1 = voxel has a NaN z (every r of it is NaN -> 0)
  int n, n_pad, T, ldz, ldb, nb;
  Threshold th;
  int weighted;
  int32_t* seg;              // [nb][n_pad]
  const int32_t* row_ptr;    // [n+1] (fill pass)
  int32_t* col_idx;          // [nnz]
  float* val;                // [nnz] or null
  long long nnz;             // fill pass: entries of col_idx / val (positions are checked)
  // near-threshold candidates (count pass appends, recompute resolves)
  uint2* cand;               // (i, j) with i < j
  unsigned long long* cand_count;
  long long cand_cap;
  // hash of resolved candidates: key (i<<32|j) -> (value, edge flag)
  unsigned long long* hkeys;
  float* hval;
  uint8_t* hedge;
  unsigned long long hmask;
  // per-tile edge lists written by the count pass, placed by the fill pass:
  // entry = (il | jl << 7 | candidate << 14, value bits); etab[4*st + q] =
  // (first entry, count) of part q of 128 x 128 sub-tile st (upper-triangle index)
  uint2* elist;
  unsigned long long* epool;
  long long ecap;
  long long echunk;  // entries per warp chunk (kElistChunkMin .. kElistChunk)
  long long* wstate; // tensor-core count pass: per epilogue warp (wcur, wend, ccur, cend)
  longlong2* etab;
  // density ties that must not become edges (sorted keys), see FormFullGraph_s
  const unsigned long long* drop_keys;
  int n_drop;
  uint32_t* err;
  unsigned long long* stats;  // [0]=band edges [1]=band within 1e-6 [2]=definite listed edges
  unsigned int* hist;         // density histogram pass: kHistBins + 1 counters
  const float* cand_val;      // density: exact values of the candidates (decide pass)
  float* cand_apx;            // density (tensor-core count pass): r~ of every candidate slot
  // multi-subject average: the averaged values (packed upper triangle) replace
  // the GEMM as the source of the plain count pass; uncertain pairs are
  // candidates
  const float* avg_packed;
  const uint32_t* avg_unc;
};

__host__ __device__ __forceinline__ long long packed_index(int i, int j, int n) {
  return (long long)i * (2LL * n - i - 1) / 2 + (j - i - 1);  // i < j, row-major
}

// Fill-pass store with a range check (an inconsistent count would otherwise
// write outside the CSR).
__device__ __forceinline__ void put_edge(const CorrArgs& a, long long pos, int col, float v) {
  if (pos < 0 || pos >= a.nnz) {
    atomicOr(a.err, ERR_RANGE);
    return;
  }
  a.col_idx[pos] = col;
  if (a.weighted) a.val[pos] = v;
}

__device__ __forceinline__ unsigned long long pair_key(int i, int j) {
  return ((unsigned long long)(uint32_t)i << 32) | (uint32_t)j;
}

__device__ __forceinline__ unsigned long long hash64(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

// Look up a resolved candidate.  Returns false (and flags ERR_HASH_MISS) if absent.
__device__ __forceinline__ bool hash_lookup(const CorrArgs& a, unsigned long long key, float& v,
                                            bool& edge) {
  unsigned long long h = hash64(key) & a.hmask;
  for (unsigned long long probe = 0; probe <= a.hmask; ++probe) {
    const unsigned long long k = a.hkeys[h];
    if (k == key) {
      v = a.hval[h];
      edge = a.hedge[h] != 0;
      return true;
    }
    if (k == ~0ull) break;
    h = (h + 1) & a.hmask;
  }
  atomicOr(a.err, ERR_HASH_MISS);
  v = 0.f;
  edge = false;
  return false;
}

// Append a near-threshold candidate (count pass).
__device__ __forceinline__ void push_candidate(const CorrArgs& a, int i, int j) {
  const unsigned long long slot = atomicAdd(a.cand_count, 1ull);
  if ((long long)slot < a.cand_cap) {
    a.cand[slot] = make_uint2((unsigned)i, (unsigned)j);
  } else {
    atomicOr(a.err, ERR_BAND_OVERFLOW);
  }
}

// Upper-triangular 128-block pair (I, J), I <= J -> its row-major index.
__host__ __device__ __forceinline__ long long subtile_index(int I, int J, int nb) {
  return (long long)I * nb - (long long)I * (I - 1) / 2 + (J - I);
}

__device__ __forceinline__ uint32_t elist_key(int il, int jl, uint32_t cand) {
  return (uint32_t)il | ((uint32_t)jl << 7) | (cand << 14);
}

// Upper-triangular tile index -> (I, J), I <= J, row-major over I.  A float
// square root gives the row to within one; integer steps settle it.
__device__ __forceinline__ void tile_coords(long long t, int nt, int& I, int& J) {
  // rows before I hold I*nt - I*(I-1)/2 tiles
  const float b = 2.0f * (float)nt + 1.0f;
  const float disc = fmaxf(b * b - 8.0f * (float)t, 0.0f);
  int i = (int)((b - sqrtf(disc)) * 0.5f);
  if (i < 0) i = 0;
  if (i > nt - 1) i = nt - 1;
  auto start = [nt](long long r) { return r * nt - r * (r - 1) / 2; };
  while (i > 0 && start(i) > t) --i;
  while (i + 1 < nt && start(i + 1) <= t) ++i;
  I = i;
  J = i + (int)(t - start(i));
}

}  // namespace bna
