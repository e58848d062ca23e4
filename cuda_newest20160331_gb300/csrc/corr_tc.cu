// Split-BF16 correlation -> CSR on the tcgen05 tensor cores.
//
// Reference: the same tile loop as the plain form (CorMat_gpu's cublasSgemm
// tiles, W/CorMat/CUCorMat/CUCorMat/CorMat.cu:87-154, then post_block /
// FormFullGraph / FormCSRGraph, CorMat.cpp:824-918), here as one persistent,
// warp-specialised kernel per pass:
//
//   warp 0      TMA producer: per K block of 64, loads A = Z[I-block] (128 rows)
//               and B = Z[2 column blocks] (256 rows) as BF16 hi and lo parts,
//               128-byte swizzled, into a 2-stage shared-memory ring;
//   warp 1      MMA issuer (one thread): per K16 step three tcgen05.mma
//               (hi*hi, hi*lo, lo*hi) accumulate a 128 x 256 FP32 tile in TMEM;
//               two TMEM accumulators (512 columns) so the epilogue of tile t
//               overlaps the MMAs of tile t+1;
//   warps 2..9  epilogue: each 128 x 128 half-tile is read from TMEM by four
//               warps (one per 32-lane quadrant, thread = row), 32 columns at
//               a time (the next load in flight), and thresholded in registers:
//               one compare per value marks the "interesting" entries (edge or
//               near-threshold candidate); a warp prefix scan gives their slots
//               in the sub-tile's compact edge list (warp-private bump
//               allocator), candidates only flagged; row counts from register
//               bitmasks, column counts from a 32 x 32 bit transpose across the
//               warp; the rare candidates also go to the candidate list
//               (warp-private chunks).  The fill pass (csr_fill.cu) places the
//               listed edges; the GEMM runs once.
//
// Every wait is bounded (4 s of wall time); on expiry the kernel raises
// ERR_TIMEOUT, drains its own copies and MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <vector>

#include "common.cuh"
#include "tc_ptx.cuh"

namespace bna {

constexpr int TC_BM = 128;
constexpr int TC_BN = 256;
// Operand forms.  Every K block is one 128-byte swizzled row per matrix row
// (64 BF16 or 32 FP32 values) and one MMA K step covers 32 bytes of it.
//   FORM_BF16X3: A hi, A lo, B hi, B lo per stage (96 KB), 2 stages, three
//                kind::f16 MMAs (hi*hi, hi*lo, lo*hi) per K16 step;
//   FORM_TF32:   A, B per stage (48 KB) from the FP32 z-scores, 4 stages, one
//                kind::tf32 MMA per K8 step.
constexpr int FORM_BF16X3 = 0, FORM_TF32 = 1;
constexpr int TC_RING_BYTES = 192 * 1024;
constexpr int TC_A_BYTES = TC_BM * 128;  // 16 KB: 128 rows x 128 bytes
constexpr int TC_B_BYTES = TC_BN * 128;  // 32 KB
template <int FORM>
struct Form {
  static constexpr int kParts = FORM == FORM_BF16X3 ? 2 : 1;           // hi/lo or one
  static constexpr int kStageBytes = kParts * (TC_A_BYTES + TC_B_BYTES);
  static constexpr int kStages = TC_RING_BYTES / kStageBytes;
  static constexpr int kElemsPerBlock = FORM == FORM_BF16X3 ? 64 : 32;   // per 128-byte row
  static constexpr int kElemsPerStep = kElemsPerBlock / 4;              // per MMA K step
};
constexpr int TC_MAX_STAGES = 4;
constexpr int TC_THREADS = 320;
constexpr int TC_EPI_THREADS = 256;
constexpr uint32_t TC_TMEM_COLS = 512;
constexpr uint64_t kWaitNs = 4000000000ull;

// Tiles are claimed one at a time from a counter in global memory (a CTA
// that starts late, its SM held by another stream's kernel, finds the tiles
// already taken instead of holding the launch open); the TMA warp claims and
// passes each tile's index to the MMA and epilogue warps through this queue.
constexpr int kTileQ = 8;
constexpr int kTileQReaders = 1 + TC_EPI_THREADS / 32;  // the MMA thread, each epilogue warp

struct TcSmem {
  uint64_t full[TC_MAX_STAGES], empty[TC_MAX_STAGES], tfull[2], tempty[2], done, hbar[2];
  uint64_t qfull[kTileQ], qempty[kTileQ];
  volatile int tq[kTileQ];  // claimed tile indices, -1 after the last
  uint32_t tmem_base;
  volatile uint32_t abort;
  uint32_t colmask[2][128][4];
  unsigned int hist[kHistBins + 1];  // density histogram pass
  CorrArgs eargs[8];                 // each epilogue warp's current subject's arguments
};

// One subject of a multi-subject count pass: its operand maps (TMA reads them
// from global memory), arguments, NaN-block flags and K steps.
struct TcSubj {  // 64-byte aligned through its CUtensorMap members
  CUtensorMap hi, lo;
  CorrArgs a;
  const uint8_t* blockbad;
  int nksteps;
};

constexpr size_t TC_SMEM_BYTES = 1024 + (size_t)TC_RING_BYTES + sizeof(TcSmem);
static_assert(TC_SMEM_BYTES <= 232448, "shared memory per CTA");

struct TcArgs {
  CorrArgs a;
  // pass 4 (multi-subject average, post_block with accumulation,
  // W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:847-883): packed[idx(i, j)] += r~
  // or its Fisher z; pairs with |r~| >= unc_lim get their uncertain bit
  float* packed;
  uint32_t* uncertain;
  int fisher;
  float unc_lim;
  // multi-subject count pass: tiles4 = (I, J-pair, subject), subj the table
  const int4* tiles4;
  const TcSubj* subj;
  const int2* tiles;        // (I, Jp): rows of block I x columns of blocks 2Jp, 2Jp+1
  int ntiles;
  // [0]: next tile to claim, [1]: CTAs finished; zero at launch, reset to
  // zero by the launch's last CTA
  unsigned int* sched;
  int nksteps;              // MMA K steps = ceil(T / elements per step)
  const uint8_t* blockbad;  // [nb]: block holds a voxel with NaN z
  float* dump;              // dump pass: 128 x 128 values of half `dump_half`
  int dump_half;
};

// v[k] for a run-time k through a 5-level select tree (no local-memory copy).
__device__ __forceinline__ uint32_t pick32(const uint32_t (&v)[32], int k) {
  uint32_t t[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) t[i] = (k & 16) ? v[i + 16] : v[i];
#pragma unroll
  for (int i = 0; i < 8; ++i) t[i] = (k & 8) ? t[i + 8] : t[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) t[i] = (k & 4) ? t[i + 4] : t[i];
#pragma unroll
  for (int i = 0; i < 2; ++i) t[i] = (k & 2) ? t[i + 2] : t[i];
  return (k & 1) ? t[1] : t[0];
}

// 32 x 32 bit transpose across a warp: lane L holds row L on entry and
// column L on exit (bit b of the result = bit L of lane b's input).
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
  const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int j = 16 >> s;
    const uint32_t m = masks[s];
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & ~m) | ((y & ~m) >> j)) : ((x & m) | ((y & m) << j));
  }
  return x;
}

// Bounded barrier of the 128 threads of one half (mbarrier based, so a lost
// peer cannot hang the CTA).
__device__ __forceinline__ bool half_sync(TcSmem& S, int h, uint32_t& phase) {
  const uint32_t bar = ptx::smem_u32(&S.hbar[h]);
  ptx::mbar_arrive(bar);
  const bool ok = ptx::mbar_wait(bar, phase, kWaitNs);
  phase ^= 1u;
  return ok;
}

// tm_hi / tm_lo: BF16 hi and lo parts (FORM_BF16X3); tm_hi: FP32 z (FORM_TF32).
// DENS (count pass of the density rule): candidates are listed per 32-column
// chunk together with their approximate value (a.cand_apx), which the device
// selection of the k-th largest value needs.
// MULTI: the tiles of several subjects in one persistent launch (count pass).
template <int PASS, bool ABS, int FORM, bool DENS, bool MULTI = false>
__global__ void __launch_bounds__(TC_THREADS, 1)
    corr_tc_kernel(const __grid_constant__ CUtensorMap tm_hi,
                   const __grid_constant__ CUtensorMap tm_lo, const TcArgs p) {
  using F = Form<FORM>;
  constexpr int TC_STAGES = F::kStages;
  constexpr int TC_STAGE_BYTES = F::kStageBytes;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  TcSmem& S = *reinterpret_cast<TcSmem*>(smem + (size_t)TC_RING_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const CorrArgs& a = p.a;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      ptx::mbar_init(ptx::smem_u32(&S.full[s]), 1);
      ptx::mbar_init(ptx::smem_u32(&S.empty[s]), 1);
    }
    for (int s = 0; s < 2; ++s) {
      ptx::mbar_init(ptx::smem_u32(&S.tfull[s]), 1);
      ptx::mbar_init(ptx::smem_u32(&S.tempty[s]), TC_EPI_THREADS);
      ptx::mbar_init(ptx::smem_u32(&S.hbar[s]), 128);
    }
    ptx::mbar_init(ptx::smem_u32(&S.done), 1);
    for (int s = 0; s < kTileQ; ++s) {
      ptx::mbar_init(ptx::smem_u32(&S.qfull[s]), 1);
      ptx::mbar_init(ptx::smem_u32(&S.qempty[s]), kTileQReaders);
    }
    S.abort = 0;
    ptx::fence_mbar_init();
  }
  if (PASS == 3)
    for (int b = threadIdx.x; b <= kHistBins; b += blockDim.x) S.hist[b] = 0u;
  if (warp == 1) {
    ptx::tmem_alloc(ptx::smem_u32(&S.tmem_base), TC_TMEM_COLS);
    ptx::tmem_relinquish();
  }
  if (!MULTI && warp == 0 && lane == 0) {
    ptx::prefetch_tensormap(&tm_hi);
    if (FORM == FORM_BF16X3) ptx::prefetch_tensormap(&tm_lo);
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = S.tmem_base;
  const int nkb = (p.nksteps + 3) / 4;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      uint32_t f = 0;
      int last_round[TC_STAGES];
      for (int s = 0; s < TC_STAGES; ++s) last_round[s] = -1;
      int m = 0;
      // the m-th claimed tile's index into the queue (bounded wait for its slot)
      auto publish = [&](int t) {
        const int qs = m % kTileQ;
        const uint32_t qr = (uint32_t)(m / kTileQ);
        if (!ptx::mbar_wait(ptx::smem_u32(&S.qempty[qs]), (qr & 1u) ^ 1u, kWaitNs)) return false;
        S.tq[qs] = t;
        ptx::mbar_arrive(ptx::smem_u32(&S.qfull[qs]));
        ++m;
        return true;
      };
      // the next tile is claimed while this one's copies are issued
      int t = (int)atomicAdd(p.sched, 1u);
      for (int t_next; t < p.ntiles && !S.abort; t = t_next) {
        if (!publish(t)) {
          atomicOr(a.err, ERR_TIMEOUT);
          S.abort = 1;
          break;
        }
        t_next = (int)atomicAdd(p.sched, 1u);
        int2 tile;
        const CUtensorMap* mh = &tm_hi;
        const CUtensorMap* ml = &tm_lo;
        int nkb_t = nkb;
        if (MULTI) {
          const int4 t4 = p.tiles4[t];
          tile = make_int2(t4.x, t4.y);
          mh = &p.subj[t4.z].hi;
          ml = &p.subj[t4.z].lo;
          nkb_t = (p.subj[t4.z].nksteps + 3) / 4;
        } else {
          tile = p.tiles[t];
        }
        for (int kb = 0; kb < nkb_t; ++kb, ++f) {
          const int s = f % TC_STAGES;
          const uint32_t round = f / TC_STAGES;
          const uint32_t empty = ptx::smem_u32(&S.empty[s]);
          if (!ptx::mbar_wait(empty, (round & 1u) ^ 1u, kWaitNs)) {
            atomicOr(a.err, ERR_TIMEOUT);
            S.abort = 1;
            break;
          }
          const uint32_t full = ptx::smem_u32(&S.full[s]);
          const uint32_t base = ptx::smem_u32(smem + (size_t)s * TC_STAGE_BYTES);
          ptx::mbar_arrive_expect_tx(full, TC_STAGE_BYTES);
          const int k0 = kb * F::kElemsPerBlock;
          const int ra = tile.x * TC_BM, rb = tile.y * TC_BN;
          // stage layout: A parts, then B parts (B = two 128-row boxes each)
          ptx::tma_load_2d(base, mh, full, k0, ra);
          if (FORM == FORM_BF16X3) ptx::tma_load_2d(base + TC_A_BYTES, ml, full, k0, ra);
          const uint32_t bb = base + F::kParts * TC_A_BYTES;
          ptx::tma_load_2d(bb, mh, full, k0, rb);
          ptx::tma_load_2d(bb + TC_B_BYTES / 2, mh, full, k0, rb + 128);
          if (FORM == FORM_BF16X3) {
            ptx::tma_load_2d(bb + TC_B_BYTES, ml, full, k0, rb);
            ptx::tma_load_2d(bb + TC_B_BYTES + TC_B_BYTES / 2, ml, full, k0, rb + 128);
          }
          last_round[s] = (int)round;
        }
      }
      publish(-1);  // the end (on a timeout the readers' own bounded waits end)
      // drain: every issued copy must have landed before the CTA exits
      for (int s = 0; s < TC_STAGES; ++s)
        if (last_round[s] >= 0)
          ptx::mbar_wait(ptx::smem_u32(&S.full[s]), (uint32_t)last_round[s] & 1u, kWaitNs);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      // BF16 x BF16 (kind::f16, format 1) or TF32 x TF32 (kind::tf32, format 2)
      constexpr uint32_t idesc = FORM == FORM_BF16X3 ? ptx::make_idesc(1, 1, TC_BM, TC_BN)
                                                     : ptx::make_idesc(2, 2, TC_BM, TC_BN);
      uint32_t f = 0;
      bool ok = true;
      for (int m = 0; !S.abort; ++m) {
        const int qs = m % kTileQ;
        if (!ptx::mbar_wait(ptx::smem_u32(&S.qfull[qs]), (uint32_t)(m / kTileQ) & 1u, kWaitNs)) {
          ok = false;
          break;
        }
        const int t = S.tq[qs];
        ptx::mbar_arrive(ptx::smem_u32(&S.qempty[qs]));
        if (t < 0) break;
        const int acc = m & 1;
        const uint32_t ar = (uint32_t)(m >> 1);
        if (!ptx::mbar_wait(ptx::smem_u32(&S.tempty[acc]), (ar & 1u) ^ 1u, kWaitNs)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(acc * TC_BN);
        const int nkb_t = MULTI ? (p.subj[p.tiles4[t].z].nksteps + 3) / 4 : nkb;
        const int nks_t = MULTI ? p.subj[p.tiles4[t].z].nksteps : p.nksteps;
        for (int kb = 0; kb < nkb_t; ++kb, ++f) {
          const int s = f % TC_STAGES;
          const uint32_t round = f / TC_STAGES;
          if (!ptx::mbar_wait(ptx::smem_u32(&S.full[s]), round & 1u, kWaitNs)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t base = ptx::smem_u32(smem + (size_t)s * TC_STAGE_BYTES);
          const int steps = min(4, nks_t - kb * 4);
          if (FORM == FORM_BF16X3) {
            for (int kk = 0; kk < steps; ++kk) {
              const uint64_t ahi = ptx::sw128_desc(base + kk * 32);
              const uint64_t alo = ptx::sw128_desc(base + TC_A_BYTES + kk * 32);
              const uint64_t bhi = ptx::sw128_desc(base + 2 * TC_A_BYTES + kk * 32);
              const uint64_t blo = ptx::sw128_desc(base + 2 * TC_A_BYTES + TC_B_BYTES + kk * 32);
              ptx::mma_bf16(d, ahi, bhi, idesc, (kb | kk) != 0);
              ptx::mma_bf16(d, ahi, blo, idesc, 1);
              ptx::mma_bf16(d, alo, bhi, idesc, 1);
            }
          } else {
            for (int kk = 0; kk < steps; ++kk) {
              const uint64_t ad = ptx::sw128_desc(base + kk * 32);
              const uint64_t bd = ptx::sw128_desc(base + TC_A_BYTES + kk * 32);
              ptx::mma_tf32(d, ad, bd, idesc, (kb | kk) != 0);
            }
          }
          ptx::mma_commit(ptx::smem_u32(&S.empty[s]));
        }
        if (!ok) break;
        ptx::mma_commit(ptx::smem_u32(&S.tfull[acc]));
      }
      if (!ok) {
        atomicOr(a.err, ERR_TIMEOUT);
        S.abort = 1;
      }
      // no MMA may still be running when TMEM is freed
      ptx::mma_commit(ptx::smem_u32(&S.done));
      ptx::mbar_wait(ptx::smem_u32(&S.done), 0, kWaitNs);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;         // TMEM lane quadrant
    const int h = (warp - 2) >> 2;  // which 128-column half of the tile
    const int il = q * 32 + lane;   // row within the tile
    // this warp's copy of the current subject's arguments (shared memory)
    CorrArgs& a = S.eargs[warp - 2];
    float tau = 0, delta = 0, lim = 0, lo_thr = 0;
    bool simple = false, zero_int = false;
    uint32_t hphase = 0;
    // this warp's current edge-list chunk [wcur, wend) and candidate chunk
    // [ccur, cend), carried from launch to launch of a pass in a.wstate
    const int wid = (int)blockIdx.x * 8 + (warp - 2);
    long long wcur = 0, wend = 0, ccur = 0, cend = 0;
    bool wok = true;
    unsigned long long n_def = 0, n_cand = 0;  // this lane's definite edges and candidates
    int cur_s = -1;
    // the fields the per-value path reads, kept in registers
    int s_n = 0, s_npad = 0, s_nb = 0;
    const uint8_t* s_bad = nullptr;
    uint2* s_elist = nullptr;
    int32_t* s_seg = nullptr;
    longlong2* s_etab = nullptr;
    // switch to subject s: arguments, thresholds and chunk state
    auto enter = [&](int s) {
      if (lane == 0) a = MULTI ? p.subj[s].a : p.a;
      __syncwarp();
      cur_s = s;
      s_n = a.n;
      s_npad = a.n_pad;
      s_nb = a.nb;
      s_bad = a.bad;
      s_elist = a.elist;
      s_seg = a.seg;
      s_etab = a.etab;
      tau = a.th.tau;
      delta = a.th.delta;
      lim = 1.0f - a.th.delta;
      lo_thr = tau - delta;
      // Near +1 is always covered by x >= tau - delta when tau < 1 - delta; near
      // -1 can be an edge only through post_block's 0 for tau <= 0 in the signed
      // rules (|r| rules cover -1 like +1).
      simple = (tau < lim) && (ABS || lo_thr > 0.0f);
      // a pair with a NaN voxel has the exact value 0 (post_block); in the 2mm
      // tools' rule it stays NaN and is never an edge
      zero_int = a.th.mode != BNA_THR_R_EPS && ((0.0f >= lo_thr) || (0.0f >= lim));
      if (PASS == 0) {
        long long x = 0;
        if (lane < 4) x = a.wstate[wid * 4 + lane];
        wcur = __shfl_sync(0xffffffffu, x, 0);
        wend = __shfl_sync(0xffffffffu, x, 1);
        ccur = __shfl_sync(0xffffffffu, x, 2);
        cend = __shfl_sync(0xffffffffu, x, 3);
      }
      wok = wend <= a.ecap;
    };
    // leave the current subject: its chunks stay open for the next launch or
    // visit (seal_candidates_kernel closes the candidate chunks after the
    // pass); the warp's counts go to its statistics
    auto leave = [&]() {
      if (PASS == 0 && cur_s >= 0) {
        if (lane < 4)
          a.wstate[wid * 4 + lane] = lane == 0 ? wcur : lane == 1 ? wend : lane == 2 ? ccur : cend;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          n_def += __shfl_xor_sync(0xffffffffu, n_def, o);
          n_cand += __shfl_xor_sync(0xffffffffu, n_cand, o);
        }
        if (lane == 0 && n_def) atomicAdd(&a.stats[2], n_def);
        if (lane == 0 && n_cand) atomicAdd(&a.stats[3], n_cand);
        n_def = n_cand = 0;
      }
      __syncwarp();
    };
    auto tile_at = [&](int t, int2& tl, int& ts) {
      if (MULTI) {
        const int4 t4 = p.tiles4[t];
        tl = make_int2(t4.x, t4.y);
        ts = t4.z;
      } else {
        tl = p.tiles[t];
        ts = 0;
      }
    };
    auto flags_of = [&](int2 tl, int ts, uint8_t& fi, uint8_t& fj) {
      const uint8_t* bbad = MULTI ? p.subj[ts].blockbad : p.blockbad;
      const int nbs = MULTI ? p.subj[ts].a.nb : p.a.nb;
      fi = bbad[tl.x];
      const int jj = 2 * tl.y + h;
      fj = jj < nbs ? bbad[jj] : 0;
    };
    for (int m = 0;; ++m) {
      if (S.abort) break;
      const int qs = m % kTileQ;
      if (!ptx::mbar_wait(ptx::smem_u32(&S.qfull[qs]), (uint32_t)(m / kTileQ) & 1u, kWaitNs)) {
        atomicOr(p.a.err, ERR_TIMEOUT);  // (this warp's `a` is set by its first tile)
        S.abort = 1;
        break;
      }
      const int t = S.tq[qs];
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(ptx::smem_u32(&S.qempty[qs]));
      if (t < 0) break;
      int2 tile;
      int tile_s;
      uint8_t nbi, nbj;
      tile_at(t, tile, tile_s);
      flags_of(tile, tile_s, nbi, nbj);
      const bool bad_i = nbi != 0, bad_j = nbj != 0;
      if (tile_s != cur_s) {  // the first tile, or another subject's
        leave();
        enter(tile_s);
      }
      const int I = tile.x, J = 2 * tile.y + h;
      const int acc = m & 1;
      const uint32_t ar = (uint32_t)(m >> 1);
      const bool active = (PASS == 2) ? (J < s_nb) : ((J >= I) && (J < s_nb));
      const bool listing = (PASS == 0);
      const int gi = I * 128 + il;
      long long start = 0;
      if (listing && active) {
        // room for this warp's worst case (32 rows x 128 columns) in one chunk
        if (wend - wcur < 32 * 128) {
          long long base = 0;
          if (lane == 0) base = (long long)atomicAdd(a.epool, (unsigned long long)a.echunk);
          base = __shfl_sync(0xffffffffu, base, 0);
          wcur = base;
          wend = base + a.echunk;
          wok = wend <= a.ecap;
          if (!wok && lane == 0) atomicOr(a.err, ERR_ELIST);
        }
        start = wcur;
      }
      if (!half_sync(S, h, hphase)) {  // previous tile's shared-memory readers are done
        atomicOr(a.err, ERR_TIMEOUT);
        S.abort = 1;
        break;
      }
      if (!ptx::mbar_wait(ptx::smem_u32(&S.tfull[acc]), ar & 1u, kWaitNs)) {
        atomicOr(a.err, ERR_TIMEOUT);
        S.abort = 1;
        break;
      }
      ptx::tc_fence_after();
      const uint32_t taddr =
          tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * TC_BN + h * 128);
      const bool diag = (I == J);
      const bool slow = active && (bad_i || bad_j);
      const bool rowbad = slow && s_bad[gi];
      int rowcount = 0;
      uint32_t cmk4[4] = {0u, 0u, 0u, 0u};
      if (active) {
        uint32_t vb[2][32];
        ptx::tmem_ld32_async(taddr, vb[0]);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint32_t(&v)[32] = vb[c & 1];
          ptx::tmem_wait32(v);
          if (c + 1 < 4) ptx::tmem_ld32_async(taddr + (c + 1) * 32, vb[(c + 1) & 1]);
          if (PASS == 2) {
            if (h == p.dump_half)
              for (int k = 0; k < 32; ++k) p.dump[il * 128 + c * 32 + k] = __uint_as_float(v[k]);
            continue;
          }
          const int jb = J * 128 + c * 32;
          uint32_t valid = (jb + 32 <= s_n) ? 0xffffffffu
                                            : (jb >= s_n ? 0u : ((1u << (s_n - jb)) - 1u));
          if (diag) {
            const int lo = il - c * 32 + 1;  // first column index k with jl > il
            valid &= (lo <= 0) ? 0xffffffffu : (lo >= 32 ? 0u : (0xffffffffu << lo));
          }
          if (PASS == 4) {
            uint32_t badm4 = 0;
            if (slow)
              for (int k = 0; k < 32; ++k)
                if (rowbad || (jb + k < s_npad && s_bad[jb + k])) badm4 |= 1u << k;
            if (gi < s_n) {
              // packed upper-triangle index of (gi, j): gi (2n - gi - 1) / 2 + j - gi - 1
              const long long rowbase = (long long)gi * (2LL * s_n - gi - 1) / 2 - gi - 1;
#pragma unroll
              for (int k = 0; k < 32; ++k) {
                if (!((valid >> k) & 1u)) continue;
                const bool badk = (badm4 >> k) & 1u;
                const float r = badk ? 0.0f : __uint_as_float(v[k]);
                const long long idx = rowbase + jb + k;
                if (!badk && !(fabsf(r) < p.unc_lim))
                  atomicOr(&p.uncertain[idx >> 5], 1u << (idx & 31));
                float add = 0.0f;
                if (r >= -1.0f && r <= 1.0f) add = p.fisher ? fisher_z(r) : r;
                p.packed[idx] = __fadd_rn(p.packed[idx], add);
              }
            }
            continue;
          }
          if (PASS == 3) {
            // density histogram of the approximate values (exact 0 for NaN voxels)
            uint32_t badm3 = 0;
            if (slow)
              for (int k = 0; k < 32; ++k)
                if (rowbad || (jb + k < s_npad && s_bad[jb + k])) badm3 |= 1u << k;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
              if ((valid >> k) & 1u) {
                const bool badk = (badm3 >> k) & 1u;
                const float r = badk ? 0.0f : __uint_as_float(v[k]);
                atomicAdd(&S.hist[(!badk && !(fabsf(r) < lim)) ? kHistBins : hist_bin(r)], 1u);
              }
            }
            continue;
          }
          // "interesting" = an edge or a candidate: x >= tau - delta, or
          // |r| >= 1 - delta; 8 partial masks so no long dependency chain forms
          uint32_t pm[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
          if (simple) {
#pragma unroll
            for (int k = 0; k < 32; ++k) {
              const float r = __uint_as_float(v[k]);
              pm[k & 7] |= ((ABS ? fabsf(r) : r) >= lo_thr) ? (1u << k) : 0u;
            }
          } else {
#pragma unroll
            for (int k = 0; k < 32; ++k) {
              const float r = __uint_as_float(v[k]);
              pm[k & 7] |= (((ABS ? fabsf(r) : r) >= lo_thr) | (fabsf(r) >= lim)) ? (1u << k) : 0u;
            }
          }
          uint32_t it = ((pm[0] | pm[1]) | (pm[2] | pm[3])) | ((pm[4] | pm[5]) | (pm[6] | pm[7]));
          uint32_t badm = 0;
          if (slow) {
            for (int k = 0; k < 32; ++k)
              if (rowbad || (jb + k < s_npad && s_bad[jb + k])) badm |= 1u << k;
            it = (it & ~badm) | (zero_int ? badm : 0u);
          }
          it &= valid;
          // slots in the warp's edge-list chunk: warp prefix scan of the counts
          const int ne = __popc(it);
          int incl = ne;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          const int total = __shfl_sync(0xffffffffu, incl, 31);
          uint2* dst = s_elist + wcur + (incl - ne);
          // classify this lane's few interesting entries; candidates are only
          // flagged here (collected for the exact recompute after the pass)
          uint32_t eb = 0;
          uint32_t w2 = it;
          while (w2) {
            const int k = __ffs(w2) - 1;
            w2 &= w2 - 1;
            const bool badk = (badm >> k) & 1u;
            uint32_t val = badk ? 0u : pick32(v, k);  // NaN voxel: exact r = 0
            const float r = __uint_as_float(val);
            const float x = ABS ? fabsf(r) : r;
            uint32_t cf = 0;
            if (!((x - tau > delta) && (fabsf(r) < lim))) {
              cf = 1u;  // candidate: collected for the exact recompute after the pass
              val = 0u;
            }
            eb |= (cf ^ 1u) << k;
            if (wok) *dst++ = make_uint2(elist_key(il, c * 32 + k, cf), val);
          }
          rowcount += __popc(eb);
          n_def += __popc(eb);
          S.colmask[h][c * 32 + lane][q] = transpose32(eb, lane);
          wcur += total;
          if (!DENS) {
            cmk4[c] = it & ~eb;  // candidates of this chunk (listed after the tile)
          } else if (__any_sync(0xffffffffu, (it & ~eb) != 0u)) {
            // candidates with their approximate values, listed now (v[] is live)
            const uint32_t cmk = it & ~eb;
            const int nc = __popc(cmk);
            int cinc = nc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const int y = __shfl_up_sync(0xffffffffu, cinc, o);
              if (lane >= o) cinc += y;
            }
            const int ctot = __shfl_sync(0xffffffffu, cinc, 31);
            if (ccur + ctot > cend) {
              for (long long sl = ccur + lane; sl < cend && sl < a.cand_cap; sl += 32)
                a.cand[sl] = make_uint2(kCandNone, kCandNone);
              const long long need = (ctot + kCandChunk - 1) / kCandChunk * kCandChunk;
              unsigned long long cb = 0;
              if (lane == 0) cb = atomicAdd(a.cand_count, (unsigned long long)need);
              ccur = (long long)__shfl_sync(0xffffffffu, cb, 0);
              cend = ccur + need;
            }
            long long slot = ccur + (cinc - nc);
            uint32_t w3 = cmk;
            while (w3) {
              const int k = __ffs(w3) - 1;
              w3 &= w3 - 1;
              const bool badk = (badm >> k) & 1u;
              const float r = badk ? 0.0f : __uint_as_float(pick32(v, k));
              if (slot < a.cand_cap) {
                a.cand[slot] = make_uint2((unsigned)gi, (unsigned)(J * 128 + c * 32 + k));
                a.cand_apx[slot] = r;
              } else {
                atomicOr(a.err, ERR_BAND_OVERFLOW);
              }
              ++slot;
            }
            ccur += ctot;
            n_cand += nc;
          }
        }
      }
      // the accumulator has been read: hand it back to the MMA warp
      ptx::tc_fence_before();
      ptx::mbar_arrive(ptx::smem_u32(&S.tempty[acc]));
      if (PASS == 2 || PASS == 3 || PASS == 4) continue;
      // candidates (rare): warp prefix scan into the warp's candidate chunk
      if (!DENS && active &&
          __any_sync(0xffffffffu, (cmk4[0] | cmk4[1] | cmk4[2] | cmk4[3]) != 0u)) {
        const int nc = __popc(cmk4[0]) + __popc(cmk4[1]) + __popc(cmk4[2]) + __popc(cmk4[3]);
        int cinc = nc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, cinc, o);
          if (lane >= o) cinc += y;
        }
        const int ctot = __shfl_sync(0xffffffffu, cinc, 31);
        if (ccur + ctot > cend) {
          // seal the rest of the chunk, take enough new chunks for this batch
          for (long long sl = ccur + lane; sl < cend && sl < a.cand_cap; sl += 32)
            a.cand[sl] = make_uint2(kCandNone, kCandNone);
          const long long need = (ctot + kCandChunk - 1) / kCandChunk * kCandChunk;
          unsigned long long cb = 0;
          if (lane == 0) cb = atomicAdd(a.cand_count, (unsigned long long)need);
          ccur = (long long)__shfl_sync(0xffffffffu, cb, 0);
          cend = ccur + need;
        }
        long long slot = ccur + (cinc - nc);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint32_t w3 = cmk4[c];
          while (w3) {
            const int k = __ffs(w3) - 1;
            w3 &= w3 - 1;
            if (slot < a.cand_cap)
              a.cand[slot] = make_uint2((unsigned)gi, (unsigned)(J * 128 + c * 32 + k));
            else
              atomicOr(a.err, ERR_BAND_OVERFLOW);
            ++slot;
          }
        }
        ccur += ctot;
        n_cand += nc;
      }
      if (active && lane == 0)
        s_etab[subtile_index(I, J, s_nb) * 4 + q] =
            wok ? make_longlong2(start, wcur - start) : make_longlong2(0, 0);
      if (!half_sync(S, h, hphase)) {
        atomicOr(a.err, ERR_TIMEOUT);
        S.abort = 1;
        break;
      }
      if (active) {
        const uint32_t* cm = S.colmask[h][il];
        const int cc = __popc(cm[0]) + __popc(cm[1]) + __popc(cm[2]) + __popc(cm[3]);
        if (diag) {
          s_seg[(size_t)I * s_npad + gi] = rowcount + cc;
        } else {
          s_seg[(size_t)J * s_npad + gi] = rowcount;
          s_seg[(size_t)I * s_npad + J * 128 + il] = cc;
        }
      }
    }
    leave();
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, TC_TMEM_COLS);
  }
  if (PASS == 3)
    for (int b = threadIdx.x; b <= kHistBins; b += blockDim.x)
      if (S.hist[b]) atomicAdd(&a.hist[b], S.hist[b]);
  // every CTA has stopped claiming by now: the last one resets the counters
  if (threadIdx.x == 0 && atomicAdd(p.sched + 1, 1u) == gridDim.x - 1) {
    p.sched[0] = 0;
    p.sched[1] = 0;
  }
}

// After the last launch of a count pass: mark the unused slots of every
// warp's open candidate chunk (warp states are (wcur, wend, ccur, cend)).
__global__ void seal_candidates_kernel(CorrArgs a, int nwarps) {
  const int lane = threadIdx.x & 31;
  for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nwarps;
       w += gridDim.x * (blockDim.x >> 5)) {
    const long long ccur = a.wstate[w * 4 + 2], cend = a.wstate[w * 4 + 3];
    for (long long sl = ccur + lane; sl < cend && sl < a.cand_cap; sl += 32)
      if (sl >= 0) a.cand[sl] = make_uint2(kCandNone, kCandNone);
  }
}

__global__ void block_bad_kernel(const uint8_t* bad, int nb, uint8_t* blockbad) {
  const int b = blockIdx.x;
  const int any = __syncthreads_or(bad[b * 128 + threadIdx.x] != 0);
  if (threadIdx.x == 0 && b < nb) blockbad[b] = any ? 1 : 0;
}

// ---------------------------------------------------------------- host side

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2-D map over [rows][ld] elements (BF16 or FP32) with a 128-byte x 128-row
// box, 128-byte swizzle (the K-major layout the MMA descriptors expect).
bool make_map(CUtensorMap* m, const void* base, int ld, int rows, bool fp32) {
  auto fn = encode_fn();
  if (!fn) return false;
  const int esz = fp32 ? 4 : 2;
  cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * esz};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esz), TC_BM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                  const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

// Tile list (I, Jp) of the upper triangle in 128 x 256 tiles (rows of block
// I, columns of blocks 2Jp and 2Jp+1, Jp >= I/2), in bands of `band` row
// blocks: band b holds rows [b*band, (b+1)*band) and lists them column by
// column (Jp ascending, then I ascending).  The CTAs of a persistent launch
// take consecutive tiles, so at any time they work on a few column pairs of
// one band: every column pair's operands are read from DRAM about once per
// band and the band's row operands stay in L2 (a row-major list sweeps all
// columns at once and re-reads them from DRAM for every row block).
__host__ __device__ inline long long tile_row_offset(int I, int njp) {
  // tiles in rows [0, I): row I' holds njp - floor(I'/2) tiles
  const long long m = I / 2;
  return (long long)I * njp - ((I & 1) ? m * m : m * (m - 1));
}

long long tc_tile_count(int nb) { return tile_row_offset(nb, (nb + 1) / 2); }

// Position of column pair jp's first tile inside band [i0, i1).
__host__ __device__ inline long long band_col_offset(int i0, int i1, int jp) {
  long long off = 0;
  for (int I = i0; I < i1; ++I) off += jp > I / 2 ? jp - I / 2 : 0;
  return off;
}

void tc_tile_list(int nb, int band, std::vector<int2>& out) {
  out.clear();
  const int njp = (nb + 1) / 2;
  if (band < 1) band = 1;
  for (int i0 = 0; i0 < nb; i0 += band) {
    const int i1 = i0 + band < nb ? i0 + band : nb;
    for (int jp = i0 / 2; jp < njp; ++jp)
      for (int I = i0; I < i1 && I / 2 <= jp; ++I) out.push_back(make_int2(I, jp));
  }
}

// The same list built on the device (no host round trip): one thread per
// (band, column pair) writes that column's tiles of the band.
__global__ void tile_list_kernel(int nb, int band, long long total, int2* out) {
  const int njp = (nb + 1) / 2;
  const int nbands = (nb + band - 1) / band;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)nbands * njp) return;
  const int b = (int)(k / njp), jp = (int)(k % njp);
  const int i0 = b * band, i1 = i0 + band < nb ? i0 + band : nb;
  if (jp < i0 / 2) return;
  const long long base = tile_row_offset(i0, njp) + band_col_offset(i0, i1, jp);
  for (int I = i0; I < i1 && I / 2 <= jp; ++I) {
    const long long pos = base + (I - i0);
    if (pos < total) out[pos] = make_int2(I, jp);
  }
}

// Every s-th tile of the list (the density histogram's sample).
__global__ void tile_sample_kernel(const int2* tiles, long long n_smp, int s, int2* out) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_smp) out[k] = tiles[k * s];
}

cudaError_t launch_tile_lists(int nb, int band, int2* tiles, long long n_smp, int s, int2* smp,
                              cudaStream_t st) {
  if (nb <= 0) return cudaSuccess;
  if (band < 1) band = 1;
  const long long work = (long long)((nb + band - 1) / band) * ((nb + 1) / 2);
  tile_list_kernel<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(nb, band, tc_tile_count(nb),
                                                                   tiles);
  if (n_smp > 0)
    tile_sample_kernel<<<(unsigned)((n_smp + 255) / 256), 256, 0, st>>>(tiles, n_smp, s, smp);
  return cudaGetLastError();
}

size_t tc_smem_bytes() { return TC_SMEM_BYTES; }

cudaError_t launch_block_bad(const uint8_t* bad, int nb, uint8_t* blockbad, cudaStream_t st) {
  block_bad_kernel<<<nb, 128, 0, st>>>(bad, nb, blockbad);
  return cudaGetLastError();
}

size_t tc_subj_bytes() { return sizeof(TcSubj); }

// Table entry s (host memory, tc_subj_bytes() per entry) of a multi-subject
// count pass: the subject's operand maps, arguments and NaN-block flags.
bool tc_subj_fill(void* host, int s, const CorrArgs& a, const uint8_t* blockbad, int form) {
  TcSubj* e = static_cast<TcSubj*>(host) + s;
  std::memset(e, 0, sizeof *e);
  if (form == FORM_BF16X3) {
    if (!a.zhi || !a.zlo || a.ldb % 64 != 0) return false;
    if (!make_map(&e->hi, a.zhi, a.ldb, a.n_pad, false) ||
        !make_map(&e->lo, a.zlo, a.ldb, a.n_pad, false))
      return false;
    e->nksteps = (a.T + Form<FORM_BF16X3>::kElemsPerStep - 1) / Form<FORM_BF16X3>::kElemsPerStep;
  } else {
    if (!a.z || a.ldz % 32 != 0) return false;
    if (!make_map(&e->hi, a.z, a.ldz, a.n_pad, true)) return false;
    e->lo = e->hi;
    e->nksteps = (a.T + Form<FORM_TF32>::kElemsPerStep - 1) / Form<FORM_TF32>::kElemsPerStep;
  }
  e->a = a;
  e->blockbad = blockbad;
  return true;
}

// Count pass over the tiles of several subjects in one persistent launch:
// tiles4 = (I, J-pair, subject); subj_dev = the device copy of the table;
// batch.err receives timeouts of the producer and MMA warps.
// The multi-subject kernel of a form, with its shared-memory limit set (a
// call outside any stream capture; the launcher sets it too).
static void (*tc_multi_kernel(int form, bool dens, bool absm))(CUtensorMap, CUtensorMap, TcArgs) {
  if (form == FORM_BF16X3)
    return dens ? corr_tc_kernel<0, false, FORM_BF16X3, true, true>
           : absm ? corr_tc_kernel<0, true, FORM_BF16X3, false, true>
                  : corr_tc_kernel<0, false, FORM_BF16X3, false, true>;
  return dens ? corr_tc_kernel<0, false, FORM_TF32, true, true>
         : absm ? corr_tc_kernel<0, true, FORM_TF32, false, true>
                : corr_tc_kernel<0, false, FORM_TF32, false, true>;
}

cudaError_t prepare_corr_tc_multi(int form, bool dens, bool absm) {
  if (dens && absm) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(tc_multi_kernel(form, dens, absm),
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM_BYTES);
}

cudaError_t launch_corr_tc_multi(const CorrArgs& batch, const void* subj_dev, const int4* tiles4,
                                 int ntiles, int form, bool dens, bool absm, int grid,
                                 unsigned int* sched, cudaStream_t st) {
  if ((dens && absm) || !sched) return cudaErrorInvalidValue;
  TcArgs p{};
  p.a = batch;
  p.sched = sched;
  p.tiles4 = tiles4;
  p.subj = static_cast<const TcSubj*>(subj_dev);
  p.ntiles = ntiles;
  p.nksteps = 0;
  const int g = grid < ntiles ? grid : ntiles;
  if (g <= 0) return cudaSuccess;
  void (*kern)(CUtensorMap, CUtensorMap, TcArgs) = tc_multi_kernel(form, dens, absm);
  CUtensorMap dummy;
  std::memset(&dummy, 0, sizeof dummy);
  kern<<<g, TC_THREADS, TC_SMEM_BYTES, st>>>(dummy, dummy, p);
  return cudaGetLastError();
}

cudaError_t launch_seal_candidates(const CorrArgs& a, int nwarps, cudaStream_t st) {
  seal_candidates_kernel<<<(nwarps + 7) / 8, 256, 0, st>>>(a, nwarps);
  return cudaGetLastError();
}

// pass 0 count (+ edge lists), 2 dump (tiles must then hold the one tile to dump),
// 3 density histogram; form FORM_BF16X3 or FORM_TF32
cudaError_t launch_corr_tc(const CorrArgs& a, int pass, int form, const int2* tiles, int ntiles,
                           const uint8_t* blockbad, float* dump, int dump_half, int grid,
                           unsigned int* sched, cudaStream_t st, const AvgPass* avg) {
  if (!sched) return cudaErrorInvalidValue;
  CUtensorMap mh, ml;
  if (form == FORM_BF16X3) {
    if (!a.zhi || !a.zlo || a.ldb % 64 != 0) return cudaErrorInvalidValue;
    if (!make_map(&mh, a.zhi, a.ldb, a.n_pad, false) ||
        !make_map(&ml, a.zlo, a.ldb, a.n_pad, false))
      return cudaErrorInvalidValue;
  } else {
    if (!a.z || a.ldz % 32 != 0) return cudaErrorInvalidValue;
    if (!make_map(&mh, a.z, a.ldz, a.n_pad, true)) return cudaErrorInvalidValue;
    ml = mh;
  }
  TcArgs p{};
  p.a = a;
  p.sched = sched;
  p.tiles = tiles;
  p.ntiles = ntiles;
  const int per_step = form == FORM_BF16X3 ? Form<FORM_BF16X3>::kElemsPerStep
                                           : Form<FORM_TF32>::kElemsPerStep;
  p.nksteps = (a.T + per_step - 1) / per_step;
  p.blockbad = blockbad;
  p.dump = dump;
  p.dump_half = dump_half;
  p.packed = avg ? avg->packed : nullptr;
  p.uncertain = avg ? avg->uncertain : nullptr;
  p.fisher = avg ? avg->fisher : 0;
  p.unc_lim = avg ? avg->unc_lim : 1.0f;
  if (pass == 4 && !avg) return cudaErrorInvalidValue;
  const int g = grid < ntiles ? grid : ntiles;
  if (g <= 0) return cudaSuccess;
  const bool absm = (a.th.mode == BNA_THR_ABS_GT || a.th.mode == BNA_THR_ABS_GE);
  const bool dens = pass == 0 && a.cand_apx != nullptr;
  if (dens && absm) return cudaErrorInvalidValue;  // the density rule is signed
  void (*kern)(CUtensorMap, CUtensorMap, TcArgs);
  if (form == FORM_BF16X3)
    kern = pass == 0   ? (dens   ? corr_tc_kernel<0, false, FORM_BF16X3, true>
                          : absm ? corr_tc_kernel<0, true, FORM_BF16X3, false>
                                 : corr_tc_kernel<0, false, FORM_BF16X3, false>)
           : pass == 3 ? corr_tc_kernel<3, false, FORM_BF16X3, false>
           : pass == 4 ? corr_tc_kernel<4, false, FORM_BF16X3, false>
                       : corr_tc_kernel<2, false, FORM_BF16X3, false>;
  else
    kern = pass == 0   ? (dens   ? corr_tc_kernel<0, false, FORM_TF32, true>
                          : absm ? corr_tc_kernel<0, true, FORM_TF32, false>
                                 : corr_tc_kernel<0, false, FORM_TF32, false>)
           : pass == 3 ? corr_tc_kernel<3, false, FORM_TF32, false>
           : pass == 4 ? corr_tc_kernel<4, false, FORM_TF32, false>
                       : corr_tc_kernel<2, false, FORM_TF32, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)TC_SMEM_BYTES);
  if (e != cudaSuccess) return e;
  kern<<<g, TC_THREADS, TC_SMEM_BYTES, st>>>(mh, ml, p);
  return cudaGetLastError();
}

}  // namespace bna
