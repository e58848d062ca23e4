// Exact density rule on the device: FormFullGraph_s
// (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:705-822) without host round trips.
//
// The reference keeps exactly k undirected edges: tau* = the k-th largest r
// over all pairs (quickselect, :770-771); every larger pair is an edge; of the
// pairs equal to tau*, the first ones in row-major (i < j) order are kept
// (the others are popped off its stack, :797-808).
//
// The count pass ran with a window [A, B] that holds tau* (from a histogram
// pass): pairs with r~ above the window were listed as definite edges
// (n_def), pairs inside as candidates with their approximate value r~
// (|r~ - r| <= delta for every pair).  Here:
//   1. tau~ = the need-th largest r~ among the candidates (need = k - n_def);
//      the order statistics of r~ and r differ by at most delta, so
//      |tau* - tau~| <= delta;
//   2. candidates with r~ > tau~ + 2 delta are surely above tau* (G of them),
//      those below tau~ - 2 delta surely below; only the rest (set E, plus
//      every |r~| >= 1 - delta, where post_block may clamp the exact value to
//      0) get their exact reference value;
//   3. tau* = the (need - G)-th largest exact value in E; A <= tau* <= B is
//      checked (the window may come from a sample);
//   4. the pairs of E equal to tau* are sorted by (i, j); the first
//      k - (pairs above tau*) stay, the rest are dropped;
//   5. every candidate is decided and stored in the hash the fill pass reads.
// The k-th largest is found by a three-digit radix select (11 + 11 + 10 bits
// of an order-preserving integer key of the float).
#include "common.cuh"
#include "exact_r.cuh"

namespace bna {

constexpr int kMaxTies = 4096;

struct DensState {
  long long k;          // undirected edges wanted
  float delta;          // per-pair bound |r~ - r|
  double A, B;          // the count pass window (tau* must lie in it)
  int err;              // DENS_ERR_* (0: selection done)
  long long need;       // k - definite
  uint32_t prefix, mask;
  long long kk;         // rank wanted within the current prefix class
  float tau_apx;        // tau~
  float tau;            // tau*
  long long n_above;    // G
  long long n_exact;    // |E|
  long long n_exact_gt; // E items above tau*
  long long n_ties;
  long long greater;    // pairs above tau*
  int n_drop;
};

enum : int {
  DENS_ERR_WINDOW = 1,  // tau* outside the window (a sampled window missed)
  DENS_ERR_TIES = 2,    // more ties at tau* than the device sort holds
  DENS_ERR_RANK = 3,    // inconsistent ranks
};

__device__ __forceinline__ uint32_t okey(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float okey_inv(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__global__ void dens_init_kernel(DensState* ds, const unsigned long long* stats) {
  ds->need = ds->k - (long long)stats[2];
  ds->err = 0;
  ds->prefix = 0;
  ds->mask = 0;
  ds->n_above = ds->n_exact = ds->n_exact_gt = ds->n_ties = 0;
  ds->n_drop = 0;
  if (ds->need < 1) ds->err = DENS_ERR_WINDOW;
}

// Histogram of one key digit over the selected items whose key matches the
// prefix so far.  which = 0: candidate slots (r~); 1: the E list (exact).
__global__ void dens_hist_kernel(CorrArgs a, DensState* ds, const float* exact, int which,
                                 int shift, int nbits, unsigned int* hist) {
  __shared__ unsigned int h[2048];
  const int nb = 1 << nbits;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) h[b] = 0;
  __syncthreads();
  if (ds->err == 0) {
    const uint32_t prefix = ds->prefix, mask = ds->mask;
    long long n;
    if (which == 0) {
      const long long c = (long long)*a.cand_count;
      n = c < a.cand_cap ? c : a.cand_cap;
    } else {
      n = ds->n_exact;
    }
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
      float v;
      if (which == 0) {
        if (a.cand[i].x == kCandNone) continue;
        v = a.cand_apx[i];
      } else {
        v = exact[i];
      }
      const uint32_t key = okey(v);
      if ((key & mask) == prefix) atomicAdd(&h[(key >> shift) & (uint32_t)(nb - 1)], 1u);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}

// One block: pick the digit value that holds the kk-th largest item.
// first: set kk from the rank wanted; last: store the selected value.
__global__ void dens_pick_kernel(DensState* ds, unsigned int* hist, int which, int shift,
                                 int nbits, int first, int last) {
  __shared__ long long part[1024];
  __shared__ int found;
  const int nb = 1 << nbits;
  const int per = nb / 1024 > 0 ? nb / 1024 : 1;  // bins per thread (1 or 2)
  if (ds->err) return;
  if (first && threadIdx.x == 0) {
    ds->kk = which == 0 ? ds->need : ds->need - ds->n_above;
    ds->prefix = 0;
    ds->mask = 0;
  }
  __syncthreads();
  const long long kk = ds->kk;
  // thread t owns bins [nb - per*(t+1), nb - per*t): descending order
  long long mine = 0;
  const int hi = nb - per * (int)threadIdx.x;
  for (int q = 1; q <= per; ++q)
    if (hi - q >= 0) mine += hist[hi - q];
  part[threadIdx.x] = mine;
  if (threadIdx.x == 0) found = -1;
  __syncthreads();
  // inclusive scan over threads (descending bins)
  for (int o = 1; o < 1024; o <<= 1) {
    const long long y = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += y;
    __syncthreads();
  }
  const long long before = threadIdx.x ? part[threadIdx.x - 1] : 0;
  if (kk >= 1 && before < kk && part[threadIdx.x] >= kk && hi > 0) {
    long long c = before;
    for (int q = 1; q <= per; ++q) {
      const int b = hi - q;
      if (b < 0) break;
      if (c + hist[b] >= kk) {
        ds->kk = kk - c;
        ds->prefix |= (uint32_t)b << shift;
        ds->mask |= (uint32_t)(nb - 1) << shift;
        found = 1;
        break;
      }
      c += hist[b];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (found < 0) {
      ds->err = which == 0 ? DENS_ERR_WINDOW : DENS_ERR_RANK;
    } else if (last) {
      const float v = okey_inv(ds->prefix);
      if (which == 0) ds->tau_apx = v;
      else ds->tau = v;
      ds->prefix = 0;  // the next selection's first histogram starts unfiltered
      ds->mask = 0;
    }
  }
  for (int b = threadIdx.x; b < nb; b += blockDim.x) hist[b] = 0;  // ready for the next digit
}

// Classify the candidates against tau~: 1 surely above, 3 surely below,
// 2 exact value needed (listed in eidx).
__global__ void dens_classify_kernel(CorrArgs a, DensState* ds, uint8_t* cls, int* eidx) {
  const long long c = (long long)*a.cand_count;
  const long long n = c < a.cand_cap ? c : a.cand_cap;
  const int lane = threadIdx.x & 31;
  if (ds->err) return;
  const float tq = ds->tau_apx, d2 = 2.0f * ds->delta * 1.0001f, lim = 1.0f - ds->delta;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // whole warps iterate together (warp-aggregated appends)
  for (long long i0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); i0 < n;
       i0 += stride) {
    const long long i = i0 + lane;
    uint8_t k = 0;
    if (i < n && a.cand[i].x != kCandNone) {
      const float r = a.cand_apx[i];
      if (fabsf(r) >= lim || fabsf(r - tq) <= d2) k = 2;
      else k = r > tq ? 1 : 3;
    }
    if (i < n) cls[i] = k;
    const uint32_t m2 = __ballot_sync(0xffffffffu, k == 2);
    const uint32_t m1 = __ballot_sync(0xffffffffu, k == 1);
    long long base = 0;
    if (lane == 0) {
      if (m1) atomicAdd((unsigned long long*)&ds->n_above, (unsigned long long)__popc(m1));
      if (m2) base = (long long)atomicAdd((unsigned long long*)&ds->n_exact,
                                          (unsigned long long)__popc(m2));
    }
    base = __shfl_sync(0xffffffffu, base, 0);
    if (k == 2) eidx[base + __popc(m2 & ((1u << lane) - 1u))] = (int)i;
  }
}

// Exact values of E (warp per item).
__global__ void dens_exact_kernel(CorrArgs a, DensState* ds, const int* eidx, float* exact,
                                  float* slot_val) {
  if (ds->err) return;
  const long long n = ds->n_exact;
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long e = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); e < n;
       e += nw) {
    const int slot = eidx[e];
    const uint2 p = a.cand[slot];
    const float r = exact_r_warp(a, (int)p.x, (int)p.y, lane);
    if (lane == 0) {
      exact[e] = r;
      slot_val[slot] = r;
    }
  }
}

// Count E above tau*, collect the ties, check the window.
__global__ void dens_ties_kernel(CorrArgs a, DensState* ds, const int* eidx, const float* exact,
                                 unsigned long long* ties) {
  if (ds->err) return;
  const double tau = (double)ds->tau;
  if (blockIdx.x == 0 && threadIdx.x == 0 && !(tau >= ds->A && tau <= ds->B))
    ds->err = DENS_ERR_WINDOW;
  const long long n = ds->n_exact;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const float r = exact[e];
    if (r > ds->tau) {
      atomicAdd((unsigned long long*)&ds->n_exact_gt, 1ull);
    } else if (r == ds->tau) {
      const unsigned long long t = atomicAdd((unsigned long long*)&ds->n_ties, 1ull);
      const uint2 p = a.cand[eidx[e]];
      if (t < (unsigned long long)kMaxTies) ties[t] = pair_key((int)p.x, (int)p.y);
    }
  }
}

// One block: sort the ties, keep the first ones in (i, j) order, list the rest.
__global__ void dens_drop_kernel(DensState* ds, const unsigned long long* stats,
                                 const unsigned long long* ties, unsigned long long* drop) {
  __shared__ unsigned long long s[kMaxTies];
  if (ds->err) return;
  const long long nt = ds->n_ties;
  if (nt > kMaxTies) {
    if (threadIdx.x == 0) ds->err = DENS_ERR_TIES;
    return;
  }
  const long long greater = (long long)stats[2] + ds->n_above + ds->n_exact_gt;
  const long long keep = ds->k - greater;
  if (keep < 1 || keep > nt) {
    if (threadIdx.x == 0) ds->err = DENS_ERR_RANK;
    return;
  }
  int n2 = 1;
  while (n2 < nt) n2 <<= 1;
  for (int i = threadIdx.x; i < n2; i += blockDim.x) s[i] = i < nt ? ties[i] : ~0ull;
  __syncthreads();
  // bitonic sort, ascending
  for (int size = 2; size <= n2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned long long x = s[i], y = s[j];
          if ((x > y) == up) {
            s[i] = y;
            s[j] = x;
          }
        }
      }
      __syncthreads();
    }
  }
  for (long long i = keep + threadIdx.x; i < nt; i += blockDim.x) drop[i - keep] = s[i];
  if (threadIdx.x == 0) {
    ds->greater = greater;
    ds->n_drop = (int)(nt - keep);
  }
}

// Decide every candidate, count the edges into seg, fill the hash.
__global__ void dens_decide_kernel(CorrArgs a, DensState* ds, const uint8_t* cls,
                                   const float* slot_val, const unsigned long long* drop) {
  if (ds->err) return;
  const long long c = (long long)*a.cand_count;
  const long long n = c < a.cand_cap ? c : a.cand_cap;
  const float tau = ds->tau;
  const int n_drop = ds->n_drop;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const uint8_t k = cls[i];
    if (k == 0) continue;
    const uint2 p = a.cand[i];
    const int pi = (int)p.x, pj = (int)p.y;
    const unsigned long long key = pair_key(pi, pj);
    float r = a.cand_apx[i];
    bool e = k == 1;
    if (k == 2) {
      r = slot_val[i];
      e = r > tau || (r == tau && !(n_drop > 0 && in_sorted(drop, n_drop, key)));
      if (fabsf(r - tau) <= 1e-6f) atomicAdd(&a.stats[1], 1ull);
    }
    if (e) {
      atomicAdd(&a.seg[(size_t)(pj / kBlk) * a.n_pad + pi], 1);
      atomicAdd(&a.seg[(size_t)(pi / kBlk) * a.n_pad + pj], 1);
      atomicAdd(&a.stats[0], 1ull);
    }
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

size_t dens_state_bytes() { return sizeof(DensState); }
size_t dens_ties_cap() { return kMaxTies; }

// Host-side view of the state.
void dens_state_read(const void* host, int* err, float* tau, long long* n_exact,
                     long long* n_ties, int* n_drop) {
  const DensState* d = static_cast<const DensState*>(host);
  *err = d->err;
  *tau = d->tau;
  *n_exact = d->n_exact;
  *n_ties = d->n_ties;
  *n_drop = d->n_drop;
}

// The whole selection and decision (15 kernels, no host synchronisation).
// Buffers: state (dens_state_bytes, k/delta/A/B filled by dens_set), hist
// (2048 uint, zero), cls (cand_cap bytes), eidx (cand_cap int), exact
// (cand_cap float), slot_val (cand_cap float), ties (kMaxTies u64), drop
// (kMaxTies u64).
cudaError_t launch_density_select(const CorrArgs& a, void* state, unsigned int* hist,
                                  uint8_t* cls, int* eidx, float* exact, float* slot_val,
                                  unsigned long long* ties, unsigned long long* drop, int sms,
                                  cudaStream_t st) {
  DensState* ds = static_cast<DensState*>(state);
  dens_init_kernel<<<1, 1, 0, st>>>(ds, a.stats);
  const int digits[3][2] = {{21, 11}, {10, 11}, {0, 10}};
  for (int which = 0; which < 2; ++which) {
    if (which == 1) {
      dens_classify_kernel<<<sms * 4, 256, 0, st>>>(a, ds, cls, eidx);
      dens_exact_kernel<<<sms * 8, 256, 0, st>>>(a, ds, eidx, exact, slot_val);
    }
    for (int d = 0; d < 3; ++d) {
      dens_hist_kernel<<<sms * 2, 256, 0, st>>>(a, ds, exact, which, digits[d][0], digits[d][1],
                                                hist);
      dens_pick_kernel<<<1, 1024, 0, st>>>(ds, hist, which, digits[d][0], digits[d][1], d == 0,
                                           d == 2);
    }
  }
  dens_ties_kernel<<<sms * 2, 256, 0, st>>>(a, ds, eidx, exact, ties);
  dens_drop_kernel<<<1, 1024, 0, st>>>(ds, a.stats, ties, drop);
  dens_decide_kernel<<<sms * 4, 256, 0, st>>>(a, ds, cls, slot_val, drop);
  return cudaGetLastError();
}

// Fill the inputs of the state (host values) before launch_density_select.
cudaError_t dens_set(void* state, long long k, float delta, double A, double B,
                     cudaStream_t st) {
  DensState h{};
  h.k = k;
  h.delta = delta;
  h.A = A;
  h.B = B;
  return cudaMemcpyAsync(state, &h, sizeof h, cudaMemcpyHostToDevice, st);
}

}  // namespace bna
