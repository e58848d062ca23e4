// Deterministic synthetic BOLD generator (factor model) for the voxel-network
// builder workloads.
//
//   x_i(t) = sum_{k<K} L_ik * f_k(t) + eps_i(t)
//
// f_k is an AR(1) series with coefficient phi and unit stationary variance
// (innovation sd = sqrt(1 - phi^2), 100 burn-in steps from 0), eps ~ N(0, 1).
// Loadings:
//   BNA_SYNTH_IID       L_ik ~ N(0, load_sd^2) independently per voxel;
//   BNA_SYNTH_BLOCKNET  voxels form contiguous blocks of `block` voxels; block b
//                       belongs to network (b mod n_net) and
//                       L_ik = load_sd * g_{net,k} + jitter_sd * h_ik,
//                       so every block shares its network's loading vector.
//
// The output is float32, time-major [T][N] (the layout the reference builds
// from NIfTI: BOLD[l*N+i], CorMat.cpp:219/234).
//
// Bit-identical on every host: counter-based hashing for the random stream,
// only IEEE-754 basic operations and sqrt (correctly rounded), a home-made
// natural logarithm (no libm), and the file is compiled with
// -ffp-contract=off so no multiply-add is fused.  Every output element is a
// pure function of (seed, indices), so the thread count does not matter.
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>
#include <cmath>

#include "../../include/bna.h"

namespace {

inline uint64_t fmix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

// Uniform double in (0, 1) from a (seed, stream, index, draw) counter.
inline double uniform01(uint64_t seed, uint64_t stream, uint64_t idx, uint64_t draw) {
  uint64_t x = seed * 0x9E3779B97F4A7C15ULL;
  x = fmix64(x ^ (stream * 0xD1B54A32D192ED03ULL));
  x = fmix64(x ^ (idx * 0x8CB92BA72F3D8DD7ULL));
  x = fmix64(x ^ (draw * 0xABC98388FB8FAC03ULL + 0x632BE59BD9B4E019ULL));
  return (double)(x >> 11) * 0x1.0p-53 + 0x1.0p-54;
}

// ln(x) for finite x > 0 from x = m * 2^e, m in [sqrt(1/2), sqrt(2)),
// ln(m) = 2 atanh(s), s = (m-1)/(m+1), evaluated by its odd power series.
inline double det_log(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  b = (b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
  double m;
  std::memcpy(&m, &b, 8);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double p = 1.0 / 25.0;
  for (int k = 11; k >= 0; --k) p = p * s2 + 1.0 / (double)(2 * k + 1);
  const double ln2 = 0x1.62e42fefa39efp-1;
  return (double)e * ln2 + 2.0 * s * p;
}

// Standard normal by Marsaglia's polar method on the counter stream.
inline double normal(uint64_t seed, uint64_t stream, uint64_t idx) {
  for (uint64_t d = 0;; d += 2) {
    const double v1 = 2.0 * uniform01(seed, stream, idx, d) - 1.0;
    const double v2 = 2.0 * uniform01(seed, stream, idx, d + 1) - 1.0;
    const double s = v1 * v1 + v2 * v2;
    if (s > 0.0 && s < 1.0) return v1 * std::sqrt(-2.0 * det_log(s) / s);
  }
}

enum : uint64_t { S_FACTOR = 1, S_LOAD = 2, S_NET = 3, S_NOISE = 4 };

}  // namespace

extern "C" int bna_synth_bold(const bna_synth_params* p, float* out, int n_threads) {
  if (!p || !out) return BNA_BAD_ARG;
  const int N = p->N, T = p->T, K = p->K;
  if (N <= 0 || T <= 0 || K < 0) return BNA_BAD_ARG;
  if (p->kind == BNA_SYNTH_BLOCKNET && (p->block <= 0 || p->n_net <= 0)) return BNA_BAD_ARG;
  const uint64_t seed = p->seed;
  const int burn = 100;
  const double phi = p->phi;
  const double innov = std::sqrt(1.0 - phi * phi);

  // Factor series f[k][t].
  std::vector<double> f((size_t)K * T);
  for (int k = 0; k < K; ++k) {
    double v = 0.0;
    for (int t = 0; t < burn + T; ++t) {
      v = phi * v + innov * normal(seed, S_FACTOR, (uint64_t)k * (burn + T) + t);
      if (t >= burn) f[(size_t)k * T + (t - burn)] = v;
    }
  }
  // Network loading vectors (block-network kind only).
  std::vector<double> g;
  if (p->kind == BNA_SYNTH_BLOCKNET) {
    g.resize((size_t)p->n_net * K);
    for (int n = 0; n < p->n_net; ++n)
      for (int k = 0; k < K; ++k) g[(size_t)n * K + k] = normal(seed, S_NET, (uint64_t)n * K + k);
  }

  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  const int chunk = 256;
  const int n_chunks = (N + chunk - 1) / chunk;
  auto work = [&](int tid) {
    std::vector<double> L((size_t)chunk * (K > 0 ? K : 1));
    for (int c = tid; c < n_chunks; c += n_threads) {
      const int i0 = c * chunk, i1 = std::min(N, i0 + chunk);
      for (int i = i0; i < i1; ++i) {
        double* Li = &L[(size_t)(i - i0) * K];
        for (int k = 0; k < K; ++k) {
          const double h = normal(seed, S_LOAD, (uint64_t)i * K + k);
          if (p->kind == BNA_SYNTH_BLOCKNET) {
            const int net = (i / p->block) % p->n_net;
            Li[k] = p->load_sd * g[(size_t)net * K + k] + p->jitter_sd * h;
          } else {
            Li[k] = p->load_sd * h;
          }
        }
      }
      for (int t = 0; t < T; ++t) {
        float* row = out + (size_t)t * N;
        for (int i = i0; i < i1; ++i) {
          const double* Li = &L[(size_t)(i - i0) * K];
          double x = 0.0;
          for (int k = 0; k < K; ++k) x = x + Li[k] * f[(size_t)k * T + t];
          x = x + normal(seed, S_NOISE, (uint64_t)i * T + t);
          row[i] = (float)x;
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& t : th) t.join();
  return BNA_OK;
}
