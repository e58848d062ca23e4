// bna_modularity: command-line drop-in for the reference's Newman modularity
// tool (U/Newman_Modularity_CPU/Modularity_CPU/Modularity_CPU.cpp, main
// :35-162): for every .csr file of the directory (name order), the spectral
// modules of its binary graph as <name>_modu.nm (int32 N, float label[N],
// :122-131) and the round-by-round log <name>_modu.txt (the lines the tool
// writes to its log stream, :196-203, 268-283, 362-363, 226-229).  Then, as
// the tool does (:131-143), num_of_random_networks degree-preserving random
// rewirings of the network (Maslov-Sneppen edge swaps, the reference's Rewire
// in W/Newman_Modularity_GPU/CUmodularity/Maslov.cpp:7-66) are divided too
// and only logged.  The reference seeds its swaps with time(0); here the
// swaps come from a fixed-seed generator (BNA_SEED overrides the seed), so a
// run can be repeated.
//
//   bna_modularity dir_for_csr num_of_random_networks
#include <cuda_runtime.h>
#include <dirent.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <unordered_set>
#include <vector>

#include "bna.h"

namespace {

// Degree-preserving rewiring of a symmetric binary CSR: 2M attempts, each
// picks two edges (i<j listing), drops the attempt when they share a node,
// else reconnects them one of the two ways at random unless a new edge
// already exists (Maslov.cpp:17-63).  Rows come back with ascending columns.
void maslov(const std::vector<int32_t>& R, const std::vector<int32_t>& C,
            std::vector<int32_t>& Cout, uint64_t& seed) {
  const int n = (int)R.size() - 1;
  std::vector<int32_t> ea, eb;
  std::unordered_set<uint64_t> has;
  for (int i = 0; i < n; ++i)
    for (int32_t k = R[i]; k < R[i + 1]; ++k)
      if (C[k] > i) {
        ea.push_back(i);
        eb.push_back(C[k]);
        has.insert((uint64_t)i * n + C[k]);
      }
  auto key = [n](int a, int b) { return a < b ? (uint64_t)a * n + b : (uint64_t)b * n + a; };
  auto next = [&seed]() {  // splitmix64
    uint64_t z = (seed += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  };
  const long long m = (long long)ea.size();
  for (long long t = 0; m > 1 && t < 2 * m; ++t) {
    const long long i = (long long)(next() % (uint64_t)m), j = (long long)(next() % (uint64_t)m);
    const int v1 = ea[i], v2 = eb[i], v3 = ea[j], v4 = eb[j];
    if (v1 == v3 || v1 == v4 || v2 == v3 || v2 == v4) continue;
    if (next() & 1) {  // 1-3, 2-4
      if (has.count(key(v1, v3)) || has.count(key(v2, v4))) continue;
      has.erase(key(v1, v2));
      has.erase(key(v3, v4));
      has.insert(key(v1, v3));
      has.insert(key(v2, v4));
      eb[i] = v3;
      ea[j] = v2;
    } else {  // 1-4, 3-2
      if (has.count(key(v1, v4)) || has.count(key(v2, v3))) continue;
      has.erase(key(v1, v2));
      has.erase(key(v3, v4));
      has.insert(key(v1, v4));
      has.insert(key(v2, v3));
      eb[i] = v4;
      eb[j] = v2;
    }
  }
  std::vector<std::vector<int32_t>> rows(n);
  for (long long e = 0; e < m; ++e) {
    rows[ea[e]].push_back(eb[e]);
    rows[eb[e]].push_back(ea[e]);
  }
  Cout.clear();
  for (int i = 0; i < n; ++i) {
    std::sort(rows[i].begin(), rows[i].end());
    Cout.insert(Cout.end(), rows[i].begin(), rows[i].end());
  }
}

// One partition of (R, C) on the device; its lines go to `log`.
bool partition(bna_ctx* ctx, const std::vector<int32_t>& R, const std::vector<int32_t>& C,
               std::vector<int32_t>* labels, FILE* log) {
  const int n = (int)R.size() - 1;
  bna_csr d{};
  d.n = n;
  d.nnz = (int64_t)C.size();
  int32_t* lab = nullptr;
  bool ok = cudaMalloc(&d.row_ptr, R.size() * 4) == cudaSuccess &&
            cudaMalloc(&d.col_idx, std::max<size_t>(C.size(), 1) * 4) == cudaSuccess &&
            cudaMalloc(&lab, (size_t)n * 4) == cudaSuccess &&
            cudaMemcpy(d.row_ptr, R.data(), R.size() * 4, cudaMemcpyHostToDevice) ==
                cudaSuccess &&
            (C.empty() || cudaMemcpy(d.col_idx, C.data(), C.size() * 4,
                                     cudaMemcpyHostToDevice) == cudaSuccess);
  std::vector<bna_mod_round> recs((size_t)2 * n + 2);
  int32_t modules = 0, nrec = 0;
  double q = 0;
  const auto t0 = std::chrono::steady_clock::now();
  int32_t s = ok ? bna_modularity(ctx, &d, 0.0, lab, &modules, &q, recs.data(),
                                  (int32_t)recs.size(), &nrec, nullptr)
                 : BNA_CUDA_ERROR;
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (s == BNA_OK && labels) {
    labels->resize(n);
    ok = cudaMemcpy(labels->data(), lab, (size_t)n * 4, cudaMemcpyDeviceToHost) == cudaSuccess;
    if (!ok) s = BNA_CUDA_ERROR;
  }
  cudaFree(d.row_ptr);
  cudaFree(d.col_idx);
  cudaFree(lab);
  if (s != BNA_OK) {
    std::fprintf(stderr, "modularity failed: %s (%s)\n", bna_status_string(s),
                 bna_ctx_last_error(ctx));
    return false;
  }
  for (int32_t r = 0; r < nrec && r < (int32_t)recs.size(); ++r) {
    const bna_mod_round& e = recs[r];
    std::string line = "\nRound:\t" + std::to_string(e.round) + "\tnumber of nodes:\t" +
                       std::to_string(e.nodes) + "\t";
    char buf[160];
    for (int c = 0; c < 2; ++c) {
      if (c == 1 && e.iters[1] == 0) break;  // no retry
      std::snprintf(buf, sizeof buf, "Iterations:\t%d\tresidual:\t%g\t", e.iters[c],
                    e.residual[c]);
      line += buf;
    }
    std::snprintf(buf, sizeof buf, "Eigen Value: %g\tDivide?: %d\t", e.lambda, e.divided);
    line += buf;
    std::fputs(line.c_str(), stdout);
    if (log) std::fputs(line.c_str(), log);
  }
  char tail[200];
  std::snprintf(tail, sizeof tail, "\nNumber of Modules: %d,\tQ=%g\nElapsed time:   %gs\n",
                modules, q, secs);
  std::fputs(tail, stdout);
  if (log) std::fputs(tail, log);
  return true;
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc != 3) {
    std::fprintf(stderr,
                 "Input format: bna_modularity dir_for_csr num_of_random_networks\n"
                 "For example: bna_modularity /data 10\n");
    return 1;
  }
  std::string dir = argv[1];
  while (dir.size() > 1 && (dir.back() == '/' || dir.back() == '\\')) dir.pop_back();
  const int nrand = std::atoi(argv[2]);
  DIR* dp = opendir(dir.c_str());
  if (!dp) {
    std::printf("can't open %s", dir.c_str());
    return 1;
  }
  std::vector<std::string> files;
  while (dirent* e = readdir(dp)) {
    const std::string n = e->d_name;
    if (n.size() > 4 && n.compare(n.size() - 4, 4, ".csr") == 0) files.push_back(n);
  }
  closedir(dp);
  std::sort(files.begin(), files.end());
  std::printf("%zu files to be processed.\n", files.size());
  bna_ctx* ctx = nullptr;
  if (bna_ctx_create(0, &ctx) != BNA_OK) {
    std::fprintf(stderr, "no CUDA device\n");
    return 1;
  }
  uint64_t seed = 20160115;
  if (const char* e = std::getenv("BNA_SEED")) seed = std::strtoull(e, nullptr, 10);
  int rc = 0;
  for (const std::string& fn : files) {
    const std::string a = dir + "/" + fn;
    std::printf("\nModular analysis for %s ...\n", a.c_str());
    bna_csr h{};
    if (bna_csr_read(a.c_str(), &h) != BNA_OK) {
      std::printf("Can't open\t%s\n", a.c_str());
      break;
    }
    std::vector<int32_t> R(h.row_ptr, h.row_ptr + h.n + 1), C(h.col_idx, h.col_idx + h.nnz);
    bna_csr_free_host(&h);
    const std::string stem = a.substr(0, a.find_last_of('.'));
    FILE* log = std::fopen((stem + "_modu.txt").c_str(), "w");
    std::vector<int32_t> labels;
    if (!partition(ctx, R, C, &labels, log)) {
      rc = 1;
      if (log) std::fclose(log);
      break;
    }
    const std::string x = stem + "_modu.nm";
    std::printf("Save partition results as %s\n", x.c_str());
    if (bna_modu_write(x.c_str(), labels.data(), (int32_t)labels.size()) != BNA_OK) rc = 1;
    if (nrand > 0) std::printf("Modular analysis for random networks...\n");
    std::vector<int32_t> Cr;
    for (int r = 0; r < nrand && rc == 0; ++r) {
      maslov(R, C, Cr, seed);
      if (!partition(ctx, R, Cr, nullptr, log)) rc = 1;
    }
    if (log) std::fclose(log);
    if (rc) break;
  }
  std::printf("===========================================================\n");
  bna_ctx_destroy(ctx);
  return rc;
}
