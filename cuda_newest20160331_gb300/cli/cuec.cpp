// bna_cuec: command-line drop-in for the reference's CUEC
// (W/CUEC/weighted-net.cu:222-331): for every .csr file of the directory
// (name order), eigenvector centrality by power iteration (Lead_Vector_GPU
// semantics, 10,000 iterations at most, stop at 1e-6), written as
// <name>_ec.nm (int32 N, float ec[N]) and <name>_evalue.txt (the eigenvalue,
// six significant digits).
//
//   bna_cuec Dir_of_csr_files
#include <dirent.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "bna.h"

int main(int argc, char* argv[]) {
  if (argc < 2) {
    std::fprintf(stderr, "Input format: bna_cuec Dir_of_csr_files\n");
    return 1;
  }
  std::string dir = argv[1];
  while (dir.size() > 1 && (dir.back() == '/' || dir.back() == '\\')) dir.pop_back();
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
  int st = bna_ctx_create(0, &ctx);
  if (st) {
    std::fprintf(stderr, "bna_ctx_create: %s\n", bna_status_string(st));
    return 1;
  }
  for (const std::string& fn : files) {
    const std::string a = dir + "/" + fn;
    std::printf("\ncalculating eigenvalue centrality for %s ...\n", a.c_str());
    bna_csr c{};
    st = bna_csr_read(a.c_str(), &c);
    if (st == BNA_CORRUPT_FILE) {
      std::printf("Your csr file %s is damaged!\n", a.c_str());  // weighted-net.cu:283
      continue;
    }
    if (st) {
      std::printf("Can't open\t%s\n", a.c_str());
      return 0;
    }
    std::vector<double> V;
    if (c.val) V.assign(c.val, c.val + c.nnz);  // float V promoted (weighted-net.cu:295-297)
    std::vector<double> ec(c.n);
    double lambda = 0;
    int32_t iters = 0;
    st = bna_lead_vector(ctx, c.row_ptr, c.col_idx, c.val ? V.data() : nullptr, c.n, ec.data(),
                         &lambda, &iters);
    if (st != BNA_OK && st != BNA_NOT_CONVERGED) {
      std::fprintf(stderr, "bna_lead_vector: %s (%s)\n", bna_status_string(st),
                   bna_ctx_last_error(ctx));
      return 1;
    }
    const std::string stem = a.substr(0, a.find_last_of('.'));
    std::printf("Save eigenvector centrality for each node as %s_ec.nm\n", stem.c_str());
    bna_ec_write((stem + "_ec.nm").c_str(), ec.data(), c.n);
    FILE* f = std::fopen((stem + "_evalue.txt").c_str(), "w");
    if (f) {
      std::fprintf(f, "%.6g\n", lambda);  // setprecision(6) << x << endl
      std::fclose(f);
    }
    bna_csr_free_host(&c);
  }
  bna_ctx_destroy(ctx);
  return 0;
}
