// bna_degree: command-line drop-in for the reference's Degree tool
// (W/Degree/Degree/Degree.cpp): for every .csr file of the directory (name
// order), the degree of each vertex (the float sum of its row's values) as
// <name>_deg.nm (int32 N, float deg[N]).
//
//   bna_degree dir_for_csr
#include <cuda_runtime.h>
#include <dirent.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "bna.h"

int main(int argc, char* argv[]) {
  if (argc < 2) {
    std::fprintf(stderr, "Input format: bna_degree dir_for_csr\n");
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
  for (const std::string& fn : files) {
    const std::string a = dir + "/" + fn;
    std::printf("\ncalculating Degree for %s ...\n", a.c_str());
    bna_csr h{};
    if (bna_csr_read(a.c_str(), &h) != BNA_OK) {
      std::printf("Can't open\t%s\n", a.c_str());
      return 0;
    }
    bna_csr d{};
    d.n = h.n;
    d.nnz = h.nnz;
    float* deg = nullptr;
    bool ok = cudaMalloc(&d.row_ptr, (size_t)(h.n + 1) * 4) == cudaSuccess &&
              cudaMalloc(&deg, (size_t)h.n * 4) == cudaSuccess &&
              cudaMemcpy(d.row_ptr, h.row_ptr, (size_t)(h.n + 1) * 4, cudaMemcpyHostToDevice) ==
                  cudaSuccess;
    if (ok && h.val && h.nnz > 0)
      ok = cudaMalloc(&d.val, (size_t)h.nnz * 4) == cudaSuccess &&
           cudaMemcpy(d.val, h.val, (size_t)h.nnz * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    std::vector<float> out(h.n);
    ok = ok && bna_degree(&d, deg, nullptr) == BNA_OK &&
         cudaMemcpy(out.data(), deg, (size_t)h.n * 4, cudaMemcpyDeviceToHost) == cudaSuccess;
    if (!ok) {
      std::fprintf(stderr, "device error\n");
      return 1;
    }
    const std::string x = a.substr(0, a.find_last_of('.')) + "_deg.nm";
    std::printf("Save degree data for each node as %s\n", x.c_str());
    FILE* f = std::fopen(x.c_str(), "wb");
    if (f) {
      const int n = h.n;
      std::fwrite(&n, 4, 1, f);
      std::fwrite(out.data(), 4, (size_t)n, f);
      std::fclose(f);
    }
    cudaFree(d.row_ptr);
    cudaFree(d.val);
    cudaFree(deg);
    bna_csr_free_host(&h);
  }
  return 0;
}
