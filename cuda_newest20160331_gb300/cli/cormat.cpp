// bna_cormat: command-line drop-in for the reference's CUCorMat
// (W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:52-670), same arguments and outputs:
//
//   bna_cormat Dir_for_BOLD Path_for_mask threshold_for_mask(0~1)
//              to_average(yf/yn/bf/bn/n) to_save_cormatrix(y/n)
//              threshold_type(r/s) threshold(s)...
//
// Every .nii file of Dir except mask.nii is a subject (taken in name order).
// n / b: per subject, Dir/weighted/<name>_<N>_spa<s>%_cor<r>_weighted.csr for
// every threshold (r: edges r > tau; s: exactly the density's edge count),
// plus <name>_<N>.cormat with y.  y / b: the average over subjects (second
// letter f: Fisher z) to Dir/<dirname>_<files>_<N>_spa<s>%_cor<r>.csr.
// The correlation form comes from BNA_PRECISION (bf16x3 by default, or tf32 /
// fp32); every form gives the same edge set.
//
// Built a second time with BNA_UNWEIGHTED_TREE as bna_cormat_u, the drop-in
// for the unweighted tree's CUCorMat (U/CorMat/CUCorMat/CUCORMAT/CorMat.cpp,
// same arguments): per-subject files go to Dir/unweighted/<name>_<N>_spa<s>%
// _cor<r>.csr and every .csr is binary (R and C only, :340-345).
#include <cuda_runtime.h>
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bna.h"

namespace {

bna_ctx* g_ctx = nullptr;

#ifdef BNA_UNWEIGHTED_TREE
const char* const kSubdir = "unweighted";  // U/.../CUCORMAT/CorMat.cpp:290-296
const char* const kSuffix = "";
constexpr bool kWeighted = false;
#else
const char* const kSubdir = "weighted";
const char* const kSuffix = "_weighted";
constexpr bool kWeighted = true;
#endif

void die(const char* what, int st) {
  std::fprintf(stderr, "%s: %s (%s)\n", what, bna_status_string(st),
               g_ctx ? bna_ctx_last_error(g_ctx) : "");
  std::exit(1);
}

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    std::exit(1);
  }
}

bool ends_with_nii(const std::string& n) {
  return n.size() > 4 && n.compare(n.size() - 4, 4, ".nii") == 0;
}

int precision_from_env() {
  const char* p = std::getenv("BNA_PRECISION");
  if (!p || !*p || !std::strcmp(p, "bf16x3")) return BNA_PREC_BF16X3;
  if (!std::strcmp(p, "tf32")) return BNA_PREC_TF32;
  if (!std::strcmp(p, "fp32")) return BNA_PREC_FP32;
  std::fprintf(stderr, "BNA_PRECISION must be bf16x3, tf32 or fp32\n");
  std::exit(1);
}

std::string fmt_spa(double s, double r) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "_spa%.3f%%_cor%.3f", s, r);
  return buf;
}

void write_cormat(const std::string& path, const float* packed_dev, long long M1) {
  std::vector<float> h((size_t)M1);
  ck(cudaMemcpy(h.data(), packed_dev, (size_t)M1 * 4, cudaMemcpyDeviceToHost), "cormat copy");
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    std::fprintf(stderr, "can't write %s\n", path.c_str());
    std::exit(1);
  }
  const int m32 = (int)M1;  // the reference writes M1 as an int (CorMat.cpp:306)
  std::fwrite(&m32, 4, 1, f);
  std::fwrite(h.data(), 4, (size_t)M1, f);
  std::fclose(f);
}

// CSR to host and to the .csr file (CorMat.cpp:353-360); the unweighted
// tree's files hold no value section.
void write_csr_dev(const std::string& path, const bna_csr& d) {
  bna_csr h{};
  h.n = d.n;
  h.nnz = d.nnz;
  std::vector<int32_t> rp(d.n + 1), ci(std::max<int64_t>(d.nnz, 1));
  std::vector<float> va(std::max<int64_t>(d.nnz, 1));
  ck(cudaMemcpy(rp.data(), d.row_ptr, (size_t)(d.n + 1) * 4, cudaMemcpyDeviceToHost), "copy");
  const bool vals = kWeighted && d.val;
  if (d.nnz) {
    ck(cudaMemcpy(ci.data(), d.col_idx, (size_t)d.nnz * 4, cudaMemcpyDeviceToHost), "copy");
    if (vals)
      ck(cudaMemcpy(va.data(), d.val, (size_t)d.nnz * 4, cudaMemcpyDeviceToHost), "copy");
  }
  h.row_ptr = rp.data();
  h.col_idx = ci.data();
  h.val = vals ? va.data() : nullptr;
  std::printf("generating %s...\n", path.c_str());
  const int st = bna_csr_write(path.c_str(), &h);
  if (st) die("bna_csr_write", st);
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc < 7) {
    std::fprintf(stderr,
                 "Input format: bna_cormat Dir_for_BOLD Path_for_mask threshold_for_mask(0~1) "
                 "to_average(yf/yn/bf/bn/n) to_save_cormatrix(y/n) threshold_type(r/s) "
                 "threshold_for_correletaion_coefficient(s)(0~1)\n"
                 "For example: bna_cormat /data/BOLD /data/MASK/mask.nii 0.5 y n r 0.2 0.25 0.3\n");
    return 1;
  }
  std::string dir = argv[1];
  while (dir.size() > 1 && (dir.back() == '/' || dir.back() == '\\')) dir.pop_back();
  const char avg0 = argv[4][0], avg1 = argv[4][1];
  const bool per_subject = avg0 == 'n' || avg0 == 'N' || avg0 == 'b' || avg0 == 'B';
  const bool average = avg0 == 'y' || avg0 == 'Y' || avg0 == 'b' || avg0 == 'B';
  bool cormat_flag;
  if (argv[5][0] == 'y' || argv[5][0] == 'Y') cormat_flag = true;
  else if (argv[5][0] == 'n' || argv[5][0] == 'N') cormat_flag = false;
  else {
    std::printf("to_save_cor_matrix type error! \ny to save the whole correlation matrix \n"
                "n to save only csr format of adjacency matrix\n");
    return 1;
  }
  bool rs_flag;
  if (argv[6][0] == 'r' || argv[6][0] == 'R') rs_flag = true;
  else if (argv[6][0] == 's' || argv[6][0] == 'S') rs_flag = false;
  else {
    std::printf("threshold type error! \nr for correlation threshold\ns for spasity threshold\n");
    return 1;
  }
  if (average && avg1 != 'f' && avg1 != 'F' && avg1 != 'n' && avg1 != 'N') {
    std::printf("to_average must be yf, yn, bf, bn or n\n");
    return 1;
  }
  const bool fisher = avg1 == 'f' || avg1 == 'F';
  std::vector<double> thr;
  for (int k = 7; k < argc; ++k) thr.push_back((float)std::atof(argv[k]));
  const int prec = precision_from_env();

  std::vector<std::string> files;
  DIR* dp = opendir(dir.c_str());
  if (!dp) {
    std::printf("can't open %s", dir.c_str());
    return 1;
  }
  while (dirent* e = readdir(dp)) {
    const std::string n = e->d_name;
    if (ends_with_nii(n) && n != "mask.nii") files.push_back(n);
  }
  closedir(dp);
  std::sort(files.begin(), files.end());
  std::printf("%zu file(s) to be processed.\n", files.size());

  int32_t dims[3];
  int64_t total = 0;
  int32_t N = 0;
  int st = bna_nifti_mask(argv[2], std::atof(argv[3]), dims, &total, &N, nullptr);
  if (st) die(argv[2], st);
  std::vector<uint8_t> sel((size_t)total);
  bna_nifti_mask(argv[2], std::atof(argv[3]), dims, &total, &N, sel.data());
  std::printf("Data size: %dx%dx%d, Grey voxel count: %d.\n", dims[0], dims[1], dims[2], N);
  if (N < 2) return 1;
  const long long M1 = (long long)N * (N - 1) / 2;

  if ((st = bna_ctx_create(0, &g_ctx))) die("bna_ctx_create", st);
  std::vector<float*> bold_dev;
  std::vector<int32_t> Ts;
  for (const std::string& fn : files) {  // every subject to the device once
    const std::string path = dir + "/" + fn;
    int32_t T = 0;
    if ((st = bna_nifti_bold(path.c_str(), sel.data(), total, N, nullptr, &T))) die(path.c_str(), st);
    std::vector<float> h((size_t)T * N);
    if ((st = bna_nifti_bold(path.c_str(), sel.data(), total, N, h.data(), &T))) die(path.c_str(), st);
    std::printf("BOLD length: %d, %s\n", T, fn.c_str());
    float* d;
    ck(cudaMalloc(&d, h.size() * 4), "cudaMalloc");
    ck(cudaMemcpy(d, h.data(), h.size() * 4, cudaMemcpyHostToDevice), "copy");
    bold_dev.push_back(d);
    Ts.push_back(T);
  }
  float* packed = nullptr;
  if (cormat_flag) ck(cudaMalloc(&packed, (size_t)M1 * 4), "cudaMalloc");
  const int pk_prec = prec == BNA_PREC_FP32 ? BNA_PREC_BF16X3 : prec;

  if (per_subject) {
    mkdir((dir + "/" + kSubdir).c_str(), 0755);
    for (size_t f = 0; f < files.size(); ++f) {
      std::printf("\ncalculating correlation for %s/%s ...\n", dir.c_str(), files[f].c_str());
      const std::string stem = files[f].substr(0, files[f].find_last_of('.'));
      const std::string out = dir + "/" + kSubdir + "/" + stem + "_" + std::to_string(N);
      if (cormat_flag) {
        if ((st = bna_corr_packed(g_ctx, 1, &bold_dev[f], N, &Ts[f], 0, pk_prec, packed, nullptr)))
          die("bna_corr_packed", st);
        write_cormat(out + ".cormat", packed, M1);
      }
      bna_corr_opts o{};
      o.precision = prec;
      o.weighted = 1;
      bna_corr_stats s{};
      if (rs_flag) {
        // one correlation pass at the lowest threshold, the others derived
        std::vector<double> sorted = thr;
        std::sort(sorted.begin(), sorted.end());
        o.mode = BNA_THR_R_GT;  // FormFullGraph: r > tau (CorMat.cpp:696)
        o.value = sorted.empty() ? 1.0 : sorted[0];
        bna_csr base{};
        if ((st = bna_corr_csr(g_ctx, bold_dev[f], N, Ts[f], &o, &base, &s, nullptr)))
          die("bna_corr_csr", st);
        for (double t : thr) {
          bna_csr c = base;
          if ((float)t != (float)o.value &&
              (st = bna_csr_rethreshold(g_ctx, &base, BNA_THR_R_GT, t, &c, nullptr, nullptr)))
            die("bna_csr_rethreshold", st);
          const double spa = 100.0 * (double)c.nnz / (double)M1 / 2;  // CorMat.cpp:323
          write_csr_dev(out + fmt_spa(spa, (float)t) + kSuffix + ".csr", c);
        }
      } else {
        for (double sp : thr) {
          std::printf("\nthreshold for sparsity = %g\n", sp);
          o.mode = BNA_THR_DENSITY;
          o.value = sp;
          bna_csr c{};
          if ((st = bna_corr_csr(g_ctx, bold_dev[f], N, Ts[f], &o, &c, &s, nullptr)))
            die("bna_corr_csr", st);
          write_csr_dev(out + fmt_spa((float)sp, (float)s.tau) + kSuffix + ".csr", c);
        }
      }
    }
  }
  if (average && !files.empty()) {
    const std::string base = dir.substr(dir.find_last_of("/\\") == std::string::npos
                                            ? 0 : dir.find_last_of("/\\") + 1);
    const std::string out = dir + "/" + base + "_" + std::to_string(files.size()) + "_" +
                            std::to_string(N);
    const int nsub = (int)files.size();
    if (cormat_flag) {
      if ((st = bna_corr_packed(g_ctx, nsub, bold_dev.data(), N, Ts.data(), fisher ? 1 : 0,
                                pk_prec, packed, nullptr)))
        die("bna_corr_packed", st);
      write_cormat(out + ".cormat", packed, M1);
    }
    for (double t : thr) {
      bna_corr_opts o{};
      o.precision = pk_prec;
      o.weighted = 1;
      o.mode = rs_flag ? BNA_THR_R_GT : BNA_THR_DENSITY;
      o.value = t;
      bna_csr c{};
      bna_corr_stats s{};
      if ((st = bna_corr_csr_avg(g_ctx, nsub, bold_dev.data(), N, Ts.data(), fisher ? 1 : 0, &o,
                                 &c, &s, nullptr)))
        die("bna_corr_csr_avg", st);
      const double spa = rs_flag ? 100.0 * (double)c.nnz / (double)M1 / 2 : (float)t;
      const double cor = rs_flag ? (float)t : (float)s.tau;
      write_csr_dev(out + fmt_spa(spa, cor) + ".csr", c);
    }
  }
  for (float* d : bold_dev) cudaFree(d);
  if (packed) cudaFree(packed);
  bna_ctx_destroy(g_ctx);
  return 0;
}
