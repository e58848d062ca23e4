// .csr and _ec.nm file formats of the reference.
//
// .csr writer: W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:353-360 (weighted:
//   int Rlength; int R[Rlength]; int Clength; int C[Clength]; int Clength; float V[Clength]);
//   the unweighted tree writes only R and C (U/CorMat/CUCorMat/CUCORMAT/CorMat.cpp).
// .csr reader: W/CUEC/weighted-net.cu:275-287 (reports a damaged file when
//   Vlength != Clength, :283-284).
// _ec.nm writer: W/CUEC/weighted-net.cu:309-318 (int N; float ec[N]).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/bna.h"

namespace {

bool write_all(FILE* f, const void* p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }
bool read_all(FILE* f, void* p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

}  // namespace

extern "C" int32_t bna_csr_write(const char* path, const bna_csr* c) {
  if (!path || !c || c->n < 0 || !c->row_ptr || c->nnz < 0 || (c->nnz > 0 && !c->col_idx))
    return BNA_BAD_ARG;
  if (c->nnz > 0x7fffffffLL || c->n >= 0x7fffffff) return BNA_NNZ_OVERFLOW_INT32;
  FILE* f = std::fopen(path, "wb");
  if (!f) return BNA_IO_ERROR;
  const int32_t rlen = c->n + 1;
  const int32_t clen = (int32_t)c->nnz;
  bool ok = write_all(f, &rlen, 4) && write_all(f, c->row_ptr, (size_t)rlen * 4) &&
            write_all(f, &clen, 4) && write_all(f, c->col_idx, (size_t)clen * 4);
  if (ok && c->val) ok = write_all(f, &clen, 4) && write_all(f, c->val, (size_t)clen * 4);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BNA_OK : BNA_IO_ERROR;
}

extern "C" int32_t bna_csr_read(const char* path, bna_csr* out) {
  if (!path || !out) return BNA_BAD_ARG;
  std::memset(out, 0, sizeof *out);
  FILE* f = std::fopen(path, "rb");
  if (!f) return BNA_IO_ERROR;
  int32_t rlen = 0, clen = 0, vlen = 0;
  int32_t st = BNA_OK;
  if (!read_all(f, &rlen, 4) || rlen < 1) {
    st = BNA_CORRUPT_FILE;
  } else {
    out->n = rlen - 1;
    out->row_ptr = (int32_t*)std::malloc((size_t)rlen * 4);
    if (!out->row_ptr) st = BNA_OOM;
    else if (!read_all(f, out->row_ptr, (size_t)rlen * 4) || !read_all(f, &clen, 4) || clen < 0)
      st = BNA_CORRUPT_FILE;
    else {
      out->nnz = clen;
      out->col_idx = (int32_t*)std::malloc((size_t)(clen > 0 ? clen : 1) * 4);
      if (!out->col_idx) st = BNA_OOM;
      else if (!read_all(f, out->col_idx, (size_t)clen * 4)) st = BNA_CORRUPT_FILE;
      else if (read_all(f, &vlen, 4)) {
        if (vlen != clen) st = BNA_CORRUPT_FILE;  // "Your csr file ... is damaged"
        else {
          out->val = (float*)std::malloc((size_t)(clen > 0 ? clen : 1) * 4);
          if (!out->val) st = BNA_OOM;
          else if (!read_all(f, out->val, (size_t)clen * 4)) st = BNA_CORRUPT_FILE;
        }
      }
      // no V section: binary (unweighted) graph
    }
  }
  if (st == BNA_OK) {
    // structural checks: R monotone, R[0] == 0, R[N] == Clength, columns in range
    if (out->row_ptr[0] != 0 || out->row_ptr[out->n] != clen) st = BNA_CORRUPT_FILE;
    for (int32_t i = 0; st == BNA_OK && i < out->n; ++i)
      if (out->row_ptr[i + 1] < out->row_ptr[i]) st = BNA_CORRUPT_FILE;
    for (int64_t k = 0; st == BNA_OK && k < out->nnz; ++k)
      if (out->col_idx[k] < 0 || out->col_idx[k] >= out->n) st = BNA_CORRUPT_FILE;
  }
  std::fclose(f);
  if (st != BNA_OK) bna_csr_free_host(out);
  return st;
}

extern "C" int32_t bna_ec_write(const char* path, const double* ec, int32_t N) {
  if (!path || !ec || N < 0) return BNA_BAD_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return BNA_IO_ERROR;
  bool ok = write_all(f, &N, 4);
  for (int32_t i = 0; ok && i < N; ++i) {
    const float v = (float)ec[i];
    ok = write_all(f, &v, 4);
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BNA_OK : BNA_IO_ERROR;
}

extern "C" int32_t bna_modu_write(const char* path, const int32_t* labels, int32_t N) {
  if (!path || (!labels && N > 0) || N < 0) return BNA_BAD_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return BNA_IO_ERROR;
  bool ok = write_all(f, &N, 4);
  for (int32_t i = 0; ok && i < N; ++i) {
    const float v = (float)labels[i];
    ok = write_all(f, &v, 4);
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BNA_OK : BNA_IO_ERROR;
}
