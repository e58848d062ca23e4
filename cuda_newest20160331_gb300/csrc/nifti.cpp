// NIfTI-1 ingest with the reference's semantics (W/CorMat/CUCorMat/CUCorMat/
// CorMat.cpp:141-242): the 352-byte header is read as 176 shorts; dim[1..3]
// = hdr[21..23] give the voxel count, dim[4] = hdr[24] the series length;
// the mask's datatype hdr[35] must be 2 (unsigned char) or 16 (float) and a
// voxel is kept when mask >= cut (compared in float); a series' sample type
// follows its bitpix hdr[36] (64: double, 32: float) and the kept voxels are
// gathered, in the file's linear order, into the time-major layout
// BOLD[t * N + i] (doubles narrowed to float).  The voxel data follow the
// header directly, as the reference reads them; files are little-endian.
#include <cstdio>
#include <cstring>
#include <vector>

#include "bna.h"

namespace {

constexpr int kHdrLen = 352;

bool read_header(FILE* f, short hdr[kHdrLen / 2]) {
  return std::fread(hdr, 1, kHdrLen, f) == (size_t)kHdrLen;
}

}  // namespace

extern "C" {

int32_t bna_nifti_mask(const char* path, double cut, int32_t dims_out[3], int64_t* total_out,
                       int32_t* n_out, uint8_t* sel_out) {
  if (!path || !total_out || !n_out) return BNA_BAD_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return BNA_IO_ERROR;
  short hdr[kHdrLen / 2];
  if (!read_header(f, hdr)) {
    std::fclose(f);
    return BNA_CORRUPT_FILE;
  }
  const long long total = (long long)hdr[21] * hdr[22] * hdr[23];
  const int dt = hdr[35];
  if (total <= 0 || (dt != 2 && dt != 16)) {
    std::fclose(f);
    return BNA_CORRUPT_FILE;  // "mask data-type error" (CorMat.cpp:166-171)
  }
  std::vector<float> mask((size_t)total);
  bool ok;
  if (dt == 2) {
    std::vector<unsigned char> m((size_t)total);
    ok = std::fread(m.data(), 1, (size_t)total, f) == (size_t)total;
    for (long long k = 0; k < total; ++k) mask[k] = (float)m[k];
  } else {
    ok = std::fread(mask.data(), sizeof(float), (size_t)total, f) == (size_t)total;
  }
  std::fclose(f);
  if (!ok) return BNA_CORRUPT_FILE;
  const float c = (float)cut;  // ProbCut is a float (CorMat.cpp:96)
  long long n = 0;
  for (long long k = 0; k < total; ++k) {
    const bool keep = mask[k] >= c;
    n += keep;
    if (sel_out) sel_out[k] = keep ? 1 : 0;
  }
  if (n > 0x7fffffffLL) return BNA_UNSUPPORTED;
  if (dims_out) {
    dims_out[0] = hdr[21];
    dims_out[1] = hdr[22];
    dims_out[2] = hdr[23];
  }
  *total_out = total;
  *n_out = (int32_t)n;
  return BNA_OK;
}

int32_t bna_nifti_bold(const char* path, const uint8_t* sel, int64_t total, int32_t N,
                       float* bold_out, int32_t* T_out) {
  if (!path || !sel || total <= 0 || N < 1 || !T_out) return BNA_BAD_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return BNA_IO_ERROR;
  short hdr[kHdrLen / 2];
  if (!read_header(f, hdr)) {
    std::fclose(f);
    return BNA_CORRUPT_FILE;
  }
  const int L = hdr[24];
  const int bitpix = hdr[36];
  if ((long long)hdr[21] * hdr[22] * hdr[23] != total || L < 1 ||
      (bitpix != 32 && bitpix != 64)) {
    std::fclose(f);
    return BNA_CORRUPT_FILE;  // "Data type is neither float nor double" (CorMat.cpp:236-239)
  }
  *T_out = L;
  if (!bold_out) {  // size query
    std::fclose(f);
    return BNA_OK;
  }
  // one time point (one volume) at a time: the gather needs no full copy
  std::vector<double> vd(bitpix == 64 ? (size_t)total : 0);
  std::vector<float> vf(bitpix == 32 ? (size_t)total : 0);
  int32_t rc = BNA_OK;
  for (int l = 0; l < L && rc == BNA_OK; ++l) {
    const size_t got = bitpix == 64 ? std::fread(vd.data(), 8, (size_t)total, f)
                                    : std::fread(vf.data(), 4, (size_t)total, f);
    if (got != (size_t)total) {
      rc = BNA_CORRUPT_FILE;
      break;
    }
    long long i = 0;
    for (long long k = 0; k < total; ++k)
      if (sel[k]) {
        if (i >= N) {
          rc = BNA_BAD_ARG;  // the selection holds more voxels than N
          break;
        }
        bold_out[(size_t)l * N + i] = bitpix == 64 ? (float)vd[k] : vf[k];
        ++i;
      }
    if (rc == BNA_OK && i != N) rc = BNA_BAD_ARG;
  }
  std::fclose(f);
  return rc;
}

}  // extern "C"
