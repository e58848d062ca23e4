/* Linux stand-ins for the few Win32 calls the reference's CPU sources make
 * outside the computation (directory checks, itoa, sprintf_s).  Oracle build
 * only: lets the reference's own CorMat.cpp / CorMat_CPU.cpp compile with g++
 * so its CPU functions can be called from tests. */
#ifndef BNA_REFSHIM_SHLWAPI_H
#define BNA_REFSHIM_SHLWAPI_H
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <sys/stat.h>
#include <sys/types.h>

inline bool PathIsDirectory(const char* p) {
  struct stat s;
  return stat(p, &s) == 0 && S_ISDIR(s.st_mode);
}
inline int CreateDirectory(const char* p, void*) { return mkdir(p, 0755) == 0; }
inline char* itoa(int v, char* buf, int base) {
  if (base == 10) std::sprintf(buf, "%d", v);
  else std::sprintf(buf, "%x", v);
  return buf;
}
template <size_t N>
inline int sprintf_s(char (&buf)[N], const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int r = std::vsnprintf(buf, N, fmt, ap);
  va_end(ap);
  return r;
}
#endif
