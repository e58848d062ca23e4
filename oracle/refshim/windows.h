/* Linux stand-ins for the Win32 thread and system-info calls of the
 * reference's multi-threaded CPU correlation (oracle build only). */
#ifndef BNA_REFSHIM_WINDOWS_H
#define BNA_REFSHIM_WINDOWS_H
#include <pthread.h>
#include <unistd.h>
#include <cstdint>
#include "shlwapi.h"

typedef void* HANDLE;
#define INFINITE 0xFFFFFFFFu
struct SYSTEM_INFO { unsigned long dwNumberOfProcessors; };
inline void GetSystemInfo(SYSTEM_INFO* s) {
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  s->dwNumberOfProcessors = n > 0 ? (unsigned long)n : 1ul;
}
inline unsigned long WaitForSingleObject(HANDLE h, unsigned long) {
  pthread_join((pthread_t)(uintptr_t)h, nullptr);
  return 0;
}
#endif
