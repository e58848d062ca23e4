/* _beginthread on pthreads (oracle build of the reference's CPU tool). */
#ifndef BNA_REFSHIM_PROCESS_H
#define BNA_REFSHIM_PROCESS_H
#include <pthread.h>
#include <cstdint>
#include <new>

namespace bna_refshim {
struct start { void (*fn)(void*); void* arg; };
inline void* trampoline(void* p) {
  start s = *static_cast<start*>(p);
  delete static_cast<start*>(p);
  s.fn(s.arg);
  return nullptr;
}
}  // namespace bna_refshim

inline uintptr_t _beginthread(void (*fn)(void*), unsigned, void* arg) {
  pthread_t t;
  auto* s = new bna_refshim::start{fn, arg};
  if (pthread_create(&t, nullptr, bna_refshim::trampoline, s) != 0) {
    delete s;
    return (uintptr_t)-1;
  }
  return (uintptr_t)t;
}
#endif
