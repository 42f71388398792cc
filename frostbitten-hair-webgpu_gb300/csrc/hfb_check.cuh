// Address checks of the self-checking build (HFB_DEVICE_CHECKS).
//
// HFB_G(p) wraps the address of every global-memory access of the kernels.
// In the normal build it is `p`.  In the self-checking build the host
// registers the byte range of every buffer a frame touches (hfb_debug_*
// entry points of that build only), and HFB_G(p) checks that the access
// lies inside one of them: if not, it counts the failure, records the first
// failing address and source line, and returns a pointer to a dummy block,
// so that the access lands there instead of faulting.  Each launch of that
// build is also followed by a stream synchronisation that names a failing
// kernel.
#pragma once

#include <cstdint>
#include <cstdio>

#include <cuda_runtime.h>

#ifndef HFB_TU
#define HFB_TU 0  // translation unit id recorded with a failure
#endif

namespace hfb {

#ifdef HFB_DEVICE_CHECKS
constexpr uint32_t CHECK_MAX_RANGES = 2048;  // sorted by lo, without overlaps
struct CheckState {
  uint32_t nRanges;
  uint32_t fails;
  uint32_t firstWhere;  // translation unit << 16 | line
  uint32_t pad;
  unsigned long long firstAddr;
  unsigned long long firstBytes;
  unsigned long long lo[CHECK_MAX_RANGES], hi[CHECK_MAX_RANGES];
  unsigned long long dummy[128];  // where a failed access goes
};
static __device__ CheckState* hfbCheck;  // one per translation unit, bound by the host

__device__ inline bool checkAddr(const void* p, uint32_t bytes, uint32_t where) {
  CheckState* s = hfbCheck;
  if (!s) return true;
  const unsigned long long a = (unsigned long long)p;
  uint32_t lo = 0, hi = s->nRanges;  // last range with lo <= a
  while (hi - lo > 1u) {
    const uint32_t mid = (lo + hi) >> 1;
    if (s->lo[mid] <= a) lo = mid; else hi = mid;
  }
  if (s->nRanges && a >= s->lo[lo] && a + bytes <= s->hi[lo]) return true;
  if (atomicAdd(&s->fails, 1u) == 0u) {
    s->firstWhere = where;
    s->firstAddr = a;
    s->firstBytes = bytes;
  }
  return false;
}

// a failed HFB_EXPECT condition: recorded like an address outside every range (address 0)
__device__ inline bool checkFail(uint32_t line) {
  CheckState* s = hfbCheck;
  if (s && atomicAdd(&s->fails, 1u) == 0u) {
    s->firstWhere = ((uint32_t)HFB_TU << 16) | line;
    s->firstAddr = 0ull;
    s->firstBytes = 0ull;
  }
  return false;
}

template <class T>
__device__ inline T* checked(T* p, uint32_t line) {
  static_assert(sizeof(T) <= sizeof(((CheckState*)nullptr)->dummy), "access wider than the dummy block");
  if (checkAddr((const void*)p, (uint32_t)sizeof(T), ((uint32_t)HFB_TU << 16) | line)) return p;
  return reinterpret_cast<T*>(hfbCheck->dummy);
}
#define HFB_G(p) ::hfb::checked((p), __LINE__)
#define HFB_EXPECT(cond) ((cond) ? true : ::hfb::checkFail(__LINE__))

// Host: binds this translation unit's hfbCheck to the context's state.
static inline cudaError_t checkBindTU(void* state) {
  static void* bound = nullptr;
  if (!state || bound == state) return cudaSuccess;
  cudaError_t e = cudaMemcpyToSymbol(hfbCheck, &state, sizeof(state));
  if (e == cudaSuccess) bound = state;
  return e;
}
#define HFB_CHECK_BIND(c)                                                \
  do {                                                                   \
    cudaError_t e_ = ::hfb::checkBindTU((c)->checkDev);                  \
    if (e_ != cudaSuccess) return e_;                                    \
  } while (0)
// every launch is waited for, and a failing kernel is named on stderr
#define HFB_AFTER_LAUNCH(c, name)                                                         \
  do {                                                                                    \
    cudaError_t e_ = cudaGetLastError();                                                  \
    if (e_ == cudaSuccess) e_ = cudaStreamSynchronize((c)->stream);                       \
    if (e_ != cudaSuccess) {                                                              \
      fprintf(stderr, "hairfb checked build: kernel %s: %s\n", name, cudaGetErrorString(e_)); \
      fflush(stderr);                                                                     \
      return e_;                                                                          \
    }                                                                                     \
  } while (0)
#else
#define HFB_G(p) (p)
#define HFB_EXPECT(cond) true
#define HFB_CHECK_BIND(c) do {} while (0)
#define HFB_AFTER_LAUNCH(c, name) do {} while (0)
#endif

}  // namespace hfb
