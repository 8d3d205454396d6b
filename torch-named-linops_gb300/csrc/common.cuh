// Shared helpers of the tlgb CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "tlgb.h"

namespace tlgb {

// Message of the last failing call on this host thread (see tlgb_last_error).
void set_error(const std::string& msg);

#define TLGB_FAIL(code, msg)      \
  do {                            \
    ::tlgb::set_error(msg);       \
    return (code);                \
  } while (0)

#define TLGB_CUDA(call)                                                              \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      ::tlgb::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));          \
      return TLGB_ERR_CUDA;                                                          \
    }                                                                                \
  } while (0)

#define TLGB_CHECK_LAUNCH()                                                          \
  do {                                                                               \
    cudaError_t e_ = cudaGetLastError();                                             \
    if (e_ != cudaSuccess) {                                                         \
      ::tlgb::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_));     \
      return TLGB_ERR_CUDA;                                                          \
    }                                                                                \
  } while (0)

#define TLGB_TRY(expr)          \
  do {                          \
    int s_ = (expr);            \
    if (s_ != TLGB_OK) return s_; \
  } while (0)

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Exclusive prefix sum of n uint32 values (in may alias out), deterministic;
// *total_dev (if given) receives the sum. Long inputs are scanned by many CTAs
// with scratch_len(n) uint32 of device scratch (not overlapping in/out);
// without scratch one CTA does it. Used while building plans.
int64_t scan_scratch_len(int64_t n);
int exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev, uint32_t* scratch,
                       cudaStream_t s);

// Stable LSD radix sort of (key, val) pairs by the low `bits` bits of key.
// keys/vals are sorted in place; keys_tmp/vals_tmp are ping-pong buffers of
// the same length; counts_tmp needs radix_counts_len(n) uint32 entries.
int64_t radix_counts_len(int64_t n);
int radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp, int32_t* vals_tmp,
                     uint32_t* counts_tmp, int64_t n, int bits, cudaStream_t s);

// Device status word of the convolution kernels (read and optionally cleared;
// synchronous). tlgb_device_status combines it with the interpolation one.
int conv_device_status(int* v, int clear);

// Streaming multiprocessors of the current device (cached per device).
int sm_count();

// Debug builds (-DTLGB_CHECKED, the library libtlgb_checked.so) range-check
// the index of selected global and shared-memory accesses: an index outside
// [0, n) sets this translation unit's checked-failure word to the source line
// (the first one wins) and the access is skipped. tlgb_device_status reports
// such a failure as bit 4. Release builds compile the checks away.
#ifdef TLGB_CHECKED
static __device__ int g_tlgb_checked_line;
static __device__ __forceinline__ bool checked_index(long long i, long long n, int line) {
  if (i >= 0 && i < n) return true;
  atomicCAS(&g_tlgb_checked_line, 0, line);
  return false;
}
#define TLGB_IN_RANGE(i, n) (::tlgb::checked_index((long long)(i), (long long)(n), __LINE__))
// this translation unit's failure word (0 = none), read and optionally cleared
static inline int checked_status(int* line, int clear) {
  TLGB_CUDA(cudaMemcpyFromSymbol(line, g_tlgb_checked_line, sizeof(int)));
  if (clear) {
    const int z = 0;
    TLGB_CUDA(cudaMemcpyToSymbol(g_tlgb_checked_line, &z, sizeof(int)));
  }
  return TLGB_OK;
}
#else
#define TLGB_IN_RANGE(i, n) true
static inline int checked_status(int* line, int) {
  *line = 0;
  return TLGB_OK;
}
#endif

// The blocks translation unit's checked-failure word (see above).
int blocks_checked_status(int* line, int clear);

}  // namespace tlgb
