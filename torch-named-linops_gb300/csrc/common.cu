// Error reporting, version, and the plan-time scan / stable radix sort.

#include <string>

#include "common.cuh"

namespace tlgb {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

namespace {

constexpr int kScanThreads = 1024;

// Single-CTA exclusive scan: each thread scans a contiguous segment.
__global__ void __launch_bounds__(kScanThreads) scan_kernel(const uint32_t* in, uint32_t* out, int64_t n,
                                                             uint32_t* total) {
  __shared__ uint32_t part[kScanThreads];
  const int64_t per = (n + kScanThreads - 1) / kScanThreads;
  const int64_t b = threadIdx.x * per;
  const int64_t e = b + per < n ? b + per : n;
  uint32_t s = 0;
  for (int64_t i = b; i < e; ++i) s += in[i];
  part[threadIdx.x] = s;
  __syncthreads();
  // Hillis-Steele inclusive scan of the partials
  for (int off = 1; off < kScanThreads; off <<= 1) {
    uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (int64_t i = b; i < e; ++i) {
    const uint32_t v = in[i];
    out[i] = run;
    run += v;
  }
  if (threadIdx.x == kScanThreads - 1 && total) *total = part[kScanThreads - 1];
}

constexpr int kRadixBits = 8;
constexpr int kBuckets = 1 << kRadixBits;
constexpr int kRadixWarps = 4;
constexpr int kChunk = 32 * 64;  // entries per warp-chunk

// Per warp-chunk digit histogram, written digit-major: counts[d * nchunks + c].
__global__ void __launch_bounds__(32 * kRadixWarps) radix_hist_kernel(const uint32_t* keys, int64_t n, int shift,
                                                                      uint32_t* counts, int64_t nchunks) {
  __shared__ uint32_t hist[kRadixWarps][kBuckets];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t chunk = (int64_t)blockIdx.x * kRadixWarps + warp;
  for (int d = lane; d < kBuckets; d += 32) hist[warp][d] = 0;
  __syncwarp();
  if (chunk < nchunks) {
    const int64_t b = chunk * kChunk;
    const int64_t e = b + kChunk < n ? b + kChunk : n;
    for (int64_t i = b + lane; i < e; i += 32) atomicAdd(&hist[warp][(keys[i] >> shift) & (kBuckets - 1)], 1u);
    __syncwarp();
    for (int d = lane; d < kBuckets; d += 32) counts[(int64_t)d * nchunks + chunk] = hist[warp][d];
  }
}

// Stable scatter: each warp walks its chunk in order, 32 entries at a time;
// equal digits inside a round are ranked by lane (match_any), rounds in order.
__global__ void __launch_bounds__(32 * kRadixWarps) radix_scatter_kernel(const uint32_t* keys_in, const int32_t* vals_in,
                                                                         uint32_t* keys_out, int32_t* vals_out,
                                                                         int64_t n, int shift, const uint32_t* offs,
                                                                         int64_t nchunks) {
  __shared__ uint32_t run[kRadixWarps][kBuckets];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t chunk = (int64_t)blockIdx.x * kRadixWarps + warp;
  if (chunk >= nchunks) return;
  for (int d = lane; d < kBuckets; d += 32) run[warp][d] = offs[(int64_t)d * nchunks + chunk];
  __syncwarp();
  const int64_t b = chunk * kChunk;
  const int64_t e = b + kChunk < n ? b + kChunk : n;
  const unsigned lt = (1u << lane) - 1u;
  for (int64_t base = b; base < e; base += 32) {
    const int64_t i = base + lane;
    const bool valid = i < e;
    uint32_t key = 0;
    int32_t val = 0;
    int digit = kBuckets + lane;  // unique dummy for idle lanes
    if (valid) {
      key = keys_in[i];
      val = vals_in[i];
      digit = (key >> shift) & (kBuckets - 1);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const uint32_t rank = __popc(peers & lt);
    uint32_t pos = 0;
    if (valid) pos = run[warp][digit] + rank;
    __syncwarp();
    if (valid) {
      keys_out[pos] = key;
      vals_out[pos] = val;
      if (rank == 0) run[warp][digit] += __popc(peers);
    }
    __syncwarp();
  }
}

}  // namespace

int exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev, cudaStream_t s) {
  if (n <= 0) {
    if (total_dev) TLGB_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), s));
    return TLGB_OK;
  }
  scan_kernel<<<1, kScanThreads, 0, s>>>(in, out, n, total_dev);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

int64_t radix_counts_len(int64_t n) { return (int64_t)kBuckets * ((n + kChunk - 1) / kChunk) + 1; }

int radix_sort_pairs(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp, int32_t* vals_tmp, uint32_t* counts_tmp,
                     int64_t n, int bits, cudaStream_t s) {
  if (n <= 1) return TLGB_OK;
  const int64_t nchunks = (n + kChunk - 1) / kChunk;
  const unsigned grid = (unsigned)((nchunks + kRadixWarps - 1) / kRadixWarps);
  uint32_t* ka = keys;
  int32_t* va = vals;
  uint32_t* kb = keys_tmp;
  int32_t* vb = vals_tmp;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += kRadixBits, ++passes) {
    radix_hist_kernel<<<grid, 32 * kRadixWarps, 0, s>>>(ka, n, shift, counts_tmp, nchunks);
    TLGB_CHECK_LAUNCH();
    TLGB_TRY(exclusive_scan_u32(counts_tmp, counts_tmp, (int64_t)kBuckets * nchunks, nullptr, s));
    radix_scatter_kernel<<<grid, 32 * kRadixWarps, 0, s>>>(ka, va, kb, vb, n, shift, counts_tmp, nchunks);
    TLGB_CHECK_LAUNCH();
    uint32_t* tk = ka;
    ka = kb;
    kb = tk;
    int32_t* tv = va;
    va = vb;
    vb = tv;
  }
  if (passes & 1) {
    TLGB_CUDA(cudaMemcpyAsync(keys, ka, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    TLGB_CUDA(cudaMemcpyAsync(vals, va, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  }
  return TLGB_OK;
}

}  // namespace tlgb

extern "C" const char* tlgb_last_error(void) { return tlgb::g_last_error.c_str(); }

extern "C" int tlgb_version(void) { return 100; }
