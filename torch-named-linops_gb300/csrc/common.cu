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

// Multi-CTA exclusive scan for long inputs: per-block sums, a scan of the
// sums (scan_kernel, one CTA), then each block's scan plus its offset.
constexpr int kScanBlock = 4096;  // elements per CTA (256 threads x 16)

__device__ __forceinline__ uint32_t block_sum_256(uint32_t v) {
  __shared__ uint32_t ws[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t t = 0;
  if (threadIdx.x < 8) t = ws[threadIdx.x];
  if (threadIdx.x < 32) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

__global__ void __launch_bounds__(256) scan_block_sums_kernel(const uint32_t* __restrict__ in, int64_t n,
                                                              uint32_t* __restrict__ sums) {
  const int64_t b0 = (int64_t)blockIdx.x * kScanBlock;
  uint32_t s = 0;
  for (int i = threadIdx.x; i < kScanBlock; i += 256) {
    const int64_t k = b0 + i;
    if (k < n) s += in[k];
  }
  s = block_sum_256(s);
  if (threadIdx.x == 0) sums[blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) scan_blocks_kernel(const uint32_t* in, uint32_t* out, int64_t n,
                                                          const uint32_t* __restrict__ offsets) {
  __shared__ uint32_t tile[kScanBlock];
  __shared__ uint32_t wsum[8];
  const int64_t b0 = (int64_t)blockIdx.x * kScanBlock;
  for (int i = threadIdx.x; i < kScanBlock; i += 256) {
    const int64_t k = b0 + i;
    tile[i] = k < n ? in[k] : 0u;
  }
  __syncthreads();
  // each thread scans its 16 consecutive elements
  uint32_t loc[16], run = 0;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    loc[j] = run;
    run += tile[threadIdx.x * 16 + j];
  }
  // exclusive scan of the thread totals: warp shuffles, then warp totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  uint32_t wbase = 0;
  for (int w = 0; w < warp; ++w) wbase += wsum[w];
  const uint32_t base = offsets[blockIdx.x] + wbase + x - run;
  __syncthreads();  // every thread has read its inputs from the tile
#pragma unroll
  for (int j = 0; j < 16; ++j) tile[threadIdx.x * 16 + j] = base + loc[j];
  __syncthreads();
  for (int i = threadIdx.x; i < kScanBlock; i += 256) {
    const int64_t k = b0 + i;
    if (k < n) out[k] = tile[i];
  }
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

int64_t scan_scratch_len(int64_t n) { return (n + kScanBlock - 1) / kScanBlock + 1; }

int exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev, uint32_t* scratch,
                       cudaStream_t s) {
  if (n <= 0) {
    if (total_dev) TLGB_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), s));
    return TLGB_OK;
  }
  if (!scratch || n <= 4 * kScanBlock) {
    scan_kernel<<<1, kScanThreads, 0, s>>>(in, out, n, total_dev);
    TLGB_CHECK_LAUNCH();
    return TLGB_OK;
  }
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  scan_block_sums_kernel<<<(unsigned)nb, 256, 0, s>>>(in, n, scratch);
  TLGB_CHECK_LAUNCH();
  scan_kernel<<<1, kScanThreads, 0, s>>>(scratch, scratch, nb, total_dev);
  TLGB_CHECK_LAUNCH();
  scan_blocks_kernel<<<(unsigned)nb, 256, 0, s>>>(in, out, n, scratch);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

static int64_t radix_counts_only(int64_t n) { return (int64_t)kBuckets * ((n + kChunk - 1) / kChunk); }

int64_t radix_counts_len(int64_t n) {
  const int64_t c = radix_counts_only(n);
  return c + 1 + scan_scratch_len(c);
}

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
    TLGB_TRY(exclusive_scan_u32(counts_tmp, counts_tmp, (int64_t)kBuckets * nchunks, nullptr,
                                counts_tmp + radix_counts_only(n) + 1, s));
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

int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (cache[dev] == 0) {
    int n = 0;
    cache[dev] = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0 ? n : 152;
  }
  return cache[dev];
}

}  // namespace tlgb

extern "C" const char* tlgb_last_error(void) { return tlgb::g_last_error.c_str(); }

extern "C" int tlgb_version(void) { return 100; }
