// 3^3 convolution, 16 -> 16 channels, BF16 operands with FP32 accumulation, on
// the tensor cores: the layers of the learned CG preconditioner (no
// counterpart in the reference; it replaces nothing there).
//
// Layout: activations channels-last [D][H][W][16] bf16, zero padding 1, same
// spatial size in and out. Weights [27][16 out][16 in] bf16, tap t = (kd*3 +
// kh)*3 + kw. Forward and data-gradient are one implicit-GEMM kernel (the
// data gradient is the forward with flipped, transposed weights); the weight
// gradient is a second kernel with a fixed-order cross-CTA reduction.

#include <cuda_bf16.h>

#include <cstring>

#include "common.cuh"
#include "sm100.cuh"

namespace tlgb {
namespace {

constexpr int kTileW = 64;               // output voxels along W per CTA (4 warps x 16)
constexpr int kHaloW = kTileW + 2;       // input voxels along W per (kd, kh) row
constexpr int kHaloRows = 9;             // (kd, kh) rows
constexpr int kVoxBytes = 32;            // 16 bf16 channels
constexpr int kTaps = 27;

// 16-byte chunk c of row j in a 32-byte-row tile, XOR-swizzled so that the 8
// row addresses of one ldmatrix phase fall in distinct banks
__device__ __forceinline__ uint32_t swz(int j, int c) { return (uint32_t)(j * 32 + ((c ^ ((j >> 2) & 1)) << 4)); }

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
// D(16x8, f32) += A(16x16, bf16, row) * B(16x8, bf16, col)
__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// The 9 (kd, kh) input rows of kHaloW voxels around output row (d, h, w0..):
// zero outside the volume. Row r = kd*3 + kh, voxel j = input w0 - 1 + j.
__device__ __forceinline__ void load_halo(unsigned char* halo, const uint4* __restrict__ x, int D, int H, int W, int d,
                                          int h, int w0) {
  for (int i = threadIdx.x; i < kHaloRows * kHaloW * 2; i += blockDim.x) {
    const int c = i & 1;
    const int j = (i >> 1) % kHaloW;
    const int r = (i >> 1) / kHaloW;
    const int di = d + r / 3 - 1, hi = h + r % 3 - 1, wi = w0 - 1 + j;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (di >= 0 && di < D && hi >= 0 && hi < H && wi >= 0 && wi < W)
      v = __ldg(x + ((((long long)di * H + hi) * W + wi) * 2 + c));
    *reinterpret_cast<uint4*>(halo + r * kHaloW * kVoxBytes + swz(j, c)) = v;
  }
}

// ---- the tcgen05 path of the forward / data gradient
//
// Persistent CTAs of 4 warps. A work unit is a column segment of up to kTcRows
// output rows (fixed d, consecutive h) of 128 voxels along W (MMA M = 128)
// x 16 output channels (N = 16). Input rows (d + kd - 1, h') sit in a ring of
// 4 slots per kd; output row h reads rows h - 1, h, h + 1 of each kd, so
// after the first row each output row needs 3 new rows (6 TMA copies of 8
// channels x 130 voxels, zero fill outside the volume) instead of 9. Layout:
// the canonical no-swizzle K-major one, 16-byte rows, the two 8-channel
// halves of a row 2176 bytes apart; tap (kd, kh, kw) is the A operand kw rows
// into slot (h + kh - 1) mod 4 of kd, and the 27 taps are 27 MMAs of K = 16
// into one 128 x 16 FP32 TMEM accumulator. Two accumulators alternate, so
// the MMAs of row r overlap the epilogue of row r - 1. Weights stay in
// shared memory ([tap][k half][n group][8][16 B]) for the CTA's lifetime.
// Thread 0 issues copies and MMAs; every wait is bounded, and a timeout sets
// the status word and ends the CTA's work after freeing its TMEM.
constexpr int kTcM = 128;
constexpr int kTcHalo = kTcM + 2;
constexpr int kTcRows = 16;                               // output rows per work unit
constexpr int kTcHalfBytes = 2176;                       // >= 130 * 16, a multiple of 128
constexpr int kTcSlotBytes = 2 * kTcHalfBytes;
constexpr uint32_t kTcABytes = 3 * 4 * kTcSlotBytes;     // 3 kd x 4 ring slots
constexpr uint32_t kTcBBytes = kTaps * 512;              // 13824
constexpr uint32_t kTcCopyBytes = kTcHalo * 16;          // one 8-channel row copy
constexpr uint32_t kTcSmem = kTcABytes + kTcBBytes + 64;
constexpr uint32_t kTcCols = 32;                         // two 16-column accumulators
constexpr uint32_t kTcWait = 1u << 22;

__device__ int g_conv_status;

template <int MODE, bool OUTF32>
__global__ void __launch_bounds__(128) conv3d_tc_kernel(const __grid_constant__ CUtensorMap xmap, int D, int H, int W,
                                                        const uint4* __restrict__ wts,
                                                        const __nv_bfloat16* __restrict__ aux,
                                                        void* __restrict__ y) {
  using namespace sm100;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sa = smem;
  unsigned char* sb = smem + kTcABytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sb + kTcBBytes);  // [0,1] copies, [2,3] MMAs
  uint32_t* slot = reinterpret_cast<uint32_t*>(bars + 4);        // [0] TMEM address, [1] failure flag
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntw = (W + kTcM - 1) / kTcM, nseg = (H + kTcRows - 1) / kTcRows;
  const long long nunits = (long long)D * ntw * nseg;
  if (warp == 0) {
    tmem_alloc(slot, kTcCols);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) mbar_init(&bars[i], 1);
    fence_mbar_init();
    slot[1] = 0;
  }
  for (int i = tid; i < kTaps * 16 * 2; i += 128) {
    const int kh2 = i & 1, co = (i >> 1) & 15, t = i >> 5;
    *reinterpret_cast<uint4*>(sb + t * 512 + kh2 * 256 + (co >> 3) * 128 + (co & 7) * 16) = __ldg(wts + i);
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = slot[0];
  const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
  constexpr uint32_t idesc = idesc_bf16_f32(kTcM, 16);
  uint32_t lg = 0;     // copy groups issued (thread 0): group k arms bars[k & 1]
  uint32_t lw = 0;     // copy groups waited on (thread 0)
  uint32_t og = 0;     // output rows issued in this CTA: row k uses accumulator k & 1 and bars[2 + (k & 1)]
  bool fail = false;

  auto load_row = [&](int d, int hr, int w0) {  // the 3 kd rows (d + kd - 1, hr) into slot hr mod 4
    for (int kd = 0; kd < 3; ++kd)
      for (int hf = 0; hf < 2; ++hf)
        tma_load_4d(sa + (kd * 4 + (hr & 3)) * kTcSlotBytes + hf * kTcHalfBytes, &xmap, &bars[lg & 1], hf * 8, w0 - 1,
                    hr, d + kd - 1);
  };

  for (long long u = blockIdx.x; u < nunits && !fail; u += gridDim.x) {
    const int hs = (int)(u % nseg);
    const long long dw = u / nseg;
    const int wt = (int)(dw % ntw), d = (int)(dw / ntw);
    const int w0 = wt * kTcM, h0 = hs * kTcRows;
    const int R = min(kTcRows, H - h0);
    if (tid == 0) {
      mbar_arrive_expect_tx(&bars[lg & 1], 9 * 2 * kTcCopyBytes);
      for (int hr = h0 - 1; hr <= h0 + 1; ++hr) load_row(d, hr, w0);
      ++lg;
    }
    for (int r = 0; r <= R; ++r) {
      const int h = h0 + r;
      if (tid == 0 && r < R && !fail) {
        if (r + 1 < R) {
          // row h + 2 (for output h + 1) replaces row h - 2, last read by output h - 1
          if (r >= 1 && !mbar_wait_bounded(&bars[2 + ((og - 1) & 1)], ((og - 1) >> 1) & 1, kTcWait)) fail = true;
          mbar_arrive_expect_tx(&bars[lg & 1], 3 * 2 * kTcCopyBytes);
          load_row(d, h + 2, w0);
          ++lg;
        }
        if (!mbar_wait_bounded(&bars[lw & 1], (lw >> 1) & 1, kTcWait)) fail = true;
        ++lw;
        if (!fail) {
          tc_fence_after();
          const uint32_t acc = tmem + (og & 1) * 16;
          for (int t = 0; t < kTaps; ++t) {
            const int kd = t / 9, kh = (t / 3) % 3, kw = t % 3;
            const uint32_t aa = a0 + (kd * 4 + ((h + kh - 1) & 3)) * kTcSlotBytes + kw * 16;
            umma_bf16(acc, smem_desc(aa, kTcHalfBytes, 128), smem_desc(b0 + t * 512, 256, 128), idesc,
                      t > 0 ? 1u : 0u);
          }
          umma_commit(&bars[2 + (og & 1)]);
        }
        if (fail) slot[1] = 1;
      }
      if (r < R) ++og;
      if (r >= 1) {
        // epilogue of output h - 1 (accumulator (og - 2) & 1 after this row's increment)
        const uint32_t k = r < R ? og - 2 : og - 1;
        const bool done = mbar_wait_bounded(&bars[2 + (k & 1)], (k >> 1) & 1, kTcWait);
        if (!done) slot[1] = 1;
        if (__syncthreads_and(done)) {
          tc_fence_after();
          float v[16];
          tmem_ld16(tmem + (k & 1) * 16 + ((uint32_t)(warp * 32) << 16), v);
          const int w = w0 + warp * 32 + lane;
          if (w < W) {
            const long long vox = ((long long)d * H + (h - 1)) * W + w;
            if (MODE == 1) {
#pragma unroll
              for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.f);
            } else if (MODE == 2) {
              const uint4* m4 = reinterpret_cast<const uint4*>(aux + vox * 16);
              uint4 mm[2] = {__ldg(m4), __ldg(m4 + 1)};
              const __nv_bfloat16* mb = reinterpret_cast<const __nv_bfloat16*>(mm);
#pragma unroll
              for (int i = 0; i < 16; ++i) v[i] = __bfloat162float(mb[i]) > 0.f ? v[i] : 0.f;
            }
            if (OUTF32) {
              float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(y) + vox * 16);
#pragma unroll
              for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            } else {
              uint4 pk[2];
              __nv_bfloat162* pb = reinterpret_cast<__nv_bfloat162*>(pk);
#pragma unroll
              for (int i = 0; i < 8; ++i) pb[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
              uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(y) + vox * 16);
              o[0] = pk[0];
              o[1] = pk[1];
            }
          }
        }
      }
      tc_fence_before();
      __syncthreads();
      if (slot[1]) {
        fail = true;
        break;
      }
    }
  }
  if (fail && tid == 0) atomicExch(&g_conv_status, 2);
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTcCols);
}

// Weight gradient: dW[t][co][ci] = sum over output voxels v of gy[v][co] *
// x[v + offset(t)][ci]. CTA b takes output rows b, b + grid, ... (fixed), warp
// w the taps w, w + 4, ...; partial sums per CTA are reduced in CTA order.
constexpr int kWgTapsPerWarp = 7;

__global__ void __launch_bounds__(128) conv3d_wgrad_kernel(int D, int H, int W, const uint4* __restrict__ x,
                                                           const uint4* __restrict__ gy, float* __restrict__ partial) {
  __shared__ __align__(128) unsigned char halo[kHaloRows * kHaloW * kVoxBytes];
  __shared__ __align__(128) unsigned char gsm[kTileW * kVoxBytes];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ntw = (W + kTileW - 1) / kTileW;
  const long long nrows = (long long)D * H * ntw;
  float acc[kWgTapsPerWarp][2][4];
#pragma unroll
  for (int i = 0; i < kWgTapsPerWarp; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  // ldmatrix.trans roles. A = gy^T (16 out x 16 voxels) from gsm [voxel][co]:
  // matrix q holds voxels 8*(q >> 1).., channels 8*(q & 1)..
  const int ga_row = (lane & 7) + 8 * (lane >> 4), ga_chunk = (lane >> 3) & 1;
  // B = x (16 voxels x 8 in) from the halo [voxel][ci]: matrix q holds
  // voxels 8*(q & 1).., channels 8*(q >> 1)..
  const int xb_row = (lane & 7) + 8 * ((lane >> 3) & 1), xb_chunk = lane >> 4;
  const uint32_t hbase = smem_addr(halo), gbase = smem_addr(gsm);
  for (long long row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int wt = (int)(row % ntw);
    const long long dh = row / ntw;
    const int h = (int)(dh % H), d = (int)(dh / H);
    const int w0 = wt * kTileW;
    __syncthreads();  // the previous row's tiles have been read
    load_halo(halo, x, D, H, W, d, h, w0);
    for (int i = threadIdx.x; i < kTileW * 2; i += blockDim.x) {
      const int c = i & 1, j = i >> 1;
      const int w = w0 + j;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (w < W) v = __ldg(gy + ((((long long)d * H + h) * W + w) * 2 + c));
      *reinterpret_cast<uint4*>(gsm + swz(j, c)) = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int ks = 0; ks < kTileW / 16; ++ks) {
      uint32_t a0, a1, a2, a3;
      ldsm_x4_t(gbase + swz(ks * 16 + ga_row, ga_chunk), a0, a1, a2, a3);
      // A fragment order: (co 0-7, v 0-7), (co 8-15, v 0-7), (co 0-7, v 8-15), (co 8-15, v 8-15)
      // = stored blocks (v lo, c lo), (v lo, c hi), (v hi, c lo), (v hi, c hi): a0, a1, a2, a3
#pragma unroll
      for (int i = 0; i < kWgTapsPerWarp; ++i) {
        const int t = warp + 4 * i;
        if (t < kTaps) {
          const int r = t / 3, kw = t % 3;
          uint32_t b0, b1, b2, b3;
          ldsm_x4_t(hbase + r * kHaloW * kVoxBytes + swz(ks * 16 + kw + xb_row, xb_chunk), b0, b1, b2, b3);
          // b0: (v lo, ci lo), b1: (v hi, ci lo), b2: (v lo, ci hi), b3: (v hi, ci hi)
          mma_bf16(acc[i][0], a0, a1, a2, a3, b0, b1);
          mma_bf16(acc[i][1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
  const int gid = lane >> 2, tig = lane & 3;
  float* dst = partial + (long long)blockIdx.x * kTaps * 256;
#pragma unroll
  for (int i = 0; i < kWgTapsPerWarp; ++i) {
    const int t = warp + 4 * i;
    if (t >= kTaps) continue;
#pragma unroll
    for (int ch = 0; ch < 2; ++ch)
#pragma unroll
      for (int hr = 0; hr < 2; ++hr) {
        const int co = gid + 8 * hr, ci = ch * 8 + 2 * tig;
        *reinterpret_cast<float2*>(dst + t * 256 + co * 16 + ci) = make_float2(acc[i][ch][2 * hr], acc[i][ch][2 * hr + 1]);
      }
  }
}

__global__ void wgrad_reduce_kernel(const float* __restrict__ partial, int nparts, float* __restrict__ dw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kTaps * 256) return;
  float s = 0.f;
  for (int b = 0; b < nparts; ++b) s += partial[(long long)b * kTaps * 256 + i];
  dw[i] = s;
}

// complex64 [V] * scale -> bf16 [V][16]: channels 0, 1 = re, im rounded to
// bf16; with hilo, channels 2, 3 = the rounding remainders (a two-term bf16
// split carrying 16 mantissa bits); the rest 0
__global__ void pack_c64_kernel(const float2* __restrict__ z, long long nvox, const float* __restrict__ scale,
                                int hilo, uint4* __restrict__ out) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvox) return;
  const float s = scale ? *scale : 1.f;
  const float2 a = z[v];
  const float re = a.x * s, im = a.y * s;
  const __nv_bfloat162 p = __floats2bfloat162_rn(re, im);
  uint32_t q = 0u;
  if (hilo) {
    const __nv_bfloat162 r = __floats2bfloat162_rn(re - __bfloat162float(p.x), im - __bfloat162float(p.y));
    q = *reinterpret_cast<const uint32_t*>(&r);
  }
  out[2 * v] = make_uint4(*reinterpret_cast<const uint32_t*>(&p), q, 0u, 0u);
  out[2 * v + 1] = make_uint4(0u, 0u, 0u, 0u);
}

// float32 [V][16] channels 0, 1 -> complex64 [V]: out = scale * y + skip * z
__global__ void unpack_c64_kernel(const float* __restrict__ y, const float2* __restrict__ z, long long nvox,
                                  const float* __restrict__ scale, float skip, float2* __restrict__ out) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvox) return;
  const float s = scale ? *scale : 1.f;
  const float2 a = *reinterpret_cast<const float2*>(y + v * 16);
  float2 r = make_float2(a.x * s, a.y * s);
  if (z) {
    const float2 b = z[v];
    r.x = fmaf(skip, b.x, r.x);
    r.y = fmaf(skip, b.y, r.y);
  }
  out[v] = r;
}

int check_conv(const tlgb_conv3d_desc* d) {
  if (!d) TLGB_FAIL(TLGB_ERR_INVALID, "null conv descriptor");
  if (d->D < 1 || d->H < 1 || d->W < 1) TLGB_FAIL(TLGB_ERR_INVALID, "conv3d: spatial sizes must be >= 1");
  if (d->H > 65535 || d->D > 65535) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "conv3d: D and H must be <= 65535");
  if (d->cin != 16 || d->cout != 16) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "conv3d: 16 input and 16 output channels (pad)");
  if (d->mode < 0 || d->mode > 2) TLGB_FAIL(TLGB_ERR_INVALID, "conv3d: unknown epilogue mode");
  return TLGB_OK;
}

// 4D tensor map over an activation [D][H][W][16] bf16 for 8-channel x 130-voxel boxes
bool conv_tensor_map(const tlgb_conv3d_desc* d, const void* x, CUtensorMap* map) {
  auto enc = sm100::tensor_map_encoder();
  if (!enc || ((uintptr_t)x & 15)) return false;
  memset(map, 0, sizeof(*map));
  const cuuint64_t dims[4] = {16, (cuuint64_t)d->W, (cuuint64_t)d->H, (cuuint64_t)d->D};
  const cuuint64_t strides[3] = {32, (cuuint64_t)d->W * 32, (cuuint64_t)d->W * d->H * 32};
  const cuuint32_t box[4] = {8, (cuuint32_t)kTcHalo, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int MODE, bool OUTF32>
int launch_conv_tc(const tlgb_conv3d_desc* d, const CUtensorMap& map, const void* w, const void* aux, void* y,
                   cudaStream_t s) {
  auto* k = conv3d_tc_kernel<MODE, OUTF32>;
  TLGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
  const long long units = (long long)d->D * ((d->W + kTcM - 1) / kTcM) * ((d->H + kTcRows - 1) / kTcRows);
  const unsigned grid = (unsigned)std::min<long long>(units, 3ll * sm_count());  // 3 CTAs of 66 KB per SM
  k<<<grid, 128, kTcSmem, s>>>(map, d->D, d->H, d->W, (const uint4*)w, (const __nv_bfloat16*)aux, y);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

int wgrad_parts(const tlgb_conv3d_desc* d) {
  const long long rows = (long long)d->D * d->H * ((d->W + kTileW - 1) / kTileW);
  return (int)std::min<long long>(rows, 4 * 152);
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_conv3d_fwd(const tlgb_conv3d_desc* d, const void* x, const void* w, const void* aux, void* y,
                               tlgb_stream_t stream) {
  TLGB_TRY(check_conv(d));
  if (!x || !w || !y || (d->mode == 2 && !aux)) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  if (((uintptr_t)x | (uintptr_t)w | (uintptr_t)y | (uintptr_t)aux) & 15)
    TLGB_FAIL(TLGB_ERR_INVALID, "conv3d: buffers must be 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  CUtensorMap map;
  if (conv_tensor_map(d, x, &map)) {
    if (d->out_f32) {
      if (d->mode == 0) return launch_conv_tc<0, true>(d, map, w, aux, y, s);
      if (d->mode == 1) return launch_conv_tc<1, true>(d, map, w, aux, y, s);
      return launch_conv_tc<2, true>(d, map, w, aux, y, s);
    }
    if (d->mode == 0) return launch_conv_tc<0, false>(d, map, w, aux, y, s);
    if (d->mode == 1) return launch_conv_tc<1, false>(d, map, w, aux, y, s);
    return launch_conv_tc<2, false>(d, map, w, aux, y, s);
  }
  TLGB_FAIL(TLGB_ERR_UNSUPPORTED,
            "conv3d: the driver offers no tensor-map encoder, which the TMA-fed tcgen05 kernel needs");
}

extern "C" int tlgb_conv3d_wgrad_scratch_size(const tlgb_conv3d_desc* d, size_t* bytes) {
  TLGB_TRY(check_conv(d));
  if (!bytes) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  *bytes = (size_t)wgrad_parts(d) * kTaps * 256 * sizeof(float);
  return TLGB_OK;
}

extern "C" int tlgb_conv3d_wgrad(const tlgb_conv3d_desc* d, const void* x, const void* gy, float* dw, void* scratch,
                                 size_t scratch_bytes, tlgb_stream_t stream) {
  TLGB_TRY(check_conv(d));
  if (!x || !gy || !dw || !scratch) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  if (((uintptr_t)x | (uintptr_t)gy | (uintptr_t)scratch) & 15)
    TLGB_FAIL(TLGB_ERR_INVALID, "conv3d: buffers must be 16-byte aligned");
  size_t need = 0;
  TLGB_TRY(tlgb_conv3d_wgrad_scratch_size(d, &need));
  if (scratch_bytes < need) TLGB_FAIL(TLGB_ERR_WORKSPACE, "conv3d wgrad scratch too small");
  cudaStream_t s = (cudaStream_t)stream;
  const int parts = wgrad_parts(d);
  conv3d_wgrad_kernel<<<parts, 128, 0, s>>>(d->D, d->H, d->W, (const uint4*)x, (const uint4*)gy, (float*)scratch);
  TLGB_CHECK_LAUNCH();
  wgrad_reduce_kernel<<<(kTaps * 256 + 255) / 256, 256, 0, s>>>((const float*)scratch, parts, dw);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_conv3d_pack(const void* z, int64_t nvox, const float* scale, int32_t hilo, void* out,
                                tlgb_stream_t stream) {
  if (nvox < 0 || (nvox > 0 && (!z || !out))) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer or negative size");
  if (nvox == 0) return TLGB_OK;
  if ((uintptr_t)out & 15) TLGB_FAIL(TLGB_ERR_INVALID, "pack: output must be 16-byte aligned");
  pack_c64_kernel<<<(unsigned)cdiv(nvox, 256), 256, 0, (cudaStream_t)stream>>>((const float2*)z, nvox, scale, hilo,
                                                                               (uint4*)out);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_conv3d_unpack(const float* y, const void* z, int64_t nvox, const float* scale, float skip,
                                  void* out, tlgb_stream_t stream) {
  if (nvox < 0 || (nvox > 0 && (!y || !out))) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer or negative size");
  if (nvox == 0) return TLGB_OK;
  unpack_c64_kernel<<<(unsigned)cdiv(nvox, 256), 256, 0, (cudaStream_t)stream>>>(y, (const float2*)z, nvox, scale,
                                                                                 skip, (float2*)out);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

namespace tlgb {
int conv_device_status(int* v, int clear) {
  int x = 0;
  TLGB_CUDA(cudaMemcpyFromSymbol(&x, g_conv_status, sizeof(int)));
  if (clear) {
    const int z = 0;
    TLGB_CUDA(cudaMemcpyToSymbol(g_conv_status, &z, sizeof(int)));
  }
  *v = x;
  return TLGB_OK;
}
}  // namespace tlgb
