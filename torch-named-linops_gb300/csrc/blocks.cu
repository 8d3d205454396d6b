// ArrayToBlocks / BlocksToArray (unfold / fold) for sm_103a.
//
// Replaces the reference's Triton _unfold{1,2,3}d / _fold{1,2,3}d
// (functional/_unfold/unfold.py:166-522, fold.py:151-475). Arrays of 1 or 2
// spatial dims run through the same kernels as 3D ones with leading extents
// of 1. Layouts: array [nbatch, im0, im1, im2], blocks [nbatch, nb0, nb1, nb2,
// B0, B1, B2] (or [..., nb2, nnz] with a mask).
//
// unfold: one CTA per (batch, b0, b1) "slab" whose output is one contiguous
//   run of nb2 * prod(B) elements; copied in 16/8/4-byte units chosen from the
//   alignment of every stride, so the stores are fully coalesced vectors.
// fold: output-stationary. Each thread owns one array element and sums its
//   covering block entries in ascending (b0, b1, b2) order starting from zero
//   -- the reference's own order (fold.py:436-474, _fold_torch :508-516) -- so
//   results are deterministic and equal to the reference bit for bit.

#include "common.cuh"

#include <type_traits>

namespace tlgb {
namespace {

// q = n / d for 0 <= n < 2^31 (multiply-shift with a 33-bit magic number).
struct FastDiv {
  uint32_t d;
  uint32_t shift;
  unsigned long long mul;
};

FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  uint32_t s = 0;
  while ((1ull << s) < d) ++s;
  f.shift = s;
  f.mul = ((1ull << (32 + s)) + d - 1) / d;
  return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  return (uint32_t)(((unsigned long long)n * f.mul) >> (32 + f.shift));
}

struct BlkGeo {
  int64_t im[3];
  int64_t B[3];
  int64_t s[3];
  int64_t nb[3];
  int64_t nbatch;
  int64_t nnz;
};

template <typename U>
__global__ void __launch_bounds__(256) unfold_rows_kernel(const U* __restrict__ in, U* __restrict__ out,
                                                          BlkGeo g, int64_t bu2, int64_t s2u, int64_t im2u,
                                                          FastDiv div_bu2, FastDiv div_B1, FastDiv div_B0,
                                                          uint32_t slab_units) {
  // slab = (n, b0, b1); output of a slab is contiguous
  const int64_t slab = blockIdx.x;
  const int64_t b1 = slab % g.nb[1];
  const int64_t t = slab / g.nb[1];
  const int64_t b0 = t % g.nb[0];
  const int64_t n = t / g.nb[0];
  const int64_t row_in = g.im[1] * im2u;                 // units per x1 row of the array
  const int64_t plane_in = g.im[0] * row_in;             // units per batch entry
  const U* src = in + n * plane_in + (b0 * g.s[0]) * row_in + (b1 * g.s[1]) * im2u;
  U* dst = out + (int64_t)slab * slab_units;
  for (uint32_t u = threadIdx.x; u < slab_units; u += blockDim.x) {
    const uint32_t row = fdiv(u, div_bu2);
    const uint32_t i2 = u - row * (uint32_t)bu2;
    const uint32_t r1 = fdiv(row, div_B1);
    const uint32_t i1 = row - r1 * (uint32_t)g.B[1];
    const uint32_t b2 = fdiv(r1, div_B0);
    const uint32_t i0 = r1 - b2 * (uint32_t)g.B[0];
    const int64_t off = (int64_t)i0 * row_in + (int64_t)i1 * im2u + (int64_t)b2 * s2u + i2;
    if (TLGB_IN_RANGE((src - in) + off, g.nbatch * plane_in)) dst[u] = __ldg(src + off);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) unfold_masked_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                            BlkGeo g, const int32_t* __restrict__ mask_idx,
                                                            FastDiv div_nnz, FastDiv div_B2, FastDiv div_B1,
                                                            uint32_t slab_elems) {
  const int64_t slab = blockIdx.x;
  const int64_t b1 = slab % g.nb[1];
  const int64_t t = slab / g.nb[1];
  const int64_t b0 = t % g.nb[0];
  const int64_t n = t / g.nb[0];
  const int64_t row_in = g.im[1] * g.im[2];
  const T* src = in + n * g.im[0] * row_in + (b0 * g.s[0]) * row_in + (b1 * g.s[1]) * g.im[2];
  T* dst = out + slab * (int64_t)slab_elems;
  for (uint32_t u = threadIdx.x; u < slab_elems; u += blockDim.x) {
    const uint32_t b2 = fdiv(u, div_nnz);
    const uint32_t j = u - b2 * (uint32_t)g.nnz;
    const uint32_t k = (uint32_t)__ldg(mask_idx + j);
    const uint32_t k01 = fdiv(k, div_B2);
    const uint32_t i2 = k - k01 * (uint32_t)g.B[2];
    const uint32_t i0 = fdiv(k01, div_B1);
    const uint32_t i1 = k01 - i0 * (uint32_t)g.B[1];
    const int64_t off = (int64_t)i0 * row_in + (int64_t)i1 * g.im[2] + (int64_t)b2 * g.s[2] + i2;
    if (TLGB_IN_RANGE((src - in) + off, g.nbatch * g.im[0] * row_in)) dst[u] = __ldg(src + off);
  }
}

template <typename T>
struct Acc;
template <>
struct Acc<float> {
  __device__ static float zero() { return 0.f; }
  __device__ static void add(float& a, float b) { a = __fadd_rn(a, b); }
};
template <>
struct Acc<double> {
  __device__ static double zero() { return 0.0; }
  __device__ static void add(double& a, double b) { a = __dadd_rn(a, b); }
};
template <>
struct Acc<float2> {
  __device__ static float2 zero() { return make_float2(0.f, 0.f); }
  __device__ static void add(float2& a, float2 b) {
    a.x = __fadd_rn(a.x, b.x);
    a.y = __fadd_rn(a.y, b.y);
  }
};
template <>
struct Acc<double2> {
  __device__ static double2 zero() { return make_double2(0.0, 0.0); }
  __device__ static void add(double2& a, double2 b) {
    a.x = __dadd_rn(a.x, b.x);
    a.y = __dadd_rn(a.y, b.y);
  }
};

// first / last block index covering array coordinate x along one dim
__device__ __forceinline__ void cover(int64_t x, int64_t B, int64_t s, int64_t nb, const FastDiv& ds,
                                      int64_t& lo, int64_t& hi) {
  const int64_t a = x - B + 1;  // first block start that still covers x
  lo = a > 0 ? (int64_t)fdiv((uint32_t)(a + s - 1), ds) : 0;
  hi = (int64_t)fdiv((uint32_t)x, ds);
  if (hi > nb - 1) hi = nb - 1;
}

template <typename T, bool MASKED>
__global__ void __launch_bounds__(256) fold_kernel(const T* __restrict__ in, T* __restrict__ out, BlkGeo g,
                                                   const int32_t* __restrict__ mask_inv, FastDiv div_im2,
                                                   FastDiv ds0, FastDiv ds1, FastDiv ds2) {
  // one CTA per (n, x0) plane of the output
  const int64_t plane = blockIdx.x;
  const int64_t x0 = plane % g.im[0];
  const int64_t n = plane / g.im[0];
  const int64_t bvol = MASKED ? g.nnz : g.B[0] * g.B[1] * g.B[2];
  const int64_t full_bvol = g.B[0] * g.B[1] * g.B[2];
  const int64_t nbl = g.nb[0] * g.nb[1] * g.nb[2];
  const T* src = in + n * nbl * bvol;
  T* dst = out + plane * (g.im[1] * g.im[2]);
  const uint32_t plane_elems = (uint32_t)(g.im[1] * g.im[2]);
  int64_t lo0, hi0;
  cover(x0, g.B[0], g.s[0], g.nb[0], ds0, lo0, hi0);
  for (uint32_t u = threadIdx.x; u < plane_elems; u += blockDim.x) {
    const uint32_t x1 = fdiv(u, div_im2);
    const uint32_t x2 = u - x1 * (uint32_t)g.im[2];
    int64_t lo1, hi1, lo2, hi2;
    cover(x1, g.B[1], g.s[1], g.nb[1], ds1, lo1, hi1);
    cover(x2, g.B[2], g.s[2], g.nb[2], ds2, lo2, hi2);
    T acc = Acc<T>::zero();
    for (int64_t b0 = lo0; b0 <= hi0; ++b0) {
      const int64_t i0 = x0 - b0 * g.s[0];
      for (int64_t b1 = lo1; b1 <= hi1; ++b1) {
        const int64_t i1 = x1 - b1 * g.s[1];
        const int64_t blk01 = (b0 * g.nb[1] + b1) * g.nb[2];
        for (int64_t b2 = lo2; b2 <= hi2; ++b2) {
          const int64_t i2 = x2 - b2 * g.s[2];
          const int64_t k = (i0 * g.B[1] + i1) * g.B[2] + i2;
          int64_t j = k;
          if (MASKED) {
            j = __ldg(mask_inv + k);
            if (j < 0) continue;
          }
          (void)full_bvol;
          if (TLGB_IN_RANGE((blk01 + b2) * bvol + j, nbl * bvol)) Acc<T>::add(acc, __ldg(src + (blk01 + b2) * bvol + j));
        }
      }
    }
    dst[u] = acc;
  }
}

// Fold of adjacent element pairs along the innermost dimension. When the
// innermost block size and stride are both even (and the extent is even),
// elements 2h and 2h + 1 are covered by the same blocks and sit next to each
// other in every block, so one 2-element load per covering block serves both;
// offsets inside one batch entry fit in 32 bits (checked by the caller). Each
// element still sums its covering block entries in ascending block order,
// starting from 0: the same float additions as fold_kernel.
template <typename E, typename V>
__global__ void __launch_bounds__(256) fold_pairs_kernel(const E* __restrict__ in, E* __restrict__ out, BlkGeo g,
                                                         FastDiv div_half2, FastDiv ds0, FastDiv ds1, FastDiv ds2) {
  static_assert(sizeof(V) == 2 * sizeof(E), "a pair of elements");
  const int64_t plane = blockIdx.x;  // (n, x0)
  const int64_t x0 = plane % g.im[0];
  const int64_t n = plane / g.im[0];
  const uint32_t B1 = (uint32_t)g.B[1], B2 = (uint32_t)g.B[2], s0 = (uint32_t)g.s[0], s1 = (uint32_t)g.s[1],
                 s2 = (uint32_t)g.s[2], nb1 = (uint32_t)g.nb[1], nb2 = (uint32_t)g.nb[2];
  const uint32_t bvol = (uint32_t)(g.B[0] * g.B[1] * g.B[2]);
  const E* src = in + n * (g.nb[0] * g.nb[1] * g.nb[2]) * (int64_t)bvol;
  E* dst = out + plane * (g.im[1] * g.im[2]);
  const uint32_t half2 = (uint32_t)(g.im[2] / 2), tasks = (uint32_t)g.im[1] * half2;
  int64_t lo0, hi0;
  cover(x0, g.B[0], g.s[0], g.nb[0], ds0, lo0, hi0);
  for (uint32_t t = threadIdx.x; t < tasks; t += blockDim.x) {
    const uint32_t x1 = fdiv(t, div_half2);
    const uint32_t x2 = 2 * (t - x1 * half2);
    int64_t lo1, hi1, lo2, hi2;
    cover(x1, g.B[1], g.s[1], g.nb[1], ds1, lo1, hi1);
    cover(x2, g.B[2], g.s[2], g.nb[2], ds2, lo2, hi2);
    E a0 = Acc<E>::zero(), a1 = Acc<E>::zero();
    for (uint32_t b0 = (uint32_t)lo0; b0 <= (uint32_t)hi0 && lo0 <= hi0; ++b0) {
      const uint32_t i0 = (uint32_t)x0 - b0 * s0;
      for (uint32_t b1 = (uint32_t)lo1; (int64_t)b1 <= hi1; ++b1) {
        const uint32_t i1 = x1 - b1 * s1;
        const uint32_t blk01 = (b0 * nb1 + b1) * nb2;
        const uint32_t k01 = (i0 * B1 + i1) * B2;
        for (uint32_t b2 = (uint32_t)lo2; (int64_t)b2 <= hi2; ++b2) {
          const uint32_t off = (blk01 + b2) * bvol + k01 + (x2 - b2 * s2);
          const V v = __ldg(reinterpret_cast<const V*>(src + off));
          const E* e = reinterpret_cast<const E*>(&v);
          Acc<E>::add(a0, e[0]);
          Acc<E>::add(a1, e[1]);
        }
      }
    }
    V r;
    E* re = reinterpret_cast<E*>(&r);
    re[0] = a0;
    re[1] = a1;
    *reinterpret_cast<V*>(dst + (int64_t)x1 * g.im[2] + x2) = r;
  }
}

int check_desc(const tlgb_blocks_desc* d, BlkGeo& g, int& esize) {
  if (!d) TLGB_FAIL(TLGB_ERR_INVALID, "null blocks descriptor");
  if (d->ndim < 1 || d->ndim > 3) TLGB_FAIL(TLGB_ERR_INVALID, "ndim must be 1, 2 or 3");
  switch (d->dtype) {
    case TLGB_F32: esize = 4; break;
    case TLGB_F64: esize = 8; break;
    case TLGB_C64: esize = 8; break;
    case TLGB_C128: esize = 16; break;
    default: TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "unsupported dtype for blocks op");
  }
  if (d->nbatch < 0) TLGB_FAIL(TLGB_ERR_INVALID, "negative batch");
  const int off = 3 - d->ndim;
  for (int e = 0; e < 3; ++e) {
    if (e < off) {
      g.im[e] = 1;
      g.B[e] = 1;
      g.s[e] = 1;
    } else {
      g.im[e] = d->im_size[e - off];
      g.B[e] = d->block[e - off];
      g.s[e] = d->stride[e - off];
    }
    if (g.im[e] < 1 || g.B[e] < 1 || g.s[e] < 1)
      TLGB_FAIL(TLGB_ERR_INVALID, "sizes, blocks and strides must be positive");
    g.nb[e] = g.im[e] >= g.B[e] ? (g.im[e] - g.B[e]) / g.s[e] + 1 : 0;
    if (g.nb[e] < 1) TLGB_FAIL(TLGB_ERR_INVALID, "block larger than the array: no block fits");
  }
  g.nbatch = d->nbatch;
  const int64_t bvol = g.B[0] * g.B[1] * g.B[2];
  const bool masked = d->mask_idx != nullptr;
  if (masked != (d->mask_inv != nullptr)) TLGB_FAIL(TLGB_ERR_INVALID, "mask_idx and mask_inv go together");
  g.nnz = masked ? d->nnz : bvol;
  if (masked && (g.nnz < 0 || g.nnz > bvol)) TLGB_FAIL(TLGB_ERR_INVALID, "mask nnz out of range");
  // 32-bit index arithmetic inside one slab / plane
  if (g.nb[2] * bvol >= (1ll << 31) || g.im[1] * g.im[2] >= (1ll << 31) || g.im[0] >= (1ll << 31))
    TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "block op too large for 32-bit slab indexing");
  // one CTA per slab (unfold) or array plane (fold): grid x below 2^31
  const int64_t lim = (1ll << 31) - 1;
  if (g.nbatch > 0 && (g.nbatch > lim / (g.nb[0] * g.nb[1]) || g.nbatch > lim / g.im[0]))
    TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "block op batch too large for one launch: split the batch");
  return TLGB_OK;
}

template <typename U>
int launch_unfold_rows(const BlkGeo& g, int esize, int ubytes, const void* in, void* out, cudaStream_t s) {
  const int64_t per = ubytes / esize;  // elements per unit (>= 1)
  const int64_t bu2 = g.B[2] / per;
  const int64_t s2u = g.s[2] / per;
  const int64_t im2u = g.im[2] / per;
  const int64_t slab_units = g.nb[2] * g.B[0] * g.B[1] * bu2;
  const int64_t nslab = g.nbatch * g.nb[0] * g.nb[1];
  if (nslab == 0 || slab_units == 0) return TLGB_OK;
  if (nslab >= (1ll << 31)) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "too many slabs");
  unfold_rows_kernel<U><<<(unsigned)nslab, 256, 0, s>>>(
      (const U*)in, (U*)out, g, bu2, s2u, im2u, make_fastdiv((uint32_t)bu2), make_fastdiv((uint32_t)g.B[1]),
      make_fastdiv((uint32_t)g.B[0]), (uint32_t)slab_units);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

template <typename T>
int launch_unfold_masked(const BlkGeo& g, const int32_t* mask_idx, const void* in, void* out, cudaStream_t s) {
  const int64_t slab = g.nb[2] * g.nnz;
  const int64_t nslab = g.nbatch * g.nb[0] * g.nb[1];
  if (nslab == 0 || slab == 0) return TLGB_OK;
  unfold_masked_kernel<T><<<(unsigned)nslab, 256, 0, s>>>(
      (const T*)in, (T*)out, g, mask_idx, make_fastdiv((uint32_t)g.nnz), make_fastdiv((uint32_t)g.B[2]),
      make_fastdiv((uint32_t)g.B[1]), (uint32_t)slab);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

template <typename T>
int launch_fold(const BlkGeo& g, const int32_t* mask_inv, const void* in, void* out, cudaStream_t s) {
  const int64_t nplane = g.nbatch * g.im[0];
  if (nplane == 0) return TLGB_OK;
  const FastDiv d2 = make_fastdiv((uint32_t)g.im[2]);
  const FastDiv s0 = make_fastdiv((uint32_t)g.s[0]), s1 = make_fastdiv((uint32_t)g.s[1]),
                s2 = make_fastdiv((uint32_t)g.s[2]);
  if constexpr (!std::is_same<T, double2>::value) {
    // element pairs: even innermost block, stride and extent, 32-bit offsets
    // inside a batch entry, pair-aligned pointers
    using V = typename std::conditional<std::is_same<T, float>::value, float2,
                                        typename std::conditional<std::is_same<T, double>::value, double2,
                                                                  float4>::type>::type;
    const int64_t per_entry = g.nb[0] * g.nb[1] * g.nb[2] * g.B[0] * g.B[1] * g.B[2];
    if (!mask_inv && g.B[2] % 2 == 0 && g.s[2] % 2 == 0 && g.im[2] >= 2 && g.im[2] % 2 == 0 && per_entry < (1ll << 31) &&
        g.im[1] * g.im[2] < (1ll << 31) && ((uintptr_t)in % sizeof(V)) == 0 && ((uintptr_t)out % sizeof(V)) == 0) {
      const FastDiv h2 = make_fastdiv((uint32_t)(g.im[2] / 2));
      fold_pairs_kernel<T, V><<<(unsigned)nplane, 256, 0, s>>>((const T*)in, (T*)out, g, h2, s0, s1, s2);
      TLGB_CHECK_LAUNCH();
      return TLGB_OK;
    }
  }
  if (mask_inv)
    fold_kernel<T, true><<<(unsigned)nplane, 256, 0, s>>>((const T*)in, (T*)out, g, mask_inv, d2, s0, s1, s2);
  else
    fold_kernel<T, false><<<(unsigned)nplane, 256, 0, s>>>((const T*)in, (T*)out, g, mask_inv, d2, s0, s1, s2);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

bool aligned(const void* p, int a) { return ((uintptr_t)p % (uintptr_t)a) == 0; }

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_unfold(const tlgb_blocks_desc* d, const void* array, void* blocks, tlgb_stream_t stream) {
  BlkGeo g;
  int esize = 0;
  TLGB_TRY(check_desc(d, g, esize));
  if (!array || !blocks) TLGB_FAIL(TLGB_ERR_INVALID, "null data pointer");
  if (!aligned(array, esize) || !aligned(blocks, esize)) TLGB_FAIL(TLGB_ERR_INVALID, "misaligned data pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (d->mask_idx) {
    switch (esize) {
      case 4: return launch_unfold_masked<uint32_t>(g, d->mask_idx, array, blocks, s);
      case 8: return launch_unfold_masked<uint2>(g, d->mask_idx, array, blocks, s);
      default: return launch_unfold_masked<uint4>(g, d->mask_idx, array, blocks, s);
    }
  }
  // widest copy unit that every innermost extent, stride and pointer allows
  for (int ub = 16; ub >= esize; ub /= 2) {
    if ((g.B[2] * esize) % ub || (g.s[2] * esize) % ub || (g.im[2] * esize) % ub) continue;
    if (!aligned(array, ub) || !aligned(blocks, ub)) continue;
    switch (ub) {
      case 16: return launch_unfold_rows<uint4>(g, esize, ub, array, blocks, s);
      case 8: return launch_unfold_rows<uint2>(g, esize, ub, array, blocks, s);
      default: return launch_unfold_rows<uint32_t>(g, esize, ub, array, blocks, s);
    }
  }
  TLGB_FAIL(TLGB_ERR_INVALID, "no copy unit fits the element size");
}

extern "C" int tlgb_fold(const tlgb_blocks_desc* d, const void* blocks, void* array, tlgb_stream_t stream) {
  BlkGeo g;
  int esize = 0;
  TLGB_TRY(check_desc(d, g, esize));
  if (!array || !blocks) TLGB_FAIL(TLGB_ERR_INVALID, "null data pointer");
  if (!aligned(array, esize) || !aligned(blocks, esize)) TLGB_FAIL(TLGB_ERR_INVALID, "misaligned data pointer");
  cudaStream_t s = (cudaStream_t)stream;
  switch (d->dtype) {
    case TLGB_F32: return launch_fold<float>(g, d->mask_inv, blocks, array, s);
    case TLGB_F64: return launch_fold<double>(g, d->mask_inv, blocks, array, s);
    case TLGB_C64: return launch_fold<float2>(g, d->mask_inv, blocks, array, s);
    default: return launch_fold<double2>(g, d->mask_inv, blocks, array, s);
  }
}

namespace tlgb {
int blocks_checked_status(int* line, int clear) { return checked_status(line, clear); }
}  // namespace tlgb
