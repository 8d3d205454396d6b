// Circular padding of the trailing dims and its adjoint: the padding of the
// Convolution linop's circular mode (linops/convolution.py:120-130,148-150).
//
// The reference pads up to three dims at a time with torch's
// F.pad(mode="circular"), cycling the dims through the back of the tensor
// for more (functional/_interp/_circ_pad.py:10-83), and forms the adjoint by
// autograd through that (circular_pad_adjoint, :119-134). Here one gather
// pads any number of dims (up to 8) in one pass, and the adjoint is one
// output-stationary pass: each element sums the padded elements that are
// copies of it, in ascending padded order (deterministic; no atomics).
//
// Both kernels work on rows: one CTA per output row (all dims but the last),
// its source rows found once per CTA, the threads running along the
// innermost dim.

#include <algorithm>

#include "common.cuh"

namespace tlgb {
namespace {

struct PadGeo {
  int ndim;
  int64_t n[TLGB_CIRCPAD_MAX_DIM];   // unpadded sizes
  int64_t np[TLGB_CIRCPAD_MAX_DIM];  // padded sizes
  int64_t lo[TLGB_CIRCPAD_MAX_DIM];
  int64_t nbatch;
};

template <typename E>
__global__ void __launch_bounds__(256) circpad_kernel(PadGeo g, const E* __restrict__ in, E* __restrict__ out,
                                                      int64_t out_rows) {
  const int D = g.ndim;
  const int64_t nl = g.n[D - 1], npl = g.np[D - 1], lol = g.lo[D - 1];
  for (int64_t r = blockIdx.x; r < out_rows; r += gridDim.x) {
    // padded row r = (b, j_0 .. j_{D-2}) -> source row (b, i_0 .. i_{D-2})
    int64_t t = r, src = 0, mul = 1;
    for (int d = D - 2; d >= 0; --d) {
      const int64_t j = t % g.np[d];
      t /= g.np[d];
      int64_t i = j - g.lo[d];
      if (i < 0) i += g.n[d];
      if (i >= g.n[d]) i -= g.n[d];
      src += i * mul;
      mul *= g.n[d];
    }
    src += t * mul;  // t is now the batch index
    const E* s = in + src * nl;
    E* dst = out + r * npl;
    for (int64_t j = threadIdx.x; j < npl; j += blockDim.x) {
      int64_t i = j - lol;
      if (i < 0) i += nl;
      if (i >= nl) i -= nl;
      dst[j] = s[i];
    }
  }
}

template <typename T>
__device__ __forceinline__ T add_elem(T a, T b) { return a + b; }
template <>
__device__ __forceinline__ float2 add_elem(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
template <>
__device__ __forceinline__ double2 add_elem(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// out[b, i] = sum over the padded elements j that copy element i, in
// ascending padded (row-major) order: per dim j = i + lo + k n for the k
// with 0 <= j < np (k in -1..1, since lo, hi <= n)
template <typename T>
__global__ void __launch_bounds__(256) circpad_adj_kernel(PadGeo g, const T* __restrict__ in, T* __restrict__ out,
                                                          int64_t out_rows) {
  const int D = g.ndim;
  const int64_t nl = g.n[D - 1], npl = g.np[D - 1], lol = g.lo[D - 1];
  for (int64_t r = blockIdx.x; r < out_rows; r += gridDim.x) {
    // unpadded row r = (b, i_0 .. i_{D-2}): per dim its padded copies (at most 3)
    int64_t t = r;
    int64_t cand[TLGB_CIRCPAD_MAX_DIM][3];
    int ncand[TLGB_CIRCPAD_MAX_DIM];
    for (int d = D - 2; d >= 0; --d) {
      const int64_t i = t % g.n[d];
      t /= g.n[d];
      int c = 0;
      for (int k = -1; k <= 1; ++k) {
        const int64_t j = i + g.lo[d] + k * g.n[d];
        if (j >= 0 && j < g.np[d]) cand[d][c++] = j;
      }
      ncand[d] = c;
    }
    const int64_t b = t;
    int64_t prow = 1;
    for (int d = 0; d < D - 1; ++d) prow *= g.np[d];
    int total = 1;
    for (int d = 0; d < D - 1; ++d) total *= ncand[d];
    T* dst = out + r * nl;
    for (int64_t i = threadIdx.x; i < nl; i += blockDim.x) {
      T acc{};
      // source rows in ascending order: odometer over the candidates, dim 0 slowest
      for (int q = 0; q < total; ++q) {
        int rem = q;
        int64_t row = 0;
        for (int d = D - 2; d >= 0; --d) {
          const int k = rem % ncand[d];
          rem /= ncand[d];
          int64_t m = 1;
          for (int e = d + 1; e < D - 1; ++e) m *= g.np[e];
          row += cand[d][k] * m;
        }
        const T* s = in + (b * prow + row) * npl;
        for (int k = -1; k <= 1; ++k) {
          const int64_t j = i + lol + k * nl;
          if (j >= 0 && j < npl) acc = add_elem(acc, s[j]);
        }
      }
      dst[i] = acc;
    }
  }
}

int make_pad_geo(const tlgb_circpad_desc* d, PadGeo& g, int64_t& in_rows, int64_t& out_rows) {
  if (!d) TLGB_FAIL(TLGB_ERR_INVALID, "null circular pad descriptor");
  if (d->ndim < 1 || d->ndim > TLGB_CIRCPAD_MAX_DIM) TLGB_FAIL(TLGB_ERR_INVALID, "circular pad: ndim must be in [1, 8]");
  if (d->nbatch < 0) TLGB_FAIL(TLGB_ERR_INVALID, "circular pad: negative batch");
  g.ndim = d->ndim;
  g.nbatch = d->nbatch;
  in_rows = d->nbatch;
  out_rows = d->nbatch;
  for (int e = 0; e < d->ndim; ++e) {
    const int64_t n = d->size[e], lo = d->pad_lo[e], hi = d->pad_hi[e];
    if (n < 1) TLGB_FAIL(TLGB_ERR_INVALID, "circular pad: sizes must be positive");
    if (lo < 0 || hi < 0 || lo > n || hi > n)
      TLGB_FAIL(TLGB_ERR_INVALID, "circular pad: each pad must lie in [0, size] (padding wraps around at most once)");
    g.n[e] = n;
    g.lo[e] = lo;
    g.np[e] = n + lo + hi;
    if (e < d->ndim - 1) {
      in_rows *= n;
      out_rows *= g.np[e];
    }
  }
  if (in_rows > ((int64_t)1 << 40) || out_rows > ((int64_t)1 << 40))
    TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "circular pad: too many rows");
  return TLGB_OK;
}

unsigned rows_grid(int64_t rows) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(rows, (int64_t)sm_count() * 16));
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_circular_pad(const tlgb_circpad_desc* d, const void* in, void* out, tlgb_stream_t stream) {
  PadGeo g;
  int64_t in_rows = 0, out_rows = 0;
  TLGB_TRY(make_pad_geo(d, g, in_rows, out_rows));
  if (out_rows == 0) return TLGB_OK;
  if (!in || !out) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned grd = rows_grid(out_rows);
  switch (d->dtype) {
    case TLGB_RAW8: circpad_kernel<uint8_t><<<grd, 256, 0, s>>>(g, (const uint8_t*)in, (uint8_t*)out, out_rows); break;
    case TLGB_RAW16: circpad_kernel<uint16_t><<<grd, 256, 0, s>>>(g, (const uint16_t*)in, (uint16_t*)out, out_rows); break;
    case TLGB_F32: case TLGB_I32:
      circpad_kernel<uint32_t><<<grd, 256, 0, s>>>(g, (const uint32_t*)in, (uint32_t*)out, out_rows); break;
    case TLGB_F64: case TLGB_C64: case TLGB_I64:
      circpad_kernel<uint2><<<grd, 256, 0, s>>>(g, (const uint2*)in, (uint2*)out, out_rows); break;
    case TLGB_C128: circpad_kernel<uint4><<<grd, 256, 0, s>>>(g, (const uint4*)in, (uint4*)out, out_rows); break;
    default: TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "circular pad: unsupported element type");
  }
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_circular_pad_adjoint(const tlgb_circpad_desc* d, const void* in, void* out, tlgb_stream_t stream) {
  PadGeo g;
  int64_t in_rows = 0, out_rows = 0;
  TLGB_TRY(make_pad_geo(d, g, in_rows, out_rows));
  if (in_rows == 0) return TLGB_OK;
  if (!in || !out) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned grd = rows_grid(in_rows);
  switch (d->dtype) {
    case TLGB_F32: circpad_adj_kernel<float><<<grd, 256, 0, s>>>(g, (const float*)in, (float*)out, in_rows); break;
    case TLGB_F64: circpad_adj_kernel<double><<<grd, 256, 0, s>>>(g, (const double*)in, (double*)out, in_rows); break;
    case TLGB_C64: circpad_adj_kernel<float2><<<grd, 256, 0, s>>>(g, (const float2*)in, (float2*)out, in_rows); break;
    case TLGB_C128: circpad_adj_kernel<double2><<<grd, 256, 0, s>>>(g, (const double2*)in, (double2*)out, in_rows); break;
    case TLGB_I32: circpad_adj_kernel<int32_t><<<grd, 256, 0, s>>>(g, (const int32_t*)in, (int32_t*)out, in_rows); break;
    case TLGB_I64: circpad_adj_kernel<long long><<<grd, 256, 0, s>>>(g, (const long long*)in, (long long*)out, in_rows); break;
    default: TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "circular pad adjoint: unsupported element type");
  }
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}
