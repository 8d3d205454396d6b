// FP64 reductions and fused vector updates of the conjugate-gradient loop.
//
// The reference CG (alg/pcg.py:13-88) forms its dot products and the
// alpha / beta / residual scalars in the input precision (complex64 -> float32)
// and reads them on the host. Here every dot product accumulates in float64
// with a fixed reduction tree (deterministic for a given length), and the
// scalars stay in a small float64 state vector on the device, so an iteration
// needs no host synchronisation.
//
// State vector layout (doubles): see enum CgSlot in tlgb.h.

#include <algorithm>

#include "common.cuh"

namespace tlgb {
namespace {

constexpr int kDotThreads = 256;
constexpr int kDotBlocks = 2048;  // fixed partial count -> fixed summation order (enough CTAs to hide FP64 latency)

__device__ __forceinline__ double2 warp_sum2(double2 v) {
  for (int m = 16; m > 0; m >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, m);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, m);
  }
  return v;
}

__device__ __forceinline__ double2 block_sum2(double2 v) {
  __shared__ double2 part[kDotThreads / 32];
  v = warp_sum2(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) part[w] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  if (w == 0) {
    s = l < kDotThreads / 32 ? part[l] : make_double2(0.0, 0.0);
    s = warp_sum2(s);
  }
  __syncthreads();
  return s;  // valid in thread 0
}

// partial[b] = sum over this block's slice of conj(x) * y (complex) or x * y
__global__ void __launch_bounds__(kDotThreads) dot_partial_kernel(const float* __restrict__ x,
                                                                  const float* __restrict__ y, int64_t n,
                                                                  int cplx, double2* __restrict__ partial) {
  double2 acc = make_double2(0.0, 0.0);
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b = (int64_t)blockIdx.x * per;
  const int64_t e = b + per < n ? b + per : n;
  if (cplx) {
    const float2* x2 = reinterpret_cast<const float2*>(x);
    const float2* y2 = reinterpret_cast<const float2*>(y);
    // two independent accumulators (the FP64 add latency, not bandwidth, bounds this loop)
    double2 acc2 = make_double2(0.0, 0.0);
    int64_t i = b + threadIdx.x;
    for (; i + kDotThreads < e; i += 2 * kDotThreads) {
      const float2 a = x2[i], c = y2[i], a2 = x2[i + kDotThreads], c2 = y2[i + kDotThreads];
      acc.x += (double)a.x * c.x + (double)a.y * c.y;
      acc.y += (double)a.x * c.y - (double)a.y * c.x;
      acc2.x += (double)a2.x * c2.x + (double)a2.y * c2.y;
      acc2.y += (double)a2.x * c2.y - (double)a2.y * c2.x;
    }
    if (i < e) {
      const float2 a = x2[i], c = y2[i];
      acc.x += (double)a.x * c.x + (double)a.y * c.y;
      acc.y += (double)a.x * c.y - (double)a.y * c.x;
    }
    acc.x += acc2.x;
    acc.y += acc2.y;
  } else {
    for (int64_t i = b + threadIdx.x; i < e; i += kDotThreads) acc.x += (double)x[i] * y[i];
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kDotThreads) dot_final_kernel(const double2* __restrict__ partial, int np,
                                                                double* __restrict__ out) {
  double2 acc = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < np; i += kDotThreads) {
    acc.x += partial[i].x;
    acc.y += partial[i].y;
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) {
    out[0] = acc.x;
    out[1] = acc.y;
  }
}

// x += a p ; r -= a Ap with a = st[RS] / st[PAP_RE]; partial |r|^2
__global__ void __launch_bounds__(kDotThreads) cg_step_kernel(float* __restrict__ x, float* __restrict__ r,
                                                              const float* __restrict__ p,
                                                              const float* __restrict__ ap, int64_t nf,
                                                              const double* __restrict__ st,
                                                              double2* __restrict__ partial) {
  const double rs = st[TLGB_CG_RS], pap = st[TLGB_CG_PAP];
  const float a = (float)(pap != 0.0 ? rs / pap : 0.0);
  double2 acc = make_double2(0.0, 0.0);
  const int64_t per = (nf + gridDim.x - 1) / gridDim.x;
  const int64_t b = (int64_t)blockIdx.x * per;
  const int64_t e = b + per < nf ? b + per : nf;
  for (int64_t i = b + threadIdx.x; i < e; i += kDotThreads) {
    x[i] = fmaf(a, p[i], x[i]);
    const float rn = fmaf(-a, ap[i], r[i]);
    r[i] = rn;
    acc.x += (double)rn * rn;
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// new rs from the partials; beta = rs_new / rs_old; rolls the state
__global__ void cg_scalars_kernel(const double2* __restrict__ partial, int np, double* __restrict__ st) {
  double2 acc = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < np; i += kDotThreads) acc.x += partial[i].x;
  acc = block_sum2(acc);
  if (threadIdx.x == 0) {
    const double rs_old = st[TLGB_CG_RS];
    st[TLGB_CG_ALPHA] = st[TLGB_CG_PAP] != 0.0 ? rs_old / st[TLGB_CG_PAP] : 0.0;
    st[TLGB_CG_RS_OLD] = rs_old;
    st[TLGB_CG_RS] = acc.x;
    st[TLGB_CG_BETA] = rs_old != 0.0 ? acc.x / rs_old : 0.0;
    st[TLGB_CG_ITERS] += 1.0;
  }
}

// p = r + beta p
__global__ void __launch_bounds__(kDotThreads) cg_dir_kernel(float* __restrict__ p, const float* __restrict__ r,
                                                             int64_t nf, const double* __restrict__ st) {
  const float beta = (float)st[TLGB_CG_BETA];
  for (int64_t i = (int64_t)blockIdx.x * kDotThreads + threadIdx.x; i < nf; i += (int64_t)gridDim.x * kDotThreads)
    p[i] = fmaf(beta, p[i], r[i]);
}

// Flexible preconditioned CG (st[RS] holds <r, z>): x += a p ; r -= a Ap
// with a = st[RS] / st[PAP], rounded once to float32 as in cg_step_kernel.
__global__ void __launch_bounds__(kDotThreads) pcg_update_kernel(float* __restrict__ x, float* __restrict__ r,
                                                                 const float* __restrict__ p,
                                                                 const float* __restrict__ ap, int64_t nf,
                                                                 const double* __restrict__ st) {
  const double rz = st[TLGB_CG_RS], pap = st[TLGB_CG_PAP];
  const float a = (float)(pap != 0.0 ? rz / pap : 0.0);
  for (int64_t i = (int64_t)blockIdx.x * kDotThreads + threadIdx.x; i < nf; i += (int64_t)gridDim.x * kDotThreads) {
    x[i] = fmaf(a, p[i], x[i]);
    r[i] = fmaf(-a, ap[i], r[i]);
  }
}

// partial[b] = (Re <r, z>, Re <Ap, z>) over this block's slice (complex
// values as interleaved floats: the real part of the Hermitian product is
// the plain sum over both components)
__global__ void __launch_bounds__(kDotThreads) pcg_dots_kernel(const float* __restrict__ r,
                                                               const float* __restrict__ z,
                                                               const float* __restrict__ ap, int64_t nf,
                                                               double2* __restrict__ partial) {
  double2 acc = make_double2(0.0, 0.0);
  const int64_t per = (nf + gridDim.x - 1) / gridDim.x;
  const int64_t b = (int64_t)blockIdx.x * per;
  const int64_t e = b + per < nf ? b + per : nf;
  for (int64_t i = b + threadIdx.x; i < e; i += kDotThreads) {
    const double zi = z[i];
    acc.x += (double)r[i] * zi;
    acc.y += (double)ap[i] * zi;
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// <r, z> and the flexible (Polak-Ribiere) beta = <r_new - r_old, z> / <r_old, z_old>,
// with r_new - r_old = -a Ap (the form that does not subtract two nearly equal
// residuals), clamped at 0; rolls the state
__global__ void pcg_scalars_kernel(const double2* __restrict__ partial, int np, double* __restrict__ st) {
  double2 acc = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < np; i += kDotThreads) {
    acc.x += partial[i].x;
    acc.y += partial[i].y;
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) {
    const double rz_old = st[TLGB_CG_RS], pap = st[TLGB_CG_PAP];
    const double a = pap != 0.0 ? rz_old / pap : 0.0;
    const double beta = rz_old != 0.0 ? -a * acc.y / rz_old : 0.0;
    st[TLGB_CG_ALPHA] = a;
    st[TLGB_CG_RS_OLD] = rz_old;
    st[TLGB_CG_RS] = acc.x;
    st[TLGB_CG_BETA] = beta > 0.0 ? beta : 0.0;
    st[TLGB_CG_ITERS] += 1.0;
  }
}

__global__ void copy_pap_kernel(const double* __restrict__ dot, double* __restrict__ st) {
  st[TLGB_CG_PAP] = dot[0];
}

int nblocks_for(int64_t n) { return (int)std::min<int64_t>(kDotBlocks, std::max<int64_t>(1, cdiv(n, 4 * kDotThreads))); }

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" size_t tlgb_cg_scratch_bytes(void) { return (size_t)kDotBlocks * sizeof(double2) + 64; }

extern "C" int tlgb_dot_f64(const float* x, const float* y, int64_t n, int is_complex, double* out, void* scratch,
                            size_t scratch_bytes, tlgb_stream_t stream) {
  if (n < 0 || !out || (n > 0 && (!x || !y))) TLGB_FAIL(TLGB_ERR_INVALID, "bad dot arguments");
  if (scratch_bytes < tlgb_cg_scratch_bytes() || !scratch) TLGB_FAIL(TLGB_ERR_WORKSPACE, "dot scratch too small");
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = nblocks_for(n);
  double2* part = (double2*)scratch;
  dot_partial_kernel<<<nb, kDotThreads, 0, s>>>(x, y, n, is_complex ? 1 : 0, part);
  TLGB_CHECK_LAUNCH();
  dot_final_kernel<<<1, kDotThreads, 0, s>>>(part, nb, out);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_cg_set_pap(const float* p, const float* ap, int64_t n, int is_complex, double* state,
                               void* scratch, size_t scratch_bytes, tlgb_stream_t stream) {
  TLGB_TRY(tlgb_dot_f64(p, ap, n, is_complex, state + TLGB_CG_TMP, scratch, scratch_bytes, stream));
  copy_pap_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(state + TLGB_CG_TMP, state);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_cg_step(float* x, float* r, float* p, const float* ap, int64_t n, int is_complex, double* state,
                            void* scratch, size_t scratch_bytes, tlgb_stream_t stream) {
  if (n < 0 || !state || (n > 0 && (!x || !r || !p || !ap))) TLGB_FAIL(TLGB_ERR_INVALID, "bad cg arguments");
  if (scratch_bytes < tlgb_cg_scratch_bytes() || !scratch) TLGB_FAIL(TLGB_ERR_WORKSPACE, "cg scratch too small");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nf = is_complex ? 2 * n : n;
  const int nb = nblocks_for(nf);
  double2* part = (double2*)scratch;
  cg_step_kernel<<<nb, kDotThreads, 0, s>>>(x, r, p, ap, nf, state, part);
  TLGB_CHECK_LAUNCH();
  cg_scalars_kernel<<<1, kDotThreads, 0, s>>>(part, nb, state);
  TLGB_CHECK_LAUNCH();
  const int nd = (int)std::min<int64_t>(4 * 152, std::max<int64_t>(1, cdiv(nf, kDotThreads)));
  cg_dir_kernel<<<nd, kDotThreads, 0, s>>>(p, r, nf, state);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_pcg_update(float* x, float* r, const float* p, const float* ap, int64_t n, int is_complex,
                               const double* state, tlgb_stream_t stream) {
  if (n < 0 || !state || (n > 0 && (!x || !r || !p || !ap))) TLGB_FAIL(TLGB_ERR_INVALID, "bad pcg arguments");
  const int64_t nf = is_complex ? 2 * n : n;
  if (nf == 0) return TLGB_OK;
  const int nd = (int)std::min<int64_t>(4 * 152, std::max<int64_t>(1, cdiv(nf, kDotThreads)));
  pcg_update_kernel<<<nd, kDotThreads, 0, (cudaStream_t)stream>>>(x, r, p, ap, nf, state);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_pcg_direction(const float* r, const float* z, const float* ap, float* p, int64_t n,
                                  int is_complex, double* state, void* scratch, size_t scratch_bytes,
                                  tlgb_stream_t stream) {
  if (n < 0 || !state || (n > 0 && (!r || !z || !ap || !p))) TLGB_FAIL(TLGB_ERR_INVALID, "bad pcg arguments");
  if (scratch_bytes < tlgb_cg_scratch_bytes() || !scratch) TLGB_FAIL(TLGB_ERR_WORKSPACE, "cg scratch too small");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nf = is_complex ? 2 * n : n;
  const int nb = nblocks_for(nf);
  double2* part = (double2*)scratch;
  pcg_dots_kernel<<<nb, kDotThreads, 0, s>>>(r, z, ap, nf, part);
  TLGB_CHECK_LAUNCH();
  pcg_scalars_kernel<<<1, kDotThreads, 0, s>>>(part, nb, state);
  TLGB_CHECK_LAUNCH();
  const int nd = (int)std::min<int64_t>(4 * 152, std::max<int64_t>(1, cdiv(nf, kDotThreads)));
  cg_dir_kernel<<<nd, kDotThreads, 0, s>>>(p, z, nf, state);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}
