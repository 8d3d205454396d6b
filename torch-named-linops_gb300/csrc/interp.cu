// Kaiser-Bessel / spline interpolation (ungrid), gridding (adjoint) and the
// trajectory gradient, 1D-3D, for sm_103a.
//
// Replaces the reference's Triton kernels _ungrid{1,2,3}d (functional/_interp/
// ungrid.py:162-503) and _grid{1,2,3}d (grid.py:169-513); the arithmetic of a
// tap follows the reference's pure-torch path (ungrid_torch ungrid.py:624-684,
// grid_torch grid.py:571-639, weights_torch kernels.py:108-147,
// kaiser_bessel_torch kernels.py:28-89) operation for operation in float32.
//
// Design (GB300 first, not a translation of the Triton programs):
//  * Plan (once per trajectory): every point is paired with each output tile
//    its valid taps touch; the pairs are sorted by tile with a stable LSD
//    radix sort, "home" pairs (the tile holding the point's first valid tap)
//    first. Work items are chunks of at most `chunk` pairs of one tile, so
//    dense k-space centres are spread over many CTAs.
//  * Forward (gather): a CTA stages its tile plus the kernel halo for a group
//    of up to 8 batch entries in shared memory ([x][y][z][batch] order, batch
//    fastest) and each warp interpolates one home point at a time; lanes are
//    (tap along the last dim, batch entry) so one warp load reads 4 taps x 8
//    entries = 256 contiguous bytes, conflict-free.
//  * Adjoint (scatter, deterministic, no global atomics): output-stationary.
//    A CTA owns one output tile in shared memory and visits every point whose
//    window touches it, in plan order. Warp w owns the tile planes with
//    (outer index) % 8 == w, so every shared-memory cell is updated by one
//    fixed warp in one fixed order: results are bit-identical run to run.
//    Each tile is written to HBM exactly once. Tiles denser than `chunk`
//    pairs are split: each part writes a partial tile to scratch and a second
//    kernel sums the parts in order.
//  * Kernel values are evaluated directly with the reference's A&S formula
//    (expf/sqrtf, IEEE division), not from a lookup table: a table would add
//    an interpolation error on top of the 1e-5 budget, and the 3 x (W+1)
//    evaluations per point visit are shared by every batch entry of the visit.

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "sm100.cuh"

namespace tlgb {
namespace {

constexpr int NTMAX = 16;  // taps per dimension supported (width < 15)
constexpr int NWARP = 8;   // warps per CTA
constexpr int NTHR = 32 * NWARP;
constexpr int CGMAX = 8;   // batch entries per coil group

struct Geo {
  int ndim;
  int N[3];   // internal dims (x, y, z); leading inactive dims have N = 1
  int T[3];   // tile edge
  int nt[3];  // tiles per dim
  int NT[3];  // taps per dim (inactive: 1)
  float r[3]; // kernel radius W/2 per dim
  float rinv[3];  // 1/r, used when r is a power of two (the product is then exact)
  int rpow2[3];
  int act[3];
  int kernel, norm, pad, cplx;
  float beta;
  long long npts, nbatch;
  int wrap_safe;  // every active N >= NT: a window never overlaps itself
  long long tv_off;  // gridding: byte offset in scratch of the point-major values, -1 = none
  int skip_copy;     // test hook (tlgb_test_skip_region_copy): TMA kernels skip their region copy
};

// ---------------------------------------------------------------- kernels math

// A&S 9.8.1 / 9.8.2 coefficients (the reference's kernels.py:65-88)
__device__ __forceinline__ float kb_value(float x, float beta) {
  const float z = beta * __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(x, x)));
  const float t = __fdiv_rn(z, 3.75f);
  const float t2 = t * t;
  if (z < 3.75f) {
    const float t4 = t2 * t2, t6 = t4 * t2, t8 = t4 * t4, t10 = t6 * t4, t12 = t6 * t6;
    return 1.0f + 3.5156229f * t2 + 3.0899424f * t4 + 1.2067492f * t6 + 0.2659732f * t8 + 0.0360768f * t10 +
           0.0045813f * t12;
  }
  const float t3 = t2 * t, t4 = t2 * t2, t5 = t3 * t2, t6 = t4 * t2, t7 = t5 * t2, t8 = t4 * t4;
  const float poly = 0.39894228f + __fdiv_rn(0.01328592f, t) + __fdiv_rn(0.00225319f, t2) -
                     __fdiv_rn(0.00157565f, t3) + __fdiv_rn(0.00916281f, t4) - __fdiv_rn(0.02057706f, t5) +
                     __fdiv_rn(0.02635537f, t6) - __fdiv_rn(0.01647633f, t7) + __fdiv_rn(0.00392377f, t8);
  return __fdiv_rn(expf(z), __fsqrt_rn(z)) * poly;
}

// d KB(x) / dx of the same A&S expressions (x signed, |x| <= 1)
__device__ __forceinline__ float kb_deriv(float x, float beta) {
  const float z = beta * __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(x, x)));
  const float b2 = beta * beta;
  if (z < 3.75f) {
    const float u = (z / 3.75f) * (z / 3.75f);
    // P(u) = 1 + a1 u + ... + a6 u^6 ; P'(u)
    const float dp = 3.5156229f + u * (2.f * 3.0899424f + u * (3.f * 1.2067492f + u * (4.f * 0.2659732f +
                     u * (5.f * 0.0360768f + u * (6.f * 0.0045813f)))));
    return -2.0f * b2 * x * dp / (3.75f * 3.75f);
  }
  const float v = 3.75f / z;
  const float q = 0.39894228f + v * (0.01328592f + v * (0.00225319f + v * (-0.00157565f + v * (0.00916281f +
                  v * (-0.02057706f + v * (0.02635537f + v * (-0.01647633f + v * 0.00392377f)))))));
  const float dq = 0.01328592f + v * (2.f * 0.00225319f + v * (3.f * -0.00157565f + v * (4.f * 0.00916281f +
                   v * (5.f * -0.02057706f + v * (6.f * 0.02635537f + v * (7.f * -0.01647633f +
                   v * (8.f * 0.00392377f)))))));
  const float e = expf(z) / sqrtf(z);
  const float dI = e * (q * (1.0f - 0.5f / z) - dq * 3.75f / (z * z));
  return dI * (-b2 * x / z);
}

__device__ __forceinline__ float kern_value(int kernel, float ax, float beta) {
  return kernel == TLGB_KERNEL_KAISER_BESSEL ? kb_value(ax, beta) : fmaxf(1.0f - ax, 0.0f);
}

__device__ __forceinline__ float kern_deriv(int kernel, float d, float beta) {
  if (kernel == TLGB_KERNEL_KAISER_BESSEL) return kb_deriv(d, beta);
  return (fabsf(d) < 1.0f) ? (d > 0.f ? -1.0f : (d < 0.f ? 1.0f : 0.0f)) : 0.0f;
}

__device__ __forceinline__ bool coord_ok(float x) { return isfinite(x) && fabsf(x) < 16777216.0f; }

// One tap of one dimension: the reference's dlocs = (locs - grid_locs) / radius
// and its validity (kernels.py:126-146).
struct Tap {
  float d;     // signed normalised offset
  bool valid;
};

__device__ __forceinline__ Tap tap_eval(const Geo& g, int e, float x, int lower, int k) {
  Tap t;
  const float gk = (float)(lower + k);
  const float diff = __fsub_rn(x, gk);
  t.d = g.rpow2[e] ? __fmul_rn(diff, g.rinv[e]) : __fdiv_rn(diff, g.r[e]);
  const float ad = fabsf(t.d);
  bool v = ad <= g.r[e];
  if (g.kernel == TLGB_KERNEL_KAISER_BESSEL) v = v && (ad <= 1.0f);
  if (g.pad == TLGB_PAD_ZERO) v = v && (lower + k >= 0) && (lower + k < g.N[e]);
  t.valid = v;
  return t;
}

__device__ __forceinline__ int lower_of(const Geo& g, int e, float x) {
  return (int)ceilf(__fsub_rn(x, g.r[e]));
}

__device__ __forceinline__ int wrapi(int v, int n) {
  if (v >= 0 && v < n) return v;
  int m = v % n;
  return m < 0 ? m + n : m;
}

__device__ __forceinline__ float load_coord(const Geo& g, const float* locs, long long p, int e) {
  return __ldg(locs + p * g.ndim + (e - (3 - g.ndim)));
}

// Valid tap range [s, s+n) of one dim for one point (sequential; used by the plan).
__device__ __forceinline__ bool axis_range(const Geo& g, const float* locs, long long p, int e, int& start, int& n) {
  if (!g.act[e]) {
    start = 0;
    n = 1;
    return true;
  }
  const float x = load_coord(g, locs, p, e);
  if (!coord_ok(x)) return false;
  const int lower = lower_of(g, e, x);
  int s = -1;
  n = 0;
  for (int k = 0; k < g.NT[e]; ++k) {
    if (tap_eval(g, e, x, lower, k).valid) {
      if (s < 0) s = k;
      ++n;
    }
  }
  if (n == 0) return false;
  start = lower + s;
  if (g.pad == TLGB_PAD_CIRCULAR) start = wrapi(start, g.N[e]);
  return true;
}

// --------------------------------------------------------------------- plan

// Distinct tiles touched along one dim by taps start .. start+n-1 (wrapped);
// the first is the home tile. At most 3 (a window crossing a ragged last tile
// and the wrap), see max_tiles_per_dim on the host.
__device__ __forceinline__ int axis_tiles(const Geo& g, int e, int start, int n, int* tl) {
  int cnt = 0;
  for (int k = 0; k < n; ++k) {
    int v = start + k;
    if (g.pad == TLGB_PAD_CIRCULAR) v = wrapi(v, g.N[e]);
    const int t = v / g.T[e];
    bool seen = false;
    for (int i = 0; i < cnt; ++i) seen = seen || (tl[i] == t);
    if (!seen && cnt < 3) tl[cnt++] = t;
  }
  return cnt;
}

__global__ void plan_count_kernel(Geo g, const float* __restrict__ locs, uint32_t* __restrict__ cnt) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  uint32_t c = 1;
  for (int e = 0; e < 3; ++e) {
    int st, n, tl[3];
    if (!axis_range(g, locs, p, e, st, n)) {
      c = 0;
      break;
    }
    c *= (uint32_t)axis_tiles(g, e, st, n, tl);
  }
  cnt[p] = c;
}

__global__ void plan_emit_kernel(Geo g, const float* __restrict__ locs, const uint32_t* __restrict__ off,
                                 uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  int tl[3][3], nc[3];
  for (int e = 0; e < 3; ++e) {
    int st, n;
    if (!axis_range(g, locs, p, e, st, n)) return;
    nc[e] = axis_tiles(g, e, st, n, tl[e]);
  }
  uint32_t o = off[p];
  for (int i = 0; i < nc[0]; ++i)
    for (int j = 0; j < nc[1]; ++j)
      for (int k = 0; k < nc[2]; ++k) {
        const uint32_t tile = ((uint32_t)tl[0][i] * g.nt[1] + tl[1][j]) * g.nt[2] + tl[2][k];
        const bool home = (i == 0 && j == 0 && k == 0);
        keys[o] = tile * 2u + (home ? 0u : 1u);
        vals[o] = (int32_t)p;
        ++o;
      }
}

__global__ void key_hist_kernel(const uint32_t* __restrict__ keys, long long n, uint32_t* __restrict__ hist) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(hist + keys[i], 1u);
}

// ------------------------------------------------------------- value types

template <typename V>
struct VT;
template <>
struct VT<float> {
  __device__ static float zero() { return 0.f; }
  __device__ static void fma(float& a, float w, float v) { a = fmaf(w, v, a); }
  __device__ static void add(float& a, float b) { a += b; }
  __device__ static float shfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  __device__ static float re_dot(float a, float b) { return a * b; }
};
template <>
struct VT<float2> {
  __device__ static float2 zero() { return make_float2(0.f, 0.f); }
  __device__ static void fma(float2& a, float w, float2 v) {
    a.x = fmaf(w, v.x, a.x);
    a.y = fmaf(w, v.y, a.y);
  }
  __device__ static void add(float2& a, float2 b) {
    a.x += b.x;
    a.y += b.y;
  }
  __device__ static float2 shfl_xor(float2 v, int m) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
  }
  // Re(conj(a) * b)
  __device__ static float re_dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
};

// Per point: start coordinate and valid-tap count per internal dim, and the
// per-tap value used by the inner loops: the 1D weight (norm 1) or |d|
// (norm 2). The DERIV variant adds d weight / d x (norm 1) or signed d (norm 2).
template <bool DERIV>
struct PTaps {
  int start[3];
  int n[3];
  float w[3][NTMAX];
  float dw[DERIV ? 3 : 1][DERIV ? NTMAX : 1];
};
using PointTaps = PTaps<false>;

// Warp-cooperative tap evaluation of point p into `pt` (shared memory).
// Returns false (warp-uniform) if the point has no valid tap.
template <int NORM, bool DERIV>
__device__ __forceinline__ bool warp_point_taps(const Geo& g, const float* locs, long long p, PTaps<DERIV>& pt,
                                                int lane) {
  bool ok = true;
  for (int e = 0; e < 3; ++e) {
    if (!g.act[e]) {
      if (lane == 0) {
        pt.start[e] = 0;
        pt.n[e] = 1;
        pt.w[e][0] = NORM == 1 ? 1.f : 0.f;  // weight 1, or |d| = 0 for the radial norm
        if (DERIV) pt.dw[e][0] = 0.f;
      }
      continue;
    }
    const float x = load_coord(g, locs, p, e);
    if (!coord_ok(x)) {
      ok = false;
      break;
    }
    const int lower = lower_of(g, e, x);
    const int k = lane;
    Tap t;
    t.valid = false;
    t.d = 0.f;
    if (k < g.NT[e]) t = tap_eval(g, e, x, lower, k);
    const unsigned m = __ballot_sync(0xffffffffu, t.valid);
    if (m == 0) {
      ok = false;
      break;
    }
    const int s = __ffs(m) - 1;
    const int n = __popc(m);
    if (t.valid) {
      const int j = k - s;
      const float ad = fabsf(t.d);
      if (NORM == 1) {
        pt.w[e][j] = kern_value(g.kernel, ad, g.beta);
        if (DERIV) pt.dw[e][j] = kern_deriv(g.kernel, t.d, g.beta) / g.r[e];
      } else {
        pt.w[e][j] = ad;
        if (DERIV) pt.dw[e][j] = t.d;
      }
    }
    if (lane == 0) {
      int st = lower + s;
      if (g.pad == TLGB_PAD_CIRCULAR) st = wrapi(st, g.N[e]);
      pt.start[e] = st;
      pt.n[e] = n;
    }
  }
  __syncwarp();
  return ok;
}

// norm-2 weight of one tap combination (radial), 0 outside the unit ball
__device__ __forceinline__ float radial_w(const Geo& g, float a0, float a1, float a2) {
  const float rho = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2)));
  if (rho > 1.0f) return 0.f;
  return kern_value(g.kernel, rho, g.beta);
}

__device__ __forceinline__ int lg2i(int v) { return 31 - __clz(v); }

// ------------------------------------------------- lane-per-point taps

// KB(x) by the same A&S expansions as kb_value, with one division (3.75 / z)
// and Horner evaluation instead of one division per term: equal to kb_value
// to a few float32 ulps, ~3x fewer instructions. Used on the hot paths.
__device__ __forceinline__ float kb_fast(float x, float beta) {
  const float z = beta * __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(x, x)));
  if (z < 3.75f) {
    const float u = (z * (1.0f / 3.75f)) * (z * (1.0f / 3.75f));
    return 1.0f + u * (3.5156229f + u * (3.0899424f + u * (1.2067492f + u * (0.2659732f +
           u * (0.0360768f + u * 0.0045813f)))));
  }
  const float v = __fdiv_rn(3.75f, z);
  const float q = 0.39894228f + v * (0.01328592f + v * (0.00225319f + v * (-0.00157565f + v * (0.00916281f +
                  v * (-0.02057706f + v * (0.02635537f + v * (-0.01647633f + v * 0.00392377f)))))));
  return expf(z) * rsqrtf(z) * q;
}

__device__ __forceinline__ float kb_approx(float ax, float beta);
__device__ __forceinline__ float kern_value_approx(int kernel, float ax, float beta) {
  return kernel == TLGB_KERNEL_KAISER_BESSEL ? kb_approx(ax, beta) : fmaxf(1.0f - ax, 0.0f);
}

__device__ __forceinline__ float kern_fast(int kernel, float ax, float beta) {
  return kernel == TLGB_KERNEL_KAISER_BESSEL ? kb_fast(ax, beta) : fmaxf(1.0f - ax, 0.0f);
}

// Per point record staged in shared memory: for each internal dim the taps
// that land in the CTA's tile (gridding) or region (gather), as a local
// coordinate and the 1D weight (norm 1) or |d| (norm 2). Taps outside the
// tile are dropped here, so the inner loops carry no bounds checks.
template <int NTB>
struct Rec {
  short lc[3][NTB];
  float wv[3][NTB];
  int m[3];
  int fast;  // every dim has <= 4 kept taps at consecutive local coordinates
};

// One lane builds the record of point p (coordinates x3) for the tile with
// origin o and extent T. region: gather mode, local coordinates run
// contiguously from the wrapped start (the staged region holds the wrap).
template <int NTB>
__device__ __forceinline__ void lane_rec(const Geo& g, const float (&x3)[3], const int (&o)[3], bool region,
                                         Rec<NTB>& R) {
  bool ok = true;
  for (int e = 0; e < 3; ++e) {
    if (!g.act[e]) {
      R.lc[e][0] = 0;
      R.wv[e][0] = g.norm == 1 ? 1.f : 0.f;
      R.m[e] = 1;
      continue;
    }
    const float x = x3[e];
    int cnt = 0;
    if (ok && coord_ok(x)) {
      const int lower = lower_of(g, e, x);
      int s = -1;
      for (int k = 0; k < g.NT[e]; ++k) {
        const Tap t = tap_eval(g, e, x, lower, k);
        if (!t.valid) continue;
        if (s < 0) s = k;
        int l;
        if (region) {
          int st = lower + s;
          if (g.pad == TLGB_PAD_CIRCULAR) st = wrapi(st, g.N[e]);
          l = st - o[e] + (k - s);
        } else {
          int gg = lower + k;
          if (g.pad == TLGB_PAD_CIRCULAR) gg = wrapi(gg, g.N[e]);
          l = gg - o[e];
          if (l < 0 || l >= g.T[e]) continue;
        }
        if (cnt < NTB) {
          const float ad = fabsf(t.d);
          R.lc[e][cnt] = (short)l;
          R.wv[e][cnt] = g.norm == 1 ? kern_fast(g.kernel, ad, g.beta) : ad;
          ++cnt;
        }
      }
    }
    R.m[e] = cnt;
    if (cnt == 0) ok = false;
  }
  if (!ok) R.m[0] = 0;
  bool fast = ok;
  for (int e = 0; e < 3 && fast; ++e) {
    const int m = R.m[e];
    fast = m <= 4 && (m == 0 || (int)R.lc[e][m - 1] - (int)R.lc[e][0] == m - 1);
  }
  R.fast = fast ? 1 : 0;
}

// N floats moved as one vector (a "coil unit": 1 or 2 batch entries)
template <int N>
struct VecF {
  float v[N];
};
template <int N>
__device__ __forceinline__ VecF<N> ldv(const float* p) {
  VecF<N> r;
  if constexpr (N == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
  } else if constexpr (N == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    r.v[0] = t.x; r.v[1] = t.y;
  } else {
    r.v[0] = *p;
  }
  return r;
}
template <int N>
__device__ __forceinline__ void stv(float* p, const VecF<N>& r) {
  if constexpr (N == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  } else if constexpr (N == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(r.v[0], r.v[1]);
  } else {
    *p = r.v[0];
  }
}

// Lane roles: lane = (ux, uz, cu); cu indexes coil units (lowest bits), uz
// the tap along z (4 slots), ux the tap along the split dim (x in 3D, y in
// 2D, more z slots in 1D).
struct Lanes {
  int cu, uz, ux, NUP, UX, lgn;
};
__device__ __forceinline__ Lanes lane_roles(int lane, int nunits) {
  Lanes L;
  L.NUP = nunits <= 1 ? 1 : (nunits <= 2 ? 2 : (nunits <= 4 ? 4 : 8));
  L.lgn = lg2i(L.NUP);
  L.cu = lane & (L.NUP - 1);
  L.uz = (lane >> L.lgn) & 3;
  L.ux = lane >> (L.lgn + 2);
  L.UX = 8 >> L.lgn;
  return L;
}

// Visit the taps of record R assigned to this lane: f(lx, ly, lz, w).
// 3D: x split over ux, z over uz, y looped; 2D: y over ux, z over uz;
// 1D: z over (ux, uz).
template <int NDIM, int NTB, typename F>
__device__ __forceinline__ void for_lane_taps(const Geo& g, const Rec<NTB>& R, const Lanes& L, F&& f) {
  if constexpr (NDIM == 3) {
    for (int kz = L.uz; kz < R.m[2]; kz += 4) {
      const int lz = R.lc[2][kz];
      const float wz = R.wv[2][kz];
      for (int kx = L.ux; kx < R.m[0]; kx += L.UX) {
        const int lx = R.lc[0][kx];
        const float wxz = R.wv[0][kx] * wz;
        for (int ky = 0; ky < R.m[1]; ++ky) {
          const float w = g.norm == 1 ? wxz * R.wv[1][ky] : radial_w(g, R.wv[0][kx], R.wv[1][ky], wz);
          f(lx, (int)R.lc[1][ky], lz, w);
        }
      }
    }
  } else if constexpr (NDIM == 2) {
    for (int kz = L.uz; kz < R.m[2]; kz += 4) {
      const int lz = R.lc[2][kz];
      const float wz = R.wv[2][kz];
      for (int ky = L.ux; ky < R.m[1]; ky += L.UX) {
        const float w = g.norm == 1 ? R.wv[1][ky] * wz : radial_w(g, 0.f, R.wv[1][ky], wz);
        f(0, (int)R.lc[1][ky], lz, w);
      }
    }
  } else {
    for (int kz = L.uz + 4 * L.ux; kz < R.m[2]; kz += 4 * L.UX) {
      const float w = g.norm == 1 ? R.wv[2][kz] : radial_w(g, 0.f, 0.f, R.wv[2][kz]);
      f(0, 0, (int)R.lc[2][kz], w);
    }
  }
}

// ------------------------------------------------------------------ forward

// CTA = NW warps sharing one staged region (tile + halo, [x][y][z][batch]);
// each warp interpolates 32 home points per batch.
template <int N, int NDIM, int NTB, int NW, bool F3>
__global__ void __launch_bounds__(NW * 32, 1) interp_fwd_kernel(Geo g, const int4* __restrict__ items,
                                                                const int32_t* __restrict__ entries,
                                                                const float* __restrict__ locs,
                                                                const float* __restrict__ gridv,
                                                                float* __restrict__ out, int CG) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int es = g.cplx ? 2 : 1;
  const int4 it = items[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c0 = blockIdx.y * CG;
  const int ncoil = (int)min((long long)CG, g.nbatch - c0);
  int tc[3];
  {
    int t = it.x;
    tc[2] = t % g.nt[2];
    t /= g.nt[2];
    tc[1] = t % g.nt[1];
    tc[0] = t / g.nt[1];
  }
  int o[3], S[3];
  for (int e = 0; e < 3; ++e) {
    o[e] = tc[e] * g.T[e];
    S[e] = g.T[e] + g.NT[e] - 1;
  }
  const int vstride = CG * es;  // floats per staged voxel
  float* reg = reinterpret_cast<float*>(smem);
  const size_t reg_bytes = (((size_t)S[0] * S[1] * S[2] * vstride * sizeof(float)) + 15) & ~(size_t)15;
  Rec<NTB>* rbuf = reinterpret_cast<Rec<NTB>*>(smem + reg_bytes) + warp * 32;

  // stage: rows (x, y) per warp, lanes over (z, batch entry), batch fastest
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  const int cgp = CG <= 1 ? 1 : (CG <= 2 ? 2 : (CG <= 4 ? 4 : 8));
  const int lgc = lg2i(cgp);
  const int rowlen = S[2] * cgp;
  for (int row = warp; row < S[0] * S[1]; row += NW) {
    const int x = row / S[1], y = row - x * S[1];
    int gx = o[0] + x, gy = o[1] + y;
    bool rin = true;
    if (g.pad == TLGB_PAD_CIRCULAR) {
      gx = wrapi(gx, g.N[0]);
      gy = wrapi(gy, g.N[1]);
    } else {
      rin = gx < g.N[0] && gy < g.N[1];
    }
    const long long rbase = ((long long)gx * g.N[1] + gy) * g.N[2];
    float* rdst = reg + (size_t)(x * S[1] + y) * S[2] * vstride;
    // all loads of the row first (independent), then the stores
    constexpr int MAXI = 8;
    float2 vv[MAXI];
#pragma unroll
    for (int i = 0; i < MAXI; ++i) {
      vv[i] = make_float2(0.f, 0.f);
      const int idx = lane + 32 * i;
      if (idx < rowlen) {
        const int c = idx & (cgp - 1), z = idx >> lgc;
        int gz = o[2] + z;
        bool in = rin && c < ncoil;
        if (g.pad == TLGB_PAD_CIRCULAR) gz = wrapi(gz, g.N[2]);
        else in = in && gz < g.N[2];
        if (in) {
          const long long gi = (long long)(c0 + c) * gvol + rbase + gz;
          if (es == 2) vv[i] = __ldg(reinterpret_cast<const float2*>(gridv) + gi);
          else vv[i].x = __ldg(gridv + gi);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < MAXI; ++i) {
      const int idx = lane + 32 * i;
      if (idx < rowlen) {
        const int c = idx & (cgp - 1), z = idx >> lgc;
        if (c < CG) {
          float* d = rdst + z * vstride + c * es;
          if (es == 2) *reinterpret_cast<float2*>(d) = vv[i];
          else d[0] = vv[i].x;
        }
      }
    }
    for (int idx = lane + 32 * MAXI; idx < rowlen; idx += 32) {  // long rows (1D tiles)
      const int c = idx & (cgp - 1), z = idx >> lgc;
      if (c >= CG) continue;
      int gz = o[2] + z;
      bool in = rin && c < ncoil;
      if (g.pad == TLGB_PAD_CIRCULAR) gz = wrapi(gz, g.N[2]);
      else in = in && gz < g.N[2];
      float* d = rdst + z * vstride + c * es;
      const long long gi = (long long)(c0 + c) * gvol + rbase + gz;
      if (es == 2) *reinterpret_cast<float2*>(d) = in ? __ldg(reinterpret_cast<const float2*>(gridv) + gi) : make_float2(0.f, 0.f);
      else d[0] = in ? __ldg(gridv + gi) : 0.f;
    }
  }
  __syncthreads();

  const int U = N / es;  // batch entries per unit
  const int nunits = (CG + U - 1) / U;
  const Lanes L = lane_roles(lane, nunits);
  for (int b = it.y + warp * 32; b < it.z; b += NW * 32) {
    const int j = b + lane;
    const int nb = min(32, it.z - b);
    long long p = -1;
    if (j < it.z) {
      p = entries[j];
      float x3[3];
      for (int e = 0; e < 3; ++e) x3[e] = g.act[e] ? load_coord(g, locs, p, e) : 0.f;
      lane_rec<NTB>(g, x3, o, true, rbuf[lane]);
    }
    __syncwarp();
    for (int jj = 0; jj < nb; ++jj) {
      const Rec<NTB>& R = rbuf[jj];
      const long long pj = __shfl_sync(0xffffffffu, p, jj);
      if (R.m[0] == 0) continue;  // warp-uniform
      VecF<N> acc;
#pragma unroll
      for (int i = 0; i < N; ++i) acc.v[i] = 0.f;
      bool done = false;
      if constexpr (F3) {
        // 3D, 8^3 tile + 4-wide halo (12^3 region), 8 complex batch entries
        // (16 floats per voxel), <= 4 taps per dim: unrolled, immediate offsets
        if (R.fast) {
          constexpr int SZ = 16, SY = 12 * 16, SX = 12 * 12 * 16;
          const bool zin = L.uz < R.m[2];
          const float wz = zin ? R.wv[2][L.uz] : 0.f;
          float wy[4];
#pragma unroll
          for (int ky = 0; ky < 4; ++ky) wy[ky] = ky < R.m[1] ? R.wv[1][ky] : 0.f;
          const float* base = reg + (R.lc[0][0] * SX + R.lc[1][0] * SY + (R.lc[2][0] + L.uz) * SZ) + L.cu * 4;
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const int kx = L.ux + 2 * i;
            if (zin && kx < R.m[0]) {
              const float wxz = R.wv[0][kx] * wz;
              const float* bx = base + kx * SX;
#pragma unroll
              for (int ky = 0; ky < 4; ++ky) {
                if (ky < R.m[1]) {
                  const float w = wxz * wy[ky];
                  const float4 v = *reinterpret_cast<const float4*>(bx + ky * SY);
                  acc.v[0] = fmaf(w, v.x, acc.v[0]);
                  acc.v[1] = fmaf(w, v.y, acc.v[1]);
                  acc.v[2] = fmaf(w, v.z, acc.v[2]);
                  acc.v[3] = fmaf(w, v.w, acc.v[3]);
                }
              }
            }
          }
          done = true;
        }
      }
      if (!done && L.cu < nunits) {
        const float* base = reg + L.cu * N;
        for_lane_taps<NDIM, NTB>(g, R, L, [&](int lx, int ly, int lz, float w) {
          const VecF<N> v = ldv<N>(base + ((size_t)(lx * S[1] + ly) * S[2] + lz) * vstride);
#pragma unroll
          for (int i = 0; i < N; ++i) acc.v[i] = fmaf(w, v.v[i], acc.v[i]);
        });
      }
      for (int m = L.NUP; m < 32; m <<= 1)
#pragma unroll
        for (int i = 0; i < N; ++i) acc.v[i] += __shfl_xor_sync(0xffffffffu, acc.v[i], m);
      if (lane < L.NUP && L.cu < nunits) {
#pragma unroll
        for (int u = 0; u < N; u += (N >= 2 && es == 2) ? 2 : 1) {
          const int c = L.cu * U + u / es;
          if (c < ncoil) {
            float* dst = out + ((long long)(c0 + c) * g.npts + pj) * es;
            if (es == 2)
              *reinterpret_cast<float2*>(dst) = make_float2(acc.v[u], acc.v[u + 1]);
            else
              dst[0] = acc.v[u];
          }
        }
      }
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ adjoint

// One warp per CTA owns one output tile in shared memory ([x][y][z][batch]),
// so every cell is updated by one warp in plan order: deterministic.
template <int N, int NDIM, int NTB, bool F3>
__global__ void __launch_bounds__(32) interp_adj_kernel(Geo g, const int4* __restrict__ items,
                                                        const int32_t* __restrict__ entries,
                                                        const float* __restrict__ locs,
                                                        const float* __restrict__ vals, float* __restrict__ gridv,
                                                        float* __restrict__ partial, int CG) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int es = g.cplx ? 2 : 1;
  const int4 it = items[blockIdx.x];
  const int lane = threadIdx.x;
  const int cg = blockIdx.y;
  const int c0 = cg * CG;
  const int ncoil = (int)min((long long)CG, g.nbatch - c0);
  int tc[3];
  {
    int t = it.x;
    tc[2] = t % g.nt[2];
    t /= g.nt[2];
    tc[1] = t % g.nt[1];
    tc[0] = t / g.nt[1];
  }
  int o[3];
  for (int e = 0; e < 3; ++e) o[e] = tc[e] * g.T[e];
  const int T1 = g.T[1], T2 = g.T[2];
  const int tvol = g.T[0] * T1 * T2;
  const int vstride = CG * es;
  const int tfl = (tvol * vstride + 3) & ~3;  // tile floats, rounded to whole float4
  float* acc = reinterpret_cast<float*>(smem);
  Rec<NTB>* rbuf = reinterpret_cast<Rec<NTB>*>(smem + (size_t)tfl * sizeof(float));
  float* pv = reinterpret_cast<float*>(rbuf + 32);  // [32][vstride]
  for (int i = lane * 4; i < tfl; i += 128) *reinterpret_cast<float4*>(acc + i) = make_float4(0.f, 0.f, 0.f, 0.f);

  const int U = N / es;
  const int nunits = (CG + U - 1) / U;
  const Lanes L = lane_roles(lane, nunits);

  // registers of the next batch (prefetched while the current one is spread)
  long long np_ = -1;
  float nx3[3] = {0.f, 0.f, 0.f};
  float nv[2 * CGMAX];
  auto prefetch = [&](int b) {
    const int j = b + lane;
    np_ = -1;
    if (j < it.z) {
      np_ = entries[j];
      for (int e = 0; e < 3; ++e) nx3[e] = g.act[e] ? load_coord(g, locs, np_, e) : 0.f;
#pragma unroll
      for (int c = 0; c < CGMAX; ++c) {
        if (c < ncoil) {
          if (es == 2) {
            const float2 v = __ldg(reinterpret_cast<const float2*>(vals) + (long long)(c0 + c) * g.npts + np_);
            nv[2 * c] = v.x;
            nv[2 * c + 1] = v.y;
          } else {
            nv[c] = __ldg(vals + (long long)(c0 + c) * g.npts + np_);
          }
        }
      }
    }
  };
  if (it.y < it.z) prefetch(it.y);
  for (int b = it.y; b < it.z; b += 32) {
    const int nb = min(32, it.z - b);
    __syncwarp();
    if (np_ >= 0) {
      lane_rec<NTB>(g, nx3, o, false, rbuf[lane]);
#pragma unroll
      for (int c = 0; c < CGMAX; ++c)
        if (c < CG) {
          if (es == 2) {
            pv[lane * vstride + 2 * c] = c < ncoil ? nv[2 * c] : 0.f;
            pv[lane * vstride + 2 * c + 1] = c < ncoil ? nv[2 * c + 1] : 0.f;
          } else {
            pv[lane * vstride + c] = c < ncoil ? nv[c] : 0.f;
          }
        }
    }
    __syncwarp();
    if (b + 32 < it.z) prefetch(b + 32);
    for (int jj = 0; jj < nb; ++jj) {
      const Rec<NTB>& R = rbuf[jj];
      // lanes of one warp update cells of consecutive points: order them
      __syncwarp();
      if (R.m[0] == 0 || L.cu >= nunits) continue;
      const VecF<N> v = ldv<N>(pv + jj * vstride + L.cu * N);
      float* base = acc + L.cu * N;
      if constexpr (F3) {
        // 3D, 8^3 tile, 8 complex batch entries (16 floats per cell), <= 4
        // taps per dim at consecutive cells: unrolled, immediate offsets
        if (R.fast && g.wrap_safe) {
          constexpr int SZ = 16, SY = 8 * 16, SX = 8 * 8 * 16;
          const bool zin = L.uz < R.m[2];
          const float wz = zin ? R.wv[2][L.uz] : 0.f;
          float wy[4];
#pragma unroll
          for (int ky = 0; ky < 4; ++ky) wy[ky] = ky < R.m[1] ? R.wv[1][ky] : 0.f;
          float* b0 = base + (R.lc[0][0] * SX + R.lc[1][0] * SY + (R.lc[2][0] + L.uz) * SZ);
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const int kx = L.ux + 2 * i;
            if (zin && kx < R.m[0]) {
              const float wxz = R.wv[0][kx] * wz;
              float* bx = b0 + kx * SX;
              float4 r[4];
#pragma unroll
              for (int ky = 0; ky < 4; ++ky)
                if (ky < R.m[1]) r[ky] = *reinterpret_cast<const float4*>(bx + ky * SY);
#pragma unroll
              for (int ky = 0; ky < 4; ++ky) {
                if (ky < R.m[1]) {
                  const float w = wxz * wy[ky];
                  r[ky].x = fmaf(w, v.v[0], r[ky].x);
                  r[ky].y = fmaf(w, v.v[1], r[ky].y);
                  r[ky].z = fmaf(w, v.v[2], r[ky].z);
                  r[ky].w = fmaf(w, v.v[3], r[ky].w);
                  *reinterpret_cast<float4*>(bx + ky * SY) = r[ky];
                }
              }
            }
          }
          continue;
        }
      }
      if (g.wrap_safe) {
        for_lane_taps<NDIM, NTB>(g, R, L, [&](int lx, int ly, int lz, float w) {
          float* a = base + ((size_t)(lx * T1 + ly) * T2 + lz) * vstride;
          VecF<N> r = ldv<N>(a);
#pragma unroll
          for (int i = 0; i < N; ++i) r.v[i] = fmaf(w, v.v[i], r.v[i]);
          stv<N>(a, r);
        });
      } else if (L.ux == 0 && L.uz == 0) {
        // a window longer than the grid reaches a cell twice: taps in order,
        // lanes split by coil unit only
        for (int kx = 0; kx < R.m[0]; ++kx)
          for (int ky = 0; ky < R.m[1]; ++ky)
            for (int kz = 0; kz < R.m[2]; ++kz) {
              const float w = g.norm == 1 ? R.wv[0][kx] * R.wv[1][ky] * R.wv[2][kz]
                                          : radial_w(g, R.wv[0][kx], R.wv[1][ky], R.wv[2][kz]);
              float* a = base + ((size_t)(R.lc[0][kx] * T1 + R.lc[1][ky]) * T2 + R.lc[2][kz]) * vstride;
              VecF<N> r = ldv<N>(a);
#pragma unroll
              for (int i = 0; i < N; ++i) r.v[i] = fmaf(w, v.v[i], r.v[i]);
              stv<N>(a, r);
            }
      }
    }
  }
  __syncwarp();
  if (it.w >= 0) {
    float* dst = partial + ((long long)it.w * gridDim.y + cg) * tfl;
    for (int i = lane * 4; i < tfl; i += 128)
      *reinterpret_cast<float4*>(dst + i) = *reinterpret_cast<const float4*>(acc + i);
    return;
  }
  // write the tile: per (x, y) row, lanes over (batch entry, z) with the
  // batch entry fastest, so shared-memory reads are contiguous
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  const int cgp = CG <= 1 ? 1 : (CG <= 2 ? 2 : (CG <= 4 ? 4 : 8));
  const int lgc = lg2i(cgp);
  for (int row = 0; row < g.T[0] * T1; ++row) {
    const int x = row / T1, y = row - x * T1;
    const int gx = o[0] + x, gy = o[1] + y;
    if (gx >= g.N[0] || gy >= g.N[1]) continue;
    const float* srow = acc + (size_t)(x * T1 + y) * T2 * vstride;
    float* drow = gridv + (((long long)gx * g.N[1] + gy) * g.N[2] + o[2]) * es;
    for (int idx = lane; idx < T2 * cgp; idx += 32) {
      const int cc = idx & (cgp - 1);
      const int z = idx >> lgc;
      if (cc >= ncoil || o[2] + z >= g.N[2]) continue;
      const float* sp = srow + z * vstride + cc * es;
      float* d = drow + ((long long)(c0 + cc) * gvol + z) * es;
      if (es == 2)
        *reinterpret_cast<float2*>(d) = *reinterpret_cast<const float2*>(sp);
      else
        d[0] = sp[0];
    }
  }
}

// ----------------------------------------- unrolled kernels of the 3D default
//
// 3D grids, 8^3 tiles, widths in (3, 4] (5 tap slots, <= 4 kept for
// non-integer coordinates), 8 complex batch entries per CTA: the benchmark
// configuration and the NUFFT default. Each point's taps are packed into a
// 64-byte record read with vector loads; tap offsets are compile-time.

// KB value for the weights only (the tap masks stay exact): the same A&S
// expansions as kb_value evaluated with the approximate square root, divide
// and exponential intrinsics; agrees with kb_value to ~3e-7 relative.
__device__ __forceinline__ float kb_approx(float ax, float beta) {
  const float u1 = __fsub_rn(1.0f, __fmul_rn(ax, ax));
  const float z = beta * (u1 > 0.f ? u1 * rsqrtf(u1) : 0.f);
  if (z < 3.75f) {
    const float u = (z * (1.0f / 3.75f)) * (z * (1.0f / 3.75f));
    return 1.0f + u * (3.5156229f + u * (3.0899424f + u * (1.2067492f + u * (0.2659732f +
           u * (0.0360768f + u * 0.0045813f)))));
  }
  const float rz = __frcp_rn(z);
  const float v = 3.75f * rz;
  const float q = 0.39894228f + v * (0.01328592f + v * (0.00225319f + v * (-0.00157565f + v * (0.00916281f +
                  v * (-0.02057706f + v * (0.02635537f + v * (-0.01647633f + v * 0.00392377f)))))));
  return __expf(z) * rsqrtf(z) * q;
}

// A staged entry of the 3D 8-entry kernels in shared memory: the point's
// weights, its view word (grid_view or region_view) and the point index.
struct __align__(16) R3 {
  float4 w[3];
  unsigned view;
  int pad0, pad1;
  int p;  // point index
};

// Per-point tap record, built with the plan for 3D geometries with 8^3 tiles
// and at most 5 taps per dimension: the kernel weights of the first 4 valid
// taps of each dimension (zero beyond), the position of the first valid tap
// (wrapped into [0, N) in circular mode) and the number of valid taps per
// dimension (cnt_x | cnt_y << 4 | cnt_z << 8; a zero count marks a point
// without taps). Valid taps form one run of tap indices: |x - g| <= W/2 is
// an interval, and so is [0, N) for zero padding.
struct __align__(16) PRec {
  float4 w[3];
  int st[3];
  int cnt;
};
static_assert(sizeof(PRec) == 64, "64-byte point records");

__global__ void point_records_kernel(Geo g, const float* __restrict__ locs, PRec* __restrict__ out) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  PRec R;
  int cnt = 0;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    float w0 = 0.f, w1 = 0.f, w2 = 0.f, w3 = 0.f;
    int c = 0, st = 0;
    if (!g.act[e]) {
      // a leading dimension of a 2D geometry: one tap of weight 1 at 0
      R.w[e] = make_float4(1.f, 0.f, 0.f, 0.f);
      R.st[e] = 0;
      cnt |= 1 << (4 * e);
      continue;
    }
    const float x = load_coord(g, locs, p, e);
    if (coord_ok(x)) {
      const int lower = lower_of(g, e, x);
      int s = -1;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const Tap t = tap_eval(g, e, x, lower, k);
        if (t.valid) {
          if (s < 0) s = k;
          const float v = kern_value_approx(g.kernel, fabsf(t.d), g.beta);
          w0 = c == 0 ? v : w0;
          w1 = c == 1 ? v : w1;
          w2 = c == 2 ? v : w2;
          w3 = c == 3 ? v : w3;
          ++c;
        }
      }
      if (c > 0) {
        st = lower + s;
        if (g.pad == TLGB_PAD_CIRCULAR) st = wrapi(st, g.N[e]);
      }
    }
    R.w[e] = make_float4(w0, w1, w2, w3);
    R.st[e] = st;
    cnt |= c << (4 * e);
  }
  R.cnt = cnt;
  out[p] = R;
}

// ------------------------------------------------ block lists (3D gridding)
//
// The 8-entry gridding works on output blocks of 4 x 4 x 4 cells in 3D and
// 8 x 8 cells in 2D (64 cells either way). A window of 4 taps per dimension
// meets 1.75 blocks of 4 (1.375 of 8) per dimension on average, and one warp
// holds a whole block for 8 entries. The plan lists per block the points
// whose window meets it, in point order.
constexpr int kBlkPart = 256;  // entries per work item: denser blocks are split into parts
constexpr int kZeroRun = 16;   // empty blocks written by one work item
constexpr int kCube = 4;       // blocks per edge of the cubes the gridding items visit in turn
constexpr int kSelShift = 29;  // entry = point | (its block's index per dim, 3 bits) << 29

// block edge along internal dim e: 4 in 3D; 8 along the two dims of a 2D
// grid (1 along its inactive leading dim)
__host__ __device__ __forceinline__ int block_edge(int ndim, int e) { return ndim == 3 ? 4 : (e == 0 ? 1 : 8); }
__host__ __device__ __forceinline__ int blocks_along(int n, int edge) { return (n + edge - 1) / edge; }
__host__ __device__ __forceinline__ int blocks_along(const Geo& g, int e) {
  return blocks_along(g.N[e], block_edge(g.ndim, e));
}
// floats of tap rows per point: 2 rows per active dim, one weight per cell
__host__ __device__ __forceinline__ int row_floats(int ndim) { return ndim == 3 ? 24 : 32; }

// Distinct blocks met along one dim by the cells st .. st+c-1 of a window
// (st in [0, N); wrapped once in circular mode, where N >= 16 > c). At most
// 2: 5 taps over blocks of 4 or 8 cells (circular grids are multiples of the
// block edge).
__device__ __forceinline__ int axis_blocks(const Geo& g, int e, int st, int c, int* bl) {
  const int edge = block_edge(g.ndim, e);
  int cnt = 0;
  for (int k = 0; k < c; ++k) {
    int v = st + k;
    if (v >= g.N[e]) v -= g.N[e];
    const int b = v / edge;
    bool seen = false;
    for (int i = 0; i < cnt; ++i) seen = seen || bl[i] == b;
    if (!seen && cnt < 3) bl[cnt++] = b;
  }
  return cnt;
}

__global__ void blk_count_kernel(Geo g, const PRec* __restrict__ precs, uint32_t* __restrict__ cnt) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  const PRec R = precs[p];
  uint32_t c = 1;
  for (int e = 0; e < 3; ++e) {
    const int ce = (R.cnt >> (4 * e)) & 15;
    int bl[3];
    c *= ce ? (uint32_t)axis_blocks(g, e, R.st[e], ce, bl) : 0u;
  }
  cnt[p] = c;
}

__global__ void blk_emit_kernel(Geo g, const PRec* __restrict__ precs, const uint32_t* __restrict__ off,
                                uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  const PRec R = precs[p];
  int bl[3][3], nc[3];
  for (int e = 0; e < 3; ++e) {
    const int ce = (R.cnt >> (4 * e)) & 15;
    if (!ce) return;
    nc[e] = axis_blocks(g, e, R.st[e], ce, bl[e]);
  }
  const uint32_t nb1 = (uint32_t)blocks_along(g, 1), nb2 = (uint32_t)blocks_along(g, 2);
  uint32_t o = off[p];
  for (int i = 0; i < nc[0]; ++i)
    for (int j = 0; j < nc[1]; ++j)
      for (int k = 0; k < nc[2]; ++k) {
        keys[o] = ((uint32_t)bl[0][i] * nb1 + (uint32_t)bl[1][j]) * nb2 + (uint32_t)bl[2][k];
        vals[o] = (int32_t)((uint32_t)p | (uint32_t)(i | j << 1 | k << 2) << kSelShift);
        ++o;
      }
}

// The tap weights of a point over each block it meets: per active dim the
// rows of its first and second block (in axis_blocks order), one weight per
// cell of the block (4 in 3D, 8 in 2D), from the coordinate as the tap
// records; a cell outside the window holds -0.0 (valid weights are >= +0), so
// the sign bit tells the gridding which cells the window covers.
__global__ void blk_rows_kernel(Geo g, const float* __restrict__ locs, const PRec* __restrict__ precs,
                                float* __restrict__ rows) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  const PRec R = precs[p];
  float* out = rows + p * row_floats(g.ndim);
  for (int e = 3 - g.ndim; e < 3; ++e) {
    const int edge = block_edge(g.ndim, e);
    const int ce = (R.cnt >> (4 * e)) & 15;
    int bl[3] = {0, 0, 0};
    const int nb = ce ? axis_blocks(g, e, R.st[e], ce, bl) : 0;
    const float x = load_coord(g, locs, p, e);
    const int lower = coord_ok(x) ? lower_of(g, e, x) : 0;
    for (int i = 0; i < 2; ++i) {
      for (int q = 0; q < edge; ++q) {
        const int v = edge * bl[i] + q;
        int k = v - lower;
        if (g.pad == TLGB_PAD_CIRCULAR) k = wrapi(k, g.N[e]);
        float w = -0.0f;
        if (i < nb && v < g.N[e] && k >= 0 && k < g.NT[e]) {
          const Tap t = tap_eval(g, e, x, lower, k);
          if (t.valid) w = kern_value_approx(g.kernel, fabsf(t.d), g.beta);
        }
        *out++ = w;
      }
    }
  }
}

// View of one dimension of a record from the tile at o (8 wide, grid N):
// f = first local position, m = taps inside the tile, k0 = index of the
// first of them in the record; packed f | m << 3 | k0 << 6. fast is cleared
// when the window has 5 taps or, in circular mode on a grid below 16, could
// meet the tile twice.
__device__ __forceinline__ int tile_view(int st, int c, int o, int N, bool circ, bool& fast) {
  const int te = min(8, N - o);
  int d = st - o;
  if (circ && d < 0) d += N;
  int f, k0, m;
  if (d >= 0 && d < te) {
    f = d;
    k0 = 0;
    m = min(c, te - d);
  } else {
    f = 0;
    k0 = circ ? N - d : -d;  // the window enters from below (wrapping around in circular mode)
    m = (d >= te && !circ) ? 0 : min(c - k0, te);
  }
  if (m < 0 || k0 < 0) m = 0, k0 = 0;
  if (c > 4 || (circ && N < 16)) fast = false;
  return f | (m << 3) | (min(k0, 7) << 6);
}

// The gridding view of a point record in the tile at o, as one word: three
// 9-bit tile views (x, y, z) | fast << 27 | ok << 28.
__device__ __forceinline__ unsigned grid_view(const Geo& g, const PRec& R, const int (&o)[3]) {
  bool fast = true;
  const bool circ = g.pad == TLGB_PAD_CIRCULAR;
  const int c = R.cnt;
  const bool ok = (c & 15) && ((c >> 4) & 15) && ((c >> 8) & 15);
  unsigned v = 0;
#pragma unroll
  for (int e = 0; e < 3; ++e) v |= (unsigned)tile_view(R.st[e], (c >> (4 * e)) & 15, o[e], g.N[e], circ, fast) << (9 * e);
  return v | ((fast ? 1u : 0u) << 27) | ((ok ? 1u : 0u) << 28);
}

// The gather view of a home record in the 12^3 region at o: region base
// (11 bits) | mx << 11 | my << 14 | mz << 17 | fast << 20 | ok << 21. The
// region is staged with wrap, so the window is always one run there.
__device__ __forceinline__ unsigned region_view(const Geo& g, const PRec& R, const int (&o)[3]) {
  const int c = R.cnt;
  const int cx = c & 15, cy = (c >> 4) & 15, cz = (c >> 8) & 15;
  const bool ok = cx && cy && cz;
  int f[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    int d = R.st[e] - o[e];
    if (g.pad == TLGB_PAD_CIRCULAR && d < 0) d += g.N[e];
    f[e] = d;
  }
  const bool fast = ok && cx <= 4 && cy <= 4 && cz <= 4 && f[0] >= 0 && f[0] < 8 && f[1] >= 0 && f[1] < 8 &&
                    f[2] >= 0 && f[2] < 8;
  const unsigned base = fast ? (unsigned)((f[0] * 12 + f[1]) * 12 + f[2]) : 0u;
  return base | (min(cx, 7) << 11) | (min(cy, 7) << 14) | (min(cz, 7) << 17) | ((fast ? 1u : 0u) << 20) |
         ((ok ? 1u : 0u) << 21);
}

__device__ __forceinline__ PRec load_prec(const PRec* __restrict__ recs, long long p) {
  const float4* q = reinterpret_cast<const float4*>(recs + p);
  PRec R;
  R.w[0] = __ldg(q);
  R.w[1] = __ldg(q + 1);
  R.w[2] = __ldg(q + 2);
  const int4 t = __ldg(reinterpret_cast<const int4*>(q + 3));
  R.st[0] = t.x;
  R.st[1] = t.y;
  R.st[2] = t.z;
  R.cnt = t.w;
  return R;
}

// Compensated summation (Neumaier's variant of Kahan's method): s + c
// carries the running sum; c collects the low-order bits each addition
// loses, whichever operand is larger.
__device__ __forceinline__ void comp_add(float& s, float& c, float x) {
  const float t = s + x;
  c += fabsf(s) >= fabsf(x) ? (s - t) + x : (x - t) + s;
  s = t;
}

__device__ __forceinline__ float pick4(const float4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

using sm100::fence_mbar_init;
using sm100::mbar_arrive_expect_tx;
using sm100::mbar_init;
using sm100::mbar_wait_bounded;
using sm100::smem_u32;
using sm100::tma_load_4d;

// device status word: set when a bounded wait gave up (see tlgb_interp_forward)
__device__ int g_tlgb_status;

// Point values [batch][npts] (complex) -> point-major [group][npts][8]: the
// gridding reads 64 contiguous bytes per (point, tile) pair instead of 8
// scattered 8-byte values. CTA = 128 points x 8 entries of one group: warp c
// loads entry c two points per 16-byte load (when the rows are 16-byte
// aligned), each thread stores two 16-byte pairs of entries; 32 bytes in
// flight per thread each way. Block (0, group) also zeroes the group's work
// counter of the gridding launched after it (ctr, when given).
constexpr int kTrPts = 128;
__global__ void __launch_bounds__(256) transpose_vals_kernel(const float2* __restrict__ vals, long long npts,
                                                             long long nbatch, float2* __restrict__ tv,
                                                             int* __restrict__ ctr) {
  __shared__ __align__(16) float2 sm[kTrPts][10];  // rows of 80 bytes: entry pairs 16-byte aligned
  const int grp = blockIdx.y;
  const long long p0 = (long long)blockIdx.x * kTrPts;
  const int t = threadIdx.x;
  if (ctr && blockIdx.x == 0 && t == 0) ctr[grp] = 0;
  {
    const int c = t >> 5, lane = t & 31;
    const long long cc = (long long)grp * 8 + c;
    const float2* src = vals + cc * npts;
    const bool vec = ((reinterpret_cast<uintptr_t>(vals) | (uintptr_t)(npts * 8)) & 15) == 0;
    float2 a[2], b[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long p = p0 + h * 64 + 2 * lane;
      a[h] = b[h] = make_float2(0.f, 0.f);
      if (cc < nbatch) {
        if (vec && p + 1 < npts) {
          const float4 v = __ldg(reinterpret_cast<const float4*>(src + p));
          a[h] = make_float2(v.x, v.y), b[h] = make_float2(v.z, v.w);
        } else {
          if (p < npts) a[h] = __ldg(src + p);
          if (p + 1 < npts) b[h] = __ldg(src + p + 1);
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      sm[h * 64 + 2 * lane][c] = a[h];
      sm[h * 64 + 2 * lane + 1][c] = b[h];
    }
  }
  __syncthreads();
  float4* dst = reinterpret_cast<float4*>(tv) + (long long)grp * npts * 4;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int j = h * 256 + t, i = j >> 2, q = j & 3;  // point i, entries 2q and 2q + 1
    const long long p = p0 + i;
    if (p < npts) dst[p * 4 + q] = *reinterpret_cast<const float4*>(&sm[i][2 * q]);
  }
}

// Sum the partial tiles of one split tile (8^3 x 8 entries) in slot order,
// compensated (the dense k-space centre piles thousands of points onto a
// cell; each partial holds at most one chunk of them). CTA = one x-plane
// (blockIdx.z) of one split tile: 256 threads x one float4 of the plane per
// partial, four partials in flight; then warp w writes row y = w of the
// plane, lane = (entry, z pair), 16 bytes per lane.
__global__ void __launch_bounds__(256) adj_reduce_f3_kernel(Geo g, const int4* __restrict__ split,
                                                            const float* __restrict__ partial,
                                                            float* __restrict__ gridv) {
  constexpr int TFL = 512 * 16, PFL = 64 * 16, VS = 16;
  __shared__ __align__(16) float acc[PFL];
  const int4 sp = split[blockIdx.x];
  const int cg = blockIdx.y, ncg = gridDim.y, x = blockIdx.z;
  const int c0 = cg * 8;
  const int ncoil = (int)min(8ll, g.nbatch - c0);
  int o[3];
  {
    int t = sp.x;
    o[2] = (t % g.nt[2]) * 8;
    t /= g.nt[2];
    o[1] = (t % g.nt[1]) * 8;
    o[0] = (t / g.nt[1]) * 8;
  }
  const int tid = threadIdx.x;
  const long long step = (long long)ncg * TFL / 4;  // float4s between consecutive partials
  const float4* src = reinterpret_cast<const float4*>(partial + ((long long)sp.y * ncg + cg) * TFL + x * PFL) + tid;
  float4 sum = __ldg(src), comp = make_float4(0.f, 0.f, 0.f, 0.f);
  int k = 1;
  for (; k + 4 <= sp.z; k += 4) {
    float4 v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __ldg(src + (k + i) * step);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      comp_add(sum.x, comp.x, v[i].x);
      comp_add(sum.y, comp.y, v[i].y);
      comp_add(sum.z, comp.z, v[i].z);
      comp_add(sum.w, comp.w, v[i].w);
    }
  }
  for (; k < sp.z; ++k) {
    const float4 v = __ldg(src + k * step);
    comp_add(sum.x, comp.x, v.x);
    comp_add(sum.y, comp.y, v.y);
    comp_add(sum.z, comp.z, v.z);
    comp_add(sum.w, comp.w, v.w);
  }
  reinterpret_cast<float4*>(acc)[tid] =
      make_float4(sum.x + comp.x, sum.y + comp.y, sum.z + comp.z, sum.w + comp.w);
  __syncthreads();
  const int yy = tid >> 5, lane = tid & 31;
  const int gx = o[0] + x, gy = o[1] + yy;
  if (gx >= g.N[0] || gy >= g.N[1]) return;
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  const int c = lane >> 2, zp = lane & 3;
  if (c >= ncoil) return;
  const float* srow = acc + yy * 8 * VS;
  const float2 a0 = *reinterpret_cast<const float2*>(srow + (2 * zp) * VS + c * 2);
  const float2 a1 = *reinterpret_cast<const float2*>(srow + (2 * zp + 1) * VS + c * 2);
  float* drow = gridv + ((long long)(c0 + c) * gvol + ((long long)gx * g.N[1] + gy) * g.N[2] + o[2]) * 2;
  // 16-byte stores need an even Z extent (row starts at even elements) and an aligned base
  const bool vec = o[2] + 8 <= g.N[2] && (g.N[2] & 1) == 0 && (reinterpret_cast<uintptr_t>(gridv) & 15) == 0;
  if (vec) {
    *reinterpret_cast<float4*>(drow + 4 * zp) = make_float4(a0.x, a0.y, a1.x, a1.y);
  } else {
    if (o[2] + 2 * zp < g.N[2]) *reinterpret_cast<float2*>(drow + 4 * zp) = a0;
    if (o[2] + 2 * zp + 1 < g.N[2]) *reinterpret_cast<float2*>(drow + 4 * zp + 2) = a1;
  }
}

// Packed single-precision arithmetic of sm_100+ (two independent IEEE fp32
// operations, round to nearest: the same results as two scalar ones).
__device__ __forceinline__ unsigned long long f2_bits(float2 v) { return *reinterpret_cast<unsigned long long*>(&v); }
__device__ __forceinline__ float2 bits_f2(unsigned long long b) { return *reinterpret_cast<float2*>(&b); }
// acc += (w, w) * v
__device__ __forceinline__ void fma2_bcast(float2& acc, float w, float2 v) {
  unsigned long long a = f2_bits(acc);
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(a) : "l"(f2_bits(make_float2(w, w))), "l"(f2_bits(v)));
  acc = bits_f2(a);
}
// (s, s) * v
__device__ __forceinline__ float2 mul2_bcast(float s, float2 v) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(make_float2(s, s))), "l"(f2_bits(v)));
  return bits_f2(r);
}

// Gridding: CTA = 8 warps owning one 8^3 x 8-entry output tile, held in
// registers: warp w owns x-plane w, lane (y, entry quad, z pair) the cells
// (w, y, z) for z in {2 zp, 2 zp + 1, 2 zp + 4, 2 zp + 5} and 4 of the 8
// entries, so no two threads update the same value. Entries are staged in
// batches of kAB, one thread per entry: its 8 point values, its view of the
// tile turned into three rows of tap weights (8 per dimension, zero where
// the window has no tap), and per plane a bitmask of the entries with taps
// in it (warp ballots). Each warp then applies its plane's entries in plan
// order, one packed (re, im) FMA per cell and entry, then the entries that
// need the generic record, also in order. The finished tile is stored from
// registers.
constexpr int kAB = 256;

// Rows are padded (28 and 20 floats) so that the staging threads' 16-byte
// stores, one row per thread, spread over all banks.
struct AdjStage {
  float wrow[kAB][28];  // tap weights at tile-local x (0-7), y (8-15), z (16-23)
  float pv[kAB][20];    // point values, 8 entries complex (16 floats)
  int pidx[kAB];
  unsigned fmask[8][kAB / 32];  // per plane: entries on the row path with taps there
  unsigned smask[kAB / 32];     // entries on the generic path (all planes)
};

static_assert(kAB == 256, "one staged pair per thread of the 8 warps; every warp owns a mask word");
constexpr size_t adj_f3_smem() { return sizeof(AdjStage) + 8 * sizeof(Rec<5>); }

__global__ void __launch_bounds__(256, 4) adj_f3_kernel(Geo g, const int4* __restrict__ items,
                                                        const int32_t* __restrict__ entries,
                                                        const PRec* __restrict__ precs,
                                                        const float* __restrict__ locs, const float* __restrict__ vals,
                                                        const float4* __restrict__ tv, float* __restrict__ gridv,
                                                        float* __restrict__ partial) {
  constexpr int CG = 8, VS = 16, TFL = 512 * 16, NW = 8, MW = kAB / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  AdjStage& S = *reinterpret_cast<AdjStage*>(smem);
  Rec<5>* slow = reinterpret_cast<Rec<5>*>(smem + sizeof(AdjStage));  // [NW]
  const int4 it = items[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cg = blockIdx.y;
  const int c0 = cg * CG;
  const int ncoil = (int)min((long long)CG, g.nbatch - c0);
  int o[3];
  {
    int t = it.x;
    o[2] = (t % g.nt[2]) * 8;
    t /= g.nt[2];
    o[1] = (t % g.nt[1]) * 8;
    o[0] = (t / g.nt[1]) * 8;
  }
  const int y = lane >> 2, cq = (lane >> 1) & 1, zp = lane & 1;
  float2 acc[4][4];  // [z slot: 2zp, 2zp+1, 2zp+4, 2zp+5][entry 4cq + k]
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[q][k] = make_float2(0.f, 0.f);
  for (int b = it.y; b < it.z; b += kAB) {
    const int nb = min(kAB, it.z - b);
    __syncthreads();  // the previous batch has been applied
    {
      // entry tid: record and point values -> view -> rows of tap weights;
      // ballots per plane. Entries with a non-finite value take the generic
      // path, which touches only the cells of the window, as the row path's
      // zero weights would not keep a NaN or Inf out of the other cells.
      unsigned view = 0;
      bool finite = true;
      if (tid < nb && TLGB_IN_RANGE(entries[b + tid], g.npts)) {
        const int p = entries[b + tid];
        const PRec R = load_prec(precs, p);
        float4 v[4];
        if (tv) {
          const float4* src = tv + ((long long)cg * g.npts + p) * 4;
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = __ldg(src + q);
        } else {
          const float2* v2 = reinterpret_cast<const float2*>(vals);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int c = 2 * q;
            const float2 a = c < ncoil ? __ldg(v2 + (long long)(c0 + c) * g.npts + p) : make_float2(0.f, 0.f);
            const float2 d = c + 1 < ncoil ? __ldg(v2 + (long long)(c0 + c + 1) * g.npts + p) : make_float2(0.f, 0.f);
            v[q] = make_float4(a.x, a.y, d.x, d.y);
          }
        }
        float4* pd = reinterpret_cast<float4*>(&S.pv[tid][0]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          pd[q] = v[q];
          finite = finite && isfinite(v[q].x) && isfinite(v[q].y) && isfinite(v[q].z) && isfinite(v[q].w);
        }
        view = grid_view(g, R, o);
        S.pidx[tid] = p;
        if (((view >> 27) & 1) && finite) {
#pragma unroll
          for (int e = 0; e < 3; ++e) {
            const unsigned u = (view >> (9 * e)) & 511;
            const int f = u & 7, m = (u >> 3) & 7, k0 = u >> 6;
            float r[8];
#pragma unroll
            for (int l = 0; l < 8; ++l) {
              const int k = l - f;
              r[l] = (k >= 0 && k < m) ? pick4(R.w[e], k0 + k) : 0.f;
            }
            float4* d = reinterpret_cast<float4*>(&S.wrow[tid][8 * e]);
            d[0] = make_float4(r[0], r[1], r[2], r[3]);
            d[1] = make_float4(r[4], r[5], r[6], r[7]);
          }
        }
      }
      const bool ok = (view >> 28) & 1, fast = ((view >> 27) & 1) && finite;
      const int f = view & 7, n = (view >> 3) & 7;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const unsigned bal = __ballot_sync(0xffffffffu, ok && fast && w >= f && w < f + n);
        if (lane == 0) S.fmask[w][warp] = bal;
      }
      const unsigned bs = __ballot_sync(0xffffffffu, ok && !fast);
      if (lane == 0) S.smask[warp] = bs;
    }
    __syncthreads();
    // row path: every lane updates its 4 cells x 4 entries (zero weights
    // outside the window), one entry at a time in entry order (at 64
    // registers 4 CTAs fit per SM; that beats two entries per step at 3)
    struct Visit {
      float2 wa, wb;  // weights of the lane's z slots
      float4 v0, v1;  // the lane's 4 entries, complex
    };
    auto fetch = [&](int j) {
      const float* wr = S.wrow[j];
      const float wxy = wr[warp] * wr[8 + y];
      Visit d;
      d.wa = mul2_bcast(wxy, *reinterpret_cast<const float2*>(wr + 16 + 2 * zp));
      d.wb = mul2_bcast(wxy, *reinterpret_cast<const float2*>(wr + 20 + 2 * zp));
      d.v0 = *reinterpret_cast<const float4*>(&S.pv[j][8 * cq]);
      d.v1 = *reinterpret_cast<const float4*>(&S.pv[j][8 * cq + 4]);
      return d;
    };
    auto apply = [&](const Visit& d) {
      const float2 v[4] = {make_float2(d.v0.x, d.v0.y), make_float2(d.v0.z, d.v0.w), make_float2(d.v1.x, d.v1.y),
                           make_float2(d.v1.z, d.v1.w)};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        fma2_bcast(acc[0][k], d.wa.x, v[k]);
        fma2_bcast(acc[1][k], d.wa.y, v[k]);
        fma2_bcast(acc[2][k], d.wb.x, v[k]);
        fma2_bcast(acc[3][k], d.wb.y, v[k]);
      }
    };
#pragma unroll 1
    for (int mw = 0; mw < MW; ++mw) {
      unsigned bits = S.fmask[warp][mw];
      while (bits) {
        const int j0 = mw * 32 + __ffs(bits) - 1;
        bits &= bits - 1;
        apply(fetch(j0));
      }
    }
    // generic path: exact-integer coordinates (5 taps) or a window wrapping
    // inside the tile; the record is rebuilt from the coordinates by lane 0
#pragma unroll 1
    for (int mw = 0; mw < MW; ++mw) {
      unsigned bits = S.smask[mw];
      while (bits) {
        const int j = mw * 32 + __ffs(bits) - 1;
        bits &= bits - 1;
        __syncwarp();  // the previous record has been read
        if (lane == 0) {
          float x3[3];
          for (int e = 0; e < 3; ++e) x3[e] = load_coord(g, locs, S.pidx[j], e);
          lane_rec<5>(g, x3, o, false, slow[warp]);
        }
        __syncwarp();
        const Rec<5>& Q = slow[warp];
        const float4 v0 = *reinterpret_cast<const float4*>(&S.pv[j][8 * cq]);
        const float4 v1 = *reinterpret_cast<const float4*>(&S.pv[j][8 * cq + 4]);
        const float2 v[4] = {make_float2(v0.x, v0.y), make_float2(v0.z, v0.w), make_float2(v1.x, v1.y),
                             make_float2(v1.z, v1.w)};
        for (int kx = 0; kx < Q.m[0]; ++kx) {
          if (Q.lc[0][kx] != warp) continue;
          for (int kyy = 0; kyy < Q.m[1]; ++kyy) {
            if (Q.lc[1][kyy] != y) continue;
            for (int kz = 0; kz < Q.m[2]; ++kz) {
              const int z = Q.lc[2][kz];
              const float w = g.norm == 1 ? Q.wv[0][kx] * Q.wv[1][kyy] * Q.wv[2][kz]
                                          : radial_w(g, Q.wv[0][kx], Q.wv[1][kyy], Q.wv[2][kz]);
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                if (z != 2 * zp + (q & 1) + 4 * (q >> 1)) continue;
#pragma unroll
                for (int k = 0; k < 4; ++k) fma2_bcast(acc[q][k], w, v[k]);
              }
            }
          }
        }
      }
    }
  }
  // Write-out from registers. A split tile's part goes to its partial slot
  // in the [x][y][z][entry] layout; a whole tile goes to the grid, where the
  // lanes of z pairs 0 and 1 write 32 contiguous bytes of an entry's row.
  if (it.w >= 0) {
    float* dst = partial + ((long long)it.w * gridDim.y + cg) * TFL;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int z = 2 * zp + (q & 1) + 4 * (q >> 1);
      float4* d = reinterpret_cast<float4*>(dst + ((warp * 8 + y) * 8 + z) * VS + 8 * cq);
      d[0] = make_float4(acc[q][0].x, acc[q][0].y, acc[q][1].x, acc[q][1].y);
      d[1] = make_float4(acc[q][2].x, acc[q][2].y, acc[q][3].x, acc[q][3].y);
    }
    return;
  }
  const int gx = o[0] + warp, gy = o[1] + y;
  if (gx >= g.N[0] || gy >= g.N[1]) return;
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  // 16-byte stores need an even Z extent (row starts at even elements) and an aligned base
  const bool vec = o[2] + 8 <= g.N[2] && (g.N[2] & 1) == 0 && (reinterpret_cast<uintptr_t>(gridv) & 15) == 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = 4 * cq + k;
    if (c >= ncoil) continue;
    float* row = gridv + ((long long)(c0 + c) * gvol + ((long long)gx * g.N[1] + gy) * g.N[2] + o[2]) * 2;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int z = 2 * zp + 4 * h;  // slots 2h, 2h + 1
      const float2 a = acc[2 * h][k], b = acc[2 * h + 1][k];
      if (vec) {
        *reinterpret_cast<float4*>(row + 2 * z) = make_float4(a.x, a.y, b.x, b.y);
      } else {
        if (o[2] + z < g.N[2]) *reinterpret_cast<float2*>(row + 2 * z) = a;
        if (o[2] + z + 1 < g.N[2]) *reinterpret_cast<float2*>(row + 2 * z + 2) = b;
      }
    }
  }
}

// ------------------------------------------------- block gridding (3D, 8 entries)
//
// Work items are blocks, parts of dense blocks and runs of empty blocks. A
// persistent grid's warps take them one at a time, in list order, from a
// counter in global memory, so a dense block costs one warp, not a CTA, no
// SM idles behind a CTA's last items, and which warp takes an item does not
// change its result. A warp holds its item's 4 x 4 x 4-cell output
// block x 8 complex entries as the accumulators of warp-level tensor-core
// products (mma.sync m16n8k8, tf32 inputs, fp32 accumulation): the block's
// 64 cells are the 4 row tiles (one per x, rows (y, z)), the 8 entries'
// real and imaginary parts the 2 column tiles. The warp walks the block's
// list in chunks of 32 entries: each lane copies one entry's values and the
// point's three rows of tap weights over this block (from the plan) into the
// warp's staging slots (cp.async). Then each group of 8 entries is one rank-8
// update of the block: weights (x row * y row * z row, built in registers)
// times values. fp32 accuracy from tf32 inputs: each operand is split into a
// high and a low tf32 part and the update is hi*hi + hi*lo + lo*hi (the
// lo*lo term is below 2^-22 of the product). The result depends only on the
// plan's order: bit-identical run to run. A chunk with a non-finite value is
// applied entry by entry on the CUDA cores instead, each such entry to the
// cells of its window only (a zero weight would carry its NaN or Inf to the
// whole block); the rows mark the cells outside the window with -0.0.
constexpr int kBC = 32;       // entries per chunk (one per lane while staging)
constexpr int kB3Ctas = 3;    // resident CTAs per SM of the persistent grid
constexpr int kBS = 40;       // floats per staged entry: x row 0-3 | y row 4-7 | z row 8-11 | values 16-31
                              // (40: the tensor-core operand loads of a group of 8 entries are free of
                              // bank conflicts)

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// x = hi + lo with hi, lo tf32 (round to nearest); x - hi is exact in fp32
__device__ __forceinline__ void split_tf32(float x, unsigned& hi, unsigned& lo) {
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
  const float r = x - __uint_as_float(hi);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
}

// d += a * b, m16n8k8, tf32 inputs, fp32 accumulators
__device__ __forceinline__ void mma_tf32(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void block_origin(const Geo& g, int key, int& bx, int& by, int& bz) {
  const int nb1 = blocks_along(g, 1), nb2 = blocks_along(g, 2);
  bz = key % nb2;
  const int t = key / nb2;
  by = t % nb1;
  bx = t / nb1;
}

// The accumulator fragment of lane (g8, t4): D[m][nt][2h + c] holds entry
// 4 nt + t4 (real part c = 0, imaginary c = 1) of the block cell
// 3D: (x m, y (g8 >> 2) + 2h, z g8 & 3); 2D: (y 2m + h, z g8).
template <int NDIM>
__device__ __forceinline__ void frag_cell(int m, int h, int g8, int& x, int& y, int& z) {
  if constexpr (NDIM == 3) {
    x = m, y = (g8 >> 2) + 2 * h, z = g8 & 3;
  } else {
    x = 0, y = 2 * m + h, z = g8;
  }
}
// index of a block cell in [x][y][z] order (64 cells)
template <int NDIM>
__device__ __forceinline__ int cell_index(int x, int y, int z) {
  return NDIM == 3 ? (x * 4 + y) * 4 + z : y * 8 + z;
}

// Stores the lane's cells of block key `blk` for entries below ncoil.
template <int NDIM>
__device__ __forceinline__ void frag_store(const Geo& g, float* __restrict__ gridv, int c0, int ncoil, int blk, int g8,
                                           int t4, const float (&D)[4][2][4]) {
  int bx, by, bz;
  block_origin(g, blk, bx, by, bz);
  const int B0 = bx * block_edge(NDIM, 0), B1 = by * block_edge(NDIM, 1), B2 = bz * block_edge(NDIM, 2);
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int lx, ly, lz;
      frag_cell<NDIM>(m, h, g8, lx, ly, lz);
      const int x = B0 + lx, y = B1 + ly, z = B2 + lz;
      if (x >= g.N[0] || y >= g.N[1] || z >= g.N[2]) continue;
      const long long cell = ((long long)x * g.N[1] + y) * g.N[2] + z;
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        const int e = 4 * nt + t4;
        if (e < ncoil)
          *reinterpret_cast<float2*>(gridv + ((long long)(c0 + e) * gvol + cell) * 2) =
              make_float2(D[m][nt][2 * h], D[m][nt][2 * h + 1]);
      }
    }
  }
}

template <int NDIM>
__global__ void __launch_bounds__(256, kB3Ctas) adj_b3_kernel(Geo g, const int4* __restrict__ items, int nitems,
                                                        const uint32_t* __restrict__ bentries,
                                                        const float* __restrict__ rows,
                                                        const float2* __restrict__ vals,
                                                        const float4* __restrict__ tv, float* __restrict__ gridv,
                                                        float* __restrict__ partial, int* __restrict__ ctr) {
  extern __shared__ __align__(16) float bsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* S = bsm + warp * (kBC * kBS);
  const int cg = blockIdx.y, c0 = cg * 8;
  const int ncoil = (int)min(8ll, g.nbatch - c0);
  const int g8 = lane >> 2, t4 = lane & 3;
  const int last = nitems;
  // the warps of all CTAs take the items in list order from the group's
  // counter (zeroed before the launch), so the items worked on at one time
  // are neighbours in the list; the warps never wait for one another
  auto grab = [&]() {
    int i = 0;
    if (lane == 0) i = atomicAdd(ctr + cg, 1);
    return __shfl_sync(0xffffffffu, i, 0);
  };
  // one item and the next chunk's point indices ahead: a chunk's copies wait
  // only for their own data, not for the descriptor and index loads before it
  int item = grab();
  if (item >= last) return;
  int4 itn = items[item];
  int inext = grab();
  int4 itnn = inext < last ? items[inext] : make_int4(0, 0, 0, 0);
  uint32_t enext = lane < min(kBC, itn.z - itn.y) ? bentries[itn.y + lane] : 0u;
  for (;;) {
    if (item >= last) return;
    const int4 it = itn;
    itn = itnn;
    item = inext;
    if (item < last) {
      inext = grab();
      itnn = inext < last ? items[inext] : make_int4(0, 0, 0, 0);
    }
    float D[4][2][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i) D[m][nt][i] = 0.f;
    if (it.y == it.z) {  // a run of -it.w empty blocks
      for (int b = 0; b < -it.w; ++b) frag_store<NDIM>(g, gridv, c0, ncoil, it.x + b, g8, t4, D);
      if (item < last) enext = lane < min(kBC, itn.z - itn.y) ? bentries[itn.y + lane] : 0u;
      continue;
    }
    for (int c = it.y; c < it.z; c += kBC) {
      const int n = min(kBC, it.z - c);
      const int n8 = (n + 7) & ~7;  // the tensor-core steps read whole groups of 8 entries
      float* sl = S + lane * kBS;
      const uint32_t en = enext;
      // the point indices of the next chunk: this item's, or the next item's first
      if (c + kBC < it.z)
        enext = lane < min(kBC, it.z - c - kBC) ? bentries[c + kBC + lane] : 0u;
      else if (item < last)
        enext = lane < min(kBC, itn.z - itn.y) ? bentries[itn.y + lane] : 0u;
      if (lane < n) {
        long long p = en & ((1u << kSelShift) - 1u);
        if (!TLGB_IN_RANGE(p, g.npts)) p = 0;
        const float* rsrc = rows + p * row_floats(NDIM);
        if constexpr (NDIM == 3) {  // rows of 4 cells: x 0-3, y 4-7, z 8-11
          cp_async16(sl + 0, rsrc + 4 * (0 + ((en >> kSelShift) & 1)));
          cp_async16(sl + 4, rsrc + 4 * (2 + ((en >> (kSelShift + 1)) & 1)));
          cp_async16(sl + 8, rsrc + 4 * (4 + ((en >> (kSelShift + 2)) & 1)));
        } else {  // rows of 8 cells: y 0-7, z 8-15
          const float* ry = rsrc + 8 * (0 + ((en >> (kSelShift + 1)) & 1));
          const float* rz = rsrc + 8 * (2 + ((en >> (kSelShift + 2)) & 1));
          cp_async16(sl + 0, ry);
          cp_async16(sl + 4, ry + 4);
          cp_async16(sl + 8, rz);
          cp_async16(sl + 12, rz + 4);
        }
        if (tv) {
          const float4* vsrc = tv + ((long long)cg * g.npts + p) * 4;
#pragma unroll
          for (int q = 0; q < 4; ++q) cp_async16(sl + 16 + 4 * q, vsrc + q);
        } else {
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            if (k < ncoil)
              cp_async8(sl + 16 + 2 * k, vals + (long long)(c0 + k) * g.npts + p);
            else
              *reinterpret_cast<float2*>(sl + 16 + 2 * k) = make_float2(0.f, 0.f);
          }
        }
      } else if (lane < n8) {  // padding entries of the last group: zero weights and values
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float4* q4 = reinterpret_cast<float4*>(sl);
        q4[0] = q4[1] = q4[2] = q4[3] = z4;
        q4[4] = q4[5] = q4[6] = q4[7] = z4;
      }
      cp_async_wait_all();
      bool nonfinite = false;
      if (lane < n) {  // a non-finite value turns the zero product into NaN
        float chk = 0.f;
        const float4* vq = reinterpret_cast<const float4*>(sl + 16);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 v = vq[q];
          chk = fmaf(v.x, 0.f, chk);
          chk = fmaf(v.y, 0.f, chk);
          chk = fmaf(v.z, 0.f, chk);
          chk = fmaf(v.w, 0.f, chk);
        }
        nonfinite = !(chk == 0.f);
      }
      const unsigned guarded = __ballot_sync(0xffffffffu, nonfinite);
      __syncwarp();
      if (!guarded) {
        for (int kk = 0; kk < n8; kk += 8) {  // entries kk + t4 and kk + t4 + 4 of this lane's fragments
          const float* e0 = S + (kk + t4) * kBS;
          const float* e1 = e0 + 4 * kBS;
          unsigned bh[2][2], bl[2][2];
#pragma unroll
          for (int nt = 0; nt < 2; ++nt) {
            split_tf32(e0[16 + 8 * nt + g8], bh[nt][0], bl[nt][0]);
            split_tf32(e1[16 + 8 * nt + g8], bh[nt][1], bl[nt][1]);
          }
          // weights of rows g8 and g8 + 8 of row tile m, for entries e0 and e1
          float wa[4][2], wb[4][2];
          if constexpr (NDIM == 3) {  // x m * (y (g8 >> 2) + 2h * z g8 & 3)
            const float z0 = e0[8 + (g8 & 3)], z1 = e1[8 + (g8 & 3)];
            const float yz0a = e0[4 + (g8 >> 2)] * z0, yz0b = e0[6 + (g8 >> 2)] * z0;
            const float yz1a = e1[4 + (g8 >> 2)] * z1, yz1b = e1[6 + (g8 >> 2)] * z1;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
              wa[m][0] = e0[m] * yz0a, wa[m][1] = e0[m] * yz0b;
              wb[m][0] = e1[m] * yz1a, wb[m][1] = e1[m] * yz1b;
            }
          } else {  // y 2m + h * z g8
            const float z0 = e0[8 + g8], z1 = e1[8 + g8];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
              wa[m][0] = e0[2 * m] * z0, wa[m][1] = e0[2 * m + 1] * z0;
              wb[m][0] = e1[2 * m] * z1, wb[m][1] = e1[2 * m + 1] * z1;
            }
          }
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            unsigned ah[4], al[4];
            split_tf32(wa[m][0], ah[0], al[0]);
            split_tf32(wa[m][1], ah[1], al[1]);
            split_tf32(wb[m][0], ah[2], al[2]);
            split_tf32(wb[m][1], ah[3], al[3]);
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
              mma_tf32(D[m][nt], ah, bh[nt][0], bh[nt][1]);
              mma_tf32(D[m][nt], ah, bl[nt][0], bl[nt][1]);
              mma_tf32(D[m][nt], al, bh[nt][0], bh[nt][1]);
            }
          }
        }
      } else {
        // entry by entry on the CUDA cores, in order; a non-finite entry only
        // reaches the cells of its window (weights with a clear sign bit)
        for (int j = 0; j < n; ++j) {
          const float* e = S + j * kBS;
          const bool nf = (guarded >> j) & 1u;
#pragma unroll
          for (int m = 0; m < 4; ++m) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              int lx, ly, lz;
              frag_cell<NDIM>(m, h, g8, lx, ly, lz);
              // weights of the cell along each dim: 3D rows x 0-3, y 4-7, z 8-11; 2D y 0-7, z 8-15
              const float wx = NDIM == 3 ? e[lx] : 1.f;
              const float y = NDIM == 3 ? e[4 + ly] : e[ly], z = e[8 + lz];
              const float w = wx * (y * z);
              const bool ok = !nf || (!signbit(wx) && !signbit(y) && !signbit(z));
#pragma unroll
              for (int nt = 0; nt < 2; ++nt) {
                const float2 v = *reinterpret_cast<const float2*>(e + 16 + 2 * (4 * nt + t4));
                if (ok) {
                  D[m][nt][2 * h] = fmaf(w, v.x, D[m][nt][2 * h]);
                  D[m][nt][2 * h + 1] = fmaf(w, v.y, D[m][nt][2 * h + 1]);
                }
              }
            }
          }
        }
      }
      __syncwarp();  // the chunk has been read before the next one is staged
    }
    if (it.w >= 0) {  // a part of a split block: its slot of the partial blocks, [cell][entry] complex
      float* dst = partial + ((long long)it.w * gridDim.y + cg) * 64 * 16;
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          int lx, ly, lz;
          frag_cell<NDIM>(m, h, g8, lx, ly, lz);
          const int cell = cell_index<NDIM>(lx, ly, lz);
#pragma unroll
          for (int nt = 0; nt < 2; ++nt)
            *reinterpret_cast<float2*>(dst + cell * 16 + 2 * (4 * nt + t4)) =
                make_float2(D[m][nt][2 * h], D[m][nt][2 * h + 1]);
        }
    } else {
      frag_store<NDIM>(g, gridv, c0, ncoil, it.x, g8, t4, D);
    }
  }
}

// Sum the partial blocks of one split block in slot order, compensated (as
// adj_reduce_f3_kernel). CTA = 256 threads, thread (cell, entry pair) sums
// one float4 of every part, eight in flight. Most split blocks have a few
// parts, so small CTAs keep many blocks in flight per SM; the plan lists the
// blocks with the most parts (a few hundred at the centre of a dense
// trajectory) first, so their longer chains overlap the rest.
template <int NDIM>
__global__ void __launch_bounds__(256) adj_reduce_b3_kernel(Geo g, const int4* __restrict__ split,
                                                            const float* __restrict__ partial,
                                                            float* __restrict__ gridv) {
  const int4 sp = split[blockIdx.x];
  const int cg = blockIdx.y, ncg = gridDim.y, c0 = cg * 8;
  const int ncoil = (int)min(8ll, g.nbatch - c0);
  const int r = threadIdx.x;
  const int cell = r >> 2, ep = r & 3;  // entries 2 ep, 2 ep + 1
  const long long step = (long long)ncg * 64 * 4;  // float4s between consecutive partials
  const float4* src = reinterpret_cast<const float4*>(partial + ((long long)sp.y * ncg + cg) * 64 * 16) + r;
  float4 sum = make_float4(0.f, 0.f, 0.f, 0.f), comp = sum;
  int k = 0;
  for (; k + 8 <= sp.z; k += 8) {
    float4 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __ldg(src + (k + i) * step);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      comp_add(sum.x, comp.x, v[i].x);
      comp_add(sum.y, comp.y, v[i].y);
      comp_add(sum.z, comp.z, v[i].z);
      comp_add(sum.w, comp.w, v[i].w);
    }
  }
  if (k < sp.z) {  // the last 1-7 parts, loaded together
    float4 v[7];
#pragma unroll
    for (int i = 0; i < 7; ++i)
      if (k + i < sp.z) v[i] = __ldg(src + (k + i) * step);
#pragma unroll
    for (int i = 0; i < 7; ++i)
      if (k + i < sp.z) {
        comp_add(sum.x, comp.x, v[i].x);
        comp_add(sum.y, comp.y, v[i].y);
        comp_add(sum.z, comp.z, v[i].z);
        comp_add(sum.w, comp.w, v[i].w);
      }
  }
  int bx, by, bz;
  block_origin(g, sp.x, bx, by, bz);
  const int x = bx * block_edge(NDIM, 0) + (NDIM == 3 ? cell >> 4 : 0);
  const int y = by * block_edge(NDIM, 1) + (NDIM == 3 ? (cell >> 2) & 3 : cell >> 3);
  const int z = bz * block_edge(NDIM, 2) + (NDIM == 3 ? cell & 3 : cell & 7);
  if (x >= g.N[0] || y >= g.N[1] || z >= g.N[2]) return;
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  float* dst = gridv + ((long long)(c0 + 2 * ep) * gvol + ((long long)x * g.N[1] + y) * g.N[2] + z) * 2;
  if (2 * ep < ncoil) *reinterpret_cast<float2*>(dst) = make_float2(sum.x + comp.x, sum.y + comp.y);
  if (2 * ep + 1 < ncoil) *reinterpret_cast<float2*>(dst + gvol * 2) = make_float2(sum.z + comp.z, sum.w + comp.w);
}


// ------------------------------------ block gridding (3D, 1, 2 or 4 entries)
//
// The same work items, counter and staging as adj_b3_kernel, with the block
// factored the other way: accumulator rows are the 16 (y, z) cells of a block
// and columns (x, real/imaginary) for each entry, so one 16 x 8 tile per
// entry holds the whole 4 x 4 x 4 block. A rank-8 update is then
// A[(y, z), e] = y row * z row (shared by the entries) times
// B[e, (x, c)] = x row * value: one m16n8k8 product (three with the tf32
// split) per batch entry and group of 8 (point, block) entries, and 8 bytes
// of values staged per batch entry instead of a 64-byte row of 8. D[j] of lane (g8, t4) holds entry j of the cells (x t4, y g8 >> 2,
// z g8 & 3) (d0, d1) and (x t4, y (g8 >> 2) + 2, z g8 & 3) (d2, d3).
constexpr int kBSn = 20;  // floats per staged entry: x row 0-3 | y row 4-7 | z row 8-11 | E values 12-19
                          // (20: the operand loads of a group of 8 entries are free of bank conflicts)
constexpr int kBnCtas = 4;  // resident CTAs per SM of the persistent grid

template <int E>
__device__ __forceinline__ void bn_store(const Geo& g, float* __restrict__ gridv, int ncoil, int blk, int g8, int t4,
                                         const float (&D)[E][4]) {
  int bx, by, bz;
  block_origin(g, blk, bx, by, bz);
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  const int x = bx * 4 + t4, z = bz * 4 + (g8 & 3);
  if (x >= g.N[0] || z >= g.N[2]) return;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int y = by * 4 + (g8 >> 2) + 2 * h;
    if (y >= g.N[1]) continue;
    const long long cell = ((long long)x * g.N[1] + y) * g.N[2] + z;
#pragma unroll
    for (int j = 0; j < E; ++j)
      if (j < ncoil)
        *reinterpret_cast<float2*>(gridv + ((long long)j * gvol + cell) * 2) = make_float2(D[j][2 * h], D[j][2 * h + 1]);
  }
}

template <int E>
__global__ void __launch_bounds__(256, kBnCtas) adj_bn_kernel(Geo g, const int4* __restrict__ items, int nitems,
                                                             const uint32_t* __restrict__ bentries,
                                                             const float* __restrict__ rows,
                                                             const float2* __restrict__ vals,
                                                             float* __restrict__ gridv, float* __restrict__ partial,
                                                             int* __restrict__ ctr) {
  extern __shared__ __align__(16) float bsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* S = bsm + warp * (kBC * kBSn);
  const int ncoil = (int)min((long long)E, g.nbatch);
  const int g8 = lane >> 2, t4 = lane & 3;
  const int last = nitems;
  auto grab = [&]() {
    int i = 0;
    if (lane == 0) i = atomicAdd(ctr, 1);
    return __shfl_sync(0xffffffffu, i, 0);
  };
  int item = grab();
  if (item >= last) return;
  int4 itn = items[item];
  int inext = grab();
  int4 itnn = inext < last ? items[inext] : make_int4(0, 0, 0, 0);
  uint32_t enext = lane < min(kBC, itn.z - itn.y) ? bentries[itn.y + lane] : 0u;
  for (;;) {
    if (item >= last) return;
    const int4 it = itn;
    itn = itnn;
    item = inext;
    if (item < last) {
      inext = grab();
      itnn = inext < last ? items[inext] : make_int4(0, 0, 0, 0);
    }
    float D[E][4];
#pragma unroll
    for (int j = 0; j < E; ++j)
#pragma unroll
      for (int i = 0; i < 4; ++i) D[j][i] = 0.f;
    if (it.y == it.z) {  // a run of -it.w empty blocks
      for (int b = 0; b < -it.w; ++b) bn_store<E>(g, gridv, ncoil, it.x + b, g8, t4, D);
      if (item < last) enext = lane < min(kBC, itn.z - itn.y) ? bentries[itn.y + lane] : 0u;
      continue;
    }
    for (int c = it.y; c < it.z; c += kBC) {
      const int n = min(kBC, it.z - c);
      const int n8 = (n + 7) & ~7;
      float* sl = S + lane * kBSn;
      const uint32_t en = enext;
      if (c + kBC < it.z)
        enext = lane < min(kBC, it.z - c - kBC) ? bentries[c + kBC + lane] : 0u;
      else if (item < last)
        enext = lane < min(kBC, itn.z - itn.y) ? bentries[itn.y + lane] : 0u;
      if (lane < n) {
        long long p = en & ((1u << kSelShift) - 1u);
        if (!TLGB_IN_RANGE(p, g.npts)) p = 0;
        const float* rsrc = rows + p * row_floats(3);
        cp_async16(sl + 0, rsrc + 4 * (0 + ((en >> kSelShift) & 1)));
        cp_async16(sl + 4, rsrc + 4 * (2 + ((en >> (kSelShift + 1)) & 1)));
        cp_async16(sl + 8, rsrc + 4 * (4 + ((en >> (kSelShift + 2)) & 1)));
#pragma unroll
        for (int j = 0; j < E; ++j) {
          if (j < ncoil)
            cp_async8(sl + 12 + 2 * j, vals + (long long)j * g.npts + p);
          else
            *reinterpret_cast<float2*>(sl + 12 + 2 * j) = make_float2(0.f, 0.f);
        }
      } else if (lane < n8) {  // padding entries of the last group: zero weights and values
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float4* q4 = reinterpret_cast<float4*>(sl);
        q4[0] = q4[1] = q4[2] = z4;
#pragma unroll
        for (int j = 0; j < E; ++j) *reinterpret_cast<float2*>(sl + 12 + 2 * j) = make_float2(0.f, 0.f);
      }
      cp_async_wait_all();
      bool nonfinite = false;
      if (lane < n) {  // a non-finite value turns the zero product into NaN
        float chk = 0.f;
#pragma unroll
        for (int j = 0; j < 2 * E; ++j) chk = fmaf(sl[12 + j], 0.f, chk);
        nonfinite = !(chk == 0.f);
      }
      const unsigned guarded = __ballot_sync(0xffffffffu, nonfinite);
      __syncwarp();
      if (!guarded) {
        for (int kk = 0; kk < n8; kk += 8) {  // entries kk + t4 and kk + t4 + 4 of this lane's fragments
          const float* e0 = S + (kk + t4) * kBSn;
          const float* e1 = e0 + 4 * kBSn;
          // A: rows g8 and g8 + 8 = (y (g8 >> 2) + 2h, z g8 & 3)
          const float z0 = e0[8 + (g8 & 3)], z1 = e1[8 + (g8 & 3)];
          unsigned ah[4], al[4];
          split_tf32(e0[4 + (g8 >> 2)] * z0, ah[0], al[0]);
          split_tf32(e0[6 + (g8 >> 2)] * z0, ah[1], al[1]);
          split_tf32(e1[4 + (g8 >> 2)] * z1, ah[2], al[2]);
          split_tf32(e1[6 + (g8 >> 2)] * z1, ah[3], al[3]);
          // B: column g8 = (x g8 >> 1, c g8 & 1) of entry j
          const float x0 = e0[g8 >> 1], x1 = e1[g8 >> 1];
#pragma unroll
          for (int j = 0; j < E; ++j) {
            unsigned bh0, bl0, bh1, bl1;
            split_tf32(x0 * e0[12 + 2 * j + (g8 & 1)], bh0, bl0);
            split_tf32(x1 * e1[12 + 2 * j + (g8 & 1)], bh1, bl1);
            mma_tf32(D[j], ah, bh0, bh1);
            mma_tf32(D[j], ah, bl0, bl1);
            mma_tf32(D[j], al, bh0, bh1);
          }
        }
      } else {
        // entry by entry on the CUDA cores, in order; a non-finite entry only
        // reaches the cells of its window (weights with a clear sign bit)
        for (int q = 0; q < n; ++q) {
          const float* e = S + q * kBSn;
          const bool nf = (guarded >> q) & 1u;
          const float wx = e[t4], z = e[8 + (g8 & 3)];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float y = e[4 + (g8 >> 2) + 2 * h];
            const float w = wx * (y * z);
            const bool ok = !nf || (!signbit(wx) && !signbit(y) && !signbit(z));
#pragma unroll
            for (int j = 0; j < E; ++j) {
              const float2 v = *reinterpret_cast<const float2*>(e + 12 + 2 * j);
              if (ok) {
                D[j][2 * h] = fmaf(w, v.x, D[j][2 * h]);
                D[j][2 * h + 1] = fmaf(w, v.y, D[j][2 * h + 1]);
              }
            }
          }
        }
      }
      __syncwarp();  // the chunk has been read before the next one is staged
    }
    if (it.w >= 0) {  // a part of a split block: its slot of the partial blocks, [cell][entry] complex
      float* dst = partial + (long long)it.w * 64 * 2 * E;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int cell = cell_index<3>(t4, (g8 >> 2) + 2 * h, g8 & 3);
#pragma unroll
        for (int j = 0; j < E; ++j)
          *reinterpret_cast<float2*>(dst + (cell * E + j) * 2) = make_float2(D[j][2 * h], D[j][2 * h + 1]);
      }
    } else {
      bn_store<E>(g, gridv, ncoil, it.x, g8, t4, D);
    }
  }
}

// Sum the partial blocks of one split block of adj_bn_kernel in slot order,
// compensated. CTA = 256 threads: thread (range r, cell, entry) sums one
// complex value of every part of the r-th of 256 / (64 E) consecutive part
// ranges, eight in flight; then the ranges are added in order. With one or
// two entries the ranges cut the longest chain (the densest block has a few
// hundred parts) by 4 or 2.
template <int E>
__global__ void __launch_bounds__(256) adj_reduce_bn_kernel(Geo g, const int4* __restrict__ split,
                                                           const float* __restrict__ partial,
                                                           float* __restrict__ gridv) {
  constexpr int U = 64 * E, R = 256 / U;  // values per part, part ranges
  __shared__ float2 rs[R > 1 ? R - 1 : 1][U], rc[R > 1 ? R - 1 : 1][U];
  const int4 sp = split[blockIdx.x];
  const int r = threadIdx.x / U, t = threadIdx.x % U, cell = t / E, j = t % E;
  const int ncoil = (int)min((long long)E, g.nbatch);
  const float2* src = reinterpret_cast<const float2*>(partial) + (long long)sp.y * U + t;
  const int k0 = (int)((long long)sp.z * r / R), k1 = (int)((long long)sp.z * (r + 1) / R);
  float2 sum = make_float2(0.f, 0.f), comp = sum;
  int k = k0;
  for (; k + 8 <= k1; k += 8) {
    float2 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __ldg(src + (long long)(k + i) * U);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      comp_add(sum.x, comp.x, v[i].x);
      comp_add(sum.y, comp.y, v[i].y);
    }
  }
  for (; k < k1; ++k) {
    const float2 v = __ldg(src + (long long)k * U);
    comp_add(sum.x, comp.x, v.x);
    comp_add(sum.y, comp.y, v.y);
  }
  if constexpr (R > 1) {
    if (r > 0) {
      rs[r - 1][t] = sum;
      rc[r - 1][t] = comp;
    }
    __syncthreads();
    if (r > 0) return;
#pragma unroll
    for (int i = 0; i < R - 1; ++i) {  // the later ranges in order, their compensations with them
      const float2 s2 = rs[i][t], c2 = rc[i][t];
      comp_add(sum.x, comp.x, s2.x);
      comp_add(sum.y, comp.y, s2.y);
      comp.x += c2.x, comp.y += c2.y;
    }
  }
  if (j >= ncoil) return;
  int bx, by, bz;
  block_origin(g, sp.x, bx, by, bz);
  const int x = bx * 4 + (cell >> 4), y = by * 4 + ((cell >> 2) & 3), z = bz * 4 + (cell & 3);
  if (x >= g.N[0] || y >= g.N[1] || z >= g.N[2]) return;
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  *reinterpret_cast<float2*>(gridv + ((long long)j * gvol + ((long long)x * g.N[1] + y) * g.N[2] + z) * 2) =
      make_float2(sum.x + comp.x, sum.y + comp.y);
}

// 2D gridding. The view of one dimension of a record from a 16-wide tile at o
// (grid N): f | m << 4 | k0 << 7, as tile_view (f first local position, m
// taps inside the tile, k0 the first of them in the record). fast is
// cleared for 5-tap windows and, in circular mode on a grid below 32, for
// windows that could meet the tile twice.
__device__ __forceinline__ int tile_view16(int st, int c, int o, int N, bool circ, bool& fast) {
  const int te = min(16, N - o);
  int d = st - o;
  if (circ && d < 0) d += N;
  int f, k0, m;
  if (d >= 0 && d < te) {
    f = d;
    k0 = 0;
    m = min(c, te - d);
  } else {
    f = 0;
    k0 = circ ? N - d : -d;
    m = (d >= te && !circ) ? 0 : min(c - k0, te);
  }
  if (m < 0 || k0 < 0) m = 0, k0 = 0;
  if (c > 4 || (circ && N < 32)) fast = false;
  return f | (m << 4) | (min(k0, 7) << 7);
}

// (y view) | (z view) << 10 | fast << 27 | ok << 28
__device__ __forceinline__ unsigned grid_view2(const Geo& g, const PRec& R, const int (&o)[3]) {
  bool fast = true;
  const bool circ = g.pad == TLGB_PAD_CIRCULAR;
  const int c = R.cnt;
  const bool ok = (c & 15) && ((c >> 4) & 15) && ((c >> 8) & 15);
  const unsigned vy = tile_view16(R.st[1], (c >> 4) & 15, o[1], g.N[1], circ, fast);
  const unsigned vz = tile_view16(R.st[2], (c >> 8) & 15, o[2], g.N[2], circ, fast);
  return vy | (vz << 10) | ((fast ? 1u : 0u) << 27) | ((ok ? 1u : 0u) << 28);
}

// CTA = 8 warps owning one 16 x 16 x 8-entry output tile of a 2D grid, held
// in registers: warp w owns rows 2w and 2w + 1, lane (row, z pair, entry
// half) the cells (y, 2 zq) and (y, 2 zq + 1) for 4 of the 8 entries. Pairs
// are staged in batches of kAB2, one thread per pair: its 8 point values,
// its rows of tap weights over the tile (16 in y, 16 in z, zero where the
// window has no tap), and per 2-row slab a bitmask of the pairs with taps
// there. Each warp applies its slab's pairs in plan order, two per step, then
// the pairs that need the generic record (5 taps, a window wrapping inside
// the tile, a non-finite value), also in order.
constexpr int kAB2 = 224;

// Rows padded as in AdjStage (36 and 20 floats); 224 pairs keep 4 CTAs per SM.
struct AdjStage2 {
  float wrow[kAB2][36];  // tap weights at tile-local y (0-15) and z (16-31)
  float pv[kAB2][20];    // point values, 8 entries complex (16 floats)
  int pidx[kAB2];
  unsigned fmask[8][kAB2 / 32];  // per slab: pairs on the row path with taps there
  unsigned smask[kAB2 / 32];     // pairs on the generic path (all slabs)
};

constexpr size_t adj_f2_smem() { return sizeof(AdjStage2) + 8 * sizeof(Rec<5>); }

__global__ void __launch_bounds__(256, 4) adj_f2_kernel(Geo g, const int4* __restrict__ items,
                                                        const int32_t* __restrict__ entries,
                                                        const PRec* __restrict__ precs,
                                                        const float* __restrict__ locs, const float* __restrict__ vals,
                                                        const float4* __restrict__ tv, float* __restrict__ gridv,
                                                        float* __restrict__ partial) {
  constexpr int CG = 8, VS = 16, TFL = 256 * 16, NW = 8, MW = kAB2 / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  AdjStage2& S = *reinterpret_cast<AdjStage2*>(smem);
  Rec<5>* slow = reinterpret_cast<Rec<5>*>(smem + sizeof(AdjStage2));  // [NW]
  const int4 it = items[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cg = blockIdx.y;
  const int c0 = cg * CG;
  const int ncoil = (int)min((long long)CG, g.nbatch - c0);
  int o[3];
  {
    int t = it.x;
    o[2] = (t % g.nt[2]) * 16;
    t /= g.nt[2];
    o[1] = (t % g.nt[1]) * 16;
    o[0] = 0;
  }
  const int r = lane >> 4, zq = (lane >> 1) & 7, eh = lane & 1;
  const int y = 2 * warp + r;
  float2 acc[2][4];  // [z = 2 zq + i][entry 4 eh + k]
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[i][k] = make_float2(0.f, 0.f);
  for (int b = it.y; b < it.z; b += kAB2) {
    const int nb = min(kAB2, it.z - b);
    __syncthreads();  // the previous batch has been applied
    {
      unsigned view = 0;
      bool finite = true;
      if (tid < nb) {
        const int p = entries[b + tid];
        const PRec R = load_prec(precs, p);
        float4 v[4];
        if (tv) {
          const float4* src = tv + ((long long)cg * g.npts + p) * 4;
#pragma unroll
          for (int q = 0; q < 4; ++q) v[q] = __ldg(src + q);
        } else {
          const float2* v2 = reinterpret_cast<const float2*>(vals);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int c = 2 * q;
            const float2 a = c < ncoil ? __ldg(v2 + (long long)(c0 + c) * g.npts + p) : make_float2(0.f, 0.f);
            const float2 d = c + 1 < ncoil ? __ldg(v2 + (long long)(c0 + c + 1) * g.npts + p) : make_float2(0.f, 0.f);
            v[q] = make_float4(a.x, a.y, d.x, d.y);
          }
        }
        float4* pd = reinterpret_cast<float4*>(&S.pv[tid][0]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          pd[q] = v[q];
          finite = finite && isfinite(v[q].x) && isfinite(v[q].y) && isfinite(v[q].z) && isfinite(v[q].w);
        }
        view = grid_view2(g, R, o);
        S.pidx[tid] = p;
        if (((view >> 27) & 1) && finite) {
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const unsigned u = (view >> (10 * e)) & 1023;
            const int f = u & 15, m = (u >> 4) & 7, k0 = u >> 7;
            const float4 w = R.w[1 + e];
            float4* d = reinterpret_cast<float4*>(&S.wrow[tid][16 * e]);
#pragma unroll
            for (int l4 = 0; l4 < 4; ++l4) {
              float rr[4];
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                const int k = 4 * l4 + i - f;
                rr[i] = (k >= 0 && k < m) ? pick4(w, k0 + k) : 0.f;
              }
              d[l4] = make_float4(rr[0], rr[1], rr[2], rr[3]);
            }
          }
        }
      }
      const bool ok = (view >> 28) & 1, fast = ((view >> 27) & 1) && finite;
      const int fy = view & 15, my = (view >> 4) & 7;
      // warps past kAB2 / 32 stage no pairs and own no mask word
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const unsigned bal = __ballot_sync(0xffffffffu, ok && fast && fy <= 2 * w + 1 && fy + my > 2 * w);
        if (lane == 0 && warp < MW) S.fmask[w][warp] = bal;
      }
      const unsigned bs = __ballot_sync(0xffffffffu, ok && !fast);
      if (lane == 0 && warp < MW) S.smask[warp] = bs;
    }
    __syncthreads();
    struct Visit {
      float w0, w1;   // weights of the lane's two cells
      float4 v0, v1;  // the lane's 4 entries, complex
    };
    auto fetch = [&](int j) {
      const float* wr = S.wrow[j];
      const float wy = wr[y];
      const float2 wz = *reinterpret_cast<const float2*>(wr + 16 + 2 * zq);
      Visit d;
      d.w0 = wy * wz.x;
      d.w1 = wy * wz.y;
      d.v0 = *reinterpret_cast<const float4*>(&S.pv[j][8 * eh]);
      d.v1 = *reinterpret_cast<const float4*>(&S.pv[j][8 * eh + 4]);
      return d;
    };
    auto apply = [&](const Visit& d) {
      const float2 v[4] = {make_float2(d.v0.x, d.v0.y), make_float2(d.v0.z, d.v0.w), make_float2(d.v1.x, d.v1.y),
                           make_float2(d.v1.z, d.v1.w)};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        fma2_bcast(acc[0][k], d.w0, v[k]);
        fma2_bcast(acc[1][k], d.w1, v[k]);
      }
    };
#pragma unroll 1
    for (int mw = 0; mw < MW; ++mw) {
      unsigned bits = S.fmask[warp][mw];
      while (bits) {
        const int j0 = mw * 32 + __ffs(bits) - 1;
        bits &= bits - 1;
        const Visit d0 = fetch(j0);
        if (bits) {
          const int j1 = mw * 32 + __ffs(bits) - 1;
          bits &= bits - 1;
          const Visit d1 = fetch(j1);
          apply(d0);
          apply(d1);
        } else {
          apply(d0);
        }
      }
    }
#pragma unroll 1
    for (int mw = 0; mw < MW; ++mw) {
      unsigned bits = S.smask[mw];
      while (bits) {
        const int j = mw * 32 + __ffs(bits) - 1;
        bits &= bits - 1;
        __syncwarp();  // the previous record has been read
        if (lane == 0) {
          float x3[3] = {0.f, 0.f, 0.f};
          for (int e = 1; e < 3; ++e) x3[e] = load_coord(g, locs, S.pidx[j], e);
          lane_rec<5>(g, x3, o, false, slow[warp]);
        }
        __syncwarp();
        const Rec<5>& Q = slow[warp];
        const float4 v0 = *reinterpret_cast<const float4*>(&S.pv[j][8 * eh]);
        const float4 v1 = *reinterpret_cast<const float4*>(&S.pv[j][8 * eh + 4]);
        const float2 v[4] = {make_float2(v0.x, v0.y), make_float2(v0.z, v0.w), make_float2(v1.x, v1.y),
                             make_float2(v1.z, v1.w)};
        if (Q.m[0] > 0)
          for (int kyy = 0; kyy < Q.m[1]; ++kyy) {
            if (Q.lc[1][kyy] != y) continue;
            for (int kz = 0; kz < Q.m[2]; ++kz) {
              const int z = Q.lc[2][kz];
              const float w = Q.wv[1][kyy] * Q.wv[2][kz];
#pragma unroll
              for (int i = 0; i < 2; ++i) {
                if (z != 2 * zq + i) continue;
#pragma unroll
                for (int k = 0; k < 4; ++k) fma2_bcast(acc[i][k], w, v[k]);
              }
            }
          }
      }
    }
  }
  // write-out from registers: a split tile's part to its partial slot
  // ([y][z][entry], 16 floats per cell); a whole tile to the grid, 16
  // contiguous bytes (two z) of an entry's row per lane
  if (it.w >= 0) {
    float* dst = partial + ((long long)it.w * gridDim.y + cg) * TFL;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      float4* d = reinterpret_cast<float4*>(dst + (y * 16 + 2 * zq + i) * VS + 8 * eh);
      d[0] = make_float4(acc[i][0].x, acc[i][0].y, acc[i][1].x, acc[i][1].y);
      d[1] = make_float4(acc[i][2].x, acc[i][2].y, acc[i][3].x, acc[i][3].y);
    }
    return;
  }
  const int gy = o[1] + y;
  if (gy >= g.N[1]) return;
  const long long gvol = (long long)g.N[1] * g.N[2];
  // 16-byte stores need an even Z extent (row starts at even elements) and an aligned base
  const bool vec = o[2] + 16 <= g.N[2] && (g.N[2] & 1) == 0 && (reinterpret_cast<uintptr_t>(gridv) & 15) == 0;
  const int z = 2 * zq;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = 4 * eh + k;
    if (c >= ncoil) continue;
    float* row = gridv + ((long long)(c0 + c) * gvol + (long long)gy * g.N[2] + o[2]) * 2;
    const float2 a = acc[0][k], bb = acc[1][k];
    if (vec) {
      *reinterpret_cast<float4*>(row + 2 * z) = make_float4(a.x, a.y, bb.x, bb.y);
    } else {
      if (o[2] + z < g.N[2]) *reinterpret_cast<float2*>(row + 2 * z) = a;
      if (o[2] + z + 1 < g.N[2]) *reinterpret_cast<float2*>(row + 2 * z + 2) = bb;
    }
  }
}

// Gather: CTA = 8 warps sharing one 12^3 x CG-entry region ([entry][x][y][z],
// loaded by one TMA bulk tensor copy when the region needs no wrap). Each warp
// takes every 8th point of the item, building the records of its next 8
// points itself (kGB = 8 warps x 8 slots). Lanes = (point, entry, z-tap): a
// lane sums its entry's 4 y-taps x 4 x-taps, then the 4 z-tap lanes add up.
// CG = 8 (two CTAs per SM): one point per step across the lanes, two steps
// interleaved. CG = 1, 2 or 4 (batches of at most 4 entries, 4 CTAs per SM):
// 8 / CG points per step, so a one-entry batch stages and reads an eighth
// of the region.
constexpr int kGB = 64;

template <int CG>
__global__ void __launch_bounds__(256, CG == 8 ? 2 : 4) fwd_f3_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                      int use_tma, Geo g,
                                                                      const int4* __restrict__ items,
                                                                      const int32_t* __restrict__ entries,
                                                                      const PRec* __restrict__ precs,
                                                                      const float* __restrict__ locs,
                                                                      const float* __restrict__ gridv,
                                                                      float* __restrict__ out) {
  constexpr int S = 12, PLANE = S * S, VOL = S * S * S, NW = 8;
  constexpr int PPW = 8 / CG;  // points per warp step
  constexpr uint32_t RBYTES = VOL * CG * 8;
  extern __shared__ __align__(128) unsigned char smem[];
  float2* reg = reinterpret_cast<float2*>(smem);               // [8][12][12][12]
  R3* rec = reinterpret_cast<R3*>(smem + RBYTES);              // [kGB]
  Rec<5>* slow = reinterpret_cast<Rec<5>*>(rec + kGB);         // [NW]
  static_assert((kGB * sizeof(R3) + NW * sizeof(Rec<5>)) % 8 == 0, "mbarrier alignment");
  uint64_t* bar = reinterpret_cast<uint64_t*>(slow + NW);
  const int4 it = items[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.y * CG;
  int o[3];
  {
    int t = it.x;
    o[2] = (t % g.nt[2]) * 8;
    t /= g.nt[2];
    o[1] = (t % g.nt[1]) * 8;
    o[0] = (t / g.nt[1]) * 8;
  }
  // the region needs wrap in circular mode when it crosses the upper edge
  const bool wraps = g.pad == TLGB_PAD_CIRCULAR && (o[0] + S > g.N[0] || o[1] + S > g.N[1] || o[2] + S > g.N[2]);
  const bool tma = use_tma && !wraps;
  if (tma) {
    if (tid == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
      if (!g.skip_copy) {  // test hook: nothing in flight, so the bounded wait runs out
        mbar_arrive_expect_tx(bar, RBYTES);
        tma_load_4d(reg, &tmap, bar, o[2], o[1], o[0], c0);
      }
    }
  } else {
    // plain loads with wrap / zero fill: rows (entry, x, y) of 12 z
    const int ncoil = (int)min((long long)CG, g.nbatch - c0);
    const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
    for (int idx = tid; idx < CG * VOL; idx += NW * 32) {
      const int z = idx % S;
      const int r = idx / S;
      const int y = r % S, x = (r / S) % S, c = r / PLANE;
      int gx = o[0] + x, gy = o[1] + y, gz = o[2] + z;
      bool in = c < ncoil;
      if (g.pad == TLGB_PAD_CIRCULAR) {
        gx = wrapi(gx, g.N[0]);
        gy = wrapi(gy, g.N[1]);
        gz = wrapi(gz, g.N[2]);
      } else {
        in = in && gx < g.N[0] && gy < g.N[1] && gz < g.N[2];
      }
      reg[idx] = in ? __ldg(reinterpret_cast<const float2*>(gridv) + (long long)(c0 + c) * gvol +
                           ((long long)gx * g.N[1] + gy) * g.N[2] + gz)
                    : make_float2(0.f, 0.f);
    }
  }
  // lane = (point q, entry c, z tap kz). Iteration t reads y tap (t + lane /
  // 4) & 3: the 8 entries' regions are 13,824 B apart (the same banks), so
  // rotating the y taps by lane group spreads one load instruction over 4
  // bank windows.
  const int q = lane / (4 * CG), c = (lane >> 2) % CG, kz = lane & 3;
  int kyo[4], rowoff[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    kyo[t] = (t + (lane >> 2)) & 3;
    rowoff[t] = kyo[t] * S;
  }
  // Each warp takes the item's points warp, warp + 8, ... in mini-batches of
  // 8 and keeps its own 8 record slots. Lanes 0-7 run two mini-batches
  // ahead: the point indices of mini-batch m + 2 and the point records of
  // m + 1 are in flight in registers while the warp gathers mini-batch m.
  R3* wrec = rec + warp * 8;
  const int npt = it.z - it.y;
  auto point_at = [&](int base) -> int {
    const int j = base + 8 * lane;
    return (lane < 8 && j < npt) ? entries[it.y + j] : -1;
  };
  auto fetch = [&](int p) {
    PRec R;
    if (p >= 0) R = load_prec(precs, p);
    return R;
  };
  auto publish = [&](int p, const PRec& R) {
    if (p >= 0) {
      R3& S = wrec[lane];
      S.w[0] = R.w[0];
      S.w[1] = R.w[1];
      S.w[2] = R.w[2];
      S.view = region_view(g, R, o);
      S.p = p;
    }
    __syncwarp();
  };
  int pc = point_at(warp);           // mini-batch 0: indices
  int pn = point_at(warp + 8 * NW);  // mini-batch 1: indices
  PRec Rc = fetch(pc);               // mini-batch 0: records
  auto build_records = [&](int base) {
    publish(pc, Rc);  // the mini-batch at base
    Rc = fetch(pn);   // the next one's records (its indices are in)
    pc = pn;
    pn = point_at(base + 16 * NW);  // the one after's indices
  };
  build_records(warp);  // while the region copy is in flight
  {
    // the copy must have landed: one thread polls (bounded), the others
    // wait at the barrier without taking issue slots; then a CTA-wide vote
    bool ok = true;
    if (tma && tid == 0) ok = mbar_wait_bounded(bar, 0, g.skip_copy ? 1u : 1u << 22);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicExch(&g_tlgb_status, 1);
      return;
    }
  }
  {
    // points of the plain-run view, two per step: sum over y taps of
    // wy wz (sum over x taps of wx v). A record's weights are zero past its
    // tap count, so taps outside the window contribute 0; every tap of the
    // 4^3 box lies inside the staged region.
    auto gather_box = [&](const R3& R) {
      const float4 wx = R.w[0];
      const float wz = (&R.w[2].x)[kz];
      const float* wy = &R.w[1].x;
      const float2* a = reg + c * VOL + (R.view & 2047) + kz;
      // the box's farthest cell: 3 x, 3 y and the last z lane from the base
      if (!TLGB_IN_RANGE((R.view & 2047) + kz + 3 * PLANE + 3 * S, VOL)) return make_float2(0.f, 0.f);
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const float wyz = wy[kyo[t]] * wz;
        const float2* ar = a + rowoff[t];
        float2 sx = mul2_bcast(wx.x, ar[0]);
        fma2_bcast(sx, wx.y, ar[PLANE]);
        fma2_bcast(sx, wx.z, ar[2 * PLANE]);
        fma2_bcast(sx, wx.w, ar[3 * PLANE]);
        acc.x = fmaf(wyz, sx.x, acc.x);
        acc.y = fmaf(wyz, sx.y, acc.y);
      }
      return acc;
    };
    // the generic record path (exact-integer coordinates); with CG < 8 only
    // the lanes of point group 0 sum (warp-uniform call)
    auto gather_rec = [&](const R3& R) {
      if (lane == 0) {
        float x3[3];
        for (int e = 0; e < 3; ++e) x3[e] = load_coord(g, locs, R.p, e);
        lane_rec<5>(g, x3, o, true, slow[warp]);
      }
      __syncwarp();
      const Rec<5>& Sr = slow[warp];
      float2 acc = make_float2(0.f, 0.f);
      if (q == 0)
      for (int kzz = kz; kzz < Sr.m[2]; kzz += 4)
        for (int kyy = 0; kyy < Sr.m[1]; ++kyy)
          for (int kx = 0; kx < Sr.m[0]; ++kx) {
            const float w = g.norm == 1 ? Sr.wv[0][kx] * Sr.wv[1][kyy] * Sr.wv[2][kzz]
                                        : radial_w(g, Sr.wv[0][kx], Sr.wv[1][kyy], Sr.wv[2][kzz]);
            const int ri = c * VOL + (Sr.lc[0][kx] * S + Sr.lc[1][kyy]) * S + Sr.lc[2][kzz];
            if (TLGB_IN_RANGE(ri, CG * VOL)) fma2_bcast(acc, w, reg[ri]);
          }
      __syncwarp();
      return acc;
    };
    // sum over the 4 z-tap lanes of each entry, then lane kz = 0 stores
    auto finish = [&](float2 acc, int p, bool store) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 1);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 1);
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 2);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 2);
      if (store && kz == 0 && c0 + c < g.nbatch && TLGB_IN_RANGE(p, g.npts))
        *reinterpret_cast<float2*>(out + ((long long)(c0 + c) * g.npts + p) * 2) = acc;
    };
    auto one = [&](const R3& R) {
      const unsigned view = R.view;
      if (!((view >> 21) & 1)) return;  // no valid tap (warp-uniform)
      const bool box = (view >> 20) & 1;
      finish(box ? gather_box(R) : gather_rec(R), R.p, box || q == 0);
    };
    for (int base = warp; base < npt; base += 8 * NW) {
      if (base != warp) {
        __syncwarp();  // the previous mini-batch has been read
        build_records(base);
      }
      const int nb = min(8, (npt - base + NW - 1) / NW);
      if constexpr (CG == 8) {
        int i = 0;
        for (; i + 1 < nb; i += 2) {
          const R3& R0 = wrec[i];
          const R3& R1 = wrec[i + 1];
          if ((R0.view & R1.view) >> 20 & 1) {
            // both on the plain-run path (which implies a valid tap): interleaved
            const float2 a0 = gather_box(R0), a1 = gather_box(R1);
            finish(a0, R0.p, true);
            finish(a1, R1.p, true);
          } else {
            one(R0);
            one(R1);
          }
        }
        if (i < nb) one(wrec[i]);
      } else {
        for (int i0 = 0; i0 < nb; i0 += PPW) {
          // the plain-run points of this step, one per lane group
          const int i = i0 + q;
          const R3& R = wrec[i < nb ? i : i0];
          const bool box = i < nb && ((R.view >> 20) & 1);
          finish(box ? gather_box(R) : make_float2(0.f, 0.f), R.p, box);
          // then the step's points with a valid tap off that path, one at a
          // time by the whole warp
#pragma unroll 1
          for (int k = 0; k < PPW && i0 + k < nb; ++k) {
            const unsigned v = wrec[i0 + k].view;
            if (((v >> 21) & 1) && !((v >> 20) & 1)) finish(gather_rec(wrec[i0 + k]), wrec[i0 + k].p, q == 0);
          }
        }
      }
    }
  }
}

// The gather view of a home record in the 20 x 20 region of a 2D tile at o:
// region base (y * 20 + z, 9 bits) | my << 11 | mz << 14 | fast << 20 |
// ok << 21 (the bit positions of region_view).
__device__ __forceinline__ unsigned region_view2(const Geo& g, const PRec& R, const int (&o)[3]) {
  const int c = R.cnt;
  const int cy = (c >> 4) & 15, cz = (c >> 8) & 15;
  const bool ok = (c & 15) && cy && cz;
  int f[3];
#pragma unroll
  for (int e = 1; e < 3; ++e) {
    int d = R.st[e] - o[e];
    if (g.pad == TLGB_PAD_CIRCULAR && d < 0) d += g.N[e];
    f[e] = d;
  }
  const bool fast = ok && cy <= 4 && cz <= 4 && f[1] >= 0 && f[1] < 16 && f[2] >= 0 && f[2] < 16;
  const unsigned base = fast ? (unsigned)(f[1] * 20 + f[2]) : 0u;
  return base | (min(cy, 7) << 11) | (min(cz, 7) << 14) | ((fast ? 1u : 0u) << 20) | ((ok ? 1u : 0u) << 21);
}

// 2D gather: CTA = 8 warps sharing the 20 x 20 x 8-entry region
// ([entry][y][z]) of one 16 x 16 tile, loaded by one TMA bulk tensor copy
// when the region needs no wrap. Each warp takes every 8th point of the
// item, building the records of its next 8 points itself, two mini-batches
// ahead. Lanes = (entry, z-tap): a lane sums its entry's 4 y-taps, two points
// at a time, then the 4 z-tap lanes of each entry add up; the y taps of entry
// c start at row (c & 3), so one load instruction spans 4 bank windows.
__global__ void __launch_bounds__(256, 3) fwd_f2_kernel(const __grid_constant__ CUtensorMap tmap, int use_tma, Geo g,
                                                        const int4* __restrict__ items,
                                                        const int32_t* __restrict__ entries,
                                                        const PRec* __restrict__ precs,
                                                        const float* __restrict__ locs,
                                                        const float* __restrict__ gridv, float* __restrict__ out) {
  constexpr int CG = 8, S = 20, VOL = S * S, NW = 8;
  constexpr uint32_t RBYTES = VOL * CG * 8;
  extern __shared__ __align__(128) unsigned char smem[];
  float2* reg = reinterpret_cast<float2*>(smem);               // [8][20][20]
  R3* rec = reinterpret_cast<R3*>(smem + RBYTES);              // [8 warps][8]
  Rec<5>* slow = reinterpret_cast<Rec<5>*>(rec + 64);          // [NW]
  static_assert((64 * sizeof(R3) + NW * sizeof(Rec<5>)) % 8 == 0, "mbarrier alignment");
  uint64_t* bar = reinterpret_cast<uint64_t*>(slow + NW);
  const int4 it = items[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.y * CG;
  int o[3];
  {
    int t = it.x;
    o[2] = (t % g.nt[2]) * g.T[2];
    t /= g.nt[2];
    o[1] = (t % g.nt[1]) * g.T[1];
    o[0] = 0;
  }
  const bool wraps = g.pad == TLGB_PAD_CIRCULAR && (o[1] + S > g.N[1] || o[2] + S > g.N[2]);
  const bool tma = use_tma && !wraps;
  if (tma) {
    if (tid == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
      if (!g.skip_copy) {  // test hook: nothing in flight, so the bounded wait runs out
        mbar_arrive_expect_tx(bar, RBYTES);
        tma_load_4d(reg, &tmap, bar, o[2], o[1], 0, c0);
      }
    }
  } else {
    // plain loads with wrap / zero fill: rows (entry, y) of 20 z
    const int ncoil = (int)min((long long)CG, g.nbatch - c0);
    const long long gvol = (long long)g.N[1] * g.N[2];
    for (int idx = tid; idx < CG * VOL; idx += NW * 32) {
      const int z = idx % S;
      const int r = idx / S;
      const int y = r % S, c = r / S;
      int gy = o[1] + y, gz = o[2] + z;
      bool in = c < ncoil;
      if (g.pad == TLGB_PAD_CIRCULAR) {
        gy = wrapi(gy, g.N[1]);
        gz = wrapi(gz, g.N[2]);
      } else {
        in = in && gy < g.N[1] && gz < g.N[2];
      }
      reg[idx] = in ? __ldg(reinterpret_cast<const float2*>(gridv) + (long long)(c0 + c) * gvol +
                           (long long)gy * g.N[2] + gz)
                    : make_float2(0.f, 0.f);
    }
  }
  const int c = lane >> 2, kz = lane & 3;
  int kyo[4], rowoff[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    kyo[t] = (t + c) & 3;
    rowoff[t] = kyo[t] * S;
  }
  R3* wrec = rec + warp * 8;
  const int npt = it.z - it.y;
  auto point_at = [&](int base) -> int {
    const int j = base + 8 * lane;
    return (lane < 8 && j < npt) ? entries[it.y + j] : -1;
  };
  auto fetch = [&](int p) {
    PRec R;
    if (p >= 0) R = load_prec(precs, p);
    return R;
  };
  auto publish = [&](int p, const PRec& R) {
    if (p >= 0) {
      R3& Sr = wrec[lane];
      Sr.w[0] = R.w[0];
      Sr.w[1] = R.w[1];
      Sr.w[2] = R.w[2];
      Sr.view = region_view2(g, R, o);
      Sr.p = p;
    }
    __syncwarp();
  };
  int pc = point_at(warp);
  int pn = point_at(warp + 8 * NW);
  PRec Rc = fetch(pc);
  auto build_records = [&](int base) {
    publish(pc, Rc);
    Rc = fetch(pn);
    pc = pn;
    pn = point_at(base + 16 * NW);
  };
  build_records(warp);  // while the region copy is in flight
  {
    bool ok = true;
    if (tma && tid == 0) ok = mbar_wait_bounded(bar, 0, g.skip_copy ? 1u : 1u << 22);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicExch(&g_tlgb_status, 1);
      return;
    }
  }
  // sum over y taps of wy wz v; weights are zero past a record's tap count
  // and every tap of the 4 x 4 box lies inside the region
  auto gather_box = [&](const R3& R) {
    const float wz = (&R.w[2].x)[kz];
    const float* wy = &R.w[1].x;
    const float2* a = reg + c * VOL + (R.view & 2047) + kz;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const float w = wy[kyo[t]] * wz;
      const float2 v = a[rowoff[t]];
      acc.x = fmaf(w, v.x, acc.x);
      acc.y = fmaf(w, v.y, acc.y);
    }
    return acc;
  };
  auto gather_rec = [&](const R3& R) {
    if (lane == 0) {
      float x3[3] = {0.f, 0.f, 0.f};
      for (int e = 1; e < 3; ++e) x3[e] = load_coord(g, locs, R.p, e);
      lane_rec<5>(g, x3, o, true, slow[warp]);
    }
    __syncwarp();
    const Rec<5>& Sr = slow[warp];
    float2 acc = make_float2(0.f, 0.f);
    if (Sr.m[0] > 0)
      for (int kzz = kz; kzz < Sr.m[2]; kzz += 4)
        for (int kyy = 0; kyy < Sr.m[1]; ++kyy) {
          const float w = Sr.wv[1][kyy] * Sr.wv[2][kzz];
          const int ri = c * VOL + Sr.lc[1][kyy] * S + Sr.lc[2][kzz];
          const float2 v = TLGB_IN_RANGE(ri, CG * VOL) ? reg[ri] : make_float2(0.f, 0.f);
          acc.x = fmaf(w, v.x, acc.x);
          acc.y = fmaf(w, v.y, acc.y);
        }
    __syncwarp();
    return acc;
  };
  auto finish = [&](float2 acc, int p) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 1);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 1);
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 2);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 2);
    if (kz == 0 && c0 + c < g.nbatch)
      *reinterpret_cast<float2*>(out + ((long long)(c0 + c) * g.npts + p) * 2) = acc;
  };
  auto one = [&](const R3& R) {
    const unsigned view = R.view;
    if (!((view >> 21) & 1)) return;  // no valid tap (warp-uniform)
    finish((view >> 20) & 1 ? gather_box(R) : gather_rec(R), R.p);
  };
  for (int base = warp; base < npt; base += 8 * NW) {
    if (base != warp) {
      __syncwarp();  // the previous mini-batch has been read
      build_records(base);
    }
    const int nb = min(8, (npt - base + NW - 1) / NW);
    int i = 0;
    for (; i + 1 < nb; i += 2) {
      const R3& R0 = wrec[i];
      const R3& R1 = wrec[i + 1];
      if ((R0.view & R1.view) >> 20 & 1) {
        const float2 a0 = gather_box(R0), a1 = gather_box(R1);
        finish(a0, R0.p);
        finish(a1, R1.p);
      } else {
        one(R0);
        one(R1);
      }
    }
    if (i < nb) one(wrec[i]);
  }
}

// Sum the partial tiles of one split tile in slot order, compensated, and
// write it out.
__global__ void __launch_bounds__(NTHR) adj_reduce_kernel(Geo g, const int4* __restrict__ split,
                                                          const float* __restrict__ partial,
                                                          float* __restrict__ gridv, int CG, int ncg) {
  const int4 sp = split[blockIdx.x];
  const int cg = blockIdx.y;
  const int c0 = cg * CG;
  const int es = g.cplx ? 2 : 1;
  const int ncoil = (int)min((long long)CG, g.nbatch - c0);
  int tc[3];
  {
    int t = sp.x;
    tc[2] = t % g.nt[2];
    t /= g.nt[2];
    tc[1] = t % g.nt[1];
    tc[0] = t / g.nt[1];
  }
  const int tvol = g.T[0] * g.T[1] * g.T[2];
  const int vstride = CG * es;
  const int tfl = (tvol * vstride + 3) & ~3;
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  for (int i = threadIdx.x; i < tvol * ncoil * es; i += NTHR) {
    const int f = i % es;
    int r = i / es;
    const int z = r % g.T[2];
    r /= g.T[2];
    const int y = r % g.T[1];
    r /= g.T[1];
    const int x = r % g.T[0];
    const int cc = r / g.T[0];
    const int gx = tc[0] * g.T[0] + x, gy = tc[1] * g.T[1] + y, gz = tc[2] * g.T[2] + z;
    if (gx >= g.N[0] || gy >= g.N[1] || gz >= g.N[2]) continue;
    const int li = ((x * g.T[1] + y) * g.T[2] + z) * vstride + cc * es + f;
    float s = partial[((long long)sp.y * ncg + cg) * tfl + li], c = 0.f;
    for (int k = 1; k < sp.z; ++k) comp_add(s, c, partial[((long long)(sp.y + k) * ncg + cg) * tfl + li]);
    gridv[((long long)(c0 + cc) * gvol + ((long long)gx * g.N[1] + gy) * g.N[2] + gz) * es + f] = s + c;
  }
}

// ------------------------------------------------------------ trajectory grad

template <typename V, int NORM>
__global__ void __launch_bounds__(NTHR) interp_grad_kernel(Geo g, const int4* __restrict__ items,
                                                              const int32_t* __restrict__ entries,
                                                              const float* __restrict__ locs,
                                                              const V* __restrict__ gridv, const V* __restrict__ a,
                                                              float* __restrict__ grad, int CG, int chunk,
                                                              float* __restrict__ partial) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int4 it = items[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int tc[3];
  {
    int t = it.x;
    tc[2] = t % g.nt[2];
    t /= g.nt[2];
    tc[1] = t % g.nt[1];
    tc[0] = t / g.nt[1];
  }
  int o[3], S[3];
  for (int e = 0; e < 3; ++e) {
    o[e] = tc[e] * g.T[e];
    S[e] = g.T[e] + g.NT[e] - 1;
  }
  const int vol = S[0] * S[1] * S[2];
  V* reg = reinterpret_cast<V*>(smem);
  PTaps<true>* ptb = reinterpret_cast<PTaps<true>*>(smem + (size_t)vol * CG * sizeof(V));
  float* gacc = reinterpret_cast<float*>(ptb + NWARP);  // [chunk][3]
  PTaps<true>& pt = ptb[warp];
  const int npt = it.z - it.y;
  for (int i = threadIdx.x; i < npt * 3; i += NTHR) gacc[i] = 0.f;
  const long long gvol = (long long)g.N[0] * g.N[1] * g.N[2];
  const int CGP = CG <= 1 ? 1 : (CG <= 2 ? 2 : (CG <= 4 ? 4 : 8));
  const int lgc = lg2i(CGP);
  const int c = lane & (CGP - 1);
  const int q = lane >> lgc;
  const int QN = 32 >> lgc;
  const int ncg = (int)((g.nbatch + CG - 1) / CG);
  // blockIdx.y takes a contiguous share of the coil groups (all of them when
  // gridDim.y == 1); its sums go to its partial slot
  const int gps = (ncg + (int)gridDim.y - 1) / (int)gridDim.y;
  const int cg_end = min(ncg, ((int)blockIdx.y + 1) * gps);
  for (int cg = (int)blockIdx.y * gps; cg < cg_end; ++cg) {
    const int c0 = cg * CG;
    const int ncoil = (int)min((long long)CG, g.nbatch - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < vol * ncoil; i += NTHR) {
      int z = i % S[2];
      int r = i / S[2];
      const int y = r % S[1];
      r /= S[1];
      const int x = r % S[0];
      const int cc = r / S[0];
      int gx = o[0] + x, gy = o[1] + y, gz = o[2] + z;
      V v = VT<V>::zero();
      bool in = true;
      if (g.pad == TLGB_PAD_CIRCULAR) {
        gx = wrapi(gx, g.N[0]);
        gy = wrapi(gy, g.N[1]);
        gz = wrapi(gz, g.N[2]);
      } else {
        in = gx < g.N[0] && gy < g.N[1] && gz < g.N[2];
      }
      if (in) v = __ldg(gridv + (long long)(c0 + cc) * gvol + ((long long)gx * g.N[1] + gy) * g.N[2] + gz);
      reg[((x * S[1] + y) * S[2] + z) * CG + cc] = v;
    }
    __syncthreads();
    for (int ei = it.y + warp; ei < it.z; ei += NWARP) {
      const long long p = entries[ei];
      if (!warp_point_taps<NORM, true>(g, locs, p, pt, lane)) continue;
      int l[3];
      for (int e = 0; e < 3; ++e) l[e] = pt.start[e] - o[e];
      V d0 = VT<V>::zero(), d1 = VT<V>::zero(), d2 = VT<V>::zero();
      for (int ka = 0; ka < pt.n[0]; ++ka) {
        for (int kb = 0; kb < pt.n[1]; ++kb) {
          const V* row = reg + (((l[0] + ka) * S[1] + (l[1] + kb)) * S[2] + l[2]) * CG + c;
          for (int kc = q; kc < pt.n[2]; kc += QN) {
            if (c >= ncoil) continue;
            const V gv = row[kc * CG];
            float w0, w1, w2;
            if (NORM == 1) {
              const float wa = pt.w[0][ka], wb = pt.w[1][kb], wc = pt.w[2][kc];
              w0 = pt.dw[0][ka] * wb * wc;
              w1 = wa * pt.dw[1][kb] * wc;
              w2 = wa * wb * pt.dw[2][kc];
            } else {
              const float a0 = pt.w[0][ka], a1 = pt.w[1][kb], a2 = pt.w[2][kc];
              const float rho = sqrtf(a0 * a0 + a1 * a1 + a2 * a2);
              float kd = 0.f;
              if (rho <= 1.0f && rho > 0.f) kd = kern_deriv(g.kernel, rho, g.beta) / rho;
              w0 = g.act[0] ? kd * pt.dw[0][ka] / g.r[0] : 0.f;
              w1 = g.act[1] ? kd * pt.dw[1][kb] / g.r[1] : 0.f;
              w2 = g.act[2] ? kd * pt.dw[2][kc] / g.r[2] : 0.f;
            }
            VT<V>::fma(d0, w0, gv);
            VT<V>::fma(d1, w1, gv);
            VT<V>::fma(d2, w2, gv);
          }
        }
      }
      float r0 = 0.f, r1 = 0.f, r2 = 0.f;
      if (c < ncoil) {
        const V av = __ldg(a + (long long)(c0 + c) * g.npts + p);
        r0 = VT<V>::re_dot(av, d0);
        r1 = VT<V>::re_dot(av, d1);
        r2 = VT<V>::re_dot(av, d2);
      }
      for (int m = 1; m < 32; m <<= 1) {
        r0 += __shfl_xor_sync(0xffffffffu, r0, m);
        r1 += __shfl_xor_sync(0xffffffffu, r1, m);
        r2 += __shfl_xor_sync(0xffffffffu, r2, m);
      }
      if (lane == 0) {
        float* ga = gacc + (ei - it.y) * 3;
        ga[0] += r0;
        ga[1] += r1;
        ga[2] += r2;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  float* dst = gridDim.y == 1 ? grad : partial + (long long)blockIdx.y * g.npts * g.ndim;
  for (int i = threadIdx.x; i < npt; i += NTHR) {
    const long long p = entries[it.y + i];
    for (int e = 3 - g.ndim; e < 3; ++e) dst[p * g.ndim + (e - (3 - g.ndim))] = gacc[i * 3 + e];
  }
}

// grad[i] = sum over slots s of partial[s][i], in slot order
__global__ void __launch_bounds__(256) grad_reduce_kernel(const float* __restrict__ partial, int nsplit, long long n,
                                                          float* __restrict__ grad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = partial[i];
  for (int k = 1; k < nsplit; ++k) s += partial[(long long)k * n + i];
  grad[i] = s;
}

// ------------------------------------------------ 2D trajectory gradient
//
// Per-point gradient records for 2D geometries (built per call, since the
// trajectory may change between calls): the weights and derivative weights
// of the first 4 valid taps in y and z (zero beyond), the first valid tap's
// position (wrapped in circular mode) and the tap counts (cy | cz << 4; a
// zero count marks a point without taps). The taps follow tap_eval; weights
// and derivatives are kern_value and kern_deriv / r, as in warp_point_taps.
struct __align__(16) GRec2 {
  float4 w[2], dw[2];
  int st[2];
  int cnt;
  int pad;
};
static_assert(sizeof(GRec2) == 80, "80-byte gradient records");

__global__ void __launch_bounds__(256) grad_records2_kernel(Geo g, const float* __restrict__ locs,
                                                            GRec2* __restrict__ out) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= g.npts) return;
  GRec2 R;
  int cnt = 0;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int e = 1 + i;
    float w[4] = {0.f, 0.f, 0.f, 0.f}, dw[4] = {0.f, 0.f, 0.f, 0.f};
    int c = 0, st = 0;
    const float x = load_coord(g, locs, p, e);
    if (coord_ok(x)) {
      const int lower = lower_of(g, e, x);
      int s = -1;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const Tap t = tap_eval(g, e, x, lower, k);
        if (!t.valid) continue;
        if (s < 0) s = k;
        if (c < 4) {
          w[c] = kern_value(g.kernel, fabsf(t.d), g.beta);
          dw[c] = kern_deriv(g.kernel, t.d, g.beta) / g.r[e];
        }
        ++c;
      }
      if (c > 0) {
        st = lower + s;
        if (g.pad == TLGB_PAD_CIRCULAR) st = wrapi(st, g.N[e]);
      }
    }
    R.w[i] = make_float4(w[0], w[1], w[2], w[3]);
    R.dw[i] = make_float4(dw[0], dw[1], dw[2], dw[3]);
    R.st[i] = st;
    cnt |= c << (4 * i);
  }
  R.cnt = cnt;
  R.pad = 0;
  out[p] = R;
}

// d/d(y, z) of sum_b Re(conj(a[b, p]) ungrid(grid)[b, p]) for one coil group
// (blockIdx.y) of a 2D geometry with 8 complex entries per group: CTA = 8
// warps sharing the 20 x 20 x 8-entry region of one 16 x 16 tile, as
// fwd_f2_kernel. Lanes = (entry, z-tap): a lane sums its entry's 4 y-taps
// for both derivatives, then all 32 lanes add up. With several coil groups
// the group's sums go to its partial slot (added in order afterwards).
__global__ void __launch_bounds__(256, 3) grad_f2_kernel(const __grid_constant__ CUtensorMap tmap, int use_tma, Geo g,
                                                         const int4* __restrict__ items,
                                                         const int32_t* __restrict__ entries,
                                                         const GRec2* __restrict__ grecs,
                                                         const float* __restrict__ locs,
                                                         const float* __restrict__ gridv, const float2* __restrict__ a,
                                                         float* __restrict__ grad, float* __restrict__ partial) {
  constexpr int CG = 8, S = 20, VOL = S * S, NW = 8;
  constexpr uint32_t RBYTES = VOL * CG * 8;
  extern __shared__ __align__(128) unsigned char smem[];
  float2* reg = reinterpret_cast<float2*>(smem);                  // [8][20][20]
  GRec2* rec = reinterpret_cast<GRec2*>(smem + RBYTES);           // [8 warps][8]
  PTaps<true>* slow = reinterpret_cast<PTaps<true>*>(rec + 64);   // [NW]
  uint64_t* bar = reinterpret_cast<uint64_t*>(slow + NW);
  const int4 it = items[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cg = blockIdx.y;
  const int c0 = cg * CG;
  float* dst = gridDim.y == 1 ? grad : partial + (long long)cg * g.npts * 2;
  int o[3];
  {
    int t = it.x;
    o[2] = (t % g.nt[2]) * g.T[2];
    t /= g.nt[2];
    o[1] = (t % g.nt[1]) * g.T[1];
    o[0] = 0;
  }
  const bool wraps = g.pad == TLGB_PAD_CIRCULAR && (o[1] + S > g.N[1] || o[2] + S > g.N[2]);
  const bool tma = use_tma && !wraps;
  if (tma) {
    if (tid == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
      if (!g.skip_copy) {  // test hook: nothing in flight, so the bounded wait runs out
        mbar_arrive_expect_tx(bar, RBYTES);
        tma_load_4d(reg, &tmap, bar, o[2], o[1], 0, c0);
      }
    }
  } else {
    const int ncoil = (int)min((long long)CG, g.nbatch - c0);
    const long long gvol = (long long)g.N[1] * g.N[2];
    for (int idx = tid; idx < CG * VOL; idx += NW * 32) {
      const int z = idx % S;
      const int r = idx / S;
      const int y = r % S, c = r / S;
      int gy = o[1] + y, gz = o[2] + z;
      bool in = c < ncoil;
      if (g.pad == TLGB_PAD_CIRCULAR) {
        gy = wrapi(gy, g.N[1]);
        gz = wrapi(gz, g.N[2]);
      } else {
        in = in && gy < g.N[1] && gz < g.N[2];
      }
      reg[idx] = in ? __ldg(reinterpret_cast<const float2*>(gridv) + (long long)(c0 + c) * gvol +
                           (long long)gy * g.N[2] + gz)
                    : make_float2(0.f, 0.f);
    }
  }
  const int c = lane >> 2, kz = lane & 3;
  int kyo[4], rowoff[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    kyo[t] = (t + c) & 3;
    rowoff[t] = kyo[t] * S;
  }
  GRec2* wrec = rec + warp * 8;
  const int npt = it.z - it.y;
  // records of the warp's next 8 points: lanes 0-7 copy them into the
  // warp's slots; pad = region base | fast << 20 | ok << 21, cnt unchanged
  auto build_records = [&](int base) {
    const int j = base + 8 * lane;
    if (lane < 8 && j < npt) {
      const int p = entries[it.y + j];
      GRec2 R = grecs[p];
      const int cy = R.cnt & 15, cz = (R.cnt >> 4) & 15;
      const bool ok = cy && cz;
      int f[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        int d = R.st[i] - o[1 + i];
        if (g.pad == TLGB_PAD_CIRCULAR && d < 0) d += g.N[1 + i];
        f[i] = d;
      }
      const bool fast = ok && cy <= 4 && cz <= 4 && f[0] >= 0 && f[0] < 16 && f[1] >= 0 && f[1] < 16;
      R.pad = (fast ? (f[0] * S + f[1]) : 0) | ((fast ? 1 : 0) << 20) | ((ok ? 1 : 0) << 21);
      R.st[0] = p;  // the point index replaces the start (no longer needed)
      wrec[lane] = R;
    }
    __syncwarp();
  };
  build_records(warp);  // while the region copy is in flight
  {
    bool ok = true;
    if (tma && tid == 0) ok = mbar_wait_bounded(bar, 0, g.skip_copy ? 1u : 1u << 22);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicExch(&g_tlgb_status, 1);
      return;
    }
  }
  auto finish = [&](float ry, float rz, int p) {
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
      ry += __shfl_xor_sync(0xffffffffu, ry, m);
      rz += __shfl_xor_sync(0xffffffffu, rz, m);
    }
    if (lane == 0) *reinterpret_cast<float2*>(dst + (long long)p * 2) = make_float2(ry, rz);
  };
  for (int base = warp; base < npt; base += 8 * NW) {
    if (base != warp) {
      __syncwarp();  // the previous mini-batch has been read
      build_records(base);
    }
    const int nb = min(8, (npt - base + NW - 1) / NW);
    for (int i = 0; i < nb; ++i) {
      const GRec2& R = wrec[i];
      const int p = R.st[0];
      const int info = R.pad;
      if (!((info >> 21) & 1)) {
        if (lane == 0) *reinterpret_cast<float2*>(dst + (long long)p * 2) = make_float2(0.f, 0.f);
        continue;
      }
      const float2 av = c0 + c < g.nbatch ? __ldg(a + (long long)(c0 + c) * g.npts + p) : make_float2(0.f, 0.f);
      float2 gy = make_float2(0.f, 0.f), gz = make_float2(0.f, 0.f);
      if ((info >> 20) & 1) {
        const float wz = (&R.w[1].x)[kz], dwz = (&R.dw[1].x)[kz];
        const float* wy = &R.w[0].x;
        const float* dwy = &R.dw[0].x;
        const float2* ab = reg + c * VOL + (info & 1023) + kz;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const float2 v = ab[rowoff[t]];
          const float a1 = dwy[kyo[t]] * wz, a2 = wy[kyo[t]] * dwz;
          gy.x = fmaf(a1, v.x, gy.x);
          gy.y = fmaf(a1, v.y, gy.y);
          gz.x = fmaf(a2, v.x, gz.x);
          gz.y = fmaf(a2, v.y, gz.y);
        }
      } else {
        // 5-tap windows: the warp evaluates the taps, as interp_grad_kernel
        PTaps<true>& pt = slow[warp];
        if (warp_point_taps<1, true>(g, locs, p, pt, lane)) {
          const int l1 = pt.start[1] - o[1], l2 = pt.start[2] - o[2];
          for (int kb = 0; kb < pt.n[1]; ++kb) {
            int yy = l1 + kb;
            if (g.pad == TLGB_PAD_CIRCULAR && yy < 0) yy += g.N[1];
            for (int kc = kz; kc < pt.n[2]; kc += 4) {
              int zz = l2 + kc;
              if (g.pad == TLGB_PAD_CIRCULAR && zz < 0) zz += g.N[2];
              if (yy < 0 || yy >= S || zz < 0 || zz >= S) continue;
              const int ri = c * VOL + yy * S + zz;
              const float2 v = TLGB_IN_RANGE(ri, 8 * VOL) ? reg[ri] : make_float2(0.f, 0.f);
              const float a1 = pt.dw[1][kb] * pt.w[2][kc], a2 = pt.w[1][kb] * pt.dw[2][kc];
              gy.x = fmaf(a1, v.x, gy.x);
              gy.y = fmaf(a1, v.y, gy.y);
              gz.x = fmaf(a2, v.x, gz.x);
              gz.y = fmaf(a2, v.y, gz.y);
            }
          }
        }
        __syncwarp();
      }
      // Re(conj(a) g)
      finish(av.x * gy.x + av.y * gy.y, av.x * gz.x + av.y * gz.y, p);
    }
  }
}

// ------------------------------------------------------------- host helpers

struct PlanLayout {
  int64_t e_max, max_fwd, max_adj, ntiles;
  int64_t off_entries, off_fwd, off_adj, off_split, off_recs, bytes;
  // block lists of the 3D 8-entry gridding (off_blk_entries == 0: none)
  int64_t nblocks, eb_max, max_blk_items, off_blk_entries, off_blk_items, off_blk_split, off_blk_rows;
  // tmp
  int64_t t_cnt, t_keys, t_keys2, t_vals2, t_counts, t_hist, t_total, t_bytes;
};

constexpr int64_t kFwdChunk = 512;
constexpr int64_t kAdjChunk = 1024;

std::atomic<int> g_test_skip_copy{0};  // tlgb_test_skip_region_copy

int make_geo(const tlgb_interp_desc* d, Geo& g) {
  if (!d) TLGB_FAIL(TLGB_ERR_INVALID, "null interp descriptor");
  if (d->ndim < 1 || d->ndim > 3) TLGB_FAIL(TLGB_ERR_INVALID, "ndim must be 1, 2 or 3");
  if (d->kernel != TLGB_KERNEL_KAISER_BESSEL && d->kernel != TLGB_KERNEL_SPLINE)
    TLGB_FAIL(TLGB_ERR_INVALID, "unknown kernel");
  if (d->norm != 1 && d->norm != 2) TLGB_FAIL(TLGB_ERR_INVALID, "norm must be 1 or 2");
  if (d->pad_mode != TLGB_PAD_CIRCULAR && d->pad_mode != TLGB_PAD_ZERO) TLGB_FAIL(TLGB_ERR_INVALID, "unknown pad mode");
  if (d->npts < 0 || d->nbatch < 0) TLGB_FAIL(TLGB_ERR_INVALID, "negative size");
  // the 8-entry kernels launch one grid row per 8 batch entries (at most 65535)
  if (d->nbatch > TLGB_INTERP_MAX_BATCH)
    TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "batch above 524280 entries in one call: split the batch");
  memset(&g, 0, sizeof(g));
  g.skip_copy = g_test_skip_copy.load();
  g.ndim = d->ndim;
  const int off = 3 - d->ndim;
  int maxnt = 1;
  for (int e = 0; e < 3; ++e) {
    if (e < off) {
      g.N[e] = 1;
      g.NT[e] = 1;
      g.r[e] = 1.f;
      g.act[e] = 0;
      continue;
    }
    const int64_t n = d->grid_size[e - off];
    const float w = d->width[e - off];
    if (n < 1 || n > (1 << 24)) TLGB_FAIL(TLGB_ERR_INVALID, "grid size must be in [1, 2^24]");
    if (!(w > 0.f)) TLGB_FAIL(TLGB_ERR_INVALID, "kernel width must be positive");
    // len(torch.arange(w + 1)) taps, as the reference's diff grid
    const int nt = (int)ceil((double)w + 1.0);
    if (nt > NTMAX) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "kernel width must be below 15 grid units");
    g.N[e] = (int)n;
    g.NT[e] = nt;
    g.r[e] = w / 2.0f;
    {
      int ex = 0;
      const float mant = frexpf(g.r[e], &ex);
      g.rpow2[e] = (mant == 0.5f) ? 1 : 0;
      g.rinv[e] = 1.0f / g.r[e];
    }
    g.act[e] = 1;
    maxnt = std::max(maxnt, nt);
  }
  if (d->ndim == 3 && maxnt > 9) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "3D kernel width must be below 8 grid units");
  const int T3[3] = {8, 8, 8}, T2[3] = {1, 16, 16}, T1[3] = {1, 1, 512};
  const int* T = d->ndim == 3 ? T3 : (d->ndim == 2 ? T2 : T1);
  g.wrap_safe = 1;
  g.tv_off = -1;
  for (int e = 0; e < 3; ++e) {
    g.T[e] = std::min(T[e], g.N[e]);
    g.nt[e] = (int)cdiv(g.N[e], g.T[e]);
    if (g.act[e] && g.N[e] < g.NT[e]) g.wrap_safe = 0;
  }
  g.kernel = d->kernel;
  g.norm = d->norm;
  g.pad = d->pad_mode;
  g.cplx = d->is_complex ? 1 : 0;
  g.beta = d->beta;
  g.npts = d->npts;
  g.nbatch = d->nbatch;
  if ((int64_t)g.nt[0] * g.nt[1] * g.nt[2] >= (1ll << 30)) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "too many tiles");
  return TLGB_OK;
}

// Tiles one point can touch along a dim: 2 for T >= taps - 1, 3 where a
// circular window can cross both a ragged last tile and the wrap.
int64_t max_tiles_per_dim(const Geo& g, int e) {
  if (g.nt[e] == 1) return 1;
  const int m = g.N[e] % g.T[e];
  if (g.pad == TLGB_PAD_CIRCULAR && m != 0 && m < g.NT[e] - 1) return std::min(3, g.nt[e]);
  return 2;
}

// Geometries whose plan carries per-point tap records (the 3D 8-entry kernels)
bool records_ok(const Geo& g) {
  if (g.norm != 1) return false;
  if (g.ndim == 3)
    return g.T[0] == 8 && g.T[1] == 8 && g.T[2] == 8 && g.NT[0] == 5 && g.NT[1] == 5 && g.NT[2] == 5;
  return g.ndim == 2 && g.T[1] == 16 && g.T[2] == 16 && g.NT[1] == 5 && g.NT[2] == 5;
}

// Geometries whose plans also carry block lists (adj_b3_kernel): those of
// the tap records (3D 8^3 or 2D 16 x 16 tiles, at most 5 taps per dim), and
// in circular mode every active dim a multiple of the block edge and at
// least 16 cells, so that a wrapped window meets at most 2 blocks per dim and
// each of them once.
bool blocks_ok(const Geo& g) {
  if (g.ndim < 2 || !records_ok(g) || g.npts >= (1ll << kSelShift)) return false;
  if (g.pad == TLGB_PAD_CIRCULAR)
    for (int e = 3 - g.ndim; e < 3; ++e)
      if (g.N[e] < 16 || g.N[e] % block_edge(g.ndim, e) != 0) return false;
  const int64_t nb = (int64_t)blocks_along(g, 0) * blocks_along(g, 1) * blocks_along(g, 2);
  return nb < (1ll << 31);
}

// Blocks one window can meet along a dim: 2 (at most 5 taps over 4 cells)
int64_t max_blocks_per_dim(const Geo& g, int e) { return blocks_along(g, e) == 1 ? 1 : 2; }

// The kernel, norm and beta a plan's records hold weights for
int64_t kernel_key(const Geo& g) {
  uint32_t bits;
  memcpy(&bits, &g.beta, 4);
  return (int64_t)bits | ((int64_t)g.kernel << 32) | ((int64_t)g.norm << 40) | ((int64_t)1 << 48);
}

PlanLayout layout(const Geo& g) {
  PlanLayout L;
  L.e_max = g.npts * max_tiles_per_dim(g, 0) * max_tiles_per_dim(g, 1) * max_tiles_per_dim(g, 2);
  L.ntiles = (int64_t)g.nt[0] * g.nt[1] * g.nt[2];
  L.max_fwd = L.ntiles + cdiv(g.npts, kFwdChunk) + 1;
  L.max_adj = L.ntiles + cdiv(L.e_max, kAdjChunk) + 1;
  size_t o = 0;
  L.off_entries = o;
  o = align_up(o + (size_t)std::max<int64_t>(L.e_max, 1) * 4, 256);
  L.off_fwd = o;
  o = align_up(o + (size_t)L.max_fwd * 16, 256);
  L.off_adj = o;
  o = align_up(o + (size_t)L.max_adj * 16, 256);
  L.off_split = o;
  o = align_up(o + (size_t)(L.ntiles + 1) * 16, 256);
  L.off_recs = 0;
  if (records_ok(g) && g.npts > 0) {
    L.off_recs = o;
    o = align_up(o + (size_t)g.npts * 64, 256);
  }
  L.nblocks = L.eb_max = L.max_blk_items = 0;
  L.off_blk_entries = L.off_blk_items = L.off_blk_split = L.off_blk_rows = 0;
  if (blocks_ok(g) && g.npts > 0) {
    L.nblocks = (int64_t)blocks_along(g, 0) * blocks_along(g, 1) * blocks_along(g, 2);
    L.eb_max = g.npts * max_blocks_per_dim(g, 0) * max_blocks_per_dim(g, 1) * max_blocks_per_dim(g, 2);
    L.max_blk_items = L.nblocks + cdiv(L.eb_max, kBlkPart) + 1;
    L.off_blk_entries = o;
    o = align_up(o + (size_t)L.eb_max * 4, 256);
    L.off_blk_items = o;
    o = align_up(o + (size_t)L.max_blk_items * 16, 256);
    L.off_blk_split = o;
    o = align_up(o + (size_t)(L.nblocks + 1) * 16, 256);
    L.off_blk_rows = o;
    o = align_up(o + (size_t)g.npts * row_floats(g.ndim) * 4, 256);
  }
  L.bytes = o;
  const int64_t pairs = std::max<int64_t>(std::max(L.e_max, L.eb_max), 1);  // sort buffers serve both lists
  size_t t = 0;
  L.t_cnt = t;
  t = align_up(t + (size_t)(g.npts + 1) * 4, 256);
  L.t_keys = t;
  t = align_up(t + (size_t)pairs * 4, 256);
  L.t_keys2 = t;
  t = align_up(t + (size_t)pairs * 4, 256);
  L.t_vals2 = t;
  t = align_up(t + (size_t)pairs * 4, 256);
  L.t_counts = t;
  t = align_up(t + (size_t)radix_counts_len(pairs) * 4, 256);
  L.t_hist = t;
  t = align_up(t + (size_t)(std::max(2 * L.ntiles, L.nblocks) + 1) * 4, 256);
  L.t_total = t;
  t = align_up(t + 16, 256);
  L.t_bytes = t;
  return L;
}

int value_size(const Geo& g) { return g.cplx ? 8 : 4; }

constexpr int NWF = 16;  // warps of a forward CTA (one CTA per SM shares one staged region)

// taps stored per dim by the kernels: 5 covers widths < 4 (the NUFFT default)
int ntb_for(const Geo& g) {
  const int m = std::max(g.NT[0], std::max(g.NT[1], g.NT[2]));
  if (m <= 5) return 5;
  return g.ndim == 3 ? 9 : 16;
}
size_t pt_bytes(int ntb) {
  return ntb == 5 ? sizeof(Rec<5>) : (ntb == 9 ? sizeof(Rec<9>) : sizeof(Rec<16>));
}

int64_t region_vol(const Geo& g) {
  return (int64_t)(g.T[0] + g.NT[0] - 1) * (g.T[1] + g.NT[1] - 1) * (g.T[2] + g.NT[2] - 1);
}

// batch entries staged per forward CTA
bool fast3(const Geo& g, int cg);
bool fast2(const Geo& g, int cg);

// A batch of fewer than 8 entries on a geometry of the dedicated 8-entry
// kernels (3D 8^3 or 2D 16 x 16 tiles, width in (3, 4], norm 1, complex) runs
// on them as one group: the missing entries are staged as zeros and never
// written. Those kernels stage each point once for all entries, so even one
// entry runs faster there than on the generic kernels.
bool small_batch_on_fast_kernels(const Geo& g) { return g.nbatch < 8 && (fast3(g, 8) || fast2(g, 8)); }

int fwd_cg(const Geo& g) {
  if (small_batch_on_fast_kernels(g)) return 8;
  int cg = (int)std::min<long long>(std::max<long long>(g.nbatch, 1), CGMAX);
  const int64_t cap = 220 * 1024 - NWF * 32 * (int64_t)pt_bytes(ntb_for(g));
  while (cg > 1 && region_vol(g) * cg * value_size(g) > cap) --cg;
  return cg;
}

size_t fwd_smem(const Geo& g, int cg) {
  return align_up((size_t)region_vol(g) * cg * value_size(g), 16) + NWF * 32 * pt_bytes(ntb_for(g));
}

int adj_cg(const Geo& g) {
  if (small_batch_on_fast_kernels(g)) return 8;
  return (int)std::min<long long>(std::max<long long>(g.nbatch, 1), CGMAX);
}

int64_t tile_floats(const Geo& g, int cg) {
  return ((int64_t)g.T[0] * g.T[1] * g.T[2] * cg * (g.cplx ? 2 : 1) + 3) & ~3ll;
}

size_t adj_smem(const Geo& g, int cg) {
  return (size_t)tile_floats(g, cg) * 4 + 32 * pt_bytes(ntb_for(g)) + 32 * (size_t)cg * (g.cplx ? 2 : 1) * 4;
}

// the grad kernel keeps the warp-cooperative tap buffers
int grad_cg(const Geo& g, size_t taps_bytes) {
  int cg = (int)std::min<long long>(std::max<long long>(g.nbatch, 1), CGMAX);
  const int64_t cap = 112 * 1024 - NWARP * (int64_t)taps_bytes - 1024;
  while (cg > 1 && region_vol(g) * cg * value_size(g) > cap) --cg;
  return cg;
}

size_t grad_smem(const Geo& g, int cg, size_t taps_bytes) {
  return (size_t)region_vol(g) * cg * value_size(g) + NWARP * taps_bytes;
}

// Parts the coil groups of the trajectory gradient are split into: enough
// CTAs to fill the device when a plan has few tiles and the batch many
// groups (each part restages the region and re-evaluates the taps).
int grad_splits(const Geo& g, const tlgb_interp_plan_info* info) {
  const int cg = grad_cg(g, sizeof(PTaps<true>));
  const long long ncg = cdiv(std::max<long long>(g.nbatch, 1), cg);
  const long long items = std::max<long long>(info->n_fwd_items, 1);
  const long long want = cdiv(8ll * sm_count(), items);  // ~8 CTAs per SM
  return (int)std::max(1ll, std::min(ncg, want));
}

size_t grad_scratch_bytes(const Geo& g, int nsplit) {
  return nsplit > 1 ? (size_t)nsplit * g.npts * g.ndim * sizeof(float) : 0;
}

bool fast2(const Geo& g, int cg);

// The 2D 8-entry gradient (grad_f2_kernel): complex values, norm 1, 8
// entries per coil group. Its scratch holds the per-point gradient records
// and, with more than one coil group, one partial slot per group.
bool grad_fast2(const Geo& g) { return g.cplx && g.norm == 1 && g.nbatch >= 8 && fast2(g, 8); }

size_t grad2_records_bytes(const Geo& g) { return align_up((size_t)g.npts * sizeof(GRec2), 256); }

size_t grad2_scratch_bytes(const Geo& g) {
  const long long ncg = cdiv(g.nbatch, 8);
  return grad2_records_bytes(g) + (ncg > 1 ? (size_t)ncg * g.npts * 2 * sizeof(float) : 0);
}

int check_plan(const Geo& g, const tlgb_interp_plan_info* info, const void* plan) {
  if (!info || !plan) TLGB_FAIL(TLGB_ERR_INVALID, "missing plan");
  for (int e = 0; e < 3; ++e)
    if (info->tile[e] != g.T[e] || info->n_tile[e] != g.nt[e])
      TLGB_FAIL(TLGB_ERR_INVALID, "plan was built for another grid");
  if (info->off_records > 0 && records_ok(g) && info->kernel_key != kernel_key(g))
    TLGB_FAIL(TLGB_ERR_INVALID, "plan was built for another kernel, norm or beta (its tap weights are stored)");
  return TLGB_OK;
}

template <typename F>
int set_smem(F* kernel, size_t bytes) {
  TLGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  TLGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_interp_plan_size(const tlgb_interp_desc* d, size_t* plan_bytes, size_t* tmp_bytes) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  const PlanLayout L = layout(g);
  if (std::max(L.e_max, L.eb_max) >= (1ll << 31)) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "too many points for one plan");
  if (plan_bytes) *plan_bytes = (size_t)L.bytes;
  if (tmp_bytes) *tmp_bytes = (size_t)L.t_bytes;
  return TLGB_OK;
}

extern "C" int tlgb_interp_plan_build(const tlgb_interp_desc* d, const float* locs, void* plan, size_t plan_bytes,
                                      void* tmp, size_t tmp_bytes, tlgb_interp_plan_info* info,
                                      tlgb_stream_t stream) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  const PlanLayout L = layout(g);
  if (std::max(L.e_max, L.eb_max) >= (1ll << 31)) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "too many points for one plan");
  if (!info || !plan || !tmp || (g.npts > 0 && !locs)) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  if (plan_bytes < (size_t)L.bytes || tmp_bytes < (size_t)L.t_bytes) TLGB_FAIL(TLGB_ERR_WORKSPACE, "plan workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  char* P = (char*)plan;
  char* Tm = (char*)tmp;
  uint32_t* cnt = (uint32_t*)(Tm + L.t_cnt);
  uint32_t* keys = (uint32_t*)(Tm + L.t_keys);
  uint32_t* keys2 = (uint32_t*)(Tm + L.t_keys2);
  int32_t* vals2 = (int32_t*)(Tm + L.t_vals2);
  uint32_t* counts = (uint32_t*)(Tm + L.t_counts);
  uint32_t* hist = (uint32_t*)(Tm + L.t_hist);
  uint32_t* total = (uint32_t*)(Tm + L.t_total);
  int32_t* entries = (int32_t*)(P + L.off_entries);

  uint32_t E = 0;
  if (g.npts > 0) {
    const unsigned nb = (unsigned)cdiv(g.npts, 256);
    plan_count_kernel<<<nb, 256, 0, s>>>(g, locs, cnt);
    TLGB_CHECK_LAUNCH();
    TLGB_TRY(exclusive_scan_u32(cnt, cnt, g.npts, total, counts, s));  // counts is free until the sort
    plan_emit_kernel<<<nb, 256, 0, s>>>(g, locs, cnt, keys, entries);
    TLGB_CHECK_LAUNCH();
    if (L.off_recs > 0) point_records_kernel<<<nb, 256, 0, s>>>(g, locs, (PRec*)(P + L.off_recs));
    TLGB_CHECK_LAUNCH();
    TLGB_CUDA(cudaMemcpyAsync(&E, total, 4, cudaMemcpyDeviceToHost, s));
    TLGB_CUDA(cudaStreamSynchronize(s));
  }
  int bits = 1;
  while ((1ll << bits) < 2 * L.ntiles) ++bits;
  TLGB_TRY(radix_sort_pairs(keys, entries, keys2, vals2, counts, (int64_t)E, bits, s));
  TLGB_CUDA(cudaMemsetAsync(hist, 0, (size_t)(2 * L.ntiles) * 4, s));
  if (E > 0) {
    key_hist_kernel<<<(unsigned)cdiv(E, 256), 256, 0, s>>>(keys, E, hist);
    TLGB_CHECK_LAUNCH();
  }
  std::vector<uint32_t> h((size_t)(2 * L.ntiles));
  TLGB_CUDA(cudaMemcpyAsync(h.data(), hist, h.size() * 4, cudaMemcpyDeviceToHost, s));
  TLGB_CUDA(cudaStreamSynchronize(s));

  // work items (host). Results do not depend on the order, because every
  // item writes its own tile, slot or points. Gather items stay in tile
  // order, so neighbouring regions are read while their shared halos are in
  // L2. Gridding items go heaviest first, for load balance.
  std::vector<int4> fwd, adj, split;
  int64_t pos = 0, n_home = 0, n_partials = 0;
  for (int64_t t = 0; t < L.ntiles; ++t) {
    const int64_t nh = h[2 * t], nn = h[2 * t + 1];
    const int64_t beg = pos, hend = pos + nh, end = pos + nh + nn;
    n_home += nh;
    for (int64_t b = beg; b < hend; b += kFwdChunk)
      fwd.push_back(make_int4((int)t, (int)b, (int)std::min(hend, b + kFwdChunk), -1));
    const int64_t na = end - beg;
    if (na <= kAdjChunk) {
      adj.push_back(make_int4((int)t, (int)beg, (int)end, -1));
    } else {
      const int64_t nch = cdiv(na, kAdjChunk);
      split.push_back(make_int4((int)t, (int)n_partials, (int)nch, 0));
      for (int64_t k = 0; k < nch; ++k)
        adj.push_back(make_int4((int)t, (int)(beg + k * kAdjChunk), (int)std::min(end, beg + (k + 1) * kAdjChunk),
                                (int)(n_partials + k)));
      n_partials += nch;
    }
    pos = end;
  }
  auto heavier = [](const int4& a, const int4& b) { return (a.z - a.y) > (b.z - b.y); };
  std::stable_sort(adj.begin(), adj.end(), heavier);
  if ((int64_t)fwd.size() > L.max_fwd || (int64_t)adj.size() > L.max_adj)
    TLGB_FAIL(TLGB_ERR_DEVICE, "work list larger than its bound");
  if (!fwd.empty()) TLGB_CUDA(cudaMemcpyAsync(P + L.off_fwd, fwd.data(), fwd.size() * 16, cudaMemcpyHostToDevice, s));
  if (!adj.empty()) TLGB_CUDA(cudaMemcpyAsync(P + L.off_adj, adj.data(), adj.size() * 16, cudaMemcpyHostToDevice, s));
  if (!split.empty())
    TLGB_CUDA(cudaMemcpyAsync(P + L.off_split, split.data(), split.size() * 16, cudaMemcpyHostToDevice, s));
  // host vectors are freed on return: make the copies complete first
  TLGB_CUDA(cudaStreamSynchronize(s));

  // Block lists (3D 8-entry gridding): (point, block) pairs from the tap
  // records, sorted stably by block; work items of at most kBlkPart entries
  // (dense blocks split into parts summed in order afterwards) and runs of
  // up to kZeroRun empty blocks. A point's blocks are neighbours, so items
  // in spatial order read its rows and values again while they are still in
  // L2 (in heaviest-first order nearly every read of them went to DRAM).
  uint32_t Eb = 0;
  std::vector<int4> bitems, bsplit;
  int64_t n_bpartials = 0;
  if (L.off_blk_entries > 0) {
    const PRec* recs = (const PRec*)(P + L.off_recs);
    int32_t* bentries = (int32_t*)(P + L.off_blk_entries);
    const unsigned nb = (unsigned)cdiv(g.npts, 256);
    blk_count_kernel<<<nb, 256, 0, s>>>(g, recs, cnt);
    TLGB_CHECK_LAUNCH();
    TLGB_TRY(exclusive_scan_u32(cnt, cnt, g.npts, total, counts, s));
    blk_emit_kernel<<<nb, 256, 0, s>>>(g, recs, cnt, keys, bentries);
    TLGB_CHECK_LAUNCH();
    blk_rows_kernel<<<nb, 256, 0, s>>>(g, locs, recs, (float*)(P + L.off_blk_rows));
    TLGB_CHECK_LAUNCH();
    TLGB_CUDA(cudaMemcpyAsync(&Eb, total, 4, cudaMemcpyDeviceToHost, s));
    TLGB_CUDA(cudaStreamSynchronize(s));
    int bbits = 1;
    while ((1ll << bbits) < L.nblocks) ++bbits;
    TLGB_TRY(radix_sort_pairs(keys, bentries, keys2, vals2, counts, (int64_t)Eb, bbits, s));
    TLGB_CUDA(cudaMemsetAsync(hist, 0, (size_t)L.nblocks * 4, s));
    if (Eb > 0) {
      key_hist_kernel<<<(unsigned)cdiv(Eb, 256), 256, 0, s>>>(keys, Eb, hist);
      TLGB_CHECK_LAUNCH();
    }
    std::vector<uint32_t> hb((size_t)L.nblocks);
    TLGB_CUDA(cudaMemcpyAsync(hb.data(), hist, hb.size() * 4, cudaMemcpyDeviceToHost, s));
    TLGB_CUDA(cudaStreamSynchronize(s));
    // items in cube order: cubes of kCube^3 blocks, blocks in key order
    // inside a cube, so that the blocks a point meets are worked on close
    // together in time and find its rows and values in L2
    std::vector<int64_t> bstart((size_t)L.nblocks + 1, 0);
    for (int64_t b = 0; b < L.nblocks; ++b) bstart[(size_t)b + 1] = bstart[(size_t)b] + hb[(size_t)b];
    const int64_t nbx = blocks_along(g, 0), nby = blocks_along(g, 1), nbz = blocks_along(g, 2);
    auto add_block = [&](int64_t b) {
      const int64_t n = hb[(size_t)b], bpos = bstart[(size_t)b];
      if (n == 0) {
        int4* last = bitems.empty() ? nullptr : &bitems.back();
        if (last && last->y == last->z && last->x - last->w == b && -last->w < kZeroRun)
          --last->w;  // extends the run of empty blocks ending at block b - 1
        else
          bitems.push_back(make_int4((int)b, (int)bpos, (int)bpos, -1));
        return;
      }
      if (n <= kBlkPart) {
        bitems.push_back(make_int4((int)b, (int)bpos, (int)(bpos + n), -1));
        return;
      }
      const int64_t nch = cdiv(n, kBlkPart);
      bsplit.push_back(make_int4((int)b, (int)n_bpartials, (int)nch, 0));
      for (int64_t k = 0; k < nch; ++k)
        bitems.push_back(make_int4((int)b, (int)(bpos + k * kBlkPart), (int)std::min(bpos + n, bpos + (k + 1) * kBlkPart),
                                   (int)(n_bpartials + k)));
      n_bpartials += nch;
    };
    for (int64_t cx = 0; cx < nbx; cx += kCube)
      for (int64_t cy = 0; cy < nby; cy += kCube)
        for (int64_t cz = 0; cz < nbz; cz += kCube)
          for (int64_t bx = cx; bx < std::min(nbx, cx + kCube); ++bx)
            for (int64_t by = cy; by < std::min(nby, cy + kCube); ++by)
              for (int64_t bz = cz; bz < std::min(nbz, cz + kCube); ++bz) add_block((bx * nby + by) * nbz + bz);
    if ((int64_t)bitems.size() > L.max_blk_items) TLGB_FAIL(TLGB_ERR_DEVICE, "block work list larger than its bound");
    // split blocks with the most parts first: their sums are the longest
    // chains of the reduction, so they start in its first wave
    std::stable_sort(bsplit.begin(), bsplit.end(), [](const int4& a, const int4& b) { return a.z > b.z; });
    if (!bitems.empty())
      TLGB_CUDA(cudaMemcpyAsync(P + L.off_blk_items, bitems.data(), bitems.size() * 16, cudaMemcpyHostToDevice, s));
    if (!bsplit.empty())
      TLGB_CUDA(cudaMemcpyAsync(P + L.off_blk_split, bsplit.data(), bsplit.size() * 16, cudaMemcpyHostToDevice, s));
    TLGB_CUDA(cudaStreamSynchronize(s));
  }

  memset(info, 0, sizeof(*info));
  info->n_entries = E;
  info->n_tiles = L.ntiles;
  for (int e = 0; e < 3; ++e) {
    info->tile[e] = g.T[e];
    info->n_tile[e] = g.nt[e];
  }
  info->n_fwd_items = (int64_t)fwd.size();
  info->n_adj_items = (int64_t)adj.size();
  info->n_partials = n_partials;
  info->n_split_tiles = (int64_t)split.size();
  info->chunk = kAdjChunk;
  info->off_entries = L.off_entries;
  info->off_fwd_items = L.off_fwd;
  info->off_adj_items = L.off_adj;
  info->off_split = L.off_split;
  info->plan_bytes = L.bytes;
  info->off_records = L.off_recs;
  info->kernel_key = L.off_recs > 0 ? kernel_key(g) : 0;
  info->n_home = n_home;
  if (L.off_blk_entries > 0) {
    info->n_blk_entries = Eb;
    info->n_blk_items = (int64_t)bitems.size();
    info->n_blk_partials = n_bpartials;
    info->n_blk_split = (int64_t)bsplit.size();
    info->off_blk_entries = L.off_blk_entries;
    info->off_blk_items = L.off_blk_items;
    info->off_blk_split = L.off_blk_split;
    info->off_blk_rows = L.off_blk_rows;
  }
  return TLGB_OK;
}

namespace tlgb {
namespace {
bool fast3(const Geo& g, int cg);
bool fast2(const Geo& g, int cg);

// Batch entries per group of the block gridding: 1, 2 or 4 for 3D batches of
// at most 4 entries (adj_bn_kernel), else 8 (adj_b3_kernel).
int blk_entries(const Geo& g) {
  if (g.ndim != 3 || g.nbatch > 4) return 8;
  return g.nbatch <= 1 ? 1 : (g.nbatch <= 2 ? 2 : 4);
}

// bytes of the block path's partial blocks: 64 cells x E complex entries per
// part and group
size_t blk_partial_bytes(const tlgb_interp_plan_info* info, int64_t ncg, int E) {
  return align_up((size_t)info->n_blk_partials * ncg * 64 * 2 * E * sizeof(float), 256);
}

// Gridding scratch: the partial tiles of split tiles (block path: the partial
// blocks and the work counters), then (8-entry paths) the point values
// transposed to point-major order.
void adj_scratch_parts(const Geo& g, const tlgb_interp_plan_info* info, size_t& partial_bytes, size_t& tv_bytes) {
  const int cg = adj_cg(g);
  const int64_t ncg = cdiv(std::max<long long>(g.nbatch, 1), cg);
  const bool blocks = (fast3(g, cg) || fast2(g, cg)) && info->n_blk_items > 0;
  partial_bytes = blocks ? blk_partial_bytes(info, ncg, blk_entries(g)) + align_up((size_t)ncg * sizeof(int), 256)
                         : align_up((size_t)info->n_partials * ncg * tile_floats(g, cg) * sizeof(float), 256);
  // adj_bn_kernel reads the values in place
  tv_bytes = ((fast3(g, cg) || fast2(g, cg)) && info->off_records > 0 && !(blocks && blk_entries(g) < 8))
                 ? (size_t)ncg * g.npts * 8 * 8
                 : 0;
}
}  // namespace
}  // namespace tlgb

extern "C" int tlgb_interp_adjoint_scratch_size(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info,
                                                size_t* bytes) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  if (!info || !bytes) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  size_t pb = 0, tb = 0;
  adj_scratch_parts(g, info, pb, tb);
  *bytes = pb + tb;
  return TLGB_OK;
}

namespace tlgb {
namespace {

// the unrolled paths: 3D, 8^3 tiles, 5 taps per dim (width in (3, 4]), 8 complex batch entries
bool fast3(const Geo& g, int cg) {
  return g.ndim == 3 && g.cplx && cg == 8 && g.norm == 1 && g.T[0] == 8 && g.T[1] == 8 && g.T[2] == 8 && g.NT[0] == 5 &&
         g.NT[1] == 5 && g.NT[2] == 5;
}

template <int N, int NDIM, int NTB, bool F3>
int launch_fwd_t2(const Geo& g, int cg, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                  const void* grid, void* out, cudaStream_t s) {
  const int64_t ncg = cdiv(g.nbatch, cg);
  const size_t sm = fwd_smem(g, cg);
  auto* k = interp_fwd_kernel<N, NDIM, NTB, NWF, F3>;
  TLGB_TRY(set_smem(k, sm));
  dim3 grd((unsigned)info->n_fwd_items, (unsigned)ncg);
  k<<<grd, NWF * 32, sm, s>>>(g, (const int4*)(P + info->off_fwd_items), (const int32_t*)(P + info->off_entries),
                             locs, (const float*)grid, (float*)out, cg);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

template <int N, int NDIM, int NTB, bool F3>
int launch_adj_t2(const Geo& g, int cg, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                  const void* vals, void* grid, void* scratch, cudaStream_t s) {
  const int64_t ncg = cdiv(g.nbatch, cg);
  const size_t sm = adj_smem(g, cg);
  auto* k = interp_adj_kernel<N, NDIM, NTB, F3>;
  TLGB_TRY(set_smem(k, sm));
  dim3 grd((unsigned)info->n_adj_items, (unsigned)ncg);
  k<<<grd, 32, sm, s>>>(g, (const int4*)(P + info->off_adj_items), (const int32_t*)(P + info->off_entries), locs,
                       (const float*)vals, (float*)grid, (float*)scratch, cg);
  TLGB_CHECK_LAUNCH();
  if (info->n_split_tiles > 0) {
    dim3 g2((unsigned)info->n_split_tiles, (unsigned)ncg);
    adj_reduce_kernel<<<g2, NTHR, 0, s>>>(g, (const int4*)(P + info->off_split), (const float*)scratch, (float*)grid,
                                          cg, (int)ncg);
    TLGB_CHECK_LAUNCH();
  }
  return TLGB_OK;
}

using sm100::tensor_map_encoder;

template <int CG>
int launch_fwd_f3_t(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                    const void* grid, void* out, cudaStream_t s) {
  const int64_t ncg = cdiv(g.nbatch, CG);
  const size_t sm = 12 * 12 * 12 * CG * 8 + kGB * sizeof(R3) + 8 * sizeof(Rec<5>) + 8;
  // 4D tensor map over [batch][X][Y][Z] complex64 (8-byte elements), box 12^3 x CG
  CUtensorMap tmap;
  memset(&tmap, 0, sizeof(tmap));
  int use_tma = 0;
  auto enc = tensor_map_encoder();
  const uint64_t zb = (uint64_t)g.N[2] * 8;
  if (enc && (zb % 16) == 0 && ((uintptr_t)grid % 16) == 0) {
    const cuuint64_t dims[4] = {(cuuint64_t)g.N[2], (cuuint64_t)g.N[1], (cuuint64_t)g.N[0], (cuuint64_t)g.nbatch};
    const cuuint64_t strides[3] = {zb, zb * g.N[1], zb * g.N[1] * g.N[0]};
    const cuuint32_t box[4] = {12, 12, 12, (cuuint32_t)CG};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<void*>(grid), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    use_tma = (r == CUDA_SUCCESS) ? 1 : 0;
  }
  TLGB_TRY(set_smem(fwd_f3_kernel<CG>, sm));
  dim3 grd((unsigned)info->n_fwd_items, (unsigned)ncg);
  fwd_f3_kernel<CG><<<grd, 256, sm, s>>>(tmap, use_tma, g, (const int4*)(P + info->off_fwd_items),
                                         (const int32_t*)(P + info->off_entries), (const PRec*)(P + info->off_records),
                                         locs, (const float*)grid, (float*)out);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

// batches of at most 4 entries stage only their own entries' regions
int launch_fwd_f3(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                  const void* grid, void* out, cudaStream_t s) {
  if (g.nbatch <= 1) return launch_fwd_f3_t<1>(g, info, P, locs, grid, out, s);
  if (g.nbatch <= 2) return launch_fwd_f3_t<2>(g, info, P, locs, grid, out, s);
  if (g.nbatch <= 4) return launch_fwd_f3_t<4>(g, info, P, locs, grid, out, s);
  return launch_fwd_f3_t<8>(g, info, P, locs, grid, out, s);
}

bool fast2(const Geo& g, int cg) {
  return g.ndim == 2 && g.cplx && cg == 8 && g.norm == 1 && g.T[1] == 16 && g.T[2] == 16 && g.NT[1] == 5 &&
         g.NT[2] == 5;
}

// [batch][Y][Z] complex64 as a 4D map {Z, Y, 1, batch}, box 20 x 20 x 1 x 8
// (the staged region of a 16 x 16 tile); 0 when TMA cannot be used
int region_map2(const Geo& g, const void* grid, CUtensorMap& tmap) {
  memset(&tmap, 0, sizeof(tmap));
  auto enc = tensor_map_encoder();
  const uint64_t zb = (uint64_t)g.N[2] * 8;
  if (!enc || (zb % 16) != 0 || ((uintptr_t)grid % 16) != 0) return 0;
  const cuuint64_t dims[4] = {(cuuint64_t)g.N[2], (cuuint64_t)g.N[1], 1, (cuuint64_t)g.nbatch};
  const cuuint64_t strides[3] = {zb, zb * g.N[1], zb * g.N[1]};
  const cuuint32_t box[4] = {20, 20, 1, 8};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<void*>(grid), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 1 : 0;
}

int launch_fwd_f2(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                  const void* grid, void* out, cudaStream_t s) {
  const int64_t ncg = cdiv(g.nbatch, 8);
  const size_t sm = 20 * 20 * 8 * 8 + 64 * sizeof(R3) + 8 * sizeof(Rec<5>) + 8;
  CUtensorMap tmap;
  const int use_tma = region_map2(g, grid, tmap);
  TLGB_TRY(set_smem(fwd_f2_kernel, sm));
  dim3 grd((unsigned)info->n_fwd_items, (unsigned)ncg);
  fwd_f2_kernel<<<grd, 256, sm, s>>>(tmap, use_tma, g, (const int4*)(P + info->off_fwd_items),
                                     (const int32_t*)(P + info->off_entries), (const PRec*)(P + info->off_records), locs,
                                     (const float*)grid, (float*)out);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

int launch_adj_f3(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                  const void* vals, void* grid, void* scratch, cudaStream_t s) {
  const int64_t ncg = cdiv(g.nbatch, 8);
  const size_t sm = adj_f3_smem();
  TLGB_TRY(set_smem(adj_f3_kernel, sm));
  // 16-byte asynchronous copies of the point records and transposed values
  if (((uintptr_t)(P + info->off_records) & 15) || ((uintptr_t)scratch & 15))
    TLGB_FAIL(TLGB_ERR_INVALID, "interp adjoint: plan and scratch must be 16-byte aligned");
  const float4* tv = nullptr;
  if (g.tv_off >= 0 && g.npts > 0) {
    float2* t = reinterpret_cast<float2*>(static_cast<char*>(scratch) + g.tv_off);
    dim3 gt((unsigned)cdiv(g.npts, kTrPts), (unsigned)ncg);
    transpose_vals_kernel<<<gt, 256, 0, s>>>((const float2*)vals, g.npts, g.nbatch, t, nullptr);
    TLGB_CHECK_LAUNCH();
    tv = reinterpret_cast<const float4*>(t);
  }
  dim3 grd((unsigned)info->n_adj_items, (unsigned)ncg);
  adj_f3_kernel<<<grd, 256, sm, s>>>(g, (const int4*)(P + info->off_adj_items), (const int32_t*)(P + info->off_entries),
                                    (const PRec*)(P + info->off_records), locs, (const float*)vals, tv, (float*)grid,
                                    (float*)scratch);
  TLGB_CHECK_LAUNCH();
  if (info->n_split_tiles > 0) {
    dim3 g2((unsigned)info->n_split_tiles, (unsigned)ncg, 8);
    adj_reduce_f3_kernel<<<g2, 256, 0, s>>>(g, (const int4*)(P + info->off_split), (const float*)scratch,
                                             (float*)grid);
    TLGB_CHECK_LAUNCH();
  }
  return TLGB_OK;
}

template <int E>
int launch_adj_bn(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const void* vals, void* grid,
                  void* scratch, cudaStream_t s) {
  const size_t sm = 8 * kBC * kBSn * sizeof(float);
  TLGB_TRY(set_smem(adj_bn_kernel<E>, sm));
  if (((uintptr_t)P & 15) || ((uintptr_t)scratch & 15))
    TLGB_FAIL(TLGB_ERR_INVALID, "interp adjoint: plan and scratch must be 16-byte aligned");
  if ((uintptr_t)vals & 7) TLGB_FAIL(TLGB_ERR_INVALID, "interp adjoint: values must be 8-byte aligned");
  // the work counter follows the partial blocks
  int* ctr = reinterpret_cast<int*>(static_cast<char*>(scratch) + blk_partial_bytes(info, 1, E));
  TLGB_CUDA(cudaMemsetAsync(ctr, 0, sizeof(int), s));
  const int64_t nctas = std::min<int64_t>(cdiv(info->n_blk_items, 8), (int64_t)kBnCtas * sm_count());
  adj_bn_kernel<E><<<(unsigned)std::max<int64_t>(nctas, 1), 256, sm, s>>>(
      g, (const int4*)(P + info->off_blk_items), (int)info->n_blk_items, (const uint32_t*)(P + info->off_blk_entries),
      (const float*)(P + info->off_blk_rows), (const float2*)vals, (float*)grid, (float*)scratch, ctr);
  TLGB_CHECK_LAUNCH();
  if (info->n_blk_split > 0) {
    adj_reduce_bn_kernel<E><<<(unsigned)info->n_blk_split, 256, 0, s>>>(g, (const int4*)(P + info->off_blk_split),
                                                                       (const float*)scratch, (float*)grid);
    TLGB_CHECK_LAUNCH();
  }
  return TLGB_OK;
}

template <int NDIM>
int launch_adj_b3(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                  const void* vals, void* grid, void* scratch, cudaStream_t s) {
  if constexpr (NDIM == 3) {
    switch (blk_entries(g)) {
      case 1: return launch_adj_bn<1>(g, info, P, vals, grid, scratch, s);
      case 2: return launch_adj_bn<2>(g, info, P, vals, grid, scratch, s);
      case 4: return launch_adj_bn<4>(g, info, P, vals, grid, scratch, s);
      default: break;
    }
  }
  const int64_t ncg = cdiv(g.nbatch, 8);
  const size_t sm = 8 * kBC * kBS * sizeof(float);
  TLGB_TRY(set_smem(adj_b3_kernel<NDIM>, sm));
  // 16-byte asynchronous copies of the weight rows and transposed values
  if (((uintptr_t)P & 15) || ((uintptr_t)scratch & 15))
    TLGB_FAIL(TLGB_ERR_INVALID, "interp adjoint: plan and scratch must be 16-byte aligned");
  if ((uintptr_t)vals & 7) TLGB_FAIL(TLGB_ERR_INVALID, "interp adjoint: values must be 8-byte aligned");
  // the work counters (one per group of 8 entries) follow the partial blocks
  int* ctr = reinterpret_cast<int*>(static_cast<char*>(scratch) + blk_partial_bytes(info, ncg, 8));
  const float4* tv = nullptr;
  if (g.tv_off >= 0 && g.npts > 0) {
    float2* t = reinterpret_cast<float2*>(static_cast<char*>(scratch) + g.tv_off);
    dim3 gt((unsigned)cdiv(g.npts, kTrPts), (unsigned)ncg);
    transpose_vals_kernel<<<gt, 256, 0, s>>>((const float2*)vals, g.npts, g.nbatch, t, ctr);
    TLGB_CHECK_LAUNCH();
    tv = reinterpret_cast<const float4*>(t);
  } else {
    TLGB_CUDA(cudaMemsetAsync(ctr, 0, (size_t)ncg * sizeof(int), s));
  }
  // persistent: kB3Ctas CTAs per SM (fewer when there are few items), any
  // number of which may be resident at once
  const int64_t nctas = std::min<int64_t>(cdiv(info->n_blk_items, 8), (int64_t)kB3Ctas * sm_count());
  dim3 grd((unsigned)std::max<int64_t>(nctas, 1), (unsigned)ncg);
  adj_b3_kernel<NDIM><<<grd, 256, sm, s>>>(g, (const int4*)(P + info->off_blk_items), (int)info->n_blk_items,
                                          (const uint32_t*)(P + info->off_blk_entries),
                                          (const float*)(P + info->off_blk_rows), (const float2*)vals, tv,
                                          (float*)grid, (float*)scratch, ctr);
  TLGB_CHECK_LAUNCH();
  if (info->n_blk_split > 0) {
    dim3 g2((unsigned)info->n_blk_split, (unsigned)ncg);
    adj_reduce_b3_kernel<NDIM><<<g2, 256, 0, s>>>(g, (const int4*)(P + info->off_blk_split),
                                                 (const float*)scratch, (float*)grid);
    TLGB_CHECK_LAUNCH();
  }
  return TLGB_OK;
}

int launch_adj_f2(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                  const void* vals, void* grid, void* scratch, cudaStream_t s) {
  const int64_t ncg = cdiv(g.nbatch, 8);
  const size_t sm = adj_f2_smem();
  TLGB_TRY(set_smem(adj_f2_kernel, sm));
  if (((uintptr_t)(P + info->off_records) & 15) || ((uintptr_t)scratch & 15))
    TLGB_FAIL(TLGB_ERR_INVALID, "interp adjoint: plan and scratch must be 16-byte aligned");
  const float4* tv = nullptr;
  if (g.tv_off >= 0 && g.npts > 0) {
    float2* t = reinterpret_cast<float2*>(static_cast<char*>(scratch) + g.tv_off);
    dim3 gt((unsigned)cdiv(g.npts, kTrPts), (unsigned)ncg);
    transpose_vals_kernel<<<gt, 256, 0, s>>>((const float2*)vals, g.npts, g.nbatch, t, nullptr);
    TLGB_CHECK_LAUNCH();
    tv = reinterpret_cast<const float4*>(t);
  }
  dim3 grd((unsigned)info->n_adj_items, (unsigned)ncg);
  adj_f2_kernel<<<grd, 256, sm, s>>>(g, (const int4*)(P + info->off_adj_items), (const int32_t*)(P + info->off_entries),
                                    (const PRec*)(P + info->off_records), locs, (const float*)vals, tv, (float*)grid,
                                    (float*)scratch);
  TLGB_CHECK_LAUNCH();
  if (info->n_split_tiles > 0) {
    // parts in the generic [y][z][entry] layout of a 16 x 16 x 8-entry tile
    dim3 g2((unsigned)info->n_split_tiles, (unsigned)ncg);
    adj_reduce_kernel<<<g2, NTHR, 0, s>>>(g, (const int4*)(P + info->off_split), (const float*)scratch, (float*)grid,
                                          8, (int)ncg);
    TLGB_CHECK_LAUNCH();
  }
  return TLGB_OK;
}

template <int N, int NDIM, int NTB>
int launch_fwd_t(const Geo& g, int cg, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                 const void* grid, void* out, cudaStream_t s) {
  if constexpr (N == 4 && NDIM == 3 && NTB == 5)
    if (fast3(g, cg) && info->off_records > 0) return launch_fwd_f3(g, info, P, locs, grid, out, s);
  if constexpr (NDIM == 2 && NTB == 5)
    if (fast2(g, cg) && info->off_records > 0) return launch_fwd_f2(g, info, P, locs, grid, out, s);
  return launch_fwd_t2<N, NDIM, NTB, false>(g, cg, info, P, locs, grid, out, s);
}

template <int N, int NDIM, int NTB>
int launch_adj_t(const Geo& g, int cg, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                 const void* vals, void* grid, void* scratch, cudaStream_t s) {
  if constexpr (N == 4 && NDIM == 3 && NTB == 5)
    if (fast3(g, cg) && info->off_records > 0 && info->n_blk_items > 0)
      return launch_adj_b3<3>(g, info, P, locs, vals, grid, scratch, s);
    if (fast3(g, cg) && info->off_records > 0) return launch_adj_f3(g, info, P, locs, vals, grid, scratch, s);
  if constexpr (NDIM == 2 && NTB == 5)
    if (fast2(g, cg) && info->off_records > 0 && info->n_blk_items > 0)
      return launch_adj_b3<2>(g, info, P, locs, vals, grid, scratch, s);
    if (fast2(g, cg) && info->off_records > 0) return launch_adj_f2(g, info, P, locs, vals, grid, scratch, s);
  return launch_adj_t2<N, NDIM, NTB, false>(g, cg, info, P, locs, vals, grid, scratch, s);
}

// floats per coil unit: 2 batch entries per unit when the group size is even
inline int unit_floats(const Geo& g, int cg) { return (g.cplx ? 2 : 1) * ((cg % 2 == 0) ? 2 : 1); }

template <int NDIM, int NTB>
int dispatch_fwd_n(const Geo& g, int cg, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                   const void* grid, void* out, cudaStream_t s) {
  switch (unit_floats(g, cg)) {
    case 4: return launch_fwd_t<4, NDIM, NTB>(g, cg, info, P, locs, grid, out, s);
    case 2: return launch_fwd_t<2, NDIM, NTB>(g, cg, info, P, locs, grid, out, s);
    default: return launch_fwd_t<1, NDIM, NTB>(g, cg, info, P, locs, grid, out, s);
  }
}

template <int NDIM, int NTB>
int dispatch_adj_n(const Geo& g, int cg, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                   const void* vals, void* grid, void* scratch, cudaStream_t s) {
  switch (unit_floats(g, cg)) {
    case 4: return launch_adj_t<4, NDIM, NTB>(g, cg, info, P, locs, vals, grid, scratch, s);
    case 2: return launch_adj_t<2, NDIM, NTB>(g, cg, info, P, locs, vals, grid, scratch, s);
    default: return launch_adj_t<1, NDIM, NTB>(g, cg, info, P, locs, vals, grid, scratch, s);
  }
}

int launch_fwd_rows(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                    const void* grid, void* out, cudaStream_t s) {
  const int cg = fwd_cg(g);
  const bool small = ntb_for(g) == 5;
  if (g.ndim == 3) return small ? dispatch_fwd_n<3, 5>(g, cg, info, P, locs, grid, out, s) : dispatch_fwd_n<3, 9>(g, cg, info, P, locs, grid, out, s);
  if (g.ndim == 2) return small ? dispatch_fwd_n<2, 5>(g, cg, info, P, locs, grid, out, s) : dispatch_fwd_n<2, 16>(g, cg, info, P, locs, grid, out, s);
  return small ? dispatch_fwd_n<1, 5>(g, cg, info, P, locs, grid, out, s) : dispatch_fwd_n<1, 16>(g, cg, info, P, locs, grid, out, s);
}

// Launch grids have at most 65535 rows of batch groups. Wide 3D kernels
// stage fewer than 8 entries per group (their region would not fit shared
// memory), so a batch below TLGB_INTERP_MAX_BATCH can still need more rows:
// batch entries are independent, so such a batch is launched in parts.
int launch_fwd(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs, const void* grid,
               void* out, cudaStream_t s) {
  const int64_t per = (int64_t)65535 * fwd_cg(g);
  if (g.nbatch <= per) return launch_fwd_rows(g, info, P, locs, grid, out, s);
  const int64_t vs = value_size(g), vol = (int64_t)g.N[0] * g.N[1] * g.N[2];
  for (int64_t b0 = 0; b0 < g.nbatch; b0 += per) {
    Geo gc = g;
    gc.nbatch = std::min(per, (int64_t)g.nbatch - b0);
    TLGB_TRY(launch_fwd_rows(gc, info, P, locs, static_cast<const char*>(grid) + b0 * vol * vs,
                             static_cast<char*>(out) + b0 * g.npts * vs, s));
  }
  return TLGB_OK;
}

int launch_adj(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs, const void* vals,
               void* grid, void* scratch, cudaStream_t s) {
  // adj_cg is min(nbatch, 8): TLGB_INTERP_MAX_BATCH keeps the grid at <= 65535 rows
  if (cdiv(g.nbatch, adj_cg(g)) > 65535) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "interp adjoint: too many batch groups");
  const int cg = adj_cg(g);
  const bool small = ntb_for(g) == 5;
  if (g.ndim == 3) return small ? dispatch_adj_n<3, 5>(g, cg, info, P, locs, vals, grid, scratch, s) : dispatch_adj_n<3, 9>(g, cg, info, P, locs, vals, grid, scratch, s);
  if (g.ndim == 2) return small ? dispatch_adj_n<2, 5>(g, cg, info, P, locs, vals, grid, scratch, s) : dispatch_adj_n<2, 16>(g, cg, info, P, locs, vals, grid, scratch, s);
  return small ? dispatch_adj_n<1, 5>(g, cg, info, P, locs, vals, grid, scratch, s) : dispatch_adj_n<1, 16>(g, cg, info, P, locs, vals, grid, scratch, s);
}

int launch_grad_f2(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs,
                   const void* grid, const void* a, float* grad, void* scratch, cudaStream_t s) {
  const long long ncg = cdiv(g.nbatch, 8);
  GRec2* recs = static_cast<GRec2*>(scratch);
  float* partial = reinterpret_cast<float*>(static_cast<char*>(scratch) + grad2_records_bytes(g));
  grad_records2_kernel<<<(unsigned)cdiv(g.npts, 256), 256, 0, s>>>(g, locs, recs);
  TLGB_CHECK_LAUNCH();
  const long long n = (long long)g.npts * 2;
  if (ncg > 1 && info->n_home < g.npts)  // points without taps get no partial writes
    TLGB_CUDA(cudaMemsetAsync(partial, 0, (size_t)ncg * n * sizeof(float), s));
  CUtensorMap tmap;
  const int use_tma = region_map2(g, grid, tmap);
  const size_t sm = 20 * 20 * 8 * 8 + 64 * sizeof(GRec2) + 8 * sizeof(PTaps<true>) + 8;
  TLGB_TRY(set_smem(grad_f2_kernel, sm));
  dim3 grd((unsigned)info->n_fwd_items, (unsigned)ncg);
  grad_f2_kernel<<<grd, 256, sm, s>>>(tmap, use_tma, g, (const int4*)(P + info->off_fwd_items),
                                      (const int32_t*)(P + info->off_entries), recs, locs, (const float*)grid,
                                      (const float2*)a, grad, partial);
  TLGB_CHECK_LAUNCH();
  if (ncg > 1) {
    grad_reduce_kernel<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(partial, (int)ncg, n, grad);
    TLGB_CHECK_LAUNCH();
  }
  return TLGB_OK;
}

template <typename V, int NORM>
int launch_grad(const Geo& g, const tlgb_interp_plan_info* info, const char* P, const float* locs, const void* grid,
                const void* a, float* grad, void* scratch, size_t scratch_bytes, cudaStream_t s) {
  if constexpr (std::is_same<V, float2>::value && NORM == 1)
    if (grad_fast2(g) && info->off_records > 0 && scratch && scratch_bytes >= grad2_scratch_bytes(g) &&
        ((uintptr_t)scratch & 15) == 0)
      return launch_grad_f2(g, info, P, locs, grid, a, grad, scratch, s);
  const int cg = grad_cg(g, sizeof(PTaps<true>));
  const size_t sm = grad_smem(g, cg, sizeof(PTaps<true>)) + kFwdChunk * 3 * sizeof(float);
  auto* k = interp_grad_kernel<V, NORM>;
  TLGB_TRY(set_smem(k, sm));
  int nsplit = grad_splits(g, info);
  const size_t need = grad_scratch_bytes(g, nsplit);
  if (!scratch || scratch_bytes < need) nsplit = 1;  // one pass over all coil groups per tile
  float* partial = static_cast<float*>(scratch);
  const long long n = (long long)g.npts * g.ndim;
  if (nsplit > 1 && info->n_home < g.npts)  // points without taps get no partial writes
    TLGB_CUDA(cudaMemsetAsync(partial, 0, need, s));
  dim3 grd((unsigned)info->n_fwd_items, (unsigned)nsplit);
  k<<<grd, NTHR, sm, s>>>(g, (const int4*)(P + info->off_fwd_items), (const int32_t*)(P + info->off_entries), locs,
                          (const V*)grid, (const V*)a, grad, cg, (int)kFwdChunk, partial);
  TLGB_CHECK_LAUNCH();
  if (nsplit > 1) {
    grad_reduce_kernel<<<(unsigned)cdiv(n, 256), 256, 0, s>>>(partial, nsplit, n, grad);
    TLGB_CHECK_LAUNCH();
  }
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

extern "C" int tlgb_interp_forward(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, const void* plan,
                                   const float* locs, const void* grid, void* out, tlgb_stream_t stream) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  TLGB_TRY(check_plan(g, info, plan));
  if (g.npts == 0 || g.nbatch == 0) return TLGB_OK;
  if (!locs || !grid || !out) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (info->n_home < g.npts)  // points without a valid tap read as zero
    TLGB_CUDA(cudaMemsetAsync(out, 0, (size_t)g.nbatch * g.npts * value_size(g), s));
  if (info->n_fwd_items == 0) return TLGB_OK;
  const char* P = (const char*)plan;
  return launch_fwd(g, info, P, locs, grid, out, s);
}

extern "C" int tlgb_interp_adjoint(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, const void* plan,
                                   const float* locs, const void* vals, void* grid, void* scratch,
                                   size_t scratch_bytes, tlgb_stream_t stream) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  TLGB_TRY(check_plan(g, info, plan));
  if (g.nbatch == 0) return TLGB_OK;
  if (!grid || (g.npts > 0 && (!locs || !vals))) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  size_t pb = 0, tb = 0;
  adj_scratch_parts(g, info, pb, tb);
  if (scratch_bytes < pb + tb || (pb + tb > 0 && !scratch)) TLGB_FAIL(TLGB_ERR_WORKSPACE, "adjoint scratch too small");
  g.tv_off = tb > 0 ? (long long)pb : -1;
  cudaStream_t s = (cudaStream_t)stream;
  const char* P = (const char*)plan;
  return launch_adj(g, info, P, locs, vals, grid, scratch, s);
}

extern "C" int tlgb_interp_grad_scratch_size(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info,
                                             size_t* bytes) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  if (!info || !bytes) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  *bytes = grad_fast2(g) && info->off_records > 0 ? grad2_scratch_bytes(g) : grad_scratch_bytes(g, grad_splits(g, info));
  return TLGB_OK;
}

extern "C" int tlgb_interp_grad_locs(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, const void* plan,
                                     const float* locs, const void* grid, const void* a, float* grad_locs,
                                     void* scratch, size_t scratch_bytes, tlgb_stream_t stream) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  TLGB_TRY(check_plan(g, info, plan));
  if (g.npts == 0) return TLGB_OK;
  if (!locs || !grid || !a || !grad_locs) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (info->n_home < g.npts || g.nbatch == 0)
    TLGB_CUDA(cudaMemsetAsync(grad_locs, 0, (size_t)g.npts * g.ndim * sizeof(float), s));
  if (g.nbatch == 0 || info->n_fwd_items == 0) return TLGB_OK;
  const char* P = (const char*)plan;
  if (g.cplx)
    return g.norm == 1 ? launch_grad<float2, 1>(g, info, P, locs, grid, a, grad_locs, scratch, scratch_bytes, s)
                       : launch_grad<float2, 2>(g, info, P, locs, grid, a, grad_locs, scratch, scratch_bytes, s);
  return g.norm == 1 ? launch_grad<float, 1>(g, info, P, locs, grid, a, grad_locs, scratch, scratch_bytes, s)
                     : launch_grad<float, 2>(g, info, P, locs, grid, a, grad_locs, scratch, scratch_bytes, s);
}

// ------------------------------------------------ gridding without allocation
//
// Some callers cannot allocate device memory at the moment they grid: a
// host framework that hands out memory only from a pool reserved at start-up
// (a scanner's real-time reconstruction loop, a service with a fixed memory
// budget), or an FFI caller (cgo, JNI) that has no allocator of its own and
// for which cudaMalloc would synchronise the device in the middle of a
// pipeline. For them tlgb_interp_adjoint_fixed takes the partial-tile scratch
// of dense tiles from this file-scope device buffer instead of from the
// caller. The buffer is part of the loaded module: every GPU that loads the
// library holds it until the process exits.

namespace tlgb {
namespace {
constexpr size_t kFixedScratchBytes = TLGB_ADJOINT_FIXED_SCRATCH_BYTES;
}  // namespace
}  // namespace tlgb

static __device__ __align__(256) unsigned char g_adjoint_fixed_scratch[tlgb::kFixedScratchBytes];

namespace tlgb {
namespace {

// The buffer's device address differs per CUDA context: the primary context
// of each device, and any context a caller made itself with the driver API
// (FFI hosts often do). The address is looked up once per context, with that
// context current, and remembered; the first lookup in a context may load the
// module there, which is when the buffer is allocated on that GPU.
std::mutex g_fixed_mu;
std::vector<std::pair<CUcontext, void*>> g_fixed_addr;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  return fn;
}

// Device address of the fixed buffer in the current context.
int fixed_scratch_address(void** out) {
  CtxGetCurrentFn get = ctx_get_current();
  if (!get) TLGB_FAIL(TLGB_ERR_CUDA, "cuCtxGetCurrent is not available from the driver");
  CUcontext ctx = nullptr;
  if (get(&ctx) != CUDA_SUCCESS) TLGB_FAIL(TLGB_ERR_CUDA, "cuCtxGetCurrent failed");
  std::lock_guard<std::mutex> lock(g_fixed_mu);
  if (ctx != nullptr)
    for (const auto& e : g_fixed_addr)
      if (e.first == ctx) {
        *out = e.second;
        return TLGB_OK;
      }
  // with no context current, this first runtime call makes the current
  // device's primary context current on this thread
  void* p = nullptr;
  TLGB_CUDA(cudaGetSymbolAddress(&p, g_adjoint_fixed_scratch));
  if (ctx == nullptr && (get(&ctx) != CUDA_SUCCESS || ctx == nullptr))
    TLGB_FAIL(TLGB_ERR_CUDA, "no current CUDA context");
  for (const auto& e : g_fixed_addr)
    if (e.first == ctx) {
      *out = e.second;
      return TLGB_OK;
    }
  g_fixed_addr.emplace_back(ctx, p);
  *out = p;
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

extern "C" int tlgb_interp_adjoint_fixed(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info,
                                         const void* plan, const float* locs, const void* vals, void* grid,
                                         tlgb_stream_t stream) {
  Geo g;
  TLGB_TRY(make_geo(d, g));
  TLGB_TRY(check_plan(g, info, plan));
  if (g.nbatch == 0) return TLGB_OK;
  if (!grid || (g.npts > 0 && (!locs || !vals))) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  size_t need = 0, tb = 0;
  adj_scratch_parts(g, info, need, tb);
  if (need > kFixedScratchBytes)
    TLGB_FAIL(TLGB_ERR_WORKSPACE, "this plan needs " + std::to_string(need) +
                                      " bytes of partial-tile scratch, more than the fixed " +
                                      std::to_string(kFixedScratchBytes) +
                                      "-byte device buffer of tlgb_interp_adjoint_fixed; use "
                                      "tlgb_interp_adjoint with caller scratch");
  // the point-major copy of the values is used only when it fits as well
  g.tv_off = (tb > 0 && need + tb <= kFixedScratchBytes) ? (long long)need : -1;
  void* scratch = nullptr;
  if (need + (g.tv_off >= 0 ? tb : 0) > 0) TLGB_TRY(fixed_scratch_address(&scratch));
  return launch_adj(g, info, (const char*)plan, locs, vals, grid, scratch, (cudaStream_t)stream);
}

extern "C" int tlgb_test_skip_region_copy(int32_t on) {
  return tlgb::g_test_skip_copy.exchange(on ? 1 : 0);
}

extern "C" int tlgb_device_status(int32_t* status, int32_t clear) {
  if (status == nullptr) TLGB_FAIL(TLGB_ERR_INVALID, "status is NULL");
  int v = 0;
  TLGB_CUDA(cudaDeviceSynchronize());
  TLGB_CUDA(cudaMemcpyFromSymbol(&v, tlgb::g_tlgb_status, sizeof(int)));
  if (clear) {
    const int z = 0;
    TLGB_CUDA(cudaMemcpyToSymbol(tlgb::g_tlgb_status, &z, sizeof(int)));
  }
  int vc = 0;
  TLGB_TRY(tlgb::conv_device_status(&vc, clear));
  // debug builds: an index outside its range in a checked access (bit 4)
  int li = 0, lb = 0;
  TLGB_TRY(tlgb::checked_status(&li, clear));
  TLGB_TRY(tlgb::blocks_checked_status(&lb, clear));
  *status = v | vc | ((li | lb) ? 4 : 0);
  return TLGB_OK;
}
