// Sampling at integer locations (the Sampling linop, NUFFT mode "sampling"):
// a gather (index) and its adjoint, a scatter-add (index_adjoint).
//
// The reference (functional/_index/index.py:17-49,75-100) ravels the D index
// tensors with Python's non-negative modulo (ravel, :187-201), gathers with
// index_select, and scatters with index_add_ (multi_grid, :141-184): float
// atomics on a GPU, so its adjoint is not deterministic there. Here a plan,
// built once per index set, holds the raveled cell of every sample and the
// samples sorted by cell (a stable radix sort, so the samples of a cell stay
// in ascending order) with per-cell offsets. The adjoint is output-stationary:
// each cell sums its samples in ascending sample order starting from zero, the
// order of a sequential index_add_, so it is bit-identical to the reference's
// CPU path and to itself run to run. No atomics touch the values.

#include <algorithm>
#include <string>

#include "common.cuh"

namespace tlgb {
namespace {

struct IdxGeo {
  int ndim;
  int64_t size[TLGB_INDEX_MAX_DIM];
  int64_t stride[TLGB_INDEX_MAX_DIM];  // row-major cell strides
  int64_t ncells, npts, nbatch;
};

// Plan layout: flat[npts] int32 | perm[npts] int32 | off[ncells + 1] uint32
struct IdxLayout {
  int64_t off_flat, off_perm, off_cells, bytes;
  int64_t t_keys, t_keys2, t_vals2, t_counts, t_cnt, t_scan, t_bad, t_bytes;
};

// cell of sample m (Python modulo per dim, as the reference's ravel); the
// lowest out-of-range dim (index >= size or < -size, the reference's
// IndexError) is recorded in *bad
__global__ void index_ravel_kernel(IdxGeo g, const int64_t* __restrict__ idx, int32_t* __restrict__ flat,
                                   uint32_t* __restrict__ keys, int32_t* __restrict__ vals, uint32_t* __restrict__ cnt,
                                   int* __restrict__ bad) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < g.npts; m += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = 0;
    int worst = TLGB_INDEX_MAX_DIM;
    for (int d = 0; d < g.ndim; ++d) {
      const int64_t i = idx[(int64_t)d * g.npts + m];
      const int64_t s = g.size[d];
      if (i >= s || i < -s) worst = min(worst, d);
      int64_t r = i % s;
      if (r < 0) r += s;
      c += r * g.stride[d];
    }
    if (worst < TLGB_INDEX_MAX_DIM) {
      atomicMin(bad, worst);
      c = 0;  // keeps the plan in range; the build reports the error
    }
    flat[m] = (int32_t)c;
    keys[m] = (uint32_t)c;
    vals[m] = (int32_t)m;
    atomicAdd(cnt + c, 1u);  // integer counts: the same totals in any order
  }
}

// out[b][m] = vals[b][flat[m]]: a copy of E-sized elements
template <typename E>
__global__ void index_fwd_kernel(const E* __restrict__ vals, const int32_t* __restrict__ flat, E* __restrict__ out,
                                 int64_t npts, int64_t ncells, int64_t nbatch) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < npts; m += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = flat[m];
    for (int64_t b = 0; b < nbatch; ++b) out[b * npts + m] = vals[b * ncells + c];
  }
}

template <typename T>
struct Acc {
  T v;
  __device__ Acc() : v(T(0)) {}
  __device__ void add(const T& x) { v = v + x; }
};
template <>
struct Acc<float2> {
  float2 v;
  __device__ Acc() : v(make_float2(0.f, 0.f)) {}
  __device__ void add(const float2& x) {
    v.x = v.x + x.x;
    v.y = v.y + x.y;
  }
};
template <>
struct Acc<double2> {
  double2 v;
  __device__ Acc() : v(make_double2(0.0, 0.0)) {}
  __device__ void add(const double2& x) {
    v.x = v.x + x.x;
    v.y = v.y + x.y;
  }
};

// out[b][c] = sum over the samples of cell c, in ascending sample order,
// starting from zero; every cell is written
template <typename T>
__global__ void index_adj_kernel(const T* __restrict__ vals, const int32_t* __restrict__ perm,
                                 const uint32_t* __restrict__ off, T* __restrict__ out, int64_t npts, int64_t ncells,
                                 int64_t nbatch) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t k0 = off[c], k1 = off[c + 1];
    for (int64_t b = 0; b < nbatch; ++b) {
      Acc<T> a;
      const T* vb = vals + b * npts;
      for (uint32_t k = k0; k < k1; ++k) a.add(vb[perm[k]]);
      out[b * ncells + c] = a.v;
    }
  }
}

int make_idx_geo(const tlgb_index_desc* d, IdxGeo& g) {
  if (!d) TLGB_FAIL(TLGB_ERR_INVALID, "null index descriptor");
  if (d->ndim < 1 || d->ndim > TLGB_INDEX_MAX_DIM) TLGB_FAIL(TLGB_ERR_INVALID, "index: ndim must be in [1, 8]");
  if (d->npts < 0 || d->nbatch < 0) TLGB_FAIL(TLGB_ERR_INVALID, "index: negative size");
  g.ndim = d->ndim;
  int64_t n = 1;
  for (int e = d->ndim - 1; e >= 0; --e) {
    if (d->grid_size[e] < 1) TLGB_FAIL(TLGB_ERR_INVALID, "index: grid sizes must be positive");
    g.size[e] = d->grid_size[e];
    g.stride[e] = n;
    if (n > (int64_t)INT32_MAX / d->grid_size[e]) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "index: grid above 2^31 - 1 cells");
    n *= d->grid_size[e];
  }
  g.ncells = n;
  if (d->npts > (int64_t)INT32_MAX - 1) TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "index: 2^31 - 1 samples or more");
  g.npts = d->npts;
  g.nbatch = d->nbatch;
  return TLGB_OK;
}

IdxLayout idx_layout(const IdxGeo& g) {
  IdxLayout L;
  const int64_t m = std::max<int64_t>(g.npts, 1);
  size_t o = 0;
  L.off_flat = o;
  o = align_up(o + (size_t)m * 4, 256);
  L.off_perm = o;
  o = align_up(o + (size_t)m * 4, 256);
  L.off_cells = o;
  o = align_up(o + (size_t)(g.ncells + 1) * 4, 256);
  L.bytes = o;
  size_t t = 0;
  L.t_keys = t;
  t = align_up(t + (size_t)m * 4, 256);
  L.t_keys2 = t;
  t = align_up(t + (size_t)m * 4, 256);
  L.t_vals2 = t;
  t = align_up(t + (size_t)m * 4, 256);
  L.t_counts = t;
  t = align_up(t + (size_t)radix_counts_len(m) * 4, 256);
  L.t_cnt = t;
  t = align_up(t + (size_t)g.ncells * 4, 256);
  L.t_scan = t;
  t = align_up(t + (size_t)scan_scratch_len(g.ncells) * 4, 256);
  L.t_bad = t;
  t = align_up(t + 16, 256);
  L.t_bytes = t;
  return L;
}

int elem_bytes(int dtype) {
  switch (dtype) {
    case TLGB_F32: case TLGB_I32: return 4;
    case TLGB_F64: case TLGB_C64: case TLGB_I64: return 8;
    case TLGB_C128: return 16;
    case TLGB_RAW8: return 1;
    case TLGB_RAW16: return 2;
    default: return 0;
  }
}

int check_index_plan(const IdxGeo& g, const tlgb_index_plan_info* info, const void* plan) {
  if (!info || !plan) TLGB_FAIL(TLGB_ERR_INVALID, "index: null plan");
  if (info->ncells != g.ncells || info->npts != g.npts)
    TLGB_FAIL(TLGB_ERR_INVALID, "index: plan was built for another grid or sample count");
  return TLGB_OK;
}

unsigned grid_for(int64_t n) {
  const int64_t cap = (int64_t)sm_count() * 8;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cap, cdiv(n, 256)));
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_index_plan_size(const tlgb_index_desc* d, size_t* plan_bytes, size_t* tmp_bytes) {
  IdxGeo g;
  TLGB_TRY(make_idx_geo(d, g));
  if (!plan_bytes || !tmp_bytes) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  const IdxLayout L = idx_layout(g);
  *plan_bytes = (size_t)L.bytes;
  *tmp_bytes = (size_t)L.t_bytes;
  return TLGB_OK;
}

extern "C" int tlgb_index_plan_build(const tlgb_index_desc* d, const int64_t* idx, void* plan, size_t plan_bytes,
                                     void* tmp, size_t tmp_bytes, tlgb_index_plan_info* info, tlgb_stream_t stream) {
  IdxGeo g;
  TLGB_TRY(make_idx_geo(d, g));
  if (!plan || !tmp || !info || (g.npts > 0 && !idx)) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  const IdxLayout L = idx_layout(g);
  if (plan_bytes < (size_t)L.bytes || tmp_bytes < (size_t)L.t_bytes)
    TLGB_FAIL(TLGB_ERR_WORKSPACE, "index plan or temporary buffer too small");
  cudaStream_t s = (cudaStream_t)stream;
  char* P = static_cast<char*>(plan);
  char* T = static_cast<char*>(tmp);
  int32_t* flat = reinterpret_cast<int32_t*>(P + L.off_flat);
  int32_t* perm = reinterpret_cast<int32_t*>(P + L.off_perm);
  uint32_t* off = reinterpret_cast<uint32_t*>(P + L.off_cells);
  uint32_t* keys = reinterpret_cast<uint32_t*>(T + L.t_keys);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(T + L.t_cnt);
  int* bad = reinterpret_cast<int*>(T + L.t_bad);
  TLGB_CUDA(cudaMemsetAsync(cnt, 0, (size_t)g.ncells * 4, s));
  const int none = 0x7f7f7f7f;  // every byte 0x7f: above any dimension index
  TLGB_CUDA(cudaMemsetAsync(bad, 0x7f, sizeof(int), s));
  if (g.npts > 0) {
    index_ravel_kernel<<<grid_for(g.npts), 256, 0, s>>>(g, idx, flat, keys, perm, cnt, bad);
    TLGB_CHECK_LAUNCH();
    int bits = 1;
    while (bits < 32 && ((int64_t)1 << bits) < g.ncells) ++bits;
    TLGB_TRY(radix_sort_pairs(keys, perm, reinterpret_cast<uint32_t*>(T + L.t_keys2),
                              reinterpret_cast<int32_t*>(T + L.t_vals2), reinterpret_cast<uint32_t*>(T + L.t_counts),
                              g.npts, bits, s));
  }
  TLGB_TRY(exclusive_scan_u32(cnt, off, g.ncells, off + g.ncells, reinterpret_cast<uint32_t*>(T + L.t_scan), s));
  int worst = none;
  TLGB_CUDA(cudaMemcpyAsync(&worst, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  TLGB_CUDA(cudaStreamSynchronize(s));
  if (worst < none) {
    std::string shape;
    for (int e = 0; e < g.ndim; ++e) shape += (e ? ", " : "") + std::to_string(g.size[e]);
    if (g.ndim == 1) shape += ",";  // as Python prints a 1-tuple
    TLGB_FAIL(TLGB_ERR_INVALID, "Out-of-bounds index for grid of shape (" + shape + "): idx[" +
                                    std::to_string(worst) + "]");
  }
  memset(info, 0, sizeof(*info));
  info->ncells = g.ncells;
  info->npts = g.npts;
  info->off_flat = L.off_flat;
  info->off_perm = L.off_perm;
  info->off_cells = L.off_cells;
  info->plan_bytes = L.bytes;
  return TLGB_OK;
}

extern "C" int tlgb_index_forward(const tlgb_index_desc* d, const tlgb_index_plan_info* info, const void* plan,
                                  const void* vals, void* out, tlgb_stream_t stream) {
  IdxGeo g;
  TLGB_TRY(make_idx_geo(d, g));
  TLGB_TRY(check_index_plan(g, info, plan));
  if (g.npts == 0 || g.nbatch == 0) return TLGB_OK;
  if (!vals || !out) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const int32_t* flat = reinterpret_cast<const int32_t*>(static_cast<const char*>(plan) + info->off_flat);
  const unsigned grd = grid_for(g.npts);
  switch (elem_bytes(d->dtype)) {
    case 1: index_fwd_kernel<uint8_t><<<grd, 256, 0, s>>>((const uint8_t*)vals, flat, (uint8_t*)out, g.npts, g.ncells, g.nbatch); break;
    case 2: index_fwd_kernel<uint16_t><<<grd, 256, 0, s>>>((const uint16_t*)vals, flat, (uint16_t*)out, g.npts, g.ncells, g.nbatch); break;
    case 4: index_fwd_kernel<uint32_t><<<grd, 256, 0, s>>>((const uint32_t*)vals, flat, (uint32_t*)out, g.npts, g.ncells, g.nbatch); break;
    case 8: index_fwd_kernel<uint2><<<grd, 256, 0, s>>>((const uint2*)vals, flat, (uint2*)out, g.npts, g.ncells, g.nbatch); break;
    case 16: index_fwd_kernel<uint4><<<grd, 256, 0, s>>>((const uint4*)vals, flat, (uint4*)out, g.npts, g.ncells, g.nbatch); break;
    default: TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "index: unsupported element type");
  }
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_index_adjoint(const tlgb_index_desc* d, const tlgb_index_plan_info* info, const void* plan,
                                  const void* vals, void* out, tlgb_stream_t stream) {
  IdxGeo g;
  TLGB_TRY(make_idx_geo(d, g));
  TLGB_TRY(check_index_plan(g, info, plan));
  if (g.nbatch == 0) return TLGB_OK;
  if (!out || (g.npts > 0 && !vals)) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const char* P = static_cast<const char*>(plan);
  const int32_t* perm = reinterpret_cast<const int32_t*>(P + info->off_perm);
  const uint32_t* off = reinterpret_cast<const uint32_t*>(P + info->off_cells);
  const unsigned grd = grid_for(g.ncells);
  switch (d->dtype) {
    case TLGB_F32: index_adj_kernel<float><<<grd, 256, 0, s>>>((const float*)vals, perm, off, (float*)out, g.npts, g.ncells, g.nbatch); break;
    case TLGB_F64: index_adj_kernel<double><<<grd, 256, 0, s>>>((const double*)vals, perm, off, (double*)out, g.npts, g.ncells, g.nbatch); break;
    case TLGB_C64: index_adj_kernel<float2><<<grd, 256, 0, s>>>((const float2*)vals, perm, off, (float2*)out, g.npts, g.ncells, g.nbatch); break;
    case TLGB_C128: index_adj_kernel<double2><<<grd, 256, 0, s>>>((const double2*)vals, perm, off, (double2*)out, g.npts, g.ncells, g.nbatch); break;
    case TLGB_I32: index_adj_kernel<int32_t><<<grd, 256, 0, s>>>((const int32_t*)vals, perm, off, (int32_t*)out, g.npts, g.ncells, g.nbatch); break;
    case TLGB_I64: index_adj_kernel<long long><<<grd, 256, 0, s>>>((const long long*)vals, perm, off, (long long*)out, g.npts, g.ncells, g.nbatch); break;
    default: TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "index adjoint: unsupported element type");
  }
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}
