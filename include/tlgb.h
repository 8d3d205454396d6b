/*
 * tlgb -- GB300 (sm_103a) kernels for the torchlinops interpolation and block
 * hot path, behind a plain C ABI (pointers, sizes, a CUDA stream; no torch
 * types). Every entry point returns TLGB_OK (0) or an error code and never
 * throws; tlgb_last_error() gives the message of the last failing call made
 * on the calling host thread. All device pointers are raw CUDA device memory;
 * every launch goes on the given stream and no call synchronises the device,
 * except tlgb_interp_plan_build (it reads the bin histogram back once) and
 * tlgb_index_plan_build (it reads its bounds check back once).
 *
 * Reference interfaces each entry replaces (paths in the torchlinops source):
 *   tlgb_interp_forward    -> ungrid / _ungrid, functional/_interp/ungrid.py:37,70
 *   tlgb_interp_adjoint    -> grid / _grid,     functional/_interp/grid.py:37,75
 *   tlgb_interp_grad_locs  -> (new) trajectory gradient; the reference's
 *                             InterpolateFn.backward returns None for locs,
 *                             functional/_interp/interp.py:46-70
 *   tlgb_interp_plan_*     -> (new) point binning; the reference launches one
 *                             Triton program per ~npts/65535 points instead,
 *                             functional/_interp/ungrid.py:135-160
 *   tlgb_unfold            -> unfold / _unfold, functional/_unfold/unfold.py:31,72
 *   tlgb_fold              -> fold / _fold,     functional/_unfold/fold.py:32,66
 *   tlgb_index_forward     -> index,            functional/_index/index.py:17
 *   tlgb_index_adjoint     -> index_adjoint,    functional/_index/index.py:75
 *   tlgb_circular_pad      -> circular_pad,     functional/_interp/_circ_pad.py:10
 *   tlgb_circular_pad_adjoint -> circular_pad_adjoint, _circ_pad.py:119
 */
#ifndef TLGB_H_
#define TLGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cudaStream_t; NULL is the legacy default stream. */
typedef void* tlgb_stream_t;

enum {
  TLGB_OK = 0,
  TLGB_ERR_INVALID = 1,     /* bad shape, size, pointer, alignment or argument */
  TLGB_ERR_UNSUPPORTED = 2, /* valid input outside what the kernels implement   */
  TLGB_ERR_CUDA = 3,        /* a CUDA runtime call or launch failed             */
  TLGB_ERR_WORKSPACE = 4,   /* caller-provided workspace too small              */
  TLGB_ERR_DEVICE = 5       /* a kernel reported an error through its status word */
};

const char* tlgb_last_error(void);
int tlgb_version(void);

/* Reads (and, if `clear`, resets) the device status word of the current
 * device. Kernels whose internal waits are bounded set a bit instead of
 * hanging when a wait gives up, and their outputs are then incomplete:
 * 1 = the TMA-staged gather, 2 = the tensor-core convolution; in the
 * range-checked debug build (libtlgb_checked.so), 4 = an index outside its
 * range in a checked access. Synchronises
 * the device. *status = 0 means no kernel has reported an error since the
 * last clear. */
int tlgb_device_status(int32_t* status, int32_t clear);

/* Test hook for the failure path of the bounded waits, off by default.
 * While `on` is nonzero, calls made afterwards launch the TMA-staged gathers
 * and the 2D trajectory gradient without their region copy, and those
 * kernels poll the copy's mbarrier once: the wait runs out with nothing in
 * flight, the kernel sets status bit 1 and its CTAs return, leaving the
 * output incomplete. Returns the previous setting. For tests of
 * tlgb_device_status only; no counterpart in the reference. */
int tlgb_test_skip_region_copy(int32_t on);

/* ------------------------------------------------------------------------ */
/* Interpolation: Kaiser-Bessel / spline ungridding and gridding, 1D-3D.      */
/* ------------------------------------------------------------------------ */

enum { TLGB_KERNEL_KAISER_BESSEL = 0, TLGB_KERNEL_SPLINE = 1 };
enum { TLGB_PAD_CIRCULAR = 0, TLGB_PAD_ZERO = 1 };

/* Problem description shared by every interpolation call.
 * Layouts (C order): grid values [nbatch, grid_size[0..ndim-1]], point values
 * [nbatch, npts], locs [npts, ndim] float32 in grid units ('ij' order).
 * is_complex: values are complex64 stored as interleaved (re, im) float32.
 * nbatch is at most TLGB_INTERP_MAX_BATCH per call (larger batches return
 * TLGB_ERR_UNSUPPORTED before any launch; split them, as consecutive batch
 * entries are independent). */
#define TLGB_INTERP_MAX_BATCH 524280 /* 65535 launch rows of 8 entries */
typedef struct tlgb_interp_desc {
  int32_t ndim;         /* 1, 2 or 3 */
  int32_t kernel;       /* TLGB_KERNEL_* */
  int32_t norm;         /* 1: product of 1D weights; 2: radial weight */
  int32_t pad_mode;     /* TLGB_PAD_* */
  int32_t is_complex;
  int32_t reserved;
  int64_t grid_size[3];
  float width[3];       /* kernel width per dimension, grid units */
  float beta;           /* Kaiser-Bessel shape parameter */
  int64_t nbatch;
  int64_t npts;
} tlgb_interp_desc;

/* Host-side summary of a plan, filled by tlgb_interp_plan_build and passed
 * back unchanged to the calls that use the plan. */
typedef struct tlgb_interp_plan_info {
  int64_t n_entries;      /* (point, tile) pairs, home pairs first per tile */
  int64_t n_tiles;
  int32_t tile[3];        /* tile edge per internal dim */
  int32_t n_tile[3];      /* tiles per internal dim */
  int64_t n_fwd_items;    /* work items of tlgb_interp_forward / grad_locs */
  int64_t n_adj_items;    /* work items of tlgb_interp_adjoint */
  int64_t n_partials;     /* partial tiles of split (dense) output tiles */
  int64_t n_split_tiles;  /* output tiles summed from partials */
  int64_t chunk;          /* max entries per work item */
  int64_t off_entries;    /* byte offsets of the plan sections */
  int64_t off_fwd_items;
  int64_t off_adj_items;
  int64_t off_split;
  int64_t plan_bytes;
  int64_t n_home;         /* points with at least one valid tap (home pairs) */
  int64_t off_records;    /* byte offset of the per-point tap records, 0 = none */
  int64_t kernel_key;     /* kernel, norm and beta the records were built for */
  /* Block lists of the 2D/3D gridding of complex batches (0 when the plan has
   * none): the (point, block) pairs of 4x4x4-cell (3D) or 8x8-cell (2D) output
   * blocks, sorted stably by block, and their work items (dense blocks are
   * split into parts summed after). */
  int64_t n_blk_entries;
  int64_t n_blk_items;
  int64_t n_blk_partials; /* partial blocks of split (dense) blocks */
  int64_t n_blk_split;    /* blocks summed from partials */
  int64_t off_blk_entries;
  int64_t off_blk_items;
  int64_t off_blk_split;
  int64_t off_blk_rows;   /* per point, the tap weights over each block it meets */
} tlgb_interp_plan_info;

/* Bytes of device memory needed by a plan for this description (worst case)
 * and of temporary device memory needed only while it is built. Plan and
 * scratch buffers are 16-byte aligned (cudaMalloc gives 256). */
int tlgb_interp_plan_size(const tlgb_interp_desc* d, size_t* plan_bytes, size_t* tmp_bytes);

/* Bin the points: sort (point, tile) pairs by output tile (stable, so points
 * keep their original order inside a tile) and cut the work into items of at
 * most `chunk` pairs. Synchronises `stream` once to size the work lists. */
int tlgb_interp_plan_build(const tlgb_interp_desc* d, const float* locs, void* plan, size_t plan_bytes,
                           void* tmp, size_t tmp_bytes, tlgb_interp_plan_info* info, tlgb_stream_t stream);

/* Scratch bytes tlgb_interp_adjoint needs for this plan: the partial tiles
 * (or blocks) of split output tiles, on the block-list path a work counter per
 * group of 8 entries, and for the 8-entry 2D/3D gridding kernels a
 * point-major copy of the point values (64 bytes per point and group of 8
 * entries), so that each (point, block) pair reads its values in one
 * contiguous run. 3D block-list gridding of at most 4 entries reads the values
 * in place and needs no copy. The scratch needs no initial contents. */
int tlgb_interp_adjoint_scratch_size(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info,
                                     size_t* bytes);

/* out[b, p] = sum over taps of w(p, tap) * grid[b, tap]         (ungrid) */
int tlgb_interp_forward(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, const void* plan,
                        const float* locs, const void* grid, void* out, tlgb_stream_t stream);

/* grid[b, v] = sum over points p with v in their window of w(p, v) * vals[b, p]
 * (gridding). Every element of `grid` is written (no accumulation into the
 * caller's contents); the summation order is fixed, so results are
 * bit-identical run to run; no global atomics. Output tiles with more pairs
 * than one work item holds are summed in parts of at most `chunk` pairs, and
 * the parts are added in a fixed order with compensated (Kahan-Neumaier)
 * summation. */
int tlgb_interp_adjoint(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, const void* plan,
                        const float* locs, const void* vals, void* grid, void* scratch, size_t scratch_bytes,
                        tlgb_stream_t stream);

/* Gridding exactly as tlgb_interp_adjoint, for callers that cannot allocate
 * device memory when they grid: a host framework that only hands out memory
 * from a pool reserved at start-up (a real-time reconstruction loop, a
 * service with a fixed memory budget), or an FFI caller (cgo, JNI) with no
 * allocator of its own, for which cudaMalloc would also synchronise the
 * device mid-pipeline. It allocates nothing: the partial tiles of dense
 * output tiles go to one file-scope device buffer of
 * TLGB_ADJOINT_FIXED_SCRATCH_BYTES bytes that the library holds on every GPU
 * it is loaded on until the process exits. The caller still provides the
 * plan, the inputs and the output.
 *  - A plan whose partial tiles alone need more than the buffer is rejected
 *    with TLGB_ERR_WORKSPACE before anything is launched. The point-major
 *    copy of the values is made only when it fits beside them; otherwise
 *    the values are read in place (same result, bit for bit).
 *  - The first call in each CUDA context (the primary context of a device,
 *    or a context the caller created with the driver API) looks up the
 *    buffer's device address in that context and remembers it. Under CUDA's
 *    lazy module loading that first lookup may also load the module, which
 *    is when the 32 MiB buffer is allocated on the GPU: make the first call
 *    at start-up, before reserving the rest of the device memory, and before
 *    any stream capture.
 *  - Every call shares the one buffer and it keeps the last call's contents;
 *    nothing in it has to start at zero, because every partial tile is
 *    written in full before it is read. Calls whose work overlaps on the GPU
 *    (other streams, other host threads) race on the buffer: serialise them.
 * No counterpart in the reference: torchlinops allocates its outputs and has
 * no scratch. */
#define TLGB_ADJOINT_FIXED_SCRATCH_BYTES ((size_t)32 << 20)
int tlgb_interp_adjoint_fixed(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, const void* plan,
                              const float* locs, const void* vals, void* grid, tlgb_stream_t stream);

/* Scratch bytes tlgb_interp_grad_locs can use to split a batch of many
 * coil groups over several CTAs per tile (0 when it would not split). */
int tlgb_interp_grad_scratch_size(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, size_t* bytes);

/* grad_locs[p, e] = sum_b Re( conj(a[b, p]) * sum_taps dw(p, tap)/dx_e * grid[b, tap] )
 * -- the gradient w.r.t. the trajectory of sum Re(conj(a) * ungrid(grid)),
 * and (with grid := the output cotangent, a := the point values) of the
 * gridding operator. Written, not accumulated. With scratch of at least
 * tlgb_interp_grad_scratch_size bytes the coil groups are split over CTAs
 * and their partial sums added in a fixed order (deterministic); with less
 * (or NULL) one CTA per tile walks all coil groups. */
int tlgb_interp_grad_locs(const tlgb_interp_desc* d, const tlgb_interp_plan_info* info, const void* plan,
                          const float* locs, const void* grid, const void* a, float* grad_locs, void* scratch,
                          size_t scratch_bytes, tlgb_stream_t stream);

/* ------------------------------------------------------------------------ */
/* ArrayToBlocks / BlocksToArray (unfold / fold), 1D-3D.                      */
/* ------------------------------------------------------------------------ */

/* Element types of the block and sampling ops. Complex types are pairs of
 * the real type. The integer and raw types are for the sampling ops only
 * (raw: 1- or 2-byte elements that tlgb_index_forward copies unchanged). */
enum {
  TLGB_F32 = 0,
  TLGB_F64 = 1,
  TLGB_C64 = 2,
  TLGB_C128 = 3,
  TLGB_I32 = 4,
  TLGB_I64 = 5,
  TLGB_RAW8 = 6,
  TLGB_RAW16 = 7
};

/* array [nbatch, im_size...]  <->  blocks [nbatch, nblocks..., block...]
 * or, with a mask, blocks [nbatch, nblocks..., nnz] where mask_idx[j] (int32,
 * device) is the row-major offset inside one block of the j-th kept element
 * (ascending) and mask_inv[k] (int32, device, prod(block) entries) is the
 * index j of block offset k, or -1 where the mask is false. Both NULL means
 * no mask. nblocks[e] = (im_size[e]-block[e])/stride[e]+1. One call handles
 * below 2^31 rows of blocks (nbatch * nblocks[0] * nblocks[1]) and below 2^31
 * array planes (nbatch * im_size[0] of a 3D array); above that it returns
 * TLGB_ERR_UNSUPPORTED before any launch. */
typedef struct tlgb_blocks_desc {
  int32_t ndim;
  int32_t dtype;       /* TLGB_F32 ... TLGB_C128 */
  int64_t nbatch;
  int64_t im_size[3];
  int64_t block[3];
  int64_t stride[3];
  int64_t nnz;         /* kept elements per block (mask) or prod(block) */
  const int32_t* mask_idx;
  const int32_t* mask_inv;
} tlgb_blocks_desc;

/* blocks = unfold(array): a copy, bit-exact. */
int tlgb_unfold(const tlgb_blocks_desc* d, const void* array, void* blocks, tlgb_stream_t stream);

/* array = fold(blocks): each element is the sum of its (at most
 * prod(ceil(block/stride))) block entries in ascending block order, starting
 * from zero -- deterministic; every element of `array` is written. */
int tlgb_fold(const tlgb_blocks_desc* d, const void* blocks, void* array, tlgb_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Sampling at integer locations (Sampling linop; NUFFT mode "sampling").      */
/* Replaces index / index_adjoint, functional/_index/index.py:17,75, whose    */
/* adjoint is index_add_ (multi_grid, :141-184): float atomics on a GPU.       */
/* ------------------------------------------------------------------------ */

#define TLGB_INDEX_MAX_DIM 8

/* vals [nbatch, grid_size...] <-> samples [nbatch, npts]; the sample m sits
 * at cell (idx[0][m], ..., idx[ndim-1][m]) of the grid, each index taken
 * modulo its size (Python's non-negative modulo, so -size <= idx < size).
 * Below 2^31 cells and 2^31 - 1 samples. */
typedef struct tlgb_index_desc {
  int32_t ndim;  /* indexed (trailing) dims, 1..TLGB_INDEX_MAX_DIM */
  int32_t dtype; /* TLGB_F32 ... TLGB_RAW16 */
  int64_t nbatch;
  int64_t grid_size[TLGB_INDEX_MAX_DIM];
  int64_t npts;
} tlgb_index_desc;

typedef struct tlgb_index_plan_info {
  int64_t ncells, npts;
  int64_t off_flat;  /* byte offsets of the plan sections: the cell of each sample, */
  int64_t off_perm;  /* the samples sorted by cell (ascending within a cell),       */
  int64_t off_cells; /* and the first sorted position of every cell (ncells + 1)   */
  int64_t plan_bytes;
} tlgb_index_plan_info;

int tlgb_index_plan_size(const tlgb_index_desc* d, size_t* plan_bytes, size_t* tmp_bytes);

/* idx: [ndim][npts] int64 device indices. Ravels them, sorts the samples by
 * cell (stable) and sizes each cell's run. Synchronises `stream` once; an
 * index outside [-size, size) returns TLGB_ERR_INVALID with the first such
 * dimension in the message (the reference raises IndexError). */
int tlgb_index_plan_build(const tlgb_index_desc* d, const int64_t* idx, void* plan, size_t plan_bytes, void* tmp,
                          size_t tmp_bytes, tlgb_index_plan_info* info, tlgb_stream_t stream);

/* out[b, m] = vals[b, cell(m)]: a copy (any element type). */
int tlgb_index_forward(const tlgb_index_desc* d, const tlgb_index_plan_info* info, const void* plan,
                       const void* vals, void* out, tlgb_stream_t stream);

/* out[b, c] = sum of vals[b, m] over the samples m of cell c, in ascending m,
 * starting from zero: the order of a sequential index_add_, so bit-identical
 * to it and run to run (no atomics). Every cell is written. Float, complex
 * and integer element types. */
int tlgb_index_adjoint(const tlgb_index_desc* d, const tlgb_index_plan_info* info, const void* plan,
                       const void* vals, void* out, tlgb_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Circular padding of the trailing dims (Convolution linop, circular mode).  */
/* Replaces circular_pad / circular_pad_adjoint,                              */
/* functional/_interp/_circ_pad.py:10,119 (F.pad three dims at a time, and    */
/* autograd through it for the adjoint).                                      */
/* ------------------------------------------------------------------------ */

#define TLGB_CIRCPAD_MAX_DIM 8

/* in [nbatch, size...] -> out [nbatch, size[e] + pad_lo[e] + pad_hi[e] ...],
 * dims listed leading to trailing; 0 <= pad <= size per dim (the padding
 * wraps around at most once, as torch's circular F.pad requires). */
typedef struct tlgb_circpad_desc {
  int32_t ndim;  /* padded trailing dims, 1..TLGB_CIRCPAD_MAX_DIM */
  int32_t dtype; /* TLGB_F32 ... TLGB_RAW16 (the adjoint: not the raw types) */
  int64_t nbatch;
  int64_t size[TLGB_CIRCPAD_MAX_DIM];
  int64_t pad_lo[TLGB_CIRCPAD_MAX_DIM];
  int64_t pad_hi[TLGB_CIRCPAD_MAX_DIM];
} tlgb_circpad_desc;

/* out[b, j] = in[b, (j - pad_lo) mod size] per dim: a copy. */
int tlgb_circular_pad(const tlgb_circpad_desc* d, const void* in, void* out, tlgb_stream_t stream);

/* The adjoint: out (unpadded) [b, i] = sum of in (padded) [b, j] over the j
 * that tlgb_circular_pad copies from i, in ascending padded order
 * (deterministic). Every element of out is written. */
int tlgb_circular_pad_adjoint(const tlgb_circpad_desc* d, const void* in, void* out, tlgb_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Conjugate gradients with float64 scalars.                                   */
/* Replaces the complex64/float32 zdot and alpha/beta of the reference CG loop */
/* (alg/pcg.py:67-87; inner product utils/_adjoint_helpers.py:8).              */
/* ------------------------------------------------------------------------ */

/* Slots of the float64 CG state vector (device, TLGB_CG_STATE_LEN doubles). */
enum {
  TLGB_CG_RS = 0,      /* |r|^2 of the current residual            */
  TLGB_CG_RS_OLD = 1,  /* |r|^2 of the previous residual           */
  TLGB_CG_PAP = 2,     /* Re <p, A p>                               */
  TLGB_CG_ALPHA = 3,   /* last step length                          */
  TLGB_CG_BETA = 4,    /* last direction update                     */
  TLGB_CG_ITERS = 5,   /* iterations taken                          */
  TLGB_CG_TMP = 6,     /* two doubles of scratch (re, im of a dot)  */
  TLGB_CG_STATE_LEN = 8
};

/* Device scratch bytes the calls below need. */
size_t tlgb_cg_scratch_bytes(void);

/* out[0] + i out[1] = sum_k conj(x_k) y_k (complex64 vectors as float pairs)
 * or sum_k x_k y_k (float32), accumulated in float64 with a fixed reduction
 * order (bit-identical for a given n). out is device memory. */
int tlgb_dot_f64(const float* x, const float* y, int64_t n, int is_complex, double* out, void* scratch,
                 size_t scratch_bytes, tlgb_stream_t stream);

/* state[TLGB_CG_PAP] = Re <p, Ap> in float64. */
int tlgb_cg_set_pap(const float* p, const float* ap, int64_t n, int is_complex, double* state, void* scratch,
                    size_t scratch_bytes, tlgb_stream_t stream);

/* One CG update with alpha = state[RS] / state[PAP]:  x += alpha p,
 * r -= alpha Ap, state[RS] = |r|^2 (float64), beta = RS / RS_OLD,
 * p = r + beta p. No host synchronisation. */
int tlgb_cg_step(float* x, float* r, float* p, const float* ap, int64_t n, int is_complex, double* state,
                 void* scratch, size_t scratch_bytes, tlgb_stream_t stream);

/* Flexible preconditioned CG (state[TLGB_CG_RS] holds <r, z>):
 * x += a p, r -= a Ap with a = state[RS] / state[PAP] (float64, applied
 * rounded to float32). After z = M(r): state[RS] = Re <r, z>, the flexible
 * Polak-Ribiere beta = -a Re <Ap, z> / <r_old, z_old> clamped at 0, and
 * p = z + beta p, all on the device (no host synchronisation). The reference's
 * CG has no preconditioner; these extend its step and direction updates
 * (alg/pcg.py:73-87) to the flexible PCG of the learned preconditioner. */
int tlgb_pcg_update(float* x, float* r, const float* p, const float* ap, int64_t n, int is_complex,
                    const double* state, tlgb_stream_t stream);
int tlgb_pcg_direction(const float* r, const float* z, const float* ap, float* p, int64_t n, int is_complex,
                       double* state, void* scratch, size_t scratch_bytes, tlgb_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Centred-FFT shifts folded into the NUFFT's pad and crop (complex64).      */
/* The reference's cfftn = fftshift . fftn . ifftshift (utils/_fft.py:7-60)  */
/* costs two extra grid passes per transform; here the image-side shift is   */
/* part of one pad / crop gather, and the k-side shift is the modulation     */
/* fftshift(fftn(z)) = fftn(z . m), m[j] = prod_e exp(2 pi i j_e h_e / Np_e), */
/* h_e = floor(Np_e / 2) (the sign (-1)^j_e for even Np_e), applied in the   */
/* same gather, so the interpolation reads the reference's own coordinates.  */
/* ------------------------------------------------------------------------ */

/* Zero pad with the ifftshift folded in: for the padded-grid index j,
 * i = ((j + shift) mod np) - off per dim; out[b*C + c][j] =
 * mod[j] * maps[c][i] * apod[i] * x[b][i] where i lies in the image, else 0,
 * with mod[j] = m[j] above when `modulate` is nonzero, else 1.
 * Dims: the last `ndim` (1-3) of x [nbatch][n] and out [nbatch*C][np];
 * shift = floor(np / 2) gives the reference's ifftshift(pad(x)); off is the
 * left padding. apod (float, [n]) and maps (complex64, [C][n], C = nmaps)
 * may be NULL (then C = 1). */
int tlgb_pad_shift_c64(const void* x, int64_t nbatch, int32_t ndim, const int64_t* n, const int64_t* np,
                       const int64_t* off, const int64_t* shift, int32_t modulate, const float* apod,
                       const void* maps, int32_t nmaps, void* out, tlgb_stream_t stream);

/* Crop with the fftshift folded in, the adjoint of tlgb_pad_shift plus an
 * axpy: out[b][i] = alpha * apod[i] * sum_c conj(maps[c][i]) *
 * conj(mod[j]) * z[b*C + c][j(i)] + beta * add[b][i], with
 * j = (i + off - shift) mod np per dim. add may be NULL (then beta is
 * ignored). */
int tlgb_crop_shift_c64(const void* z, int64_t nbatch, int32_t ndim, const int64_t* n, const int64_t* np,
                        const int64_t* off, const int64_t* shift, int32_t modulate, const float* apod,
                        const void* maps, int32_t nmaps, float alpha, const void* add, float beta, void* out,
                        tlgb_stream_t stream);

/* ------------------------------------------------------------------------ */
/* 3^3 convolution on the tensor cores (BF16 operands, FP32 accumulation):    */
/* the layers of the learned CG preconditioner. No counterpart in the         */
/* reference (torchlinops has no learned preconditioner).                     */
/* ------------------------------------------------------------------------ */

/* Epilogue of tlgb_conv3d_fwd. */
enum {
  TLGB_CONV_PLAIN = 0, /* y = conv(x, w)                                     */
  TLGB_CONV_RELU = 1,  /* y = max(conv(x, w), 0)                             */
  TLGB_CONV_MASK = 2   /* y = conv(x, w) * (aux > 0): data gradient through a
                          ReLU whose output is aux                           */
};

typedef struct tlgb_conv3d_desc {
  int32_t D, H, W;   /* spatial size, the same in and out (zero padding 1)  */
  int32_t cin, cout; /* 16 and 16: pad narrower layers with zero channels    */
  int32_t mode;      /* TLGB_CONV_*                                          */
  int32_t out_f32;   /* 1: float32 output [D][H][W][16], else bfloat16       */
  int32_t reserved;
} tlgb_conv3d_desc;

/* y[v][co] = sum_{t, ci} w[t][co][ci] x[v + off(t)][ci], activations
 * channels-last [D][H][W][16] bfloat16, weights [27][16][16] bfloat16 with
 * tap t = (kd*3 + kh)*3 + kw reading input offset (kd-1, kh-1, kw-1).
 * The data gradient is this call with w'[26 - t][ci][co] = w[t][co][ci].
 * Buffers 16-byte aligned. */
int tlgb_conv3d_fwd(const tlgb_conv3d_desc* d, const void* x, const void* w, const void* aux, void* y,
                    tlgb_stream_t stream);

/* Device scratch for tlgb_conv3d_wgrad. */
int tlgb_conv3d_wgrad_scratch_size(const tlgb_conv3d_desc* d, size_t* bytes);

/* dw[t][co][ci] = sum_v gy[v][co] x[v + off(t)][ci] (float32), summed in a
 * fixed order (bit-identical run to run). */
int tlgb_conv3d_wgrad(const tlgb_conv3d_desc* d, const void* x, const void* gy, float* dw, void* scratch,
                      size_t scratch_bytes, tlgb_stream_t stream);

/* complex64 z[V] times *scale (device float; NULL = 1) -> bfloat16 [V][16]
 * with channels 0, 1 = real, imaginary rounded to bfloat16 and, if hilo,
 * channels 2, 3 = their rounding remainders (a two-term split with 16
 * significant bits); the other channels zero. */
int tlgb_conv3d_pack(const void* z, int64_t nvox, const float* scale, int32_t hilo, void* out,
                     tlgb_stream_t stream);

/* out[v] = *scale * (y[v][0] + i y[v][1]) + skip * z[v] (z may be NULL):
 * float32 [V][16] network output back to complex64. */
int tlgb_conv3d_unpack(const float* y, const void* z, int64_t nvox, const float* scale, float skip, void* out,
                       tlgb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* TLGB_H_ */
