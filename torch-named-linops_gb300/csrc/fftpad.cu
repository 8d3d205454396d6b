// Centred-FFT shifts folded into the pad and crop of the NUFFT chain, with
// the apodization and (for SENSE) the coil sensitivities fused in.
//
// The reference's NUFFT is Apodize -> Pad -> cfftn -> Interpolate, with
// cfftn = fftshift . fftn . ifftshift (linops/nufft.py:170-184,
// utils/_fft.py:7-60). Each shift is a full-grid pass. Here:
//   ifftshift(Pad(a x))[j] = a[i] x[i], i = (j + floor(Np/2)) mod Np - off
// is one gather (tlgb_pad_shift), and the k-space fftshift is a modulation
// of the same gather's output:
//   fftshift(fftn(z)) = fftn(z . m),  m[j] = prod_e exp(2 pi i j_e h_e / Np_e),
//   h_e = floor(Np_e / 2),
// which for even Np_e is the sign (-1)^j_e (exact). So an uncentred fftn of
// the gather's output is the reference's centred k-space, read at the
// reference's own interpolation coordinates. On the way back,
//   Crop(fftshift(ifftn(ifftshift(G))))[i] = conj(m[j]) ifftn(G)[j],
//   j = (i + off - floor(Np/2)) mod Np,
// is one gather (tlgb_crop_shift), which can also apply the conjugate coil
// maps, the coil sum and an axpy.

#include "common.cuh"

namespace tlgb {
namespace {

struct PadGeo {
  int n[3], np[3], off[3], sh[3];  // internal dims padded to 3 (leading 1s)
  long long nvol, npvol;
  int modulate;  // multiply by m[j] (pad) / conj(m[j]) (crop)
};

// m[j] of the uncentred index j: a sign for even extents, a phase otherwise
__device__ __forceinline__ float2 modulation(const PadGeo& G, int j0, int j1, int j2) {
  const int j[3] = {j0, j1, j2};
  int sign = 0;
  float ph = 0.f;  // in units of pi
  bool odd = false;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    if ((G.np[e] & 1) == 0) {
      sign ^= j[e] & 1;
    } else {
      odd = true;
      // 2 j h / Np with h = floor(Np / 2), reduced mod 2 in integers first
      ph += (float)((2ll * j[e] * (G.np[e] / 2)) % (2ll * G.np[e])) / (float)G.np[e];
    }
  }
  float c = 1.f, s = 0.f;
  if (odd) sincospif(ph, &s, &c);
  return sign ? make_float2(-c, -s) : make_float2(c, s);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ int wrapm(int v, int m) {
  v %= m;
  return v < 0 ? v + m : v;
}

// out[(b*C + c)][j] = maps[c][i] * apod[i] * x[b][i] for the source i of j, else 0
__global__ void pad_shift_kernel(PadGeo G, const float2* __restrict__ x, long long nbatch, const float* __restrict__ apod,
                                 const float2* __restrict__ maps, int nmaps, float2* __restrict__ out) {
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= G.npvol) return;
  const int j2 = (int)(j % G.np[2]);
  const long long r = j / G.np[2];
  const int j1 = (int)(r % G.np[1]), j0 = (int)(r / G.np[1]);
  const int i0 = wrapm(j0 + G.sh[0], G.np[0]) - G.off[0];
  const int i1 = wrapm(j1 + G.sh[1], G.np[1]) - G.off[1];
  const int i2 = wrapm(j2 + G.sh[2], G.np[2]) - G.off[2];
  const bool in = i0 >= 0 && i0 < G.n[0] && i1 >= 0 && i1 < G.n[1] && i2 >= 0 && i2 < G.n[2];
  const long long i = in ? ((long long)i0 * G.n[1] + i1) * G.n[2] + i2 : 0;
  const float a = (in && apod) ? apod[i] : 1.f;
  const int C = maps ? nmaps : 1;
  const float2 md = G.modulate ? modulation(G, j0, j1, j2) : make_float2(1.f, 0.f);
  for (long long b = 0; b < nbatch; ++b) {
    float2 v = make_float2(0.f, 0.f);
    if (in) {
      v = x[b * G.nvol + i];
      v.x *= a;
      v.y *= a;
    }
    for (int c = 0; c < C; ++c) {
      float2 o = v;
      if (maps && in) {
        const float2 m = maps[(long long)c * G.nvol + i];
        o = make_float2(m.x * v.x - m.y * v.y, m.x * v.y + m.y * v.x);
      }
      if (G.modulate) o = cmul(o, md);
      out[(b * C + c) * G.npvol + j] = o;
    }
  }
}

// out[b][i] = alpha * apod[i] * sum_c conj(maps[c][i]) z[(b*C + c)][src(i)] + beta * add[b][i]
__global__ void crop_shift_kernel(PadGeo G, const float2* __restrict__ z, long long nbatch, const float* __restrict__ apod,
                                  const float2* __restrict__ maps, int nmaps, float alpha, const float2* __restrict__ add,
                                  float beta, float2* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nvol) return;
  const int i2 = (int)(i % G.n[2]);
  const long long r = i / G.n[2];
  const int i1 = (int)(r % G.n[1]), i0 = (int)(r / G.n[1]);
  const int j0 = wrapm(i0 + G.off[0] - G.sh[0], G.np[0]);
  const int j1 = wrapm(i1 + G.off[1] - G.sh[1], G.np[1]);
  const int j2 = wrapm(i2 + G.off[2] - G.sh[2], G.np[2]);
  const long long j = ((long long)j0 * G.np[1] + j1) * G.np[2] + j2;
  const float a = (apod ? apod[i] : 1.f) * alpha;
  const int C = maps ? nmaps : 1;
  float2 md = make_float2(1.f, 0.f);
  if (G.modulate) {
    md = modulation(G, j0, j1, j2);
    md.y = -md.y;  // conj(m[j])
  }
  for (long long b = 0; b < nbatch; ++b) {
    float sx = 0.f, sy = 0.f;
    for (int c = 0; c < C; ++c) {
      float2 v = z[(b * C + c) * G.npvol + j];
      if (G.modulate) v = cmul(v, md);
      if (maps) {
        const float2 m = maps[(long long)c * G.nvol + i];
        sx += m.x * v.x + m.y * v.y;  // conj(m) * v
        sy += m.x * v.y - m.y * v.x;
      } else {
        sx += v.x;
        sy += v.y;
      }
    }
    float2 o = make_float2(a * sx, a * sy);
    if (add) {
      const float2 q = add[b * G.nvol + i];
      o.x = fmaf(beta, q.x, o.x);
      o.y = fmaf(beta, q.y, o.y);
    }
    out[b * G.nvol + i] = o;
  }
}

int make_pad_geo(int32_t ndim, const int64_t* n, const int64_t* np, const int64_t* off, const int64_t* shift,
                 int32_t modulate, PadGeo& G) {
  G.modulate = modulate ? 1 : 0;
  if (ndim < 1 || ndim > 3 || !n || !np || !off || !shift) TLGB_FAIL(TLGB_ERR_INVALID, "pad/crop: bad dims");
  G.nvol = G.npvol = 1;
  for (int e = 0; e < 3; ++e) {
    const int a = e - (3 - ndim);
    const int64_t ne = a >= 0 ? n[a] : 1, pe = a >= 0 ? np[a] : 1, oe = a >= 0 ? off[a] : 0, se = a >= 0 ? shift[a] : 0;
    if (ne < 1 || pe < ne || oe < 0 || oe + ne > pe || pe >= (1ll << 30) || se < 0 || se >= pe)
      TLGB_FAIL(TLGB_ERR_INVALID, "pad/crop: sizes, offsets or shifts out of range");
    G.n[e] = (int)ne;
    G.np[e] = (int)pe;
    G.off[e] = (int)oe;
    G.sh[e] = (int)se;
    // one thread per padded voxel: grid x below 2^31 CTAs of 256
    if (G.npvol > ((1ll << 38) - 1) / pe)
      TLGB_FAIL(TLGB_ERR_UNSUPPORTED, "pad/crop: padded volume too large for one launch");
    G.nvol *= ne;
    G.npvol *= pe;
  }
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_pad_shift_c64(const void* x, int64_t nbatch, int32_t ndim, const int64_t* n, const int64_t* np,
                                  const int64_t* off, const int64_t* shift, int32_t modulate, const float* apod,
                                  const void* maps, int32_t nmaps, void* out, tlgb_stream_t stream) {
  PadGeo G;
  TLGB_TRY(make_pad_geo(ndim, n, np, off, shift, modulate, G));
  if (nbatch < 0 || (maps && nmaps < 1)) TLGB_FAIL(TLGB_ERR_INVALID, "pad_shift: bad batch or map count");
  if (nbatch == 0) return TLGB_OK;
  if (!x || !out) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  pad_shift_kernel<<<(unsigned)cdiv(G.npvol, 256), 256, 0, (cudaStream_t)stream>>>(
      G, (const float2*)x, nbatch, apod, (const float2*)maps, nmaps, (float2*)out);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}

extern "C" int tlgb_crop_shift_c64(const void* z, int64_t nbatch, int32_t ndim, const int64_t* n, const int64_t* np,
                                   const int64_t* off, const int64_t* shift, int32_t modulate, const float* apod,
                                   const void* maps, int32_t nmaps, float alpha, const void* add, float beta,
                                   void* out, tlgb_stream_t stream) {
  PadGeo G;
  TLGB_TRY(make_pad_geo(ndim, n, np, off, shift, modulate, G));
  if (nbatch < 0 || (maps && nmaps < 1)) TLGB_FAIL(TLGB_ERR_INVALID, "crop_shift: bad batch or map count");
  if (nbatch == 0) return TLGB_OK;
  if (!z || !out) TLGB_FAIL(TLGB_ERR_INVALID, "null pointer");
  crop_shift_kernel<<<(unsigned)cdiv(G.nvol, 256), 256, 0, (cudaStream_t)stream>>>(
      G, (const float2*)z, nbatch, apod, (const float2*)maps, nmaps, alpha, (const float2*)add, beta, (float2*)out);
  TLGB_CHECK_LAUNCH();
  return TLGB_OK;
}
