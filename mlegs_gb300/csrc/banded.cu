// banded.cu — banded radial operators and solves per (m, k) column.
//
//   matvec: xxdx (tridiagonal), del2h, del2 (pentadiagonal), mlegs_scalar_ops.f90:418-573, with the
//           bands of mlegs_spectfm_diff.f90:6-152 precomputed once per m (kit.cu); del2 adds -ak^2 on
//           the diagonal per k.  One CTA per (m, k) column stages the column in shared memory and
//           applies the band in place.
//   solve:  ihelm, idel2 (pre/pro ln), ihelmp (:575-1000) through lsolve -> zgbtrf + zgbtrs
//           (mlegs_bndmat_ops.f90:369-457): LU with partial pivoting over kl rows, multipliers by the
//           reciprocal pivot, U of bandwidth kl+ku, one right-hand side.  One thread per system;
//           the factor lives in a scratch band laid out [row][diagonal][system] so that a warp's
//           32 systems touch consecutive addresses.
// Every per-(m,k) loop of the reference visits k = 1..nzc and then k = nzcu..nzdim; when nzc == nzcu
// (nzchop = nz/2+1) the shared slot is processed twice, and so it is here.
#include "common.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>

namespace mlg {

__device__ __forceinline__ int k_count(int k0, int nzc, int nzcu, int nzdim) {  // 0-based k
  int kk = k0 + 1;
  return (kk <= min(nzdim, nzc) ? 1 : 0) + (kk >= max(nzcu, 1) ? 1 : 0);
}

// op: 0 = xxdx, 1 = del2h, 2 = del2
// ln handling (column (m=0,k=0) only): the ln terms added after the band product, and ln <- 0.
// T = double: the plain form; T = float: the mixed form (stencil in FP32, conversions on the integer
// pipe, the ln terms still in FP64).
template <typename T> struct BC;
template <> struct BC<double> {
  typedef double2 C;
  static __device__ __forceinline__ C ld(const double2* p) { return *p; }
  static __device__ __forceinline__ void st(double2* p, C v) { *p = v; }
  static __device__ __forceinline__ double cv(double v) { return v; }
};
template <> struct BC<float> {
  typedef float2 C;
  static __device__ __forceinline__ C ld(const double2* p) { return ld_c32(p); }
  static __device__ __forceinline__ void st(double2* p, C v) { st_c32(p, v); }
  static __device__ __forceinline__ float cv(double v) { return d2f_fast(v); }
};
// the band tables in T: FP64 as built, or their FP32 copies (made once with the kit)
struct BandTabs {
  const double *bd2, *bxx, *ak;
  const float *bd2f, *bxxf, *ak2f;
};
template <typename T> __device__ __forceinline__ T btab(const double* d, const float* f, size_t i);
template <> __device__ __forceinline__ double btab<double>(const double* d, const float* f, size_t i) { (void)f; return d[i]; }
template <> __device__ __forceinline__ float btab<float>(const double* d, const float* f, size_t i) { (void)d; return f[i]; }
template <typename T> __device__ __forceinline__ T bakv2(const BandTabs& t, int k);   // akval**2 (mlegs_spectfm_diff.f90:144)
template <> __device__ __forceinline__ double bakv2<double>(const BandTabs& t, int k) { return t.ak[k] * t.ak[k]; }
template <> __device__ __forceinline__ float bakv2<float>(const BandTabs& t, int k) { return t.ak2f[k]; }
// -v exactly, by the sign bits (off the FP64 pipe)
__device__ __forceinline__ double2 neg_d2(double2 v) {
  return make_double2(__hiloint2double(__double2hiint(v.x) ^ (int)0x80000000, __double2loint(v.x)),
                      __hiloint2double(__double2hiint(v.y) ^ (int)0x80000000, __double2loint(v.y)));
}

// one (m, k) column of nn rows, applied cnt times in place through shared memory
template <typename T>
__device__ __forceinline__ void band_col(double2* __restrict__ g, const BandTabs& tb, int k, int op, int m, int ne,
                                         int nn, int cnt, unsigned char* smem, int nrdim) {
  typedef typename BC<T>::C C;
  C* c0 = (C*)smem;
  C* c1 = c0 + nrdim;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = BC<T>::ld(g + i);
  __syncthreads();
  const T akv2 = bakv2<T>(tb, k);
  for (int rep = 0; rep < cnt; ++rep) {
    for (int i = threadIdx.x; i < nn; i += blockDim.x) {
      C acc; acc.x = 0; acc.y = 0;
      if (op == 0) {
        const size_t b = 3 * ((size_t)i + (size_t)ne * m);
        if (i - 1 >= 0) { T v = btab<T>(tb.bxx, tb.bxxf, b); acc.x += v * c0[i - 1].x; acc.y += v * c0[i - 1].y; }
        if (i + 1 < nn) { T v = btab<T>(tb.bxx, tb.bxxf, b + 2); acc.x += v * c0[i + 1].x; acc.y += v * c0[i + 1].y; }
      } else {
        const size_t b = 5 * ((size_t)i + (size_t)ne * m);
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          int j = i - 2 + c;
          if (j < 0 || j >= nn) continue;
          T v = btab<T>(tb.bd2, tb.bd2f, b + c);
          if (c == 2 && op == 2) v = v - akv2;
          acc.x += v * c0[j].x;
          acc.y += v * c0[j].y;
        }
      }
      c1[i] = acc;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = c1[i];
    __syncthreads();
  }
  for (int i = threadIdx.x; i < nn; i += blockDim.x) BC<T>::st(g + i, c0[i]);
  __syncthreads();
}

// grid (k, m).  The mixed form (T = float) still applies the m = 0 columns in FP64: they hold the
// axisymmetric mean flow, and their radial sums cancel toward the axis.
template <typename T>
__global__ void k_band_apply(double2* __restrict__ e, BandTabs tb, double* __restrict__ lnp, const double* __restrict__ lognorm,
                             int op, int nrdim, int npdim, int ne, int nrc, int npc, int nzc, int nzcu, int nzdim,
                             double ell) {
  extern __shared__ __align__(16) unsigned char band_smem[];
  int m = blockIdx.y, k = blockIdx.x;
  int nn = max(min(nrc, nrc - m), 0);
  int cnt = k_count(k, nzc, nzcu, nzdim);
  double2* g = e + (size_t)nrdim * (m + (size_t)npdim * k);
  bool lnblk = (m == 0 && k == 0);
  double lnin = 0.0;
  if (lnblk) lnin = *lnp;
  if (m < npc && nn > 0 && cnt > 0) {
    if (m == 0) band_col<double>(g, tb, k, op, m, ne, nn, cnt, band_smem, nrdim);
    else band_col<T>(g, tb, k, op, m, ne, nn, cnt, band_smem, nrdim);
  }
  if (lnblk && threadIdx.x == 0) {
    // the log-term contributions land on e(1..3,1,1) whether or not the column was active
    double e2 = ell * ell;
    if (op == 0) {   // r d/dr of the log term (:452-456)
      g[0].x += 1.0 / exp(lognorm[0]) * lnin;
      g[1].x += 1.0 / exp(lognorm[1]) * lnin;
    } else {         // (:506-511, :561-566)
      g[0].x += 4.0 / 3.0 / e2 / exp(lognorm[0]) * lnin;
      g[1].x -= 2.0 / 1.0 / e2 / exp(lognorm[1]) * lnin;
      g[2].x += 2.0 / 3.0 / e2 / exp(lognorm[2]) * lnin;
    }
    *lnp = 0.0;
  }
}

// The right-hand side of abcn (mlegs_scalar_ops.f90:1200-1262) with hyperpow = 0, fused:
//   svis = s; svis = del2(svis) (band rows, with the log terms of (0,0)); svis = visc*svis;
//   s = a*(s + 1.5 dt nl - 0.5 dt nl_p + dt/2 svis)   (e and ln; svis%ln = 0 after del2)
// One CTA per (m, k) column of the whole array, the same operations and order as the copy, band
// apply, scale and four-term combination it replaces.  The mixed form runs the m >= 1 stencils in FP32.
template <typename T>
__global__ void k_abcn_rhs(double2* __restrict__ e, const double2* __restrict__ nl, const double2* __restrict__ nlp,
                           double* __restrict__ lnp, const double* __restrict__ lnnl, const double* __restrict__ lnnlp,
                           BandTabs tb, const double* __restrict__ lognorm,
                           int nrdim, int npdim, int ne, int nrc, int npc, int nzc, int nzcu, int nzdim, double ell,
                           double visc, double c1, double c2, double c3, double post) {
  extern __shared__ __align__(16) unsigned char rhs_smem[];
  double2* sv = (double2*)rhs_smem;               // svis of the column (FP64)
  int m = blockIdx.y, k = blockIdx.x;
  int nn = max(min(nrc, nrc - m), 0);
  int cnt = k_count(k, nzc, nzcu, nzdim);
  size_t off = (size_t)nrdim * (m + (size_t)npdim * k);
  double2* g = e + off;
  const double2* n0 = nl + off;
  const double2* n1 = nlp + off;
  const bool act = m < npc && nn > 0 && cnt > 0;
  if (m > 0 && sizeof(T) == sizeof(float)) {
    // the mixed form's m >= 1 columns: the increment 1.5 dt nl - 0.5 dt nl_p + dt/2 visc del2(s) summed
    // in FP32 (its terms carry the FP32 contractions' rounding already), added to the FP64 state
    typedef float2 C;
    C* c0 = (C*)rhs_smem;
    C* c1b = c0 + nrdim;
    if (act) {
      for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = ld_c32(g + i);
      __syncthreads();
      const float akv2 = tb.ak2f[k];
      for (int rep = 0; rep < cnt; ++rep) {
        for (int i = threadIdx.x; i < nn; i += blockDim.x) {
          C acc; acc.x = 0; acc.y = 0;
          const float* b = tb.bd2f + 5 * ((size_t)i + (size_t)ne * m);
#pragma unroll
          for (int c = 0; c < 5; ++c) {
            int j = i - 2 + c;
            if (j < 0 || j >= nn) continue;
            float v = b[c];
            if (c == 2) v = v - akv2;
            acc.x += v * c0[j].x;
            acc.y += v * c0[j].y;
          }
          c1b[i] = acc;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = c1b[i];
        __syncthreads();
      }
    }
    const float f1 = d2f_fast(c1), f2 = d2f_fast(c2), f3 = d2f_fast(c3 * visc);
    for (int i = threadIdx.x; i < nrdim; i += blockDim.x) {
      double2 x = g[i];
      float2 a1 = ld_c32(n0 + i), a2 = ld_c32(n1 + i);
      float2 s3 = (act && i < nn) ? c0[i] : make_float2(d2f_fast(x.x), d2f_fast(x.y));
      float dx = f1 * a1.x, dy = f1 * a1.y;
      dx = fmaf(f2, a2.x, dx); dy = fmaf(f2, a2.y, dy);
      dx = fmaf(f3, s3.x, dx); dy = fmaf(f3, s3.y, dy);
      g[i] = make_double2(post * (x.x + f2d_fast(dx)), post * (x.y + f2d_fast(dy)));
    }
    return;
  }
  bool lnblk = (m == 0 && k == 0);
  double lnin = lnblk ? *lnp : 0.0;
  for (int i = threadIdx.x; i < nrdim; i += blockDim.x) sv[i] = g[i];
  __syncthreads();
  if (act) {
    double2* c0 = sv;
    double2* c1b = sv + nrdim;
    double akv2 = tb.ak[k] * tb.ak[k];
    for (int rep = 0; rep < cnt; ++rep) {
      for (int i = threadIdx.x; i < nn; i += blockDim.x) {
        double2 acc; acc.x = 0; acc.y = 0;
        const double* b = tb.bd2 + 5 * ((size_t)i + (size_t)ne * m);
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          int j = i - 2 + c;
          if (j < 0 || j >= nn) continue;
          double v = b[c];
          if (c == 2) v = v - akv2;
          acc.x += v * c0[j].x;
          acc.y += v * c0[j].y;
        }
        c1b[i] = acc;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = c1b[i];
      __syncthreads();
    }
  }
  if (lnblk && threadIdx.x == 0) {   // the log terms of del2 (:561-566) on svis(1..3, 1, 1)
    double e2 = ell * ell;
    sv[0].x += 4.0 / 3.0 / e2 / exp(lognorm[0]) * lnin;
    sv[1].x -= 2.0 / 1.0 / e2 / exp(lognorm[1]) * lnin;
    sv[2].x += 2.0 / 3.0 / e2 / exp(lognorm[2]) * lnin;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nrdim; i += blockDim.x) {
    double2 x = g[i], a1 = n0[i], a2 = n1[i], s3 = sv[i];
    s3 = make_double2(0.0 + visc * s3.x, 0.0 + visc * s3.y);   // svis = visc*svis
    double2 acc = make_double2(0, 0);
    acc.x += 1.0 * x.x; acc.y += 1.0 * x.y;
    acc.x += c1 * a1.x; acc.y += c1 * a1.y;
    acc.x += c2 * a2.x; acc.y += c2 * a2.y;
    acc.x += c3 * s3.x; acc.y += c3 * s3.y;
    g[i] = make_double2(post * acc.x, post * acc.y);
  }
  if (lnblk && threadIdx.x == 0) {
    double l = 0.0;
    l += 1.0 * lnin;
    l += c1 * *lnnl;
    l += c2 * *lnnlp;
    l += c3 * 0.0;
    *lnp = post * l;
  }
}

static BandTabs band_tabs() { return BandTabs{G.bd2, G.bxx, G.ak, G.bd2f, G.bxxf, G.ak2f}; }

int launch_abcn_rhs(Scalar& s, const Scalar& nl, const Scalar& nl_p, double dt, double a) {
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  dim3 grid(G.nzdim, G.npdim);
  size_t sm = 2ull * G.nrdim * sizeof(double2);
  kt_begin(2);
  if (G.precision == MLG_MIXED) {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_abcn_rhs<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_abcn_rhs<float><<<grid, 128, sm, G.stream>>>(s.e, nl.e, nl_p.e, s.ln, nl.ln, nl_p.ln, band_tabs(), G.lognorm, G.nrdim,
                                                   G.npdim, G.ne, c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell, G.P.visc,
                                                   1.5 * dt, -.5 * dt, dt / 2.0, a);
  } else {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_abcn_rhs<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_abcn_rhs<double><<<grid, 128, sm, G.stream>>>(s.e, nl.e, nl_p.e, s.ln, nl.ln, nl_p.ln, band_tabs(), G.lognorm, G.nrdim,
                                                    G.npdim, G.ne, c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell, G.P.visc,
                                                    1.5 * dt, -.5 * dt, dt / 2.0, a);
  }
  MLG_LAUNCH();
  kt_end(2, 5.0 * G.fsize * 16);
  return 0;
}

// dst = scale * band(src), out of place: the same values as copying src to dst, applying the band
// operator in place and multiplying dst by scale (dst%ln = 0), in one pass over every column
template <typename T>
__global__ void __launch_bounds__(128, 16) k_band_apply_to(double2* __restrict__ dst, const double2* __restrict__ src, const double* __restrict__ lnsrc,
                                double* __restrict__ lndst, BandTabs tb, const double* __restrict__ lognorm, int op,
                                int nrdim, int npdim, int ne, int nrc, int npc, int nzc, int nzcu, int nzdim, double ell,
                                double scale, int smode, PostChop pc) {
  extern __shared__ __align__(16) unsigned char bat_smem[];
  double2* sv = (double2*)bat_smem;   // the column, then its band product on the active rows (FP64)
  int m = blockIdx.y, k = blockIdx.x;
  int nn = max(min(nrc, nrc - m), 0);
  int cnt = k_count(k, nzc, nzcu, nzdim);
  size_t off = (size_t)nrdim * (m + (size_t)npdim * k);
  bool lnblk = (m == 0 && k == 0);
  for (int i = threadIdx.x; i < nrdim; i += blockDim.x) sv[i] = src[off + i];
  __syncthreads();
  if (m < npc && nn > 0 && cnt > 0) {
    if (m == 0) {
      double2* c0 = sv;
      double2* c1 = sv + nrdim;
      double akv2 = tb.ak[k] * tb.ak[k];
      for (int rep = 0; rep < cnt; ++rep) {
        for (int i = threadIdx.x; i < nn; i += blockDim.x) {
          double2 acc; acc.x = 0; acc.y = 0;
          if (op == 0) {
            const double* b = tb.bxx + 3 * ((size_t)i + (size_t)ne * m);
            if (i - 1 >= 0) { double v = b[0]; acc.x += v * c0[i - 1].x; acc.y += v * c0[i - 1].y; }
            if (i + 1 < nn) { double v = b[2]; acc.x += v * c0[i + 1].x; acc.y += v * c0[i + 1].y; }
          } else {
            const double* b = tb.bd2 + 5 * ((size_t)i + (size_t)ne * m);
#pragma unroll
            for (int c = 0; c < 5; ++c) {
              int j = i - 2 + c;
              if (j < 0 || j >= nn) continue;
              double v = b[c];
              if (c == 2 && op == 2) v = v - akv2;
              acc.x += v * c0[j].x;
              acc.y += v * c0[j].y;
            }
          }
          c1[i] = acc;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = c1[i];
        __syncthreads();
      }
    } else {
      typedef typename BC<T>::C C;
      C* c0 = (C*)(sv + 2 * nrdim);
      C* c1 = c0 + nrdim;
      for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = BC<T>::ld(sv + i);
      __syncthreads();
      const T akv2 = bakv2<T>(tb, k);
      for (int rep = 0; rep < cnt; ++rep) {
        for (int i = threadIdx.x; i < nn; i += blockDim.x) {
          C acc; acc.x = 0; acc.y = 0;
          if (op == 0) {
            const size_t b = 3 * ((size_t)i + (size_t)ne * m);
            if (i - 1 >= 0) { T v = btab<T>(tb.bxx, tb.bxxf, b); acc.x += v * c0[i - 1].x; acc.y += v * c0[i - 1].y; }
            if (i + 1 < nn) { T v = btab<T>(tb.bxx, tb.bxxf, b + 2); acc.x += v * c0[i + 1].x; acc.y += v * c0[i + 1].y; }
          } else {
            const size_t b = 5 * ((size_t)i + (size_t)ne * m);
#pragma unroll
            for (int c = 0; c < 5; ++c) {
              int j = i - 2 + c;
              if (j < 0 || j >= nn) continue;
              T v = btab<T>(tb.bd2, tb.bd2f, b + c);
              if (c == 2 && op == 2) v = v - akv2;
              acc.x += v * c0[j].x;
              acc.y += v * c0[j].y;
            }
          }
          c1[i] = acc;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = c1[i];
        __syncthreads();
      }
      for (int i = threadIdx.x; i < nn; i += blockDim.x) BC<T>::st(sv + i, c0[i]);
    }
    __syncthreads();
  }
  if (lnblk && threadIdx.x == 0) {
    double lnin = *lnsrc;
    double e2 = ell * ell;
    if (op == 0) {   // (:452-456)
      sv[0].x += 1.0 / exp(lognorm[0]) * lnin;
      sv[1].x += 1.0 / exp(lognorm[1]) * lnin;
    } else {         // (:506-511, :561-566)
      sv[0].x += 4.0 / 3.0 / e2 / exp(lognorm[0]) * lnin;
      sv[1].x -= 2.0 / 1.0 / e2 / exp(lognorm[1]) * lnin;
      sv[2].x += 2.0 / 3.0 / e2 / exp(lognorm[2]) * lnin;
    }
    *lndst = 0.0;
  }
  __syncthreads();
  const int zf = chop_from(pc, m, k, nrdim);
  for (int i = threadIdx.x; i < nrdim; i += blockDim.x) {
    double2 v = sv[i];
    if (smode == 1) v = neg_d2(v);
    else if (smode == 2) v = make_double2(0.0 + scale * v.x, 0.0 + scale * v.y);
    if (i >= zf) v = make_double2(0.0, 0.0);   // the chop that follows
    dst[off + i] = v;
  }
}

// ------------------------------------------------------------------------------------------------
// (ur, up) of vector_reconstruction (mlegs_scalar_ops.f90:1455-1502: ur = r d/dr chi, up = r d/dr psi,
// then ur = i m psi + i kv ur, up = -up - m kv chi on the active window) per (m, k) column in one pass: the
// two xxdx stencils run side by side in shared memory, the mix follows, and the rows outside the
// window keep the band products' copies of their inputs (with the log terms of (0,0)); ln(ur) =
// ln(up) = 0.  U = double for m = 0 (and the plain form), float for the mixed form's m >= 1.
template <typename U>
__device__ __forceinline__ void uv_col(double2* __restrict__ ur, double2* __restrict__ up, const double2* __restrict__ psi,
                                       const double2* __restrict__ chi, double lnp, double lnc, const BandTabs& tb,
                                       const double* __restrict__ lognorm, int nrdim, int ne, int nn, int cnt, bool act,
                                       int m, int k, bool lnblk, int zf, unsigned char* smem) {
  typedef typename BC<U>::C C;
  C* a0 = (C*)smem;
  C* a1 = a0 + nrdim;
  C* b0 = a1 + nrdim;
  C* b1 = b0 + nrdim;
  if (act) {
    for (int i = threadIdx.x; i < nn; i += blockDim.x) { a0[i] = BC<U>::ld(chi + i); b0[i] = BC<U>::ld(psi + i); }
    __syncthreads();
    for (int rep = 0; rep < cnt; ++rep) {
      for (int i = threadIdx.x; i < nn; i += blockDim.x) {
        C sa, sb;
        sa.x = 0; sa.y = 0; sb.x = 0; sb.y = 0;
        const size_t b = 3 * ((size_t)i + (size_t)ne * m);
        if (i - 1 >= 0) {
          U v = btab<U>(tb.bxx, tb.bxxf, b);
          sa.x += v * a0[i - 1].x; sa.y += v * a0[i - 1].y;
          sb.x += v * b0[i - 1].x; sb.y += v * b0[i - 1].y;
        }
        if (i + 1 < nn) {
          U v = btab<U>(tb.bxx, tb.bxxf, b + 2);
          sa.x += v * a0[i + 1].x; sa.y += v * a0[i + 1].y;
          sb.x += v * b0[i + 1].x; sb.y += v * b0[i + 1].y;
        }
        a1[i] = sa;
        b1[i] = sb;
      }
      __syncthreads();
      C* t = a0; a0 = a1; a1 = t;
      t = b0; b0 = b1; b1 = t;
    }
  }
  const double kv = tb.ak[k], mv = (double)m;
  for (int i = threadIdx.x; i < nrdim; i += blockDim.x) {
    if (i >= zf) {   // the chop that follows
      ur[i] = make_double2(0.0, 0.0);
      up[i] = make_double2(0.0, 0.0);
      continue;
    }
    const double2 c = chi[i], p = psi[i];
    const bool in = act && i < nn;
    double2 av = c, bv = p;
    if (in) { BC<U>::st(&av, a0[i]); BC<U>::st(&bv, b0[i]); }
    if (lnblk && i < 2) {   // r d/dr of the log terms (mlegs_scalar_ops.f90:452-456)
      av.x += 1.0 / exp(lognorm[i]) * lnc;
      bv.x += 1.0 / exp(lognorm[i]) * lnp;
    }
    if (!in) { ur[i] = av; up[i] = bv; continue; }
    if (sizeof(U) == sizeof(double)) {
      ur[i] = make_double2(-mv * p.y - kv * av.y, mv * p.x + kv * av.x);
      up[i] = make_double2(-bv.x - mv * kv * c.x, -bv.y - mv * kv * c.y);
    } else {
      const float mf = (float)m, kf = d2f_fast(kv), mk = d2f_fast(mv * kv);
      const C af = a0[i], bf = b0[i];
      const float2 pf = ld_c32(psi + i), cf = ld_c32(chi + i);
      st_c32(ur + i, make_float2(-mf * pf.y - kf * (float)af.y, mf * pf.x + kf * (float)af.x));
      st_c32(up + i, make_float2(-(float)bf.x - mk * cf.x, -(float)bf.y - mk * cf.y));
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(128, 12) k_tp2vec_uv(double2* __restrict__ ur, double2* __restrict__ up, const double2* __restrict__ psi,
                            const double2* __restrict__ chi, const double* __restrict__ lnpsi,
                            const double* __restrict__ lnchi, double* __restrict__ lnur, double* __restrict__ lnup,
                            BandTabs tb, const double* __restrict__ lognorm, int nrdim, int npdim, int ne, int nrc,
                            int npc, int nzc, int nzcu, int nzdim, PostChop pc) {
  extern __shared__ __align__(16) unsigned char uv_smem[];
  const int m = blockIdx.y, k = blockIdx.x;
  const int nn = max(min(nrc, nrc - m), 0);
  const int cnt = k_count(k, nzc, nzcu, nzdim);
  const size_t off = (size_t)nrdim * (m + (size_t)npdim * k);
  const bool lnblk = m == 0 && k == 0;
  const double lnp = lnblk ? *lnpsi : 0.0, lnc = lnblk ? *lnchi : 0.0;
  const bool act = m < npc && nn > 0 && cnt > 0;
  const int zf = chop_from(pc, m, k, nrdim);
  if (m == 0) uv_col<double>(ur + off, up + off, psi + off, chi + off, lnp, lnc, tb, lognorm, nrdim, ne, nn, cnt, act, m, k, lnblk, zf, uv_smem);
  else uv_col<T>(ur + off, up + off, psi + off, chi + off, lnp, lnc, tb, lognorm, nrdim, ne, nn, cnt, act, m, k, lnblk, zf, uv_smem);
  if (lnblk && threadIdx.x == 0) { *lnur = 0.0; *lnup = 0.0; }
}

int launch_tp2vec_uv(Scalar& ur, Scalar& up, const Scalar& psi, const Scalar& chi, const ChopIdx& c, PostChop pc) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  dim3 grid(G.nzdim, G.npdim);
  size_t sm = 4ull * G.nrdim * sizeof(double2);
  kt_begin(KT_BAND);
  if (G.precision == MLG_MIXED) {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_tp2vec_uv<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_tp2vec_uv<float><<<grid, 128, sm, G.stream>>>(ur.e, up.e, psi.e, chi.e, psi.ln, chi.ln, ur.ln, up.ln, band_tabs(),
                                                    G.lognorm, G.nrdim, G.npdim, G.ne, c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, pc);
  } else {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_tp2vec_uv<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_tp2vec_uv<double><<<grid, 128, sm, G.stream>>>(ur.e, up.e, psi.e, chi.e, psi.ln, chi.ln, ur.ln, up.ln, band_tabs(),
                                                     G.lognorm, G.nrdim, G.npdim, G.ne, c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, pc);
  }
  MLG_LAUNCH();
  kt_end(KT_BAND, 4.0 * G.fsize * 16);
  return 0;
}

int launch_band_apply_to(Scalar& dst, const Scalar& src, int op, const ChopIdx& c, double scale, PostChop pc,
                         cudaStream_t st) {
  if (!st) st = G.stream;
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  const int smode = scale == 1.0 ? 0 : scale == -1.0 ? 1 : 2;   // identity, exact negation, FP64 product
  dim3 grid(G.nzdim, G.npdim);
  size_t sm = 4ull * G.nrdim * sizeof(double2);
  kt_begin(KT_BAND);
  if (G.precision == MLG_MIXED) {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_band_apply_to<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_band_apply_to<float><<<grid, 128, sm, st>>>(dst.e, src.e, src.ln, dst.ln, band_tabs(), G.lognorm, op,
                                                        G.nrdim, G.npdim, G.ne, c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell,
                                                        scale, smode, pc);
  } else {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_band_apply_to<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_band_apply_to<double><<<grid, 128, sm, st>>>(dst.e, src.e, src.ln, dst.ln, band_tabs(), G.lognorm, op,
                                                         G.nrdim, G.npdim, G.ne, c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell,
                                                         scale, smode, pc);
  }
  MLG_LAUNCH();
  kt_end(KT_BAND, 2.0 * G.fsize * 16);
  return 0;
}

int launch_band_apply(Scalar& s, int op, const ChopIdx& c) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  dim3 grid(G.nzdim, std::max(c.npc, 1));
  kt_begin(2);
  if (G.precision == MLG_MIXED) {
    size_t sm = 2ull * G.nrdim * sizeof(double2);   // the m = 0 columns run in FP64
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_band_apply<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_band_apply<float><<<grid, 128, sm, G.stream>>>(s.e, band_tabs(), s.ln, G.lognorm, op, G.nrdim, G.npdim, G.ne,
                                                     c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell);
  } else {
    size_t sm = 2ull * G.nrdim * sizeof(double2);
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_band_apply<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_band_apply<double><<<grid, 128, sm, G.stream>>>(s.e, band_tabs(), s.ln, G.lognorm, op, G.nrdim, G.npdim, G.ne,
                                                      c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell);
  }
  MLG_LAUNCH();
  kt_end(2, 2.0 * G.fsize * 16);
  return 0;
}

// ------------------------------------------------------------------------------------------------
// banded LU solve, one thread per (m, k) system.
// mode 0: ihelm / idel2 generic:  A = D0(m) - ak^2 I + alpha I             (kl = ku = 2)
// mode 1: idel2_proln on (0,0):   A = D0(0) with the column-1 log-term additions (:705-711)
// mode 2: idel2_preln on (0,0):   rows shifted down, bordered by the ln unknown (:609-625), kl = 3
// mode 3: ihelmp:                 A = D^q + beta D + alpha I, q = power/2   (kl = ku = power)
// flags (per launch): pre-solve ln handling for ihelm/ihelmp, post-solve ln for idel2.
struct SolveArgs {
  double2* e;
  double* ws;           // scratch band [row][W][nsys]
  double* lnp;
  const double* bd2;
  const double* ak;
  const double* lognorm;
  int* status;
  int nrdim, npdim, ne, nrc, npc, nzc, nzcu, nzdim;
  int nsys;             // npc * nzdim (the cached-factor paths: the positions of sys_mk)
  int nsp = 0;          // the factor image's system stride: nsys rounded up to 32
  double alpha, beta, ell, preln;
  int kind;             // 0 ihelm, 1 idel2_proln, 2 idel2_preln, 3 ihelmp
  int power;
  int skip_root;        // substitution: leave the (0,0) column to the bordered solve
  int transpose;        // factor / solve A^T (kinds 0 and 1): the adjoint's systems
  int no_ln;            // substitution: skip the log-term handling of the (0,0) column
  double2* e2 = nullptr;  // substitution: a second field with the same matrices (paired solve), or null
  double* lnp2 = nullptr;
  int* pivflag = nullptr;  // per 32 systems: non-zero when one of them exchanges rows (factor writes, substitution reads)
  int lead = 0;            // cached factors: positions of the twice-solved systems (a multiple of 32; sys_mk)
};

// The order of the systems in the cached factors and in the substitution's blocks (position p -> (m, k);
// false for a position that holds no system).  The k that both halves of the reference's k loop visit
// (the shared slot when nzc == nzcu) are solved twice in a row, and a block holding one of them runs
// both passes twice.  Those systems come first, m by m, in blocks of their own (`lead` positions, padded
// to a whole block); then every (m, k) follows m-major as p = lead + m nzdim + k, with the twice-solved
// k left idle there.  The 32-system blocks of the second part are those of the plain order, so the
// systems that exchange rows (and take the substitution's slower paths) fall into the same blocks.
__device__ __forceinline__ bool sys_mk(const SolveArgs& a, int p, int& m, int& k) {
  const int klo = max(a.nzcu, 1) - 1, khi = min(a.nzdim, a.nzc) - 1;
  if (p < a.lead) {
    const int nd = max(khi - klo + 1, 1);
    m = p / nd;
    k = klo + (p - m * nd);
    return m < a.npc;
  }
  const int q = p - a.lead;
  m = q / a.nzdim;
  k = q - m * a.nzdim;
  return a.lead == 0 || k < klo || k > khi;
}

// entry (i, j) (0-based) of D(m,k) = D0(m) - ak^2 I for an n x n truncation
__device__ __forceinline__ double dmat(const SolveArgs& a, int m, double akv, int n, int i, int j) {
  if (i < 0 || j < 0 || i >= n || j >= n) return 0.0;
  int c = j - i + 2;
  if (c < 0 || c > 4) return 0.0;
  double v = a.bd2[c + 5 * ((size_t)i + (size_t)a.ne * m)];
  if (c == 2) v = v - akv * akv;
  return v;
}

__global__ void k_band_solve(SolveArgs a) {
  int sys = blockIdx.x * blockDim.x + threadIdx.x;
  if (sys >= a.nsys) return;
  int m = sys / a.nzdim, k = sys % a.nzdim;
  int cnt = k_count(k, a.nzc, a.nzcu, a.nzdim);
  int nn = max(min(a.nrc, a.nrc - m), 0);
  bool root = (m == 0 && k == 0);
  double e2 = pow(a.ell, 2.0);
  // ln handling before the solves (ihelm :818-824, ihelmp :937-951 is done separately)
  if (root && a.kind == 0) {
    double lnin = *a.lnp;
    double lno = lnin / a.alpha;
    *a.lnp = lno;
    double2* g = a.e;
    g[0].x -= 4.0 / 3.0 / e2 / exp(a.lognorm[0]) * lno;
    g[1].x += 2.0 / 1.0 / e2 / exp(a.lognorm[1]) * lno;
    g[2].x -= 2.0 / 3.0 / e2 / exp(a.lognorm[2]) * lno;
  }
  if (m >= a.npc || nn < 1 || cnt == 0) return;
  bool special = root && (a.kind == 1 || a.kind == 2);
  int kl = 2, ku = 2;
  if (special && a.kind == 2) { kl = 3; ku = 2; }
  if (a.kind == 3) { kl = a.power; ku = a.power; }
  int W = 2 * kl + ku + 1;
  double akv = a.ak[k];
  double2* x = a.e + (size_t)a.nrdim * (m + (size_t)a.npdim * k);
  double alpha = (a.kind == 0 || a.kind == 3) ? a.alpha : 0.0;
  size_t ns = a.nsys;
#define U(i, j) a.ws[((size_t)(i) * W + ((j) - (i) + kl)) * ns + sys]
  for (int rep = 0; rep < cnt; ++rep) {
    // build the band rows (columns i-kl .. i+ku) into the work band
    for (int i = 0; i < nn; ++i) {
      for (int c = 0; c < W; ++c) a.ws[((size_t)i * W + c) * ns + sys] = 0.0;
      if (a.kind == 3) {
        // row i of the truncated power D^q, q = power/2 (the band products of mulrbrb,
        // mlegs_bndmat_ops.f90:251-318, on nn x nn matrices), window i-8 .. i+8
        int q = a.power / 2;
        double rv[17], nv[17];
        int w0 = i - 8;
        for (int u = 0; u < 17; ++u) rv[u] = 0.0;
        for (int jj = max(0, i - 2); jj <= min(nn - 1, i + 2); ++jj) rv[jj - w0] = dmat(a, m, akv, nn, i, jj);
        for (int t = 2; t <= q; ++t) {
          for (int u = 0; u < 17; ++u) nv[u] = 0.0;
          for (int u = 0; u < 17; ++u) {
            int col = w0 + u;
            if (col < 0 || col >= nn) continue;
            for (int jj = max(0, col - 2); jj <= min(nn - 1, col + 2); ++jj) {
              int uu = jj - w0;
              if (uu >= 0 && uu < 17) nv[uu] += rv[u] * dmat(a, m, akv, nn, col, jj);
            }
          }
          for (int u = 0; u < 17; ++u) rv[u] = nv[u];
        }
        for (int j = max(0, i - kl); j <= min(nn - 1, i + ku); ++j) {
          double v = rv[j - w0] + a.beta * dmat(a, m, akv, nn, i, j);
          if (i == j) v += alpha;
          U(i, j) = v;
        }
        continue;
      }
      for (int j = max(0, i - kl); j <= min(nn - 1, i + ku); ++j) {
        double v;
        if (special && a.kind == 1) {
          v = dmat(a, 0, akv, nn, i, j);
          if (j == 0) {
            if (i == 0) v += 4.0 / 3.0 / e2;
            if (i == 1) v -= 2.0 / 1.0 / e2 * exp(a.lognorm[0] - a.lognorm[1]);
            if (i == 2) v += 2.0 / 3.0 / e2 * exp(a.lognorm[0] - a.lognorm[2]);
          }
        } else if (special && a.kind == 2) {
          // del2_pre(2:nn,:) = del2_pre(1:nn-1,:); row 1 = e_1; column-1 additions (:609-617)
          if (i == 0) v = (j == 0) ? 1.0 : 0.0;
          else {
            v = dmat(a, 0, akv, nn, i - 1, j);
            if (j == 0) {
              if (i == 1) v += 4.0 / 3.0 / e2;
              if (i == 2) v -= 2.0 / 1.0 / e2 * exp(a.lognorm[0] - a.lognorm[1]);
              if (i == 3) v += 2.0 / 3.0 / e2 * exp(a.lognorm[0] - a.lognorm[2]);
            }
          }
        } else {
          v = dmat(a, m, akv, nn, i, j);
          if (i == j) v += alpha;
        }
        U(i, j) = v;
      }
    }
    if (special && a.kind == 2 && rep == 0) {
      for (int i = nn - 1; i >= 1; --i) x[i] = x[i - 1];
      x[0] = make_double2(a.preln / exp(a.lognorm[0]), 0.0);
    }
    // factor + forward substitution (gbtrf/gbtrs 'N')
    for (int j = 0; j < nn; ++j) {
      int km = min(kl, nn - 1 - j), p = j;
      double best = fabs(U(j, j));
      for (int i = j + 1; i <= j + km; ++i) {
        double t = fabs(U(i, j));
        if (t > best) { best = t; p = i; }
      }
      if (U(p, j) == 0.0) { atomicExch(a.status, 1); return; }
      int ju = min(nn - 1, j + kl + ku);
      if (p != j) {
        for (int c = j; c <= ju; ++c) { double t = U(p, c); U(p, c) = U(j, c); U(j, c) = t; }
        double2 t = x[p]; x[p] = x[j]; x[j] = t;
      }
      double rp = 1.0 / U(j, j);
      double2 xj = x[j];
      for (int i = j + 1; i <= j + km; ++i) {
        double l = U(i, j) * rp;
        U(i, j) = l;
        for (int c = j + 1; c <= ju; ++c) U(i, c) -= l * U(j, c);
        x[i].x -= l * xj.x;
        x[i].y -= l * xj.y;
      }
    }
    for (int j = nn - 1; j >= 0; --j) {
      double d = U(j, j);
      double2 xj = make_double2(x[j].x / d, x[j].y / d);
      x[j] = xj;
      for (int i = j - 1; i >= max(0, j - kl - ku); --i) {
        double u = U(i, j);
        x[i].x -= xj.x * u;
        x[i].y -= xj.y * u;
      }
    }
  }
#undef U
  if (special) *a.lnp = x[0].x * exp(a.lognorm[0]);
}

// Entry (i, j) of the system matrix of (m, k) for kinds 0..2 (0-based, n x n truncation).
__device__ __forceinline__ double sys_entry(const SolveArgs& a, int kind, bool special, int m, double akv, int nn,
                                            double alpha, double e2, int i, int j) {
  if (a.transpose) { int t = i; i = j; j = t; }
  if (i < 0 || j < 0 || i >= nn || j >= nn) return 0.0;
  if (special && kind == 1) {
    double v = dmat(a, 0, akv, nn, i, j);
    if (j == 0) {
      if (i == 0) v += 4.0 / 3.0 / e2;
      if (i == 1) v -= 2.0 / 1.0 / e2 * exp(a.lognorm[0] - a.lognorm[1]);
      if (i == 2) v += 2.0 / 3.0 / e2 * exp(a.lognorm[0] - a.lognorm[2]);
    }
    return v;
  }
  if (special && kind == 2) {   // shifted rows, bordered by the ln unknown (:609-617)
    if (i == 0) return (j == 0) ? 1.0 : 0.0;
    double v = dmat(a, 0, akv, nn, i - 1, j);
    if (j == 0) {
      if (i == 1) v += 4.0 / 3.0 / e2;
      if (i == 2) v -= 2.0 / 1.0 / e2 * exp(a.lognorm[0] - a.lognorm[1]);
      if (i == 3) v += 2.0 / 3.0 / e2 * exp(a.lognorm[0] - a.lognorm[2]);
    }
    return v;
  }
  double v = dmat(a, m, akv, nn, i, j);
  if (i == j) v += alpha;
  return v;
}

// Banded LU with partial pivoting (gbtrf semantics) on a sliding window held in registers: at
// column j only rows j..j+KL and columns j..j+KL+KU are live.  The finished U row (KL+KU+1 values)
// and its transformed right-hand side are streamed to the scratch band ([row][slot][system], so a
// warp writes consecutive addresses) and read back in reverse for the back substitution.
template <int KL, int KU>
__device__ void window_solve(const SolveArgs& a, int sys, int kind, bool special, int m, double akv, int nn,
                             double alpha, double e2, double2* __restrict__ x) {
  constexpr int WC = KL + KU + 1;     // window columns
  constexpr int SL = WC + 2;          // scratch slots per row: U row + complex rhs
  const size_t ns = a.nsys;
  double W[KL + 1][WC];
  double2 r[KL + 1];
#pragma unroll
  for (int t = 0; t <= KL; ++t) {
#pragma unroll
    for (int c = 0; c < WC; ++c) W[t][c] = sys_entry(a, kind, special, m, akv, nn, alpha, e2, t, c);
    r[t] = (t < nn) ? x[t] : make_double2(0.0, 0.0);
  }
  for (int j = 0; j < nn; ++j) {
    int km = min(KL, nn - 1 - j);
    // pivot: first row of maximal |a| among window rows 0..km
    int p = 0;
    double best = fabs(W[0][0]);
#pragma unroll
    for (int t = 1; t <= KL; ++t)
      if (t <= km && fabs(W[t][0]) > best) { best = fabs(W[t][0]); p = t; }
    if (best == 0.0) { atomicExch(a.status, 1); return; }
#pragma unroll
    for (int t = 1; t <= KL; ++t)
      if (t == p) {
#pragma unroll
        for (int c = 0; c < WC; ++c) { double q = W[0][c]; W[0][c] = W[t][c]; W[t][c] = q; }
        double2 q = r[0]; r[0] = r[t]; r[t] = q;
      }
    double rp = 1.0 / W[0][0];
#pragma unroll
    for (int t = 1; t <= KL; ++t)
      if (t <= km) {
        double l = W[t][0] * rp;
#pragma unroll
        for (int c = 1; c < WC; ++c) W[t][c] -= l * W[0][c];
        r[t].x -= l * r[0].x;
        r[t].y -= l * r[0].y;
      }
    // stream out U row j (its diagonal as the reciprocal) and its right-hand side
    a.ws[((size_t)j * SL) * ns + sys] = rp;
#pragma unroll
    for (int c = 1; c < WC; ++c) a.ws[((size_t)j * SL + c) * ns + sys] = W[0][c];
    a.ws[((size_t)j * SL + WC) * ns + sys] = r[0].x;
    a.ws[((size_t)j * SL + WC + 1) * ns + sys] = r[0].y;
    // slide the window by one row and one column; the new last row enters unreduced
#pragma unroll
    for (int t = 0; t < KL; ++t) {
#pragma unroll
      for (int c = 0; c < WC - 1; ++c) W[t][c] = W[t + 1][c + 1];
      W[t][WC - 1] = 0.0;
      r[t] = r[t + 1];
    }
    int nr_ = j + 1 + KL;
#pragma unroll
    for (int c = 0; c < WC; ++c) W[KL][c] = sys_entry(a, kind, special, m, akv, nn, alpha, e2, nr_, j + 1 + c);
    r[KL] = (nr_ < nn) ? x[nr_] : make_double2(0.0, 0.0);
  }
  // back substitution with U (bandwidth KL+KU), x(j+1..j+KL+KU) kept in registers
  double2 xs[WC - 1];
#pragma unroll
  for (int c = 0; c < WC - 1; ++c) xs[c] = make_double2(0.0, 0.0);
  for (int j = nn - 1; j >= 0; --j) {
    double2 acc;
    acc.x = a.ws[((size_t)j * SL + WC) * ns + sys];
    acc.y = a.ws[((size_t)j * SL + WC + 1) * ns + sys];
#pragma unroll
    for (int c = 1; c < WC; ++c) {
      double u = a.ws[((size_t)j * SL + c) * ns + sys];
      acc.x -= u * xs[c - 1].x;
      acc.y -= u * xs[c - 1].y;
    }
    double rd = a.ws[((size_t)j * SL) * ns + sys];
    double2 xj = make_double2(acc.x * rd, acc.y * rd);
    x[j] = xj;
#pragma unroll
    for (int c = WC - 2; c >= 1; --c) xs[c] = xs[c - 1];
    xs[0] = xj;
  }
}

// ------------------------------------------------------------------------------------------------
// Factor cache.  The matrix of system (m, k) depends only on (kind, alpha, m, k), and the steppers
// call ihelm with the same alpha every step (and vec2tp calls idel2), so the LU factors are computed
// once per key and every later call is a forward and a back substitution.  Per row j the cache
// holds, [row][slot][system] so that a warp reads consecutive addresses:
//   slot 0..KL-1     multipliers l(j+1..j+KL) (0 beyond the matrix)
//   slot KL          pivot row offset p in 0..KL (gbtrf's ipiv(j) - j)
//   slot KL+1        1 / U(j, j)
//   slot KL+2 ..     U(j, j+1 .. j+KL+KU)
constexpr int FKL = 2, FKU = 2, FSL = 2 * FKL + FKU + 2;

__global__ void __launch_bounds__(32) k_band_factor(SolveArgs a, double* __restrict__ fac) {
  int sys = blockIdx.x * blockDim.x + threadIdx.x;   // position in the system order (sys_mk)
  if (sys >= a.nsys) return;
  int m, k;
  if (!sys_mk(a, sys, m, k)) return;
  int nn = max(min(a.nrc, a.nrc - m), 0);
  if (m >= a.npc || nn < 1 || k_count(k, a.nzc, a.nzcu, a.nzdim) == 0) return;
  bool special = (m == 0 && k == 0) && a.kind == 1;
  double akv = a.ak[k];
  double alpha = (a.kind == 0) ? a.alpha : 0.0;
  double e2 = a.ell * a.ell;
  constexpr int WC = FKL + FKU + 1;
  const size_t ns = a.nsp;
  double W[FKL + 1][WC];
#pragma unroll
  for (int t = 0; t <= FKL; ++t)
#pragma unroll
    for (int c = 0; c < WC; ++c) W[t][c] = sys_entry(a, a.kind, special, m, akv, nn, alpha, e2, t, c);
  for (int j = 0; j < nn; ++j) {
    int km = min(FKL, nn - 1 - j);
    int p = 0;
    double best = fabs(W[0][0]);
#pragma unroll
    for (int t = 1; t <= FKL; ++t)
      if (t <= km && fabs(W[t][0]) > best) { best = fabs(W[t][0]); p = t; }
    if (best == 0.0) { atomicExch(a.status, 1); return; }
    if (p != 0 && a.pivflag) atomicOr(&a.pivflag[sys >> 5], 1);
#pragma unroll
    for (int t = 1; t <= FKL; ++t)
      if (t == p) {
#pragma unroll
        for (int c = 0; c < WC; ++c) { double q = W[0][c]; W[0][c] = W[t][c]; W[t][c] = q; }
      }
    double rp = 1.0 / W[0][0];
    double* f = fac + (size_t)j * FSL * ns + sys;
#pragma unroll
    for (int t = 1; t <= FKL; ++t) {
      double l = 0.0;
      if (t <= km) {
        l = W[t][0] * rp;
#pragma unroll
        for (int c = 1; c < WC; ++c) W[t][c] -= l * W[0][c];
      }
      f[(t - 1) * ns] = l;
    }
    f[FKL * ns] = (double)p;
    f[(FKL + 1) * ns] = rp;
    // U(j, j+c) / U(j, j): the back substitution then has one dependent FMA per row
#pragma unroll
    for (int c = 1; c < WC; ++c) f[(FKL + 1 + c) * ns] = W[0][c] * rp;
#pragma unroll
    for (int t = 0; t < FKL; ++t) {
#pragma unroll
      for (int c = 0; c < WC - 1; ++c) W[t][c] = W[t + 1][c + 1];
      W[t][WC - 1] = 0.0;
    }
    int nr_ = j + 1 + FKL;
#pragma unroll
    for (int c = 0; c < WC; ++c) W[FKL][c] = sys_entry(a, a.kind, special, m, akv, nn, alpha, e2, nr_, j + 1 + c);
  }
}

// cp.async helpers: 16 bytes through L2 only (the staged rows include rows that other threads of the
// block have just stored; a zero source size fills the destination with zeros)
__device__ __forceinline__ void cpa16cg(void* sdst, const void* gsrc, bool pred) {
  unsigned d = (unsigned)__cvta_generic_to_shared(sdst);
  int sz = pred ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gsrc), "r"(sz));
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cpa_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// forward and back substitution with the cached factors (gbtrs 'N', one or two right-hand sides), in
// place on the column.  One warp = 32 systems; factor rows and right-hand-side values are staged into shared
// memory SST groups ahead of use by cp.async, so DRAM latency overlaps the recurrences.
constexpr int SGR = 8, SST = 4, SNU = FKL + FKU, SFS = SNU + 1;
static_assert(FKL == 2, "the substitution compares the pivot index by the high words of 1.0 and 2.0");
template <int NR>
struct SubstSmem {
  double f[SST][SFS][SGR][32];   // factor rows by group: [slot][row in group][system]
  double2 v[NR][SST][SGR][32];   // field rows by group: fwd the entering rows, bwd y(j)
  double2 o[NR][2][SGR][32];     // outgoing rows by group parity: fwd y(j), bwd x(j)
  long long off[32];             // the block's systems: column offset, active rows, passes
  int nn[32], cnt[32];
};

// ihelm's pre-solve log-term handling of one field (:818-824): so%ln = s%ln/alpha, the log terms on
// e(1..3, 1, 1)
__device__ __forceinline__ void subst_root_pre(const SolveArgs& a, double2* g, double* lnp) {
  double e2 = a.ell * a.ell;
  double lno = *lnp / a.alpha;
  *lnp = lno;
  g[0].x -= 4.0 / 3.0 / e2 / exp(a.lognorm[0]) * lno;
  g[1].x += 2.0 / 1.0 / e2 / exp(a.lognorm[1]) * lno;
  g[2].x -= 2.0 / 3.0 / e2 / exp(a.lognorm[2]) * lno;
}

// The matrices are real, so the real and imaginary parts of a right-hand side are two independent
// real systems with the same factors.  A block takes 32 consecutive systems (m, k) and has 64*NR
// threads: one per system, part (real / imaginary) and field (NR = 2 solves the psi and chi fields of
// a vortex step with the same matrices).  The systems' serial recurrences are all the parallelism
// there is (a few warps per SM), so the kernel is built to issue few instructions per row: the
// factors and field rows are staged by groups of SGR rows with 16-byte copies shared by the whole
// block (the factors laid out [row][slot][system], a field's rows 128-byte runs per system), the
// outgoing rows go back the same way, and the rows are walked by absolute index with no early exit
// (rows past a system's own count are computed on whatever was staged and never stored; in the
// backward pass they keep the recurrence at zero until the system's last row).  Only the real-part
// thread of system (0,0) touches ln and the log terms, which all act on real parts.
template <int NR>
__global__ void __launch_bounds__(64 * NR) k_band_subst(SolveArgs a, const double* __restrict__ fac) {
  typedef double R;
  constexpr int NT = 64 * NR;
  extern __shared__ __align__(16) unsigned char subst_smem[];
  SubstSmem<NR>& sm = *reinterpret_cast<SubstSmem<NR>*>(subst_smem);
  const int th = threadIdx.x, q = th >> 6, comp = (th >> 5) & 1, lane = th & 31;
  const size_t nsp = a.nsp;
  const int sys0 = blockIdx.x * 32, sys = sys0 + lane;
  double2* ev = q == 0 ? a.e : a.e2;
  double* lv = q == 0 ? a.lnp : a.lnp2;
  auto sys_info = [&](int s, int& nn, int& cnt, size_t& off) {
    bool valid = s < a.nsys;
    int m = 0, k = 0;
    if (valid) valid = sys_mk(a, s, m, k);
    cnt = valid ? k_count(k, a.nzc, a.nzcu, a.nzdim) : 0;
    nn = max(min(a.nrc, a.nrc - m), 0);
    if (valid && m == 0 && k == 0 && a.skip_root) cnt = 0;
    if (!valid || m >= a.npc || nn < 1) cnt = 0;
    off = (size_t)a.nrdim * (m + (size_t)a.npdim * k);
  };
  int nn, cnt;
  size_t off;
  sys_info(sys, nn, cnt, off);
  if (th < 32) { sm.nn[th] = nn; sm.cnt[th] = cnt; sm.off[th] = (long long)off; }
  const bool root = sys < a.nsys && off == 0;
  if (root && comp == 0 && a.kind == 0 && !a.skip_root && !a.no_ln) subst_root_pre(a, ev, lv);
  double* x = reinterpret_cast<double*>(ev + off) + comp;   // stride 2
  // every warp holds the same 32 systems: warp-wide maxima are block-wide
  int nnw = (cnt > 0) ? nn : 0;
  for (int o = 16; o; o >>= 1) nnw = max(nnw, __shfl_xor_sync(0xffffffffu, nnw, o));
  int cntw = cnt;
  for (int o = 16; o; o >>= 1) cntw = max(cntw, __shfl_xor_sync(0xffffffffu, cntw, o));
  const int ng = (nnw + SGR - 1) / SGR;
  const double* dummy = fac;   // a 256-byte aligned address for the zero-size copies
  __syncthreads();             // the system table
  // the block's field rows of a group: chunk c = th + i*NT -> field c/256, system (c%256)/8, row in
  // group c%8 (eight consecutive threads copy one system's 128-byte run); each thread's four chunks
  // keep their system for the whole kernel
  constexpr int NCH = NR * 256 / NT;   // 4
  double2* cbase[NCH];
  int cnn[NCH], ccnt[NCH];
  const int cu = th & 7;
#pragma unroll
  for (int i = 0; i < NCH; ++i) {
    const int c = th + i * NT, qq = c >> 8, sl = (c >> 3) & 31;
    cbase[i] = (qq == 0 ? a.e : a.e2) + sm.off[sl];
    cnn[i] = sm.nn[sl];
    ccnt[i] = sm.cnt[sl];
  }
  auto stage_rows = [&](int g, int rep, bool bwd) {
    const int st = g % SST;
#pragma unroll
    for (int i = 0; i < NCH; ++i) {
      const int c = th + i * NT, qq = c >> 8, sl = (c >> 3) & 31;
      const int j = bwd ? nnw - 1 - (g * SGR + cu) : g * SGR + cu + 1 + FKL;
      const bool ok = rep < ccnt[i] && j >= 0 && j < cnn[i];
      cpa16cg(&sm.v[qq][st][cu][sl], ok ? (const void*)(cbase[i] + j) : (const void*)dummy, ok);
    }
  };
  auto write_out = [&](int g, int rep, bool bwd) {
#pragma unroll
    for (int i = 0; i < NCH; ++i) {
      const int c = th + i * NT, qq = c >> 8, sl = (c >> 3) & 31;
      const int j = bwd ? nnw - 1 - (g * SGR + cu) : g * SGR + cu;
      if (rep < ccnt[i] && j >= 0 && j < cnn[i]) cbase[i][j] = sm.o[qq][g & 1][cu][sl];
    }
  };
  // the factor rows of group g: NSL slots from S0 of rows j(u), 256 bytes per (row, slot), 16 per copy
  // (backward without row exchanges: 1/U(j,j) and the FKU entries of U's own band only)
  const double* fbase = fac + sys0 + 2 * (th & 15);
  auto stage_fac_t = [&](auto bwdc, auto npc, int g) {
    constexpr bool BWD = decltype(bwdc)::value, NP = decltype(npc)::value;
    constexpr int NSL = BWD ? (NP ? FKU + 1 : SNU + 1) : (NP ? FKL : FKL + 1), S0 = BWD ? FKL + 1 : 0;
    const int st = g % SST;
#pragma unroll
    for (int c = th; c < SGR * NSL * 16; c += NT) {
      const int pr = c >> 4;
      const int u = pr / NSL, t = pr - u * NSL;
      const int j = BWD ? nnw - 1 - (g * SGR + u) : g * SGR + u;
      const bool ok = j >= 0 && j < nnw;
      cpa16cg(&sm.f[st][t][u][2 * (th & 15)], ok ? (const void*)(fbase + ((size_t)j * FSL + S0 + t) * nsp) : (const void*)dummy, ok);
    }
  };
  // the factorisation records, per 32 systems, whether any of them exchanges rows; a block whose systems
  // never do runs the forward pass without the pivot slot and the exchanges (the same result bit for bit)
  const bool blk_nopiv = a.pivflag != nullptr && __ldcg(&a.pivflag[blockIdx.x]) == 0;
  for (int rep = 0; rep < cntw; ++rep) {
    // ---- forward: L y = P b, y(j) into the field's slot of row j ----
    R r[FKL + 1];
    bool piv = false;   // a row exchange in one of this thread's staged rows
#pragma unroll
    for (int t = 0; t <= FKL; ++t) r[t] = ((rep < cnt && t < nn) ? __ldcg(x + 2 * t) : 0.0);
    auto forward = [&](auto npc) {
      constexpr bool NP = decltype(npc)::value;
      auto stage_f = [&](int g) { stage_fac_t(std::integral_constant<bool, false>(), npc, g); };
      for (int g = 0; g < SST - 1; ++g) { if (g < ng) { stage_f(g); stage_rows(g, rep, false); } cpa_commit(); }
      for (int g = 0; g < ng; ++g) {
        cpa_wait<SST - 2>();
        __syncthreads();   // group g staged; group g-1 computed; stage (g-1)%SST free
        if (g + SST - 1 < ng) { stage_f(g + SST - 1); stage_rows(g + SST - 1, rep, false); }
        cpa_commit();
        if (g > 0) write_out(g - 1, rep, false);
        const int st = g % SST;
#pragma unroll
        for (int u = 0; u < SGR; ++u) {
          if constexpr (!NP) {
            // the pivot row index p (0..FKL), stored as a double: compared by its high word, off the FP64 pipe
            const int ph = __double2hiint(sm.f[st][FKL][u][lane]);
            piv = piv || ph != 0;
#pragma unroll
            for (int t = 1; t <= FKL; ++t)
              if (ph == (t == 1 ? 0x3FF00000 : 0x40000000)) { R w = r[0]; r[0] = r[t]; r[t] = w; }
          }
#pragma unroll
          for (int t = 1; t <= FKL; ++t) r[t] = fma(-sm.f[st][t - 1][u][lane], r[0], r[t]);
          reinterpret_cast<double*>(&sm.o[q][g & 1][u][lane])[comp] = r[0];
#pragma unroll
          for (int t = 0; t < FKL; ++t) r[t] = r[t + 1];
          r[FKL] = reinterpret_cast<const double*>(&sm.v[q][st][u][lane])[comp];
        }
      }
    };
    if (blk_nopiv) forward(std::integral_constant<bool, true>());
    else forward(std::integral_constant<bool, false>());
    cpa_wait<0>();
    __syncthreads();
    if (ng > 0) write_out(ng - 1, rep, false);
    __threadfence_block();
    __syncthreads();   // y(j) in the fields, read back below by other threads' copies
    // ---- backward: U x = y from row nnw-1 down; a system joins at its own last row.  Without a row
    // exchange in any of the block's systems (every forward pass saw pivot offset 0), U keeps the
    // matrix's own FKU superdiagonals and its fill-in entries are exact zeros: the pass then stages and
    // applies only those (1 / U(j,j) and FKU ratios), with the same result bit for bit, since
    // fma(-0, x, t) = t for finite x.
    const bool nopiv = !__syncthreads_or(piv);
    auto backward = [&](auto npc) {
      constexpr bool NP = decltype(npc)::value;
      constexpr int NU = NP ? FKU : SNU;
      auto stage_b = [&](int g) { stage_fac_t(std::integral_constant<bool, true>(), npc, g); };
      R xs[SNU];
#pragma unroll
      for (int c = 0; c < SNU; ++c) xs[c] = 0.0;
      for (int g = 0; g < SST - 1; ++g) { if (g < ng) { stage_b(g); stage_rows(g, rep, true); } cpa_commit(); }
      for (int g = 0; g < ng; ++g) {
        cpa_wait<SST - 2>();
        __syncthreads();
        if (g + SST - 1 < ng) { stage_b(g + SST - 1); stage_rows(g + SST - 1, rep, true); }
        cpa_commit();
        if (g > 0) write_out(g - 1, rep, true);
        const int st = g % SST;
#pragma unroll
        for (int u = 0; u < SGR; ++u) {
          const int j = nnw - 1 - (g * SGR + u);
          const R f0 = sm.f[st][0][u][lane];
          // x(j) = y(j)/U(j,j) - sum_c (U(j,j+c)/U(j,j)) x(j+c): only the last FMA waits on x(j+1)
          const R yj = reinterpret_cast<const double*>(&sm.v[q][st][u][lane])[comp];
          R t = yj * f0;
#pragma unroll
          for (int c = 2; c <= NU; ++c) t = fma(-sm.f[st][c][u][lane], xs[c - 1], t);
          R xj = fma(-sm.f[st][1][u][lane], xs[0], t);
          if (j >= nn) xj = 0.0;
          reinterpret_cast<double*>(&sm.o[q][g & 1][u][lane])[comp] = xj;
#pragma unroll
          for (int c = SNU - 1; c >= 1; --c) xs[c] = xs[c - 1];
          xs[0] = xj;
        }
      }
    };
    if (nopiv) backward(std::integral_constant<bool, true>());
    else backward(std::integral_constant<bool, false>());
    cpa_wait<0>();
    __syncthreads();
    if (ng > 0) write_out(ng - 1, rep, true);
    __threadfence_block();
    __syncthreads();   // x complete before the next pass (or the log-term read below)
  }
  if (root && comp == 0 && a.kind == 1 && !a.skip_root && !a.no_ln && cnt > 0) *lv = __ldcg(x) * exp(a.lognorm[0]);
}

// the bordered (0,0) system of idel2_preln (KL = 3), single thread, after the batch
__global__ void k_band_solve_special(SolveArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int nn = max(a.nrc, 0);
  if (a.npc < 1 || nn < 1) return;
  int cnt = k_count(0, a.nzc, a.nzcu, a.nzdim);
  if (cnt == 0) return;
  double e2 = pow(a.ell, 2.0);
  double2* x = a.e;
  for (int i = nn - 1; i >= 1; --i) x[i] = x[i - 1];
  x[0] = make_double2(a.preln / exp(a.lognorm[0]), 0.0);
  SolveArgs b = a;
  b.nsys = 1;   // scratch rows of this single system are contiguous
  for (int rep = 0; rep < cnt; ++rep) window_solve<3, 2>(b, 0, 2, true, 0, a.ak[0], nn, 0.0, e2, x);
  *a.lnp = x[0].x * exp(a.lognorm[0]);
}

// ihelmp's log-term pre-step (mlegs_scalar_ops.f90:937-951): ln <- ln/alpha, then
// e(:nrc,1,1) -= D(0,0)^(q-1) bl2 + beta bl2 with bl2 = (4/3, -2, 2/3)/ell^2/exp(lognorm) * ln.
__global__ void k_ihelmp_pre(double2* __restrict__ e, double* __restrict__ lnp, const double* __restrict__ bd2,
                             const double* __restrict__ ak, const double* __restrict__ lognorm, double* __restrict__ tmp,
                             int nrc, int ne, int power, double alpha, double beta, double ell) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double lno = *lnp / alpha;
  *lnp = lno;
  double e2 = pow(ell, 2.0);
  double* bl = tmp;
  double* bl2 = tmp + nrc;
  double* t = tmp + 2 * nrc;
  for (int i = 0; i < nrc; ++i) bl2[i] = 0.0;
  bl2[0] = 4.0 / 3.0 / e2 / exp(lognorm[0]) * lno;
  if (nrc > 1) bl2[1] = -2.0 / e2 / exp(lognorm[1]) * lno;
  if (nrc > 2) bl2[2] = 2.0 / 3.0 / e2 / exp(lognorm[2]) * lno;
  for (int i = 0; i < nrc; ++i) bl[i] = bl2[i];
  double akv = ak[0];
  for (int n = 1; n <= power / 2 - 1; ++n) {
    for (int i = 0; i < nrc; ++i) {
      double acc = 0.0;
      for (int j = max(0, i - 2); j <= min(nrc - 1, i + 2); ++j) {
        int c = j - i + 2;
        double v = bd2[c + 5 * ((size_t)i + (size_t)ne * 0)];
        if (c == 2) v = v - pow(akv, 2.0);
        acc += v * bl[j];
      }
      t[i] = acc;
    }
    for (int i = 0; i < nrc; ++i) bl[i] = t[i];
  }
  for (int i = 0; i < nrc; ++i) e[i].x -= bl[i] + beta * bl2[i];
}

int launch_ihelmp_pre(Scalar& s, const ChopIdx& c, int power, double alpha, double beta) {
  if (3 * c.nrc > 2 * 4096) return set_error(MLG_ESIZE, "ihelmp: nrc too large for the log-term workspace");
  k_ihelmp_pre<<<1, 32, 0, G.stream>>>(s.e, s.ln, G.bd2, G.ak, G.lognorm, G.dscal + DS_CALC, c.nrc, G.ne, power, alpha,
                                       beta, G.ell);
  MLG_LAUNCH();
  return 0;
}

// ------------------------------------------------------------------------------------------------
// Helmholtz solve that allocates nothing (mlg_ihelm_noalloc).
//
// Some callers cannot let a library call cudaMalloc: Fortran or C hosts whose own device allocator
// or fixed arena owns all GPU memory (an extra cudaMalloc would fail or fragment it), and codes that
// forbid device allocation inside their time-stepping loop.  For them this variant of the ihelm
// solve keeps its only workspace (the U rows of the on-the-fly band LU) in the fixed-size device
// array below, present on every GPU that loads the library until the process exits.  Systems are
// processed in batches that fit it, so any grid size works; a single system larger than the array
// is rejected.  All calls share the array: calls that overlap on the GPU (other streams, other host
// threads) race on it.  Every word a launch reads was written earlier by the same launch, so nothing
// needs clearing between calls.
constexpr size_t NOALLOC_DOUBLES = 2u << 20;   // 16 MiB
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

__global__ void __launch_bounds__(32) k_ihelm_noalloc(SolveArgs a, int s0, int batch, double lno) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  int sys = s0 + b;
  if (b >= batch || sys >= a.nsys) return;
  int m = sys / a.nzdim, k = sys % a.nzdim;
  int cnt = k_count(k, a.nzc, a.nzcu, a.nzdim);
  int nn = max(min(a.nrc, a.nrc - m), 0);
  double e2 = a.ell * a.ell;
  if (sys == 0) {   // so%ln = s%ln/alpha is lno; its log terms on e(1..3,1,1) (:818-824)
    double2* g = a.e;
    g[0].x -= 4.0 / 3.0 / e2 / exp(a.lognorm[0]) * lno;
    g[1].x += 2.0 / 1.0 / e2 / exp(a.lognorm[1]) * lno;
    g[2].x -= 2.0 / 3.0 / e2 / exp(a.lognorm[2]) * lno;
  }
  if (m >= a.npc || nn < 1 || cnt == 0) return;
  double2* x = a.e + (size_t)a.nrdim * (m + (size_t)a.npdim * k);
  SolveArgs w = a;
  w.nsys = batch;   // scratch rows are laid out [row][slot][batch]
  for (int rep = 0; rep < cnt; ++rep) window_solve<2, 2>(w, b, 0, false, m, a.ak[k], nn, a.alpha, e2, x);
}

// per-device address of g_noalloc_scratch, looked up on the first call made with that device current
static double* g_noalloc_ptr[64] = {nullptr};

int ihelm_noalloc(void* e_dev, double* ln, double alpha) {
  int dev = 0;
  MLG_CUDA(cudaGetDevice(&dev));
  if (dev != G.device)
    return set_error(MLG_EPARAM, "ihelm_noalloc: the current CUDA device is not the one the kit was built on");
  if (dev < 0 || dev >= 64) return set_error(MLG_ESIZE, "ihelm_noalloc: device index beyond 63");
  if (!g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return set_error(MLG_ECUDA, std::string("ihelm_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_ptr[dev] = (double*)ptr;
  }
  if (std::fabs(alpha) < 5.0e-14)
    return set_error(MLG_EALPHA, "ihelm: alpha equals to zero. Inversion of 0*identity is impossible");
  int nrc = G.nrchop, npc = G.npchop;
  int nnmax = std::max(std::min(nrc, G.nrdim), 1);
  constexpr int SL = 2 + 2 + 1 + 2;   // U row (5) + complex right-hand side (2), as in window_solve<2,2>
  size_t per_sys = (size_t)nnmax * SL;
  size_t batch = NOALLOC_DOUBLES / per_sys;
  if (batch < 1)
    return set_error(MLG_ESIZE, "ihelm_noalloc: one radial system (" + std::to_string(nnmax) +
                                    " rows) exceeds the fixed 16 MiB workspace");
  size_t nsys = (size_t)npc * G.nzdim;
  double lno = *ln / alpha;
  SolveArgs a;
  std::memset(&a, 0, sizeof(a));
  a.e = (double2*)e_dev; a.ws = g_noalloc_ptr[dev]; a.lnp = nullptr; a.bd2 = G.bd2; a.ak = G.ak; a.lognorm = G.lognorm;
  a.status = (int*)(G.dscal + DS_FLAG + 1);
  a.nrdim = G.nrdim; a.npdim = G.npdim; a.ne = G.ne; a.nrc = nrc; a.npc = npc; a.nzc = G.chopzl; a.nzcu = G.chopzu;
  a.nzdim = G.nzdim; a.nsys = (int)nsys; a.alpha = alpha; a.ell = G.ell; a.kind = 0;
  for (size_t s0 = 0; s0 < nsys; s0 += batch) {
    int nb = (int)std::min(batch, nsys - s0);
    k_ihelm_noalloc<<<cdiv(nb, 32), 32, 0, G.stream>>>(a, (int)s0, nb, lno);
    MLG_LAUNCH();
  }
  *ln = lno;
  return 0;
}

// the positions of the cached-factor system order (sys_mk) for a's chop window: sets lead, nsys and nsp
static size_t set_positions(SolveArgs& a) {
  const int klo = std::max(a.nzcu, 1) - 1, khi = std::min(a.nzdim, a.nzc) - 1;
  const size_t nd = (size_t)std::max(khi - klo + 1, 0);
  a.lead = (int)(((size_t)std::max(a.npc, 0) * nd + 31) / 32 * 32);
  const size_t n = (size_t)a.lead + (size_t)std::max(a.npc, 1) * a.nzdim;
  a.nsys = (int)n;
  a.nsp = (int)((n + 31) / 32 * 32);
  return n;
}

// LRU cache of factor sets, keyed by (kind, alpha, chop window)
struct LUEntry {
  int kind; double alpha; int nrc, npc, nzc, nzcu; double* buf; size_t bytes; unsigned long long used;
};
static std::vector<LUEntry> g_lu;
static unsigned long long g_lu_clock = 0;
static const size_t LU_MAX_ENTRIES = 4;

void lu_cache_clear() {
  for (auto& e : g_lu) dfree(e.buf, e.bytes);
  g_lu.clear();
}

// the factors' per-32-system row-exchange flags follow the factor rows in the cache entry
static size_t lu_flag_offset(int nrc, size_t nsp) {
  const int nnmax = std::max(std::min(nrc, G.nrdim), 1);
  return (size_t)nnmax * FSL * nsp;
}
static int* lu_flags(double* buf, int nrc, size_t nsp) { return (int*)(buf + lu_flag_offset(nrc, nsp)); }

// the cached factors of (kind, alpha, chop window), laid out [row][slot][system] with system stride
// nsp, then nsp/32 row-exchange flags; made by factor() on a miss
template <class F>
static int lu_cache_get(int kind, double alpha, const ChopIdx& c, size_t nsp, double** out, F factor) {
  for (auto& e : g_lu)
    if (e.kind == kind && e.alpha == alpha && e.nrc == c.nrc && e.npc == c.npc && e.nzc == c.nzc && e.nzcu == c.nzcu) {
      e.used = ++g_lu_clock;
      *out = e.buf;
      return 0;
    }
  size_t bytes = lu_flag_offset(c.nrc, nsp) * sizeof(double) + (nsp / 32) * sizeof(int);
  if (g_lu.size() >= LU_MAX_ENTRIES) {
    auto it = std::min_element(g_lu.begin(), g_lu.end(), [](const LUEntry& x, const LUEntry& y) { return x.used < y.used; });
    dfree(it->buf, it->bytes);
    g_lu.erase(it);
  }
  LUEntry e{kind, alpha, c.nrc, c.npc, c.nzc, c.nzcu, nullptr, bytes, ++g_lu_clock};
  MLG_TRY(dmalloc((void**)&e.buf, bytes));
  // rows past a system's own count (and systems outside the chop) stay zero: pivot offset 0, so a
  // block's substitution can take its no-exchange paths; the flags start at zero
  MLG_CUDA(cudaMemsetAsync(e.buf, 0, bytes, G.stream));
  MLG_TRY(factor(e.buf));
  g_lu.push_back(e);
  *out = e.buf;
  return 0;
}

// the substitution launch: 64*NR threads per 32 systems
template <int NR>
static int launch_subst(const SolveArgs& a, const double* fac, size_t nsys) {
  size_t smb = sizeof(SubstSmem<NR>);
  MLG_CUDA(cudaFuncSetAttribute(k_band_subst<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb));
  k_band_subst<NR><<<cdiv(nsys, 32), 64 * NR, smb, G.stream>>>(a, fac);
  MLG_LAUNCH();
  return 0;
}
// kind as in SolveArgs; the band scratch grows to fit (kl, ku)
// algorithmic bytes of one substitution pass over nrhs fields: each field read and written once, the
// cached factors (FSL doubles per row and system) read once
static double solve_bytes(int nrhs, const ChopIdx& c) {
  double nsys = (double)std::max(c.npc, 1) * G.nzdim;
  double rows = std::max(std::min(c.nrc, G.nrdim), 1);
  return 2.0 * nrhs * G.fsize * 16 + rows * FSL * nsys * 8;
}

int launch_band_solve(Scalar& s, int kind, const ChopIdx& c, double alpha, double beta, double preln, int power) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  int kl = 2, ku = 2;
  if (kind == 2) kl = 3;
  if (kind == 3) { kl = power; ku = power; }
  int W = std::max(2 * kl + ku + 1, kl + ku + 3);
  int npc = std::max(c.npc, 1);
  size_t nsys = (size_t)npc * G.nzdim;
  int nnmax = std::max(std::min(c.nrc, G.nrdim), 1);
  size_t need = (size_t)nnmax * W * nsys * sizeof(double);
  if (need > G.band_ws_bytes) {
    if (G.band_ws) dfree(G.band_ws, G.band_ws_bytes);
    G.band_ws = nullptr;
    G.band_ws_bytes = 0;
    MLG_TRY(dmalloc((void**)&G.band_ws, need));
    G.band_ws_bytes = need;
  }
  SolveArgs a;
  a.e = s.e; a.ws = G.band_ws; a.lnp = s.ln; a.bd2 = G.bd2; a.ak = G.ak; a.lognorm = G.lognorm;
  a.status = (int*)(G.dscal + DS_FLAG + 1);
  a.nrdim = G.nrdim; a.npdim = G.npdim; a.ne = G.ne; a.nrc = c.nrc; a.npc = c.npc; a.nzc = c.nzc; a.nzcu = c.nzcu;
  a.nzdim = G.nzdim; a.nsys = (int)nsys; a.alpha = alpha; a.beta = beta; a.ell = G.ell; a.preln = preln;
  a.kind = kind; a.power = power; a.skip_root = 0; a.transpose = 0; a.no_ln = 0;
  kt_begin(KT_SOLVE);
  if (kind == 3) {
    k_band_solve<<<cdiv(nsys, 64), 64, 0, G.stream>>>(a);
    MLG_LAUNCH();
  } else {
    // kinds 0 and 1 (and the batch of kind 2): cached factors, substitution only; the bordered
    // (0,0) system of kind 2 is skipped by the batch and solved on its own afterwards
    int fkind = (kind == 2) ? 1 : kind;
    double* fac = nullptr;
    SolveArgs b = a;
    b.kind = fkind;
    b.skip_root = (kind == 2) ? 1 : 0;
    const size_t npos = set_positions(b);
    MLG_TRY(lu_cache_get(fkind, alpha, c, (size_t)b.nsp, &fac, [&](double* buf) -> int {
      SolveArgs fa = b;
      fa.pivflag = lu_flags(buf, b.nrc, (size_t)b.nsp);
      k_band_factor<<<cdiv(npos, 32), 32, 0, G.stream>>>(fa, buf);
      MLG_LAUNCH();
      return 0;
    }));
    b.pivflag = lu_flags(fac, b.nrc, (size_t)b.nsp);
    MLG_TRY(launch_subst<1>(b, fac, npos));
    if (kind == 2) {
      k_band_solve_special<<<1, 32, 0, G.stream>>>(a);
      MLG_LAUNCH();
    }
  }
  kt_end(KT_SOLVE, solve_bytes(1, c));
  return 0;
}

// ------------------------------------------------------------------------------------------------
// ihelm of two fields with the same chop window and alpha in one substitution pass (the psi and chi
// solves of a vortex step): the factors are read once for both.  Results are those of two ihelm calls.
int launch_ihelm_pair(Scalar& s1, Scalar& s2, const ChopIdx& c, double alpha) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  int npc = std::max(c.npc, 1);
  size_t nsys = (size_t)npc * G.nzdim;
  SolveArgs a;
  a.e = s1.e; a.ws = G.band_ws; a.lnp = s1.ln; a.bd2 = G.bd2; a.ak = G.ak; a.lognorm = G.lognorm;
  a.status = (int*)(G.dscal + DS_FLAG + 1);
  a.nrdim = G.nrdim; a.npdim = G.npdim; a.ne = G.ne; a.nrc = c.nrc; a.npc = c.npc; a.nzc = c.nzc; a.nzcu = c.nzcu;
  a.nzdim = G.nzdim; a.nsys = (int)nsys; a.alpha = alpha; a.beta = 0.0; a.ell = G.ell; a.preln = 0.0;
  a.kind = 0; a.power = 0; a.skip_root = 0; a.transpose = 0; a.no_ln = 0;
  a.e2 = s2.e; a.lnp2 = s2.ln;
  kt_begin(KT_SOLVE);
  double* fac = nullptr;
  const size_t npos = set_positions(a);
  MLG_TRY(lu_cache_get(0, alpha, c, (size_t)a.nsp, &fac, [&](double* buf) -> int {
    SolveArgs fa = a;
    fa.pivflag = lu_flags(buf, a.nrc, (size_t)a.nsp);
    k_band_factor<<<cdiv(npos, 32), 32, 0, G.stream>>>(fa, buf);
    MLG_LAUNCH();
    return 0;
  }));
  a.pivflag = lu_flags(fac, a.nrc, (size_t)a.nsp);
  MLG_TRY(launch_subst<2>(a, fac, npos));
  kt_end(KT_SOLVE, solve_bytes(2, c));
  return 0;
}

// transposes for the adjoint: the band products in the precision of their forwards (FP64, or FP32
// for the mixed form's m >= 1 columns), the solves FP64 in both forms

// B^T applied cnt times to the rows [0, nn) of a column held in shared memory as U (in place in c0)
template <typename U>
__device__ __forceinline__ typename BC<U>::C* band_T_col(typename BC<U>::C* c0, typename BC<U>::C* c1,
                                                         const BandTabs& tb, int k, int op, int m, int ne, int nn,
                                                         int cnt) {
  typedef typename BC<U>::C C;
  const U akv2 = bakv2<U>(tb, k);
  for (int rep = 0; rep < cnt; ++rep) {
    for (int j = threadIdx.x; j < nn; j += blockDim.x) {
      C acc; acc.x = 0; acc.y = 0;
      if (op == 0) {
        if (j + 1 < nn) {
          U v = btab<U>(tb.bxx, tb.bxxf, 3 * ((size_t)(j + 1) + (size_t)ne * m) + 0);
          acc.x += v * c0[j + 1].x; acc.y += v * c0[j + 1].y;
        }
        if (j - 1 >= 0) {
          U v = btab<U>(tb.bxx, tb.bxxf, 3 * ((size_t)(j - 1) + (size_t)ne * m) + 2);
          acc.x += v * c0[j - 1].x; acc.y += v * c0[j - 1].y;
        }
      } else {
        for (int i = max(0, j - 2); i <= min(nn - 1, j + 2); ++i) {
          U v = btab<U>(tb.bd2, tb.bd2f, (j - i + 2) + 5 * ((size_t)i + (size_t)ne * m));
          if (i == j && op == 2) v -= akv2;
          acc.x += v * c0[i].x;
          acc.y += v * c0[i].y;
        }
      }
      c1[j] = acc;
    }
    __syncthreads();
    C* t = c0; c0 = c1; c1 = t;
  }
  return c0;
}

// k_band_apply^T: x <- B^T x per active column (cnt times, as the forward), rows >= nn and inactive
// columns untouched (the forward is the identity there).  The forward adds c_n * ln to Re e(n,0,0)
// after the product and zeroes ln, so the adjoint of ln is read off the incoming adjoint of e first:
// ln_bar = sum_n c_n Re(e_bar(n,0,0)); the adjoint of the output ln (a constant zero) is dropped.
template <typename T>
__global__ void k_band_apply_T(double2* __restrict__ e, BandTabs tb, double* __restrict__ lnp,
                               const double* __restrict__ lognorm, int op, int nrdim, int npdim, int ne, int nrc,
                               int npc, int nzc, int nzcu, int nzdim, double ell) {
  extern __shared__ __align__(16) unsigned char bandt_smem[];
  int m = blockIdx.y, k = blockIdx.x;
  int nn = max(min(nrc, nrc - m), 0);
  int cnt = k_count(k, nzc, nzcu, nzdim);
  double2* g = e + (size_t)nrdim * (m + (size_t)npdim * k);
  if (m == 0 && k == 0 && threadIdx.x == 0) {
    double e2 = ell * ell;
    if (op == 0) *lnp = g[0].x / exp(lognorm[0]) + g[1].x / exp(lognorm[1]);
    else *lnp = 4.0 / 3.0 / e2 / exp(lognorm[0]) * g[0].x - 2.0 / 1.0 / e2 / exp(lognorm[1]) * g[1].x +
                2.0 / 3.0 / e2 / exp(lognorm[2]) * g[2].x;
  }
  __syncthreads();
  if (m >= npc || nn <= 0 || cnt <= 0) return;
  if (m == 0 || sizeof(T) == sizeof(double)) {
    double2* c0 = (double2*)bandt_smem;
    double2* c1 = c0 + nrdim;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = g[i];
    __syncthreads();
    c0 = band_T_col<double>(c0, c1, tb, k, op, m, ne, nn, cnt);
    for (int i = threadIdx.x; i < nn; i += blockDim.x) g[i] = c0[i];
  } else {
    float2* c0 = (float2*)bandt_smem;
    float2* c1 = c0 + nrdim;
    for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = ld_c32(g + i);
    __syncthreads();
    c0 = band_T_col<float>(c0, c1, tb, k, op, m, ne, nn, cnt);
    for (int i = threadIdx.x; i < nn; i += blockDim.x) st_c32(g + i, c0[i]);
  }
}

int launch_band_apply_T(Scalar& s, int op, const ChopIdx& c) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  dim3 grid(G.nzdim, std::max(c.npc, 1));
  size_t sm = 2ull * G.nrdim * sizeof(double2);
  kt_begin(2);
  if (G.precision == MLG_MIXED) {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_band_apply_T<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_band_apply_T<float><<<grid, 128, sm, G.stream>>>(s.e, band_tabs(), s.ln, G.lognorm, op, G.nrdim, G.npdim, G.ne,
                                                       c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell);
  } else {
    if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_band_apply_T<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_band_apply_T<double><<<grid, 128, sm, G.stream>>>(s.e, band_tabs(), s.ln, G.lognorm, op, G.nrdim, G.npdim, G.ne,
                                                        c.nrc, c.npc, c.nzc, c.nzcu, G.nzdim, G.ell);
  }
  MLG_LAUNCH();
  kt_end(2, 2.0 * G.fsize * 16);
  return 0;
}

// A^T x = b for kind 0 (D(m,k) + alpha I) and kind 1 (idel2_proln: the root system with its
// column-1 log-term entries), all columns, no log-term handling; the factors of A^T are cached
// beside those of A.
int launch_band_solve_T(Scalar& s, int kind, const ChopIdx& c, double alpha) {
  if (kind != 0 && kind != 1) return set_error(MLG_EPARAM, "transposed band solve: kinds 0 and 1 only");
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  int npc = std::max(c.npc, 1);
  size_t nsys = (size_t)npc * G.nzdim;
  SolveArgs a;
  a.e = s.e; a.ws = G.band_ws; a.lnp = s.ln; a.bd2 = G.bd2; a.ak = G.ak; a.lognorm = G.lognorm;
  a.status = (int*)(G.dscal + DS_FLAG + 1);
  a.nrdim = G.nrdim; a.npdim = G.npdim; a.ne = G.ne; a.nrc = c.nrc; a.npc = c.npc; a.nzc = c.nzc; a.nzcu = c.nzcu;
  a.nzdim = G.nzdim; a.nsys = (int)nsys; a.alpha = alpha; a.beta = 0.0; a.ell = G.ell; a.preln = 0.0;
  a.kind = kind; a.power = 0; a.skip_root = 0; a.transpose = 1; a.no_ln = 1;
  kt_begin(KT_SOLVE);
  double* fac = nullptr;
  const size_t npos = set_positions(a);
  MLG_TRY(lu_cache_get(kind + 8, alpha, c, (size_t)a.nsp, &fac, [&](double* buf) -> int {
    SolveArgs fa = a;
    fa.pivflag = lu_flags(buf, a.nrc, (size_t)a.nsp);
    k_band_factor<<<cdiv(npos, 32), 32, 0, G.stream>>>(fa, buf);
    MLG_LAUNCH();
    return 0;
  }));
  a.pivflag = lu_flags(fac, a.nrc, (size_t)a.nsp);
  MLG_TRY(launch_subst<1>(a, fac, npos));
  kt_end(KT_SOLVE, solve_bytes(1, c));
  return 0;
}

// A^T x = b for kind 0 on two fields with the same chop window and alpha, in one substitution pass
// (the psi and chi solves of the adjoint step); results are those of two launch_band_solve_T calls
int launch_band_solve_T_pair(Scalar& s1, Scalar& s2, const ChopIdx& c, double alpha) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  int npc = std::max(c.npc, 1);
  size_t nsys = (size_t)npc * G.nzdim;
  SolveArgs a;
  a.e = s1.e; a.ws = G.band_ws; a.lnp = s1.ln; a.bd2 = G.bd2; a.ak = G.ak; a.lognorm = G.lognorm;
  a.status = (int*)(G.dscal + DS_FLAG + 1);
  a.nrdim = G.nrdim; a.npdim = G.npdim; a.ne = G.ne; a.nrc = c.nrc; a.npc = c.npc; a.nzc = c.nzc; a.nzcu = c.nzcu;
  a.nzdim = G.nzdim; a.nsys = (int)nsys; a.alpha = alpha; a.beta = 0.0; a.ell = G.ell; a.preln = 0.0;
  a.kind = 0; a.power = 0; a.skip_root = 0; a.transpose = 1; a.no_ln = 1;
  a.e2 = s2.e; a.lnp2 = s2.ln;
  kt_begin(KT_SOLVE);
  double* fac = nullptr;
  const size_t npos = set_positions(a);
  MLG_TRY(lu_cache_get(0 + 8, alpha, c, (size_t)a.nsp, &fac, [&](double* buf) -> int {
    SolveArgs fa = a;
    fa.pivflag = lu_flags(buf, a.nrc, (size_t)a.nsp);
    k_band_factor<<<cdiv(npos, 32), 32, 0, G.stream>>>(fa, buf);
    MLG_LAUNCH();
    return 0;
  }));
  a.pivflag = lu_flags(fac, a.nrc, (size_t)a.nsp);
  MLG_TRY(launch_subst<2>(a, fac, npos));
  kt_end(KT_SOLVE, solve_bytes(2, c));
  return 0;
}

}  // namespace mlg
