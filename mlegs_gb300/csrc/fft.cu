// fft.cu — φ and z FFTs of a field (horizontal_fft_forward/backward, mlegs_scalar_ops.f90:1567-1717;
// vertical_fft_forward/backward, :1721-1848) in FFTE's conventions:
//   forward  X_k = sum_j x_j exp(-2 pi i jk/N), then scaled 1/N (the reference divides after FFTE);
//   backward unnormalised sum with exp(+2 pi i jk/N) (FFTE's 1/N undone by the reference's *N).
// The φ transform is real: PPP stores two real samples per complex slot, z_j = f(2j) + i f(2j+1),
// which is exactly the input of a half-length complex FFT; the usual split step turns its result
// into X_0..X_{N/2}.  Backward, the last complex slot keeps N times its input (FFTE's zdfft2d never
// writes A(NX/2+1), zdfft2d.f:119-128, and the reference then multiplies by N, :1705).
//
// Mixed form (T = float): the DC coefficient of a transform line is carried in FP64 and the FP32 FFT
// runs on the mean-free residual.  Forward, the line's FP64 sum gives the k = 0 output and its mean is
// subtracted (in FP64) before the samples are rounded to FP32; backward, the k = 0 input is left out of
// the FP32 transform and added (in FP64) to every output sample.  A vortex field is dominated by its
// axisymmetric, axially uniform mean flow; without this the FP32 rounding of that mean (relative
// 2^-24 of an O(1) value) would land on every other wavenumber, where the perturbation lives.  The
// φ lines all get it (their DC is the m = 0 coefficient).  The z lines of the m = 0 plane run in FP64.
//
// Layout: a field is (nrdim, npdim, nzdim) with r fastest.  Both transforms run along a strided
// dimension; a CTA takes TR consecutive r (the contiguous batch, so every global access is a run of
// TR*16 bytes) and TT threads per transform, keeps the TR transforms in shared memory as
// [point][TR] and runs a Stockham autosort FFT (radix 4, 2, 3, 5) between two shared buffers.
#include "common.cuh"
#include "dfloat.cuh"
#include "xs_common.cuh"
#include <type_traits>

namespace mlg {

// the mixed form's FFT arithmetic: FP32 or double-float
#ifndef MLG_MIXED_FFT_DF
#define MLG_MIXED_FFT_DF 0
#endif
typedef std::conditional<MLG_MIXED_FFT_DF != 0, dfl, float>::type MixFT;

template <typename T> struct CT;
template <> struct CT<double> { typedef double2 t; };
template <> struct CT<float> { typedef float2 t; };
template <> struct CT<dfl> { typedef dfl2 t; };

template <typename T> __device__ __forceinline__ typename CT<T>::t mk(T a, T b);
template <> __device__ __forceinline__ double2 mk<double>(double a, double b) { return make_double2(a, b); }
template <> __device__ __forceinline__ float2 mk<float>(float a, float b) { return make_float2(a, b); }
template <> __device__ __forceinline__ dfl2 mk<dfl>(dfl a, dfl b) { dfl2 r; r.x = a; r.y = b; return r; }

template <typename C> __device__ __forceinline__ C c_add(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C c_sub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C c_mul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C> __device__ __forceinline__ C c_muli(C a, int sgn) {  // a * (sgn * i), exact
  C r; r.x = sgn > 0 ? -a.y : a.y; r.y = sgn > 0 ? a.x : -a.x; return r;
}
template <typename C, typename T> __device__ __forceinline__ C c_scale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }

// twiddle tables hold exp(-2 pi i k/L) (FP64 for the plain form; FP32, or double-float as (re hi,
// re lo, im hi, im lo), for the mixed form); sgn > 0 conjugates
template <typename T> struct TW;
template <> struct TW<double> { typedef double2 t; };
template <> struct TW<float> { typedef float2 t; };
template <> struct TW<dfl> { typedef float4 t; };
template <typename T>
__device__ __forceinline__ typename CT<T>::t load_tw(const typename TW<T>::t* tw, int idx, int sgn) {
  typename TW<T>::t w = tw[idx];
  return mk<T>(w.x, sgn < 0 ? w.y : -w.y);
}
template <>
__device__ __forceinline__ dfl2 load_tw<dfl>(const float4* tw, int idx, int sgn) {
  const float4 w = tw[idx];
  const dfl im(w.z, w.w);
  return mk<dfl>(dfl(w.x, w.y), sgn < 0 ? im : -im);
}
// h + l rounded to FP64 on the integer pipe, for a normalised double-float (|l| <= ulp(h)/2, so l's
// exponent is at least 23 below h's): both significands in one 64-bit integer, h's at bits 38..61,
// then one rounding; GB300's FP64 pipe (about 2 operations per clock per SM) stays free
__device__ __forceinline__ double df_to_double(float h, float l) {
  const unsigned bh = __float_as_uint(h), bl = __float_as_uint(l);
  const int eh = (int)((bh >> 23) & 0xFFu), el = (int)((bl >> 23) & 0xFFu);
  if (eh == 0) return f2d_fast(l);
  long long X = (long long)((bh & 0x7FFFFFu) | 0x800000u) << 38;
  if (bh >> 31) X = -X;
  const int d = eh - el;
  if (el != 0 && d < 62) {
    const long long ml = (long long)((bl & 0x7FFFFFu) | 0x800000u);
    const long long L = d <= 38 ? (ml << (38 - d)) : (ml >> (d - 38));
    X += (bl >> 31) ? -L : L;
  }
  return xs_i64_to_double(X, eh - 150 - 38);
}
// a transform value to FP64 (FP32 and double-float on the integer pipe)
__device__ __forceinline__ double to_dbl(double v) { return v; }
__device__ __forceinline__ double to_dbl(float v) { return f2d_fast(v); }
__device__ __forceinline__ double to_dbl(dfl v) { return df_to_double(v.h, v.l); }

// a double-float sample in the transform's arithmetic
template <typename T> __device__ __forceinline__ T from_df(dfl v);
template <> __device__ __forceinline__ float from_df<float>(dfl v) { return v.h; }
template <> __device__ __forceinline__ dfl from_df<dfl>(dfl v) { return v; }

// small DFTs, sign sgn = -1 forward, +1 backward
template <typename T>
__device__ __forceinline__ void dft_small(typename CT<T>::t* a, int p, int sgn) {
  typedef typename CT<T>::t C;
  if (p == 2) {
    C t = a[0]; a[0] = c_add(t, a[1]); a[1] = c_sub(t, a[1]);
  } else if (p == 4) {
    C t0 = c_add(a[0], a[2]), t1 = c_sub(a[0], a[2]), t2 = c_add(a[1], a[3]), t3 = c_muli(c_sub(a[1], a[3]), sgn);
    a[0] = c_add(t0, t2); a[2] = c_sub(t0, t2); a[1] = c_add(t1, t3); a[3] = c_sub(t1, t3);
  } else if (p == 3) {
    const T c1 = (T)-0.5, s1 = (T)0.86602540378443864676372317075294;  // cos(2pi/3), sin(2pi/3)
    C t1 = c_add(a[1], a[2]), t2 = c_sub(a[1], a[2]);
    C m1 = c_add(a[0], c_scale(t1, c1));
    C m2 = c_muli(c_scale(t2, s1), sgn);
    a[0] = c_add(a[0], t1); a[1] = c_add(m1, m2); a[2] = c_sub(m1, m2);
  } else if (p == 5) {
    const T c1 = (T)0.30901699437494742410229341718282, c2 = (T)-0.80901699437494742410229341718282;
    const T s1 = (T)0.95105651629515357211643933337938, s2 = (T)0.58778525229247312916870595463907;
    C t1 = c_add(a[1], a[4]), t2 = c_add(a[2], a[3]), t3 = c_sub(a[1], a[4]), t4 = c_sub(a[2], a[3]);
    C m1 = c_add(a[0], c_add(c_scale(t1, c1), c_scale(t2, c2)));
    C m2 = c_add(a[0], c_add(c_scale(t1, c2), c_scale(t2, c1)));
    C n1 = c_muli(c_add(c_scale(t3, s1), c_scale(t4, s2)), sgn);
    C n2 = c_muli(c_sub(c_scale(t3, s2), c_scale(t4, s1)), sgn);
    a[0] = c_add(a[0], c_add(t1, t2));
    a[1] = c_add(m1, n1); a[4] = c_sub(m1, n1);
    a[2] = c_add(m2, n2); a[3] = c_sub(m2, n2);
  }
}

// Stockham FFT over the TR transforms held in s0 ([L][TR]); result left in *res.
template <typename T>
__device__ void stockham(typename CT<T>::t* s0, typename CT<T>::t* s1, typename CT<T>::t** res, int L, int TR,
                         int tr, int tt, int TT, const typename TW<T>::t* tw, int sgn) {
  typedef typename CT<T>::t C;
  C* src = s0;
  C* dst = s1;
  int rem = L;
  for (int ns = 1; ns < L;) {
    int p = (rem % 4 == 0) ? 4 : (rem % 2 == 0) ? 2 : (rem % 3 == 0) ? 3 : 5;
    int m = L / p;
    int span = ns * p, twstep = L / span;
    for (int j = tt; j < m; j += TT) {
      int k = j % ns;
      C a[5];
#pragma unroll
      for (int r = 0; r < 5; ++r)
        if (r < p) a[r] = src[(j + r * m) * TR + tr];
      if (k) {
#pragma unroll
        for (int r = 1; r < 5; ++r)
          if (r < p) a[r] = c_mul(a[r], load_tw<T>(tw, (k * r * twstep) % L, sgn));
      }
      dft_small<T>(a, p, sgn);
      int base = (j / ns) * span + k;
#pragma unroll
      for (int r = 0; r < 5; ++r)
        if (r < p) dst[(base + r * ns) * TR + tr] = a[r];
    }
    __syncthreads();
    C* t = src; src = dst; dst = t;
    ns = span;
    rem /= p;
  }
  *res = src;
}

template <typename T> __device__ __forceinline__ typename CT<T>::t ld(const double2* p);
template <> __device__ __forceinline__ double2 ld<double>(const double2* p) { return *p; }
template <> __device__ __forceinline__ float2 ld<float>(const double2* p) { return ld_c32(p); }
template <> __device__ __forceinline__ dfl2 ld<dfl>(const double2* p) {
  const double2 v = *p;
  return mk<dfl>(dfl(v.x), dfl(v.y));
}
template <typename T> __device__ __forceinline__ void st(double2* p, typename CT<T>::t v);
template <> __device__ __forceinline__ void st<double>(double2* p, double2 v) { *p = v; }
template <> __device__ __forceinline__ void st<float>(double2* p, float2 v) { st_c32(p, v); }
template <> __device__ __forceinline__ void st<dfl>(double2* p, dfl2 v) { *p = make_double2(to_dbl(v.x), to_dbl(v.y)); }

// z FFT of columns (r, m): points at stride nrdim*npdim; the grid covers m = m0, m0+1, ...
template <typename T>
__global__ void k_vfft(double2* __restrict__ e, int nrdim, int npdim, int L, int TR,
                       const typename TW<T>::t* __restrict__ tw, int sgn, T scale, int m0) {
  typedef typename CT<T>::t C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* s0 = (C*)smem_raw;
  C* s1 = s0 + (size_t)L * TR;
  int tr = threadIdx.x, tt = threadIdx.y, TT = blockDim.y;
  int r = blockIdx.x * TR + tr;
  int m = blockIdx.y + m0;
  bool ok = r < nrdim;
  size_t pstride = (size_t)nrdim * npdim;
  double2* base = e + r + (size_t)nrdim * m;
  for (int pt = tt; pt < L; pt += TT) s0[pt * TR + tr] = ok ? ld<T>(base + pt * pstride) : mk<T>(0, 0);
  __syncthreads();
  C* res;
  stockham<T>(s0, s1, &res, L, TR, tr, tt, TT, tw, sgn);
  if (ok)
    for (int pt = tt; pt < L; pt += TT) st<T>(base + pt * pstride, c_scale(res[pt * TR + tr], (T)scale));
}

// φ forward: packed reals -> X_0..X_{L} (L = np/2) scaled 1/np, in place.  Mixed form: X_0 from the
// FP64 sum of the row, the FP32 FFT on the samples minus their FP64 mean.
template <typename T>
__global__ void k_hfft_fwd(double2* __restrict__ e, int nrdim, int npdim, int L, int TR,
                           const typename TW<T>::t* __restrict__ tw, const typename TW<T>::t* __restrict__ twr, T scale,
                           double scale_d, double inv_np, const double* __restrict__ rs, int nrs) {
  typedef typename CT<T>::t C;
  constexpr bool DC = std::is_same<T, float>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* s0 = (C*)smem_raw;
  C* s1 = s0 + (size_t)L * TR;
  int tr = threadIdx.x, tt = threadIdx.y, TT = blockDim.y;
  int r = blockIdx.x * TR + tr;
  int z = blockIdx.y;
  bool ok = r < nrdim;
  double2* base = e + r + (size_t)nrdim * npdim * z;
  const double rv = (rs != nullptr && ok && r < nrs) ? rs[r] : 1.0;   // scale_r of the input row
  double sum = 0.0, mu = 0.0;
  if (DC) {
    double* red = (double*)(s1 + (size_t)L * TR);
    double part = 0.0;
    if (ok)
      for (int pt = tt; pt < L; pt += TT) { double2 v = base[(size_t)pt * nrdim]; part += v.x * rv + v.y * rv; }
    red[tt * TR + tr] = part;
    __syncthreads();
    for (int q = 0; q < TT; ++q) sum += red[q * TR + tr];
    mu = sum * inv_np;
  }
  for (int pt = tt; pt < L; pt += TT) {
    C v = mk<T>(0, 0);
    if (ok) {
      if (DC) {
        double2 d = base[(size_t)pt * nrdim];
        v = mk<T>((T)d2f_fast(d.x * rv - mu), (T)d2f_fast(d.y * rv - mu));
      } else {
        double2 d = base[(size_t)pt * nrdim];
        v = mk<T>((T)(d.x * rv), (T)(d.y * rv));
      }
    }
    s0[pt * TR + tr] = v;
  }
  __syncthreads();
  C* res;
  stockham<T>(s0, s1, &res, L, TR, tr, tt, TT, tw, -1);
  if (!ok) return;
  for (int k = tt; k <= L; k += TT) {
    C zk = res[(k % L) * TR + tr];
    C zc = res[((L - k) % L) * TR + tr];
    zc.y = -zc.y;
    C fe = c_scale(c_add(zk, zc), (T)0.5);
    C fo = c_muli(c_scale(c_sub(zk, zc), (T)0.5), -1);   // (zk - zc)/(2i)
    typename TW<T>::t wd = twr[k];
    C w = mk<T>(wd.x, wd.y);
    C x = c_scale(c_add(fe, c_mul(w, fo)), (T)scale);
    if (DC && k == 0) {
      base[0] = make_double2(f2d_fast((float)x.x) + sum * scale_d, f2d_fast((float)x.y));
    } else {
      st<T>(base + (size_t)k * nrdim, x);
    }
  }
}

// φ backward: X_0..X_L -> packed reals (unnormalised); slot L <- np * X_L (input), in place.  Mixed
// form: Re X_0 is left out of the FP32 FFT and added to every sample in FP64.
template <typename T>
__global__ void k_hfft_bwd(double2* __restrict__ e, int nrdim, int npdim, int L, int TR,
                           const typename TW<T>::t* __restrict__ tw, const typename TW<T>::t* __restrict__ twr, double np_d,
                           const double* __restrict__ rs, int nrs) {
  typedef typename CT<T>::t C;
  constexpr bool DC = std::is_same<T, float>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* s0 = (C*)smem_raw;
  C* s1 = s0 + (size_t)L * TR;
  int tr = threadIdx.x, tt = threadIdx.y, TT = blockDim.y;
  int r = blockIdx.x * TR + tr;
  int z = blockIdx.y;
  bool ok = r < nrdim;
  double2* base = e + r + (size_t)nrdim * npdim * z;
  double2 nyq = make_double2(0, 0);
  double dc = 0.0;
  if (ok && tt == 0) nyq = base[(size_t)L * nrdim];
  if (DC && ok) dc = base[0].x;
  for (int k = tt; k < L; k += TT) {
    C v = mk<T>(0, 0);
    if (ok) {
      C xk = ld<T>(base + (size_t)k * nrdim);
      C xc = ld<T>(base + (size_t)(L - k) * nrdim);
      if (k == 0) { xk.y = 0; xc.y = 0; if (DC) xk.x = 0; }
      xc.y = -xc.y;
      C g = c_add(xk, xc);
      typename TW<T>::t wd = twr[k];
      C w = mk<T>(wd.x, -wd.y);   // exp(+2 pi i k / np)
      C h = c_mul(c_sub(xk, xc), w);
      v = c_add(g, c_muli(h, 1));
    }
    s0[k * TR + tr] = v;
  }
  __syncthreads();
  C* res;
  stockham<T>(s0, s1, &res, L, TR, tr, tt, TT, tw, +1);
  if (!ok) return;
  const double rv = (rs != nullptr && r < nrs) ? rs[r] : 1.0;   // scale_r of the output row
  for (int pt = tt; pt < L; pt += TT) {
    C y = res[pt * TR + tr];
    double2 v;
    if (DC) v = make_double2(f2d_fast((float)y.x) + dc, f2d_fast((float)y.y) + dc);
    else v = make_double2((double)y.x, (double)y.y);
    base[(size_t)pt * nrdim] = make_double2(v.x * rv, v.y * rv);
  }
  if (tt == 0) base[(size_t)L * nrdim] = make_double2(nyq.x * np_d * rv, nyq.y * np_d * rv);
}

// ------------------------------------------------------------------------------------------------
// Power-of-two lengths 16..256: two passes through registers.  L = R1 * R2, n = n2 + R2 n1,
// k = k1 + R1 k2:  X_k = sum_n2 w_L^(n2 k1) [sum_n1 x_n w_R1^(n1 k1)] w_R2^(n2 k2).
// A CTA holds TRL lines (consecutive r: every global access is a run of TRL*16 bytes) and R2 threads
// per line; pass 1: each thread loads R1 points of its line and does the R1-point DFT in registers,
// multiplies by w_L^(n2 k1) and stores to shared memory [k1][n2][line]; pass 2: each thread does
// R1/R2 DFTs of R2 points and writes the results.  Every element is read and written once in HBM and
// once in shared memory, with compile-time index arithmetic.

// cos and sin of 2 pi j / 16 (j mod 16)
__host__ __device__ constexpr double cos16(int j) {
  return (j & 15) == 0 ? 1.0 : (j & 15) == 1 ? 0.92387953251128675613 : (j & 15) == 2 ? 0.70710678118654752440
       : (j & 15) == 3 ? 0.38268343236508977173 : (j & 15) == 4 ? 0.0 : (j & 15) == 5 ? -0.38268343236508977173
       : (j & 15) == 6 ? -0.70710678118654752440 : (j & 15) == 7 ? -0.92387953251128675613 : (j & 15) == 8 ? -1.0
       : (j & 15) == 9 ? -0.92387953251128675613 : (j & 15) == 10 ? -0.70710678118654752440
       : (j & 15) == 11 ? -0.38268343236508977173 : (j & 15) == 12 ? 0.0 : (j & 15) == 13 ? 0.38268343236508977173
       : (j & 15) == 14 ? 0.70710678118654752440 : 0.92387953251128675613;
}
__host__ __device__ constexpr double sin16(int j) { return cos16(j - 4); }

// v * exp(SGN 2 pi i j / 16)
template <typename T, int SGN>
__device__ __forceinline__ typename CT<T>::t tw16(typename CT<T>::t v, int j) {
  typedef typename CT<T>::t C;
  j &= 15;
  if (j == 0) return v;
  if (j == 8) { C r; r.x = -v.x; r.y = -v.y; return r; }
  if (j == 4) return c_muli(v, SGN);
  if (j == 12) return c_muli(v, -SGN);
  C w; w.x = (T)cos16(j); w.y = (T)(SGN * sin16(j));
  return c_mul(v, w);
}

__host__ __device__ constexpr int bitrev(int i, int n) {   // bit reversal of i in log2(n) bits
  int r = 0;
  for (int b = 1; b < n; b <<= 1) { r = (r << 1) | (i & 1); i >>= 1; }
  return r;
}

// in-register DFT of N <= 16 points, sign SGN: radix-2 decimation in frequency, fully unrolled, so
// every register index is a compile-time constant; the result comes out in bit-reversed order,
// a[i] = X_bitrev(i), and the callers fold the reversal into their memory addresses
template <typename T, int N, int SGN>
__device__ __forceinline__ void dft_reg(typename CT<T>::t* a) {
  typedef typename CT<T>::t C;
#pragma unroll
  for (int len = N; len >= 2; len >>= 1) {
#pragma unroll
    for (int i = 0; i < N; i += len) {
#pragma unroll
      for (int k = 0; k < len / 2; ++k) {
        C u = a[i + k], v = a[i + k + len / 2];
        a[i + k] = c_add(u, v);
        a[i + k + len / 2] = tw16<T, SGN>(c_sub(u, v), k * (16 / len));
      }
    }
  }
}

template <int L> struct Split;            // L = R1 * R2, R1 >= R2, R1 <= 16
template <> struct Split<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct Split<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct Split<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Split<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct Split<256> { static constexpr int R1 = 16, R2 = 16; };

// the two passes on a CTA's lines; a[] holds the R1 inputs of this thread (n1 order); on return
// b[q][i] holds X_(k1 + R1 bitrev(i)) for k1 = w*(R1/R2) + q
template <typename T, int L, int SGN, int TRL>
__device__ __forceinline__ void fft2pass(typename CT<T>::t* a, typename CT<T>::t (*b)[Split<L>::R2],
                                         typename CT<T>::t* S, const typename TW<T>::t* __restrict__ tw, int w,
                                         int lane) {
  constexpr int R1 = Split<L>::R1, R2 = Split<L>::R2, Q = R1 / R2;
  dft_reg<T, R1, SGN>(a);
#pragma unroll
  for (int i = 0; i < R1; ++i) {
    const int k1 = bitrev(i, R1);
    typename CT<T>::t v = a[i];
    if (k1) v = c_mul(v, load_tw<T>(tw, (w * k1) & (L - 1), SGN));
    S[(k1 * R2 + w) * TRL + lane] = v;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    int k1 = w * Q + q;
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) b[q][n2] = S[(k1 * R2 + n2) * TRL + lane];
    dft_reg<T, R2, SGN>(b[q]);
  }
}

// a set of fields transformed by one launch (the components of a vector field, stage by stage): their
// lines are taken flat, field after field, so that one launch has enough blocks to fill the GPU
constexpr int FS_MAX = 6;
struct FSet {
  double2* e[FS_MAX];
  const double* rs[FS_MAX];   // per field: the row scaling of the phi transforms, or null
  int n;
};
// field f's pointers by a chain of selects: an indexed access to the kernel parameter would copy the
// whole set to local memory
__device__ __forceinline__ double2* fset_e(const FSet& fs, int f) {
  double2* p = fs.e[0];
#pragma unroll
  for (int q = 1; q < FS_MAX; ++q) p = f == q ? fs.e[q] : p;
  return p;
}
__device__ __forceinline__ const double* fset_rs(const FSet& fs, int f) {
  const double* p = fs.rs[0];
#pragma unroll
  for (int q = 1; q < FS_MAX; ++q) p = f == q ? fs.rs[q] : p;
  return p;
}

// z FFT: the lines (r, m) of m in [m0, m0 + nm) taken flat, line r + nrdim*(m - m0) at offset
// r + nrdim*m (so a block's lanes read one run of consecutive offsets and no block is left ragged at
// the end of an m), points at stride nrdim*npdim
template <typename T, int L, int SGN, int TRL>
__global__ void __launch_bounds__(TRL * Split<L>::R2) k_zfft2(FSet fs, int nrdim, int npdim,
                                                              const typename TW<T>::t* __restrict__ tw, T scale, int m0,
                                                              int nlines) {
  typedef typename CT<T>::t C;
  constexpr int R1 = Split<L>::R1, R2 = Split<L>::R2, Q = R1 / R2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* S = (C*)smem_raw;
  int lane = threadIdx.x, w = threadIdx.y;
  const int gl = blockIdx.x * TRL + lane;     // line over the set; nlines per field
  const int f = gl / nlines, line = gl - f * nlines;
  bool ok = f < fs.n;
  size_t ps = (size_t)nrdim * npdim;
  double2* base = fset_e(fs, ok ? f : 0) + (size_t)nrdim * m0 + line;
  C a[R1];
#pragma unroll
  for (int n1 = 0; n1 < R1; ++n1) a[n1] = ok ? ld<T>(base + (size_t)(w + R2 * n1) * ps) : mk<T>(0, 0);
  C b[Q][R2];
  fft2pass<T, L, SGN, TRL>(a, b, S, tw, w, lane);
  if (!ok) return;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    int k1 = w * Q + q;
#pragma unroll
    for (int i = 0; i < R2; ++i) st<T>(base + (size_t)(k1 + R1 * bitrev(i, R2)) * ps, c_scale(b[q][i], scale));
  }
}

// φ forward: packed reals -> X_0..X_L scaled, in place (lines (r, z)); mixed form: X_0 from the FP64
// sum of the row, the FP32 transform on the samples minus their FP64 mean
template <typename T, int L, int TRL>
__global__ void __launch_bounds__(TRL * Split<L>::R2) k_pfft_fwd2(FSet fs, int nrdim, int npdim, int nzdim,
                                                                  const typename TW<T>::t* __restrict__ tw,
                                                                  const typename TW<T>::t* __restrict__ twr, T scale,
                                                                  double scale_d, double inv_np, int nrs) {
  typedef typename CT<T>::t C;
  constexpr int R1 = Split<L>::R1, R2 = Split<L>::R2, Q = R1 / R2;
  constexpr bool DC = !std::is_same<T, double>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* S = (C*)smem_raw;
  double* red = (double*)(smem_raw + (size_t)L * TRL * sizeof(C));
  int lane = threadIdx.x, w = threadIdx.y;
  const int per = nrdim * nzdim;               // the lines (r, z) of a field taken flat: r + nrdim*z
  const int gl = blockIdx.x * TRL + lane;
  const int f = gl / per, line = gl - f * per;
  bool ok = f < fs.n;
  const int r = line % nrdim, z = line / nrdim;
  double2* base = fset_e(fs, ok ? f : 0) + r + (size_t)nrdim * npdim * z;
  const double* rs = ok ? fset_rs(fs, f) : nullptr;
  const bool rsc = rs != nullptr && ok && r < nrs;   // the row's samples times rs[r] first (scale_r)
  const double rv = rsc ? rs[r] : 1.0;
  C a[R1];
  double sum = 0.0;
  if constexpr (DC) {
    // the row scale, the row sum and the mean subtraction in double-float (about 47 bits, on the FP32
    // and integer pipes; FP64 would occupy GB300's narrow FP64 pipe with 4-6 operations per sample);
    // the samples less their mean are then rounded to FP32 for the transform
    dfl dx[R1], dy[R1];
    dfl part(0);
    const dfl rvd = rsc ? dfl(rv) : dfl(1);
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      const double2 v = ok ? base[(size_t)(w + R2 * n1) * nrdim] : make_double2(0.0, 0.0);
      dx[n1] = dfl(v.x);
      dy[n1] = dfl(v.y);
      if (rsc) { dx[n1] = dx[n1] * rvd; dy[n1] = dy[n1] * rvd; }
      part = part + dx[n1] + dy[n1];
    }
    dfl* redf = reinterpret_cast<dfl*>(red);
    redf[w * TRL + lane] = part;
    __syncthreads();
    dfl sd(0);
#pragma unroll
    for (int q = 0; q < R2; ++q) sd = sd + redf[q * TRL + lane];
    const dfl mu = sd * dfl((float)inv_np, 0.f);   // inv_np = 1/np, a power of two for these lengths
    sum = f2d_fast(sd.h) + f2d_fast(sd.l);
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) a[n1] = mk<T>(from_df<T>(dx[n1] - mu), from_df<T>(dy[n1] - mu));
  } else {
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      if (rsc) {
        double2 d = base[(size_t)(w + R2 * n1) * nrdim];
        a[n1] = mk<T>((T)(d.x * rv), (T)(d.y * rv));
      } else {
        a[n1] = ok ? ld<T>(base + (size_t)(w + R2 * n1) * nrdim) : mk<T>(0, 0);
      }
    }
  }
  C b[Q][R2];
  fft2pass<T, L, -1, TRL>(a, b, S, tw, w, lane);
  __syncthreads();   // every thread has read its pass-2 inputs: S can take the spectrum
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    int k1 = w * Q + q;
#pragma unroll
    for (int i = 0; i < R2; ++i) S[(k1 * R2 + bitrev(i, R2)) * TRL + lane] = b[q][i];   // Z_(k1 + R1 k2)
  }
  __syncthreads();
  if (!ok) return;
  auto Z = [&](int k) -> C { return S[((k % R1) * R2 + k / R1) * TRL + lane]; };
  for (int k = w; k <= L; k += R2) {
    C zk = Z(k & (L - 1));
    C zc = Z((L - k) & (L - 1));
    zc.y = -zc.y;
    C fe = c_scale(c_add(zk, zc), (T)0.5);
    C fo = c_muli(c_scale(c_sub(zk, zc), (T)0.5), -1);   // (zk - zc)/(2i)
    C x = c_scale(c_add(fe, c_mul(load_tw<T>(twr, k, -1), fo)), scale);
    bool dc0 = false;
    if constexpr (DC) dc0 = k == 0;
    if (dc0) base[0] = make_double2(to_dbl(x.x) + sum * scale_d, to_dbl(x.y));
    else st<T>(base + (size_t)k * nrdim, x);
  }
}

// φ backward: X_0..X_L -> packed reals (unnormalised), slot L <- np X_L, in place; mixed form: Re X_0
// left out of the FP32 transform and added to every sample in FP64
template <typename T, int L, int TRL>
__global__ void __launch_bounds__(TRL * Split<L>::R2) k_pfft_bwd2(FSet fs, int nrdim, int npdim, int nzdim,
                                                                  const typename TW<T>::t* __restrict__ tw,
                                                                  const typename TW<T>::t* __restrict__ twr, double np_d,
                                                                  int nrs) {
  typedef typename CT<T>::t C;
  constexpr int R1 = Split<L>::R1, R2 = Split<L>::R2, Q = R1 / R2;
  constexpr bool DC = !std::is_same<T, double>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* S = (C*)smem_raw;
  int lane = threadIdx.x, w = threadIdx.y;
  const int per = nrdim * nzdim;               // the lines (r, z) of a field taken flat: r + nrdim*z
  const int gl = blockIdx.x * TRL + lane;
  const int f = gl / per, line = gl - f * per;
  bool ok = f < fs.n;
  const int r = line % nrdim, z = line / nrdim;
  double2* base = fset_e(fs, ok ? f : 0) + r + (size_t)nrdim * npdim * z;
  const double* rs = ok ? fset_rs(fs, f) : nullptr;
  double2 nyq = make_double2(0, 0);
  double dc = 0.0;
  if (ok && w == 0) nyq = base[(size_t)L * nrdim];
  if (DC && ok) dc = base[0].x;
  C a[R1];
#pragma unroll
  for (int n1 = 0; n1 < R1; ++n1) {
    int k = w + R2 * n1;
    C v = mk<T>(0, 0);
    if (ok) {
      C xk = ld<T>(base + (size_t)k * nrdim);
      C xc = ld<T>(base + (size_t)(L - k) * nrdim);
      if (k == 0) { xk.y = 0; xc.y = 0; if (DC) xk.x = 0; }
      xc.y = -xc.y;
      C g = c_add(xk, xc);
      C h = c_mul(c_sub(xk, xc), load_tw<T>(twr, k, +1));   // exp(+2 pi i k / np)
      v = c_add(g, c_muli(h, 1));
    }
    a[n1] = v;
  }
  C b[Q][R2];
  fft2pass<T, L, +1, TRL>(a, b, S, tw, w, lane);
  if (!ok) return;
  const bool rsc = rs != nullptr && r < nrs;   // every slot of the row times rs[r] last (scale_r)
  const double rv = rsc ? rs[r] : 1.0;
  const double dcr = dc * rv;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    int k1 = w * Q + q;
#pragma unroll
    for (int i = 0; i < R2; ++i) {
      C y = b[q][i];
      double2* o = base + (size_t)(k1 + R1 * bitrev(i, R2)) * nrdim;
      double2 v;
      if constexpr (DC) {
        // (y + dc) rv as one FMA per component
        v = rsc ? make_double2(fma(to_dbl(y.x), rv, dcr), fma(to_dbl(y.y), rv, dcr))
                : make_double2(to_dbl(y.x) + dc, to_dbl(y.y) + dc);
      } else {
        v = make_double2((double)y.x, (double)y.y);
        if (rsc) { v.x *= rv; v.y *= rv; }
      }
      *o = v;
    }
  }
  if (w == 0) {
    double2 v = make_double2(nyq.x * np_d, nyq.y * np_d);
    if (rsc) { v.x *= rv; v.y *= rv; }
    base[(size_t)L * nrdim] = v;
  }
}

// a host-side scale factor in the transform's arithmetic (double-float: hi = the FP32 rounding, lo =
// the FP32 rounding of the rest)
template <typename T> static T host_scale(double v) { return (T)v; }
template <> dfl host_scale<dfl>(double v) { const float h = (float)v; return dfl(h, (float)(v - (double)h)); }

// the twiddle tables of a transform's arithmetic: phi (L = np/2), phi post-processing (np), z (nz)
template <typename T> struct TwTab;
template <> struct TwTab<double> {
  static const double2* p() { return G.tw_p; }
  static const double2* pr() { return G.tw_pr; }
  static const double2* z() { return G.tw_z; }
};
template <> struct TwTab<float> {
  static const float2* p() { return G.tw_p32; }
  static const float2* pr() { return G.tw_pr32; }
  static const float2* z() { return G.tw_z32; }
};
template <> struct TwTab<dfl> {
  static const float4* p() { return G.tw_pdf; }
  static const float4* pr() { return G.tw_prdf; }
  static const float4* z() { return G.tw_zdf; }
};

static int pick_tr(int L, size_t elem) {
  // two shared buffers of L*TR complex values, at most 96 KB
  int tr = 32;
  while (tr > 1 && 2ull * L * tr * elem > 96 * 1024) tr /= 2;
  return tr;
}

template <typename T>
static int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return 0;
}

static FSet fset1(cd* e, const double* rs = nullptr) {
  FSet fs{};
  fs.e[0] = e; fs.rs[0] = rs; fs.n = 1;
  return fs;
}

template <typename T, int L, int SGN, int TRL>
static int zfft2_launch(const FSet& fs, double scale, int m0, int nm, cudaStream_t stream) {
  size_t sm = (size_t)L * TRL * sizeof(typename CT<T>::t);
  MLG_TRY(set_smem<T>((const void*)k_zfft2<T, L, SGN, TRL>, sm));
  const int nlines = G.nrdim * nm;
  dim3 grid(cdiv((long long)nlines * fs.n, TRL)), blk(TRL, Split<L>::R2);
  k_zfft2<T, L, SGN, TRL><<<grid, blk, sm, stream>>>(fs, G.nrdim, G.npdim, TwTab<T>::z(), host_scale<T>(scale), m0,
                                                     nlines);
  MLG_LAUNCH();
  return 0;
}
template <typename T, int L, int TRL>
static int zfft2_dir(const FSet& fs, int dir, double scale, int m0, int nm, cudaStream_t stream) {
  return dir < 0 ? zfft2_launch<T, L, -1, TRL>(fs, scale, m0, nm, stream) : zfft2_launch<T, L, +1, TRL>(fs, scale, m0, nm, stream);
}
template <typename T, int TRL>
static int zfft2_any(const FSet& fs, int dir, double scale, int m0, int nm, cudaStream_t stream) {
  switch (G.nz) {
    case 16: return zfft2_dir<T, 16, TRL>(fs, dir, scale, m0, nm, stream);
    case 32: return zfft2_dir<T, 32, TRL>(fs, dir, scale, m0, nm, stream);
    case 64: return zfft2_dir<T, 64, TRL>(fs, dir, scale, m0, nm, stream);
    case 128: return zfft2_dir<T, 128, TRL>(fs, dir, scale, m0, nm, stream);
    case 256: return zfft2_dir<T, 256, TRL>(fs, dir, scale, m0, nm, stream);
  }
  return -1;
}
static bool pow2_fast(int L) { return L == 16 || L == 32 || L == 64 || L == 128 || L == 256; }

template <typename T>
static int vfft_t(const FSet& fs, int dir, double scale, int m0, int nm, int tr_max, cudaStream_t stream) {
  int L = G.nz;
  if (L <= 1 || nm <= 0) return 0;
  if (pow2_fast(L)) {
    if (tr_max >= 32) return zfft2_any<T, 32>(fs, dir, scale, m0, nm, stream);
    // a single plane (m = 0): four lines per CTA, so that its few hundred lines spread over most SMs
    return tr_max >= 8 ? zfft2_any<T, 8>(fs, dir, scale, m0, nm, stream) : zfft2_any<T, 4>(fs, dir, scale, m0, nm, stream);
  }
  if constexpr (std::is_same<T, dfl>::value) {
    return vfft_t<double>(fs, dir, scale, m0, nm, tr_max, stream);   // other lengths: the FP64 Stockham kernel
  } else {
  int TR = std::min(pick_tr(L, sizeof(typename CT<T>::t)), tr_max);
  int TT = std::max(1, std::min(256 / TR, L / 2));
  size_t sm = 2ull * L * TR * sizeof(typename CT<T>::t);
  MLG_TRY(set_smem<T>((const void*)k_vfft<T>, sm));
  dim3 grid(cdiv(G.nrdim, TR), nm), blk(TR, TT);
  for (int f = 0; f < fs.n; ++f) {   // other lengths: the Stockham kernel, field by field
    k_vfft<T><<<grid, blk, sm, stream>>>(fs.e[f], G.nrdim, G.npdim, L, TR, TwTab<T>::z(), dir, (T)scale, m0);
    MLG_LAUNCH();
  }
  return 0;
  }
}

// plain form: FP64.  Mixed form: m >= 1 in FP32; the m = 0 lines (the axisymmetric part, with the mean
// flow in its k = 0 coefficient) in FP64, in small CTAs so that they spread over the SMs.
static int vfft_any(const FSet& fs, int dir, double scale) {
  kt_begin(1);
  if (G.precision == MLG_MIXED) {
    MLG_TRY(side_fork());
    MLG_TRY(vfft_t<double>(fs, dir, scale, 0, 1, 2, G.side));
    MLG_TRY(vfft_t<MixFT>(fs, dir, scale, 1, G.npdim - 1, 32, G.stream));
    MLG_TRY(side_join());
  } else {
    MLG_TRY(vfft_t<double>(fs, dir, scale, 0, G.npdim, 32, G.stream));
  }
  kt_end(1, 2.0 * fs.n * G.fsize * 16);
  return 0;
}

int launch_vfft_buf(cd* e, int dir) { return vfft_any(fset1(e), dir, dir < 0 ? 1.0 / G.nz : 1.0); }
// sum_j x_j exp(dir 2 pi i jk/nz) * scale, any direction and scale (the adjoint's FFTs)
int launch_vfft_scaled(cd* e, int dir, double scale) { return vfft_any(fset1(e), dir, scale); }
int launch_vfft(Scalar& s, int dir) { return launch_vfft_buf(s.e, dir); }
// the z transform of n fields in one pass (forward scaled by 1/nz)
int launch_vfft_multi(Scalar* const* s, int n, int dir) {
  if (n < 1 || n > FS_MAX) return set_error(MLG_EPARAM, "vertical_fft: 1 to 6 fields per batch");
  FSet fs{};
  for (int i = 0; i < n; ++i) { fs.e[i] = s[i]->e; fs.rs[i] = nullptr; }
  fs.n = n;
  return vfft_any(fs, dir, dir < 0 ? 1.0 / G.nz : 1.0);
}

template <typename T, int L>
static int pfft2_launch(const FSet& fs, int dir, double scale) {
  constexpr int TRL = 32;
  constexpr bool DC = !std::is_same<T, double>::value;
  size_t sm = (size_t)L * TRL * sizeof(typename CT<T>::t) + (DC && dir < 0 ? (size_t)Split<L>::R2 * TRL * sizeof(double) : 0);
  dim3 grid(cdiv((long long)G.nrdim * G.nzdim * fs.n, TRL)), blk(TRL, Split<L>::R2);
  if (dir < 0) {
    MLG_TRY(set_smem<T>((const void*)k_pfft_fwd2<T, L, TRL>, sm));
    k_pfft_fwd2<T, L, TRL><<<grid, blk, sm, G.stream>>>(fs, G.nrdim, G.npdim, G.nzdim, TwTab<T>::p(),
                                                        TwTab<T>::pr(), host_scale<T>(scale), scale, 1.0 / G.np, G.nr);
  } else {
    MLG_TRY(set_smem<T>((const void*)k_pfft_bwd2<T, L, TRL>, sm));
    k_pfft_bwd2<T, L, TRL><<<grid, blk, sm, G.stream>>>(fs, G.nrdim, G.npdim, G.nzdim, TwTab<T>::p(),
                                                        TwTab<T>::pr(), (double)G.np, G.nr);
  }
  MLG_LAUNCH();
  return 0;
}

template <typename T>
static int hfft_t(const FSet& fs, int dir, double scale) {
  int L = G.nph;
  if (G.np <= 1) return 0;
  kt_begin(1);
  if (pow2_fast(L)) {
    switch (L) {
      case 16: MLG_TRY((pfft2_launch<T, 16>(fs, dir, scale))); break;
      case 32: MLG_TRY((pfft2_launch<T, 32>(fs, dir, scale))); break;
      case 64: MLG_TRY((pfft2_launch<T, 64>(fs, dir, scale))); break;
      case 128: MLG_TRY((pfft2_launch<T, 128>(fs, dir, scale))); break;
      case 256: MLG_TRY((pfft2_launch<T, 256>(fs, dir, scale))); break;
    }
    kt_end(1, 2.0 * fs.n * G.fsize * 16);
    return 0;
  }
  if constexpr (std::is_same<T, dfl>::value) {
    kt_end(1, 0.0);
    return hfft_t<double>(fs, dir, scale);   // other lengths: the FP64 Stockham kernels
  } else {
  int TR = pick_tr(L, sizeof(typename CT<T>::t));
  int TT = std::max(1, std::min(256 / TR, std::max(L / 2, 1)));
  constexpr bool DC = std::is_same<T, float>::value;
  size_t sm = 2ull * L * TR * sizeof(typename CT<T>::t) + (DC ? (size_t)TT * TR * sizeof(double) : 0);
  dim3 grid(cdiv(G.nrdim, TR), G.nzdim), blk(TR, TT);
  if (dir < 0) MLG_TRY(set_smem<T>((const void*)k_hfft_fwd<T>, sm));
  else MLG_TRY(set_smem<T>((const void*)k_hfft_bwd<T>, sm));
  for (int f = 0; f < fs.n; ++f) {   // other lengths: the Stockham kernels, field by field
    if (dir < 0) {
      k_hfft_fwd<T><<<grid, blk, sm, G.stream>>>(fs.e[f], G.nrdim, G.npdim, L, TR, TwTab<T>::p(),
                                                  TwTab<T>::pr(), (T)scale,
                                                  scale, 1.0 / G.np, fs.rs[f], G.nr);
    } else {
      k_hfft_bwd<T><<<grid, blk, sm, G.stream>>>(fs.e[f], G.nrdim, G.npdim, L, TR, TwTab<T>::p(),
                                                  TwTab<T>::pr(), (double)G.np, fs.rs[f], G.nr);
    }
    MLG_LAUNCH();
  }
  kt_end(1, 2.0 * fs.n * G.fsize * 16);
  return 0;
  }
}

int launch_hfft(Scalar& s, int dir) { return launch_hfft_rs(s, dir, nullptr); }
// with rs: the rows i < nr of the field times rs[i] before the forward transform / after the
// backward one (scale_r folded into the transform)
int launch_hfft_rs(Scalar& s, int dir, const double* rs) {
  Scalar* ps = &s;
  return launch_hfft_multi(&ps, &rs, 1, dir);
}
// the phi transform of n fields in one pass, field i's rows times rs[i] (before the forward / after
// the backward transform) where rs[i] is not null
int launch_hfft_multi(Scalar* const* s, const double* const* rs, int n, int dir) {
  if (n < 1 || n > FS_MAX) return set_error(MLG_EPARAM, "horizontal_fft: 1 to 6 fields per batch");
  FSet fs{};
  for (int i = 0; i < n; ++i) {
    if (G.npchop + s[i]->off[1] > G.npdim)
      return set_error(MLG_ECHOP, dir < 0 ? "horizontal_fft_forward: chopping in p too large"
                                          : "horizontal_fft_fbackard: chopping in p too large");
    fs.e[i] = s[i]->e; fs.rs[i] = rs ? rs[i] : nullptr;
  }
  fs.n = n;
  return G.precision == MLG_MIXED ? hfft_t<MixFT>(fs, dir, 1.0 / G.np) : hfft_t<double>(fs, dir, 1.0 / G.np);
}
static FSet fset_n(cd* const* e, int n) {
  FSet fs{};
  for (int i = 0; i < n; ++i) { fs.e[i] = e[i]; fs.rs[i] = nullptr; }
  fs.n = n;
  return fs;
}
// the real-to-half-complex sum scaled by `scale` instead of 1/np (the adjoint's FFTs), of n <= 6 buffers
int launch_hfft_fwd_scaled_n(cd* const* e, int n, double scale) {
  if (n < 1 || n > FS_MAX) return set_error(MLG_EPARAM, "horizontal_fft: 1 to 6 fields per batch");
  const FSet fs = fset_n(e, n);
  return G.precision == MLG_MIXED ? hfft_t<MixFT>(fs, -1, scale) : hfft_t<double>(fs, -1, scale);
}
int launch_hfft_fwd_scaled(cd* e, double scale) { return launch_hfft_fwd_scaled_n(&e, 1, scale); }
// the half-complex-to-real sum (unnormalised, Nyquist slot kept times np), on n <= 6 raw buffers
int launch_hfft_bwd_buf_n(cd* const* e, int n) {
  if (n < 1 || n > FS_MAX) return set_error(MLG_EPARAM, "horizontal_fft: 1 to 6 fields per batch");
  const FSet fs = fset_n(e, n);
  return G.precision == MLG_MIXED ? hfft_t<MixFT>(fs, +1, 1.0) : hfft_t<double>(fs, +1, 1.0);
}
int launch_hfft_bwd_buf(cd* e) { return launch_hfft_bwd_buf_n(&e, 1); }
// the z sum of n <= 6 buffers, any direction and scale
int launch_vfft_scaled_n(cd* const* e, int n, int dir, double scale) {
  if (n < 1 || n > FS_MAX) return set_error(MLG_EPARAM, "vertical_fft: 1 to 6 fields per batch");
  return vfft_any(fset_n(e, n), dir, scale);
}

}  // namespace mlg
