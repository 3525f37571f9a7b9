// xs_common.cuh — arithmetic of the exact-slice (Ozaki) tensor-core contractions shared by
// xs_radial.cu and xs_vec2tp.cu.
//
// A value x with |x| < 2^E becomes the integer X = round(x 2^(nb - E)) of nb = w NS bits (|X| <= 2^nb),
// and X is cut into NS two's-complement digits of w bits, most significant first:
//   X = d_0 2^(w (NS-1)) + sum_{s>0} d_s 2^(w (NS-1-s)),  d_0 = X >> w (NS-1) in [-2^w, 2^w],
//   d_s in [0, 2^w) for s > 0.
// Every digit is an exact BF16 and every digit product an exact FP32 integer of magnitude <= 2^(2w), so
// a K-term sum of the products of one digit order stays exact while K (pairs of the order) 2^(2w) < 2^24.
// All conversions run on the integer and FP32 pipes: GB300 issues FP64 at about 2 operations per clock
// per SM.
#pragma once
#include "common.cuh"
#include <cstdint>
#include <type_traits>

namespace mlg {

// exponent bound of a magnitude bit pattern: |v| < 2^E for E = exponent field - 1022
__device__ __forceinline__ int xs_ebound(unsigned long long absbits) { return (int)(absbits >> 52) - 1022; }

// x 2^(nb - E) rounded to the nearest integer (halves away from zero) for |x| < 2^E (nb <= 63), from
// the FP64 bit pattern; zero, subnormal and non-finite inputs and E <= -2000 (an all-zero row or
// column) give 0.  Rounding, not truncation: a truncated fixed-point operand carries a one-signed bias
// of half a unit, and a K-term contraction against a table of one sign sums it coherently (K units
// instead of sqrt(K)), which the inverse Laplacian of the projection's chi then magnified.
__device__ __forceinline__ long long xs_fix(double x, int E, int nb) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0 || e == 0x7FF || E <= -2000) return 0;
  const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = e - 1075 + nb - E;     // |x| 2^(nb - E) = M 2^sh, and M 2^sh < 2^nb
  unsigned long long X;
  if (sh >= 0) X = (sh <= 10) ? (M << sh) : 0ull;  // sh < nb - 52 <= 11 when |x| < 2^E
  else X = (sh > -63) ? ((M + (1ull << (-sh - 1))) >> (-sh)) : 0ull;
  return (b >> 63) ? -(long long)X : (long long)X;
}

// the FP32 value of a small integer (|d| < 2^22), exactly, on the FP32 pipe
__device__ __forceinline__ float xs_i2f(int d) { return __int_as_float(0x4B400000 + d) - 12582912.0f; }

// the NS digits of X as FP32 values (each exact, so its BF16 pattern is the top half of its bits)
template <int NS>
__device__ __forceinline__ void xs_digits_f(long long X, int w, float* f) {
  const unsigned mask = (1u << w) - 1u;
  f[0] = xs_i2f((int)(X >> (w * (NS - 1))));
#pragma unroll
  for (int s = 1; s < NS; ++s) f[s] = xs_i2f((int)((unsigned)(X >> (w * (NS - 1 - s))) & mask));
}
// two FP32 digit values as one packed BF16 pair (a low, b high)
__device__ __forceinline__ uint32_t xs_pack(float a, float b) { return __byte_perm(__float_as_uint(a), __float_as_uint(b), 0x7632); }

// the exact integer value of an FP32 accumulator entry (integral, |x| < 2^24)
__device__ __forceinline__ int xs_f2i(float x) { return __float2int_rn(x); }

// f(std::integral_constant<int, 0>()), ..., f(std::integral_constant<int, N-1>())
template <int I, int N, class F> __device__ __forceinline__ void xs_static_for_(F& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>());
    xs_static_for_<I + 1, N>(f);
  }
}
template <int N, class F> __device__ __forceinline__ void xs_static_for(F f) { xs_static_for_<0, N>(f); }

// x 2^s for s >= 0, floor(x 2^s) for s < 0
__device__ __forceinline__ long long xs_shl(long long x, int s) { return s >= 0 ? (x << s) : (x >> (-s)); }

// T 2^e2 rounded once to FP64 (round to nearest even), T a signed 64-bit integer; magnitudes below the
// normal range flush to zero.  Branch-free on the integer pipe: normalise |T| so that its top bit is
// bit 63, keep 53 bits, round on the 11 below them, and let the implicit bit (and a rounding carry)
// add into the exponent field.
__device__ __forceinline__ double xs_i64_to_double(long long T, int e2) {
  const unsigned long long sign = (unsigned long long)T & 0x8000000000000000ull;
  const unsigned long long a = T < 0 ? 0ull - (unsigned long long)T : (unsigned long long)T;
  const int lz = __clzll((long long)a);
  const unsigned long long n = a << (lz & 63);                    // bit 63 set (a != 0)
  unsigned long long m = n >> 11;                                 // 53 bits, the implicit one on top
  const unsigned long long rb = (n >> 10) & 1ull, st = (n & 0x3FFull) != 0ull;
  m += rb & (st | (m & 1ull));
  const long long ex = (long long)(1023 + 63 - lz + e2);          // biased exponent of 2^(top bit)
  const unsigned long long bits = ((unsigned long long)(ex - 1) << 52) + m;
  if (a == 0ull || ex <= 0) return __longlong_as_double((long long)sign);
  if (ex >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sign | bits));
}

// y 2^e2 as FP64, exactly (FP32 subnormals and results below the normal range give zero)
__device__ __forceinline__ double xs_f2d_scaled(float y, int e2) {
  const unsigned f = __float_as_uint(y);
  const unsigned e = (f >> 23) & 0xFFu;
  if (e == 0u) return 0.0;
  const int ex = (int)e + 896 + e2;   // FP64 exponent field
  if (ex <= 0) return 0.0;
  const unsigned sign = f & 0x80000000u, m = f & 0x7FFFFFu;
  const unsigned hi = sign | ((unsigned)min(ex, 2047) << 20) | (m >> 3);
  return __hiloint2double((int)hi, (int)(m << 29));
}

// double-float accumulation of exact FP32 terms: (hi, lo) += x (Knuth's two-sum; lo collects the
// rounding errors, which are exact)
__device__ __forceinline__ void xs_df_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x), v = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, v)), __fsub_rn(x, v));
  hi = s;
  lo = __fadd_rn(lo, e);
}

// sum_d G_d 2^(-w d) of NO exact accumulator orders in double-float, then times 2^e2 as FP64 (about 46
// bits: enough for the mixed form's 35-bit digits; the plain form combines in 64-bit integers)
template <int NO>
__device__ __forceinline__ void xs_orders_df(const float* g, int w, float& hi, float& lo) {
  hi = g[0];
  lo = 0.f;
#pragma unroll
  for (int d = 1; d < NO; ++d) xs_df_add(hi, lo, g[d] * __int_as_float((127 - w * d) << 23));
}
__device__ __forceinline__ double xs_df_to_double(float hi, float lo, int e2) {
  return xs_f2d_scaled(hi, e2) + xs_f2d_scaled(lo, e2);
}

}  // namespace mlg
