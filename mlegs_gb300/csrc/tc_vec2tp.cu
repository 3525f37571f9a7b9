// tc_vec2tp.cu — the mixed form's projection contraction (vector_projection, mlegs_scalar_ops.f90:
// 1402-1438, with the eomul / oemul folds :2067-2145) for m >= 1 on the 5th-generation tensor cores.
//
// For each m and row parity par, rows j = 2t + par, radial points i < nr/2, z columns n:
//   psi = -i m V.F_s(ur) - D.F_o(up)
//   chi =  i k D.F_o(ur) + m k V.F_s(up) - T.F_s(uz)
// F_s / F_o fold ur(i) with ur(nr-1-i) by the row's own / the other parity's sign.
//
// psi and chi each take one TMEM accumulator, with every factor applied exactly or once:
//   psi = (m V).(-i F_s(ur)) + D.(-F_o(up)),   chi = k [D.(i F_o(ur)) + (m V).F_s(up)] - T.F_s(uz);
// m V is split at kit init from the FP64 product, the factors -i, i, -1 are exact swaps and signs of
// the field operand, and k multiplies chi's accumulator once.  These four products use the three-way
// BF16 split of both operands (eight products with i + j <= 3, FP32 accumulation).
//
// The T.F_s(uz) term needs more than FP32: chi ends with an inverse Laplacian that lifts its rounding
// into chi's weak low modes.  It runs as an exact integer-slice product (the Ozaki scheme): every row
// of T has a power-of-two scale 2^e_j and every column of F_s(uz) one of 2^f_n, and both are cut into
// NS signed digits of w bits, each an integer of magnitude < 2^w, exact in BF16.  A digit product is
// < 2^(2w), a sum over the nr/2 radial points and the <= NS digit pairs of one order d = s + t stays
// below 2^24, so each order's FP32 accumulator is exact; the orders are combined in double-float:
//   T.F = 2^(e_j + f_n - 2w) sum_d 2^(-w d) G_d,  G_d = sum_{s+t=d} sum_i a_t(j,i) b_s(i,n).
// With NS = 6 digits of w = 7 bits (6 when nr/2 > 173, keeping the orders exact) the term carries
// 42 (36) bits.
//
// Engine: one CTA per (m, parity, 128-row tile, 8 complex z columns), 256 threads (warp w takes role
// w % 4 in the staging -- ur, up, Re uz, Im uz -- for half the K of each group), about 64 KiB of
// shared memory and 128 TMEM columns, three CTAs per SM.  Per K chunk of
// 16 radial points the table tiles (V, D splits and T digits, laid out at kit init in the UMMA
// canonical K-major layout) arrive by one bulk copy on an mbarrier; the threads fold and split the
// field operand; one thread issues 53 tcgen05.mma (M = 128, N = 16, K = 16).  Every wait is bounded.
#include "common.cuh"
#include "tc_common.cuh"
#include <cstdint>

namespace mlg {

constexpr int PV_KC = 16;                  // K chunk (radial points): one MMA K step
constexpr int PV_NZ = 8;                   // complex z columns per CTA
constexpr int PV_N = 2 * PV_NZ;            // real columns (N of the MMA)
constexpr int PV_NS = 6;                   // digits of the T term
constexpr int PV_RW = 2;                   // warps per staging role
constexpr int PV_THREADS = 128 * PV_RW;
constexpr int PV_SBO = PV_KC * 16;         // 8 rows x 16 K x 2 B between 8-row core-matrix groups
constexpr int PV_LBO = 128;                // between the two 8-K core matrices of a row group
__host__ __device__ constexpr int pv_off(int row, int k) {
  return (row >> 3) * PV_SBO + (k >> 3) * PV_LBO + (row & 7) * 16 + (k & 7) * 2;
}
constexpr int PV_ATILE = 128 * PV_KC * 2;  // 4 KiB
constexpr int PV_BTILE = PV_N * PV_KC * 2; // 512 B
constexpr int PV_NA = 6 + PV_NS;           // A tiles per chunk: V s0..2, D s0..2, T digits 0..5
constexpr int PV_NB = 12 + PV_NS;          // B tiles: psi1 (3), psi2 (3), chi1 (3), chi2 (3), uz digits
constexpr int PV_TMEM_COLS = 128;          // psi, chi, then the NS digit orders, N columns each
static_assert((2 + PV_NS) * PV_N <= PV_TMEM_COLS, "TMEM columns");
constexpr int PV_KQ = PV_KC * PV_NZ / (32 * PV_RW);   // consecutive K per staging item

// the NS signed w-bit digits of x / 2^fexp (|x| < 2^fexp), most significant first, by integer ops
__device__ __forceinline__ void pv_digits(double x, int fexp, int w, int* d) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int e = (int)((b >> 52) & 0x7FF);
  unsigned long long X = 0;
  const int nb = w * PV_NS;
  if (e != 0 && e != 0x7FF) {
    unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    int sh = e - 1075 + nb - fexp;   // X = floor(|x| 2^(nb - fexp)) = M 2^sh, sh < 0 when |x| < 2^fexp
    if (sh < 0) X = (sh > -64) ? (M >> (-sh)) : 0ull;
    else X = (1ull << nb) - 1;       // out of range: saturate (not reached with the scales below)
    if (X >= (1ull << nb)) X = (1ull << nb) - 1;
  }
  const int sg = (b >> 63) ? -1 : 1;
  const unsigned long long mask = (1ull << w) - 1;
#pragma unroll
  for (int s = 0; s < PV_NS; ++s) d[s] = sg * (int)((X >> (w * (PV_NS - 1 - s))) & mask);
}

// binary exponent bound of a magnitude bit pattern: |v| < 2^(E - 1022) for the FP64 exponent field E
__device__ __forceinline__ int pv_ebound(unsigned long long absbits) {
  return (int)(absbits >> 52) - 1022;
}

// ------------------------------------------------------------------------------------------------
// kit-time table images
// row scales: texp[(m-1)*2 + par][t] = e with max_i |T(i, 2t+par, m)| < 2^e
__global__ void k_pv_texp(const double* __restrict__ tT, int* __restrict__ texp, int nrh, int ne, int nrc, int npc,
                          int ntr) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int mp = blockIdx.y;              // (m - 1) * 2 + par
  int m = mp / 2 + 1, par = mp & 1;
  if (t >= ntr || m >= npc) return;
  int j = 2 * t + par;
  int nn = max(min(nrc, nrc - m), 0);
  unsigned long long mx = 0;
  if (j < nn)
    for (int i = 0; i < nrh; ++i) {
      unsigned long long v = (unsigned long long)__double_as_longlong(tT[i + (size_t)nrh * (j + (size_t)ne * m)]) &
                             0x7FFFFFFFFFFFFFFFull;
      mx = v > mx ? v : mx;
    }
  texp[(size_t)mp * ntr + t] = mx ? pv_ebound(mx) : -1000;
}

// tiles per (m - 1, par, row tile mt, chunk kc): [m V s0, s1, s2 | D s0, s1, s2 | T digits 0..NS-1]
__global__ void k_pv_table(const double* __restrict__ tV, const double* __restrict__ tD, const double* __restrict__ tT,
                           const int* __restrict__ texp, uint16_t* __restrict__ img, int nrh, int ne, int nrc, int nmt,
                           int nkc, int ntr, int w) {
  size_t blk = blockIdx.x;   // ((mp * nmt) + mt) * nkc + kc
  int kc = blk % nkc;
  int mt = (blk / nkc) % nmt;
  int mp = (int)(blk / ((size_t)nkc * nmt));
  int m = mp / 2 + 1, par = mp & 1;
  int nn = max(min(nrc, nrc - m), 0);
  uint8_t* base = (uint8_t*)img + blk * (size_t)(PV_NA * PV_ATILE);
  for (int idx = threadIdx.x; idx < 128 * PV_KC; idx += blockDim.x) {
    int k = idx % PV_KC, r = idx / PV_KC;
    int t = mt * 128 + r;
    int j = 2 * t + par, i = kc * PV_KC + k;
    double v = 0.0, dd = 0.0, tt = 0.0;
    int ex = -1000;
    if (j < nn && i < nrh) {
      size_t o = i + (size_t)nrh * (j + (size_t)ne * m);
      v = (double)m * tV[o]; dd = tD[o]; tt = tT[o];
      ex = texp[(size_t)mp * ntr + t];
    }
    int off = pv_off(r, k);
    double src[2] = {v, dd};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      double a = src[q];
      uint16_t s0 = bf16_rn((float)a);
      double r1 = a - (double)bf16_f(s0);
      uint16_t s1 = bf16_rn((float)r1);
      double r2 = r1 - (double)bf16_f(s1);
      uint16_t s2 = bf16_rn((float)r2);
      *(uint16_t*)(base + (q * 3 + 0) * PV_ATILE + off) = s0;
      *(uint16_t*)(base + (q * 3 + 1) * PV_ATILE + off) = s1;
      *(uint16_t*)(base + (q * 3 + 2) * PV_ATILE + off) = s2;
    }
    int dg[PV_NS];
    pv_digits(tt, ex, w, dg);
#pragma unroll
    for (int s = 0; s < PV_NS; ++s) *(uint16_t*)(base + (6 + s) * PV_ATILE + off) = bf16_rn((float)dg[s]);
  }
}

// ------------------------------------------------------------------------------------------------
struct PvSmem {
  uint8_t a[PV_NA * PV_ATILE];   // 48 KiB, bulk-copied
  uint8_t b[PV_NB * PV_BTILE];   // 18 KiB, written by the threads
  int fexp[PV_N];                // column scales of F_s(uz)
  unsigned long long red[PV_THREADS / PV_NZ][PV_N];
  uint64_t bar_a, bar_mma;
  uint32_t tmem;
};

// PV_KQ consecutive K of one B row as three BF16 splits into tiles t0, t0+1, t0+2
__device__ __forceinline__ void pv_store_split(uint8_t* b, int t0, int n, int k0, const float* v) {
  static_assert(PV_KQ == 2, "staging items of 2 K");
  uint32_t w[3];
  split3x2(v[0], v[1], w);
#pragma unroll
  for (int s = 0; s < 3; ++s) *(uint32_t*)(b + (t0 + s) * PV_BTILE + pv_off(n, k0)) = w[s];
}

// a + b in double-float (Knuth two-sum, renormalised); b exact float
__device__ __forceinline__ float2 pv_dfadd(float2 a, float b) {
  float s = __fadd_rn(a.x, b), v = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, v)), __fsub_rn(b, v));
  e = __fadd_rn(e, a.y);
  float h = __fadd_rn(s, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ float pv_pow2(int e) {   // 2^e as float, 0 below the normal range
  return e < -126 ? 0.f : (e > 127 ? __uint_as_float(0x7F800000u) : __uint_as_float((uint32_t)(e + 127) << 23));
}

// grid (z tiles, 2 * nmt, npc - 1): blockIdx.y = mt * 2 + par, m = blockIdx.z + 1
__global__ void __launch_bounds__(PV_THREADS, 3) k_pv_contract(
    const double2* __restrict__ ur, const double2* __restrict__ up, const double2* __restrict__ uz,
    double2* __restrict__ psi, double2* __restrict__ chi, const uint16_t* __restrict__ img, const int* __restrict__ texp,
    const double* __restrict__ ak, int nr, int nrh, int nrdim, int npdim, int nzdim, int nrc, int nzc, int nzcu,
    int nmt, int nkc, int ntr, int w, int* __restrict__ status) {
  extern __shared__ __align__(1024) uint8_t pv_smem_raw[];
  PvSmem& sm = *reinterpret_cast<PvSmem*>(pv_smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int z0 = blockIdx.x * PV_NZ, par = blockIdx.y & 1, mt = blockIdx.y >> 1, m = blockIdx.z + 1;
  const int nn = max(min(nrc, nrc - m), 0);
  if (2 * (mt * 128) + par >= nn) return;
  if (tid == 0) {
    mbar_init(&sm.bar_a, 1);
    mbar_init(&sm.bar_mma, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(&sm.tmem, PV_TMEM_COLS);
    tmem_relinquish();
  }
  const float ss = par ? -1.f : 1.f;   // own-parity fold sign
  // column scales of F_s(uz): |uz(i) +- uz(nr-1-i)| <= 2 max(|uz(i)|, |uz(nr-1-i)|)
  {
    const int zz = tid % PV_NZ, g = tid / PV_NZ, z = z0 + zz;
    unsigned long long mr = 0, mi = 0;
    if (z < nzdim) {
      const double2* col = uz + (size_t)nrdim * (m + (size_t)npdim * z);
      for (int i = g; i < nrh; i += PV_THREADS / PV_NZ) {
        double2 a = col[i], b = col[nr - 1 - i];
        unsigned long long v;
        v = (unsigned long long)__double_as_longlong(a.x) & 0x7FFFFFFFFFFFFFFFull; mr = v > mr ? v : mr;
        v = (unsigned long long)__double_as_longlong(b.x) & 0x7FFFFFFFFFFFFFFFull; mr = v > mr ? v : mr;
        v = (unsigned long long)__double_as_longlong(a.y) & 0x7FFFFFFFFFFFFFFFull; mi = v > mi ? v : mi;
        v = (unsigned long long)__double_as_longlong(b.y) & 0x7FFFFFFFFFFFFFFFull; mi = v > mi ? v : mi;
      }
    }
    sm.red[g][2 * zz] = mr;
    sm.red[g][2 * zz + 1] = mi;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < PV_N) {
    unsigned long long mx = 0;
#pragma unroll
    for (int g = 0; g < PV_THREADS / PV_NZ; ++g) mx = sm.red[g][tid] > mx ? sm.red[g][tid] : mx;
    sm.fexp[tid] = mx ? pv_ebound(mx) + 1 : -1000;   // +1: the fold can double the magnitude
  }
  const uint32_t tmem = sm.tmem;
  // staging role of this warp: 0 ur, 1 up, 2 Re uz, 3 Im uz, two warps per role (half of each K group of
  // 4); lane: z column zz, K group kg; the item's K: kbase .. kbase + PV_KQ - 1 of the chunk
  const int role = warp & 3, half = warp >> 2, zz = lane % PV_NZ, kg = lane / PV_NZ;
  const int kbase = kg * (PV_KQ * PV_RW) + half * PV_KQ;
  const int z = z0 + zz;
  const bool zok = z < nzdim;
  const size_t cbase = (size_t)nrdim * (m + (size_t)npdim * (zok ? z : 0));
  float2 fa[PV_KQ], fb[PV_KQ];   // roles 0, 1: the two halves of ur / up (FP32)
  double da[PV_KQ], db[PV_KQ];   // roles 2, 3: the two halves of the uz component (FP64)
  auto fetch = [&](int kc) {
#pragma unroll
    for (int q = 0; q < PV_KQ; ++q) {
      int i = kc * PV_KC + kbase + q;
      bool ok = zok && i < nrh;
      if (role < 2) {
        const double2* src = role == 0 ? ur : up;
        fa[q] = ok ? ld_c32(src + cbase + i) : make_float2(0.f, 0.f);
        fb[q] = ok ? ld_c32(src + cbase + nr - 1 - i) : make_float2(0.f, 0.f);
      } else {
        const double* src = reinterpret_cast<const double*>(uz) + (role - 2);
        da[q] = ok ? src[2 * (cbase + i)] : 0.0;
        db[q] = ok ? src[2 * (cbase + nr - 1 - i)] : 0.0;
      }
    }
  };
  bool ok = true;
  const uint8_t* img_b = (const uint8_t*)img + (((size_t)((m - 1) * 2 + par) * nmt + mt) * nkc) * (size_t)(PV_NA * PV_ATILE);
  __syncthreads();   // fexp visible
  fetch(0);
  for (int kc = 0; kc < nkc; ++kc) {
    if (tid == 0) {
      mbar_expect_tx(&sm.bar_a, PV_NA * PV_ATILE);
      bulk_g2s(sm.a, img_b + (size_t)kc * (PV_NA * PV_ATILE), PV_NA * PV_ATILE, &sm.bar_a);
    }
    if (role < 2) {
      float v0[PV_KQ], v1[PV_KQ], v2[PV_KQ], v3[PV_KQ];
#pragma unroll
      for (int q = 0; q < PV_KQ; ++q) {
        float2 fs = make_float2(fa[q].x + ss * fb[q].x, fa[q].y + ss * fb[q].y);
        float2 fo = make_float2(fa[q].x - ss * fb[q].x, fa[q].y - ss * fb[q].y);
        if (role == 0) {   // psi1 = -i F_s(ur): columns (re, im) = (Im, -Re); chi1 = i F_o(ur): (-Im, Re)
          v0[q] = fs.y; v1[q] = -fs.x;
          v2[q] = -fo.y; v3[q] = fo.x;
        } else {           // psi2 = -F_o(up); chi2 = F_s(up)
          v0[q] = -fo.x; v1[q] = -fo.y;
          v2[q] = fs.x; v3[q] = fs.y;
        }
      }
      const int tp = role == 0 ? 0 : 3, tc = role == 0 ? 6 : 9;
      pv_store_split(sm.b, tp, 2 * zz, kbase, v0);
      pv_store_split(sm.b, tp, 2 * zz + 1, kbase, v1);
      pv_store_split(sm.b, tc, 2 * zz, kbase, v2);
      pv_store_split(sm.b, tc, 2 * zz + 1, kbase, v3);
    } else {
      const int n = 2 * zz + (role - 2);
      const int fe = sm.fexp[n];
      uint32_t h[PV_NS][PV_KQ];
#pragma unroll
      for (int q = 0; q < PV_KQ; ++q) {
        double f = ss > 0.f ? da[q] + db[q] : da[q] - db[q];   // F_s(uz), FP64
        int dg[PV_NS];
        pv_digits(f, fe, w, dg);
#pragma unroll
        for (int s = 0; s < PV_NS; ++s) h[s][q] = bf16_small_int(dg[s]);
      }
#pragma unroll
      for (int s = 0; s < PV_NS; ++s)
        *(uint32_t*)(sm.b + (12 + s) * PV_BTILE + pv_off(n, kbase)) = h[s][0] | (h[s][1] << 16);
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      ok = ok && mbar_wait(&sm.bar_a, kc & 1);
      tc_fence_after();
      if (ok) {
        const uint32_t idesc = idesc_bf16(128, PV_N);
        const uint32_t a0 = smem_u32(sm.a), b0 = smem_u32(sm.b);
        auto A = [&](int t) { return sdesc(a0 + t * PV_ATILE, PV_LBO, PV_SBO); };
        auto B = [&](int t) { return sdesc(b0 + t * PV_BTILE, PV_LBO, PV_SBO); };
        // split pairs (i, j) with i + j <= 3: the omitted (2, 2) term is 2^-32 relative
        const int SA[8] = {0, 0, 1, 0, 1, 2, 1, 2}, SB[8] = {0, 1, 0, 2, 1, 0, 2, 1};
#pragma unroll
        for (int p = 0; p < 8; ++p) {
          uint32_t acc = (kc > 0 || p > 0) ? 1u : 0u;
          umma_bf16(tmem + 0, A(0 + SA[p]), B(0 + SB[p]), idesc, acc);    // psi: mV . psi1
          umma_bf16(tmem + 0, A(3 + SA[p]), B(3 + SB[p]), idesc, 1u);     //      D . psi2
          umma_bf16(tmem + PV_N, A(3 + SA[p]), B(6 + SB[p]), idesc, acc); // chi/k: D . chi1
          umma_bf16(tmem + PV_N, A(0 + SA[p]), B(9 + SB[p]), idesc, 1u);  //        mV . chi2
        }
#pragma unroll
        for (int d = 0; d < PV_NS; ++d)
#pragma unroll
          for (int t = 0; t <= d; ++t)   // T digit t times uz digit d - t
            umma_bf16(tmem + (2 + d) * PV_N, A(6 + t), B(12 + d - t), idesc, (kc > 0 || t > 0) ? 1u : 0u);
      }
      umma_commit(&sm.bar_mma);
    }
    if (kc + 1 < nkc) fetch(kc + 1);
    bool done = mbar_wait(&sm.bar_mma, kc & 1);
    if (!done || (tid == 0 && !ok)) atomicExch(status, 2);
    __syncthreads();
  }
  tc_fence_after();
  // epilogue: warp w reads TMEM lanes 32 (w % 4) .. (rows t = mt*128 + 32 (w % 4) + lane) and the column
  // blocks cb = w / 4 (mod PV_RW)
  const int t = mt * 128 + (warp & 3) * 32 + lane;
  const int j = 2 * t + par;
  const bool rok = j < nn && t < ntr;
  const int ej = rok ? texp[(size_t)((m - 1) * 2 + par) * ntr + t] : -1000;
  const uint32_t lrow = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll 1
  for (int cb = half; cb < PV_N / 8; cb += PV_RW) {
    float pv[8], cv[8], g[PV_NS][8];
    tmem_ld8(tmem + lrow + cb * 8, pv);
    tmem_ld8(tmem + lrow + PV_N + cb * 8, cv);
#pragma unroll
    for (int d = 0; d < PV_NS; ++d) tmem_ld8(tmem + lrow + (2 + d) * PV_N + cb * 8, g[d]);
    if (!rok) continue;
#pragma unroll
    for (int c = 0; c < 8; c += 2) {
      const int n = cb * 8 + c, zc = z0 + n / 2;
      if (zc >= nzdim) continue;
      const int kk = zc + 1;
      if (!(kk <= nzc || kk >= nzcu)) continue;
      const float kz = d2f_fast(ak[zc]);
      double out[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float2 s = make_float2(0.f, 0.f);
#pragma unroll
        for (int d = PV_NS - 1; d >= 0; --d) s = pv_dfadd(s, g[d][c + q] * pv_pow2(-w * d));
        const float sc = pv_pow2(ej + sm.fexp[n + q] - 2 * w);
        s.x *= sc; s.y *= sc;
        // chi = chi' - T.F_s(uz), in double-float, rounded once to FP64
        float2 r = pv_dfadd(make_float2(-s.x, -s.y), kz * cv[c + q]);
        out[q] = f2d_fast(r.x) + f2d_fast(r.y);
      }
      size_t o = j + (size_t)nrdim * (m + (size_t)npdim * zc);
      psi[o] = make_double2(f2d_fast(pv[c]), f2d_fast(pv[c + 1]));
      chi[o] = make_double2(out[0], out[1]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, PV_TMEM_COLS);
}

// ------------------------------------------------------------------------------------------------
struct PvImg {
  uint16_t* p = nullptr;
  int* texp = nullptr;
  size_t bytes = 0, tbytes = 0;
  int nrc = -1, npc = -1, w = 0;
};
static PvImg g_pv;

void pv_free() {
  if (g_pv.p) dfree(g_pv.p, g_pv.bytes);
  if (g_pv.texp) dfree(g_pv.texp, g_pv.tbytes);
  g_pv = PvImg();
}

// psi, chi: rows of m >= 1 written (zeroed by the caller); the m = 0 plane is the caller's
int pv_contract(const cd* ur, const cd* up, const cd* uz, cd* psi, cd* chi, int nrc, int npc) {
  if (npc <= 1) return 0;
  const int ntr = (nrc + 1) / 2;                 // rows of one parity
  const int nmt = cdiv(ntr, 128), nkc = cdiv(G.nrh, PV_KC);
  // digit width: (digit pairs of one order) x (radial points) x (2^w - 1)^2 < 2^24 keeps the orders exact
  const int w = ((double)PV_NS * G.nrh * 127.0 * 127.0 < 16777216.0) ? 7 : 6;
  if ((double)PV_NS * G.nrh * 63.0 * 63.0 >= 16777216.0)
    return set_error(MLG_ESIZE, "vec2tp: too many radial points for the exact T-term digits");
  if (g_pv.nrc != nrc || g_pv.npc != npc || !g_pv.p) {
    pv_free();
    g_pv.bytes = (size_t)(npc - 1) * 2 * nmt * nkc * PV_NA * PV_ATILE;
    g_pv.tbytes = (size_t)(npc - 1) * 2 * ntr * sizeof(int);
    MLG_TRY(dmalloc((void**)&g_pv.p, g_pv.bytes));
    MLG_TRY(dmalloc((void**)&g_pv.texp, g_pv.tbytes));
    k_pv_texp<<<dim3(cdiv(ntr, 128), (npc - 1) * 2), 128, 0, G.stream>>>(G.tT, g_pv.texp, G.nrh, G.ne, nrc, npc, ntr);
    MLG_LAUNCH();
    k_pv_table<<<(npc - 1) * 2 * nmt * nkc, 256, 0, G.stream>>>(G.tV, G.tD, G.tT, g_pv.texp, g_pv.p, G.nrh, G.ne, nrc, nmt,
                                                                nkc, ntr, w);
    MLG_LAUNCH();
    g_pv.nrc = nrc; g_pv.npc = npc; g_pv.w = w;
  }
  size_t sm = sizeof(PvSmem) + 1024;
  MLG_CUDA(cudaFuncSetAttribute(k_pv_contract, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  dim3 grid(cdiv(G.nzdim, PV_NZ), 2 * nmt, npc - 1);
  int* st = (int*)(G.dscal + DS_FLAG + 1) + 1;
  k_pv_contract<<<grid, PV_THREADS, sm, G.stream>>>(ur, up, uz, psi, chi, g_pv.p, g_pv.texp, G.ak, G.nr, G.nrh, G.nrdim,
                                                    G.npdim, G.nzdim, nrc, G.chopzl, G.chopzu, nmt, nkc, ntr, g_pv.w, st);
  MLG_LAUNCH();
  return 0;
}

}  // namespace mlg
