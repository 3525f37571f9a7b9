// xs_radial.cu — the radial Legendre contractions as exact-slice products on the 5th-generation tensor
// cores (rtrans_forward, mlegs_scalar_ops.f90:1852-1927; rtrans_backward, :1931-2008).
//
// Method (the Ozaki scheme of error-free matrix products).  Every row of the table operand A has a
// power-of-two scale 2^EA (|A(row, k)| < 2^EA) and every column of the field operand B one of 2^EB;
// both are cut into NS signed digits of w bits,
//   A(row, k) ~ 2^(EA - nb) sum_t a_t 2^(w (NS-1-t)),   nb = w NS,  a_t integer, |a_t| < 2^w,
// by rounding A 2^(nb - EA) to an integer (so the representation error is at most 2^(EA - nb - 1)).  Every digit is
// an exact BF16 and every digit product an exact FP32 integer.  The products of one digit order
// d = t + s are summed over K in their own FP32 accumulator in tensor memory,
//   G_d = sum_{t+s=d} sum_k a_t(row, k) b_s(k, n),
// which stays exact while K * (d+1) * 2^(2w) < 2^24 (w = 7 up to K ~ 113 with nine orders, w = 6
// beyond).  Orders d < NO = NS are kept; the epilogue forms the exact integer
//   T = sum_d G_d 2^(w (NO-1-d))
// in 64-bit integer arithmetic (the lowest orders shifted right when T would pass 2^62: a loss below
// 2^-60 of the largest term) and rounds T 2^(EA + EB - w (NO+1)) once to FP64, on the integer pipe.
// The result differs from the exact product of the FP64 operands by about 2^-(w NS - 1) of
// max|A(row,:)| max|B(:,n)| per term: NS = 9, w = 7 (63 bits) is an FP64-grade product (the plain
// form), NS = 6 (42 bits) the mixed form's.  No floating-point rounding happens anywhere else: the
// forward fold f(i) +- f(nr-1-i) is an exact integer sum of the two rounded samples, and the
// quadrature weights are folded into the table (A = pf w, one FP64 rounding at kit init).
//
// Forward: per m and row parity par, C_par(t, n) = sum_{i < nr/2} A_par(t, i) B_par(i, n) with
//   A_par(t, i) = pf(i, 2t+par, m) w(i),  B_par(i, n) = f(i) + (-1)^par f(nr-1-i)  (n: re/im of z),
//   c(2t+par, m, z) = C_par(t, n); one column scale per n for both parities (the fold may double),
//   one row scale per (par, t).
// Backward: D_par(i, n) = sum_t A_par(i, t) B_par(t, n) with A_par(i, t) = pf(i, 2t+par, m),
//   B_par(t, n) = c(2t+par, m, z); f(i) = D_0 + D_1, f(nr-1-i) = D_0 - D_1, formed exactly in the
//   integers, so both parities share one row scale per i and one column scale per n; the log term
//   ln * lnx(i) is added at m = 0 (trans, :194).
//
// Engine: a persistent grid of one CTA per SM (512 threads).  A work item is one (m, tile of NZ complex
// z columns); the CTA
//  * bulk-copies the item's FP64 field columns (NZ runs of consecutive r, each contiguous in HBM) into
//    shared memory on the TMA engine, completing on an mbarrier;
//  * reduces the column scales there;
//  * per row tile and K chunk of 16: the table digits of both parities arrive by one bulk copy (pre-split
//    at kit init in the UMMA canonical no-swizzle K-major layout), the threads cut the field digits
//    from shared memory into the same layout (each warp's 32 stores in 32 banks), and one thread issues
//    the chunk's tcgen05.mma, commits, and as soon as the other stage is free starts the next chunk's
//    table copy into it; the stages are double-buffered, so the digits and the table copy of chunk
//    k + 1 overlap the MMAs of chunk k.  The field digits of a parity lie side by side (digit s at
//    rows s N .. s N + N-1 of the B operand) and so do the accumulators of the orders, so table digit
//    t meets all field digits s <= NO-1-t in one MMA of M = 128, N = (NO - t) 2 NZ, K = 16 whose
//    column block s lands on order t + s: NO MMAs per parity and chunk instead of NO (NO+1)/2, and
//    each table tile is read from shared memory once;
//  * reads the 2 NO accumulators back with tcgen05.ld and writes FP64 results.
// Every wait is bounded (about a second of SM clock): a timeout sets the library's timeout word and the
// CTA stops issuing work, waits (bounded) for what it issued, frees its tensor memory and returns.
#include "common.cuh"
#include "tc_common.cuh"
#include "xs_common.cuh"
#include <cstdint>

namespace mlg {

constexpr int XS_KC = 16;                         // K per chunk: one MMA K step
constexpr int XS_THREADS = 512;
constexpr int XS_ATILE = 128 * XS_KC * 2;         // 4 KiB: 128 rows x 16 K of BF16
constexpr int XS_SBO = XS_KC * 16;                // between 8-row core-matrix groups
constexpr int XS_LBO = 128;                       // between the two 8-K core matrices of a row group
__host__ __device__ constexpr int xs_off(int row, int k) {
  return (row >> 3) * XS_SBO + (k >> 3) * XS_LBO + (row & 7) * 16 + (k & 7) * 2;
}

// ------------------------------------------------------------------------------------------------
// kit-time table images
// fwd rows (par, t), K = i: A = pf(i, 2t+par, m) w(i); bwd rows i, K = t: A = pf(i, 2t+par, m)
__device__ __forceinline__ double xs_a(const double* __restrict__ pf, const double* __restrict__ w, int mode, int row,
                                       int k, int par, int m, int nn, int nrh, int ne) {
  const int i = mode == 0 ? k : row, t = mode == 0 ? row : k, j = 2 * t + par;
  if (j >= nn || i >= nrh) return 0.0;
  const double v = pf[i + (size_t)nrh * (j + (size_t)ne * m)];
  return mode == 0 ? v * w[i] : v;
}

// row scales: fwd aexp[(m * 2 + par) * nrp + t], bwd aexp[m * nrp + i] (both parities); -2000: all zero
__global__ void k_xs_aexp(const double* __restrict__ pf, const double* __restrict__ w, int* __restrict__ aexp, int mode,
                          int nrh, int ne, int nrc, int nrp, int nk) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y, nn = max(min(nrc, nrc - m), 0);
  if (row >= nrp) return;
  for (int p = 0; p < (mode == 0 ? 2 : 1); ++p) {
    unsigned long long mx = 0;
    for (int par = (mode == 0 ? p : 0); par <= (mode == 0 ? p : 1); ++par)
      for (int k = 0; k < nk; ++k) {
        unsigned long long v = (unsigned long long)__double_as_longlong(xs_a(pf, w, mode, row, k, par, m, nn, nrh, ne)) &
                               0x7FFFFFFFFFFFFFFFull;
        mx = v > mx ? v : mx;
      }
    aexp[(size_t)(mode == 0 ? m * 2 + p : m) * nrp + row] = mx ? xs_ebound(mx) : -2000;
  }
}

// digit tiles per (m, row tile mt, chunk kc): [par][digit t] of 128 rows x 16 K
template <int NS>
__global__ void k_xs_table(const double* __restrict__ pf, const double* __restrict__ w, const int* __restrict__ aexp,
                           uint16_t* __restrict__ img, int mode, int nrh, int ne, int nrc, int nmt, int nkc, int nrp,
                           int wbits) {
  const size_t blk = blockIdx.x;   // (m * nmt + mt) * nkc + kc
  const int kc = (int)(blk % nkc), mt = (int)((blk / nkc) % nmt), m = (int)(blk / ((size_t)nkc * nmt));
  const int nn = max(min(nrc, nrc - m), 0);
  uint8_t* base = (uint8_t*)img + blk * (size_t)(2 * NS * XS_ATILE);
  for (int idx = threadIdx.x; idx < 2 * 128 * XS_KC; idx += blockDim.x) {
    const int k = idx % XS_KC, r = (idx / XS_KC) % 128, par = idx / (XS_KC * 128);
    const int row = mt * 128 + r, kk = kc * XS_KC + k;
    int E = -2000;
    double a = 0.0;
    if (row < nrp) {
      E = aexp[(size_t)(mode == 0 ? m * 2 + par : m) * nrp + row];
      a = xs_a(pf, w, mode, row, kk, par, m, nn, nrh, ne);
    }
    float f[NS];
    xs_digits_f<NS>(xs_fix(a, E, wbits * NS), wbits, f);
#pragma unroll
    for (int t = 0; t < NS; ++t) *(uint16_t*)(base + (par * NS + t) * XS_ATILE + xs_off(r, k)) = (uint16_t)(__float_as_uint(f[t]) >> 16);
  }
}

// ------------------------------------------------------------------------------------------------
struct XsArgs {
  const double2* in;
  double2* out;
  const uint16_t* img;
  const int* aexp;
  const double* lnx;
  const double* lnp;
  int* status;
  int add_ln, nr, nrh, nrdim, npdim, nzdim, nrc, m0, npc, nmt, nkc, nrp, rawk, wbits, esh;
};

__device__ __forceinline__ bool xs_wait(uint64_t* bar, uint32_t phase, bool& ok) {
  if (!ok) return false;
  ok = mbar_wait(bar, phase);
  return ok;
}



// MODE 0 forward, 1 backward; NS digits, NO orders, NZ complex z columns per item
template <int MODE, int NS, int NO, int NZ>
__global__ void __launch_bounds__(XS_THREADS, 1) k_xs_rtrans(XsArgs a) {
  constexpr int N = 2 * NZ;                       // real columns (MMA N)
  constexpr int BT = N * XS_KC * 2;               // B digit tile bytes
  constexpr int ASTAGE = 2 * NS * XS_ATILE;
  constexpr int BSTAGE = 2 * NS * BT;
  constexpr int TCOLS = 2 * NO * N <= 32 ? 32 : 2 * NO * N <= 64 ? 64 : 2 * NO * N <= 128 ? 128 : 2 * NO * N <= 256 ? 256 : 512;
  constexpr int NW = XS_THREADS / 32;
  constexpr int CGW = N / 8 < 4 ? N / 8 : 4;      // column groups of 8 in the epilogue (one per 4 warps)
  constexpr int NDW = NW - 2;                     // digit warps: 2 .. NW-1
  constexpr int NDIG = NDW * 32;
  // staging blocks per chunk: (8 columns, 4 K pairs) and, backward, the parity (forward, a block writes
  // both parities from the same two samples)
  constexpr int NBLK = (MODE == 0 ? 1 : 2) * (N / 8) * 2;
  static_assert(2 * NO * N <= 512, "accumulators exceed tensor memory");
  static_assert(NO <= NS, "every order's first product (t = 0) resets its accumulator");
  static_assert(N % 16 == 0 && N >= 16 && N <= 32, "MMA N");
  static_assert(NW == 16, "the epilogue map assumes 16 warps");
  extern __shared__ __align__(1024) uint8_t xs_smem_raw[];
  uint8_t* sbase = (uint8_t*)(((uintptr_t)xs_smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = sbase;                                   // [2 stages][ASTAGE]
  uint8_t* sB = sA + 2 * ASTAGE;                         // [2 stages][BSTAGE]
  double* raw = (double*)(sB + 2 * BSTAGE);              // [NZ][rawk] complex (re, im)
  int* colexp = (int*)(raw + (size_t)2 * NZ * a.rawk);   // [N]
  uint64_t* bars = (uint64_t*)(colexp + 2 * N);         // raw, a[2], b[2], mma[2]
  uint32_t* tslot = (uint32_t*)(bars + 7);
  uint64_t* bar_raw = bars;
  uint64_t* bar_a = bars + 1;     // table stage filled (bulk copy)
  uint64_t* bar_b = bars + 3;     // field-digit stage written (the digit warps)
  uint64_t* bar_mma = bars + 5;   // the stage's MMAs completed (tcgen05.commit)

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int w = a.wbits, nb = w * NS;
  if (tid == 0) {
    mbar_init(bar_raw, 1);
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar_a + i, 1);
      mbar_init(bar_b + i, NDIG);
      mbar_init(bar_mma + i, 1);
    }
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tslot, TCOLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;
  uint32_t it = 0, raw_ph = 0;                  // chunk counter (stage and phase), raw-copy phase
  const int nzt = (a.nzdim + NZ - 1) / NZ;
  const int nitems = (a.npc - a.m0) * nzt;
  // the items of this CTA, skipping those without rows (every thread walks the same sequence)
  auto item_nn = [&](int item) { const int m = a.m0 + item / nzt; return max(min(a.nrc, a.nrc - m), 0); };
  auto next_item = [&](int item) {
    for (item += gridDim.x; item < nitems && item_nn(item) == 0; item += gridDim.x) {}
    return item;
  };
  auto issue_raw = [&](int item) {   // tid 0: the item's field columns into shared memory
    const int m = a.m0 + item / nzt, z0 = (item % nzt) * NZ;
    const int kraw = MODE == 0 ? a.nr : item_nn(item);
    fence_async_smem();
    uint32_t bytes = 0;
    for (int zz = 0; zz < NZ; ++zz)
      if (z0 + zz < a.nzdim) bytes += (uint32_t)kraw * 16u;
    mbar_expect_tx(bar_raw, bytes);
    for (int zz = 0; zz < NZ; ++zz)
      if (z0 + zz < a.nzdim)
        bulk_g2s(raw + (size_t)2 * zz * a.rawk, a.in + (size_t)a.nrdim * (m + (size_t)a.npdim * (z0 + zz)),
                 (uint32_t)kraw * 16u, bar_raw);
  };
  int item = blockIdx.x;
  while (item < nitems && item_nn(item) == 0) item += gridDim.x;
  if (tid == 0 && item < nitems) issue_raw(item);

  for (; item < nitems && ok; item = next_item(item)) {
    const int m = a.m0 + item / nzt, z0 = (item % nzt) * NZ;
    const int nn = item_nn(item);
    const int kraw = MODE == 0 ? a.nr : nn;     // field entries per column
    // K extent: fwd radial points, bwd rows of the even parity (the longer one)
    const int kext = MODE == 0 ? a.nrh : (nn + 1) / 2;
    const int nkc_m = (kext + XS_KC - 1) / XS_KC;
    const int nrows = MODE == 0 ? (nn + 1) / 2 : a.nrh;
    const int nmt_m = (nrows + 127) / 128;
    xs_wait(bar_raw, raw_ph, ok);
    raw_ph ^= 1;
    ok = __syncthreads_and(ok);   // every exit below is taken by the whole block
    if (!ok) break;
    // ---- column scales: XS_THREADS / N lanes of one warp per real column n (z = n/2, re/im = n&1)
    // reduce the largest exponent field (the high words of the staged FP64 samples) by warp shuffles
    {
      constexpr int TPC = XS_THREADS / N;
      static_assert(TPC == 16 || TPC == 32, "a column's lanes are a half or a whole warp");
      const int n = tid / TPC, sub = tid % TPC, zz = n >> 1;
      unsigned mx = 0;
      if (z0 + zz < a.nzdim) {
        const unsigned* hw = (const unsigned*)(raw + (size_t)2 * zz * a.rawk + (n & 1)) + 1;
        for (int i = sub; i < kraw; i += TPC) mx = max(mx, (hw[4 * i] >> 20) & 0x7FFu);
      }
      mx = __reduce_max_sync(TPC == 32 ? 0xFFFFFFFFu : (0xFFFFu << (lane & 16)), mx);
      // |x| < 2^(field - 1022) for every sample; an all-zero column gets -2000
      if (sub == 0) colexp[n] = mx ? (int)mx - 1022 + (MODE == 0 ? 1 : 0) : -2000;
    }
    __syncthreads();

    for (int mt = 0; mt < nmt_m && ok; ++mt) {
      const uint8_t* img_m = (const uint8_t*)a.img + ((size_t)m * a.nmt + mt) * a.nkc * (size_t)ASTAGE;
      const uint32_t it0 = it;
      if (warp == 0) {
        // ---- producer: the table chunks, each into its stage once the MMAs that read it before are done
        if (lane == 0) {
          for (int kc = 0; kc < nkc_m && ok; ++kc) {
            const uint32_t c = it0 + kc, s = c & 1;
            if (c >= 2) xs_wait(&bar_mma[s], ((c - 2) >> 1) & 1, ok);
            if (!ok) break;
            mbar_expect_tx(&bar_a[s], ASTAGE);
            bulk_g2s(sA + s * ASTAGE, img_m + (size_t)kc * ASTAGE, ASTAGE, &bar_a[s]);
          }
          // the next item's field columns, once the digit warps are done with these
          const int nxt = next_item(item);
          if (ok && mt == nmt_m - 1 && nxt < nitems) {
            const uint32_t c = it0 + nkc_m - 1;
            xs_wait(&bar_b[c & 1], (c >> 1) & 1, ok);
            if (ok) issue_raw(nxt);
          }
        }
        __syncwarp();
      } else if (warp == 1) {
        // ---- MMA issue: one thread, as soon as a stage's table and digits are in
        if (lane == 0) {
          for (int kc = 0; kc < nkc_m && ok; ++kc) {
            const uint32_t c = it0 + kc, s = c & 1;
            xs_wait(&bar_a[s], (c >> 1) & 1, ok);
            xs_wait(&bar_b[s], (c >> 1) & 1, ok);
            if (!ok) break;
            tc_fence_after();
            const uint32_t a0 = smem_u32(sA + s * ASTAGE), b0 = smem_u32(sB + s * BSTAGE);
            // table digit t times the field digits s = 0 .. NO-1-t in one MMA of N (NO - t) columns: the
            // field digits lie side by side in shared memory and the orders d = t + s side by side in
            // tensor memory, so the product of digit s lands on order t + s
#pragma unroll
            for (int par = 0; par < 2; ++par)
#pragma unroll
              for (int t = 0; t < NO; ++t) {
                const uint64_t ad = sdesc(a0 + (par * NS + t) * XS_ATILE, XS_LBO, XS_SBO);
                const uint64_t bd = sdesc(b0 + (par * NS) * BT, XS_LBO, XS_SBO);
                umma_bf16(tmem + (uint32_t)((par * NO + t) * N), ad, bd, idesc_bf16(128, (NO - t) * N),
                          (kc > 0 || t > 0) ? 1u : 0u);
              }
            umma_commit(&bar_mma[s]);
          }
        }
        __syncwarp();
      } else {
        // ---- field digits: a warp writes one (parity, 8 columns, 4 K pairs) block, its 32 four-byte
        // stores in 32 different banks
        const int dw = warp - 2;
        for (int kc = 0; kc < nkc_m && ok; ++kc) {
          const uint32_t c = it0 + kc, s = c & 1;
          if (c >= 2) xs_wait(&bar_mma[s], ((c - 2) >> 1) & 1, ok);
          if (!ok) break;
          uint8_t* bst = sB + s * BSTAGE;
          for (int blk = dw; blk < NBLK; blk += NDW) {
            const int par = MODE == 0 ? 0 : (blk & 1), bb = MODE == 0 ? blk : (blk >> 1);
            const int ng = bb % (N / 8), kh = bb / (N / 8);
            const int n = ng * 8 + (lane & 7), kp = kh * 4 + (lane >> 3), zz = n >> 1;
            const int E = colexp[n];
            const bool zok = (z0 + zz < a.nzdim) && E > -2000;
            const double* col = raw + (size_t)2 * zz * a.rawk + (n & 1);
            const int off = xs_off(n, 2 * kp);
            if (MODE == 0) {
              // B_par(i) = f(i) + (-1)^par f(nr-1-i) for both parities, exact in the integers
              float he[2][NS], ho[2][NS];
#pragma unroll
              for (int u = 0; u < 2; ++u) {
                const int i = kc * XS_KC + 2 * kp + u;
                long long x1 = 0, x2 = 0;
                if (zok && i < a.nrh) { x1 = xs_fix(col[2 * i], E, nb); x2 = xs_fix(col[2 * (a.nr - 1 - i)], E, nb); }
                xs_digits_f<NS>(x1 + x2, w, he[u]);
                xs_digits_f<NS>(x1 - x2, w, ho[u]);
              }
#pragma unroll
              for (int t = 0; t < NS; ++t) {
                *(uint32_t*)(bst + t * BT + off) = xs_pack(he[0][t], he[1][t]);
                *(uint32_t*)(bst + (NS + t) * BT + off) = xs_pack(ho[0][t], ho[1][t]);
              }
            } else {
              // B_par(t) = c(2t + par)
              float h[2][NS];
#pragma unroll
              for (int u = 0; u < 2; ++u) {
                const int j = 2 * (kc * XS_KC + 2 * kp + u) + par;
                xs_digits_f<NS>((zok && j < nn) ? xs_fix(col[2 * j], E, nb) : 0ll, w, h[u]);
              }
#pragma unroll
              for (int t = 0; t < NS; ++t) *(uint32_t*)(bst + (par * NS + t) * BT + off) = xs_pack(h[0][t], h[1][t]);
            }
          }
          fence_async_smem();
          mbar_arrive(&bar_b[s]);
        }
      }
      it = it0 + nkc_m;
      // ---- epilogue: every MMA of the tile has completed once the last chunk's commit has
      {
        const uint32_t lst = it - 1;
        xs_wait(&bar_mma[lst & 1], (lst >> 1) & 1, ok);
      }
      ok = __syncthreads_and(ok);
      if (!ok) break;
      tc_fence_after();
      const int lq = warp & 3, cg = warp >> 2;      // TMEM lane quarter, 8-column group
      // (a warp whose 32 rows all lie past the tile's valid rows has nothing to write)
      if (cg < CGW && mt * 128 + lq * 32 < nrows) {
        const int row = mt * 128 + lq * 32 + lane;
        const uint32_t lrow = (uint32_t)(lq * 32) << 16;
        const int c0 = cg * 8;
        {
          // the orders combined exactly in 64-bit integers, T = sum_d G_d 2^(w (NO-1-d) - esh), on the
          // integer pipe; T 2^(EA + EB + esh - w (NO+1)) is then rounded once to FP64
        long long T[2][8];
#pragma unroll
        for (int par = 0; par < 2; ++par)
#pragma unroll
          for (int c = 0; c < 8; ++c) T[par][c] = 0;
#pragma unroll
        for (int d = 0; d < NO; ++d) {
          const int sh = w * (NO - 1 - d) - a.esh;
          uint32_t g[2][8];
#pragma unroll
          for (int par = 0; par < 2; ++par) tmem_ld8_nw(tmem + lrow + (uint32_t)((par * NO + d) * N + c0), g[par]);
          tmem_wait_ld();
#pragma unroll
          for (int par = 0; par < 2; ++par)
#pragma unroll
            for (int c = 0; c < 8; ++c) T[par][c] += xs_shl((long long)xs_f2i(__uint_as_float(g[par][c])), sh);
        }
        const int eo = a.esh - w * (NO + 1);
        if (MODE == 0) {
#pragma unroll
          for (int par = 0; par < 2; ++par) {
            const int j = 2 * row + par;
            if (row >= nrows || j >= nn) continue;
            const int EA = a.aexp[(size_t)(m * 2 + par) * a.nrp + row];
#pragma unroll
            for (int c = 0; c < 8; c += 2) {
              const int n = c0 + c, zo = z0 + (n >> 1);
              if (zo >= a.nzdim) continue;
              const double re = EA > -2000 && colexp[n] > -2000 ? xs_i64_to_double(T[par][c], EA + colexp[n] + eo) : 0.0;
              const double im = EA > -2000 && colexp[n + 1] > -2000 ? xs_i64_to_double(T[par][c + 1], EA + colexp[n + 1] + eo) : 0.0;
              a.out[j + (size_t)a.nrdim * (m + (size_t)a.npdim * zo)] = make_double2(re, im);
            }
          }
        } else {
          const int i = row;
          if (i < a.nrh) {
            const int EA = a.aexp[(size_t)m * a.nrp + i];
            const double lnv = (a.add_ln && m == 0) ? *a.lnp : 0.0;
#pragma unroll
            for (int c = 0; c < 8; c += 2) {
              const int n = c0 + c, zo = z0 + (n >> 1);
              if (zo >= a.nzdim) continue;
              double v[4] = {0.0, 0.0, 0.0, 0.0};   // f(i) re, im; f(nr-1-i) re, im
#pragma unroll
              for (int q = 0; q < 2; ++q) {
                const int E = colexp[n + q];
                if (EA > -2000 && E > -2000) {
                  v[q] = xs_i64_to_double(T[0][c + q] + T[1][c + q], EA + E + eo);
                  v[2 + q] = xs_i64_to_double(T[0][c + q] - T[1][c + q], EA + E + eo);
                }
              }
              if (lnv != 0.0) { v[0] += lnv * a.lnx[i]; v[2] += lnv * a.lnx[a.nr - 1 - i]; }
              const size_t b0 = (size_t)a.nrdim * (m + (size_t)a.npdim * zo);
              a.out[b0 + i] = make_double2(v[0], v[1]);
              a.out[b0 + a.nr - 1 - i] = make_double2(v[2], v[3]);
            }
          }
        }
        }
      }
      tc_fence_before();
      __syncthreads();   // TMEM read out before the next tile's MMAs
    }
  }
  if (!ok) {
    if (tid == 0) atomicExch(a.status, 2);
    // let what was issued finish (bounded) before the memory goes away: the last commit completes
    // after every earlier MMA; a table or field copy completes on its own barrier
    if (tid == 0 && it > 0) {
      bool ok2 = true;
      const uint32_t lst = it - 1;
      xs_wait(&bar_mma[lst & 1], (lst >> 1) & 1, ok2);
      ok2 = true;
      xs_wait(bar_raw, raw_ph, ok2);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, TCOLS);
}

// ------------------------------------------------------------------------------------------------
struct XsImg {
  uint16_t* p = nullptr;
  int* aexp = nullptr;
  size_t bytes = 0, abytes = 0;
  int nrc = -1, npc = -1, ns = 0, w = 0, nmt = 0, nkc = 0, nrp = 0;
};
static XsImg g_xs[2][2];   // [mode][plain/mixed]

void xs_free() {
  for (auto& r : g_xs)
    for (auto& t : r) {
      if (t.p) dfree(t.p, t.bytes);
      if (t.aexp) dfree(t.aexp, t.abytes);
      t = XsImg();
    }
}

// the digit configuration: FP64-grade (plain: 63 or 60 bits) or the mixed form's 42 bits; w = 7 while
// the orders stay exact (K (pairs) 2^14 < 2^24), else w = 6 with one digit more.  The mixed form
// needs 42 bits: its transform errors are deterministic, so a slowly changing flow meets the same
// error step after step and they add up along a run; with 35-bit slices the backward transforms alone
// left the vortex step's nonlinear term 9.6e-7 from the FP64 form after 1000 steps at 192 x 128 x 128,
// with 42 bits the whole mixed step stayed within 7e-7.  The plain form
// needs more than 53 bits: the rounding is relative to the column maximum, and the nonlinear term's
// curl cancellation magnifies what that loses on small entries (at 192 x 128 x 128 the vortex step's
// nonlinear term differed from the FP64 reference by 5e-10 with 49-bit and 2.4e-11 with 56-bit digits).
struct XsCfg { int ns, w; };
static bool xs_cfg(int kmax, bool plain, XsCfg& c) {
  const double lim = 16777216.0;
  if (plain) {
    if (9.0 * kmax * 128 * 128 < lim) { c = {9, 7}; return true; }
    if (10.0 * kmax * 64 * 64 < lim) { c = {10, 6}; return true; }
  } else {
    if (6.0 * kmax * 128 * 128 < lim) { c = {6, 7}; return true; }
    if (7.0 * kmax * 64 * 64 < lim) { c = {7, 6}; return true; }
  }
  return false;
}

static size_t xs_smem(int ns, int nz, int rawk) {
  const int n = 2 * nz;
  return 1024 + 2 * (size_t)(2 * ns * XS_ATILE) + 2 * (size_t)(2 * ns * n * XS_KC * 2) + (size_t)2 * nz * rawk * sizeof(double) +
         n * (sizeof(int) + sizeof(unsigned long long)) + 64;
}
// complex z columns per work item: 16 while the accumulators (2 NS orders x 2 NZ columns) fit the
// 512 columns of tensor memory and the field columns fit shared memory, else 8
static int xs_nz(int ns) { return (G.nr <= 256 && ns <= 8) ? 16 : 8; }

// whether the exact-slice contraction covers this kit: the orders stay exact and the stages fit
bool xs_supported(int mode, int nrc, bool plain) {
  XsCfg c;
  const int kmax = mode == 0 ? G.nrh : (nrc + 1) / 2;
  return xs_cfg(kmax, plain, c) && xs_smem(c.ns, xs_nz(c.ns), std::max(G.nr, nrc) | 1) <= 227 * 1024;
}

template <int MODE, int NS, int NZ>
static int xs_launch(const XsArgs& args, int nitems) {
  const size_t sm = xs_smem(NS, NZ, args.rawk);
  if (sm > 227 * 1024) return set_error(MLG_ESIZE, "radial contraction: shared-memory stage too large");
  auto kern = k_xs_rtrans<MODE, NS, NS, NZ>;
  MLG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int grid = std::min(nitems, 152);
  kern<<<grid, XS_THREADS, sm, G.stream>>>(args);
  MLG_LAUNCH();
  return 0;
}

// mode 0 forward, 1 backward, for m0 <= m < npc; out's rows that it writes are overwritten, the rest left
int xs_rtrans(int mode, const cd* in, cd* out, int nrc, int npc, int m0, const double* lnp, bool add_ln, bool plain) {
  if (npc <= m0) return 0;
  const int nrows = mode == 0 ? (nrc + 1) / 2 : G.nrh;
  const int kmax = mode == 0 ? G.nrh : (nrc + 1) / 2;
  XsCfg cfg;
  if (!xs_cfg(kmax, plain, cfg)) return set_error(MLG_ESIZE, "radial contraction: too many radial points for exact slices");
  const int nmt = cdiv(nrows, 128), nkc = cdiv(kmax, XS_KC), nrp = nmt * 128;
  XsImg& im = g_xs[mode][plain ? 0 : 1];
  if (im.nrc != nrc || im.npc != npc || !im.p || im.ns != cfg.ns || im.w != cfg.w) {
    if (im.p) dfree(im.p, im.bytes);
    if (im.aexp) dfree(im.aexp, im.abytes);
    im = XsImg();
    im.bytes = (size_t)npc * nmt * nkc * 2 * cfg.ns * XS_ATILE;
    im.abytes = (size_t)npc * (mode == 0 ? 2 : 1) * nrp * sizeof(int);
    MLG_TRY(dmalloc((void**)&im.p, im.bytes));
    MLG_TRY(dmalloc((void**)&im.aexp, im.abytes));
    k_xs_aexp<<<dim3(cdiv(nrp, 128), npc), 128, 0, G.stream>>>(G.pf, G.w, im.aexp, mode, G.nrh, G.ne, nrc, nrp, kmax);
    MLG_LAUNCH();
    const int nblk_t = npc * nmt * nkc;
    switch (cfg.ns) {
      case 6: k_xs_table<6><<<nblk_t, 256, 0, G.stream>>>(G.pf, G.w, im.aexp, im.p, mode, G.nrh, G.ne, nrc, nmt, nkc, nrp, cfg.w); break;
      case 7: k_xs_table<7><<<nblk_t, 256, 0, G.stream>>>(G.pf, G.w, im.aexp, im.p, mode, G.nrh, G.ne, nrc, nmt, nkc, nrp, cfg.w); break;
      case 9: k_xs_table<9><<<nblk_t, 256, 0, G.stream>>>(G.pf, G.w, im.aexp, im.p, mode, G.nrh, G.ne, nrc, nmt, nkc, nrp, cfg.w); break;
      default: k_xs_table<10><<<nblk_t, 256, 0, G.stream>>>(G.pf, G.w, im.aexp, im.p, mode, G.nrh, G.ne, nrc, nmt, nkc, nrp, cfg.w); break;
    }
    MLG_LAUNCH();
    im.nrc = nrc; im.npc = npc; im.ns = cfg.ns; im.w = cfg.w; im.nmt = nmt; im.nkc = nkc; im.nrp = nrp;
  }
  XsArgs args;
  args.in = in; args.out = out; args.img = im.p; args.aexp = im.aexp; args.lnx = G.lnx; args.lnp = lnp;
  args.status = (int*)(G.dscal + DS_FLAG + 1) + 1;
  args.add_ln = add_ln ? 1 : 0; args.nr = G.nr; args.nrh = G.nrh; args.nrdim = G.nrdim; args.npdim = G.npdim;
  args.nzdim = G.nzdim; args.nrc = nrc; args.m0 = m0; args.npc = npc; args.nmt = nmt; args.nkc = nkc; args.nrp = nrp;
  // odd, so that the columns of the staged field start in different shared-memory banks
  args.rawk = std::max(G.nr, nrc) | 1;
  args.wbits = cfg.w;
  {
    // the epilogue's 64-bit integer T = sum_d G_d 2^(w (NS-1-d) - esh) stays below 2^62:
    // |G_d| <= K NS 2^(2w)
    const double mx = (double)kmax * cfg.ns * (1 << cfg.w) * (1 << cfg.w);
    args.esh = std::max(0, (int)std::ceil(std::log2(mx) + 0.05) + cfg.w * (cfg.ns - 1) - 62);
  }
  const int nz16 = xs_nz(cfg.ns) == 16;
  const int nitems = (npc - m0) * cdiv(G.nzdim, nz16 ? 16 : 8);
#define XS_CASE(NSV)                                                                                   \
  case NSV:                                                                                            \
    if (mode == 0) return nz16 ? xs_launch<0, NSV, 16>(args, nitems) : xs_launch<0, NSV, 8>(args, nitems); \
    return nz16 ? xs_launch<1, NSV, 16>(args, nitems) : xs_launch<1, NSV, 8>(args, nitems);
  switch (cfg.ns) {
    XS_CASE(6)
    XS_CASE(7)
    case 9: return mode == 0 ? xs_launch<0, 9, 8>(args, nitems) : xs_launch<1, 9, 8>(args, nitems);
    case 10: return mode == 0 ? xs_launch<0, 10, 8>(args, nitems) : xs_launch<1, 10, 8>(args, nitems);
  }
#undef XS_CASE
  return set_error(MLG_EPARAM, "radial contraction: digit configuration");
}

}  // namespace mlg
