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
//  * takes the item's column scales, which the epilogue warps computed two items ahead from global memory;
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
// up to XS_NF fields with the same chop, transformed by one launch (the components of a vector field)
constexpr int XS_NF = 3;
struct XsArgs {
  const double2* in[XS_NF];
  double2* out[XS_NF];
  const double* lnp[XS_NF];
  const uint16_t* img;
  const int* aexp;
  const double* lnx;
  int* status;
  int add_ln, nf, nr, nrh, nrdim, npdim, nzdim, nrc, m0, npc, nmt, nkc, nrp, rawk;
  int astages;   // table-chunk stages (2 or 3, as shared memory allows)
};
// field f's pointer without an indexed access to the kernel parameters (which would copy them to local
// memory)
template <class P> __device__ __forceinline__ P xs_sel(const P (&p)[XS_NF], int f) {
  return f == 0 ? p[0] : (f == 1 ? p[1] : p[2]);
}

__device__ __forceinline__ bool xs_wait(uint64_t* bar, uint32_t phase, bool& ok) {
  if (!ok) return false;
  ok = mbar_wait(bar, phase);
  return ok;
}



// Warp roles of the contraction kernel (512 threads, one CTA per SM):
//   warp 0      producer: the item's field columns and the table chunks, by bulk copy
//   warp 1      MMA issue (one thread) and the tensor-memory allocation
//   warps 2..7  field digits
//   warps 8..15 epilogue: tensor memory -> 64-bit order sums -> FP64 results; the column scales of
//               the item two ahead
// Every hand-off is an mbarrier: the table chunks and the field-digit stages are rings (2 and XS_SB
// stages), the field columns are one buffer (the next item's columns land while the MMAs and the
// epilogue of this one run), the accumulators are released by the epilogue as soon as it has read
// them, so the MMAs of the next work unit overlap the FP64 conversion and the stores of this one.
// a bounded wait whose outcome every lane of the warp shares (the warp-collective operations that
// follow need the whole warp)
__device__ __forceinline__ bool xs_wait_w(uint64_t* bar, uint32_t phase, bool& ok) {
  xs_wait(bar, phase, ok);
  ok = __all_sync(0xFFFFFFFFu, ok);
  return ok;
}

constexpr int XS_SB = 3;                 // field-digit stages
constexpr int XS_NDW = 6, XS_NEW = 8;    // digit warps (2..7), epilogue warps (8..15)
constexpr int XS_NDIG = XS_NDW * 32, XS_NEPI = XS_NEW * 32;
static_assert(2 + XS_NDW + XS_NEW == XS_THREADS / 32, "warp roles");

// MODE 0 forward, 1 backward; NS digits (and orders), NZ complex z columns per item
// digit width of a digit count (xs_cfg): 7 bits for 6 and 9 digits, 6 bits for 7 and 10
template <int NS> __host__ __device__ constexpr int xs_w() { return (NS == 6 || NS == 9) ? 7 : 6; }
// right shift of the 64-bit order sums: |G_d| < 2^24 / (pairs) keeps sum_d G_d 2^(w (NS-1-d) - ESH)
// below 2^62
template <int NS> __host__ __device__ constexpr int xs_esh() {
  return 24 + xs_w<NS>() * (NS - 1) - 62 > 0 ? 24 + xs_w<NS>() * (NS - 1) - 62 : 0;
}
// T += v 2^SH (floor for SH < 0), SH a compile-time constant: one wide multiply-add for 0 <= SH <= 30
template <int SH> __device__ __forceinline__ void xs_acc(long long& T, int v) {
  if constexpr (SH > 30) T += (long long)v << SH;
  else if constexpr (SH >= 0) T += (long long)v * (long long)(1 << SH);
  else T += (long long)v >> (-SH);
}
template <int NO, int W, int ESH, int D> __device__ __forceinline__ void xs_acc_order(long long& T, uint32_t g) {
  xs_acc<W * (NO - 1 - D) - ESH>(T, xs_f2i(__uint_as_float(g)));
}

template <int MODE, int NS, int NZ>
__global__ void __launch_bounds__(XS_THREADS, 1) k_xs_rtrans(XsArgs a) {
  constexpr int NO = NS;
  constexpr int W = xs_w<NS>(), ESH = xs_esh<NS>();
  constexpr int N = 2 * NZ;                       // real columns (MMA N per digit)
  constexpr int BT = N * XS_KC * 2;               // B digit tile bytes
  constexpr int ASTAGE = 2 * NS * XS_ATILE;
  constexpr int BSTAGE = 2 * NS * BT;
  // the accumulators of one work unit, and two sets of them where tensor memory holds both: the MMAs of
  // the next unit then run while the epilogue reads this one's
  constexpr int ACC = 2 * NO * N;
  constexpr int TB = 2 * ACC <= 512 ? 2 : 1;
  constexpr int TUSE = TB * ACC;
  constexpr int TCOLS = TUSE <= 32 ? 32 : TUSE <= 64 ? 64 : TUSE <= 128 ? 128 : TUSE <= 256 ? 256 : 512;
  constexpr int NBLK = (MODE == 0 ? 1 : 2) * (N / 8) * 2;   // digit blocks per chunk
  constexpr int CPW = N / 16;                     // 8-column groups of an epilogue warp
  static_assert(ACC <= 512, "accumulators exceed tensor memory");
  static_assert(N == 16 || N == 32, "MMA N per digit");
  static_assert((NO - 1) * N + N <= 256, "MMA N of the widest digit product");
  extern __shared__ __align__(1024) uint8_t xs_smem_raw[];
  uint8_t* sbase = (uint8_t*)(((uintptr_t)xs_smem_raw + 1023) & ~(uintptr_t)1023);
  const int AS = a.astages;
  uint8_t* sA = sbase;                                   // [AS][ASTAGE]
  uint8_t* sB = sA + AS * ASTAGE;                        // [XS_SB][BSTAGE]
  double* raw = (double*)(sB + XS_SB * BSTAGE);          // [NZ][rawk] complex (re, im)
  int* colexp = (int*)(raw + (size_t)2 * NZ * a.rawk);   // [2][N]: by item parity
  uint64_t* bars = (uint64_t*)(colexp + 2 * N);
  uint64_t* bar_rf = bars;                 // field columns landed
  uint64_t* bar_re = bars + 1;             // field columns consumed (digit threads)
  uint64_t* bar_af = bars + 2;             // [AS] table chunk landed
  uint64_t* bar_ae = bars + 5;             // [AS] table chunk consumed (MMA commit)
  uint64_t* bar_bf = bars + 8;             // [XS_SB] digit stage written (digit threads)
  uint64_t* bar_be = bar_bf + XS_SB;       // [XS_SB] digit stage consumed (MMA commit)
  uint64_t* bar_tf = bar_be + XS_SB;       // [TB] accumulators complete (MMA commit)
  uint64_t* bar_te = bar_tf + 2;           // [TB] accumulators read (epilogue threads)
  uint64_t* bar_cx = bar_te + 2;           // [2] column scales written (epilogue threads), by item parity
  uint64_t* bar_ce = bar_cx + 2;           // [2] column scales read (epilogue threads), by item parity
  uint32_t* tslot = (uint32_t*)(bar_ce + 2);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int w = W, nb = W * NS;
  if (tid == 0) {
    mbar_init(bar_rf, 1);
    mbar_init(bar_re, XS_NDIG);
    for (int i = 0; i < 3; ++i) {
      mbar_init(bar_af + i, 1);
      mbar_init(bar_ae + i, 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar_cx + i, XS_NEPI);
      mbar_init(bar_ce + i, XS_NEPI);
      mbar_init(bar_tf + i, 1);
      mbar_init(bar_te + i, XS_NEPI);
    }
    for (int i = 0; i < XS_SB; ++i) {
      mbar_init(bar_bf + i, XS_NDIG);
      mbar_init(bar_be + i, 1);
    }
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tslot, TCOLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;

  // the CTA's items (field, m, z tile), item = ((m - m0) nzt + z tile) nf + field, those without rows
  // skipped; every role walks the same sequence
  const int nzt = (a.nzdim + NZ - 1) / NZ;
  const int nitems = (a.npc - a.m0) * nzt * a.nf;
  auto item_m = [&](int item) { return a.m0 + item / (nzt * a.nf); };
  auto item_z0 = [&](int item) { return ((item / a.nf) % nzt) * NZ; };
  auto item_nn = [&](int item) { const int m = item_m(item); return max(min(a.nrc, a.nrc - m), 0); };
  auto next_item = [&](int item) {
    for (item += gridDim.x; item < nitems && item_nn(item) == 0; item += gridDim.x) {}
    return item;
  };
  int first = blockIdx.x;
  while (first < nitems && item_nn(first) == 0) first += gridDim.x;
  // per item: K extent (fwd radial points, bwd rows of the even parity), chunks, output rows, row tiles
  auto geom = [&](int nn, int& nkc_m, int& nrows, int& nmt_m) {
    const int kext = MODE == 0 ? a.nrh : (nn + 1) / 2;
    nkc_m = (kext + XS_KC - 1) / XS_KC;
    nrows = MODE == 0 ? (nn + 1) / 2 : a.nrh;
    nmt_m = (nrows + 127) / 128;
  };

  if (warp == 0) {
    // ---- producer
    if (lane == 0) {
      uint32_t c = 0, nraw = 0;   // table chunks and field-column copies issued
      int ii = 0;
      for (int item = first; item < nitems && ok; item = next_item(item), ++ii) {
        const int m = item_m(item), z0 = item_z0(item), nn = item_nn(item);
        const double2* fin = xs_sel(a.in, item % a.nf);
        int nkc_m, nrows, nmt_m;
        geom(nn, nkc_m, nrows, nmt_m);
        // the item's field columns, once the digit threads are done with the previous item's
        if (ii > 0 && !xs_wait(bar_re, (ii - 1) & 1, ok)) break;
        const int kraw = MODE == 0 ? a.nr : nn;
        fence_async_smem();
        uint32_t bytes = 0;
        for (int zz = 0; zz < NZ; ++zz)
          if (z0 + zz < a.nzdim) bytes += (uint32_t)kraw * 16u;
        mbar_expect_tx(bar_rf, bytes);
        for (int zz = 0; zz < NZ; ++zz)
          if (z0 + zz < a.nzdim)
            bulk_g2s(raw + (size_t)2 * zz * a.rawk, fin + (size_t)a.nrdim * (m + (size_t)a.npdim * (z0 + zz)),
                     (uint32_t)kraw * 16u, bar_rf);
        ++nraw;
        for (int mt = 0; mt < nmt_m && ok; ++mt) {
          const uint8_t* img_m = (const uint8_t*)a.img + ((size_t)m * a.nmt + mt) * a.nkc * (size_t)ASTAGE;
          for (int kc = 0; kc < nkc_m; ++kc, ++c) {
            const uint32_t s = c % (uint32_t)AS;
            if (c >= (uint32_t)AS && !xs_wait(&bar_ae[s], ((c - AS) / AS) & 1, ok)) break;
            mbar_expect_tx(&bar_af[s], ASTAGE);
            bulk_g2s(sA + s * ASTAGE, img_m + (size_t)kc * ASTAGE, ASTAGE, &bar_af[s]);
          }
        }
      }
      // the copies issued complete on their own: wait (bounded) for the last of them, so that no copy
      // is in flight when the CTA's shared memory goes away (at once in a run without a timeout)
      for (uint32_t j = c > (uint32_t)AS ? c - AS : 0; j < c; ++j) {
        bool ok2 = true;
        xs_wait(&bar_af[j % AS], (j / AS) & 1, ok2);
      }
      bool ok2 = true;
      if (nraw >= 1) xs_wait(bar_rf, (nraw - 1) & 1, ok2);
    }
  } else if (warp == 1) {
    // ---- MMA issue
    if (lane == 0) {
      uint32_t c = 0, u = 0;
      for (int item = first; item < nitems && ok; item = next_item(item)) {
        int nkc_m, nrows, nmt_m;
        geom(item_nn(item), nkc_m, nrows, nmt_m);
        for (int mt = 0; mt < nmt_m && ok; ++mt, ++u) {
          // the accumulator set of this unit, once the epilogue has read what it held TB units before
          const uint32_t tb = u % TB;
          if (u >= (uint32_t)TB && !xs_wait(&bar_te[tb], ((u - TB) / TB) & 1, ok)) break;
          tc_fence_after();
          const uint32_t tacc = tmem + tb * (uint32_t)ACC;
          for (int kc = 0; kc < nkc_m; ++kc, ++c) {
            const uint32_t sa = c % (uint32_t)AS, sb = c % XS_SB;
            if (!xs_wait(&bar_af[sa], (c / AS) & 1, ok)) break;
            if (!xs_wait(&bar_bf[sb], (c / XS_SB) & 1, ok)) break;
            tc_fence_after();
            const uint32_t a0 = smem_u32(sA + sa * ASTAGE), b0 = smem_u32(sB + sb * BSTAGE);
            // table digit t times the field digits s = 0 .. NO-1-t in one MMA of N (NO - t) columns: the
            // field digits lie side by side in shared memory and the orders d = t + s side by side in
            // tensor memory, so the product of digit s lands on order t + s
#pragma unroll
            for (int par = 0; par < 2; ++par)
#pragma unroll
              for (int t = 0; t < NO; ++t) {
                const uint64_t ad = sdesc(a0 + (par * NS + t) * XS_ATILE, XS_LBO, XS_SBO);
                const uint64_t bd = sdesc(b0 + (par * NS) * BT, XS_LBO, XS_SBO);
                umma_bf16(tacc + (uint32_t)((par * NO + t) * N), ad, bd, idesc_bf16(128, (NO - t) * N),
                          (kc > 0 || t > 0) ? 1u : 0u);
              }
            umma_commit(&bar_ae[sa]);
            umma_commit(&bar_be[sb]);
          }
          if (ok) umma_commit(&bar_tf[tb]);
        }
      }
      if (c > 0) {   // the MMAs issued have finished (bounded) before tensor memory is freed
        bool ok2 = true;
        xs_wait(&bar_ae[(c - 1) % AS], ((c - 1) / AS) & 1, ok2);
      }
    }
  } else if (warp < 2 + XS_NDW) {
    // ---- field digits
    const int dw = warp - 2;
    uint32_t c = 0;
    int ii = 0;
    for (int item = first; item < nitems && ok; item = next_item(item), ++ii) {
      const int z0 = item_z0(item), nn = item_nn(item);
      int nkc_m, nrows, nmt_m;
      geom(nn, nkc_m, nrows, nmt_m);
      const int* cx = colexp + (ii & 1) * N;
      if (!xs_wait_w(bar_rf, ii & 1, ok)) break;
      // the item's column scales, written by the epilogue warps two items ahead
      if (!xs_wait_w(&bar_cx[ii & 1], (ii >> 1) & 1, ok)) break;
      for (int mt = 0; mt < nmt_m && ok; ++mt) {
        for (int kc = 0; kc < nkc_m; ++kc, ++c) {
          const uint32_t s = c % XS_SB;
          if (c >= XS_SB && !xs_wait_w(&bar_be[s], ((c - XS_SB) / XS_SB) & 1, ok)) break;
          uint8_t* bst = sB + s * BSTAGE;
          // a warp writes (parity, 8 columns, 4 K pairs) blocks, each its 32 four-byte stores in 32 banks;
          // the warp's blocks unrolled, so that their independent chains interleave
#pragma unroll
          for (int bi = 0; bi < (NBLK + XS_NDW - 1) / XS_NDW; ++bi) {
            const int blk = dw + bi * XS_NDW;
            if (blk >= NBLK) break;
            const int par = MODE == 0 ? 0 : (blk & 1), bb = MODE == 0 ? blk : (blk >> 1);
            const int ng = bb % (N / 8), kh = bb / (N / 8);
            const int n = ng * 8 + (lane & 7), kp = kh * 4 + (lane >> 3), zz = n >> 1;
            const int E = cx[n];
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
          mbar_arrive(&bar_bf[s]);
        }
      }
      mbar_arrive(bar_re);   // done with the item's field columns
    }
  } else {
    // ---- epilogue: warp e reads TMEM lanes 32 (e % 4) .. +31 (rows of the tile) and the column half
    // e / 4; the orders are combined exactly in 64-bit integers, T = sum_d G_d 2^(w (NO-1-d) - esh), on the
    // integer pipe, and T 2^(EA + EB + esh - w (NO+1)) is then rounded once to FP64
    const int ew = warp - 2 - XS_NDW, lq = warp & 3, ch = ew >> 2;
    const uint32_t lrow = (uint32_t)(lq * 32) << 16;
    // The column scales of an item, into its slot of colexp: a warp per complex column z, its lanes over
    // the column's samples (read from global memory through L2, before the item's own bulk copy), the
    // largest exponent fields of the re and im parts (the high words without their sign bits order like
    // the magnitudes' exponent fields) reduced by warp shuffles; |x| < 2^(field - 1022), and the
    // forward folds may double.  The epilogue warps compute them two items ahead, in the time between
    // their last stores of one item and the accumulators of the next, so that the digit warps find them
    // ready when the item's columns land.
    auto col_scales = [&](int item, int slot) {
      const int m = item_m(item), z0 = item_z0(item);
      const int kraw = MODE == 0 ? a.nr : item_nn(item);
      const double2* fin = xs_sel(a.in, item % a.nf);
      int* cxw = colexp + slot * N;
      for (int zz = ew; zz < NZ; zz += XS_NEW) {
        unsigned mr = 0, mi = 0;
        if (z0 + zz < a.nzdim) {
          const double2* col = fin + (size_t)a.nrdim * (m + (size_t)a.npdim * (z0 + zz));
#pragma unroll 4
          for (int i = lane; i < kraw; i += 32) {
            const double2 v = __ldcg(col + i);
            mr = max(mr, (unsigned)__double2hiint(v.x) & 0x7FFFFFFFu);
            mi = max(mi, (unsigned)__double2hiint(v.y) & 0x7FFFFFFFu);
          }
        }
        mr = __reduce_max_sync(0xFFFFFFFFu, mr >> 20);
        mi = __reduce_max_sync(0xFFFFFFFFu, mi >> 20);
        if (lane == 0) {
          cxw[2 * zz] = mr ? (int)mr - 1022 + (MODE == 0 ? 1 : 0) : -2000;
          cxw[2 * zz + 1] = mi ? (int)mi - 1022 + (MODE == 0 ? 1 : 0) : -2000;
        }
      }
      mbar_arrive(&bar_cx[slot]);
    };
    if (first < nitems) {
      col_scales(first, 0);
      const int second = next_item(first);
      if (second < nitems) col_scales(second, 1);
    }
    uint32_t u = 0;
    int ii = 0;
    for (int item = first; item < nitems && ok; item = next_item(item), ++ii) {
      const int m = item_m(item), z0 = item_z0(item), nn = item_nn(item);
      double2* fout = xs_sel(a.out, item % a.nf);
      const double* flnp = xs_sel(a.lnp, item % a.nf);
      int nkc_m, nrows, nmt_m;
      geom(nn, nkc_m, nrows, nmt_m);
      const int* cx = colexp + (ii & 1) * N;
      // the item's column scales (written into this slot by all epilogue warps)
      if (!xs_wait_w(&bar_cx[ii & 1], (ii >> 1) & 1, ok)) break;
      for (int mt = 0; mt < nmt_m && ok; ++mt, ++u) {
        const int row = mt * 128 + lq * 32 + lane;
        const bool live = mt * 128 + lq * 32 < nrows;   // a warp of rows past the tile's rows reads nothing
        // the row exponents, loaded before the wait so that their latency hides behind it
        int EA0 = -2000, EA1 = -2000;
        if (MODE == 0) {
          if (row < nrows) {
            EA0 = a.aexp[(size_t)(m * 2) * a.nrp + row];
            EA1 = a.aexp[(size_t)(m * 2 + 1) * a.nrp + row];
          }
        } else if (row < a.nrh) {
          EA0 = a.aexp[(size_t)m * a.nrp + row];
        }
        const uint32_t tb = u % TB;
        if (!xs_wait_w(&bar_tf[tb], (u / TB) & 1, ok)) break;
        tc_fence_after();
        const uint32_t tacc = tmem + tb * (uint32_t)ACC;
        constexpr int eo = ESH - W * (NO + 1);
        // the warp's columns eight at a time; after the last group's loads the accumulators are free for
        // the next unit's MMAs (and, after the item's last unit, this thread is done with the item's
        // column scales), so the last group's conversions and stores overlap them
#pragma unroll 1
        for (int q = 0; q < CPW; ++q) {
          const int cb = ch * (N / 2) + q * 8;
          int E[8];
#pragma unroll
          for (int c = 0; c < 8; ++c) E[c] = cx[cb + c];
          long long T[2][8];
#pragma unroll
          for (int par = 0; par < 2; ++par)
#pragma unroll
            for (int c = 0; c < 8; ++c) T[par][c] = 0;
          if (live) {
            // two orders per load batch (one wait for four 8-column loads)
            auto order2 = [&](auto dc) {
              constexpr int D = 2 * decltype(dc)::value, D2 = D + 1 < NO ? D + 1 : D;
              uint32_t g[2][8], h[2][8];
#pragma unroll
              for (int par = 0; par < 2; ++par) {
                tmem_ld8_nw(tacc + lrow + (uint32_t)((par * NO + D) * N + cb), g[par]);
                if constexpr (D2 != D) tmem_ld8_nw(tacc + lrow + (uint32_t)((par * NO + D2) * N + cb), h[par]);
              }
              tmem_wait_ld();
#pragma unroll
              for (int par = 0; par < 2; ++par)
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                  xs_acc_order<NO, W, ESH, D>(T[par][c], g[par][c]);
                  if constexpr (D2 != D) xs_acc_order<NO, W, ESH, D2>(T[par][c], h[par][c]);
                }
            };
            xs_static_for<(NO + 1) / 2>(order2);
          }
          if (q == CPW - 1) {
            tc_fence_before();
            mbar_arrive(&bar_te[tb]);
            if (mt == nmt_m - 1) mbar_arrive(&bar_ce[ii & 1]);
          }
          if (!live) continue;
          if (MODE == 0) {
#pragma unroll
            for (int par = 0; par < 2; ++par) {
              const int j = 2 * row + par;
              if (row >= nrows || j >= nn) continue;
              const int EA = par ? EA1 : EA0;
#pragma unroll
              for (int c = 0; c < 8; c += 2) {
                const int zo = z0 + ((cb + c) >> 1);
                if (zo >= a.nzdim) continue;
                const double re = EA > -2000 && E[c] > -2000 ? xs_i64_to_double(T[par][c], EA + E[c] + eo) : 0.0;
                const double im = EA > -2000 && E[c + 1] > -2000 ? xs_i64_to_double(T[par][c + 1], EA + E[c + 1] + eo) : 0.0;
                fout[j + (size_t)a.nrdim * (m + (size_t)a.npdim * zo)] = make_double2(re, im);
              }
            }
          } else {
            const int i = row;
            if (i < a.nrh) {
              const int EA = EA0;
              // the log term is added at m = 0 only: an integer test per item, so that the other items
              // issue no FP64 compares or (predicated) FP64 additions on GB300's narrow FP64 pipe
              const bool ln_here = a.add_ln && m == 0;
#pragma unroll
              for (int c = 0; c < 8; c += 2) {
                const int zo = z0 + ((cb + c) >> 1);
                if (zo >= a.nzdim) continue;
                double v[4] = {0.0, 0.0, 0.0, 0.0};   // f(i) re, im; f(nr-1-i) re, im
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                  if (EA > -2000 && E[c + h] > -2000) {
                    // f(i) = D_0 + D_1, f(nr-1-i) = D_0 - D_1: both parities share the scales
                    v[h] = xs_i64_to_double(T[0][c + h] + T[1][c + h], EA + E[c + h] + eo);
                    v[2 + h] = xs_i64_to_double(T[0][c + h] - T[1][c + h], EA + E[c + h] + eo);
                  }
                }
                if (ln_here) {
                  const double lnv = *flnp;
                  v[0] += lnv * a.lnx[i];
                  v[2] += lnv * a.lnx[a.nr - 1 - i];
                }
                const size_t b0 = (size_t)a.nrdim * (m + (size_t)a.npdim * zo);
                fout[b0 + i] = make_double2(v[0], v[1]);
                fout[b0 + a.nr - 1 - i] = make_double2(v[2], v[3]);
              }
            }
          }
        }
      }
      // the scales of item ii+2 into this item's slot, once every epilogue thread has read it
      const int ahead = next_item(next_item(item));
      if (ok && ahead < nitems && xs_wait_w(&bar_ce[ii & 1], (ii >> 1) & 1, ok)) col_scales(ahead, ii & 1);
    }
  }
  if (!ok) atomicExch(a.status, 2);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, TCOLS);
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

static size_t xs_smem(int ns, int nz, int rawk, int astages) {
  const int n = 2 * nz;
  return 1024 + astages * (size_t)(2 * ns * XS_ATILE) + XS_SB * (size_t)(2 * ns * n * XS_KC * 2) +
         (size_t)2 * nz * rawk * sizeof(double) + 2 * n * sizeof(int) + 256;
}
// table-chunk stages: three where shared memory holds them, else two
static int xs_astages(int ns, int nz, int rawk) { return xs_smem(ns, nz, rawk, 3) <= 227 * 1024 ? 3 : 2; }
// complex z columns per work item: 16 while the accumulators (2 NS orders x 2 NZ columns) fit the 512
// columns of tensor memory and the field columns fit shared memory, else 8.  (With 8 columns two sets of
// accumulators fit for up to eight digits and the kernel double-buffers them, but at 192 x 128 x 128
// the halved items doubled the per-item costs: backward 102 -> 124 us per three-field launch.)
static int xs_nz(int ns) { return (G.nr <= 256 && ns <= 8) ? 16 : 8; }

// whether the exact-slice contraction covers this kit: the orders stay exact and the stages fit
bool xs_supported(int mode, int nrc, bool plain) {
  XsCfg c;
  const int kmax = mode == 0 ? G.nrh : (nrc + 1) / 2;
  return xs_cfg(kmax, plain, c) && xs_smem(c.ns, xs_nz(c.ns), std::max(G.nr, nrc) | 1, 2) <= 227 * 1024;
}

template <int MODE, int NS, int NZ>
static int xs_launch(const XsArgs& args, int nitems) {
  const size_t sm = xs_smem(NS, NZ, args.rawk, args.astages);
  if (sm > 227 * 1024) return set_error(MLG_ESIZE, "radial contraction: shared-memory stage too large");
  auto kern = k_xs_rtrans<MODE, NS, NZ>;
  MLG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int grid = std::min(nitems, 152);
  kern<<<grid, XS_THREADS, sm, G.stream>>>(args);
  MLG_LAUNCH();
  return 0;
}

// mode 0 forward, 1 backward, for m0 <= m < npc; out's rows that it writes are overwritten, the rest left
int xs_rtrans_multi(int mode, const cd* const* in, cd* const* out, int nf, int nrc, int npc, int m0,
                    const double* const* lnp, bool add_ln, bool plain) {
  if (npc <= m0 || nf < 1) return 0;
  if (nf > XS_NF) return set_error(MLG_EPARAM, "radial contraction: at most three fields per launch");
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
  for (int f = 0; f < XS_NF; ++f) {
    const int g = f < nf ? f : 0;
    args.in[f] = in[g]; args.out[f] = out[g]; args.lnp[f] = lnp ? lnp[g] : nullptr;
  }
  args.nf = nf;
  args.img = im.p; args.aexp = im.aexp; args.lnx = G.lnx;
  args.status = (int*)(G.dscal + DS_FLAG + 1) + 1;
  args.add_ln = add_ln ? 1 : 0; args.nr = G.nr; args.nrh = G.nrh; args.nrdim = G.nrdim; args.npdim = G.npdim;
  args.nzdim = G.nzdim; args.nrc = nrc; args.m0 = m0; args.npc = npc; args.nmt = nmt; args.nkc = nkc; args.nrp = nrp;
  // odd, so that the columns of the staged field start in different shared-memory banks
  args.rawk = std::max(G.nr, nrc) | 1;
  args.astages = xs_astages(cfg.ns, xs_nz(cfg.ns), args.rawk);
  // the kernels' compile-time digit widths (xs_w) are those of xs_cfg
  if (cfg.w != (cfg.ns == 6 || cfg.ns == 9 ? 7 : 6)) return set_error(MLG_EPARAM, "radial contraction: digit configuration");
  const int nz16 = xs_nz(cfg.ns) == 16;
  const int nitems = (npc - m0) * cdiv(G.nzdim, nz16 ? 16 : 8) * nf;
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

int xs_rtrans(int mode, const cd* in, cd* out, int nrc, int npc, int m0, const double* lnp, bool add_ln, bool plain) {
  return xs_rtrans_multi(mode, &in, &out, 1, nrc, npc, m0, &lnp, add_ln, plain);
}

// The bounded-wait path of the tensor-core kernels on its own: one thread waits on an mbarrier of
// arrival count 1.  arrive = 0: nothing arrives, so the wait runs out after `limit` clocks and the
// kernel sets the timeout word exactly as k_xs_rtrans does; arrive = 1: the thread arrives first and
// the wait ends at once.  Nothing is in flight and no tensor memory is held when it returns.
__global__ void k_wait_selftest(int* __restrict__ status, long long limit, int arrive) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(&bar)) : "memory");
  if (!mbar_wait_limit(&bar, 0, limit)) atomicExch(status, 2);
}

int wait_selftest(long long limit, int arrive) {
  if (limit < 0 || limit > 2000000000LL) return set_error(MLG_EPARAM, "wait self-test: limit must be 0 .. 2e9 clocks");
  k_wait_selftest<<<1, 32, 0, G.stream>>>((int*)(G.dscal + DS_FLAG + 1) + 1, limit, arrive ? 1 : 0);
  MLG_LAUNCH();
  return 0;
}

}  // namespace mlg
