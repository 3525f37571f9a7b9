// xs_vec2tp.cu — the projection contraction of vector_projection (mlegs_scalar_ops.f90:1402-1438, with
// the eomul / oemul folds :2067-2145) as exact-slice products on the 5th-generation tensor cores.
//
// For each m and row parity par, rows j = 2t + par, radial points i < nr/2, z columns n:
//   psi = (m V).(-i F_s(ur)) + D.(-F_o(up))
//   chi = k X - Y,   X = D.(i F_o(ur)) + (m V).F_s(up),   Y = T.F_s(uz)
// F_s / F_o fold u(i) with u(nr-1-i) by the row's own / the other parity's sign.
//
// All three sums run in the exact-slice scheme of xs_radial.cu.  psi and X each add two products in one
// set of digit-order accumulators, so the two products share their scales: one row scale per j over
// m V and D (kit init), one column scale per real column n over the two field components that land in
// it (Im ur with Re up for the real part of the output, Re ur with Im up for the imaginary part;
// the folds may double), and the digits of the folds are exact integer sums of the rounded samples.
// Y has its own row scale (T) and column scale (uz).  The orders of each sum are combined exactly in
// 64-bit integers and rounded once to FP64, on the integer pipe; chi = k X - Y is one FP64 fused
// multiply-add.  The row parity of a work item fixes the folds, so each item is one (m, parity,
// 128-row tile, NZ complex z columns).
//
// Digits: NS for psi and X, NT for Y, of w bits: the mixed form's NS = 5 (35 bits) and NT = 7 (49
// bits; 6 and 8 of 6 bits beyond about 100 radial points); w and the digit counts keep every order's
// accumulator exact: (pairs of the order) x (nr/2) x 2^(2w) < 2^24, where psi's and X's orders hold two
// products per digit pair.  Y needs the extra digits: at k = 0 chi is -Y alone, and the inverse
// Laplacian that ends the projection magnifies its error in the weak low modes; with 42-bit Y the
// (m = 1, k = 0) column left the step's nonlinear term chi 9e-6 from FP64 at 192 x 128 x 128, with
// 49 bits 2e-7.  (The plain form keeps its FP64 contraction: chi = k X - Y cancels, and even 54-bit
// slices, cut relative to the column maxima, left chi 7e-9 from the FP64 reference.)
//
// Engine: a persistent grid of one 256-thread CTA per SM over work items (m, parity, 128-row tile, 8
// complex z columns).  Per K chunk of 16 radial points the table digits (m V, D and T, laid out at kit
// init in the UMMA canonical K-major layout) arrive by one bulk copy into a two-stage ring, six warps
// cut the field digits (ur, up and uz at i and nr-1-i, fetched in FP64 a chunk ahead) into the same
// layout and arrive on the stage's mbarrier, and one thread issues the chunk's tcgen05.mma as soon as
// both halves of a stage are in: a table digit t meets every field digit s <= n-1-t of its operands in
// a single MMA (M = 128, K = 16; the field digits side by side in shared memory, the orders side by
// side in tensor memory, psi's and X's alternating), 2 NS + NT MMAs per chunk.  Every wait is bounded.
#include "common.cuh"
#include "tc_common.cuh"
#include "xs_common.cuh"
#include <cstdint>

namespace mlg {

constexpr int XV_KC = 16;
constexpr int XV_SBO = XV_KC * 16;
constexpr int XV_LBO = 128;
__host__ __device__ constexpr int xv_off(int row, int k) {
  return (row >> 3) * XV_SBO + (k >> 3) * XV_LBO + (row & 7) * 16 + (k & 7) * 2;
}
constexpr int XV_ATILE = 128 * XV_KC * 2;    // 4 KiB

__device__ __forceinline__ bool xs_wait(uint64_t* bar, uint32_t phase, bool& ok) {
  if (!ok) return false;
  ok = mbar_wait(bar, phase);
  return ok;
}

// ------------------------------------------------------------------------------------------------
// kit-time: row scales rexp[(m * 2 + par) * ntr + t] over (m V, D) and texp over T (-2000: zero row)
__global__ void k_xv_rexp(const double* __restrict__ tV, const double* __restrict__ tD, const double* __restrict__ tT,
                          int* __restrict__ rexp, int* __restrict__ texp, int nrh, int ne, int nrc, int ntr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int mp = blockIdx.y, m = mp >> 1, par = mp & 1;
  if (t >= ntr) return;
  const int j = 2 * t + par, nn = max(min(nrc, nrc - m), 0);
  unsigned long long mv = 0, mt = 0;
  if (j < nn)
    for (int i = 0; i < nrh; ++i) {
      const size_t o = i + (size_t)nrh * (j + (size_t)ne * m);
      unsigned long long a = (unsigned long long)__double_as_longlong((double)m * tV[o]) & 0x7FFFFFFFFFFFFFFFull;
      unsigned long long b = (unsigned long long)__double_as_longlong(tD[o]) & 0x7FFFFFFFFFFFFFFFull;
      unsigned long long c = (unsigned long long)__double_as_longlong(tT[o]) & 0x7FFFFFFFFFFFFFFFull;
      mv = a > mv ? a : mv;
      mv = b > mv ? b : mv;
      mt = c > mt ? c : mt;
    }
  rexp[(size_t)mp * ntr + t] = mv ? xs_ebound(mv) : -2000;
  texp[(size_t)mp * ntr + t] = mt ? xs_ebound(mt) : -2000;
}

// tiles per (m, par, row tile mt, chunk kc): [m V digits NS | D digits NS | T digits NT]
template <int NS, int NT>
__global__ void k_xv_table(const double* __restrict__ tV, const double* __restrict__ tD, const double* __restrict__ tT,
                           const int* __restrict__ rexp, const int* __restrict__ texp, uint16_t* __restrict__ img,
                           int nrh, int ne, int nrc, int nmt, int nkc, int ntr, int w) {
  const size_t blk = blockIdx.x;   // ((m * 2 + par) * nmt + mt) * nkc + kc
  const int kc = (int)(blk % nkc), mt = (int)((blk / nkc) % nmt), mp = (int)(blk / ((size_t)nkc * nmt));
  const int m = mp >> 1, par = mp & 1;
  const int nn = max(min(nrc, nrc - m), 0);
  uint8_t* base = (uint8_t*)img + blk * (size_t)((2 * NS + NT) * XV_ATILE);
  for (int idx = threadIdx.x; idx < 128 * XV_KC; idx += blockDim.x) {
    const int k = idx % XV_KC, r = idx / XV_KC;
    const int t = mt * 128 + r, j = 2 * t + par, i = kc * XV_KC + k;
    double v = 0.0, d = 0.0, tt = 0.0;
    int er = -2000, et = -2000;
    if (t < ntr && j < nn && i < nrh) {
      const size_t o = i + (size_t)nrh * (j + (size_t)ne * m);
      v = (double)m * tV[o]; d = tD[o]; tt = tT[o];
      er = rexp[(size_t)mp * ntr + t]; et = texp[(size_t)mp * ntr + t];
    }
    const int off = xv_off(r, k);
    float h[NS > NT ? NS : NT];
    xs_digits_f<NS>(xs_fix(v, er, w * NS), w, h);
#pragma unroll
    for (int s = 0; s < NS; ++s) *(uint16_t*)(base + s * XV_ATILE + off) = (uint16_t)(__float_as_uint(h[s]) >> 16);
    xs_digits_f<NS>(xs_fix(d, er, w * NS), w, h);
#pragma unroll
    for (int s = 0; s < NS; ++s) *(uint16_t*)(base + (NS + s) * XV_ATILE + off) = (uint16_t)(__float_as_uint(h[s]) >> 16);
    xs_digits_f<NT>(xs_fix(tt, et, w * NT), w, h);
#pragma unroll
    for (int s = 0; s < NT; ++s) *(uint16_t*)(base + (2 * NS + s) * XV_ATILE + off) = (uint16_t)(__float_as_uint(h[s]) >> 16);
  }
}

// ------------------------------------------------------------------------------------------------
struct XvArgs {
  const double2 *ur, *up, *uz;
  double2 *psi, *chi;
  const uint16_t* img;
  const int *rexp, *texp;
  const double* ak;
  int* status;
  int nr, nrh, nrdim, npdim, nzdim, nrc, nzc, nzcu, nmt, nkc, ntr, w, m0, npc;
  int esh_s, esh_t;   // right shifts that keep the 64-bit order sums of psi / X and of Y below 2^62
};

// NS digits for psi and X, NT for Y; 8 complex z columns per work item (N = 16).  Persistent: one CTA of
// 256 threads per SM walks the items (m, parity, row tile, z tile); warp 0 (one thread) copies the table
// chunks into a two-stage ring, warp 1 (one thread) issues the MMAs, warps 2..7 cut the field digits
// (one staging item each: field, z column, K pair), all eight warps run the epilogue.
constexpr int XV_NZ = 8;
constexpr int XV_THREADS = 256;
template <int NS, int NT>
__global__ void __launch_bounds__(XV_THREADS, 1) k_xv_contract(XvArgs a) {
  constexpr int NZ = XV_NZ;
  constexpr int N = 2 * NZ;
  constexpr int BTILE = N * XV_KC * 2;
  constexpr int NA = 2 * NS + NT;                 // A tiles per chunk
  constexpr int NB = 4 * NS + NT;                 // B tiles: [psi_ur, X_up] and [psi_up, X_ur] by digit, uz (NT)
  constexpr int ASTAGE = NA * XV_ATILE, BSTAGE = NB * BTILE;
  constexpr int COLS = (2 * NS + NT) * N;
  constexpr int TCOLS = COLS <= 128 ? 128 : COLS <= 256 ? 256 : 512;
  constexpr int NDIG = 3 * NZ * 8;                // staging items = digit threads (warps 2..7)
  static_assert(COLS <= 512, "accumulators exceed tensor memory");
  static_assert(NDIG == XV_THREADS - 64, "one staging item per digit thread");
  extern __shared__ __align__(1024) uint8_t xv_smem_raw[];
  uint8_t* sbase = (uint8_t*)(((uintptr_t)xv_smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = sbase;                            // [2][ASTAGE]
  uint8_t* sB = sA + 2 * ASTAGE;                  // [2][BSTAGE]
  int* cexp = (int*)(sB + 2 * BSTAGE);            // [N]: ur/up columns
  int* fexp = cexp + N;                           // [N]: uz columns
  uint64_t* bars = (uint64_t*)(fexp + 2 * N);     // a[2], b[2], mma[2]
  uint32_t* tslot = (uint32_t*)(bars + 6);
  uint64_t* bar_a = bars;
  uint64_t* bar_b = bars + 2;
  uint64_t* bar_mma = bars + 4;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int w = a.w, nbs = w * NS, nbt = w * NT;
  if (tid == 0) {
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
  uint32_t it = 0;   // chunk counter (stage and phase), the same in every thread
  const int nzt = (a.nzdim + NZ - 1) / NZ;
  const int nmp = a.npc - a.m0;
  const int nitems = nmp * 2 * a.nmt * nzt;   // item = ((mi * 2 + par) * nmt + mt) * nzt + zt
  // staging item of a digit thread: field f (0 ur, 1 up, 2 uz), z column zz, K pair kp (the eight K
  // pairs of a column in consecutive lanes, so that a warp's loads are runs of consecutive r)
  const int dt = tid - 64;
  const int f = dt / (NZ * 8), kp = dt % 8, zz = (dt / 8) % NZ;

  for (int item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
    const int zt = item % nzt, mt = (item / nzt) % a.nmt, par = (item / (nzt * a.nmt)) & 1;
    const int m = a.m0 + item / (nzt * a.nmt * 2);
    const int nn = max(min(a.nrc, a.nrc - m), 0);
    if (2 * (mt * 128) + par >= nn) continue;   // no rows of this parity in the tile (every thread agrees)
    const int z0 = zt * NZ;
    const int ss = par ? -1 : 1;   // own-parity fold sign
    // ---- column scales: cexp(2zz) over (Im ur, Re up), cexp(2zz+1) over (Re ur, Im up); fexp over uz.
    // Warp cz scans column z0 + cz (runs of consecutive r) for the largest exponent fields and reduces
    // them by warp shuffles; |x| < 2^(field - 1022) for every sample, +1 because the folds may double.
    {
      static_assert(XV_THREADS / 32 == NZ, "one warp per z column");
      const int cz = warp, z = z0 + cz;
      unsigned e0 = 0, e1 = 0, u0 = 0, u1 = 0;
      if (z < a.nzdim) {
        const size_t cb = (size_t)a.nrdim * (m + (size_t)a.npdim * z);
        auto ex = [](double v) { return ((unsigned)__double2hiint(v) >> 20) & 0x7FFu; };
        // unrolled, so that the loads of several rows are in flight at once (the scan waits on them)
#pragma unroll 6
        for (int i = lane; i < a.nr; i += 32) {
          const double2 r = a.ur[cb + i], pq = a.up[cb + i], q = a.uz[cb + i];
          e0 = max(e0, max(ex(r.y), ex(pq.x)));
          e1 = max(e1, max(ex(r.x), ex(pq.y)));
          u0 = max(u0, ex(q.x));
          u1 = max(u1, ex(q.y));
        }
      }
      e0 = __reduce_max_sync(0xFFFFFFFFu, e0);
      e1 = __reduce_max_sync(0xFFFFFFFFu, e1);
      u0 = __reduce_max_sync(0xFFFFFFFFu, u0);
      u1 = __reduce_max_sync(0xFFFFFFFFu, u1);
      if (lane == 0) {
        cexp[2 * cz] = e0 ? (int)e0 - 1021 : -2000;
        cexp[2 * cz + 1] = e1 ? (int)e1 - 1021 : -2000;
        fexp[2 * cz] = u0 ? (int)u0 - 1021 : -2000;
        fexp[2 * cz + 1] = u1 ? (int)u1 - 1021 : -2000;
      }
    }
    __syncthreads();
    const uint8_t* img_b = (const uint8_t*)a.img + (((size_t)(m * 2 + par) * a.nmt + mt) * a.nkc) * (size_t)ASTAGE;
    const int nkc = a.nkc;
    const uint32_t it0 = it;
    if (warp == 0) {
      // ---- producer: each table chunk into its stage once the MMAs that read the stage before are done
      if (lane == 0)
        for (int kc = 0; kc < nkc && ok; ++kc) {
          const uint32_t c = it0 + kc, s = c & 1;
          if (c >= 2) xs_wait(&bar_mma[s], ((c - 2) >> 1) & 1, ok);
          if (!ok) break;
          mbar_expect_tx(&bar_a[s], ASTAGE);
          bulk_g2s(sA + s * ASTAGE, img_b + (size_t)kc * ASTAGE, ASTAGE, &bar_a[s]);
        }
      __syncwarp();
    } else if (warp == 1) {
      // ---- MMA issue
      if (lane == 0)
        for (int kc = 0; kc < nkc && ok; ++kc) {
          const uint32_t c = it0 + kc, s = c & 1;
          xs_wait(&bar_a[s], (c >> 1) & 1, ok);
          xs_wait(&bar_b[s], (c >> 1) & 1, ok);
          if (!ok) break;
          tc_fence_after();
          const uint32_t a0 = smem_u32(sA + s * ASTAGE), b0 = smem_u32(sB + s * BSTAGE);
          auto A = [&](int t) { return sdesc(a0 + t * XV_ATILE, XV_LBO, XV_SBO); };
          auto B = [&](int t) { return sdesc(b0 + t * BTILE, XV_LBO, XV_SBO); };
          // table digit t against the field digits 0 .. n-1-t in one MMA: the field digits lie side by
          // side in shared memory and the accumulators of the orders side by side in tensor memory, so
          // the product of field digit s lands on order t + s.  psi and X alternate by order (psi_d at
          // 2d N, X_d at (2d+1) N) and their field digits alternate the same way ([psi_ur_s, X_up_s]
          // against m V, [psi_up_s, X_ur_s] against D), so one MMA of 2 N (NS - t) columns covers
          // both sums
#pragma unroll
          for (int t = 0; t < NS; ++t) {
            const uint32_t id = idesc_bf16(128, 2 * (NS - t) * N);
            umma_bf16(tmem + 2 * t * N, A(t), B(0), id, (kc > 0 || t > 0) ? 1u : 0u);   // m V . [psi_ur | X_up]
            umma_bf16(tmem + 2 * t * N, A(NS + t), B(2 * NS), id, 1u);                 // D . [psi_up | X_ur]
          }
#pragma unroll
          for (int t = 0; t < NT; ++t)
            umma_bf16(tmem + (2 * NS + t) * N, A(2 * NS + t), B(4 * NS), idesc_bf16(128, (NT - t) * N),
                      (kc > 0 || t > 0) ? 1u : 0u);
          umma_commit(&bar_mma[s]);
        }
      __syncwarp();
    } else {
      // ---- field digits: this thread's two K of its field at i and nr-1-i, fetched a chunk ahead
      const int z = z0 + zz;
      const bool zok = z < a.nzdim;
      const size_t cbase = (size_t)a.nrdim * (m + (size_t)a.npdim * (zok ? z : 0));
      const double2* src = f == 0 ? a.ur : (f == 1 ? a.up : a.uz);
      double2 va[2], vb[2];
      auto fetch = [&](int kc) {
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int i = kc * XV_KC + 2 * kp + u;
          const bool okk = zok && i < a.nrh;
          va[u] = okk ? src[cbase + i] : make_double2(0.0, 0.0);
          vb[u] = okk ? src[cbase + a.nr - 1 - i] : make_double2(0.0, 0.0);
        }
      };
      fetch(0);
      const int off = xv_off(2 * zz, 2 * kp), off1 = xv_off(2 * zz + 1, 2 * kp);
      for (int kc = 0; kc < nkc && ok; ++kc) {
        const uint32_t c = it0 + kc, s = c & 1;
        if (c >= 2) xs_wait(&bar_mma[s], ((c - 2) >> 1) & 1, ok);
        if (!ok) break;
        uint8_t* bst = sB + s * BSTAGE;
        if (f < 2) {
          // integer folds of the two components with the column scales of the columns they land in
          const int Ere = f == 0 ? cexp[2 * zz + 1] : cexp[2 * zz];       // Re ur -> col 2zz+1, Re up -> col 2zz
          const int Eim = f == 0 ? cexp[2 * zz] : cexp[2 * zz + 1];
          float h0[2][NS], h1[2][NS], g0[2][NS], g1[2][NS];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const long long ar = xs_fix(va[u].x, Ere, nbs), br = xs_fix(vb[u].x, Ere, nbs);
            const long long ai = xs_fix(va[u].y, Eim, nbs), bi = xs_fix(vb[u].y, Eim, nbs);
            const long long fs_re = ar + ss * br, fs_im = ai + ss * bi;
            const long long fo_re = ar - ss * br, fo_im = ai - ss * bi;
            if (f == 0) {   // psi_ur = -i F_s(ur): (Im, -Re); X_ur = i F_o(ur): (-Im, Re)
              xs_digits_f<NS>(fs_im, w, h0[u]); xs_digits_f<NS>(-fs_re, w, h1[u]);
              xs_digits_f<NS>(-fo_im, w, g0[u]); xs_digits_f<NS>(fo_re, w, g1[u]);
            } else {        // psi_up = -F_o(up): (-Re, -Im); X_up = F_s(up): (Re, Im)
              xs_digits_f<NS>(-fo_re, w, h0[u]); xs_digits_f<NS>(-fo_im, w, h1[u]);
              xs_digits_f<NS>(fs_re, w, g0[u]); xs_digits_f<NS>(fs_im, w, g1[u]);
            }
          }
          // B tiles: [psi_ur_s, X_up_s] at 2s, 2s+1; [psi_up_s, X_ur_s] at 2 NS + 2s, 2 NS + 2s + 1
          const int tp = f == 0 ? 0 : 2 * NS, tx = f == 0 ? 2 * NS + 1 : 1;
#pragma unroll
          for (int q = 0; q < NS; ++q) {
            *(uint32_t*)(bst + (tp + 2 * q) * BTILE + off) = xs_pack(h0[0][q], h0[1][q]);
            *(uint32_t*)(bst + (tp + 2 * q) * BTILE + off1) = xs_pack(h1[0][q], h1[1][q]);
            *(uint32_t*)(bst + (tx + 2 * q) * BTILE + off) = xs_pack(g0[0][q], g0[1][q]);
            *(uint32_t*)(bst + (tx + 2 * q) * BTILE + off1) = xs_pack(g1[0][q], g1[1][q]);
          }
        } else {
          // Y: F_s(uz) with the uz column scales
          float h0[2][NT], h1[2][NT];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const long long re = xs_fix(va[u].x, fexp[2 * zz], nbt) + ss * xs_fix(vb[u].x, fexp[2 * zz], nbt);
            const long long im = xs_fix(va[u].y, fexp[2 * zz + 1], nbt) + ss * xs_fix(vb[u].y, fexp[2 * zz + 1], nbt);
            xs_digits_f<NT>(re, w, h0[u]);
            xs_digits_f<NT>(im, w, h1[u]);
          }
#pragma unroll
          for (int q = 0; q < NT; ++q) {
            *(uint32_t*)(bst + (4 * NS + q) * BTILE + off) = xs_pack(h0[0][q], h0[1][q]);
            *(uint32_t*)(bst + (4 * NS + q) * BTILE + off1) = xs_pack(h1[0][q], h1[1][q]);
          }
        }
        fence_async_smem();
        mbar_arrive(&bar_b[s]);
        if (kc + 1 < nkc) fetch(kc + 1);
      }
    }
    it = it0 + nkc;
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. (rows t) and the 8-column block w / 4
    const int t = mt * 128 + (warp & 3) * 32 + lane;
    const int j = 2 * t + par;
    const bool rok = j < nn && t < a.ntr;
    // the row exponents, loaded before the wait so that their latency hides behind it
    const int er = rok ? a.rexp[(size_t)(m * 2 + par) * a.ntr + t] : -2000;
    const int et = rok ? a.texp[(size_t)(m * 2 + par) * a.ntr + t] : -2000;
    {
      const uint32_t lst = it - 1;
      xs_wait(&bar_mma[lst & 1], (lst >> 1) & 1, ok);
    }
    ok = __syncthreads_and(ok);
    if (!ok) break;
    tc_fence_after();
    if (mt * 128 + (warp & 3) * 32 < a.ntr) {   // a warp of rows past the tile's rows has nothing to write
      const uint32_t lrow = (uint32_t)((warp & 3) * 32) << 16;
      const int cb = warp >> 2;
#pragma unroll 1
      for (int half = 0; half < 2; ++half) {   // four columns (two complex z) at a time
        const int c0 = cb * 8 + half * 4;
        // the orders combined exactly in 64-bit integers, T = sum_d G_d 2^(w (n-1-d) - esh), then
        // T 2^(row exp + column exp + esh - w (n+1)) rounded once to FP64
        long long tp[4] = {0, 0, 0, 0}, tx[4] = {0, 0, 0, 0}, ty[4] = {0, 0, 0, 0};
        {
          uint32_t gp[NS][4], gx[NS][4];
#pragma unroll
          for (int d = 0; d < NS; ++d) {
            tmem_ld4_nw(tmem + lrow + 2 * d * N + c0, gp[d]);
            tmem_ld4_nw(tmem + lrow + (2 * d + 1) * N + c0, gx[d]);
          }
          tmem_wait_ld();
#pragma unroll
          for (int d = 0; d < NS; ++d) {
            const int sh = w * (NS - 1 - d) - a.esh_s;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              tp[c] += xs_shl((long long)xs_f2i(__uint_as_float(gp[d][c])), sh);
              tx[c] += xs_shl((long long)xs_f2i(__uint_as_float(gx[d][c])), sh);
            }
          }
        }
        {
          uint32_t gy[NT][4];
#pragma unroll
          for (int d = 0; d < NT; ++d) tmem_ld4_nw(tmem + lrow + (2 * NS + d) * N + c0, gy[d]);
          tmem_wait_ld();
#pragma unroll
          for (int d = 0; d < NT; ++d) {
            const int sh = w * (NT - 1 - d) - a.esh_t;
#pragma unroll
            for (int c = 0; c < 4; ++c) ty[c] += xs_shl((long long)xs_f2i(__uint_as_float(gy[d][c])), sh);
          }
        }
        double pv[4], xv[4], yv[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int E = cexp[c0 + c], F = fexp[c0 + c];
          const bool ox = er > -2000 && E > -2000, oy = et > -2000 && F > -2000;
          pv[c] = ox ? xs_i64_to_double(tp[c], er + E + a.esh_s - w * (NS + 1)) : 0.0;
          xv[c] = ox ? xs_i64_to_double(tx[c], er + E + a.esh_s - w * (NS + 1)) : 0.0;
          yv[c] = oy ? xs_i64_to_double(ty[c], et + F + a.esh_t - w * (NT + 1)) : 0.0;
        }
        if (rok) {
#pragma unroll
          for (int c = 0; c < 4; c += 2) {
            const int n = c0 + c, zc = z0 + n / 2;
            if (zc >= a.nzdim) continue;
            const int kk = zc + 1;
            if (!(kk <= a.nzc || kk >= a.nzcu)) continue;
            const double kz = a.ak[zc];
            const size_t o = j + (size_t)a.nrdim * (m + (size_t)a.npdim * zc);
            a.psi[o] = make_double2(pv[c], pv[c + 1]);
            a.chi[o] = make_double2(fma(kz, xv[c], -yv[c]), fma(kz, xv[c + 1], -yv[c + 1]));
          }
        }
      }
    }
    tc_fence_before();
    __syncthreads();   // TMEM read out (and cexp / fexp read) before the next item
  }
  if (!ok) {
    if (tid == 0) atomicExch(a.status, 2);
    if (tid == 0 && it > 0) {   // let what was issued finish (bounded) before the memory goes away
      bool ok2 = true;
      const uint32_t lst = it - 1;
      xs_wait(&bar_mma[lst & 1], (lst >> 1) & 1, ok2);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, TCOLS);
}

// ------------------------------------------------------------------------------------------------
struct XvImg {
  uint16_t* p = nullptr;
  int *rexp = nullptr, *texp = nullptr;
  size_t bytes = 0, ebytes = 0;
  int nrc = -1, npc = -1, ns = 0, nt = 0, w = 0;
};
static XvImg g_xv;

void xv_free() {
  if (g_xv.p) dfree(g_xv.p, g_xv.bytes);
  if (g_xv.rexp) dfree(g_xv.rexp, g_xv.ebytes);
  if (g_xv.texp) dfree(g_xv.texp, g_xv.ebytes);
  g_xv = XvImg();
}

struct XvCfg { int ns, nt, w; };
static bool xv_cfg(int k, XvCfg& c) {
  const double lim = 16777216.0;
  auto fits = [&](int ns, int nt, int w) {
    const double d = (double)(1 << w) * (1 << w);   // largest digit product (two's-complement digits)
    return 2.0 * ns * k * d < lim && (double)nt * k * d < lim;
  };
  if (fits(5, 7, 7)) { c = {5, 7, 7}; return true; }
  if (fits(6, 8, 6)) { c = {6, 8, 6}; return true; }
  return false;
}

bool xv_supported() {
  XvCfg c;
  return xv_cfg(G.nrh, c);
}

template <int NS, int NT>
static int xv_launch(const XvArgs& args, int npc) {
  constexpr int N = 2 * XV_NZ;
  const size_t sm = 1024 + 2 * (size_t)(2 * NS + NT) * XV_ATILE + 2 * (size_t)(4 * NS + NT) * N * XV_KC * 2 +
                    4 * N * sizeof(int) + 64;
  auto kern = k_xv_contract<NS, NT>;
  MLG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const int nitems = (npc - args.m0) * 2 * args.nmt * cdiv(G.nzdim, XV_NZ);
  kern<<<std::min(nitems, 152), XV_THREADS, sm, G.stream>>>(args);
  MLG_LAUNCH();
  return 0;
}

// psi, chi: the rows of m0 <= m < npc written (zeroed elsewhere by the caller)
int xv_contract(const cd* ur, const cd* up, const cd* uz, cd* psi, cd* chi, int nrc, int npc, int m0) {
  if (npc <= m0) return 0;
  XvCfg cfg;
  if (!xv_cfg(G.nrh, cfg)) return set_error(MLG_ESIZE, "vec2tp: too many radial points for exact slices");
  const int ntr = (nrc + 1) / 2;
  const int nmt = cdiv(ntr, 128), nkc = cdiv(G.nrh, XV_KC);
  XvImg& im = g_xv;
  if (im.nrc != nrc || im.npc != npc || !im.p || im.ns != cfg.ns || im.nt != cfg.nt || im.w != cfg.w) {
    if (im.p) dfree(im.p, im.bytes);
    if (im.rexp) dfree(im.rexp, im.ebytes);
    if (im.texp) dfree(im.texp, im.ebytes);
    im = XvImg();
    im.bytes = (size_t)npc * 2 * nmt * nkc * (2 * cfg.ns + cfg.nt) * XV_ATILE;
    im.ebytes = (size_t)npc * 2 * ntr * sizeof(int);
    MLG_TRY(dmalloc((void**)&im.p, im.bytes));
    MLG_TRY(dmalloc((void**)&im.rexp, im.ebytes));
    MLG_TRY(dmalloc((void**)&im.texp, im.ebytes));
    k_xv_rexp<<<dim3(cdiv(ntr, 128), npc * 2), 128, 0, G.stream>>>(G.tV, G.tD, G.tT, im.rexp, im.texp, G.nrh, G.ne, nrc, ntr);
    MLG_LAUNCH();
    const int nb = npc * 2 * nmt * nkc;
    if (cfg.ns == 5)
      k_xv_table<5, 7><<<nb, 256, 0, G.stream>>>(G.tV, G.tD, G.tT, im.rexp, im.texp, im.p, G.nrh, G.ne, nrc, nmt, nkc, ntr, cfg.w);
    else
      k_xv_table<6, 8><<<nb, 256, 0, G.stream>>>(G.tV, G.tD, G.tT, im.rexp, im.texp, im.p, G.nrh, G.ne, nrc, nmt, nkc, ntr, cfg.w);
    MLG_LAUNCH();
    im.nrc = nrc; im.npc = npc; im.ns = cfg.ns; im.nt = cfg.nt; im.w = cfg.w;
  }
  XvArgs args;
  args.ur = ur; args.up = up; args.uz = uz; args.psi = psi; args.chi = chi; args.img = im.p; args.rexp = im.rexp;
  args.texp = im.texp; args.ak = G.ak; args.status = (int*)(G.dscal + DS_FLAG + 1) + 1;
  args.nr = G.nr; args.nrh = G.nrh; args.nrdim = G.nrdim; args.npdim = G.npdim; args.nzdim = G.nzdim; args.nrc = nrc;
  args.nzc = G.chopzl; args.nzcu = G.chopzu; args.nmt = nmt; args.nkc = nkc; args.ntr = ntr; args.w = cfg.w; args.m0 = m0;
  args.npc = npc;
  {
    // the 64-bit order sums stay below 2^62: |G_d| <= K (pairs of order d) 2^(2w), with two products
    // per digit pair for psi and X
    auto esh = [&](int n, int pairs) {
      const double mx = (double)G.nrh * pairs * (1 << cfg.w) * (1 << cfg.w);
      return std::max(0, (int)std::ceil(std::log2(mx) + 0.05) + cfg.w * (n - 1) - 62);
    };
    args.esh_s = esh(cfg.ns, 2 * cfg.ns);
    args.esh_t = esh(cfg.nt, cfg.nt);
  }
  // 8 complex z columns per work item: the (2 NS + NT) orders of 2 x 8 columns fit the 512
  // tensor-memory columns
  if (cfg.ns == 5) return xv_launch<5, 7>(args, npc);
  return xv_launch<6, 8>(args, npc);
}

}  // namespace mlg
