// tc_radial.cu — the mixed form's radial Legendre contractions on the 5th-generation tensor cores.
//
// Forward (rtrans_forward, mlegs_scalar_ops.f90:1852-1927): for every azimuthal mode m and both
// row parities, C_par(t, n) = sum_i A_par(t, i) B_par(i, n) with A_par(t, i) = pf(i, 2t+par, m) and
// B_par(i, n) = (f(i) +- f(nr-1-i)) w(i) (n runs over re/im of the z columns).
//
// Precision: split BF16.  Each FP32 operand x is written as x0 + x1 + x2 with x0 = bf16(x),
// x1 = bf16(x - x0), x2 = bf16(x - x0 - x1) (each residual is exact in FP32), and the product keeps
// the six terms with i + j <= 2; every BF16 x BF16 product is exact in the FP32 accumulator, so the
// result carries ~2^-24 relative error like an FP32 contraction (the omitted terms are below 2^-24).
//
// Backward (rtrans_backward, :1931-2008): D_par(i, n) = sum_t A_par(i, t) B_par(t, n) with
// A_par(i, t) = pf(i, 2t+par, m) and B_par(t, n) = c(2t+par, m, z); the epilogue forms
// f(i) = D_0 + D_1 and f(nr-1-i) = D_0 - D_1 (and adds the log term at m = 0).
//
// Engine: one CTA per (m, 128-row tile, 32 complex z columns), 256 threads, 72 KiB of shared memory
// (three CTAs per SM).
//  * The table operand is split and laid out at kit init in the UMMA canonical no-swizzle K-major
//    layout (8x8 BF16 core matrices, 16-byte rows) per (m, row tile, K chunk): one K chunk of both
//    parities and all three splits (48 KiB) arrives by one cp.async.bulk on the TMA engine,
//    completing on an mbarrier.
//  * The field operand is folded (FP32, conversions on the integer pipe), split and stored by the
//    threads into the same layout, then made visible to the tensor core (fence.proxy.async).
//  * One elected thread issues tcgen05.mma kind::f16 (BF16 in, FP32 accumulate in TMEM, one
//    accumulator per parity; M=128, N=64, K=16 per instruction) and commits to an mbarrier; while the
//    tensor core runs, the threads already load the next K chunk of the field into registers.
//  * Epilogue: tcgen05.ld of each warp's 32 TMEM lanes, FP32 -> FP64 on the integer pipe.
// Every wait is bounded (about a second of clock); a timeout sets the library's status flag, and the
// CTA still releases its TMEM.
//
// The m = 0 plane is not done here: the mixed form contracts it in double-float (radial.cu), since
// it carries the axisymmetric mean flow and its radial sums cancel toward the axis.  The grid starts
// at m = m0.
#include "common.cuh"
#include "tc_common.cuh"
#include <cstdint>

namespace mlg {

// canonical layout of one operand tile of R rows x KC columns (BF16): byte offset of (row, k)
constexpr int TC_KC = 32;                       // K chunk
constexpr int TC_SBO = TC_KC * 16;              // 8 rows x KC cols: (KC/8) core matrices of 128 B
constexpr int TC_LBO = 128;
__host__ __device__ constexpr int tc_off(int row, int k) {
  return (row >> 3) * TC_SBO + (k >> 3) * TC_LBO + (row & 7) * 16 + (k & 7) * 2;
}
constexpr int TC_TILE_BYTES = 128 * TC_KC * 2;  // 8 KiB: 128 rows x 32 BF16 (table tiles, M = 128)
constexpr int TC_NZ = 32;                       // complex z columns per CTA (N = 64)
constexpr int TC_BTILE_BYTES = 2 * TC_NZ * TC_KC * 2;   // 4 KiB: 64 rows x 32 BF16 (field tiles)
constexpr int TC_THREADS = 512;   // 16 warps: the operand staging split in two halves (parity or fold sign)
                                  // of 8 K groups of 4, the epilogue in four column blocks of the four
                                  // TMEM lane quarters
constexpr int TC_KQ = 4;          // consecutive K per staging item

// ------------------------------------------------------------------------------------------------
// table images, split and laid out once per kit: for (m, row tile, K chunk): [par 2][split 3][tile]
//  fwd: rows t (A(t, i) = pf(i, 2t+par, m)), K = i
//  bwd: rows i (A(i, t) = pf(i, 2t+par, m)), K = t
__global__ void k_tc_table(const double* __restrict__ pf, uint16_t* __restrict__ img, int nrh, int ne, int nmt,
                           int nkc, int nrc, int bwd) {
  size_t blk = blockIdx.x;   // (m, mt, kc)
  int kc = blk % nkc;
  int mt = (blk / nkc) % nmt;
  int m = blk / ((size_t)nkc * nmt);
  int nn = max(min(nrc, nrc - m), 0);
  uint8_t* base = (uint8_t*)img + blk * (size_t)(6 * TC_TILE_BYTES);
  for (int idx = threadIdx.x; idx < 2 * 128 * TC_KC; idx += blockDim.x) {
    int k = idx % TC_KC, r = (idx / TC_KC) % 128, par = idx / (TC_KC * 128);
    int row = mt * 128 + r, kk = kc * TC_KC + k;
    int i = bwd ? row : kk, t = bwd ? kk : row;
    int j = 2 * t + par;
    double a = 0.0;
    if (j < nn && i < nrh) a = pf[i + (size_t)nrh * (j + (size_t)ne * m)];
    uint16_t s0 = bf16_rn((float)a);
    double r1 = a - (double)bf16_f(s0);
    uint16_t s1 = bf16_rn((float)r1);
    double r2 = r1 - (double)bf16_f(s1);
    uint16_t s2 = bf16_rn((float)r2);
    int off = tc_off(r, k);
    *(uint16_t*)(base + (par * 3 + 0) * TC_TILE_BYTES + off) = s0;
    *(uint16_t*)(base + (par * 3 + 1) * TC_TILE_BYTES + off) = s1;
    *(uint16_t*)(base + (par * 3 + 2) * TC_TILE_BYTES + off) = s2;
  }
}

struct TcSmem {
  uint8_t a[6 * TC_TILE_BYTES];    // [par][split] table tiles (bulk-copied), 48 KiB
  uint8_t b[6 * TC_BTILE_BYTES];   // [par][split] field tiles (written by the threads), 24 KiB
  uint64_t bar_a, bar_mma;
  uint32_t tmem;
};

// store the TC_KQ values of one K group of one field row (n) as the three BF16 splits
__device__ __forceinline__ void store_split4(uint8_t* b, int par, int n, int kg, const float* v) {
  static_assert(TC_KQ == 4, "staging items of 4 K: 8 bytes of a core-matrix row");
  uint32_t w[2][3];
#pragma unroll
  for (int q = 0; q < 2; ++q) split3x2(v[2 * q], v[2 * q + 1], w[q]);
#pragma unroll
  for (int s = 0; s < 3; ++s)
    *(uint2*)(b + (par * 3 + s) * TC_BTILE_BYTES + tc_off(n, kg * TC_KQ)) = make_uint2(w[0][s], w[1][s]);
}

// the two-parity bf16x3 MMA group of one K chunk: D_par += A_par * B_par, six split products
__device__ __forceinline__ void tc_issue_chunk(TcSmem& sm, uint32_t tmem, bool first) {
  const uint32_t idesc = idesc_bf16(128, 2 * TC_NZ);
  const int SA[6] = {0, 0, 1, 0, 1, 2}, SB[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
  for (int par = 0; par < 2; ++par)
#pragma unroll
    for (int ks = 0; ks < TC_KC / 16; ++ks)
#pragma unroll
      for (int p = 0; p < 6; ++p) {
        uint32_t aaddr = smem_u32(sm.a + (par * 3 + SA[p]) * TC_TILE_BYTES) + ks * 2 * TC_LBO;
        uint32_t baddr = smem_u32(sm.b + (par * 3 + SB[p]) * TC_BTILE_BYTES) + ks * 2 * TC_LBO;
        uint32_t acc = (!first || ks > 0 || p > 0) ? 1u : 0u;
        umma_bf16(tmem + par * (2 * TC_NZ), sdesc(aaddr, TC_LBO, TC_SBO), sdesc(baddr, TC_LBO, TC_SBO), idesc, acc);
      }
}

// mode 0 = forward (rtrans_forward), mode 1 = backward (rtrans_backward, + ln term at m = 0)
template <int MODE>
__global__ void __launch_bounds__(TC_THREADS) k_tc_rtrans(const double2* __restrict__ in, double2* __restrict__ out,
                                                          const uint16_t* __restrict__ img, const float* __restrict__ w32,
                                                          const double* __restrict__ lnx, const double* __restrict__ lnp,
                                                          int add_ln, int nr, int nrh, int nrdim, int npdim, int nzdim,
                                                          int nrc, int nmt, int nkc, int m0, int* __restrict__ status) {
  extern __shared__ __align__(1024) uint8_t tc_smem_raw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(tc_smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int z0 = blockIdx.x * TC_NZ, mt = blockIdx.y, m = blockIdx.z + m0;
  const int nn = max(min(nrc, nrc - m), 0);
  if (MODE == 0 && 2 * (mt * 128) >= nn) return;   // no rows of either parity in this tile
  if (MODE == 1 && (nn == 0 || mt * 128 >= nrh)) return;
  const int nkc_m = (MODE == 0) ? nkc : min(nkc, (((nn + 1) / 2) + TC_KC - 1) / TC_KC);   // bwd: K = rows t
  if (tid == 0) {
    mbar_init(&sm.bar_a, 1);
    mbar_init(&sm.bar_mma, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(&sm.tmem, 128);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem;
  bool ok = true;
  const uint8_t* img_m = (const uint8_t*)img + ((size_t)m * nmt + mt) * nkc * (size_t)(6 * TC_TILE_BYTES);
  // staging item of this thread: z column zz, K group kg (8 consecutive K indices) and half: the row
  // parity it writes (forward: the fold sign, backward: the parity of the rows it reads)
  constexpr int NKG = TC_KC / TC_KQ;   // K groups per chunk
  const int zz = tid % TC_NZ, kg = (tid / TC_NZ) % NKG, half = tid / (NKG * TC_NZ);
  const int z = z0 + zz;
  const double2* col = in + (size_t)nrdim * (m + (size_t)npdim * min(z, nzdim - 1));
  float2 ra[TC_KQ], rb[TC_KQ];
  float wv[TC_KQ];
  auto fetch = [&](int kc) {
#pragma unroll
    for (int q = 0; q < TC_KQ; ++q) {
      int k = kc * TC_KC + kg * TC_KQ + q;
      ra[q] = make_float2(0.f, 0.f); rb[q] = make_float2(0.f, 0.f); wv[q] = 0.f;
      if (MODE == 0) {
        if (k < nrh && z < nzdim) { ra[q] = ld_c32(col + k); rb[q] = ld_c32(col + nr - 1 - k); wv[q] = w32[k]; }
      } else {
        int j = 2 * k + half;
        if (z < nzdim && j < nn) ra[q] = ld_c32(col + j);
      }
    }
  };
  fetch(0);
  for (int kc = 0; kc < nkc_m; ++kc) {
    if (tid == 0) {
      mbar_expect_tx(&sm.bar_a, 6 * TC_TILE_BYTES);
      bulk_g2s(sm.a, img_m + (size_t)kc * (6 * TC_TILE_BYTES), 6 * TC_TILE_BYTES, &sm.bar_a);
    }
    {
      float v[TC_KQ];
      if (MODE == 0) {
        const float sg = half ? -1.f : 1.f;
#pragma unroll
        for (int q = 0; q < TC_KQ; ++q) v[q] = (ra[q].x + sg * rb[q].x) * wv[q];
        store_split4(sm.b, half, 2 * zz, kg, v);
#pragma unroll
        for (int q = 0; q < TC_KQ; ++q) v[q] = (ra[q].y + sg * rb[q].y) * wv[q];
        store_split4(sm.b, half, 2 * zz + 1, kg, v);
      } else {
#pragma unroll
        for (int q = 0; q < TC_KQ; ++q) v[q] = ra[q].x;
        store_split4(sm.b, half, 2 * zz, kg, v);
#pragma unroll
        for (int q = 0; q < TC_KQ; ++q) v[q] = ra[q].y;
        store_split4(sm.b, half, 2 * zz + 1, kg, v);
      }
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      ok = ok && mbar_wait(&sm.bar_a, kc & 1);
      tc_fence_after();
      if (ok) tc_issue_chunk(sm, tmem, kc == 0);
      umma_commit(&sm.bar_mma);
    }
    if (kc + 1 < nkc_m) fetch(kc + 1);   // the next chunk's loads overlap the MMAs
    bool done = mbar_wait(&sm.bar_mma, kc & 1);
    if (!done || (tid == 0 && !ok)) atomicExch(status, 2);
    __syncthreads();
  }
  tc_fence_after();
  // warp w reads TMEM lanes 32 (w % 4) .. +31 and the column part w / 4 of each accumulator
  const int lq = warp & 3, ch = warp >> 2;
  constexpr int NCP = TC_THREADS / 128;            // column parts
  constexpr int CBH = (2 * TC_NZ) / (16 * NCP);    // 16-column blocks per part
  static_assert(CBH >= 1, "at least one 16-column block per part");
  if (MODE == 0) {
    // lane quarter lq holds rows t = mt*128 + 32 lq + lane of both parities
    const int t = mt * 128 + lq * 32 + lane;
#pragma unroll
    for (int par = 0; par < 2; ++par) {
      int j = 2 * t + par;
#pragma unroll
      for (int cbi = 0; cbi < CBH; ++cbi) {
        const int cb = ch * CBH + cbi;
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + par * (2 * TC_NZ) + cb * 16, v);
        if (j < nn) {
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            int zo = z0 + cb * 8 + q;
            if (zo < nzdim)
              out[j + (size_t)nrdim * (m + (size_t)npdim * zo)] = make_double2(f2d_fast(v[2 * q]), f2d_fast(v[2 * q + 1]));
          }
        }
      }
    }
  } else {
    // lane quarter lq holds radial points i = mt*128 + 32 lq + lane: f(i) = be + bo, f(nr-1-i) = be - bo
    const int i = mt * 128 + lq * 32 + lane;
    const bool addl = add_ln && m == 0;
    const double lnv = addl ? *lnp : 0.0;
#pragma unroll
    for (int cbi = 0; cbi < CBH; ++cbi) {
      const int cb = ch * CBH + cbi;
      float ve[16], vo[16];
      tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + 0 * (2 * TC_NZ) + cb * 16, ve);
      tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + 1 * (2 * TC_NZ) + cb * 16, vo);
      if (i < nrh) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          int zo = z0 + cb * 8 + q;
          if (zo >= nzdim) continue;
          size_t b0 = (size_t)nrdim * (m + (size_t)npdim * zo);
          double2 p = make_double2(f2d_fast(ve[2 * q] + vo[2 * q]), f2d_fast(ve[2 * q + 1] + vo[2 * q + 1]));
          double2 qq = make_double2(f2d_fast(ve[2 * q] - vo[2 * q]), f2d_fast(ve[2 * q + 1] - vo[2 * q + 1]));
          if (addl) { p.x += lnv * lnx[i]; qq.x += lnv * lnx[nr - 1 - i]; }
          out[b0 + i] = p;
          out[b0 + nr - 1 - i] = qq;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

// ------------------------------------------------------------------------------------------------
// ------------------------------------------------------------------------------------------------
struct TcImg {
  uint16_t* p = nullptr;
  size_t bytes = 0;
  int nrc = -1, npc = -1;
};
static TcImg g_img[2];

void tc_free() {
  for (auto& t : g_img) {
    if (t.p) dfree(t.p, t.bytes);
    t = TcImg();
  }
}

// forward (mode 0) / backward (mode 1) contraction on the tensor cores; out zeroed by the caller
static int tc_rtrans(int mode, const cd* in, cd* out, int nrc, int npc, const double* lnp, bool add_ln) {
  int nrows = (mode == 0) ? (nrc + 1) / 2 : G.nrh;           // M: rows of a parity (fwd) / radial points (bwd)
  int nk = (mode == 0) ? G.nrh : (nrc + 1) / 2;              // K: radial points (fwd) / rows of a parity (bwd)
  int nmt = cdiv(nrows, 128), nkc = cdiv(nk, TC_KC);
  TcImg& im = g_img[mode];
  if (im.nrc != nrc || im.npc != npc || !im.p) {
    if (im.p) dfree(im.p, im.bytes);
    im = TcImg();
    im.bytes = (size_t)npc * nmt * nkc * 6 * TC_TILE_BYTES;
    MLG_TRY(dmalloc((void**)&im.p, im.bytes));
    k_tc_table<<<npc * nmt * nkc, 256, 0, G.stream>>>(G.pf, im.p, G.nrh, G.ne, nmt, nkc, nrc, mode);
    MLG_LAUNCH();
    im.nrc = nrc;
    im.npc = npc;
  }
  size_t sm = sizeof(TcSmem) + 1024;
  dim3 grid(cdiv(G.nzdim, TC_NZ), nmt, npc);
  int* st = (int*)(G.dscal + DS_FLAG + 1) + 1;
  // m >= 1 only: the m = 0 plane is contracted in double-float by the caller
  const int m0 = 1;
  if (npc <= m0) return 0;
  grid.z = npc - m0;
  if (mode == 0) {
    MLG_CUDA(cudaFuncSetAttribute(k_tc_rtrans<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_tc_rtrans<0><<<grid, TC_THREADS, sm, G.stream>>>(in, out, im.p, G.w32, G.lnx, lnp, 0, G.nr, G.nrh, G.nrdim, G.npdim,
                                                       G.nzdim, nrc, nmt, nkc, m0, st);
  } else {
    MLG_CUDA(cudaFuncSetAttribute(k_tc_rtrans<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_tc_rtrans<1><<<grid, TC_THREADS, sm, G.stream>>>(in, out, im.p, G.w32, G.lnx, lnp, add_ln ? 1 : 0, G.nr, G.nrh,
                                                       G.nrdim, G.npdim, G.nzdim, nrc, nmt, nkc, m0, st);
  }
  MLG_LAUNCH();
  return 0;
}

// The bounded-wait path of the tensor-core kernels on its own: one thread waits on an mbarrier of
// arrival count 1.  arrive = 0: nothing arrives, so the wait runs out after `limit` clocks and the
// kernel sets the timeout word exactly as k_tc_rtrans does; arrive = 1: the thread arrives first and
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

int tc_rtrans_fwd(const cd* in, cd* out, int nrc, int npc) { return tc_rtrans(0, in, out, nrc, npc, nullptr, false); }
int tc_rtrans_bwd(const cd* in, cd* out, int nrc, int npc, const double* lnp, bool add_ln) {
  return tc_rtrans(1, in, out, nrc, npc, lnp, add_ln);
}

}  // namespace mlg
