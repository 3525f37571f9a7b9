// radial.cu — the mapped-Legendre radial transforms as ragged batches of dense contractions, one
// group per azimuthal mode m:
//   forward  (rtrans_forward, mlegs_scalar_ops.f90:1852-1927)
//     c(j, m, z) = sum_{i<nr/2} pf(i, j, m) * (f(i) +- f(nr-1-i)) * w(i),  j < nn(m) = nrc - m,
//     '+' for even j (0-based), '-' for odd j;
//   backward (rtrans_backward, :1931-2008)
//     be(i) = sum_{j even} pf(i, j, m) c(j),  bo(i) = sum_{j odd} pf(i, j, m) c(j),
//     f(i) = be + bo,  f(nr-1-i) = be - bo;
//   vec2tp projection (:1402-1438), five contractions against the V, D, T matrices with the
//     eomul / oemul parity folds (:2067-2145), combined into psi and chi.
// Each CTA owns one m, one parity of rows and one tile of z columns; the folded input (f(i) +- f(nr-1-i))
// is formed while staging the K-chunk in shared memory.  The plain form accumulates in FP64 (DFMA).
// Where the exact-slice tensor-core contractions cover the grid (xs_radial.cu, xs_vec2tp.cu) they take
// m >= 1 in both forms and these kernels the m = 0 plane, in FP64 (plain) or double-float (mixed,
// below); beyond that range the FP64 kernels take every m.  The m = 0 plane carries the axisymmetric
// mean flow, and its radial functions do
// not vanish on the axis, so regular fields such as r d/dr(chi) reach zero there only by cancellation
// of their radial sums, which the 1/r of the velocity components then magnifies (about 40x at the
// innermost collocation point of a 192-point grid).
#include "common.cuh"
#include "dfloat.cuh"

namespace mlg {

// forward: grid (ztiles, 2*ttiles, npc); block (ZT/ZPT, MT/MPT)
template <typename T, int MT, int ZT, int KC, int MPT, int ZPT>
__global__ void __launch_bounds__((MT / MPT) * (ZT / ZPT))
k_rtrans_fwd(const double2* __restrict__ in, double2* __restrict__ out, const typename TabT<T>::t* __restrict__ pf,
             const double* __restrict__ w, const float* __restrict__ w32, int nr, int nrh, int ne, int nrdim, int npdim,
             int nzdim, int nrc) {
  typedef typename V2<T>::t C;
  __shared__ T As[KC][MT + 1];
  __shared__ C Bs[KC][ZT];
  int m = blockIdx.z;
  int par = blockIdx.y & 1;
  int t0 = (blockIdx.y >> 1) * MT;
  int nn = max(min(nrc, nrc - m), 0);
  if (2 * t0 + par >= nn) return;
  int z0 = blockIdx.x * ZT;
  int tx = threadIdx.x, ty = threadIdx.y;
  int nthr = blockDim.x * blockDim.y, tid = ty * blockDim.x + tx;
  T acc_r[MPT][ZPT], acc_i[MPT][ZPT];
#pragma unroll
  for (int a = 0; a < MPT; ++a)
#pragma unroll
    for (int b = 0; b < ZPT; ++b) { acc_r[a][b] = 0; acc_i[a][b] = 0; }
  const T sgn = par ? (T)-1 : (T)1;
  for (int i0 = 0; i0 < nrh; i0 += KC) {
    // A chunk: rows j = 2(t0+tt)+par, columns i0..i0+KC
    for (int idx = tid; idx < KC * MT; idx += nthr) {
      int ii = idx % KC, tt = idx / KC;
      int j = 2 * (t0 + tt) + par, i = i0 + ii;
      T v = 0;
      if (j < nn && i < nrh) v = tab<T>(pf, i + (size_t)nrh * (j + (size_t)ne * m));
      As[ii][tt] = v;
    }
    // B chunk: folded columns (f(i) +- f(nr-1-i)) * w(i)
    for (int idx = tid; idx < KC * ZT; idx += nthr) {
      int ii = idx % KC, zz = idx / KC;
      int i = i0 + ii, z = z0 + zz;
      C v; v.x = 0; v.y = 0;
      if (i < nrh && z < nzdim) {
        const double2* col = in + (size_t)nrdim * (m + (size_t)npdim * z);
        C a = ldc<T>(col + i), b = ldc<T>(col + nr - 1 - i);
        T wi = wsel<T>(w, w32, i);
        v.x = (a.x + sgn * b.x) * wi;
        v.y = (a.y + sgn * b.y) * wi;
      }
      Bs[ii][zz] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < KC; ++ii) {
      T av[MPT];
      C bv[ZPT];
#pragma unroll
      for (int a = 0; a < MPT; ++a) av[a] = As[ii][ty * MPT + a];
#pragma unroll
      for (int b = 0; b < ZPT; ++b) bv[b] = Bs[ii][tx + b * (ZT / ZPT)];
#pragma unroll
      for (int a = 0; a < MPT; ++a)
#pragma unroll
        for (int b = 0; b < ZPT; ++b) {
          acc_r[a][b] = tmac(av[a], bv[b].x, acc_r[a][b]);
          acc_i[a][b] = tmac(av[a], bv[b].y, acc_i[a][b]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < MPT; ++a) {
    int j = 2 * (t0 + ty * MPT + a) + par;
    if (j >= nn) continue;
#pragma unroll
    for (int b = 0; b < ZPT; ++b) {
      int z = z0 + tx + b * (ZT / ZPT);
      if (z < nzdim) out[j + (size_t)nrdim * (m + (size_t)npdim * z)] = to_d2<T>(acc_r[a][b], acc_i[a][b]);
    }
  }
}

// the m = 0 plane of the forward transform: one output (j, z) per thread of a slice, KS slices of the K
// range (radial points, chunks of KC dealt round-robin) in the block's z dimension, their partial sums
// added in shared memory in slice order; grid (ztiles, 2 * ttiles)
template <typename T, int MT, int ZT, int KC, int KS>
__global__ void __launch_bounds__(MT * ZT * KS)
k_rtrans_fwd_plane(const double2* __restrict__ in, double2* __restrict__ out, const typename TabT<T>::t* __restrict__ pf,
                   const double* __restrict__ w, const float* __restrict__ w32, int nr, int nrh, int nrdim, int npdim,
                   int nzdim, int nrc) {
  typedef typename V2<T>::t C;
  __shared__ T As[KS][KC][MT + 1];
  __shared__ C Bs[KS][KC][ZT];
  __shared__ C red[KS - 1][MT][ZT];
  const int par = blockIdx.y & 1, t0 = (blockIdx.y >> 1) * MT;
  const int nn = max(nrc, 0);
  if (2 * t0 + par >= nn) return;   // uniform over the block
  const int z0 = blockIdx.x * ZT;
  const int tx = threadIdx.x, ty = threadIdx.y, ks = threadIdx.z;
  const int nthr = MT * ZT, tid = ty * ZT + tx;
  C acc;
  acc.x = 0; acc.y = 0;
  const T sgn = par ? (T)-1 : (T)1;
  const int nchunk = (nrh + KC - 1) / KC, nround = (nchunk + KS - 1) / KS;
  for (int rd = 0; rd < nround; ++rd) {   // the same trip count in every slice (barriers below)
    const int i0 = (rd * KS + ks) * KC;
    for (int idx = tid; idx < KC * MT; idx += nthr) {
      const int ii = idx % KC, tt = idx / KC;
      const int j = 2 * (t0 + tt) + par, i = i0 + ii;
      T v = 0;
      if (j < nn && i < nrh) v = tab<T>(pf, i + (size_t)nrh * j);
      As[ks][ii][tt] = v;
    }
    for (int idx = tid; idx < KC * ZT; idx += nthr) {
      const int ii = idx % KC, zz = idx / KC;
      const int i = i0 + ii, z = z0 + zz;
      C v; v.x = 0; v.y = 0;
      if (i < nrh && z < nzdim) {
        const double2* col = in + (size_t)nrdim * npdim * z;
        const C a = ldc<T>(col + i), b = ldc<T>(col + nr - 1 - i);
        const T wi = wsel<T>(w, w32, i);
        v.x = (a.x + sgn * b.x) * wi;
        v.y = (a.y + sgn * b.y) * wi;
      }
      Bs[ks][ii][zz] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < KC; ++ii) {
      const T av = As[ks][ii][ty];
      const C bv = Bs[ks][ii][tx];
      acc.x = tmac(av, bv.x, acc.x);
      acc.y = tmac(av, bv.y, acc.y);
    }
    __syncthreads();
  }
  if (ks > 0) red[ks - 1][ty][tx] = acc;
  __syncthreads();
  if (ks > 0) return;
#pragma unroll
  for (int q = 0; q < KS - 1; ++q) {
    const C b = red[q][ty][tx];
    acc.x = acc.x + b.x; acc.y = acc.y + b.y;
  }
  const int j = 2 * (t0 + ty) + par, z = z0 + tx;
  if (j < nn && z < nzdim) out[j + (size_t)nrdim * npdim * z] = to_d2<T>(acc.x, acc.y);
}

// backward: tile (itile blockIdx.y, ztile blockIdx.x) of mode m; each thread owns IPT rows i and ZPT
// columns and both parities
template <typename T, int IT, int ZT, int KC, int IPT, int ZPT>
__device__ __forceinline__ void rtrans_bwd_tile(const double2* __restrict__ in, double2* __restrict__ out,
                                                const typename TabT<T>::t* __restrict__ pf, const double* __restrict__ lnx,
                                                const double* __restrict__ lnp, int add_ln, int nr, int nrh, int ne,
                                                int nrdim, int npdim, int nzdim, int nrc, int m) {
  typedef typename V2<T>::t C;
  __shared__ T Ae[KC][IT + 1], Ao[KC][IT + 1];
  __shared__ C Be[KC][ZT], Bo[KC][ZT];
  int i0 = blockIdx.y * IT;
  int z0 = blockIdx.x * ZT;
  int nn = max(min(nrc, nrc - m), 0);
  int tx = threadIdx.x, ty = threadIdx.y;
  int nthr = blockDim.x * blockDim.y, tid = ty * blockDim.x + tx;
  T er[IPT][ZPT], ei[IPT][ZPT], orr[IPT][ZPT], oi[IPT][ZPT];
#pragma unroll
  for (int a = 0; a < IPT; ++a)
#pragma unroll
    for (int b = 0; b < ZPT; ++b) { er[a][b] = 0; ei[a][b] = 0; orr[a][b] = 0; oi[a][b] = 0; }
  int nt = (nn + 1) / 2;
  for (int t0 = 0; t0 < nt; t0 += KC) {
    for (int idx = tid; idx < KC * IT; idx += nthr) {
      int ii = idx % IT, tt = idx / IT;
      int i = i0 + ii, je = 2 * (t0 + tt), jo = je + 1;
      T ve = 0, vo = 0;
      if (i < nrh) {
        if (je < nn) ve = tab<T>(pf, i + (size_t)nrh * (je + (size_t)ne * m));
        if (jo < nn) vo = tab<T>(pf, i + (size_t)nrh * (jo + (size_t)ne * m));
      }
      Ae[tt][ii] = ve; Ao[tt][ii] = vo;
    }
    for (int idx = tid; idx < KC * ZT * 2; idx += nthr) {
      int jj = idx % (2 * KC), zz = idx / (2 * KC);
      int j = 2 * t0 + jj, z = z0 + zz;
      C v; v.x = 0; v.y = 0;
      if (j < nn && z < nzdim) v = ldc<T>(in + j + (size_t)nrdim * (m + (size_t)npdim * z));
      if (jj & 1) Bo[jj >> 1][zz] = v; else Be[jj >> 1][zz] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int tt = 0; tt < KC; ++tt) {
      T ae[IPT], ao[IPT];
      C be[ZPT], bo[ZPT];
#pragma unroll
      for (int a = 0; a < IPT; ++a) { ae[a] = Ae[tt][ty * IPT + a]; ao[a] = Ao[tt][ty * IPT + a]; }
#pragma unroll
      for (int b = 0; b < ZPT; ++b) { be[b] = Be[tt][tx + b * (ZT / ZPT)]; bo[b] = Bo[tt][tx + b * (ZT / ZPT)]; }
#pragma unroll
      for (int a = 0; a < IPT; ++a)
#pragma unroll
        for (int b = 0; b < ZPT; ++b) {
          er[a][b] = tmac(ae[a], be[b].x, er[a][b]);
          ei[a][b] = tmac(ae[a], be[b].y, ei[a][b]);
          orr[a][b] = tmac(ao[a], bo[b].x, orr[a][b]);
          oi[a][b] = tmac(ao[a], bo[b].y, oi[a][b]);
        }
    }
    __syncthreads();
  }
  double lnv = (add_ln && m == 0) ? *lnp : 0.0;
#pragma unroll
  for (int a = 0; a < IPT; ++a) {
    int i = i0 + ty * IPT + a;
    if (i >= nrh) continue;
#pragma unroll
    for (int b = 0; b < ZPT; ++b) {
      int z = z0 + tx + b * (ZT / ZPT);
      if (z >= nzdim) continue;
      size_t base = (size_t)nrdim * (m + (size_t)npdim * z);
      double2 p = to_d2<T>(er[a][b] + orr[a][b], ei[a][b] + oi[a][b]);
      double2 q = to_d2<T>(er[a][b] - orr[a][b], ei[a][b] - oi[a][b]);
      if (lnv != 0.0) { p.x += lnv * lnx[i]; q.x += lnv * lnx[nr - 1 - i]; }
      out[base + i] = p;
      out[base + nr - 1 - i] = q;
    }
  }
}

// backward over modes m < gridDim.z: grid (ztiles, itiles, mcount)
template <typename T, int IT, int ZT, int KC, int IPT, int ZPT>
__global__ void __launch_bounds__((IT / IPT) * (ZT / ZPT))
k_rtrans_bwd(const double2* __restrict__ in, double2* __restrict__ out, const typename TabT<T>::t* __restrict__ pf,
             const double* __restrict__ lnx, const double* __restrict__ lnp, int add_ln, int nr, int nrh, int ne,
             int nrdim, int npdim, int nzdim, int nrc) {
  rtrans_bwd_tile<T, IT, ZT, KC, IPT, ZPT>(in, out, pf, lnx, lnp, add_ln, nr, nrh, ne, nrdim, npdim, nzdim, nrc,
                                           blockIdx.z);
}

// the m = 0 planes of up to three fields (the components of a vector field) in one launch: grid
// (ztiles, itiles, fields), one output pair (i, nr-1-i) of one column per thread of a slice.  The plane is
// 1/65 of the radial work at 192 x 128 x 128, so a grid over m alone would leave most SMs idle: small
// tiles, the fields in the grid and KS slices of the K range (rows t, chunks of KC dealt round-robin, in
// the block's z dimension, their partial sums added in shared memory in slice order) give it several
// thousand warps.
struct PlaneSet {
  const double2* in[3];
  double2* out[3];
  const double* lnp[3];
};
template <typename T, int IT, int ZT, int KC, int KS>
__global__ void __launch_bounds__(IT * ZT * KS)
k_rtrans_bwd_plane(PlaneSet ps, const typename TabT<T>::t* __restrict__ pf, const double* __restrict__ lnx, int add_ln,
                   int nr, int nrh, int ne, int nrdim, int npdim, int nzdim, int nrc) {
  typedef typename V2<T>::t C;
  __shared__ T Ae[KS][KC][IT + 1], Ao[KS][KC][IT + 1];
  __shared__ C Be[KS][KC][ZT], Bo[KS][KC][ZT];
  __shared__ T red[KS - 1][4][IT][ZT];
  const int f = blockIdx.z;
  const double2* in = f == 0 ? ps.in[0] : (f == 1 ? ps.in[1] : ps.in[2]);
  double2* out = f == 0 ? ps.out[0] : (f == 1 ? ps.out[1] : ps.out[2]);
  const double* lnp = f == 0 ? ps.lnp[0] : (f == 1 ? ps.lnp[1] : ps.lnp[2]);
  (void)ne;
  const int i0 = blockIdx.y * IT, z0 = blockIdx.x * ZT;
  const int nn = max(nrc, 0);
  const int tx = threadIdx.x, ty = threadIdx.y, ks = threadIdx.z;
  const int nthr = IT * ZT, tid = ty * ZT + tx;
  T er = 0, ei = 0, orr = 0, oi = 0;
  const int nt = (nn + 1) / 2, nchunk = (nt + KC - 1) / KC, nround = (nchunk + KS - 1) / KS;
  for (int rd = 0; rd < nround; ++rd) {   // the same trip count in every slice (barriers below)
    const int t0 = (rd * KS + ks) * KC;
    for (int idx = tid; idx < KC * IT; idx += nthr) {
      const int ii = idx % IT, tt = idx / IT;
      const int i = i0 + ii, je = 2 * (t0 + tt), jo = je + 1;
      T ve = 0, vo = 0;
      if (i < nrh) {
        if (je < nn) ve = tab<T>(pf, i + (size_t)nrh * je);
        if (jo < nn) vo = tab<T>(pf, i + (size_t)nrh * jo);
      }
      Ae[ks][tt][ii] = ve; Ao[ks][tt][ii] = vo;
    }
    for (int idx = tid; idx < KC * ZT * 2; idx += nthr) {
      const int jj = idx % (2 * KC), zz = idx / (2 * KC);
      const int j = 2 * t0 + jj, z = z0 + zz;
      C v; v.x = 0; v.y = 0;
      if (j < nn && z < nzdim) v = ldc<T>(in + j + (size_t)nrdim * npdim * z);
      if (jj & 1) Bo[ks][jj >> 1][zz] = v; else Be[ks][jj >> 1][zz] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int tt = 0; tt < KC; ++tt) {
      const T ae = Ae[ks][tt][ty], ao = Ao[ks][tt][ty];
      const C be = Be[ks][tt][tx], bo = Bo[ks][tt][tx];
      er = tmac(ae, be.x, er); ei = tmac(ae, be.y, ei);
      orr = tmac(ao, bo.x, orr); oi = tmac(ao, bo.y, oi);
    }
    __syncthreads();
  }
  if (ks > 0) { red[ks - 1][0][ty][tx] = er; red[ks - 1][1][ty][tx] = ei; red[ks - 1][2][ty][tx] = orr; red[ks - 1][3][ty][tx] = oi; }
  __syncthreads();
  if (ks > 0) return;
#pragma unroll
  for (int q = 0; q < KS - 1; ++q) {
    er = er + red[q][0][ty][tx]; ei = ei + red[q][1][ty][tx];
    orr = orr + red[q][2][ty][tx]; oi = oi + red[q][3][ty][tx];
  }
  const int i = i0 + ty, z = z0 + tx;
  if (i >= nrh || z >= nzdim) return;
  const size_t base = (size_t)nrdim * npdim * z;
  double2 p = to_d2<T>(er + orr, ei + oi);
  double2 q = to_d2<T>(er - orr, ei - oi);
  if (add_ln) { const double lnv = *lnp; p.x += lnv * lnx[i]; q.x += lnv * lnx[nr - 1 - i]; }
  out[base + i] = p;
  out[base + nr - 1 - i] = q;
}

// vec2tp: psi(j) = -i m (V.F_s(ur))_j - (D.F_o(up))_j,
//         chi(j) = i k (D.F_o(ur))_j + m k (V.F_s(up))_j - (T.F_s(uz))_j
// F_s is the fold of the row's own parity (eomul), F_o the other one (oemul); no weights (they are
// inside V, D, T).  Only k slots 1..nzc and nzcu..nzdim are produced.
template <typename T, int MT, int ZT, int KC, int ZPT>
__global__ void __launch_bounds__(MT * (ZT / ZPT))
k_vec2tp(const double2* __restrict__ ur, const double2* __restrict__ up, const double2* __restrict__ uz,
         double2* __restrict__ psi, double2* __restrict__ chi, const typename TabT<T>::t* __restrict__ tV,
         const typename TabT<T>::t* __restrict__ tD, const typename TabT<T>::t* __restrict__ tT, const double* __restrict__ ak, int nr, int nrh, int ne, int nrdim, int npdim,
         int nzdim, int nrc, int nzc, int nzcu, int m0) {
  typedef typename V2<T>::t C;
  __shared__ T Av[KC][MT + 1], Ad[KC][MT + 1], At[KC][MT + 1];
  __shared__ C Brs[KC][ZT], Bro[KC][ZT], Bps[KC][ZT], Bpo[KC][ZT], Bzs[KC][ZT];
  int m = blockIdx.z + m0;
  int par = blockIdx.y & 1;
  int t0 = (blockIdx.y >> 1) * MT;
  int nn = max(min(nrc, nrc - m), 0);
  if (2 * t0 + par >= nn) return;
  int z0 = blockIdx.x * ZT;
  int tx = threadIdx.x, ty = threadIdx.y;
  int nthr = blockDim.x * blockDim.y, tid = ty * blockDim.x + tx;
  C a1[ZPT], a2[ZPT], a3[ZPT], a4[ZPT], a5[ZPT];
#pragma unroll
  for (int b = 0; b < ZPT; ++b) {
    a1[b].x = a1[b].y = 0; a2[b].x = a2[b].y = 0; a3[b].x = a3[b].y = 0; a4[b].x = a4[b].y = 0; a5[b].x = a5[b].y = 0;
  }
  const T ss = par ? (T)-1 : (T)1;   // own-parity fold sign
  for (int i0 = 0; i0 < nrh; i0 += KC) {
    for (int idx = tid; idx < KC * MT; idx += nthr) {
      int ii = idx % KC, tt = idx / KC;
      int j = 2 * (t0 + tt) + par, i = i0 + ii;
      T v = 0, d = 0, t = 0;
      if (j < nn && i < nrh) {
        size_t o = i + (size_t)nrh * (j + (size_t)ne * m);
        v = tab<T>(tV, o); d = tab<T>(tD, o); t = tab<T>(tT, o);
      }
      Av[ii][tt] = v; Ad[ii][tt] = d; At[ii][tt] = t;
    }
    for (int idx = tid; idx < KC * ZT; idx += nthr) {
      int ii = idx % KC, zz = idx / KC;
      int i = i0 + ii, z = z0 + zz;
      C rs, ro, ps, po, zs;
      rs.x = rs.y = ro.x = ro.y = ps.x = ps.y = po.x = po.y = zs.x = zs.y = 0;
      if (i < nrh && z < nzdim) {
        size_t base = (size_t)nrdim * (m + (size_t)npdim * z);
        C a = ldc<T>(ur + base + i), b = ldc<T>(ur + base + nr - 1 - i);
        rs.x = a.x + ss * b.x; rs.y = a.y + ss * b.y;
        ro.x = a.x - ss * b.x; ro.y = a.y - ss * b.y;
        a = ldc<T>(up + base + i); b = ldc<T>(up + base + nr - 1 - i);
        ps.x = a.x + ss * b.x; ps.y = a.y + ss * b.y;
        po.x = a.x - ss * b.x; po.y = a.y - ss * b.y;
        a = ldc<T>(uz + base + i); b = ldc<T>(uz + base + nr - 1 - i);
        zs.x = a.x + ss * b.x; zs.y = a.y + ss * b.y;
      }
      Brs[ii][zz] = rs; Bro[ii][zz] = ro; Bps[ii][zz] = ps; Bpo[ii][zz] = po; Bzs[ii][zz] = zs;
    }
    __syncthreads();
#pragma unroll 2
    for (int ii = 0; ii < KC; ++ii) {
      T v = Av[ii][ty], d = Ad[ii][ty], t = At[ii][ty];
#pragma unroll
      for (int b = 0; b < ZPT; ++b) {
        int zz = tx + b * (ZT / ZPT);
        C rs = Brs[ii][zz], ro = Bro[ii][zz], ps = Bps[ii][zz], po = Bpo[ii][zz], zs = Bzs[ii][zz];
        a1[b].x = tmac(v, rs.x, a1[b].x); a1[b].y = tmac(v, rs.y, a1[b].y);   // V.F_s(ur)
        a2[b].x = tmac(d, po.x, a2[b].x); a2[b].y = tmac(d, po.y, a2[b].y);   // D.F_o(up)
        a3[b].x = tmac(d, ro.x, a3[b].x); a3[b].y = tmac(d, ro.y, a3[b].y);   // D.F_o(ur)
        a4[b].x = tmac(v, ps.x, a4[b].x); a4[b].y = tmac(v, ps.y, a4[b].y);   // V.F_s(up)
        a5[b].x = tmac(t, zs.x, a5[b].x); a5[b].y = tmac(t, zs.y, a5[b].y);   // T.F_s(uz)
      }
    }
    __syncthreads();
  }
  int j = 2 * (t0 + ty) + par;
  if (j >= nn) return;
  T mv = (T)m;
#pragma unroll
  for (int b = 0; b < ZPT; ++b) {
    int z = z0 + tx + b * (ZT / ZPT);
    if (z >= nzdim) continue;
    int kk = z + 1;
    if (!(kk <= nzc || kk >= nzcu)) continue;
    T kv = (T)ak[z];
    T w1x = m ? a1[b].x : (T)0, w1y = m ? a1[b].y : (T)0;
    T w2x = a2[b].x, w2y = a2[b].y;
    // psi = -i*mv*w1 - w2
    double2 p = to_d2<T>(mv * w1y - w2x, -mv * w1x - w2y);
    T v1x = a3[b].x, v1y = a3[b].y;
    T v2x = m ? a4[b].x : (T)0, v2y = m ? a4[b].y : (T)0;
    T cx = a5[b].x, cy = a5[b].y;
    // chi = i*kv*w1' + mv*kv*w2' - c
    double2 q = to_d2<T>(-kv * v1y + mv * kv * v2x - cx, kv * v1x + mv * kv * v2y - cy);
    size_t o = j + (size_t)nrdim * (m + (size_t)npdim * z);
    psi[o] = p;
    chi[o] = q;
  }
}

// the m = 0 plane of vec2tp (mixed form, double-float): the m V terms vanish at m = 0, so
//   psi = -D.F_o(up),   chi = i k D.F_o(ur) - T.F_s(uz),
// three contractions instead of five.  One output (j, z) per thread of a slice; KS slices of the K
// range (radial points, chunks of KC dealt round-robin) in the block's z dimension give the plane
// several thousand warps, and their partial sums are added in shared memory in slice order.
template <typename T, int MT, int ZT, int KC, int KS>
__global__ void __launch_bounds__(MT * ZT * KS)
k_vec2tp_plane(const double2* __restrict__ ur, const double2* __restrict__ up, const double2* __restrict__ uz,
               double2* __restrict__ psi, double2* __restrict__ chi, const typename TabT<T>::t* __restrict__ tD,
               const typename TabT<T>::t* __restrict__ tT, const double* __restrict__ ak, int nr, int nrh, int ne,
               int nrdim, int npdim, int nzdim, int nrc, int nzc, int nzcu) {
  typedef typename V2<T>::t C;
  __shared__ T Ad[KS][KC][MT + 1], At[KS][KC][MT + 1];
  __shared__ C Bro[KS][KC][ZT], Bpo[KS][KC][ZT], Bzs[KS][KC][ZT];
  __shared__ C red[KS - 1][3][MT][ZT];
  const int par = blockIdx.y & 1, t0 = (blockIdx.y >> 1) * MT;
  const int nn = max(nrc, 0);
  if (2 * t0 + par >= nn) return;   // uniform over the block
  const int z0 = blockIdx.x * ZT;
  const int tx = threadIdx.x, ty = threadIdx.y, ks = threadIdx.z;
  const int nthr = MT * ZT, tid = ty * ZT + tx;
  C a2, a3, a5;   // D.F_o(up), D.F_o(ur), T.F_s(uz)
  a2.x = a2.y = 0; a3.x = a3.y = 0; a5.x = a5.y = 0;
  const T ss = par ? (T)-1 : (T)1;
  const int nchunk = (nrh + KC - 1) / KC, nround = (nchunk + KS - 1) / KS;
  for (int rd = 0; rd < nround; ++rd) {   // the same trip count in every slice (barriers below)
    const int i0 = (rd * KS + ks) * KC;
    for (int idx = tid; idx < KC * MT; idx += nthr) {
      const int ii = idx % KC, tt = idx / KC;
      const int j = 2 * (t0 + tt) + par, i = i0 + ii;
      T d = 0, t = 0;
      if (j < nn && i < nrh) {
        const size_t o = i + (size_t)nrh * j;
        d = tab<T>(tD, o); t = tab<T>(tT, o);
      }
      Ad[ks][ii][tt] = d; At[ks][ii][tt] = t;
    }
    for (int idx = tid; idx < KC * ZT; idx += nthr) {
      const int ii = idx % KC, zz = idx / KC;
      const int i = i0 + ii, z = z0 + zz;
      C ro, po, zs;
      ro.x = ro.y = po.x = po.y = zs.x = zs.y = 0;
      if (i < nrh && z < nzdim) {
        const size_t base = (size_t)nrdim * npdim * z;
        C a = ldc<T>(ur + base + i), b = ldc<T>(ur + base + nr - 1 - i);
        ro.x = a.x - ss * b.x; ro.y = a.y - ss * b.y;
        a = ldc<T>(up + base + i); b = ldc<T>(up + base + nr - 1 - i);
        po.x = a.x - ss * b.x; po.y = a.y - ss * b.y;
        a = ldc<T>(uz + base + i); b = ldc<T>(uz + base + nr - 1 - i);
        zs.x = a.x + ss * b.x; zs.y = a.y + ss * b.y;
      }
      Bro[ks][ii][zz] = ro; Bpo[ks][ii][zz] = po; Bzs[ks][ii][zz] = zs;
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < KC; ++ii) {
      const T d = Ad[ks][ii][ty], t = At[ks][ii][ty];
      const C ro = Bro[ks][ii][tx], po = Bpo[ks][ii][tx], zs = Bzs[ks][ii][tx];
      a2.x = tmac(d, po.x, a2.x); a2.y = tmac(d, po.y, a2.y);
      a3.x = tmac(d, ro.x, a3.x); a3.y = tmac(d, ro.y, a3.y);
      a5.x = tmac(t, zs.x, a5.x); a5.y = tmac(t, zs.y, a5.y);
    }
    __syncthreads();
  }
  if (ks > 0) { red[ks - 1][0][ty][tx] = a2; red[ks - 1][1][ty][tx] = a3; red[ks - 1][2][ty][tx] = a5; }
  __syncthreads();
  if (ks > 0) return;
#pragma unroll
  for (int q = 0; q < KS - 1; ++q) {
    const C b2 = red[q][0][ty][tx], b3 = red[q][1][ty][tx], b5 = red[q][2][ty][tx];
    a2.x = a2.x + b2.x; a2.y = a2.y + b2.y;
    a3.x = a3.x + b3.x; a3.y = a3.y + b3.y;
    a5.x = a5.x + b5.x; a5.y = a5.y + b5.y;
  }
  const int j = 2 * (t0 + ty) + par, z = z0 + tx;
  if (j >= nn || z >= nzdim) return;
  const int kk = z + 1;
  if (!(kk <= nzc || kk >= nzcu)) return;
  const T kv = (T)ak[z];
  // psi = -D.F_o(up); chi = i k D.F_o(ur) - T.F_s(uz)
  const double2 p = to_d2<T>(-a2.x, -a2.y);
  const double2 q = to_d2<T>(-(kv * a3.y) - a5.x, kv * a3.x - a5.y);
  const size_t o = j + (size_t)nrdim * npdim * z;
  psi[o] = p;
  chi[o] = q;
}

static int rtrans_check(const Scalar& s, int& nrc, int& npc, const char* who) {
  nrc = G.nrchop + s.off[0];
  npc = G.npchop + s.off[1];
  if (nrc > G.nrdim || nrc > G.ne) return set_error(MLG_ECHOP, std::string(who) + ": chopping in r too large");
  if (npc > G.npdim) return set_error(MLG_ECHOP, std::string(who) + ": chopping in p too large");
  if (npc > G.npchop) return set_error(MLG_ECHOP, std::string(who) + ": chopping in p beyond the table");
  return 0;
}

static double fwd_flops(int nrc, int npc) {
  double f = 0;
  for (int m = 0; m < npc; ++m) f += 4.0 * std::max(std::min(nrc, nrc - m), 0) * G.nrh * G.nzdim;
  return f;
}

// The m = 0 plane, in double-float (mixed form) or FP64 (plain form), with small tiles: the plane is
// 1/65 of the radial work at 192 x 128 x 128, and the tiles of the all-m kernels would give it a few
// dozen CTAs.  Forward: 16 x 8 tiles with four K slices (192 CTAs of 512 threads at 192 x 128 x 128).
template <typename T>
static int plane_rtrans_fwd(const cd* in, cd* out, int nrc, cudaStream_t st) {
  constexpr int MT = 16, ZT = 8, KC = 8, KS = 4;
  int nn = std::max(nrc, 0);
  if (nn == 0) return 0;
  dim3 grid(cdiv(G.nzdim, ZT), 2 * cdiv((nn + 1) / 2, MT), 1), blk(ZT, MT, KS);
  k_rtrans_fwd_plane<T, MT, ZT, KC, KS><<<grid, blk, 0, st>>>(in, out, G.pf, G.w, G.w32, G.nr, G.nrh, G.nrdim, G.npdim,
                                                              G.nzdim, nrc);
  MLG_LAUNCH();
  return 0;
}
// Backward: the planes of n <= 3 fields in one launch, 8 x 16 tiles with four K slices (288 CTAs of 512
// threads for three fields at 192 x 128 x 128).
template <typename T>
static int plane_rtrans_bwd(const cd* const* in, cd* const* out, const double* const* lnp, int n, int nrc, bool add_ln,
                            cudaStream_t st) {
  constexpr int IT = 8, ZT = 16, KC = 8, KS = 4;
  if (nrc <= 0 || n < 1) return 0;
  if (n > 3) return set_error(MLG_EPARAM, "rtrans_backward: at most three m = 0 planes per launch");
  PlaneSet ps;
  for (int f = 0; f < 3; ++f) {
    const int g = f < n ? f : 0;
    ps.in[f] = in[g]; ps.out[f] = out[g]; ps.lnp[f] = lnp[g];
  }
  dim3 grid(cdiv(G.nzdim, ZT), cdiv(G.nrh, IT), n), blk(ZT, IT, KS);
  k_rtrans_bwd_plane<T, IT, ZT, KC, KS><<<grid, blk, 0, st>>>(ps, G.pf, G.lnx, add_ln ? 1 : 0, G.nr, G.nrh, G.ne, G.nrdim,
                                                              G.npdim, G.nzdim, nrc);
  MLG_LAUNCH();
  return 0;
}
// the m = 0 plane of one or more fields in the arithmetic of the form: double-float (mixed), FP64 (plain)
static int plane_bwd(const cd* const* in, cd* const* out, const double* const* lnp, int n, int nrc, bool add_ln,
                     cudaStream_t st) {
  return G.precision == MLG_MIXED ? plane_rtrans_bwd<dfl>(in, out, lnp, n, nrc, add_ln, st)
                                  : plane_rtrans_bwd<double>(in, out, lnp, n, nrc, add_ln, st);
}
static int plane_fwd(const cd* in, cd* out, int nrc, cudaStream_t st) {
  return G.precision == MLG_MIXED ? plane_rtrans_fwd<dfl>(in, out, nrc, st) : plane_rtrans_fwd<double>(in, out, nrc, st);
}


// the rows of each column (m, z) of a mixed-form contraction's output that its kernels leave
// unwritten, to zero: mode 0 (forward radial transform, projection) rows >= nn(m), and the whole column
// where z is outside the kept band k <= nzc or k >= nzcu; mode 1 (backward radial transform) rows >= nr
// (the padding), the whole column where nn(m) = 0; columns m >= npc whole.  One warp per column.
__global__ void k_zero_tails(double2* __restrict__ out0, double2* __restrict__ out1, double2* __restrict__ out2, int nf,
                             int mode, int nr, int nrdim, int npdim, int nzdim, int nrc, int npc, int nzc, int nzcu) {
  const int lane = threadIdx.x & 31;
  const size_t ncols = (size_t)npdim * nzdim, nw = (size_t)gridDim.x * (blockDim.x >> 5);
  for (size_t cf = blockIdx.x * (size_t)(blockDim.x >> 5) + (threadIdx.x >> 5); cf < ncols * nf; cf += nw) {
    const int f = (int)(cf / ncols);
    const size_t c = cf - (size_t)f * ncols;
    const int m = (int)(c % npdim), kk = (int)(c / npdim) + 1;
    const int nn = (m < npc && (kk <= nzc || kk >= nzcu)) ? max(min(nrc, nrc - m), 0) : 0;
    const int lim = mode == 0 ? nn : (nn > 0 ? nr : 0);
    double2* col = (f == 0 ? out0 : (f == 1 ? out1 : out2)) + (size_t)nrdim * c;
    for (int j = lim + lane; j < nrdim; j += 32) col[j] = make_double2(0.0, 0.0);
  }
}

// the tails of n <= 3 outputs with the same chop in one launch (on G.stream, or on the side stream
// beside the contraction that writes the other rows)
int launch_zero_tails_n(cd* const* out, int n, int mode, int nrc, int npc, int nzc, int nzcu, cudaStream_t st) {
  if (n < 1 || n > 3) return set_error(MLG_EPARAM, "zero_tails: one to three fields per launch");
  const size_t ncols = (size_t)G.npdim * G.nzdim * n;
  k_zero_tails<<<(int)std::min<size_t>(cdiv(ncols, 8), 152 * 8), 256, 0, st ? st : G.stream>>>(
      out[0], n > 1 ? out[1] : out[0], n > 2 ? out[2] : out[0], n, mode, G.nr, G.nrdim, G.npdim, G.nzdim, nrc, npc, nzc, nzcu);
  MLG_LAUNCH();
  return 0;
}
int launch_zero_tails(cd* out, int mode, int nrc, int npc, int nzc, int nzcu) {
  return launch_zero_tails_n(&out, 1, mode, nrc, npc, nzc, nzcu);
}

// the FP64 DFMA contractions over every m < mcount (kits the exact-slice contraction does not cover)
static int dfma_rtrans_fwd(const cd* in, cd* out, int nrc, int mcount, cudaStream_t st) {
  constexpr int MT = 32, ZT = 32, KC = 16, MPT = 2, ZPT = 4;
  int tt = cdiv((nrc + 1) / 2, MT);
  dim3 grid(cdiv(G.nzdim, ZT), 2 * tt, mcount), blk(ZT / ZPT, MT / MPT);
  k_rtrans_fwd<double, MT, ZT, KC, MPT, ZPT><<<grid, blk, 0, st>>>(in, out, G.pf, G.w, G.w32, G.nr, G.nrh, G.ne, G.nrdim,
                                                                    G.npdim, G.nzdim, nrc);
  MLG_LAUNCH();
  return 0;
}
static int dfma_rtrans_bwd(const cd* in, cd* out, int nrc, int mcount, const double* lnp, bool add_ln, cudaStream_t st) {
  constexpr int IT = 32, ZT = 32, KC = 8, IPT = 2, ZPT = 2;
  dim3 grid(cdiv(G.nzdim, ZT), cdiv(G.nrh, IT), mcount), blk(ZT / ZPT, IT / IPT);
  k_rtrans_bwd<double, IT, ZT, KC, IPT, ZPT><<<grid, blk, 0, st>>>(in, out, G.pf, G.lnx, lnp, add_ln ? 1 : 0, G.nr, G.nrh,
                                                                    G.ne, G.nrdim, G.npdim, G.nzdim, nrc);
  MLG_LAUNCH();
  return 0;
}

int launch_rtrans_fwd(Scalar& s) {
  int nrc, npc;
  MLG_TRY(rtrans_check(s, nrc, npc, "rtrans_forward"));
  cd* out = get_buf();
  if (!out) return set_error(MLG_EALLOC, "rtrans_forward: out of device memory");
  const bool mixed = G.precision == MLG_MIXED;
  const bool xs = xs_supported(0, nrc, !mixed);   // exact-slice tensor-core contraction (xs_radial.cu)
  // the tensor-core contractions write rows < nn(m) of every column m < npc: only the rest needs zeros
  // (beside them, below)
  if (xs && npc < 1) {
    MLG_TRY(launch_zero_tails(out, 0, nrc, npc, G.nzdim, G.nzdim + 1));
  } else if (!xs) {
    MLG_CUDA(cudaMemsetAsync(out, 0, G.fsize * sizeof(cd), G.stream));
  }
  kt_begin(KT_RFWD);
  if (npc > 0) {
    if (xs) {
      // m = 0 (the axisymmetric mean flow, whose large range within a column the fixed-point slices
      // would cut relative to its maximum) beside, in double-float (mixed) or FP64 (plain), after the
      // zeros of the rows that no contraction writes; m >= 1 as exact slices, 42-bit (mixed) or
      // FP64-grade (plain)
      MLG_TRY(side_fork());
      cd* o1[1] = {out};
      MLG_TRY(launch_zero_tails_n(o1, 1, 0, nrc, npc, G.nzdim, G.nzdim + 1, G.side));
      MLG_TRY(plane_fwd(s.e, out, nrc, G.side));
      MLG_TRY(xs_rtrans(0, s.e, out, nrc, npc, 1, nullptr, false, !mixed));
      MLG_TRY(side_join());
    } else {
      // beyond the slices' range (their orders would not stay exact): FP64 DFMA over every m, in both forms
      MLG_TRY(dfma_rtrans_fwd(s.e, out, nrc, npc, G.stream));
    }
  }
  kt_end(KT_RFWD, fwd_flops(nrc, npc));
  put_buf(s.e);
  s.e = out;
  return 0;
}

int launch_rtrans_bwd(Scalar& s, bool add_ln) {
  int nrc, npc;
  MLG_TRY(rtrans_check(s, nrc, npc, "rtrans_backward"));
  cd* out = get_buf();
  if (!out) return set_error(MLG_EALLOC, "rtrans_backward: out of device memory");
  const bool mixed = G.precision == MLG_MIXED;
  const bool xs = xs_supported(1, nrc, !mixed);
  // the tensor-core contractions write rows < nr of every column m < npc with nn(m) > 0 (the m = 0
  // plane included): only the rest needs zeros (beside them, below)
  if (xs && npc < 1) {
    MLG_TRY(launch_zero_tails(out, 1, nrc, npc, G.nzdim, G.nzdim + 1));
  } else if (!xs) {
    MLG_CUDA(cudaMemsetAsync(out, 0, G.fsize * sizeof(cd), G.stream));
  }
  kt_begin(KT_RBWD);
  if (npc > 0) {
    if (xs) {
      // m = 0 beside in double-float (mixed) or FP64 DFMA (plain), after the zeros; m >= 1 as exact
      // slices
      MLG_TRY(side_fork());
      cd* o1[1] = {out};
      MLG_TRY(launch_zero_tails_n(o1, 1, 1, nrc, npc, G.nzdim, G.nzdim + 1, G.side));
      MLG_TRY(plane_bwd(&s.e, &out, &s.ln, 1, nrc, add_ln, G.side));
      MLG_TRY(xs_rtrans(1, s.e, out, nrc, npc, 1, s.ln, add_ln, !mixed));
      MLG_TRY(side_join());
    } else {
      // beyond the slices' range: FP64 DFMA over every m, in both forms
      MLG_TRY(dfma_rtrans_bwd(s.e, out, nrc, npc, s.ln, add_ln, G.stream));
    }
  }
  kt_end(KT_RBWD, fwd_flops(nrc, npc));
  put_buf(s.e);
  s.e = out;
  return 0;
}

// the forward transforms of n fields (n <= 3) with the same chop: one tensor-core launch over all of
// them (the m = 0 planes beside it, one launch each), else field by field
int launch_rtrans_fwd_multi(Scalar* const* f, int n) {
  if (n == 1) return launch_rtrans_fwd(*f[0]);
  int nrc = 0, npc = 0;
  for (int i = 0; i < n; ++i) {
    int a, b;
    MLG_TRY(rtrans_check(*f[i], a, b, "rtrans_forward"));
    if (i == 0) { nrc = a; npc = b; }
    if (a != nrc || b != npc || n > 3) {   // different chops: one at a time
      for (int k = 0; k < n; ++k) MLG_TRY(launch_rtrans_fwd(*f[k]));
      return 0;
    }
  }
  const bool mixed = G.precision == MLG_MIXED;
  const bool xs = xs_supported(0, nrc, !mixed);
  if (!xs || npc < 1) {
    for (int k = 0; k < n; ++k) MLG_TRY(launch_rtrans_fwd(*f[k]));
    return 0;
  }
  cd* out[3] = {nullptr, nullptr, nullptr};
  const cd* in[3] = {nullptr, nullptr, nullptr};
  for (int i = 0; i < n; ++i) {
    out[i] = get_buf();
    if (!out[i]) {
      for (int k = 0; k < i; ++k) put_buf(out[k]);
      return set_error(MLG_EALLOC, "rtrans_forward: out of device memory");
    }
    in[i] = f[i]->e;
  }
  kt_begin(KT_RFWD);
  MLG_TRY(side_fork());
  // beside the m >= 1 contraction: the rows it does not write (zero), then the m = 0 planes
  MLG_TRY(launch_zero_tails_n(out, n, 0, nrc, npc, G.nzdim, G.nzdim + 1, G.side));
  for (int i = 0; i < n; ++i) MLG_TRY(plane_fwd(in[i], out[i], nrc, G.side));   // m = 0 beside
  MLG_TRY(xs_rtrans_multi(0, in, out, n, nrc, npc, 1, nullptr, false, !mixed));   // m >= 1, all fields
  MLG_TRY(side_join());
  kt_end(KT_RFWD, n * fwd_flops(nrc, npc));
  for (int i = 0; i < n; ++i) {
    put_buf(f[i]->e);
    f[i]->e = out[i];
  }
  return 0;
}

// the backward transforms of n fields (n <= 3, the components of a vector field) with the same chop:
// one tensor-core launch over all of them (and the m = 0 planes beside it), else field by field
int launch_rtrans_bwd_multi(Scalar* const* f, int n, bool add_ln) {
  if (n == 1) return launch_rtrans_bwd(*f[0], add_ln);
  int nrc = 0, npc = 0;
  for (int i = 0; i < n; ++i) {
    int a, b;
    MLG_TRY(rtrans_check(*f[i], a, b, "rtrans_backward"));
    if (i == 0) { nrc = a; npc = b; }
    if (a != nrc || b != npc || n > 3) {   // different chops: one at a time
      for (int k = 0; k < n; ++k) MLG_TRY(launch_rtrans_bwd(*f[k], add_ln));
      return 0;
    }
  }
  const bool mixed = G.precision == MLG_MIXED;
  const bool xs = xs_supported(1, nrc, !mixed);
  if (!xs || npc < 1) {
    for (int k = 0; k < n; ++k) MLG_TRY(launch_rtrans_bwd(*f[k], add_ln));
    return 0;
  }
  cd* out[3] = {nullptr, nullptr, nullptr};
  const cd* in[3] = {nullptr, nullptr, nullptr};
  const double* lnp[3] = {nullptr, nullptr, nullptr};
  for (int i = 0; i < n; ++i) {
    out[i] = get_buf();
    if (!out[i]) {
      for (int k = 0; k < i; ++k) put_buf(out[k]);
      return set_error(MLG_EALLOC, "rtrans_backward: out of device memory");
    }
    in[i] = f[i]->e;
    lnp[i] = f[i]->ln;
  }
  kt_begin(KT_RBWD);
  MLG_TRY(side_fork());
  // beside the m >= 1 contraction: the rows it does not write (zero), then the m = 0 planes of all
  // fields in one launch: double-float (mixed) or FP64 DFMA (plain)
  MLG_TRY(launch_zero_tails_n(out, n, 1, nrc, npc, G.nzdim, G.nzdim + 1, G.side));
  MLG_TRY(plane_bwd(in, out, lnp, n, nrc, add_ln, G.side));
  MLG_TRY(xs_rtrans_multi(1, in, out, n, nrc, npc, 1, lnp, add_ln, !mixed));   // m >= 1, all fields
  MLG_TRY(side_join());
  kt_end(KT_RBWD, n * fwd_flops(nrc, npc));
  for (int i = 0; i < n; ++i) {
    put_buf(f[i]->e);
    f[i]->e = out[i];
  }
  return 0;
}

// ur, up, uz in (r physical, m, k) space; psi and chi written in full
int launch_vec2tp_contract(const cd* ur, const cd* up, const cd* uz, cd* psi, cd* chi, int nrc_off) {
  int nrc = G.nrchop + nrc_off, npc = G.npchop;
  int nzc = G.chopzl, nzcu = G.chopzu;
  if (nrc > G.ne || nrc > G.nrdim) return set_error(MLG_ECHOP, "vec2tp: chopping in r too large");
  const bool mixed = G.precision == MLG_MIXED;
  // the exact-slice tensor-core contraction (xs_vec2tp.cu) in the mixed form; the plain form keeps the
  // FP64 contraction: chi = k X - Y cancels, and the slices' truncation relative to the column maxima
  // (54-bit digits) left chi 7e-9 from the FP64 reference on the 32^3 kit (sliced radial transforms
  // hold 1e-12 there)
  const bool xv = mixed && xv_supported();
  // the tensor-core contractions write rows < nn(m) of the kept columns: only the rest needs zeros
  // (beside them, below)
  if (!xv) {
    MLG_CUDA(cudaMemsetAsync(psi, 0, G.fsize * sizeof(cd), G.stream));
    MLG_CUDA(cudaMemsetAsync(chi, 0, G.fsize * sizeof(cd), G.stream));
  }
  kt_begin(KT_V2TP);
  constexpr int MT = 16, ZT = 32, KC = 16, ZPT = 4;
  int tt = cdiv((nrc + 1) / 2, MT);
  dim3 grid(cdiv(G.nzdim, ZT), 2 * tt, npc), blk(ZT / ZPT, MT);
  if (xv) {
    // m >= 1 on the tensor cores as exact slices, m = 0 in double-float beside it (after the zeros)
    MLG_TRY(side_fork());
    cd* pc[2] = {psi, chi};
    MLG_TRY(launch_zero_tails_n(pc, 2, 0, nrc, npc, nzc, nzcu, G.side));
    constexpr int DMT = 16, DZT = 8, DKC = 8, DKS = 4;
    dim3 dgrid(cdiv(G.nzdim, DZT), 2 * cdiv((nrc + 1) / 2, DMT), 1), dblk(DZT, DMT, DKS);
    k_vec2tp_plane<dfl, DMT, DZT, DKC, DKS><<<dgrid, dblk, 0, G.side>>>(ur, up, uz, psi, chi, G.tD, G.tT, G.ak, G.nr, G.nrh,
                                                                         G.ne, G.nrdim, G.npdim, G.nzdim, nrc, nzc, nzcu);
    MLG_LAUNCH();
    MLG_TRY(xv_contract(ur, up, uz, psi, chi, nrc, npc, 1));   // m >= 1: 35/49-bit slices
    MLG_TRY(side_join());
    kt_end(KT_V2TP, 5.0 * fwd_flops(nrc, npc));
    return 0;
  } else   // the plain form, and the mixed form beyond the slices' range: FP64 DFMA over every m
    k_vec2tp<double, MT, ZT, KC, ZPT><<<grid, blk, 0, G.stream>>>(ur, up, uz, psi, chi, G.tV, G.tD, G.tT, G.ak, G.nr,
                                                                   G.nrh, G.ne, G.nrdim, G.npdim, G.nzdim, nrc, nzc, nzcu, 0);
  MLG_LAUNCH();
  kt_end(KT_V2TP, 5.0 * fwd_flops(nrc, npc));
  return 0;
}

}  // namespace mlg
