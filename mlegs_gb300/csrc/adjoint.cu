// adjoint.cu — the discrete adjoint of the 3-D vortex step and of the operators it is built from.
// The reference has no adjoint; this is new functionality behind the same scalar API.
//
// Inner product.  <a, b> = sum over every stored entry of Re(conj(a.e) b.e) + a.ln * b.ln: the
// Euclidean product of the real and imaginary parts of the whole (nrdim, npdim, nzdim) array plus
// the log-term coefficient.  Every *_T routine applies the exact transpose, under this product, of
// the forward routine it is named after, as that routine is implemented in this library (padding
// rows, chopped slots, the shared Nyquist slot and the log-term bookkeeping included), so
// <F x, y> = <x, F^T y> holds to rounding for each of them.  An adjoint variable is stored in a
// Scalar and labelled with the space of the forward quantity it is the adjoint of.
//
// The step.  With SVV off and hyperpow = 0 the vortex step is a polynomial map of its state
// (psi, chi, nl_psi, nl_chi, nl_psi_prev, nl_chi_prev): linear operators around one bilinear
// product u x omega.  Its transpose needs the state at the end of the step (the point the next
// nonlinear term is evaluated at); the driver keeps the full state every K steps and recomputes
// each K-step segment forward before sweeping it backward.
//
// Objective.  J = 1/2 sum_{i < nr, phi, z} W_i |u'|^2 with u' the velocity of (psi, chi) without
// their axisymmetric, z-independent column (m = 0, k = 0, all n, and ln), and
// W_i = w_i r_i^2 / (1 - x_i^2) * (2 pi / np) * (zlen / nz) the quadrature of the volume integral
// r dr dphi dz over the mapped Gauss-Legendre points (dr/dx = r / (1 - x^2)).
#include "common.cuh"
#include <cstring>
#include "dfloat.cuh"
#include <cmath>
#include <vector>

namespace mlg {

int vfft_checked_T(Scalar& s, int dir);

// ------------------------------------------------------------------------------------------------
// kernels

// hfft forward^T, before the half-complex-to-real sum: slot 0 and slot L scaled 1/np, the interior
// 1/(2 np) (the forward's X_k for 0 < k < L stands for two conjugate terms of the real sum)
// up to three fields of one transposed transform, the field of a block being blockIdx.y (selected
// without an indexed access to the kernel parameter, which would copy it to local memory)
struct Fields3 {
  double2* e[3];
  double2* buf[3];
  double* ln[3];
};
template <class P> __device__ __forceinline__ P f3sel(const P (&p)[3]) {
  return blockIdx.y == 0 ? p[0] : (blockIdx.y == 1 ? p[1] : p[2]);
}

__global__ void k_hfftT_pre(Fields3 fs, int nrdim, int npdim, int nzdim, int L, double np) {
  double2* __restrict__ e = f3sel(fs.e);
  size_t n = (size_t)nrdim * (L + 1) * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int k = (int)((idx / (unsigned)nrdim) % (unsigned)(L + 1));
    int z = (int)(idx / (unsigned)(nrdim * (L + 1)));
    double f = (k == 0 || k == L) ? 1.0 / np : 0.5 / np;
    double2* p = e + i + (size_t)nrdim * (k + (size_t)npdim * z);
    p->x *= f; p->y *= f;
  }
}

// slot L of every (r, z) row: saved to buf (save = 1) or zeroed (save = 0)
__global__ void k_slotL(Fields3 fs, int nrdim, int npdim, int nzdim, int L, int save) {
  double2* __restrict__ e = f3sel(fs.e);
  double2* __restrict__ buf = f3sel(fs.buf);
  size_t n = (size_t)nrdim * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int z = (int)(idx / (unsigned)nrdim);
    double2* p = e + i + (size_t)nrdim * (L + (size_t)npdim * z);
    if (save) buf[idx] = *p;
    else *p = make_double2(0.0, 0.0);
  }
}

// hfft backward^T, after the unnormalised real-to-half-complex sum X_k = sum_j f_j e^{-2 pi i jk/np}:
// interior doubled; slot L also takes np times the saved adjoint of the forward's slot-L copy
__global__ void k_hfftT_post(Fields3 fs, int nrdim, int npdim, int nzdim, int L, double np) {
  double2* __restrict__ e = f3sel(fs.e);
  const double2* __restrict__ buf = f3sel(fs.buf);
  size_t n = (size_t)nrdim * (L + 1) * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int k = (int)((idx / (unsigned)nrdim) % (unsigned)(L + 1));
    int z = (int)(idx / (unsigned)(nrdim * (L + 1)));
    double2* p = e + i + (size_t)nrdim * (k + (size_t)npdim * z);
    if (k > 0 && k < L) { p->x *= 2.0; p->y *= 2.0; }
    if (k == L) { double2 b = buf[i + (size_t)nrdim * z]; p->x += np * b.x; p->y += np * b.y; }
  }
}

// rows i < nr of every column scaled by tab[i] (inv = 0) or divided by it (inv = 1)
__global__ void k_scale_tab(Fields3 fs, const double* __restrict__ tab, int nr, int nrdim, size_t ncol, int inv) {
  double2* __restrict__ e = f3sel(fs.e);
  size_t n = (size_t)nr * ncol;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nr);
    unsigned c = idx / (unsigned)nr;
    double2* p = e + i + (size_t)nrdim * c;
    double v = inv ? 1.0 / tab[i] : tab[i];
    p->x *= v; p->y *= v;
  }
}

// *lnp += sgn * sum_{i < nr, z} lnx_i Re e(i, 0, z): the adjoint of e(:nr, 1, :) += ln * lnx
__global__ void __launch_bounds__(1024) k_ln_dot(Fields3 fs, const double* __restrict__ lnx, int nr, int nrdim, int npdim,
                                                 int nzdim, double sgn) {
  const double2* __restrict__ e = f3sel(fs.e);
  double* __restrict__ lnp = f3sel(fs.ln);
  __shared__ double red[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double s = 0.0;
  for (int z = warp; z < nzdim; z += 32) {   // a warp per z line, its lanes over r (coalesced)
    const double2* col = e + (size_t)nrdim * npdim * z;
    for (int i = lane; i < nr; i += 32) s += lnx[i] * col[i].x;
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (warp == 0) {
    s = red[lane];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) *lnp += sgn * s;
  }
}

// zeroat1^T: the forward sets e(0,0,k) <- e(0,0,k) - sum_{n<nmax} at_n e(n,0,k) / at_0, so
// e_bar(n,0,k) -= at_n / at_0 * e_bar(0,0,k) for n < nmax (which leaves e_bar(0,0,k) = 0); warp per k
// one warp per k of e0 and, when e1 is given, of e1
__global__ void k_zeroat1_T(double2* __restrict__ e0, double2* __restrict__ e1, const double* __restrict__ at, int nmax,
                            int nrdim, int npdim, int nzdim) {
  const int kf = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (kf >= (e1 ? 2 : 1) * nzdim) return;
  const int k = kf < nzdim ? kf : kf - nzdim;
  double2* col = (kf < nzdim ? e0 : e1) + (size_t)nrdim * npdim * k;
  double bx = 0.0, by = 0.0;
  if (lane == 0) { bx = col[0].x; by = col[0].y; }
  bx = __shfl_sync(0xffffffffu, bx, 0);
  by = __shfl_sync(0xffffffffu, by, 0);
  double a0 = at[0];
  for (int n = lane; n < nmax; n += 32) {
    double f = at[n] / a0;
    col[n].x -= f * bx;
    col[n].y -= f * by;
  }
}

// ihelm^T log term, after the transposed solve: the forward took lno = ln / alpha and
// e(n,0,0).x -= cf_n lno with cf = (4/3, -2, 2/3) / (ell^2 exp(lognorm_n))
__global__ void k_ihelm_T_ln(const double2* __restrict__ e, double* __restrict__ lnp, const double* __restrict__ lognorm,
                             double ell, double alpha) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double e2 = ell * ell;
  double lno = *lnp - (4.0 / 3.0 / e2 / exp(lognorm[0]) * e[0].x - 2.0 / 1.0 / e2 / exp(lognorm[1]) * e[1].x +
                       2.0 / 3.0 / e2 / exp(lognorm[2]) * e[2].x);
  *lnp = lno / alpha;
}

// idel2_proln^T log term, before the transposed solve: the forward set ln = Re x(0,0,0) exp(lognorm_0)
// and ignored the incoming ln
__global__ void k_idel2_T_ln(double2* __restrict__ e, double* __restrict__ lnp, const double* __restrict__ lognorm) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  e[0].x += *lnp * exp(lognorm[0]);
  *lnp = 0.0;
}

// calcat^T of vec2tp: the forward set psi%ln = -1/2 Re sum_{n<nmax} at1_n up(n,0,0)
__global__ void k_calcat_T(double2* __restrict__ e, const double* __restrict__ at, int nmax, const double* __restrict__ lnbar,
                           double f) {
  double l = *lnbar;
  for (int n = threadIdx.x; n < nmax; n += blockDim.x) e[n].x += f * at[n] * l;
}

// *lnp += sum_{i < nr} (1 + x_i) Re e(i, 0, 0): the adjoint of k_add_ln_x
__global__ void k_add_ln_x_T(const double2* __restrict__ e, const double* __restrict__ x, int nr, double* __restrict__ lnp) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) s += (1.0 + x[i]) * e[i].x;
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *lnp += red[0];
}

// k_tp2vec_mix^T.  Forward on the active entries: ur <- i m psi + i k ur, up <- -up - m k uz;
// transposed (conjugate coefficients): psi_bar += -i m ur_bar, uz_bar += -m k up_bar,
// ur_bar <- -i k ur_bar, up_bar <- -up_bar; the other entries pass through unchanged.
__global__ void k_tp2vec_mix_T(double2* __restrict__ ur, double2* __restrict__ up, double2* __restrict__ psi,
                               double2* __restrict__ uz, const double* __restrict__ ak, int nrdim, int npdim, int nzdim,
                               int nrc, int npc, int nzc, int nzcu) {
  size_t n = (size_t)nrdim * npdim * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int m = (int)((idx / (unsigned)nrdim) % (unsigned)npdim);
    int k = (int)(idx / (unsigned)(nrdim * npdim));
    if (m >= npc) continue;
    int nn = max(min(nrc, nrc - m), 0);
    int kk = k + 1;
    if (i >= nn || !(kk <= nzc || kk >= nzcu)) continue;
    double kv = ak[k], mv = (double)m;
    double2 a = ur[idx], b = up[idx];
    psi[idx].x += mv * a.y;  psi[idx].y -= mv * a.x;   // -i m a
    uz[idx].x -= mv * kv * b.x;  uz[idx].y -= mv * kv * b.y;
    ur[idx] = make_double2(kv * a.y, -kv * a.x);        // -i k a
    up[idx] = make_double2(-b.x, -b.y);
  }
}

// vecprod^T around (v, w): the forward o = v x w on each packed real (i < nr, slots < np/2; zero
// elsewhere); <o_bar, dv x w + v x dw> gives v_bar = w x o_bar, w_bar = o_bar x v
__global__ void k_vecprod_T(double2* __restrict__ vbr, double2* __restrict__ vbp, double2* __restrict__ vbz,
                            double2* __restrict__ wbr, double2* __restrict__ wbp, double2* __restrict__ wbz,
                            const double2* __restrict__ vr, const double2* __restrict__ vp, const double2* __restrict__ vz,
                            const double2* __restrict__ wr, const double2* __restrict__ wp, const double2* __restrict__ wz,
                            const double2* __restrict__ obr, const double2* __restrict__ obp, const double2* __restrict__ obz,
                            int nr, int nph, int nrdim, int npdim, int nzdim) {
  size_t n = (size_t)nrdim * npdim * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int m = (int)((idx / (unsigned)nrdim) % (unsigned)npdim);
    double2 a1 = make_double2(0, 0), a2 = a1, a3 = a1, b1 = a1, b2 = a1, b3 = a1;
    if (i < nr && m < nph) {
      double2 V1 = vr[idx], V2 = vp[idx], V3 = vz[idx], W1 = wr[idx], W2 = wp[idx], W3 = wz[idx];
      double2 O1 = obr[idx], O2 = obp[idx], O3 = obz[idx];
      // w x o
      a1 = make_double2(W2.x * O3.x - W3.x * O2.x, W2.y * O3.y - W3.y * O2.y);
      a2 = make_double2(W3.x * O1.x - W1.x * O3.x, W3.y * O1.y - W1.y * O3.y);
      a3 = make_double2(W1.x * O2.x - W2.x * O1.x, W1.y * O2.y - W2.y * O1.y);
      // o x v
      b1 = make_double2(O2.x * V3.x - O3.x * V2.x, O2.y * V3.y - O3.y * V2.y);
      b2 = make_double2(O3.x * V1.x - O1.x * V3.x, O3.y * V1.y - O1.y * V3.y);
      b3 = make_double2(O1.x * V2.x - O2.x * V1.x, O1.y * V2.y - O2.y * V1.y);
    }
    vbr[idx] = a1; vbp[idx] = a2; vbz[idx] = a3;
    wbr[idx] = b1; wbp[idx] = b2; wbz[idx] = b3;
  }
}

// The vec2tp contraction transposed.  Forward, row j of parity p (sign s = +1 for even p, -1 odd):
//   psi_j = -i m (V F_s(ur))_j - (D F_o(up))_j
//   chi_j = i k (D F_o(ur))_j + m k (V F_s(up))_j - (T F_s(uz))_j
// with F_s(u)_i = u_i + s u_{nr-1-i}, F_o(u)_i = u_i - s u_{nr-1-i}, i < nr/2.  Transposed, per
// parity: S1 = V^T psi_bar, S2 = D^T psi_bar, S3 = D^T chi_bar, S4 = V^T chi_bar, S5 = T^T chi_bar
// (sums over that parity's rows), then F_s_bar(ur) = i m S1, F_o_bar(ur) = -i k S3,
// F_s_bar(up) = m k S4, F_o_bar(up) = -S2, F_s_bar(uz) = -S5, unfolded as
// u_bar_i += F_s_bar + F_o_bar, u_bar_{nr-1-i} += s (F_s_bar - F_o_bar).
// One CTA per (m, z tile, i tile); each thread one (i, z) pair; rows staged in shared memory.
template <typename T, int IT, int ZT, int KC>
__global__ void __launch_bounds__(IT * ZT / 2)
k_vec2tp_T(const double2* __restrict__ psib, const double2* __restrict__ chib, double2* __restrict__ urb,
           double2* __restrict__ upb, double2* __restrict__ uzb, const typename TabT<T>::t* __restrict__ tV,
           const typename TabT<T>::t* __restrict__ tD, const typename TabT<T>::t* __restrict__ tT,
           const double* __restrict__ ak, int nr, int nrh, int ne, int nrdim, int npdim, int nzdim, int nrc, int nzc,
           int nzcu, int m0) {
  typedef typename V2<T>::t C;
  __shared__ T Vs[KC][IT + 1], Ds[KC][IT + 1], Ts[KC][IT + 1];
  __shared__ C Ps[KC][ZT], Cs[KC][ZT];
  int m = blockIdx.z + m0;
  int i0 = blockIdx.y * IT, z0 = blockIdx.x * ZT;
  int nn = max(min(nrc, nrc - m), 0);
  int tz = threadIdx.x % ZT, ti = threadIdx.x / ZT;   // ZT columns x (IT/2) rows of threads
  constexpr int NT = IT * ZT / 2;
  // two i per thread: ti and ti + IT/2
  C S[2][2][5];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 0; q < 5; ++q) { S[a][p][q].x = 0; S[a][p][q].y = 0; }
  int z = z0 + tz;
  int kk = z + 1;
  bool zact = z < nzdim && (kk <= nzc || kk >= nzcu);
  for (int j0 = 0; j0 < nn; j0 += KC) {
    for (int idx = threadIdx.x; idx < KC * IT; idx += NT) {
      int jj = idx / IT, ii = idx % IT;
      int j = j0 + jj, i = i0 + ii;
      T v = 0, d = 0, t = 0;
      if (j < nn && i < nrh) {
        size_t o = i + (size_t)nrh * (j + (size_t)ne * m);
        v = tab<T>(tV, o); d = tab<T>(tD, o); t = tab<T>(tT, o);
      }
      Vs[jj][ii] = v; Ds[jj][ii] = d; Ts[jj][ii] = t;
    }
    for (int idx = threadIdx.x; idx < KC * ZT; idx += NT) {
      int jj = idx / ZT, zz = idx % ZT;
      int j = j0 + jj, zg = z0 + zz;
      C pv, cv;
      pv.x = 0; pv.y = 0; cv = pv;
      if (j < nn && zg < nzdim) {
        size_t o = j + (size_t)nrdim * (m + (size_t)npdim * zg);
        pv = ldc<T>(psib + o); cv = ldc<T>(chib + o);
      }
      Ps[jj][zz] = pv; Cs[jj][zz] = cv;
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < KC; ++jj) {
      int p = (j0 + jj) & 1;
      C pv = Ps[jj][tz], cv = Cs[jj][tz];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        int ii = ti + a * (IT / 2);
        T v = Vs[jj][ii], d = Ds[jj][ii], t = Ts[jj][ii];
        S[a][p][0].x = tmac(v, pv.x, S[a][p][0].x); S[a][p][0].y = tmac(v, pv.y, S[a][p][0].y);
        S[a][p][1].x = tmac(d, pv.x, S[a][p][1].x); S[a][p][1].y = tmac(d, pv.y, S[a][p][1].y);
        S[a][p][2].x = tmac(d, cv.x, S[a][p][2].x); S[a][p][2].y = tmac(d, cv.y, S[a][p][2].y);
        S[a][p][3].x = tmac(v, cv.x, S[a][p][3].x); S[a][p][3].y = tmac(v, cv.y, S[a][p][3].y);
        S[a][p][4].x = tmac(t, cv.x, S[a][p][4].x); S[a][p][4].y = tmac(t, cv.y, S[a][p][4].y);
      }
    }
    __syncthreads();
  }
  if (!zact) return;
  T kv = (T)ak[z], mv = (T)m;
  size_t base = (size_t)nrdim * (m + (size_t)npdim * z);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    int i = i0 + ti + a * (IT / 2);
    if (i >= nrh) continue;
    C r_lo, r_hi, p_lo, p_hi, z_lo, z_hi;
    r_lo.x = 0; r_lo.y = 0; r_hi = r_lo; p_lo = r_lo; p_hi = r_lo; z_lo = r_lo; z_hi = r_lo;
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      T sg = p ? (T)-1 : (T)1;
      C S1 = S[a][p][0], S2 = S[a][p][1], S3 = S[a][p][2], S4 = S[a][p][3], S5 = S[a][p][4];
      C fs_r, fo_r, fs_p, fo_p, fs_z;
      fs_r.x = -mv * S1.y; fs_r.y = mv * S1.x;              // i m S1
      fo_r.x = kv * S3.y; fo_r.y = -kv * S3.x;              // -i k S3
      fs_p.x = mv * kv * S4.x; fs_p.y = mv * kv * S4.y;
      fo_p.x = -S2.x; fo_p.y = -S2.y;
      fs_z.x = -S5.x; fs_z.y = -S5.y;
      r_lo.x = r_lo.x + (fs_r.x + fo_r.x); r_lo.y = r_lo.y + (fs_r.y + fo_r.y);
      r_hi.x = r_hi.x + sg * (fs_r.x - fo_r.x); r_hi.y = r_hi.y + sg * (fs_r.y - fo_r.y);
      p_lo.x = p_lo.x + (fs_p.x + fo_p.x); p_lo.y = p_lo.y + (fs_p.y + fo_p.y);
      p_hi.x = p_hi.x + sg * (fs_p.x - fo_p.x); p_hi.y = p_hi.y + sg * (fs_p.y - fo_p.y);
      z_lo.x = z_lo.x + fs_z.x; z_lo.y = z_lo.y + fs_z.y;
      z_hi.x = z_hi.x + sg * fs_z.x; z_hi.y = z_hi.y + sg * fs_z.y;
    }
    urb[base + i] = to_d2<T>(r_lo.x, r_lo.y); urb[base + nr - 1 - i] = to_d2<T>(r_hi.x, r_hi.y);
    upb[base + i] = to_d2<T>(p_lo.x, p_lo.y); upb[base + nr - 1 - i] = to_d2<T>(p_hi.x, p_hi.y);
    uzb[base + i] = to_d2<T>(z_lo.x, z_lo.y); uzb[base + nr - 1 - i] = to_d2<T>(z_hi.x, z_hi.y);
  }
}

// The m = 0 plane of k_vec2tp_T in double-float: one warp per output pair (i, z), the lanes over the
// row pairs (2t, 2t+1) -- the two parities.  With m = 0 the terms in S1 and S4 vanish, and the unfolded
// outputs are F_o_bar(ur) = -i k S3, F_o_bar(up) = -S2, F_s_bar(uz) = -S5 per parity: six complex sums,
// reduced by shuffles.
__global__ void __launch_bounds__(256) k_m0_vec2tp_T_df(const double2* __restrict__ psib, const double2* __restrict__ chib,
                                                        double2* __restrict__ urb, double2* __restrict__ upb,
                                                        double2* __restrict__ uzb, const double* __restrict__ tD,
                                                        const double* __restrict__ tT,
                                                        const double* __restrict__ ak, int nr, int nrh, int nrdim,
                                                        int npdim, int nzdim, int nn, int nzc, int nzcu) {
  const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  const int i = wid % nrh, z = wid / nrh;
  if (z >= nzdim) return;
  const int kk = z + 1;
  if (!(kk <= nzc || kk >= nzcu)) return;
  const size_t base = (size_t)nrdim * npdim * z;
  dfl2 S[2][5];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 5; ++q) { S[p][q].x = 0; S[p][q].y = 0; }
  for (int t = lane; 2 * t < nn; t += 32) {
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      const int j = 2 * t + p;
      if (j >= nn) break;
      const size_t o = i + (size_t)nrh * j;
      // V enters only through S1 and S4, which m = 0 multiplies by zero
      const dfl d(tD[o]), tt(tT[o]);
      const dfl2 pv = ldc<dfl>(psib + base + j), cv = ldc<dfl>(chib + base + j);
      S[p][1].x = tmac(d, pv.x, S[p][1].x); S[p][1].y = tmac(d, pv.y, S[p][1].y);
      S[p][2].x = tmac(d, cv.x, S[p][2].x); S[p][2].y = tmac(d, cv.y, S[p][2].y);
      S[p][4].x = tmac(tt, cv.x, S[p][4].x); S[p][4].y = tmac(tt, cv.y, S[p][4].y);
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1)
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 1; q < 5; ++q) {
        if (q == 3) continue;
        S[p][q].x = S[p][q].x + df_shfl_xor(S[p][q].x, o);
        S[p][q].y = S[p][q].y + df_shfl_xor(S[p][q].y, o);
      }
  if (lane != 0) return;
  const dfl kv(ak[z]);
  dfl2 r_lo, r_hi, p_lo, p_hi, z_lo, z_hi;
  r_lo.x = 0; r_lo.y = 0; r_hi = r_lo; p_lo = r_lo; p_hi = r_lo; z_lo = r_lo; z_hi = r_lo;
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const dfl sg = p ? dfl(-1) : dfl(1);
    const dfl2 S2 = S[p][1], S3 = S[p][2], S5 = S[p][4];
    dfl2 fo_r, fo_p, fs_z;
    fo_r.x = kv * S3.y; fo_r.y = -(kv * S3.x);   // -i k S3
    fo_p.x = -S2.x; fo_p.y = -S2.y;
    fs_z.x = -S5.x; fs_z.y = -S5.y;
    r_lo.x = r_lo.x + fo_r.x; r_lo.y = r_lo.y + fo_r.y;
    r_hi.x = r_hi.x + sg * (-fo_r.x); r_hi.y = r_hi.y + sg * (-fo_r.y);
    p_lo.x = p_lo.x + fo_p.x; p_lo.y = p_lo.y + fo_p.y;
    p_hi.x = p_hi.x + sg * (-fo_p.x); p_hi.y = p_hi.y + sg * (-fo_p.y);
    z_lo.x = z_lo.x + fs_z.x; z_lo.y = z_lo.y + fs_z.y;
    z_hi.x = z_hi.x + sg * fs_z.x; z_hi.y = z_hi.y + sg * fs_z.y;
  }
  urb[base + i] = to_d2<dfl>(r_lo.x, r_lo.y); urb[base + nr - 1 - i] = to_d2<dfl>(r_hi.x, r_hi.y);
  upb[base + i] = to_d2<dfl>(p_lo.x, p_lo.y); upb[base + nr - 1 - i] = to_d2<dfl>(p_hi.x, p_hi.y);
  uzb[base + i] = to_d2<dfl>(z_lo.x, z_lo.y); uzb[base + nr - 1 - i] = to_d2<dfl>(z_hi.x, z_hi.y);
}

// J = 1/2 sum W_i |u|^2 over i < nr, slots < np/2 (both packed reals), every z; u_bar = W u
// (zero elsewhere); one partial sum per block
__global__ void k_energy(double2* __restrict__ ubr, double2* __restrict__ ubp, double2* __restrict__ ubz,
                         const double2* __restrict__ vr, const double2* __restrict__ vp, const double2* __restrict__ vz,
                         const double* __restrict__ wq, int nr, int nph, int nrdim, int npdim, int nzdim,
                         double* __restrict__ partial) {
  __shared__ double red[256];
  double s = 0.0;
  size_t n = (size_t)nrdim * npdim * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int m = (int)((idx / (unsigned)nrdim) % (unsigned)npdim);
    double2 a = vr[idx], b = vp[idx], c = vz[idx];
    double q = (i < nr && m < nph) ? wq[i] : 0.0;
    s += 0.5 * q * (a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y);
    if (ubr) {
      ubr[idx] = make_double2(q * a.x, q * a.y);
      ubp[idx] = make_double2(q * b.x, q * b.y);
      ubz[idx] = make_double2(q * c.x, q * c.y);
    }
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// W_i = w_i r_i^2 / (1 - x_i^2) * dphi * dz
__global__ void k_energy_weights(double* __restrict__ wq, const double* __restrict__ x, const double* __restrict__ w,
                                 const double* __restrict__ r, int nr, double dpz) {
  for (int i = threadIdx.x; i < nr; i += blockDim.x) wq[i] = w[i] * r[i] * r[i] / (1.0 - x[i] * x[i]) * dpz;
}

// the perturbation: the (m = 0, k = 0) column and ln removed
__global__ void k_drop_mean(double2* __restrict__ e, double* __restrict__ lnp, int nrdim) {
  for (int i = threadIdx.x; i < nrdim; i += blockDim.x) e[i] = make_double2(0.0, 0.0);
  if (threadIdx.x == 0) *lnp = 0.0;
}

// ------------------------------------------------------------------------------------------------
// transposed operators on Scalars (each in place on the adjoint variable s)

static Fields3 fields3(Scalar* const* s, int n, cd* const* bufs = nullptr) {
  Fields3 f{};
  for (int i = 0; i < 3; ++i) {
    const int g = i < n ? i : 0;
    f.e[i] = s[g]->e;
    f.buf[i] = bufs ? bufs[g] : nullptr;
    f.ln[i] = s[g]->ln;
  }
  return f;
}

// The transposed transform steps of n <= 3 fields in one launch each (the components of a vector
// field, each field's own sequence of operations unchanged).
static int hfft_fwd_T_n(Scalar* const* s, int n) {   // PFP-side adjoint -> PPP-side
  if (G.np <= 1) return 0;
  const int L = G.np / 2;
  const Fields3 fs = fields3(s, n);
  k_hfftT_pre<<<dim3(nblk((size_t)G.nrdim * (L + 1) * G.nzdim), n), 256, 0, G.stream>>>(fs, G.nrdim, G.npdim, G.nzdim, L,
                                                                                       (double)G.np);
  MLG_LAUNCH();
  cd* e[3];
  for (int i = 0; i < n; ++i) e[i] = s[i]->e;
  MLG_TRY(launch_hfft_bwd_buf_n(e, n));
  k_slotL<<<dim3(nblk((size_t)G.nrdim * G.nzdim), n), 256, 0, G.stream>>>(fs, G.nrdim, G.npdim, G.nzdim, L, 0);
  MLG_LAUNCH();
  return 0;
}

static int hfft_bwd_T_n(Scalar* const* s, int n) {   // PPP-side adjoint -> PFP-side
  if (G.np <= 1) return 0;
  const int L = G.np / 2;
  cd* bufs[3] = {nullptr, nullptr, nullptr};
  for (int i = 0; i < n; ++i) {
    bufs[i] = get_buf();
    if (!bufs[i]) {
      for (int k = 0; k < i; ++k) put_buf(bufs[k]);
      return set_error(MLG_EALLOC, "adjoint: out of device memory");
    }
  }
  const Fields3 fs = fields3(s, n, bufs);
  k_slotL<<<dim3(nblk((size_t)G.nrdim * G.nzdim), n), 256, 0, G.stream>>>(fs, G.nrdim, G.npdim, G.nzdim, L, 1);
  int rc = 0;
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) rc = set_error(MLG_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(err));
  ++G.launches;
  cd* e[3];
  for (int i = 0; i < n; ++i) e[i] = s[i]->e;
  if (!rc) rc = launch_hfft_fwd_scaled_n(e, n, 1.0);
  if (!rc) {
    k_hfftT_post<<<dim3(nblk((size_t)G.nrdim * (L + 1) * G.nzdim), n), 256, 0, G.stream>>>(fs, G.nrdim, G.npdim, G.nzdim, L,
                                                                                          (double)G.np);
    ++G.launches;
    err = cudaGetLastError();
    if (err != cudaSuccess) rc = set_error(MLG_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(err));
  }
  for (int i = 0; i < n; ++i) put_buf(bufs[i]);
  return rc;
}

static int scale_tab_n(Scalar* const* s, int n, const double* tab, int inv) {
  size_t ncol = (size_t)G.npdim * G.nzdim;
  k_scale_tab<<<dim3(nblk((size_t)G.nr * ncol), n), 256, 0, G.stream>>>(fields3(s, n), tab, G.nr, G.nrdim, ncol, inv);
  MLG_LAUNCH();
  return 0;
}
static int scale_tab(Scalar& s, const double* tab, int inv) { Scalar* p = &s; return scale_tab_n(&p, 1, tab, inv); }

static int ln_dot_n(Scalar* const* s, int n, double sgn) {
  k_ln_dot<<<dim3(1, n), 1024, 0, G.stream>>>(fields3(s, n), G.lnx, G.nr, G.nrdim, G.npdim, G.nzdim, sgn);
  MLG_LAUNCH();
  return 0;
}

// the PFP -> FFP step (e(:nr,1,:) -= ln lnx, then rtrans_forward) transposed: FFP-side -> PFP-side.
// rtrans_forward^T = w * rtrans_backward (the quadrature weights are symmetric about the fold).
static int rtrans_fwd_T_n(Scalar* const* s, int n) {
  MLG_TRY(launch_rtrans_bwd_multi(s, n, false));
  MLG_TRY(scale_tab_n(s, n, G.w, 0));
  return ln_dot_n(s, n, -1.0);
}

// the FFP -> PFP step (rtrans_backward with the log term) transposed: PFP-side -> FFP-side.
// rtrans_backward^T = rtrans_forward of the input divided by the weights.
static int rtrans_bwd_T_n(Scalar* const* s, int n, bool with_ln) {
  if (with_ln) MLG_TRY(ln_dot_n(s, n, 1.0));
  MLG_TRY(scale_tab_n(s, n, G.w, 1));
  return launch_rtrans_fwd_multi(s, n);
}
static int rtrans_bwd_T(Scalar& s, bool with_ln) { Scalar* p = &s; return rtrans_bwd_T_n(&p, 1, with_ln); }

// transpose of vertical_fft (dir -1 forward, +1 backward) of n fields with the same z chop
static int vfft_checked_T_n(Scalar* const* s, int n, int dir) {
  if (G.nz <= 1) return 0;
  cd* e[3];
  for (int i = 0; i < n; ++i) {
    int nzc = G.chopzl + s[i]->off[2], nzcu = G.chopzu - s[i]->off[2];
    if (2 * s[i]->off[2] > nzcu - nzc) return set_error(MLG_ECHOP, "vertical_fft: chopping in z too large");
    e[i] = s[i]->e;
  }
  // forward: (1/nz) sum e^{-}; its transpose (1/nz) sum e^{+}.  backward: sum e^{+}; transpose sum e^{-}
  return dir < 0 ? launch_vfft_scaled_n(e, n, +1, 1.0 / G.nz) : launch_vfft_scaled_n(e, n, -1, 1.0);
}
int vfft_checked_T(Scalar& s, int dir) { Scalar* p = &s; return vfft_checked_T_n(&p, 1, dir); }

static int space_idx(const char* sp) {
  if (!std::strncmp(sp, "PPP", 3)) return 0;
  if (!std::strncmp(sp, "PFP", 3)) return 1;
  if (!std::strncmp(sp, "FFP", 3)) return 2;
  if (!std::strncmp(sp, "FFF", 3)) return 3;
  return -1;
}
static const char* SPACES[4] = {"PPP", "PFP", "FFP", "FFF"};

// trans^T: s holds the adjoint of trans(x, s.space) applied to an x in fwd_from; afterwards s holds
// the adjoint w.r.t. x (labelled fwd_from)
// n <= 3 fields in the same space: each step of the transform for all of them in one launch
static int trans_T_n(Scalar* const* s, int n, const char* fwd_from) {
  int to = space_idx(s[0]->space), from = space_idx(fwd_from);
  if (to < 0 || from < 0) return set_error(MLG_ESPACE, "trans adjoint: unknown space");
  for (int i = 1; i < n; ++i)
    if (space_idx(s[i]->space) != to) return set_error(MLG_ESPACE, "trans adjoint: a batch of fields in different spaces");
  if (from < to) {          // forward went up: undo the steps from the top
    for (int c = to; c > from; --c) {
      if (c == 3) MLG_TRY(vfft_checked_T_n(s, n, -1));
      if (c == 2) MLG_TRY(rtrans_fwd_T_n(s, n));
      if (c == 1) MLG_TRY(hfft_fwd_T_n(s, n));
      for (int i = 0; i < n; ++i) s[i]->set_space(SPACES[c - 1]);
    }
  } else if (from > to) {   // forward went down
    for (int c = to; c < from; ++c) {
      if (c == 0) MLG_TRY(hfft_bwd_T_n(s, n));
      if (c == 1) MLG_TRY(rtrans_bwd_T_n(s, n, true));
      if (c == 2) MLG_TRY(vfft_checked_T_n(s, n, +1));
      for (int i = 0; i < n; ++i) s[i]->set_space(SPACES[c + 1]);
    }
  }
  return 0;
}
int trans_T(Scalar& s, const char* fwd_from) {
  Scalar* p = &s;
  return trans_T_n(&p, 1, fwd_from);
}

int band_T(Scalar& s, int op) {   // xxdx (0), del2h (1), del2 (2)
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  return launch_band_apply_T(s, op, c);
}

int ihelm_T(Scalar& s, double alpha) {
  if (std::fabs(alpha) < 5.0e-14) return set_error(MLG_EALPHA, "ihelm: alpha equals to zero. Inversion of 0*identity is impossible");
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  MLG_TRY(launch_band_solve_T(s, 0, c, alpha));
  k_ihelm_T_ln<<<1, 32, 0, G.stream>>>(s.e, s.ln, G.lognorm, G.ell, alpha);
  MLG_LAUNCH();
  return 0;
}

// ihelm^T of two fields with the same alpha: one paired substitution when their chop windows agree
static int ihelm_T_pair(Scalar& s1, Scalar& s2, double alpha) {
  if (std::fabs(alpha) < 5.0e-14) return set_error(MLG_EALPHA, "ihelm: alpha equals to zero. Inversion of 0*identity is impossible");
  ChopIdx c1, c2;
  MLG_TRY(chop_index(s1, c1));
  MLG_TRY(chop_index(s2, c2));
  if (!(c1.nrc == c2.nrc && c1.npc == c2.npc && c1.nzc == c2.nzc && c1.nzcu == c2.nzcu)) {
    MLG_TRY(ihelm_T(s1, alpha));
    return ihelm_T(s2, alpha);
  }
  MLG_TRY(launch_band_solve_T_pair(s1, s2, c1, alpha));
  for (Scalar* s : {&s1, &s2}) {
    k_ihelm_T_ln<<<1, 32, 0, G.stream>>>(s->e, s->ln, G.lognorm, G.ell, alpha);
    MLG_LAUNCH();
  }
  return 0;
}

int idel2_proln_T(Scalar& s) {
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  k_idel2_T_ln<<<1, 32, 0, G.stream>>>(s.e, s.ln, G.lognorm);
  MLG_LAUNCH();
  return launch_band_solve_T(s, 1, c, 0.0);
}

int zeroat1_T(Scalar& s) {
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  int nmax = std::min(std::min(G.nrdim, c.nrc), G.nrchop);
  k_zeroat1_T<<<cdiv(G.nzdim, 4), 128, 0, G.stream>>>(s.e, nullptr, G.at1, nmax, G.nrdim, G.npdim, G.nzdim);
  MLG_LAUNCH();
  return 0;
}
// zeroat1^T of two distinct fields with the same chop in one launch
static int zeroat1_T2(Scalar& a, Scalar& b) {
  ChopIdx ca, cb;
  MLG_TRY(chop_index(a, ca));
  MLG_TRY(chop_index(b, cb));
  const int na = std::min(std::min(G.nrdim, ca.nrc), G.nrchop), nb = std::min(std::min(G.nrdim, cb.nrc), G.nrchop);
  if (na != nb || a.e == b.e) {
    MLG_TRY(zeroat1_T(a));
    return zeroat1_T(b);
  }
  k_zeroat1_T<<<cdiv(2 * G.nzdim, 4), 128, 0, G.stream>>>(a.e, b.e, G.at1, na, G.nrdim, G.npdim, G.nzdim);
  MLG_LAUNCH();
  return 0;
}

static int set_fff0(Scalar& s) { s.set_space("FFF"); s.off[0] = s.off[1] = s.off[2] = 0; return 0; }

// op_tp2vec^T: (vr_bar, vp_bar, vz_bar) in PPP -> (psi_bar, chi_bar) in FFF, overwritten
int tp2vec_T(const Scalar& vrb, const Scalar& vpb, const Scalar& vzb, Scalar& psib, Scalar& chib) {
  TMP(ur); TMP(up); TMP(uz);
  MLG_TRY(assign(ur, vrb)); MLG_TRY(assign(up, vpb)); MLG_TRY(assign(uz, vzb));
  for (Scalar* q : {&ur, &up, &uz}) { q->set_space("PPP"); q->off[0] = q->off[1] = q->off[2] = 0; }
  // u_z branch: del2h (offset 3), negation, chop, trans to PPP; u_r, u_phi branches: xxdx (offset 3),
  // combination, chop, trans to PPP, division by r.  The branches are independent: the transposed
  // transforms and chops of the three fields run together, each field's own sequence unchanged.
  MLG_TRY(scale_r(ur, 1)); MLG_TRY(scale_r(up, 1));
  Scalar* f3[3] = {&uz, &ur, &up};
  MLG_TRY(trans_T_n(f3, 3, "FFF"));
  MLG_TRY(op_mask_n(f3, 3, true, false));
  MLG_TRY(lincomb(uz, {{&uz, -1.0}}, {}, 1.0, false));
  uz.off[0] = 3;
  MLG_TRY(band_T(uz, 1));
  ur.off[0] = 3; up.off[0] = 3;
  ChopIdx c;
  MLG_TRY(chop_index(ur, c));
  MLG_TRY(launch_zero(psib.e));
  k_tp2vec_mix_T<<<nblk(G.fsize), 256, 0, G.stream>>>(ur.e, up.e, psib.e, uz.e, G.ak, G.nrdim, G.npdim, G.nzdim, c.nrc,
                                                       c.npc, c.nzc, c.nzcu);
  MLG_LAUNCH();
  MLG_TRY(band_T(ur, 0));
  MLG_TRY(band_T(up, 0));
  set_fff0(psib); set_fff0(chib);
  MLG_TRY(lincomb(chib, {{&ur, 1.0}, {&uz, 1.0}}, {{&ur, 1.0}, {&uz, 1.0}}));
  MLG_TRY(lincomb(psib, {{&psib, 1.0}, {&up, 1.0}}, {{&up, 1.0}}));
  return 0;
}

// op_tp2curlvec^T: tp2vec^T, then the first output through (-del2)^T
int tp2curlvec_T(const Scalar& wrb, const Scalar& wpb, const Scalar& wzb, Scalar& psib, Scalar& chib) {
  TMP(md);
  MLG_TRY(tp2vec_T(wrb, wpb, wzb, md, psib));   // tp2vec(md, psi): md is its first argument
  MLG_TRY(lincomb(md, {{&md, -1.0}}, {}, 1.0, false));
  md.off[0] = md.off[1] = md.off[2] = 0;
  MLG_TRY(band_T(md, 2));
  MLG_TRY(assign(chib, md));
  set_fff0(chib);
  return 0;
}

// op_vec2tp^T: (psi_bar, chi_bar) in FFF (with ln) -> (vr_bar, vp_bar, vz_bar) in PPP, overwritten
int vec2tp_T(const Scalar& psib_in, const Scalar& chib_in, Scalar& vrb, Scalar& vpb, Scalar& vzb) {
  TMP(pb); TMP(cb);
  MLG_TRY(assign(pb, psib_in)); MLG_TRY(assign(cb, chib_in));
  set_fff0(pb); set_fff0(cb);
  MLG_TRY(zeroat1_T2(pb, cb));
  MLG_TRY(op_chop2(pb, cb));
  MLG_TRY(idel2_proln_T(cb));
  TMP(ur); TMP(up); TMP(uz);
  MLG_TRY(launch_zero(ur.e)); MLG_TRY(launch_zero(up.e)); MLG_TRY(launch_zero(uz.e));
  {
    int nrc = G.nrchop + 3, npc = G.npchop;
    if (nrc > G.ne || nrc > G.nrdim) return set_error(MLG_ECHOP, "vec2tp: chopping in r too large");
    constexpr int IT = 32, ZT = 16, KC = 16;
    kt_begin(KT_V2TP);
    if (G.precision == MLG_MIXED) {
      // as the forward: m >= 1 in FP32, the m = 0 plane in double-float beside it
      MLG_TRY(side_fork());
      k_m0_vec2tp_T_df<<<cdiv((long long)G.nrh * G.nzdim, 8), 256, 0, G.side>>>(
          pb.e, cb.e, ur.e, up.e, uz.e, G.tD, G.tT, G.ak, G.nr, G.nrh, G.nrdim, G.npdim, G.nzdim,
          std::max(nrc, 0), G.chopzl, G.chopzu);
      MLG_LAUNCH();
      if (npc > 1) {
        dim3 grid(cdiv(G.nzdim, ZT), cdiv(G.nrh, IT), npc - 1);
        k_vec2tp_T<float, IT, ZT, KC><<<grid, IT * ZT / 2, 0, G.stream>>>(pb.e, cb.e, ur.e, up.e, uz.e, G.tV32, G.tD32,
                                                                          G.tT32, G.ak, G.nr, G.nrh, G.ne, G.nrdim,
                                                                          G.npdim, G.nzdim, nrc, G.chopzl, G.chopzu, 1);
        MLG_LAUNCH();
      }
      MLG_TRY(side_join());
    } else {
      dim3 grid(cdiv(G.nzdim, ZT), cdiv(G.nrh, IT), npc);
      k_vec2tp_T<double, IT, ZT, KC><<<grid, IT * ZT / 2, 0, G.stream>>>(pb.e, cb.e, ur.e, up.e, uz.e, G.tV, G.tD, G.tT,
                                                                         G.ak, G.nr, G.nrh, G.ne, G.nrdim, G.npdim,
                                                                         G.nzdim, nrc, G.chopzl, G.chopzu, 0);
      MLG_LAUNCH();
    }
    kt_end(KT_V2TP, 0.0);
  }
  for (Scalar* q : {&ur, &up, &uz}) { q->set_space("PFF"); q->off[0] = q->off[1] = q->off[2] = 0; }
  // psi%ln = -1/2 Re calcat1(up)(k=1), used in up(:nr,1,1) += psi%ln (1 + x) and kept as psi%ln
  MLG_TRY(launch_copy_ln(up.ln, pb.ln));
  k_add_ln_x_T<<<1, 256, 0, G.stream>>>(up.e, G.x, G.nr, up.ln);
  MLG_LAUNCH();
  MLG_TRY(rtrans_bwd_T(up, false));
  up.set_space("FFF");
  {
    ChopIdx c;
    MLG_TRY(chop_index(up, c));
    int nmax = std::min(std::min(G.nrdim, c.nrc), G.nrchop);
    k_calcat_T<<<1, 256, 0, G.stream>>>(up.e, G.at1, nmax, up.ln, -0.5);
    MLG_LAUNCH();
  }
  MLG_TRY(launch_set_ln(up.ln, 0.0));
  // trans^T of up from FFF back to PPP (z, radial, phi steps); u_r (r*vr) and u_z walk back through the
  // z and phi steps only (the PFF adjoint).  The three chains are independent: their z and phi steps run
  // together, each field's own sequence unchanged.
  Scalar* f3[3] = {&up, &ur, &uz};
  MLG_TRY(vfft_checked_T_n(f3, 3, -1));
  MLG_TRY(rtrans_fwd_T_n(f3, 1));
  MLG_TRY(hfft_fwd_T_n(f3, 3));
  up.set_space("PPP");
  MLG_TRY(scale_r(up, 0));
  MLG_TRY(launch_set_ln2(ur.ln, uz.ln, 0.0));
  MLG_TRY(scale_r(ur, 0));
  MLG_TRY(assign(vrb, ur)); MLG_TRY(assign(vpb, up)); MLG_TRY(assign(vzb, uz));
  for (Scalar* q : {&vrb, &vpb, &vzb}) { q->set_space("PPP"); q->off[0] = q->off[1] = q->off[2] = 0; }
  return 0;
}

// the nonlinear term around (psi, chi) (already dealiased, FFF): nl = dealias(vec2tp(v x w)), nl%ln = 0,
// v = tp2vec(psi, chi) + (0, 0, uz), w = tp2curlvec(psi, chi).  (nlpsi_bar, nlchi_bar) -> (psi_bar, chi_bar).
// psi and chi are read only when v and w are not kept (vw_kept null)
int nlcore_T(const Scalar* psi, const Scalar* chi, const Scalar& uzb, const Scalar& nlpb, const Scalar& nlcb, Scalar& psib,
             Scalar& chib, Scalar* const* vw_kept) {
  TMP(np_); TMP(nc_);
  MLG_TRY(assign(np_, nlpb)); MLG_TRY(assign(nc_, nlcb));
  set_fff0(np_); set_fff0(nc_);
  MLG_TRY(op_dealias2(np_, nc_));
  MLG_TRY(launch_set_ln2(np_.ln, nc_.ln, 0.0));
  TMP(obr); TMP(obp); TMP(obz);
  MLG_TRY(vec2tp_T(np_, nc_, obr, obp, obz));
  // the linearisation point: v and w of the forward, kept by the forward step (they are consumed
  // here) or recomputed from (psi, chi)
  TMP(vr_t); TMP(vp_t); TMP(vz_t); TMP(wr_t); TMP(wp_t); TMP(wz_t);
  Scalar* vw[6] = {&vr_t, &vp_t, &vz_t, &wr_t, &wp_t, &wz_t};
  if (vw_kept) for (int i = 0; i < 6; ++i) vw[i] = vw_kept[i];
  Scalar &vr = *vw[0], &vp = *vw[1], &vz = *vw[2], &wr = *vw[3], &wp = *vw[4], &wz = *vw[5];
  if (!vw_kept) {
    if (!psi || !chi) return set_error(MLG_EHANDLE, "adjoint: no linearisation point");
    for (Scalar* q : vw) q->set_space("PPP");
    MLG_TRY(op_tp2vec(*psi, *chi, vr, vp, vz));
    MLG_TRY(op_tp2curlvec(*psi, *chi, wr, wp, wz));
  }
  MLG_TRY(lincomb(vz, {{&vz, 1.0}, {&uzb, 1.0}}, {}, 1.0, false));
  TMP(vbr); TMP(vbp); TMP(vbz); TMP(wbr); TMP(wbp); TMP(wbz);
  k_vecprod_T<<<nblk(G.fsize), 256, 0, G.stream>>>(vbr.e, vbp.e, vbz.e, wbr.e, wbp.e, wbz.e, vr.e, vp.e, vz.e, wr.e, wp.e,
                                                    wz.e, obr.e, obp.e, obz.e, G.nr, G.np / 2, G.nrdim, G.npdim, G.nzdim);
  MLG_LAUNCH();
  {
    double* lns[6];
    int i = 0;
    for (Scalar* q : {&vbr, &vbp, &vbz, &wbr, &wbp, &wbz}) {
      q->set_space("PPP"); q->off[0] = q->off[1] = q->off[2] = 0;
      lns[i++] = q->ln;
    }
    MLG_TRY(launch_set_ln_n(lns, 6, 0.0));
  }
  TMP(pa); TMP(ca);
  MLG_TRY(tp2vec_T(vbr, vbp, vbz, pa, ca));
  MLG_TRY(tp2curlvec_T(wbr, wbp, wbz, psib, chib));
  MLG_TRY(lincomb_n({lin_args(psib, {{&psib, 1.0}, {&pa, 1.0}}, {{&psib, 1.0}, {&pa, 1.0}}),
                     lin_args(chib, {{&chib, 1.0}, {&ca, 1.0}}, {{&chib, 1.0}, {&ca, 1.0}})}));
  return 0;
}

// op_advection_rhs^T (its in-place dealias of psi and chi included): (psi, chi) is the point the
// forward was called at
int advection_T(const Scalar& psi, const Scalar& chi, const Scalar& uzb, const Scalar& nlpb, const Scalar& nlcb, Scalar& psib,
                Scalar& chib) {
  TMP(p3); TMP(c3);
  MLG_TRY(assign(p3, psi)); MLG_TRY(assign(c3, chi));
  MLG_TRY(op_dealias(p3)); MLG_TRY(op_dealias(c3));
  MLG_TRY(nlcore_T(&p3, &c3, uzb, nlpb, nlcb, psib, chib, nullptr));
  MLG_TRY(op_dealias(psib)); MLG_TRY(op_dealias(chib));
  return 0;
}

// abcn^T (hyperpow = 0) of the psi and chi chains of a step: pb and cb hold the adjoints of the new
// psi and chi; on return they hold the adjoints w.r.t. the old ones, and npb, nppb (ncb, ncpb) have
// received the adjoints w.r.t. nl and nl_p (added).  The two transposed Helmholtz solves run in one
// pass; the chains touch disjoint scalars, so each of their linear combinations is paired with the
// other chain's in one launch.
static int abcn_T_pair(Scalar& pb, Scalar& npb, Scalar& nppb, Scalar& cb, Scalar& ncb, Scalar& ncpb, double dt) {
  const double a = -2.0 / (dt * G.P.visc);
  MLG_TRY(ihelm_T_pair(pb, cb, a));
  // the adjoints of nl and nl_p
  MLG_TRY(lincomb_n({lin_args(npb, {{&npb, 1.0}, {&pb, 1.5 * dt * a}}, {{&npb, 1.0}, {&pb, 1.5 * dt * a}}),
                     lin_args(nppb, {{&nppb, 1.0}, {&pb, -0.5 * dt * a}}, {{&nppb, 1.0}, {&pb, -0.5 * dt * a}}),
                     lin_args(ncb, {{&ncb, 1.0}, {&cb, 1.5 * dt * a}}, {{&ncb, 1.0}, {&cb, 1.5 * dt * a}}),
                     lin_args(ncpb, {{&ncpb, 1.0}, {&cb, -0.5 * dt * a}}, {{&ncpb, 1.0}, {&cb, -0.5 * dt * a}})}));
  TMP(tp); TMP(tc);   // t = (visc a dt/2) sb with sb's ln and tags
  for (auto q : {std::make_pair(&tp, &pb), std::make_pair(&tc, &cb)}) {
    std::memcpy(q.first->space, q.second->space, 4);
    for (int i = 0; i < 3; ++i) q.first->off[i] = q.second->off[i];
  }
  MLG_TRY(lincomb_n({lin_args(tp, {{&pb, G.P.visc * a * dt / 2.0}}, {{&pb, 1.0}}),
                     lin_args(tc, {{&cb, G.P.visc * a * dt / 2.0}}, {{&cb, 1.0}})}));
  MLG_TRY(band_T(tp, 2));   // t.e <- del2^T t.e; t.ln <- the log-term adjoint
  MLG_TRY(band_T(tc, 2));
  MLG_TRY(lincomb_n({lin_args(pb, {{&pb, a}, {&tp, 1.0}}, {{&pb, a}, {&tp, 1.0}}),
                     lin_args(cb, {{&cb, a}, {&tc, 1.0}}, {{&cb, a}, {&tc, 1.0}})}));
  return 0;
}

static int adjoint_supported() {
  if (G.P.is_svv) return set_error(MLG_EPARAM, "adjoint: SVV must be off (is_svv = 0): the filter's energy gain is not differentiated");
  if (G.P.hyperpow != 0) return set_error(MLG_EPARAM, "adjoint: hyperviscosity (hyperpow > 0) is not supported");
  if (G.P.visc < 5.0e-14) return set_error(MLG_EINVISCID, "adjoint: inviscid case has no implicit step");
  return 0;
}

// One step backward.  vw = the velocity and vorticity the step's nonlinear term was formed from (kept
// by its forward, consumed here); ad = the adjoint of the state (psi, chi, nlpsi, nlchi, nlpsi_p,
// nlchi_p) at the step's end, replaced by the adjoint of the state at the step's start.
static int step_T(const Scalar& uzb, double dt, Scalar* const ad[6], Scalar* const* vw) {
  Scalar& pb = *ad[0]; Scalar& cb = *ad[1];
  Scalar& npb = *ad[2]; Scalar& ncb = *ad[3];
  Scalar& nppb = *ad[4]; Scalar& ncpb = *ad[5];
  TMP(xp); TMP(xc);
  MLG_TRY(nlcore_T(nullptr, nullptr, uzb, npb, ncb, xp, xc, vw));
  MLG_TRY(lincomb_n({lin_args(pb, {{&pb, 1.0}, {&xp, 1.0}}, {{&pb, 1.0}, {&xp, 1.0}}),
                     lin_args(cb, {{&cb, 1.0}, {&xc, 1.0}}, {{&cb, 1.0}, {&xc, 1.0}})}));
  // the psi and chi chains are independent: each transpose of the pair in one launch
  MLG_TRY(op_dealias2(pb, cb));   // advection_rhs's in-place dealias
  MLG_TRY(zeroat1_T2(pb, cb));
  MLG_TRY(op_dealias2(pb, cb));   // the step's dealias
  // nl_p(out) = nl(in); the new nl(in) and nl_p(in) adjoints come from abcn^T
  MLG_TRY(assign(npb, nppb)); MLG_TRY(assign(ncb, ncpb));
  MLG_TRY(launch_zero(nppb.e)); MLG_TRY(launch_zero(ncpb.e));
  MLG_TRY(launch_set_ln2(nppb.ln, ncpb.ln, 0.0));
  MLG_TRY(abcn_T_pair(pb, npb, nppb, cb, ncb, ncpb, dt));
  for (int i = 0; i < 6; ++i) set_fff0(*ad[i]);
  return 0;
}

// keep (optional): receives the step's velocity and vorticity for step_T
static int forward_step(Scalar* const st[6], const Scalar& uzb, double dt, Scalar* const* keep = nullptr) {
  // psi_p and chi_p of the step are not part of the state: left unwritten
  TMP(pp); TMP(cp);
  pp.set_space("FFF"); cp.set_space("FFF");
  return op_vortex_step_dev(*st[0], *st[1], *st[2], *st[3], pp, cp, *st[4], *st[5], uzb, dt, G.dscal + DS_GAIN0, keep,
                            false);
}

// startup from (psi0, chi0): psi <- dealias(psi0), nl <- advection_rhs, nl_p <- nl
static int startup(const Scalar& psi0, const Scalar& chi0, const Scalar& uzb, Scalar* const st[6]) {
  MLG_TRY(assign(*st[0], psi0)); MLG_TRY(assign(*st[1], chi0));
  for (int i = 2; i < 6; ++i) { MLG_TRY(launch_zero(st[i]->e)); MLG_TRY(launch_set_ln(st[i]->ln, 0.0)); set_fff0(*st[i]); }
  MLG_TRY(op_advection_rhs(*st[0], *st[1], *st[2], *st[3], uzb));
  MLG_TRY(assign(*st[4], *st[2])); MLG_TRY(assign(*st[5], *st[3]));
  return 0;
}

// J and, if seeds are given, (psi_bar, chi_bar) = dJ/d(psi, chi)
// J and its gradient run in FP64 in every form: the volume weights grow like r^2 toward the outer
// collocation points (about 3e5 at 128 points), and the transposed transforms sum them against the
// oscillating top-degree functions with cancellation that FP32 does not resolve.
static int energy(const Scalar& psi, const Scalar& chi, double* J, Scalar* psib, Scalar* chib) {
  PrecisionScope fp64(MLG_PLAIN_FP64);
  TMP(p); TMP(c);
  MLG_TRY(assign(p, psi)); MLG_TRY(assign(c, chi));
  k_drop_mean<<<1, 256, 0, G.stream>>>(p.e, p.ln, G.nrdim); MLG_LAUNCH();
  k_drop_mean<<<1, 256, 0, G.stream>>>(c.e, c.ln, G.nrdim); MLG_LAUNCH();
  TMP(vr); TMP(vp); TMP(vz);
  MLG_TRY(op_tp2vec(p, c, vr, vp, vz));
  double* wq = G.dscal + DS_CALC + 2 * 2048;                  // nr weights
  double* partial = wq + G.nrdim;                               // block sums
  const int NB = 152;
  if ((size_t)(DS_CALC + 2 * 2048 + G.nrdim + NB) > (size_t)DS_COUNT) return set_error(MLG_ESIZE, "adjoint: grid too large");
  double dpz = (2.0 * 3.14159265358979323846 / G.np) * (G.P.zlen / G.nz);
  k_energy_weights<<<1, 256, 0, G.stream>>>(wq, G.x, G.w, G.r, G.nr, dpz); MLG_LAUNCH();
  TMP(ur); TMP(upp); TMP(uzz);
  bool seed = psib && chib;
  k_energy<<<NB, 256, 0, G.stream>>>(seed ? ur.e : nullptr, upp.e, uzz.e, vr.e, vp.e, vz.e, wq, G.nr, G.np / 2, G.nrdim,
                                     G.npdim, G.nzdim, partial);
  MLG_LAUNCH();
  std::vector<double> h(NB);
  MLG_CUDA(cudaMemcpyAsync(h.data(), partial, NB * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
  MLG_CUDA(cudaStreamSynchronize(G.stream));
  double s = 0.0;
  for (double v : h) s += v;
  *J = s;
  if (seed) {
    for (Scalar* q : {&ur, &upp, &uzz}) {
      q->set_space("PPP"); q->off[0] = q->off[1] = q->off[2] = 0;
      MLG_TRY(launch_set_ln(q->ln, 0.0));
    }
    MLG_TRY(tp2vec_T(ur, upp, uzz, *psib, *chib));
    k_drop_mean<<<1, 256, 0, G.stream>>>(psib->e, psib->ln, G.nrdim); MLG_LAUNCH();
    k_drop_mean<<<1, 256, 0, G.stream>>>(chib->e, chib->ln, G.nrdim); MLG_LAUNCH();
  }
  return 0;
}

struct State {
  Tmp t[6];
  Scalar* p[6];
  int rc = 0;
  State() { for (int i = 0; i < 6; ++i) { p[i] = &t[i].s; if (t[i].rc) rc = t[i].rc; } }
};

static int copy_state(Scalar* const d[6], Scalar* const s[6]) {
  for (int i = 0; i < 6; ++i) MLG_TRY(assign(*d[i], *s[i]));
  return 0;
}

// the gradient of J(T) w.r.t. (psi0, chi0) through nsteps steps, the state kept every k_ckpt steps
// The state of the step sequence lives in the active subspace: psi and chi are chopped and dealiased
// at every step boundary (the step ends with dealias, and the start-up's advection_rhs dealiases
// psi0, chi0 in place), nl and nl_p are chopped and dealiased by advection_rhs, and no operator of
// the step writes outside it.  The chopped coefficients are not degrees of freedom, but the step
// does read three of them per column (the vector reconstruction runs with a chop offset of 3), and
// with SVV off their influence grows by orders of magnitude per step.  The gradient is therefore
// the one of J restricted to the active subspace: the adjoint state is projected onto it (chop,
// dealias) at every step boundary, which is the exact transpose of the step restricted to that
// invariant subspace.
static int project_active(Scalar& s) {
  set_fff0(s);
  MLG_TRY(op_chop(s));
  return op_dealias(s);
}
// the same for the six adjoint fields of the state, chop and dealias in one launch
static int project_active6(Scalar* const* ad) {
  for (int i = 0; i < 6; ++i) set_fff0(*ad[i]);
  return op_mask_n(ad, 6, true, true);
}

int adjoint_run(const Scalar& psi0, const Scalar& chi0, const Scalar& uzb, double dt, int nsteps, int k_ckpt, Scalar* gpsi,
                Scalar* gchi, double* J) {
  MLG_TRY(adjoint_supported());
  if (nsteps < 0) return set_error(MLG_EPARAM, "adjoint: nsteps must be >= 0");
  if (k_ckpt < 1) k_ckpt = 1;
  if (!psi0.is("FFF") || !chi0.is("FFF") || !uzb.is("PPP"))
    return set_error(MLG_ESPACE, "adjoint: psi0 and chi0 must be in FFF and uz in PPP");
  std::vector<State*> ck;
  int rc = 0;
  auto cleanup = [&]() { for (State* s : ck) delete s; ck.clear(); };
  State cur;
  if (cur.rc) return cur.rc;
  // forward sweep, keeping the state at steps 0, K, 2K, ...
  rc = startup(psi0, chi0, uzb, cur.p);
  for (int s = 0; s < nsteps && !rc; ++s) {
    if (s % k_ckpt == 0) {
      State* c = new State();
      if (c->rc) { rc = c->rc; delete c; break; }
      ck.push_back(c);
      rc = copy_state(c->p, cur.p);
      if (rc) break;
    }
    rc = forward_step(cur.p, uzb, dt);
  }
  if (rc) { cleanup(); return rc; }
  if (!gpsi || !gchi) {
    rc = energy(*cur.p[0], *cur.p[1], J, nullptr, nullptr);
    cleanup();
    return rc;
  }
  State ad;
  if (ad.rc) { cleanup(); return ad.rc; }
  rc = energy(*cur.p[0], *cur.p[1], J, ad.p[0], ad.p[1]);
  for (int i = 2; i < 6 && !rc; ++i) { rc = launch_zero(ad.p[i]->e); if (!rc) rc = launch_set_ln(ad.p[i]->ln, 0.0); set_fff0(*ad.p[i]); }
  for (int i = 0; i < 2 && !rc; ++i) rc = project_active(*ad.p[i]);
  // backward sweep, segment by segment: recompute the segment's steps from its checkpoint, keeping
  // each step's velocity and vorticity (the linearisation point of its nonlinear term, all that the
  // step back reads of the forward), then step back
  std::vector<State*> segvw;
  for (int c = (int)ck.size() - 1; c >= 0 && !rc; --c) {
    int s0 = c * k_ckpt, s1 = std::min(nsteps, s0 + k_ckpt);
    int len = s1 - s0;
    while ((int)segvw.size() < len) {
      State* v = new State();
      if (v->rc) { rc = v->rc; delete v; break; }
      segvw.push_back(v);
    }
    if (rc) break;
    rc = copy_state(cur.p, ck[c]->p);
    for (int q = 0; q < len && !rc; ++q) rc = forward_step(cur.p, uzb, dt, segvw[q]->p);
    for (int q = len - 1; q >= 0 && !rc; --q) {
      rc = step_T(uzb, dt, ad.p, segvw[q]->p);
      if (!rc) rc = project_active6(ad.p);
    }
  }
  for (State* t : segvw) delete t;
  if (!rc) {
    // through the startup: nl(0) = nl_p(0) = advection_rhs(psi0, chi0)
    TMP(nb); TMP(cb2);
    rc = lincomb(*ad.p[2], {{ad.p[2], 1.0}, {ad.p[4], 1.0}}, {{ad.p[2], 1.0}, {ad.p[4], 1.0}});
    if (!rc) rc = lincomb(*ad.p[3], {{ad.p[3], 1.0}, {ad.p[5], 1.0}}, {{ad.p[3], 1.0}, {ad.p[5], 1.0}});
    if (!rc) rc = advection_T(psi0, chi0, uzb, *ad.p[2], *ad.p[3], nb, cb2);
    if (!rc) rc = lincomb(*gpsi, {{ad.p[0], 1.0}, {&nb, 1.0}}, {{ad.p[0], 1.0}, {&nb, 1.0}});
    if (!rc) rc = lincomb(*gchi, {{ad.p[1], 1.0}, {&cb2, 1.0}}, {{ad.p[1], 1.0}, {&cb2, 1.0}});
    // the startup's psi <- psi0 passes through advection_rhs's in-place dealias; the gradient is
    // the one with respect to the active coefficients
    set_fff0(*gpsi); set_fff0(*gchi);
    if (!rc) rc = project_active(*gpsi);
    if (!rc) rc = project_active(*gchi);
  }
  cleanup();
  return rc;
}

int adjoint_step(Scalar* const st[6], const Scalar& uzb, double dt, Scalar* const ad[6]) {
  MLG_TRY(adjoint_supported());
  State e;
  if (e.rc) return e.rc;
  State vw;
  if (vw.rc) return vw.rc;
  MLG_TRY(copy_state(e.p, st));
  MLG_TRY(forward_step(e.p, uzb, dt, vw.p));
  return step_T(uzb, dt, ad, vw.p);
}

}  // namespace mlg

// =================================================================================================
// C ABI
using namespace mlg;

static int adj_need(void* p) {
  if (!G.kit_set) return set_error(MLG_ENOKIT, "transformation kit is not initialized");
  if (!p || !reinterpret_cast<Scalar*>(p)->e) return set_error(MLG_EHANDLE, "invalid scalar handle");
  return adjoint_supported();
}
#define ADJ_S(h) MLG_TRY(adj_need(h)); Scalar& h##_ = *reinterpret_cast<Scalar*>(h)

extern "C" {

int mlg_adjoint_run(mlg_scalar psi0, mlg_scalar chi0, mlg_scalar uz, double dt, int nsteps, int k_ckpt,
                    mlg_scalar grad_psi, mlg_scalar grad_chi, double* J) {
  ADJ_S(psi0); ADJ_S(chi0); ADJ_S(uz);
  if (!J) return set_error(MLG_EHANDLE, "adjoint: null J");
  Scalar* gp = nullptr;
  Scalar* gc = nullptr;
  if (grad_psi && grad_chi) {
    MLG_TRY(adj_need(grad_psi)); MLG_TRY(adj_need(grad_chi));
    gp = reinterpret_cast<Scalar*>(grad_psi);
    gc = reinterpret_cast<Scalar*>(grad_chi);
  }
  return adjoint_run(psi0_, chi0_, uz_, dt, nsteps, k_ckpt, gp, gc, J);
}

int mlg_adj_vortex_step(const mlg_scalar* state, mlg_scalar uz, double dt, const mlg_scalar* adj) {
  ADJ_S(uz);
  if (!state || !adj) return set_error(MLG_EHANDLE, "invalid scalar handle");
  Scalar* st[6];
  Scalar* ad[6];
  for (int i = 0; i < 6; ++i) {
    MLG_TRY(adj_need(state[i])); MLG_TRY(adj_need(adj[i]));
    st[i] = reinterpret_cast<Scalar*>(state[i]);
    ad[i] = reinterpret_cast<Scalar*>(adj[i]);
    if (!st[i]->is("FFF") || !ad[i]->is("FFF")) return set_error(MLG_ESPACE, "adjoint: the step state must be in FFF");
  }
  return adjoint_step(st, uz_, dt, ad);
}

int mlg_adj_trans(mlg_scalar s, const char* from) { ADJ_S(s); return trans_T(s_, from); }
int mlg_adj_band(mlg_scalar s, int op) {
  ADJ_S(s);
  if (op < 0 || op > 2) return set_error(MLG_EPARAM, "adjoint: band op is 0, 1 or 2");
  return band_T(s_, op);
}
int mlg_adj_ihelm(mlg_scalar s, double alpha) { ADJ_S(s); return ihelm_T(s_, alpha); }
int mlg_adj_idel2_proln(mlg_scalar s) { ADJ_S(s); return idel2_proln_T(s_); }
int mlg_adj_zeroat1(mlg_scalar s) { ADJ_S(s); return zeroat1_T(s_); }
int mlg_adj_tp2vec(mlg_scalar vr, mlg_scalar vp, mlg_scalar vz, mlg_scalar psi, mlg_scalar chi) {
  ADJ_S(vr); ADJ_S(vp); ADJ_S(vz); ADJ_S(psi); ADJ_S(chi);
  return tp2vec_T(vr_, vp_, vz_, psi_, chi_);
}
int mlg_adj_tp2curlvec(mlg_scalar wr, mlg_scalar wp, mlg_scalar wz, mlg_scalar psi, mlg_scalar chi) {
  ADJ_S(wr); ADJ_S(wp); ADJ_S(wz); ADJ_S(psi); ADJ_S(chi);
  return tp2curlvec_T(wr_, wp_, wz_, psi_, chi_);
}
int mlg_adj_vec2tp(mlg_scalar psi, mlg_scalar chi, mlg_scalar vr, mlg_scalar vp, mlg_scalar vz) {
  ADJ_S(psi); ADJ_S(chi); ADJ_S(vr); ADJ_S(vp); ADJ_S(vz);
  return vec2tp_T(psi_, chi_, vr_, vp_, vz_);
}
int mlg_adj_advection(mlg_scalar psi, mlg_scalar chi, mlg_scalar uz, mlg_scalar nlpsi_bar, mlg_scalar nlchi_bar,
                      mlg_scalar psi_bar, mlg_scalar chi_bar) {
  ADJ_S(psi); ADJ_S(chi); ADJ_S(uz); ADJ_S(nlpsi_bar); ADJ_S(nlchi_bar); ADJ_S(psi_bar); ADJ_S(chi_bar);
  return advection_T(psi_, chi_, uz_, nlpsi_bar_, nlchi_bar_, psi_bar_, chi_bar_);
}

}  // extern "C"
