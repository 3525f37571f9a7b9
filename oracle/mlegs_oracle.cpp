// mlegs_oracle.cpp — CPU restatement of the MLegS spectral hot path, used ONLY as test
// infrastructure: the parity checker for the GPU library (tests/, __graft_entry__.smoke) and the
// timed CPU baseline leg of bench.py.  Nothing in the product links or calls this file.
//
// Every routine restates the Fortran reference line by line (file:line cited on each), on one
// process (no MPI: every loc_st is 0 and every loc_sz is the global size, so the reference's
// `exchange` calls are identity maps).  Arithmetic is FP64 as in the reference; the Legendre table
// uses IEEE binary128 (libquadmath __float128 on x86-64, long double on aarch64) where the reference
// uses FM 50-digit arithmetic (mlegs_spectfm_init.f90:254-300, fm_parallel.f90:60).
//
// Third-party arithmetic restated from its published definitions (not vendored code):
//  * FFTE 7.0 conventions: zfft1d forward e^{-2 pi i jk/N} unnormalised, inverse with 1/N
//    (external/ffte-7.0/zfft1d.f:41-84, fft235.f:205-217); dzfft2d real-to-complex unnormalised
//    (dzfft2d.f:96-103 for NY=1); zdfft2d complex-to-real with 1/NX and the last complex slot left
//    untouched (zdfft2d.f:67,119-128).
//  * LAPACK 3.12 zgbtrf/zgbtrs (banded LU with partial pivoting, NRHS=1) — an empty submodule in the
//    reference checkout (external/CMake_build.sh:67); restated from the LAPACK documentation.
//
// Parity of this restatement is pinned against the reference's known answers (tests/golden):
// the two-mode backward transform and its Laplacian (docs/tutorial/transformation.md:209-223,
// operation.md:144-150), the Lamb-Oseen decay (time_integration.md:37-60) and a 50-digit mpmath
// evaluation of the P_L^m table recurrence.

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <map>
#include <mutex>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/mlegs_gb300.h"

#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 qreal;
static inline qreal q_sqrt(qreal a) { return sqrtq(a); }
static inline qreal q_exp(qreal a) { return expq(a); }
#else
typedef long double qreal;  // IEEE binary128 on aarch64
static inline qreal q_sqrt(qreal a) { return sqrtl(a); }
static inline qreal q_exp(qreal a) { return expl(a); }
#endif

typedef std::complex<double> cplx;
static const double PI = 3.14159265358979323846264338327950288;  // acos(-1.D0), mlegs_envir.f90:17

// ------------------------------------------------------------------------------------------------
// error handling: the reference `stop`s; the restatement returns the matching MLG_E* code.
static std::string g_err;
static int fail(int code, const char* msg) {
#pragma omp critical(mlg_oracle_err)
  g_err = msg;
  return code;
}
#define CHECK(x) do { int _rc = (x); if (_rc) return _rc; } while (0)

// ------------------------------------------------------------------------------------------------
// transform kit: type(tfm_kit_3d) (mlegs_spectfm.f90:14-63)
struct Kit {
  bool is_set = false;
  int nr, np, nz, nrchop, npchop, nzchop, hyperpow;
  double ell, zlen, visc, hypervisc;
  int is_svv;
  double svv_cutoff, svv_target, svv_strength, svv_relax;
  int nrdim, npdim, nzdim, chopp, chopzl, chopzu, nrh, ne;
  std::vector<double> x, w, ln, r, p, z, ak, at0, at1;
  std::vector<int> chops, m;
  std::vector<double> lognorm;  // (ne, npchop)
  std::vector<double> pf;       // (nrh, ne, npchop)
  double LN(int n1, int m1) const { return lognorm[(n1 - 1) + (size_t)ne * (m1 - 1)]; }  // 1-based
  double PF(int i1, int n1, int m1) const {
    return pf[(i1 - 1) + (size_t)nrh * ((n1 - 1) + (size_t)ne * (m1 - 1))];
  }
};
static Kit K;

// gauss_legendre (mlegs_spectfm_init.f90:181-214)
static void gauss_legendre(double x1, double x2, std::vector<double>& x, std::vector<double>& w, int n) {
  const double eps = 1.0e-15;
  int m = (int)std::ceil((n + 1) / 2.0);
  double xm = (x2 + x1) / 2.0, xl = (x2 - x1) / 2.0;
  for (int i = 1; i <= m; ++i) {
    double z = std::cos(PI * (i - .25) / (n + .5));
    double z1 = z + 1.0, p1 = 0, p2 = 0, p3 = 0, pp = 0;
    while (std::fabs(z - z1) > eps) {
      p1 = 1.0; p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        p3 = p2; p2 = p1;
        p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      z1 = z;
      z = z1 - p1 / pp;
    }
    x[i - 1] = xm - xl * z;
    x[n - i] = xm + xl * z;
    w[i - 1] = 2 * xl / ((1 - z * z) * pp * pp);
    w[n - i] = w[i - 1];
  }
}

// leg_lognorm (mlegs_spectfm_init.f90:218-250); returns (ndim, size(ms)) column-major
static std::vector<double> leg_lognorm(int ndim, const std::vector<int>& ms) {
  int me = 0;
  for (int v : ms) me = std::max(me, std::abs(v));
  std::vector<double> wk(me + 1);
  wk[0] = std::log(.5);
  for (int m = 1; m <= me; ++m)
    wk[m] = wk[m - 1] + std::log(2.0 * m + 1.0) - std::log(2.0 * m * std::pow(2.0 * m - 1.0, 2));
  std::vector<double> l((size_t)ndim * ms.size());
  for (size_t mm = 0; mm < ms.size(); ++mm) {
    int m = std::abs(ms[mm]);
    l[ndim * mm] = wk[m];
    for (int nn = 2; nn <= ndim; ++nn) {
      int n = m + (nn - 1);
      l[(nn - 1) + ndim * mm] = l[(nn - 2) + ndim * mm] + std::log(2.0 * n + 1.0) - std::log(2.0 * n - 1.0) +
                                std::log(1.0 * (n - m)) - std::log(1.0 * (n + m));
    }
    for (int nn = 1; nn <= ndim; ++nn) l[(nn - 1) + ndim * mm] *= .5;
  }
  return l;
}

// log_fact (mlegs_spectfm_init.f90:351-357)
static double log_fact(int m) { return std::lgamma(2 * m + 1.0) - m * std::log(2.0) - std::lgamma(m + 1.0); }

// leg_tbl (mlegs_spectfm_init.f90:254-300): the scaled three-term recurrence evaluated in
// binary128 (FM 50 digits in the reference), times exp(log_fact(n)+lnrm(nn,mm)), rounded to FP64.
static std::vector<double> leg_tbl(const std::vector<double>& x, int ne, const std::vector<int>& ms,
                                   const std::vector<double>& lnrm, int lnrm_ld) {
  size_t nx = x.size(), me = ms.size();
  std::vector<double> tbl(nx * ne * me, 0.0);
#pragma omp parallel for collapse(2) schedule(dynamic)
  for (long mm = 0; mm < (long)me; ++mm) {
    for (long xx = 0; xx < (long)nx; ++xx) {
      int m = std::abs(ms[mm]);
      std::vector<qreal> f(ne);
      qreal xq = (qreal)x[xx];
      qreal s = q_sqrt((qreal)1 - xq * xq);
      qreal pw = 1;
      for (int k = 0; k < m; ++k) pw *= s;
      f[0] = ((m % 2) ? (qreal)-1 : (qreal)1) * pw;        // (-1)**m * sqrt(1-x^2)**m   (:280)
      if (ne >= 2) f[1] = xq * f[0];                        // (:282)
      for (int nn = 3; nn <= ne; ++nn) {                    // (:283-288)
        int n = m + nn - 1;
        f[nn - 1] = (qreal)1 / (qreal)(n - m) *
                    (f[nn - 2] * xq - f[nn - 3] * (qreal)(n + m - 1) / (qreal)(2 * n - 1) / (qreal)(2 * n - 3));
      }
      for (int nn = 1; nn <= ne; ++nn) {                    // (:289-292)
        int n = m + nn - 1;
        qreal arg = (qreal)log_fact(n) + (qreal)lnrm[(nn - 1) + (size_t)lnrm_ld * mm];
        f[nn - 1] = f[nn - 1] * q_exp(arg);
        tbl[xx + nx * ((nn - 1) + (size_t)ne * mm)] = (double)f[nn - 1];  // to_dp (:293)
      }
    }
  }
  return tbl;
}

static bool factors235(int n) {
  while (n % 2 == 0 || n % 3 == 0 || n % 5 == 0) {
    if (n % 2 == 0) n /= 2;
    if (n % 3 == 0) n /= 3;
    if (n % 5 == 0) n /= 5;
  }
  return n == 1;
}

// tfm_kit_init (mlegs_spectfm_init.f90:6-154), tfm_kit_3d branch (:110-146)
static int kit_init(const mlg_params* P) {
  if (K.is_set) return fail(MLG_ENOKIT, "tfm_kit_init: only one MLegS transformation kit (either 1D, 2D or 3D) is permitted per program");
  Kit k;
  k.nr = P->nr; k.np = P->np; k.nz = P->nz;
  k.nrchop = P->nrchop; k.npchop = P->npchop; k.nzchop = P->nzchop;
  k.ell = P->ell; k.zlen = P->zlen; k.visc = P->visc;
  k.hyperpow = P->hyperpow; k.hypervisc = P->hypervisc; k.is_svv = P->is_svv;
  k.svv_cutoff = P->svv_cutoff; k.svv_target = P->svv_target; k.svv_strength = P->svv_strength;
  k.svv_relax = P->svv_relax;
  int nr = k.nr, np = k.np, nz = k.nz;
  if (!(nr > 0 && nr % 2 == 0)) return fail(MLG_EPARAM, "tfm_kit_init: nr must be even");
  if (!(np > 0 && (np == 1 || np % 2 == 0))) return fail(MLG_EPARAM, "tfm_kit_init: np must be even");
  if (np != 1 && !factors235(np)) return fail(MLG_EPARAM, "tfm_kit_init: np must only have factors of 2, 3 and 5");
  if (!(nz > 0 && (nz == 1 || nz % 2 == 0))) return fail(MLG_EPARAM, "tfm_kit_init: nz must be even");
  if (nz != 1 && !factors235(nz)) return fail(MLG_EPARAM, "tfm_kit_init: nz must only have factors of 2, 3 and 5");
  if (k.nrchop > nr) return fail(MLG_EPARAM, "tfm_kit_init: nrchop must be smaller than or equal to nr");
  if (np != 1 && k.npchop * 2 > np + 2) return fail(MLG_EPARAM, "tfm_kit_init: npchop <= np/2 + 1 must be satisfied");
  if (nz != 1 && k.nzchop * 2 > nz + 2) return fail(MLG_EPARAM, "tfm_kit_init: nzchop <= nz/2 + 1 must be satisfied");
  if (k.nrchop < 1 || k.npchop < 1 || k.nzchop < 1) return fail(MLG_EPARAM, "tfm_kit_init: chops must be positive");
  if (k.hyperpow != 0 && !(k.hyperpow == 4 || k.hyperpow == 6 || k.hyperpow == 8))
    return fail(MLG_EPARAM, "tfm_kit_init: hyperpow must be 0, 4, 6 or 8");

  k.x.resize(nr); k.w.resize(nr);
  gauss_legendre(-1.0, 1.0, k.x, k.w, nr);
  k.ln.resize(nr);
  for (int i = 0; i < nr; ++i) k.ln[i] = -std::log(1.0 - k.x[i]);
  k.r.resize(nr);
  for (int i = 0; i < nr; ++i) k.r[i] = k.ell * std::sqrt((1.0 + k.x[i]) / (1.0 - k.x[i]));
  k.chops.resize(k.npchop);
  for (int i = 0; i < k.npchop; ++i) k.chops[i] = std::max(k.nrchop - i, 0);
  k.nrdim = nr + std::max(3, k.hyperpow);
  k.p.resize(np + 1);
  for (int i = 0; i <= np; ++i) k.p[i] = 2 * PI / np * i;
  k.m.resize(k.npchop);
  for (int i = 0; i < k.npchop; ++i) k.m[i] = i;
  k.npdim = np / 2 + 1;
  k.chopp = k.npchop;
  k.z.resize(nz + 1);
  for (int i = 0; i <= nz; ++i) k.z[i] = k.zlen / nz * i;
  k.ak.resize(nz);
  for (int i = -nz; i <= -1; ++i) k.ak[i + nz] = 2.0 * PI / k.zlen * i;   // (:133)
  for (int i = 0; i <= nz / 2; ++i) k.ak[i] = 2.0 * PI / k.zlen * i;      // (:134)
  k.nzdim = nz;
  k.chopzl = k.nzchop;
  k.chopzu = nz - k.nzchop + 2;
  k.nrh = nr / 2;
  k.ne = k.nrchop + 14;
  k.lognorm = leg_lognorm(k.ne, k.m);
  std::vector<double> xh(k.x.begin(), k.x.begin() + k.nrh);
  k.pf = leg_tbl(xh, k.ne, k.m, k.lognorm, k.ne);
  std::vector<int> m0(1, 0);
  std::vector<double> xa(1, -1.0 + 1.0e-15), xb(1, 1.0 - 1.0e-15);
  k.at0 = leg_tbl(xa, k.nrchop, m0, k.lognorm, k.ne);   // (:147-148)
  k.at1 = leg_tbl(xb, k.nrchop, m0, k.lognorm, k.ne);   // (:149-150)
  k.is_set = true;
  K = std::move(k);
  return 0;
}

// ------------------------------------------------------------------------------------------------
// scalar: type(scalar) (mlegs_scalar.f90:15-49) on one process
struct Scalar {
  std::vector<cplx> e;
  double ln = 0.0;
  int off[3] = {0, 0, 0};
  char space[4] = {'P', 'P', 'P', 0};
  cplx& at(int i1, int j1, int k1) { return e[(i1 - 1) + (size_t)K.nrdim * ((j1 - 1) + (size_t)K.npdim * (k1 - 1))]; }
  const cplx& at(int i1, int j1, int k1) const {
    return e[(i1 - 1) + (size_t)K.nrdim * ((j1 - 1) + (size_t)K.npdim * (k1 - 1))];
  }
  void init() { e.assign((size_t)K.nrdim * K.npdim * K.nzdim, cplx(0, 0)); ln = 0; off[0] = off[1] = off[2] = 0; strcpy(space, "PPP"); }
  bool is(const char* s) const { return strncmp(space, s, 3) == 0; }
};

// chop_index (mlegs_scalar_ops.f90:2012-2063)
struct ChopIdx { int nrc, npc, nzc, nzcu; std::vector<int> nrcs; };
static int chop_index(const Scalar& s, ChopIdx& c) {
  c.nrc = K.chops[0] + s.off[0];
  c.npc = K.chopp + s.off[1];
  c.nzc = K.chopzl + s.off[2];
  c.nzcu = K.chopzu - s.off[2];
  if (c.nrc > K.nrdim) return fail(MLG_ECHOP, "chop_index: chopping in r too large");
  if (c.npc > K.npdim) return fail(MLG_ECHOP, "chop_index: chopping in p too large");
  if (2 * s.off[2] > c.nzcu - c.nzc) return fail(MLG_ECHOP, "chop_index: chopping in z too large");
  if (c.nrc > K.ne) return fail(MLG_ECHOP, "chop_index: chopping in r beyond the table");
  c.nrcs.assign(K.npdim, 0);
  for (int mm = 1; mm <= c.npc; ++mm) c.nrcs[mm - 1] = std::max(std::min(c.nrc, c.nrc - (mm - 1)), 0);
  return 0;
}

// ------------------------------------------------------------------------------------------------
// FFT in FFTE's sign convention: X_k = sum_j x_j exp(-2 pi i jk/N), mixed radix 2/3/5 (DIT)
struct FFTPlan {
  int n;
  std::vector<int> fac;
  std::vector<cplx> tw;  // exp(-2 pi i k / n)
};
static std::map<int, FFTPlan*> g_plans;
static std::mutex g_plan_mu;
static const FFTPlan* get_plan(int n) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto it = g_plans.find(n);
  if (it != g_plans.end()) return it->second;
  FFTPlan* p = new FFTPlan;
  p->n = n;
  int t = n;
  for (int f : {4, 2, 3, 5})
    while (t % f == 0) { p->fac.push_back(f); t /= f; }
  p->tw.resize(n);
  for (int k = 0; k < n; ++k) p->tw[k] = cplx(std::cos(2 * PI * k / n), -std::sin(2 * PI * k / n));
  g_plans[n] = p;
  return p;
}
static void fft_rec(const cplx* x, int stride, cplx* X, int n, const FFTPlan* P, int fi, cplx* tmp) {
  if (n == 1) { X[0] = x[0]; return; }
  int p = P->fac[fi], q = n / p;
  for (int r = 0; r < p; ++r) fft_rec(x + (size_t)r * stride, stride * p, X + (size_t)r * q, q, P, fi + 1, tmp);
  int tws = P->n / n;
  for (int k = 0; k < q; ++k) {
    cplx y[5];
    for (int r = 0; r < p; ++r) y[r] = X[(size_t)r * q + k];
    for (int s = 0; s < p; ++s) {
      cplx acc(0, 0);
      for (int r = 0; r < p; ++r) {
        long e = ((long)r * (k + (long)s * q)) % n;
        acc += y[r] * P->tw[(size_t)e * tws];
      }
      tmp[(size_t)s * q + k] = acc;
    }
  }
  for (int i = 0; i < n; ++i) X[i] = tmp[i];
}
// forward (sign -1) or unnormalised inverse (sign +1)
static void fft(const cplx* x, cplx* X, int n, int sign) {
  const FFTPlan* P = get_plan(n);
  std::vector<cplx> tmp(n), in(x, x + n);
  if (sign > 0) for (auto& v : in) v = std::conj(v);
  fft_rec(in.data(), 1, X, n, P, 0, tmp.data());
  if (sign > 0) for (int i = 0; i < n; ++i) X[i] = std::conj(X[i]);
}

// horizontal_fft_forward (mlegs_scalar_ops.f90:1567-1641) with dzfft2d (NY=1)
static int horizontal_fft_forward(Scalar& s) {
  int npdim = K.npdim, npc = K.chopp + s.off[1];
  if (npc > npdim) return fail(MLG_ECHOP, "horizontal_fft_forward: chopping in p too large");
  int nph = K.np / 2, n = K.np;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ii = 1; ii <= K.nrdim; ++ii)
    for (int kk = 1; kk <= K.nzdim; ++kk) {
      std::vector<cplx> c(n), X(n);
      for (int mm = 1; mm <= nph; ++mm) {
        c[2 * mm - 2] = cplx(s.at(ii, mm, kk).real(), 0);
        c[2 * mm - 1] = cplx(s.at(ii, mm, kk).imag(), 0);
      }
      fft(c.data(), X.data(), n, -1);
      for (int mm = 1; mm <= nph + 1; ++mm) s.at(ii, mm, kk) = X[mm - 1] / (double)(2 * nph);
    }
  return 0;
}

// horizontal_fft_backward (mlegs_scalar_ops.f90:1645-1717) with zdfft2d (NY=1):
// f_j = Re A_0 + 2 sum_{m=1}^{N/2-1} Re(A_m e^{+2pi i jm/N}) + Re(A_{N/2}) (-1)^j, packed in pairs;
// the Nyquist slot keeps its input value (zdfft2d leaves A(NX/2+1) untouched), times np.
static int horizontal_fft_backward(Scalar& s) {
  int npdim = K.npdim, npc = K.chopp + s.off[1];
  if (npc > npdim) return fail(MLG_ECHOP, "horizontal_fft_fbackard: chopping in p too large");
  int nph = K.np / 2, n = K.np;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ii = 1; ii <= K.nrdim; ++ii)
    for (int kk = 1; kk <= K.nzdim; ++kk) {
      std::vector<cplx> C(n), f(n);
      C[0] = cplx(s.at(ii, 1, kk).real(), 0);
      for (int mm = 2; mm <= nph; ++mm) {
        C[mm - 1] = s.at(ii, mm, kk);
        C[n - mm + 1] = std::conj(s.at(ii, mm, kk));
      }
      C[nph] = cplx(s.at(ii, nph + 1, kk).real(), 0);
      fft(C.data(), f.data(), n, +1);
      cplx nyq = s.at(ii, nph + 1, kk);
      for (int mm = 1; mm <= nph; ++mm) s.at(ii, mm, kk) = cplx(f[2 * mm - 2].real(), f[2 * mm - 1].real());
      s.at(ii, nph + 1, kk) = nyq * (double)(2 * nph);
    }
  return 0;
}

// vertical_fft_forward (mlegs_scalar_ops.f90:1721-1783): zfft1d(-1) then /nz
static int vertical_fft_forward(Scalar& s) {
  int nzc = K.chopzl + s.off[2], nzcu = K.chopzu - s.off[2];
  if (2 * s.off[2] > nzcu - nzc) return fail(MLG_ECHOP, "vertical_fft_forward: chopping in z too large");
  int nz = K.nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ii = 1; ii <= K.nrdim; ++ii)
    for (int jj = 1; jj <= K.npdim; ++jj) {
      std::vector<cplx> b(nz), X(nz);
      for (int k = 1; k <= nz; ++k) b[k - 1] = s.at(ii, jj, k);
      fft(b.data(), X.data(), nz, -1);
      for (int k = 1; k <= nz; ++k) s.at(ii, jj, k) = X[k - 1] / (double)nz;
    }
  return 0;
}

// vertical_fft_backward (mlegs_scalar_ops.f90:1787-1848): zfft1d(+1) (which divides by N) then *nz
static int vertical_fft_backward(Scalar& s) {
  int nzc = K.chopzl + s.off[2], nzcu = K.chopzu - s.off[2];
  if (2 * s.off[2] > nzcu - nzc) return fail(MLG_ECHOP, "vertical_fft_backward: chopping in z too large");
  int nz = K.nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int ii = 1; ii <= K.nrdim; ++ii)
    for (int jj = 1; jj <= K.npdim; ++jj) {
      std::vector<cplx> b(nz), X(nz);
      for (int k = 1; k <= nz; ++k) b[k - 1] = s.at(ii, jj, k);
      fft(b.data(), X.data(), nz, +1);
      for (int k = 1; k <= nz; ++k) s.at(ii, jj, k) = X[k - 1];
    }
  return 0;
}

static int rtrans_nrcs(const Scalar& s, int& npc, std::vector<int>& nrcs, const char* who) {
  int nrc = K.chops[0] + s.off[0];
  npc = K.chopp + s.off[1];
  if (nrc > K.nrdim) return fail(MLG_ECHOP, who);
  if (npc > K.npdim) return fail(MLG_ECHOP, who);
  if (nrc > K.ne) return fail(MLG_ECHOP, who);
  nrcs.assign(K.npdim, 0);
  for (int mm = 1; mm <= npc; ++mm) nrcs[mm - 1] = std::max(std::min(nrc, nrc - (mm - 1)), 0);
  return 0;
}

// rtrans_forward (mlegs_scalar_ops.f90:1852-1927)
static int rtrans_forward(Scalar& s) {
  int npc; std::vector<int> nrcs;
  CHECK(rtrans_nrcs(s, npc, nrcs, "rtrans_forward: chopping in r too large"));
  std::vector<cplx> se(s.e.size(), cplx(0, 0));
  int nrh = K.nrh, nr = K.nr, nzd = K.nzdim, nrd = K.nrdim, npd = K.npdim;
#pragma omp parallel for schedule(dynamic)
  for (int mm = 1; mm <= npc; ++mm) {
    std::vector<cplx> be((size_t)nrh * nzd), bo((size_t)nrh * nzd);
    for (int k = 1; k <= nzd; ++k)
      for (int i = 1; i <= nrh; ++i) {
        cplx a = s.at(i, mm, k), b = s.at(nr - i + 1, mm, k);
        be[(i - 1) + (size_t)nrh * (k - 1)] = (a + b) * K.w[i - 1];
        bo[(i - 1) + (size_t)nrh * (k - 1)] = (a - b) * K.w[i - 1];
      }
    int nn = nrcs[mm - 1];
    for (int k = 1; k <= nzd; ++k)
      for (int j = 1; j <= nn; ++j) {
        const std::vector<cplx>& bb = (j % 2 == 1) ? be : bo;
        cplx acc(0, 0);
        for (int i = 1; i <= nrh; ++i) acc += K.PF(i, j, mm) * bb[(i - 1) + (size_t)nrh * (k - 1)];
        se[(j - 1) + (size_t)nrd * ((mm - 1) + (size_t)npd * (k - 1))] = acc;
      }
  }
  s.e.swap(se);
  return 0;
}

// rtrans_backward (mlegs_scalar_ops.f90:1931-2008)
static int rtrans_backward(Scalar& s) {
  int npc; std::vector<int> nrcs;
  CHECK(rtrans_nrcs(s, npc, nrcs, "rtrans_backward: chopping in r too large"));
  std::vector<cplx> se(s.e.size(), cplx(0, 0));
  int nrh = K.nrh, nr = K.nr, nzd = K.nzdim, nrd = K.nrdim, npd = K.npdim;
#pragma omp parallel for schedule(dynamic)
  for (int mm = 1; mm <= npc; ++mm) {
    int nn = nrcs[mm - 1];
    for (int k = 1; k <= nzd; ++k)
      for (int i = 1; i <= nrh; ++i) {
        cplx be(0, 0), bo(0, 0);
        for (int j = 1; j <= nn; j += 2) be += K.PF(i, j, mm) * s.at(j, mm, k);
        for (int j = 2; j <= nn; j += 2) bo += K.PF(i, j, mm) * s.at(j, mm, k);
        se[(i - 1) + (size_t)nrd * ((mm - 1) + (size_t)npd * (k - 1))] = be + bo;
        se[(nr - i) + (size_t)nrd * ((mm - 1) + (size_t)npd * (k - 1))] = be - bo;
      }
  }
  s.e.swap(se);
  return 0;
}

static int space_code(const char* sp) {
  if (!strncmp(sp, "PPP", 3)) return 0;
  if (!strncmp(sp, "PFP", 3)) return 1;
  if (!strncmp(sp, "FFP", 3)) return 2;
  if (!strncmp(sp, "FFF", 3)) return 3;
  return -1;
}

// trans (mlegs_scalar_ops.f90:157-235)
static int trans(Scalar& s, const char* space) {
  int cur = space_code(s.space);
  if (cur < 0) return fail(MLG_ESPACE, "trans: scalar space info corrupted (only accepting PPP, PFP, FFP and FFF)");
  int nw = space_code(space);
  if (nw < 0) return fail(MLG_ESPACE, "trans: only taking PPP, PFP, FFP and FFF for spectral transformation");
  if (cur < nw) {
    while (true) {
      if (cur == 0) { if (K.np > 1) CHECK(horizontal_fft_forward(s)); strcpy(s.space, "PFP"); }
      if (cur == 1) {
        for (int kk = 1; kk <= K.nzdim; ++kk)
          for (int i = 1; i <= K.nr; ++i) s.at(i, 1, kk) -= s.ln * K.ln[i - 1];   // (:193-195)
        CHECK(rtrans_forward(s));
        strcpy(s.space, "FFP");
      }
      if (cur == 2) { if (K.nz > 1) CHECK(vertical_fft_forward(s)); strcpy(s.space, "FFF"); }
      if (cur == 3) break;
      cur++;
      if (cur == nw) break;
    }
  }
  if (cur > nw) {
    while (true) {
      if (cur == 3) { if (K.nz > 1) CHECK(vertical_fft_backward(s)); strcpy(s.space, "FFP"); }
      if (cur == 2) {
        CHECK(rtrans_backward(s));
        for (int kk = 1; kk <= K.nzdim; ++kk)
          for (int i = 1; i <= K.nr; ++i) s.at(i, 1, kk) += s.ln * K.ln[i - 1];   // (:219-221)
        strcpy(s.space, "PFP");
      }
      if (cur == 1) { if (K.np > 1) CHECK(horizontal_fft_backward(s)); strcpy(s.space, "PPP"); }
      if (cur == 0) break;
      cur--;
      if (cur == nw) break;
    }
  }
  return 0;
}

// chop (mlegs_scalar_ops.f90:6-41)
static int chop(Scalar& s) {
  ChopIdx c; CHECK(chop_index(s, c));
  if (s.space[0] == 'F')
    for (int mm = 1; mm <= K.npdim; ++mm) {
      int rc = c.nrcs[mm - 1] + 1;
      for (int kk = 1; kk <= K.nzdim; ++kk)
        for (int i = std::max(rc, 1); i <= K.nrdim; ++i) s.at(i, mm, kk) = 0;
    }
  if (s.space[1] == 'F')
    for (int mm = c.npc + 1; mm <= K.npdim; ++mm)
      for (int kk = 1; kk <= K.nzdim; ++kk)
        for (int i = 1; i <= K.nrdim; ++i) s.at(i, mm, kk) = 0;
  if (s.space[2] == 'F' && c.nzc < c.nzcu)
    for (int kk = c.nzc + 1; kk <= c.nzcu - 1; ++kk)
      for (int mm = 1; mm <= K.npdim; ++mm)
        for (int i = 1; i <= K.nrdim; ++i) s.at(i, mm, kk) = 0;
  return 0;
}

// dealias (mlegs_scalar_ops.f90:43-70)
static int dealias(Scalar& s) {
  if (K.np > 1 && s.space[1] == 'F') {
    int pcut = std::max(K.np / 3 + 1, 1);
    for (int mm = pcut + 1; mm <= K.npdim; ++mm)
      for (int kk = 1; kk <= K.nzdim; ++kk)
        for (int i = 1; i <= K.nrdim; ++i) s.at(i, mm, kk) = 0;
  }
  if (K.nz > 1 && s.space[2] == 'F') {
    int zcut = std::max(K.nz / 3 + 1, 1), zupper = K.nz - zcut + 2;
    for (int kk = 1; kk <= K.nzdim; ++kk)
      if (kk > zcut && kk < zupper)
        for (int mm = 1; mm <= K.npdim; ++mm)
          for (int i = 1; i <= K.nrdim; ++i) s.at(i, mm, kk) = 0;
  }
  return 0;
}

// svv_filter (mlegs_scalar_ops.f90:72-155)
static int svv_filter(Scalar& s, double& gain) {
  if (!K.is_svv) return 0;
  if (!s.is("FFF")) return fail(MLG_ESPACE, "svv_filter: scalar must be in FFF space");
  double total = 0, tail = 0;
  for (auto& v : s.e) { double a = std::abs(v); total += a * a; }
  double cutoff = std::min(std::max(K.svv_cutoff, 0.0), 0.99);
  double target = std::max(K.svv_target, 1.0e-12);
  double kmax = 0;
  for (double a : K.ak) kmax = std::max(kmax, std::fabs(a));
  kmax = std::max(kmax, 1.0);
  auto qval = [&](int i, int j, int k) {
    int gn = i - 1, gm = j - 1, gk = k;
    double q_r = std::min(1.0, (double)std::max(gn, 0) / std::max((double)(K.nrchop - 1), 1.0));
    double q_p = std::min(1.0, (double)std::abs(gm) / std::max((double)(K.np / 2), 1.0));
    double kv = (gk >= 1 && gk <= (int)K.ak.size()) ? std::fabs(K.ak[gk - 1]) : 0.0;
    double q_z = std::min(1.0, kv / kmax);
    return std::min(1.0, std::max(q_r, std::max(q_p, q_z)));
  };
  for (int i = 1; i <= K.nrdim; ++i)
    for (int j = 1; j <= K.npdim; ++j)
      for (int k = 1; k <= K.nzdim; ++k)
        if (qval(i, j, k) >= cutoff) { double a = std::abs(s.at(i, j, k)); tail += a * a; }
  if (total <= 2.2250738585072014e-308) return 0;   // tiny(1.D0)
  double tail_ratio = tail / total;
  double feedback = std::min(std::max(tail_ratio / target - 1.0, 0.0), 1.0);
  double rl = std::min(std::max(K.svv_relax, 0.0), 1.0);
  gain = (1.0 - rl) * gain + rl * feedback;
  double strength = std::min(std::max(K.svv_strength, 0.0) * gain, 1.0);
  if (strength <= 0.0) return 0;
  for (int i = 1; i <= K.nrdim; ++i)
    for (int j = 1; j <= K.npdim; ++j)
      for (int k = 1; k <= K.nzdim; ++k) {
        double q = qval(i, j, k);
        if (q > cutoff) {
          double shape = (q - cutoff) / (1.0 - cutoff);
          double factor = std::exp(-strength * std::pow(shape, 8));
          s.at(i, j, k) *= factor;
        }
      }
  return 0;
}

// calcat0 / calcat1 (mlegs_scalar_ops.f90:237-309)
static int calcat(const Scalar& s, std::vector<cplx>& calc, const std::vector<double>& atv) {
  ChopIdx c; CHECK(chop_index(s, c));
  Scalar st = s;
  CHECK(trans(st, "FFF"));
  calc.assign(K.nz, cplx(0, 0));
  int nmax = std::min(std::min(K.nrdim, c.nrc), (int)atv.size());
  for (int k = 1; k <= K.nz; ++k) {
    cplx acc(0, 0);
    for (int n = 1; n <= nmax; ++n) acc += st.at(n, 1, k) * atv[n - 1];
    calc[k - 1] = acc;
  }
  return 0;
}

// zeroat1 (mlegs_scalar_ops.f90:311-325)
static int zeroat1(Scalar& s) {
  if (!s.is("FFF")) CHECK(trans(s, "FFF"));
  std::vector<cplx> a1;
  CHECK(calcat(s, a1, K.at1));
  for (int k = 1; k <= K.nzdim; ++k) s.at(1, 1, k) -= a1[k - 1] / K.at1[0];
  return 0;
}

// ------------------------------------------------------------------------------------------------
// banded matrices: LAPACK band layout as type(real_bndm) (mlegs_bndmat.f90:8-16,
// mlegs_bndmat_cvrt.f90:46-68): A(i,j) stored at e(suplen+1+i-j, j), here 0-based.
struct Band {
  int n = 0, kl = 0, ku = 0;
  std::vector<double> a;   // (kl+ku+1) x n
  double get(int i, int j) const {  // 1-based, 0 outside band
    if (i < 1 || j < 1 || i > n || j > n || i - j > kl || j - i > ku) return 0.0;
    return a[(ku + i - j) + (size_t)(kl + ku + 1) * (j - 1)];
  }
  void set(int i, int j, double v) { a[(ku + i - j) + (size_t)(kl + ku + 1) * (j - 1)] = v; }
  void alloc(int n_, int kl_, int ku_) { n = n_; kl = kl_; ku = ku_; a.assign((size_t)(kl + ku + 1) * n, 0.0); }
};
static Band from_dense(const std::vector<double>& g, int n, int kl, int ku) {  // bandmatr (:46-68)
  Band b; b.alloc(n, kl, ku);
  for (int j = 1; j <= n; ++j)
    for (int i = std::max(1, j - ku); i <= std::min(n, j + kl); ++i) b.set(i, j, g[(i - 1) + (size_t)n * (j - 1)]);
  return b;
}
static std::vector<double> to_dense(const Band& b) {  // fullmatr (:6-24)
  std::vector<double> g((size_t)b.n * b.n, 0.0);
  for (int j = 1; j <= b.n; ++j)
    for (int i = std::max(1, j - b.ku); i <= std::min(b.n, j + b.kl); ++i) g[(i - 1) + (size_t)b.n * (j - 1)] = b.get(i, j);
  return g;
}

// leg_xxdx (mlegs_spectfm_diff.f90:6-43)
static Band leg_xxdx(int mval, int nin, int nout) {
  int am = std::abs(mval);
  std::vector<double> g((size_t)nin * nout, 0.0);
  auto G = [&](int i, int j) -> double& { return g[(i - 1) + (size_t)nin * (j - 1)]; };
  for (int nn = 1; nn <= nin; ++nn) {
    double n = am + (nn - 1);
    if (nn - 1 >= 1) G(nn, nn - 1) = -(n - 1.0) * (n - am) / (2.0 * n - 1.0);
    if (nn + 1 <= nout) G(nn, nn + 1) = (n + 2.0) * (n + am + 1.0) / (2.0 * n + 3.0);
  }
  for (int i = 1; i <= nin; ++i)
    for (int j = 1; j <= nout; ++j) G(i, j) = G(i, j) * std::exp(K.LN(j, am + 1) - K.LN(i, am + 1));
  return from_dense(g, nin, 1, 1);
}

// leg_del2h / leg_del2 (mlegs_spectfm_diff.f90:45-152); akval = 0 gives del2h
static Band leg_del2(int mval, double akval, int nin, int nout, bool with_k) {
  int am = std::abs(mval);
  double ell2 = std::pow(K.ell, 2.0), s = 0.0;
  std::vector<double> g((size_t)nin * nout, 0.0);
  auto G = [&](int i, int j) -> double& { return g[(i - 1) + (size_t)nin * (j - 1)]; };
  for (int nn = 1; nn <= nin; ++nn) {
    double n = am + (nn - 1);
    if (nn - 2 >= 1) G(nn, nn - 2) = -(n - am - 1.0) * (n - am) * (n - 2.0 + s) * (n - 1.0 + s) / (2.0 * n - 3.0) / (2.0 * n - 1.0);
    if (nn - 1 >= 1) G(nn, nn - 1) = 2.0 * n * (n - am) * (n - 1.0 + s) / (2.0 * n - 1.0);
    if (nn <= nout)
      G(nn, nn) = (-2.0 * n * (n + 1.0) * (3.0 * n * n + 3.0 * n - am * am - 2.0) + 2.0 * s * (s - 2.0) * (n * n + n + am * am - 1.0)) /
                  (2.0 * n - 1.0) / (2.0 * n + 3.0);
    if (nn + 1 <= nout) G(nn, nn + 1) = 2.0 * (n + 1.0) * (n + am + 1.0) * (n + 2.0 - s) / (2.0 * n + 3.0);
    if (nn + 2 <= nout)
      G(nn, nn + 2) = -(n + am + 1.0) * (n + am + 2.0) * (n + 3.0 - s) * (n + 2.0 - s) / (2.0 * n + 3.0) / (2.0 * n + 5.0);
  }
  for (auto& v : g) v = v / ell2;
  if (with_k)
    for (int nn = 1; nn <= nin; ++nn)
      if (nn <= nout) G(nn, nn) = G(nn, nn) - std::pow(akval, 2.0);
  for (int i = 1; i <= nin; ++i)
    for (int j = 1; j <= nout; ++j) G(i, j) = G(i, j) * std::exp(K.LN(j, am + 1) - K.LN(i, am + 1));
  return from_dense(g, nin, 2, 2);
}

// band x complex vector: mulrbc1 (mlegs_bndmat_ops.f90:123-133): y = A x
static void band_mulvec(const Band& A, cplx* x) {
  std::vector<cplx> y(A.n);
  for (int i = 1; i <= A.n; ++i) {
    cplx acc(0, 0);
    for (int j = std::max(1, i - A.kl); j <= std::min(A.n, i + A.ku); ++j) acc += A.get(i, j) * x[j - 1];
    y[i - 1] = acc;
  }
  for (int i = 0; i < A.n; ++i) x[i] = y[i];
}
static void band_mulvec_real(const Band& A, double* x) {
  std::vector<double> y(A.n);
  for (int i = 1; i <= A.n; ++i) {
    double acc = 0;
    for (int j = std::max(1, i - A.kl); j <= std::min(A.n, i + A.ku); ++j) acc += A.get(i, j) * x[j - 1];
    y[i - 1] = acc;
  }
  for (int i = 0; i < A.n; ++i) x[i] = y[i];
}
// band x band: mulrbrb (mlegs_bndmat_ops.f90:251-318), C = A B of two n x n band matrices
static Band band_mul(const Band& A, const Band& B) {
  Band C; C.alloc(A.n, A.kl + B.kl, A.ku + B.ku);
  for (int i = 1; i <= A.n; ++i)
    for (int j = std::max(1, i - C.kl); j <= std::min(A.n, i + C.ku); ++j) {
      double acc = 0;
      for (int k = std::max(1, std::max(i - A.kl, j - B.ku)); k <= std::min(A.n, std::min(i + A.ku, j + B.kl)); ++k)
        acc += A.get(i, k) * B.get(k, j);
      C.set(i, j, acc);
    }
  return C;
}

// lsolve(band, x): lurb/lucb + zgbtrs (mlegs_bndmat_ops.f90:369-457); LAPACK gbtrf/gbtrs semantics:
// partial pivoting over rows j..j+kl, multipliers by the reciprocal pivot, U of bandwidth kl+ku.
static int band_lsolve(const Band& A, cplx* b) {
  int n = A.n, kl = A.kl, ku = A.ku, W = 2 * kl + ku + 1;
  std::vector<double> U((size_t)n * W, 0.0);          // row i covers columns i-kl .. i+kl+ku
  auto at = [&](int i, int j) -> double& { return U[(size_t)(i - 1) * W + (j - i + kl)]; };
  for (int i = 1; i <= n; ++i)
    for (int j = std::max(1, i - kl); j <= std::min(n, i + ku); ++j) at(i, j) = A.get(i, j);
  for (int j = 1; j <= n; ++j) {
    int km = std::min(kl, n - j), p = j;
    double best = std::fabs(at(j, j));
    for (int i = j + 1; i <= j + km; ++i)
      if (std::fabs(at(i, j)) > best) { best = std::fabs(at(i, j)); p = i; }
    if (at(p, j) == 0.0) return fail(MLG_ESINGULAR, "lurc: lu factorization resulted in failure");
    int ju = std::min(n, j + kl + ku);
    if (p != j) {
      for (int c = j; c <= ju; ++c) std::swap(at(p, c), at(j, c));
      std::swap(b[p - 1], b[j - 1]);
    }
    double rp = 1.0 / at(j, j);
    for (int i = j + 1; i <= j + km; ++i) {
      double l = at(i, j) * rp;
      at(i, j) = l;
      for (int c = j + 1; c <= ju; ++c) at(i, c) -= l * at(j, c);
      b[i - 1] -= l * b[j - 1];
    }
  }
  for (int j = n; j >= 1; --j) {
    b[j - 1] = b[j - 1] / at(j, j);
    cplx t = b[j - 1];
    for (int i = j - 1; i >= std::max(1, j - kl - ku); --i) b[i - 1] -= t * at(i, j);
  }
  return 0;
}

// column vector helpers on (:nn, mm, kk)
static void get_col(const Scalar& s, int mm, int kk, int nn, std::vector<cplx>& v) {
  v.resize(nn);
  for (int i = 1; i <= nn; ++i) v[i - 1] = s.at(i, mm, kk);
}
static void put_col(Scalar& s, int mm, int kk, int nn, const std::vector<cplx>& v) {
  for (int i = 1; i <= nn; ++i) s.at(i, mm, kk) = v[i - 1];
}
// per-(m,k) loops over kk = 1..nzc and kk = nzcu..nzdim (the Nyquist slot twice when nzc == nzcu),
// as in every banded operator of mlegs_scalar_ops.f90 (e.g. :546-557).  The m columns are independent
// and run on the host threads; each m keeps the reference's k order (so a slot visited twice is still
// updated twice in sequence).  f(mm, kk, v) gets a per-thread work vector and returns a status; the
// first nonzero status in m order is returned, after every column ran.
template <class F>
static int for_each_mk(const ChopIdx& c, F f) {
  std::vector<int> st(std::max(c.npc, 0), 0);
#pragma omp parallel
  {
    std::vector<cplx> v;
#pragma omp for schedule(dynamic)
    for (int mm = 1; mm <= c.npc; ++mm) {
      int rc = 0;
      for (int kk = 1; kk <= std::min(K.nzdim, c.nzc) && !rc; ++kk) rc = f(mm, kk, v);
      for (int kk = std::max(c.nzcu, 1); kk <= K.nzdim && !rc; ++kk) rc = f(mm, kk, v);
      st[mm - 1] = rc;
    }
  }
  for (int r : st)
    if (r) return r;
  return 0;
}

static int require_fff(Scalar& s) {
  if (!s.is("FFF")) CHECK(trans(s, "FFF"));
  return 0;
}

// delsqp (mlegs_scalar_ops.f90:327-366)
static int delsqp(Scalar& s) {
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  Scalar so = s;
  so.ln = 0;
  for (int mm = 1; mm <= c.npc; ++mm)
    for (int nn = 1; nn <= c.nrcs[mm - 1]; ++nn) {
      double n = (mm - 1) + nn - 1;
      for (int kk = 1; kk <= K.nzdim; ++kk) so.at(nn, mm, kk) = -s.at(nn, mm, kk) * n * (n + 1.0) / std::pow(K.ell, 2.0);
    }
  so.at(1, 1, 1) = s.ln / std::pow(K.ell, 2.0) / std::exp(K.LN(1, 1));
  s = so;
  return 0;
}

// idelsqp (mlegs_scalar_ops.f90:368-416)
static int idelsqp(Scalar& s) {
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  Scalar so = s;
  so.ln = s.at(1, 1, 1).real() * std::pow(K.ell, 2.0) * std::exp(K.LN(1, 1));
  for (int mm = 1; mm <= c.npc; ++mm)
    for (int nn = 1; nn <= c.nrcs[mm - 1]; ++nn) {
      int n = (mm - 1) + nn - 1;
      for (int kk = 1; kk <= K.nzdim; ++kk)
        so.at(nn, mm, kk) = (n == 0) ? cplx(0, 0) : -s.at(nn, mm, kk) / (double)n / (n + 1.0) * std::pow(K.ell, 2.0);
    }
  for (int kk = 1; kk <= K.nzdim; ++kk) so.at(1, 1, kk) = 0;
  s = so;
  return 0;
}

// xxdx (mlegs_scalar_ops.f90:418-463)
static int xxdx(Scalar& s) {
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  Scalar so = s;
  so.ln = 0;
  for_each_mk(c, [&](int mm, int kk, std::vector<cplx>& v) {
    int nn = c.nrcs[mm - 1];
    if (nn < 1) return 0;
    Band B = leg_xxdx(mm - 1, nn, nn);
    get_col(so, mm, kk, nn, v); band_mulvec(B, v.data()); put_col(so, mm, kk, nn, v);
    return 0;
  });
  so.at(1, 1, 1) += 1.0 / std::exp(K.LN(1, 1)) * s.ln;
  so.at(2, 1, 1) += 1.0 / std::exp(K.LN(2, 1)) * s.ln;
  s = so;
  return 0;
}

static void ln_del2_terms(Scalar& so, double lnv, double sign) {
  double e2 = std::pow(K.ell, 2.0);
  so.at(1, 1, 1) += sign * (4.0 / 3.0 / e2 / std::exp(K.LN(1, 1)) * lnv);
  so.at(2, 1, 1) -= sign * (2.0 / 1.0 / e2 / std::exp(K.LN(2, 1)) * lnv);
  so.at(3, 1, 1) += sign * (2.0 / 3.0 / e2 / std::exp(K.LN(3, 1)) * lnv);
}

// del2h (mlegs_scalar_ops.f90:465-518) and del2 (:520-573)
static int del2_generic(Scalar& s, bool with_k) {
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  Scalar so = s;
  so.ln = 0;
  for_each_mk(c, [&](int mm, int kk, std::vector<cplx>& v) {
    int nn = c.nrcs[mm - 1];
    if (nn < 1) return 0;
    Band D = leg_del2(mm - 1, K.ak[kk - 1], nn, nn, with_k);
    get_col(so, mm, kk, nn, v); band_mulvec(D, v.data()); put_col(so, mm, kk, nn, v);
    return 0;
  });
  ln_del2_terms(so, s.ln, 1.0);
  s = so;
  return 0;
}
static int del2h(Scalar& s) { return del2_generic(s, false); }
static int del2(Scalar& s) { return del2_generic(s, true); }

// idel2_preln (mlegs_scalar_ops.f90:575-669) and idel2_proln (:671-760)
static int idel2(Scalar& s, bool pre, double preln) {
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  Scalar so = s;
  double e2 = std::pow(K.ell, 2.0);
  std::vector<int> st(std::max(c.npc, 0), 0);
  // the m columns are independent: one host thread per column, the reference's k order within it
#pragma omp parallel for schedule(dynamic)
  for (int mm = 1; mm <= c.npc; ++mm) {
    int nn = c.nrcs[mm - 1];
    if (nn < 1) continue;
    std::vector<cplx> v;
    int rc = 0;
    for (int kk = 1; kk <= std::min(K.nzdim, c.nzc) && !rc; ++kk) {
      if (mm == 1 && kk == 1) {
        Band D0 = leg_del2(0, K.ak[0], nn, nn, true);
        std::vector<double> g = to_dense(D0);
        auto G = [&](int i, int j) -> double& { return g[(i - 1) + (size_t)nn * (j - 1)]; };
        if (pre) {
          for (int j = 1; j <= nn; ++j) {
            for (int i = nn; i >= 2; --i) G(i, j) = G(i - 1, j);   // del2_pre(2:nn,:) = del2_pre(1:nn-1,:)
            G(1, j) = 0.0;
          }
          G(1, 1) = 1.0;
          if (nn >= 2) G(2, 1) = G(2, 1) + 4.0 / 3.0 / e2;
          if (nn >= 3) G(3, 1) = G(3, 1) - 2.0 / 1.0 / e2 * std::exp(K.LN(1, 1) - K.LN(2, 1));
          if (nn >= 4) G(4, 1) = G(4, 1) + 2.0 / 3.0 / e2 * std::exp(K.LN(1, 1) - K.LN(3, 1));
          Band Bm = from_dense(g, nn, 3, 2);
          get_col(so, mm, kk, nn, v);
          for (int i = nn; i >= 2; --i) v[i - 1] = v[i - 2];
          v[0] = preln / std::exp(K.LN(1, 1));
          rc = band_lsolve(Bm, v.data());
          put_col(so, mm, kk, nn, v);
        } else {
          G(1, 1) = G(1, 1) + 4.0 / 3.0 / e2;
          if (nn >= 2) G(2, 1) = G(2, 1) - 2.0 / 1.0 / e2 * std::exp(K.LN(1, 1) - K.LN(2, 1));
          if (nn >= 3) G(3, 1) = G(3, 1) + 2.0 / 3.0 / e2 * std::exp(K.LN(1, 1) - K.LN(3, 1));
          Band Bm = from_dense(g, nn, 2, 2);
          get_col(so, mm, kk, nn, v);
          rc = band_lsolve(Bm, v.data());
          put_col(so, mm, kk, nn, v);
        }
        so.ln = so.at(1, mm, kk).real() * std::exp(K.LN(1, 1));
      } else {
        Band D = leg_del2(mm - 1, K.ak[kk - 1], nn, nn, true);
        get_col(so, mm, kk, nn, v); rc = band_lsolve(D, v.data()); put_col(so, mm, kk, nn, v);
      }
    }
    for (int kk = std::max(c.nzcu, 1); kk <= K.nzdim && !rc; ++kk) {
      Band D = leg_del2(mm - 1, K.ak[kk - 1], nn, nn, true);
      get_col(so, mm, kk, nn, v); rc = band_lsolve(D, v.data()); put_col(so, mm, kk, nn, v);
    }
    st[mm - 1] = rc;
  }
  for (int r : st)
    if (r) return r;
  s = so;
  return 0;
}

// helm (mlegs_scalar_ops.f90:762-789): the reference computes del2(s)+alpha*s into a temporary and
// returns without assigning it back, so s leaves the call unchanged.
static int helm(Scalar& s, double alpha) {
  (void)alpha;
  CHECK(require_fff(s));
  return 0;
}

// ihelm (mlegs_scalar_ops.f90:791-854)
static int ihelm(Scalar& s, double alpha) {
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  if (std::fabs(alpha) < 5.0e-14) return fail(MLG_EALPHA, "ihelm: alpha equals to zero. Inversion of 0*identity is impossible");
  Scalar so = s;
  so.ln = s.ln / alpha;
  ln_del2_terms(so, so.ln, -1.0);
  int rc = for_each_mk(c, [&](int mm, int kk, std::vector<cplx>& v) {
    int nn = c.nrcs[mm - 1];
    if (nn < 1) return 0;
    Band H = leg_del2(mm - 1, K.ak[kk - 1], nn, nn, true);
    for (int j = 1; j <= nn; ++j) H.set(j, j, H.get(j, j) + alpha);
    get_col(so, mm, kk, nn, v);
    int r = band_lsolve(H, v.data());
    put_col(so, mm, kk, nn, v);
    return r;
  });
  if (rc) return rc;
  s = so;
  return 0;
}

// helmp (mlegs_scalar_ops.f90:856-903)
static int helmp(Scalar& s, int power, double alpha, double beta) {
  if (!(power % 2 == 0 && power >= 4)) return fail(MLG_EPOWER, "helmp: even power greater than or equal to 4");
  if (power > 8) return fail(MLG_EPOWER, "helmp: power must be less than or equal to 8 (supported power = 4, 6 or 8)");
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  Scalar so = s, s2 = s;
  CHECK(del2(s2));
  Scalar sp = s2;
  for (int n = 1; n <= power / 2 - 1; ++n) CHECK(del2(sp));
  for (size_t i = 0; i < so.e.size(); ++i) so.e[i] = sp.e[i] + beta * s2.e[i] + alpha * s.e[i];
  so.ln = alpha * s.ln;
  s = so;
  return 0;
}

// ihelmp (mlegs_scalar_ops.f90:905-1000)
static int ihelmp(Scalar& s, int power, double alpha, double beta) {
  if (!(power % 2 == 0 && power >= 4)) return fail(MLG_EPOWER, "ihelmp: even power greater than or equal to 4");
  if (power > 8) return fail(MLG_EPOWER, "ihelmp: power must be less than or equal to 8 (supported power = 4, 6 or 8)");
  ChopIdx c; CHECK(chop_index(s, c));
  CHECK(require_fff(s));
  if (std::fabs(alpha) < 5.0e-14) return fail(MLG_EALPHA, "ihelmp: alpha equals to zero. Inversion of 0*identity is impossible");
  Scalar so = s;
  so.ln = s.ln / alpha;
  double e2 = std::pow(K.ell, 2.0);
  int nrc = c.nrc;
  std::vector<double> bl(nrc, 0.0), bl2(nrc, 0.0);
  bl2[0] = 4.0 / 3.0 / e2 / std::exp(K.LN(1, 1)) * so.ln;
  if (nrc > 1) bl2[1] = -2.0 / e2 / std::exp(K.LN(2, 1)) * so.ln;
  if (nrc > 2) bl2[2] = 2.0 / 3.0 / e2 / std::exp(K.LN(3, 1)) * so.ln;
  bl = bl2;
  {
    Band D = leg_del2(0, K.ak[0], nrc, nrc, true);
    for (int n = 1; n <= power / 2 - 1; ++n) band_mulvec_real(D, bl.data());
    for (int i = 1; i <= nrc; ++i) so.at(i, 1, 1) -= bl[i - 1] + beta * bl2[i - 1];
  }
  int rc = for_each_mk(c, [&](int mm, int kk, std::vector<cplx>& v) {
    int nn = c.nrcs[mm - 1];
    if (nn < 1) return 0;
    Band D = leg_del2(mm - 1, K.ak[kk - 1], nn, nn, true);
    Band Hp = D;
    for (int n = 1; n <= power / 2 - 1; ++n) Hp = band_mul(D, Hp);
    std::vector<double> w = to_dense(Hp), d = to_dense(D);
    for (size_t i = 0; i < w.size(); ++i) w[i] += beta * d[i];
    Band H = from_dense(w, nn, power, power);
    for (int j = 1; j <= nn; ++j) H.set(j, j, H.get(j, j) + alpha);
    get_col(so, mm, kk, nn, v);
    int r = band_lsolve(H, v.data());
    put_col(so, mm, kk, nn, v);
    return r;
  });
  if (rc) return rc;
  s = so;
  return 0;
}

// smooth (mlegs_scalar_ops.f90:2149-2175)
static std::vector<cplx> smooth(const std::vector<cplx>& a) {
  int ni = (int)a.size();
  std::vector<cplx> as(ni, cplx(0, 0));
  const double fae[3] = {.2, .3, .5};
  as[0] = a[0];
  for (int t = 0; t < 3; ++t) as[ni - 3 + t] += a[ni - 1] * fae[t];
  for (int i = 2; i <= ni - 1; ++i) {
    double f = (1.0 + (ni - i) / (ni - 1.0)) * 0.5;
    as[i - 2] += a[i - 1] * ((1.0 - f) / 2.0);
    as[i - 1] += a[i - 1] * f;
    as[i] += a[i - 1] * ((1.0 - f) / 2.0);
  }
  return as;
}

// fftreat (mlegs_scalar_ops.f90:1002-1063)
static int fftreat(Scalar& s) {
  ChopIdx c; CHECK(chop_index(s, c));
  int nr = K.nr, ns = nr * 3 / 4, ns0 = std::min(ns + 4, nr);
  if (nr - ns + 1 < 3) return fail(MLG_EPARAM, "smooth: the input length must be longer than or equal to 3.");
  Scalar so = s;
  double lnv = s.ln;
  so.ln = 0;
  CHECK(delsqp(so));
  CHECK(rtrans_backward(so));
  auto active_k = [&](int kk) { return kk <= c.nzc || kk >= c.nzcu; };
  for (int mm = 1; mm <= c.npc; ++mm)
    for (int kk = 1; kk <= K.nzdim; ++kk)
      if (active_k(kk))
        for (int i = 1; i <= nr; ++i) so.at(i, mm, kk) *= std::pow(1.0 - K.x[i - 1], 2.0);
  for (int mm = 2; mm <= c.npc; ++mm)
    for (int kk = 1; kk <= K.nzdim; ++kk)
      for (int i = ns0; i <= K.nrdim; ++i) so.at(i, mm, kk) = 0;
  for (int mm = 1; mm <= c.npc; ++mm)
    for (int kk = 1; kk <= K.nzdim; ++kk)
      if (active_k(kk)) {
        std::vector<cplx> a(K.nrdim - ns + 1);
        for (int i = ns; i <= K.nrdim; ++i) a[i - ns] = so.at(i, mm, kk);
        for (int t = 0; t < 5; ++t) a = smooth(a);
        for (int i = ns; i <= K.nrdim; ++i) so.at(i, mm, kk) = a[i - ns];
      }
  for (int mm = 1; mm <= c.npc; ++mm)
    for (int kk = 1; kk <= K.nzdim; ++kk)
      if (active_k(kk))
        for (int i = 1; i <= nr; ++i) so.at(i, mm, kk) /= std::pow(1.0 - K.x[i - 1], 2.0);
  strcpy(so.space, "FFF");
  CHECK(rtrans_forward(so));
  CHECK(idelsqp(so));
  so.ln = lnv;
  CHECK(zeroat1(so));
  s = so;
  return 0;
}

// ------------------------------------------------------------------------------------------------
// time steppers (mlegs_scalar_ops.f90:1065-1262)
static double hsign() { return (double)(((K.hyperpow / 2 + 1) % 2 == 0) ? 1 : -1); }  // (-1)**(hyperpow/2+1)

static int lterm(Scalar& svis) {   // svis <- visc*del2(svis) or the hyperviscous operator
  if (K.hyperpow == 0) {
    if (K.visc < 5.0e-14) { for (auto& v : svis.e) v = 0; }
    else { CHECK(del2(svis)); for (auto& v : svis.e) v *= K.visc; }
  } else {
    double hv = K.hypervisc * hsign();
    CHECK(helmp(svis, K.hyperpow, 0.0, K.visc / hv));
    for (auto& v : svis.e) v *= hv;
  }
  return 0;
}

static int fefe(Scalar& s, const Scalar& nl, double dt) {
  if (!s.is("FFF") || !nl.is("FFF")) return fail(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  Scalar svis = s;
  CHECK(lterm(svis));
  for (size_t i = 0; i < s.e.size(); ++i) s.e[i] = s.e[i] + dt * (nl.e[i] + svis.e[i]);
  s.ln = s.ln + dt * (nl.ln + svis.ln);
  return 0;
}

static int abab(Scalar& s, Scalar& s_p, Scalar& nl, Scalar& nl_p, double dt, bool is2nd) {
  if (!s.is("FFF") || !nl.is("FFF") || !s_p.is("FFF") || !nl_p.is("FFF"))
    return fail(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  Scalar svis = s;
  CHECK(lterm(svis));
  Scalar svis_p = s_p;
  if (!is2nd) {
    if (K.hyperpow == 0) {
      if (K.visc < 5.0e-14) { for (auto& v : svis.e) v = 0; }   // (:1135) zeroes svis, not svis_p
      else { CHECK(del2(svis_p)); for (auto& v : svis_p.e) v *= K.visc; }
    } else {
      double hv = K.hypervisc * hsign();
      CHECK(helmp(svis_p, K.hyperpow, 0.0, K.visc / hv));
      for (auto& v : svis_p.e) v *= hv;
    }
  }
  for (size_t i = 0; i < s.e.size(); ++i)
    s.e[i] = s.e[i] + dt * (1.5 * (nl.e[i] + svis.e[i]) - .5 * (nl_p.e[i] + svis_p.e[i]));
  s.ln = s.ln + dt * (1.5 * (nl.ln + svis.ln) - .5 * (nl_p.ln + svis_p.ln));
  s_p = s;
  nl_p = nl;
  return 0;
}

static int febe(Scalar& s, const Scalar& nl, double dt) {
  if (!s.is("FFF") || !nl.is("FFF")) return fail(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  Scalar sh = s;
  for (size_t i = 0; i < s.e.size(); ++i) sh.e[i] = s.e[i] + dt * nl.e[i];
  sh.ln = s.ln + dt * nl.ln;
  if (K.hyperpow == 0) {
    if (K.visc < 5.0e-14) return fail(MLG_EINVISCID, "febe: inviscid case and no linear term in rhs. semi-implicit time adv is impossible");
    double a = -1.0 / (dt * K.visc);
    sh.ln = a * sh.ln;
    for (auto& v : sh.e) v = a * v;
    CHECK(ihelm(sh, a));
    s = sh;
  } else {
    double hv = K.hypervisc * hsign();
    double a = -1.0 / (dt * hv), b = K.visc / hv;
    sh.ln = a * sh.ln;
    for (auto& v : sh.e) v = a * v;
    CHECK(ihelmp(sh, K.hyperpow, a, b));
    s = sh;
  }
  return 0;
}

static int abcn(Scalar& s, Scalar& s_p, Scalar& nl, Scalar& nl_p, double dt) {
  if (!s.is("FFF") || !nl.is("FFF") || !s_p.is("FFF") || !nl_p.is("FFF"))
    return fail(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  Scalar sh = s;
  for (size_t i = 0; i < s.e.size(); ++i) sh.e[i] = s.e[i] + dt * (1.5 * nl.e[i] - .5 * nl_p.e[i]);
  sh.ln = s.ln + dt * (1.5 * nl.ln - .5 * nl_p.ln);
  Scalar svis = s;
  CHECK(lterm(svis));
  if (K.hyperpow == 0) {
    if (K.visc < 5.0e-14) return fail(MLG_EINVISCID, "abcn: inviscid case and no linear term in rhs. semi-implicit time adv is impossible");
    double a = -2.0 / (dt * K.visc);
    sh.ln = a * (sh.ln + dt / 2.0 * svis.ln);
    for (size_t i = 0; i < sh.e.size(); ++i) sh.e[i] = a * (sh.e[i] + dt / 2.0 * svis.e[i]);
    CHECK(ihelm(sh, a));
    s = sh;
  } else {
    double hv = K.hypervisc * hsign();
    double a = -2.0 / (dt * hv), b = K.visc / hv;
    sh.ln = a * (sh.ln + dt / 2.0 * svis.ln);
    for (size_t i = 0; i < sh.e.size(); ++i) sh.e[i] = a * (sh.e[i] + dt / 2.0 * svis.e[i]);
    CHECK(ihelmp(sh, K.hyperpow, a, b));
    s = sh;
  }
  s_p = s;
  nl_p = nl;
  return 0;
}

// ------------------------------------------------------------------------------------------------
// vector fields (mlegs_scalar_ops.f90:1264-1560)
static int vecprod(Scalar& vr, Scalar& vp, Scalar& vz, const Scalar& ur, const Scalar& up, const Scalar& uz) {
  for (const Scalar* q : {(const Scalar*)&vr, (const Scalar*)&vp, (const Scalar*)&vz, &ur, &up, &uz})
    if (!q->is("PPP")) return fail(MLG_ESPACE, "vector_product: to compute v x u, all inputs must be in PPP");
  Scalar a, b, c;
  a.init(); b.init(); c.init();
  for (int kk = 1; kk <= K.nz; ++kk)
    for (int mm = 1; mm <= K.np / 2; ++mm)
      for (int nn = 1; nn <= K.nr; ++nn) {
        double a1 = vr.at(nn, mm, kk).real(), a2 = vp.at(nn, mm, kk).real(), a3 = vz.at(nn, mm, kk).real();
        double b1 = ur.at(nn, mm, kk).real(), b2 = up.at(nn, mm, kk).real(), b3 = uz.at(nn, mm, kk).real();
        double c1 = vr.at(nn, mm, kk).imag(), c2 = vp.at(nn, mm, kk).imag(), c3 = vz.at(nn, mm, kk).imag();
        double d1 = ur.at(nn, mm, kk).imag(), d2 = up.at(nn, mm, kk).imag(), d3 = uz.at(nn, mm, kk).imag();
        a.at(nn, mm, kk) = cplx(a2 * b3 - a3 * b2, c2 * d3 - c3 * d2);
        b.at(nn, mm, kk) = cplx(a3 * b1 - a1 * b3, c3 * d1 - c1 * d3);
        c.at(nn, mm, kk) = cplx(a1 * b2 - a2 * b1, c1 * d2 - c2 * d1);
      }
  vr = a; vp = b; vz = c;
  return 0;
}

// eomul / oemul (mlegs_scalar_ops.f90:2067-2145); A is (ni, nj/2) column-major, b has nj entries
static void eoemul(const std::vector<double>& A, int lda, int ni, int njh, const cplx* b, cplx* c, bool eo) {
  std::vector<cplx> be(njh), bo(njh);
  int nj = 2 * njh;
  for (int i = 0; i < njh; ++i) { be[i] = b[i] + b[nj - 1 - i]; bo[i] = b[i] - b[nj - 1 - i]; }
  for (int i = 1; i <= ni; ++i) {
    const std::vector<cplx>& src = ((i % 2 == 1) == eo) ? be : bo;
    cplx acc(0, 0);
    for (int j = 0; j < njh; ++j) acc += A[(i - 1) + (size_t)lda * j] * src[j];
    c[i - 1] = acc;
  }
}

static int vec2tp(const Scalar& vr, const Scalar& vp, const Scalar& vz, Scalar& psi, Scalar& chi) {
  if (!vr.is("PPP") || !vp.is("PPP") || !vz.is("PPP")) return fail(MLG_ESPACE, "vector_projection: vr must be in PPP");
  if (!psi.is("FFF")) return fail(MLG_ESPACE, "vector_projection: psi must be in FFF");
  if (!chi.is("FFF")) return fail(MLG_ESPACE, "vector_projection: chi must be in FFF");
  int nr = K.nr, nrh = K.nrh;
  for (auto& v : psi.e) v = 0;
  for (auto& v : chi.e) v = 0;
  psi.ln = 0; chi.ln = 0;
  Scalar ur = vr, up = vp, uz = vz;
  for (int mm = 1; mm <= K.npdim; ++mm)
    for (int kk = 1; kk <= K.nzdim; ++kk)
      for (int i = 1; i <= nr; ++i) { ur.at(i, mm, kk) *= K.r[i - 1]; up.at(i, mm, kk) *= K.r[i - 1]; }
  CHECK(trans(ur, "PFP"));
  if (K.nz > 1) CHECK(vertical_fft_forward(ur));
  strcpy(ur.space, "PFF");
  CHECK(trans(up, "FFF"));
  std::vector<cplx> inf;
  CHECK(calcat(up, inf, K.at1));
  psi.ln = -1.0 / 2.0 * inf[0].real();
  CHECK(rtrans_backward(up));
  strcpy(up.space, "PFF");
  for (int i = 1; i <= nr; ++i) up.at(i, 1, 1) += psi.ln * (1.0 + K.x[i - 1]);
  CHECK(trans(uz, "PFP"));
  if (K.nz > 1) CHECK(vertical_fft_forward(uz));
  strcpy(uz.space, "PFF");
  ur.off[0] = 3; up.off[0] = 3; uz.off[0] = 3;
  ur.off[1] = ur.off[2] = up.off[1] = up.off[2] = uz.off[1] = uz.off[2] = 0;
  ChopIdx c; CHECK(chop_index(ur, c));
  int nrc = c.nrc;
  std::vector<double> fff(nrh);
  for (int i = 0; i < nrh; ++i) fff[i] = (1.0 - std::pow(K.x[i], 2.0)) / K.w[i];
  int rc = 0;
#pragma omp parallel for schedule(dynamic)
  for (int mm = 1; mm <= c.npc; ++mm) {
    int nn = c.nrcs[mm - 1], mv = mm - 1;
    if (nn < 1) continue;
    std::vector<double> v((size_t)nrc * nrh, 0.0), d((size_t)nrc * nrh, 0.0), t((size_t)nrc * nrh, 0.0);
    std::vector<double> pfd((size_t)nrh * (nn + 1), 0.0);
    Band X = leg_xxdx(mv, nn + 1, nn + 1);
    for (int x = 1; x <= nrh; ++x)       // pfd = pf(:nrh, :nn+1, m) .mul. leg_xxdx(mv, nn+1, nn+1)  (:1405)
      for (int j = 1; j <= nn + 1; ++j) {
        double acc = 0;
        for (int i = std::max(1, j - X.ku); i <= std::min(nn + 1, j + X.kl); ++i) acc += K.PF(x, i, mm) * X.get(i, j);
        pfd[(x - 1) + (size_t)nrh * (j - 1)] = acc;
      }
    for (int i = 1; i <= nn; ++i) {      // (:1406-1411)
      int n = std::max(1, mv + i - 1);
      for (int x = 1; x <= nrh; ++x) {
        v[(i - 1) + (size_t)nrc * (x - 1)] = K.PF(x, i, mm) / n / (n + 1) / fff[x - 1];
        d[(i - 1) + (size_t)nrc * (x - 1)] = pfd[(x - 1) + (size_t)nrh * (i - 1)] / n / (n + 1) / fff[x - 1];
        t[(i - 1) + (size_t)nrc * (x - 1)] = K.PF(x, i, mm) * K.w[x - 1];
      }
    }
    std::vector<cplx> w1(nrc), w2(nrc), col(nr), colp(nr), colz(nr), chv(nn);
    auto body = [&](int kk) {
      for (int i = 1; i <= nr; ++i) { col[i - 1] = ur.at(i, mm, kk); colp[i - 1] = up.at(i, mm, kk); colz[i - 1] = uz.at(i, mm, kk); }
      std::fill(w1.begin(), w1.end(), cplx(0, 0)); std::fill(w2.begin(), w2.end(), cplx(0, 0));
      if (mv != 0) eoemul(v, nrc, nn, nrh, col.data(), w1.data(), true);
      eoemul(d, nrc, nn, nrh, colp.data(), w2.data(), false);
      for (int i = 1; i <= nn; ++i) psi.at(i, mm, kk) = -cplx(0, 1) * (double)mv * w1[i - 1] - w2[i - 1];
      std::fill(w1.begin(), w1.end(), cplx(0, 0)); std::fill(w2.begin(), w2.end(), cplx(0, 0));
      eoemul(d, nrc, nn, nrh, col.data(), w1.data(), false);
      if (mv != 0) eoemul(v, nrc, nn, nrh, colp.data(), w2.data(), true);
      eoemul(t, nrc, nn, nrh, colz.data(), chv.data(), true);
      double kv = K.ak[kk - 1];
      for (int i = 1; i <= nn; ++i) chi.at(i, mm, kk) = cplx(0, 1) * kv * w1[i - 1] + (double)mv * kv * w2[i - 1] - chv[i - 1];
    };
    for (int kk = 1; kk <= std::min(K.nzdim, c.nzc); ++kk) body(kk);
    for (int kk = std::max(c.nzcu, 1); kk <= K.nzdim; ++kk) body(kk);
  }
  if (rc) return rc;
  CHECK(idel2(chi, false, 0.0));
  psi.off[0] = psi.off[1] = psi.off[2] = 0;
  chi.off[0] = chi.off[1] = chi.off[2] = 0;
  CHECK(chop(psi)); CHECK(chop(chi));
  CHECK(zeroat1(psi)); CHECK(zeroat1(chi));
  return 0;
}

static int tp2vec(const Scalar& psi, const Scalar& chi, Scalar& vr, Scalar& vp, Scalar& vz) {
  if (!psi.is("FFF") || !chi.is("FFF")) return fail(MLG_ESPACE, "vector_projection: psi must be in FFF");
  if (!vr.is("PPP") || !vp.is("PPP") || !vz.is("PPP")) return fail(MLG_ESPACE, "vector_projection: vr must be in PPP");
  Scalar ur = chi, up = psi, uz = chi;
  ur.off[0] = 3; ur.off[1] = ur.off[2] = 0;
  up.off[0] = 3; up.off[1] = up.off[2] = 0;
  uz.off[0] = 3; uz.off[1] = uz.off[2] = 0;
  ChopIdx c; CHECK(chop_index(ur, c));
  CHECK(xxdx(ur));
  CHECK(xxdx(up));
  for (int mm = 1; mm <= c.npc; ++mm) {
    int nn = c.nrcs[mm - 1], mv = mm - 1;
    for (int kk = 1; kk <= K.nzdim; ++kk)
      if (kk <= c.nzc || kk >= c.nzcu) {
        double kv = K.ak[kk - 1];
        for (int i = 1; i <= std::min(K.nrdim, nn); ++i) {
          ur.at(i, mm, kk) = cplx(0, 1) * (double)mv * psi.at(i, mm, kk) + cplx(0, 1) * kv * ur.at(i, mm, kk);
          up.at(i, mm, kk) = -up.at(i, mm, kk) - (double)mv * kv * uz.at(i, mm, kk);
        }
      }
  }
  ur.off[0] = 0; up.off[0] = 0;
  CHECK(chop(ur)); CHECK(chop(up));
  CHECK(trans(ur, "PPP")); CHECK(trans(up, "PPP"));
  for (int mm = 1; mm <= K.npdim; ++mm)
    for (int kk = 1; kk <= K.nzdim; ++kk)
      for (int i = 1; i <= K.nr; ++i) { ur.at(i, mm, kk) /= K.r[i - 1]; up.at(i, mm, kk) /= K.r[i - 1]; }
  CHECK(del2h(uz));
  for (auto& v : uz.e) v = -v;
  uz.off[0] = 0;
  CHECK(chop(uz));
  CHECK(trans(uz, "PPP"));
  vr = ur; vp = up; vz = uz;
  return 0;
}

static int tp2curlvec(const Scalar& psi, const Scalar& chi, Scalar& wr, Scalar& wp, Scalar& wz) {
  Scalar md = chi;
  strcpy(md.space, "FFF");
  CHECK(del2(md));
  for (auto& v : md.e) v = -v;
  return tp2vec(md, psi, wr, wp, wz);
}

// advection_rhs (vortical_flow_3d.f90:353-395)
static int advection_rhs(Scalar& psi, Scalar& chi, Scalar& nlpsi, Scalar& nlchi, const Scalar& uz) {
  if (!psi.is("FFF") || !chi.is("FFF") || !nlpsi.is("FFF") || !nlchi.is("FFF") || !uz.is("PPP"))
    return fail(MLG_ESPACE, "advection_rhs: space mismatch");
  CHECK(dealias(psi)); CHECK(dealias(chi));
  Scalar vr, vp, vz, wr, wp, wz;
  vr.init(); vp.init(); vz.init(); wr.init(); wp.init(); wz.init();
  CHECK(tp2vec(psi, chi, vr, vp, vz));
  for (size_t i = 0; i < vz.e.size(); ++i) vz.e[i] += uz.e[i];
  CHECK(tp2curlvec(psi, chi, wr, wp, wz));
  CHECK(vecprod(vr, vp, vz, wr, wp, wz));
  CHECK(vec2tp(vr, vp, vz, nlpsi, nlchi));
  nlpsi.ln = 0; nlchi.ln = 0;
  CHECK(dealias(nlpsi)); CHECK(dealias(nlchi));
  return 0;
}

static bool all_finite(const Scalar& s) {
  for (auto& v : s.e) if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return false;
  return true;
}

// main-loop step (vortical_flow_3d.f90:168-180)
static int vortex_step(Scalar& psi, Scalar& chi, Scalar& nlpsi, Scalar& nlchi, Scalar& psip, Scalar& chip,
                       Scalar& nlpsip, Scalar& nlchip, const Scalar& uz, double dt, double* gains) {
  for (Scalar* q : {&psi, &chi, &nlpsi, &nlchi, &psip, &chip, &nlpsip, &nlchip}) CHECK(trans(*q, "FFF"));
  CHECK(abcn(psi, psip, nlpsi, nlpsip, dt));
  CHECK(abcn(chi, chip, nlchi, nlchip, dt));
  CHECK(dealias(psi)); CHECK(dealias(chi));
  CHECK(svv_filter(psi, gains[0])); CHECK(svv_filter(chi, gains[1]));
  CHECK(zeroat1(psi)); CHECK(zeroat1(chi));
  CHECK(advection_rhs(psi, chi, nlpsi, nlchi, uz));
  if (!all_finite(psi) || !all_finite(chi)) return fail(MLG_ENONFINITE, "ERROR: non-finite vortex state");
  return 0;
}

// ================================================================================================
// C ABI of the oracle (handle-based, mirroring include/mlegs_gb300.h)
static std::vector<Scalar*> g_sc;
static Scalar* H(int h) { return (h >= 0 && h < (int)g_sc.size()) ? g_sc[h] : nullptr; }
#define HS(name, h) Scalar* name = H(h); if (!name) return fail(MLG_EHANDLE, "oracle: bad handle")
#define NEED_KIT if (!K.is_set) return fail(MLG_ENOKIT, "oracle: kit not initialised")

extern "C" {
const char* orc_last_error(void) { return g_err.c_str(); }
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
int orc_init(const mlg_params* p) { return kit_init(p); }
int orc_finalize(void) {
  for (auto* s : g_sc) delete s;
  g_sc.clear();
  K = Kit();
  return 0;
}
int orc_kit_dims(int* d) {
  NEED_KIT;
  d[0] = K.nrdim; d[1] = K.npdim; d[2] = K.nzdim; d[3] = K.chopzl; d[4] = K.chopzu; d[5] = K.nrh; d[6] = K.ne;
  d[7] = K.npchop; d[8] = K.nr;
  return 0;
}
int orc_kit_get(const char* name, double* out, long long count) {
  NEED_KIT;
  const std::vector<double>* v = nullptr;
  std::string n(name);
  if (n == "x") v = &K.x; else if (n == "w") v = &K.w; else if (n == "r") v = &K.r; else if (n == "ln") v = &K.ln;
  else if (n == "ak") v = &K.ak; else if (n == "lognorm") v = &K.lognorm; else if (n == "pf") v = &K.pf;
  else if (n == "at0") v = &K.at0; else if (n == "at1") v = &K.at1;
  if (!v) return fail(MLG_EHANDLE, "oracle: unknown kit array");
  if (count < (long long)v->size()) return fail(MLG_ESIZE, "oracle: output too small");
  std::memcpy(out, v->data(), v->size() * sizeof(double));
  return 0;
}
int orc_new(void) {
  if (!K.is_set) { fail(MLG_ENOKIT, "oracle: kit not initialised"); return -1; }
  Scalar* s = new Scalar; s->init();
  for (size_t i = 0; i < g_sc.size(); ++i) if (!g_sc[i]) { g_sc[i] = s; return (int)i; }
  g_sc.push_back(s);
  return (int)g_sc.size() - 1;
}
int orc_free(int h) { HS(s, h); delete s; g_sc[h] = nullptr; return 0; }
int orc_set(int h, const double* e, double ln, const char* space, const int* offs) {
  HS(s, h);
  std::memcpy(s->e.data(), e, s->e.size() * sizeof(cplx));
  s->ln = ln;
  std::memcpy(s->space, space, 3); s->space[3] = 0;
  if (offs) for (int i = 0; i < 3; ++i) s->off[i] = offs[i];
  return 0;
}
int orc_get(int h, double* e, double* ln, char* space4, int* offs) {
  HS(s, h);
  if (e) std::memcpy(e, s->e.data(), s->e.size() * sizeof(cplx));
  if (ln) *ln = s->ln;
  if (space4) { std::memcpy(space4, s->space, 3); space4[3] = 0; }
  if (offs) for (int i = 0; i < 3; ++i) offs[i] = s->off[i];
  return 0;
}
int orc_copy(int dst, int src) { HS(d, dst); HS(s, src); *d = *s; return 0; }
int orc_axpby(int d, double a, int x, double b, int y) {
  HS(D, d); HS(X, x);
  Scalar* Y = (y >= 0) ? H(y) : nullptr;
  std::vector<cplx> out(D->e.size());
  for (size_t i = 0; i < out.size(); ++i) out[i] = a * X->e[i] + (Y ? b * Y->e[i] : cplx(0, 0));
  D->e.swap(out);
  return 0;
}
int orc_chop_offset(int h, int a, int b, int c) { HS(s, h); s->off[0] = a; s->off[1] = b; s->off[2] = c; return 0; }
int orc_trans(int h, const char* sp) { NEED_KIT; HS(s, h); return trans(*s, sp); }
int orc_chop(int h) { NEED_KIT; HS(s, h); return chop(*s); }
int orc_dealias(int h) { NEED_KIT; HS(s, h); return dealias(*s); }
int orc_svv_filter(int h, double* gain) { NEED_KIT; HS(s, h); return svv_filter(*s, *gain); }
int orc_calcat0(int h, double* out) {
  NEED_KIT; HS(s, h); std::vector<cplx> c; CHECK(calcat(*s, c, K.at0));
  std::memcpy(out, c.data(), c.size() * sizeof(cplx)); return 0;
}
int orc_calcat1(int h, double* out) {
  NEED_KIT; HS(s, h); std::vector<cplx> c; CHECK(calcat(*s, c, K.at1));
  std::memcpy(out, c.data(), c.size() * sizeof(cplx)); return 0;
}
int orc_zeroat1(int h) { NEED_KIT; HS(s, h); return zeroat1(*s); }
int orc_delsqp(int h) { NEED_KIT; HS(s, h); return delsqp(*s); }
int orc_idelsqp(int h) { NEED_KIT; HS(s, h); return idelsqp(*s); }
int orc_xxdx(int h) { NEED_KIT; HS(s, h); return xxdx(*s); }
int orc_del2h(int h) { NEED_KIT; HS(s, h); return del2h(*s); }
int orc_del2(int h) { NEED_KIT; HS(s, h); return del2(*s); }
int orc_idel2_preln(int h, double preln) { NEED_KIT; HS(s, h); return idel2(*s, true, preln); }
int orc_idel2_proln(int h) { NEED_KIT; HS(s, h); return idel2(*s, false, 0.0); }
int orc_helm(int h, double a) { NEED_KIT; HS(s, h); return helm(*s, a); }
int orc_ihelm(int h, double a) { NEED_KIT; HS(s, h); return ihelm(*s, a); }
int orc_helmp(int h, int p, double a, double b) { NEED_KIT; HS(s, h); return helmp(*s, p, a, b); }
int orc_ihelmp(int h, int p, double a, double b) { NEED_KIT; HS(s, h); return ihelmp(*s, p, a, b); }
int orc_fftreat(int h) { NEED_KIT; HS(s, h); return fftreat(*s); }
int orc_fefe(int h, int nl, double dt) { NEED_KIT; HS(s, h); HS(n, nl); return fefe(*s, *n, dt); }
int orc_abab(int h, int hp, int nl, int nlp, double dt, int is2nd) {
  NEED_KIT; HS(s, h); HS(sp, hp); HS(n, nl); HS(np_, nlp); return abab(*s, *sp, *n, *np_, dt, is2nd != 0);
}
int orc_febe(int h, int nl, double dt) { NEED_KIT; HS(s, h); HS(n, nl); return febe(*s, *n, dt); }
int orc_abcn(int h, int hp, int nl, int nlp, double dt) {
  NEED_KIT; HS(s, h); HS(sp, hp); HS(n, nl); HS(np_, nlp); return abcn(*s, *sp, *n, *np_, dt);
}
int orc_vecprod(int a, int b, int c, int d, int e, int f) {
  NEED_KIT; HS(vr, a); HS(vp, b); HS(vz, c); HS(ur, d); HS(up, e); HS(uz, f);
  return vecprod(*vr, *vp, *vz, *ur, *up, *uz);
}
int orc_vec2tp(int a, int b, int c, int d, int e) {
  NEED_KIT; HS(vr, a); HS(vp, b); HS(vz, c); HS(psi, d); HS(chi, e);
  return vec2tp(*vr, *vp, *vz, *psi, *chi);
}
int orc_tp2vec(int a, int b, int c, int d, int e) {
  NEED_KIT; HS(psi, a); HS(chi, b); HS(vr, c); HS(vp, d); HS(vz, e);
  return tp2vec(*psi, *chi, *vr, *vp, *vz);
}
int orc_tp2curlvec(int a, int b, int c, int d, int e) {
  NEED_KIT; HS(psi, a); HS(chi, b); HS(vr, c); HS(vp, d); HS(vz, e);
  return tp2curlvec(*psi, *chi, *vr, *vp, *vz);
}
int orc_advection_rhs(int a, int b, int c, int d, int e) {
  NEED_KIT; HS(psi, a); HS(chi, b); HS(nlpsi, c); HS(nlchi, d); HS(uz, e);
  return advection_rhs(*psi, *chi, *nlpsi, *nlchi, *uz);
}
int orc_vortex_step(int a, int b, int c, int d, int e, int f, int g, int h, int u, double dt, double* gains) {
  NEED_KIT; HS(psi, a); HS(chi, b); HS(nlpsi, c); HS(nlchi, d); HS(psip, e); HS(chip, f); HS(nlpsip, g);
  HS(nlchip, h); HS(uz, u);
  return vortex_step(*psi, *chi, *nlpsi, *nlchi, *psip, *chip, *nlpsip, *nlchip, *uz, dt, gains);
}
}  // extern "C"
