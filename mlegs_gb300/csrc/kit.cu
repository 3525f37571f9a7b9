// kit.cu — the transform kit (tfm_kit_init, src/submodules/mlegs_spectfm_init.f90:6-154) on GB300.
//
// Host FP64, with the reference's own operation order: the O(nr) / O(ne*npchop) scalar arrays
// (Gauss-Legendre nodes and weights :181-214, the map r(x) :112, -log(1-x) :68, ak :133-134,
// lognorm :218-250, log_fact :351-357).  These are a few thousand numbers; computing them with the
// same libm as the reference keeps them bit-identical.
//
// GPU: the P_L^m table (leg_tbl :254-300), which the reference evaluates in FM 50-digit arithmetic
// (9.88 s at NR=200, NPCHOP=65, docs/tutorial/initialization.md:85).  Here one thread per (x_i, m)
// runs the same scaled three-term recurrence in double-double arithmetic (~32 digits) with a
// separate binary exponent, so (1-x^2)^(m/2) never underflows, then multiplies by
// exp(log_fact(n)+lognorm(n,m)) evaluated in double-double and rounds to FP64.  Derived tables
// (del2 / xxdx band coefficients, the vec2tp projection matrices, FFT twiddles, FP32 copies) are
// built on the GPU from it.
#include "common.cuh"
#include <cmath>
#include <algorithm>

namespace mlg {

static const double PI = 3.14159265358979323846264338327950288;

// ------------------------------------------------------------------------------------------------
// double-double arithmetic (Dekker / Knuth error-free transformations)
struct dd { double hi, lo; };
__device__ __forceinline__ dd two_sum(double a, double b) {
  double s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dd quick_two_sum(double a, double b) { double s = a + b; return {s, b - (s - a)}; }
__device__ __forceinline__ dd two_prod(double a, double b) { double p = a * b; return {p, fma(a, b, -p)}; }
__device__ __forceinline__ dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
  s.lo += t.hi; s = quick_two_sum(s.hi, s.lo); s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
__device__ __forceinline__ dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd dd_mul_d(dd a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd dd_div(dd a, dd b) {
  double q1 = a.hi / b.hi;
  dd r = dd_sub(a, dd_mul_d(b, q1));
  double q2 = r.hi / b.hi;
  r = dd_sub(r, dd_mul_d(b, q2));
  double q3 = r.hi / b.hi;
  dd q = quick_two_sum(q1, q2);
  return dd_add(q, {q3, 0.0});
}
__device__ __forceinline__ dd dd_div_d(dd a, double b) { return dd_div(a, {b, 0.0}); }
__device__ __forceinline__ dd dd_sqrt(dd a) {  // Karp-Markstein: one Newton step on a double seed
  if (a.hi <= 0.0) return {0.0, 0.0};
  double x = 1.0 / sqrt(a.hi), y = a.hi * x;
  dd y2 = two_prod(y, y);
  double d = dd_sub(a, y2).hi * (x * 0.5);
  return two_sum(y, d);
}
__device__ __forceinline__ dd dd_ldexp(dd a, int e) { return {ldexp(a.hi, e), ldexp(a.lo, e)}; }

// exp of a double-double argument, returned as mantissa * 2^k (k separate: the result can exceed
// the FP64 range).  Range reduction by k*ln2, scaling by 2^-10, Taylor series to degree 12 in
// Horner form, then ten squarings of (1+s) kept as s -> 2s + s^2.
__device__ dd dd_exp2k(dd a, int* kout) {
  const dd LN2 = {6.93147180559945286226764e-01, 2.319046813846299558417771e-17};
  double kd = rint(a.hi / LN2.hi);
  dd r = dd_sub(a, dd_mul_d(LN2, kd));
  r = dd_ldexp(r, -10);
  dd s = {1.0, 0.0};
  // e^r - 1 = r (1 + r/2 (1 + r/3 (1 + ... (1 + r/13))))
  for (int n = 13; n >= 2; --n) s = dd_add({1.0, 0.0}, dd_mul(dd_div_d(r, (double)n), s));
  s = dd_mul(r, s);
  for (int i = 0; i < 10; ++i) s = dd_add(dd_mul_d(s, 2.0), dd_mul(s, s));
  *kout = (int)kd;
  return dd_add({1.0, 0.0}, s);
}

// leg_tbl (mlegs_spectfm_init.f90:254-300): tbl(xx, nn, mm), nn = 1..ne_out, for the m of column mm
__global__ void k_leg_tbl(const double* __restrict__ xs, int nx, int ne_out, int nm,
                          const double* __restrict__ lnrm, int lnrm_ld, const double* __restrict__ logfact,
                          int m_is_zero, double* __restrict__ tbl) {
  int xx = blockIdx.x * blockDim.x + threadIdx.x;
  int mm = blockIdx.y;
  if (xx >= nx || mm >= nm) return;
  int m = m_is_zero ? 0 : mm;
  double x = xs[xx];
  // (-1)^m * sqrt(1-x^2)^m (:280) with a running binary exponent
  dd omx2 = dd_sub({1.0, 0.0}, two_prod(x, x));
  dd s = dd_sqrt(omx2);
  dd pw = {1.0, 0.0};
  int E = 0;
  for (int k = 0; k < m; ++k) {
    pw = dd_mul(pw, s);
    if (fabs(pw.hi) < 0x1p-400 && pw.hi != 0.0) { pw = dd_ldexp(pw, 600); E -= 600; }
  }
  dd f2 = (m & 1) ? dd_neg(pw) : pw;  // f(nn-2) in the loop below
  dd f1 = dd_mul_d(f2, x);            // (:282)
  for (int nn = 1; nn <= ne_out; ++nn) {
    int n = m + nn - 1;
    dd f;
    if (nn == 1) f = f2;
    else if (nn == 2) f = f1;
    else {
      // (:285-287): 1/(n-m) * (f(nn-1)*x - f(nn-2)*(n+m-1)/(2n-1)/(2n-3))
      dd c = dd_div_d(dd_div_d({(double)(n + m - 1), 0.0}, (double)(2 * n - 1)), (double)(2 * n - 3));
      f = dd_div_d(dd_sub(dd_mul_d(f1, x), dd_mul(f2, c)), (double)(n - m));
      f2 = f1; f1 = f;
      double a = fabs(f.hi);
      if (a > 0x1p+400) { f1 = dd_ldexp(f1, -600); f2 = dd_ldexp(f2, -600); f = f1; E += 600; }
      else if (a < 0x1p-400 && a != 0.0 && fabs(f2.hi) < 0x1p-400) {
        f1 = dd_ldexp(f1, 600); f2 = dd_ldexp(f2, 600); f = f1; E -= 600;
      }
    }
    // (:291): * exp(log_fact(n) + lnrm(nn, mm)), both FP64, summed exactly as FM does
    dd arg = two_sum(logfact[n], lnrm[(nn - 1) + (size_t)lnrm_ld * (m_is_zero ? 0 : mm)]);
    int k;
    dd ex = dd_exp2k(arg, &k);
    dd v = dd_mul(f, ex);
    double out = ldexp(v.hi + v.lo, E + k);
    tbl[xx + (size_t)nx * ((nn - 1) + (size_t)ne_out * mm)] = out;
  }
}

// del2 band without the -ak^2 term and xxdx band for each (row, m) (mlegs_spectfm_diff.f90:6-152),
// with the exp(lognorm_j - lognorm_i) scaling; entries whose column lies outside 1..ne are zero.
__global__ void k_bands(int ne, int npchop, double ell, const double* __restrict__ lognorm,
                        double* __restrict__ bd2, double* __restrict__ bxx) {
  int nn = blockIdx.x * blockDim.x + threadIdx.x + 1;  // 1-based row
  int mm = blockIdx.y;
  if (nn > ne) return;
  int am = mm;
  double n = am + (nn - 1), s = 0.0, ell2 = pow(ell, 2.0);
  const double* L = lognorm + (size_t)ne * mm;
  double g[5] = {0, 0, 0, 0, 0};
  if (nn - 2 >= 1) g[0] = -(n - am - 1.0) * (n - am) * (n - 2.0 + s) * (n - 1.0 + s) / (2.0 * n - 3.0) / (2.0 * n - 1.0);
  if (nn - 1 >= 1) g[1] = 2.0 * n * (n - am) * (n - 1.0 + s) / (2.0 * n - 1.0);
  g[2] = (-2.0 * n * (n + 1.0) * (3.0 * n * n + 3.0 * n - am * am - 2.0) + 2.0 * s * (s - 2.0) * (n * n + n + am * am - 1.0)) /
         (2.0 * n - 1.0) / (2.0 * n + 3.0);
  g[3] = 2.0 * (n + 1.0) * (n + am + 1.0) * (n + 2.0 - s) / (2.0 * n + 3.0);
  g[4] = -(n + am + 1.0) * (n + am + 2.0) * (n + 3.0 - s) * (n + 2.0 - s) / (2.0 * n + 3.0) / (2.0 * n + 5.0);
  for (int c = 0; c < 5; ++c) {
    int j = nn - 2 + c;
    double v = 0.0;
    if (j >= 1 && j <= ne) v = (g[c] / ell2) * exp(L[j - 1] - L[nn - 1]);
    if (c == 2) v = g[c] / ell2;  // diagonal: exp(0) = 1; the -ak^2 term is added per k
    bd2[c + 5 * ((size_t)(nn - 1) + (size_t)ne * mm)] = v;
  }
  double x[3] = {0, 0, 0};
  if (nn - 1 >= 1) x[0] = -(n - 1.0) * (n - am) / (2.0 * n - 1.0);
  x[2] = (n + 2.0) * (n + am + 1.0) / (2.0 * n + 3.0);
  for (int c = 0; c < 3; c += 2) {
    int j = nn - 1 + c;
    double v = 0.0;
    if (j >= 1 && j <= ne) v = x[c] * exp(L[j - 1] - L[nn - 1]);
    bxx[c + 3 * ((size_t)(nn - 1) + (size_t)ne * mm)] = v;
  }
  bxx[1 + 3 * ((size_t)(nn - 1) + (size_t)ne * mm)] = 0.0;
}

// vec2tp projection matrices (mlegs_scalar_ops.f90:1395-1411) for the row offset 3 used there:
// V(i,x) = pf(x,i)/n/(n+1)/fff(x), D(i,x) = pfd(x,i)/n/(n+1)/fff(x), T(i,x) = pf(x,i)*w(x),
// pfd = pf .mul. leg_xxdx, fff = (1-x^2)/w, n = max(1, m+i-1); stored (nrh, ne, npchop) like pf.
__global__ void k_vec2tp_mats(int nrh, int ne, int npchop, int nrchop, const double* __restrict__ pf,
                              const double* __restrict__ bxx, const double* __restrict__ x,
                              const double* __restrict__ w, double* __restrict__ V, double* __restrict__ D,
                              double* __restrict__ T) {
  int xi = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y + 1;  // 1-based row
  int mm = blockIdx.z;
  if (xi >= nrh) return;
  int mv = mm;
  int nn = nrchop + 3 - mv;  // nrcs(m) with offset 3
  size_t o = xi + (size_t)nrh * ((i - 1) + (size_t)ne * mm);
  if (i > nn || i > ne) { V[o] = 0; D[o] = 0; T[o] = 0; return; }
  auto PF = [&](int r1) { return pf[xi + (size_t)nrh * ((r1 - 1) + (size_t)ne * mm)]; };
  auto XX = [&](int r1, int c1) -> double {  // leg_xxdx(mv, nn+1, nn+1)(r1, c1)
    if (r1 < 1 || c1 < 1 || r1 > nn + 1 || c1 > nn + 1) return 0.0;
    int c = c1 - r1 + 1;
    if (c < 0 || c > 2) return 0.0;
    return bxx[c + 3 * ((size_t)(r1 - 1) + (size_t)ne * mm)];
  };
  // pfd(x, i) = sum_r pf(x, r) * XX(r, i), r in i-1..i+1 (mulrrb, mlegs_bndmat_ops.f90:135-160)
  double pfd = 0.0;
  for (int r1 = max(1, i - 1); r1 <= min(nn + 1, i + 1); ++r1) pfd += PF(r1) * XX(r1, i);
  double xv = x[xi], wv = w[xi];
  double fff = (1.0 - pow(xv, 2.0)) / wv;
  int n = max(1, mv + i - 1);
  V[o] = PF(i) / n / (n + 1) / fff;
  D[o] = pfd / n / (n + 1) / fff;
  T[o] = PF(i) * wv;
}

__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// ------------------------------------------------------------------------------------------------
// host-side FP64 pieces, same operation order as the reference
static void gauss_legendre(double x1, double x2, std::vector<double>& x, std::vector<double>& w, int n) {
  const double eps = 1.0e-15;   // (:187)
  int m = (int)std::ceil((n + 1) / 2.0);
  double xm = (x2 + x1) / 2.0, xl = (x2 - x1) / 2.0;
  for (int i = 1; i <= m; ++i) {
    volatile double z = std::cos(PI * (i - .25) / (n + .5));
    double z1 = z + 1.0, p1 = 0, p2 = 0, p3 = 0, pp = 0;
    while (std::fabs(z - z1) > eps) {
      p1 = 1.0; p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        p3 = p2; p2 = p1;
        volatile double t = (2 * j - 1) * z * p2;   // no contraction into FMA: matches the reference
        volatile double u = (j - 1) * p3;
        p1 = (t - u) / j;
      }
      volatile double zz = z * p1;
      volatile double z2 = z * z;
      pp = n * (zz - p2) / (z2 - 1);
      z1 = z;
      z = z1 - p1 / pp;
    }
    x[i - 1] = xm - xl * z;
    x[n - i] = xm + xl * z;
    volatile double zz = z * z;
    volatile double q = (1 - zz) * pp;
    w[i - 1] = 2 * xl / (q * pp);
    w[n - i] = w[i - 1];
  }
}

static std::vector<double> leg_lognorm(int ndim, int nm) {
  int me = nm - 1;
  std::vector<double> wk(me + 1);
  wk[0] = std::log(.5);
  for (int m = 1; m <= me; ++m)
    wk[m] = wk[m - 1] + std::log(2.0 * m + 1.0) - std::log(2.0 * m * std::pow(2.0 * m - 1.0, 2));
  std::vector<double> l((size_t)ndim * nm);
  for (int mm = 0; mm < nm; ++mm) {
    int m = mm;
    l[(size_t)ndim * mm] = wk[m];
    for (int nn = 2; nn <= ndim; ++nn) {
      int n = m + (nn - 1);
      l[(nn - 1) + (size_t)ndim * mm] = l[(nn - 2) + (size_t)ndim * mm] + std::log(2.0 * n + 1.0) - std::log(2.0 * n - 1.0) +
                                        std::log(1.0 * (n - m)) - std::log(1.0 * (n + m));
    }
    for (int nn = 1; nn <= ndim; ++nn) l[(nn - 1) + (size_t)ndim * mm] *= .5;
  }
  return l;
}

static bool factors235(int n) {
  while (n % 2 == 0 || n % 3 == 0 || n % 5 == 0) {
    if (n % 2 == 0) n /= 2;
    if (n % 3 == 0) n /= 3;
    if (n % 5 == 0) n /= 5;
  }
  return n == 1;
}

template <class T>
static int upload(T** d, const std::vector<T>& h) {
  MLG_TRY(dmalloc((void**)d, h.size() * sizeof(T)));
  MLG_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

int kit_build(const mlg_params* P) {
  if (G.kit_set)
    return set_error(MLG_ENOKIT, "tfm_kit_init: only one MLegS transformation kit (either 1D, 2D or 3D) is permitted per program");
  int nr = P->nr, np = P->np, nz = P->nz;
  // parameter checks (mlegs_spectfm_init.f90:35-62)
  if (!(nr > 0 && nr % 2 == 0)) return set_error(MLG_EPARAM, "tfm_kit_init: nr must be even");
  if (!(np > 0 && (np == 1 || np % 2 == 0))) return set_error(MLG_EPARAM, "tfm_kit_init: np must be even");
  if (np != 1 && !factors235(np)) return set_error(MLG_EPARAM, "tfm_kit_init: np must only have factors of 2, 3 and 5");
  if (!(nz > 0 && (nz == 1 || nz % 2 == 0))) return set_error(MLG_EPARAM, "tfm_kit_init: nz must be even");
  if (nz != 1 && !factors235(nz)) return set_error(MLG_EPARAM, "tfm_kit_init: nz must only have factors of 2, 3 and 5");
  if (P->nrchop > nr) return set_error(MLG_EPARAM, "tfm_kit_init: nrchop must be smaller than or equal to nr");
  if (np != 1 && P->npchop * 2 > np + 2) return set_error(MLG_EPARAM, "tfm_kit_init: npchop <= np/2 + 1 must be satisfied");
  if (nz != 1 && P->nzchop * 2 > nz + 2) return set_error(MLG_EPARAM, "tfm_kit_init: nzchop <= nz/2 + 1 must be satisfied");
  if (P->nrchop < 1 || P->npchop < 1 || P->nzchop < 1) return set_error(MLG_EPARAM, "tfm_kit_init: chops must be positive");
  if (P->hyperpow != 0 && !(P->hyperpow == 4 || P->hyperpow == 6 || P->hyperpow == 8))
    return set_error(MLG_EPARAM, "tfm_kit_init: hyperpow must be 0, 4, 6 or 8");
  if (np > 2 * 1024 || nz > 1024) return set_error(MLG_ESIZE, "tfm_kit_init: np <= 2048 and nz <= 1024 supported");

  G.P = *P;
  G.nr = nr; G.np = np; G.nz = nz;
  G.nrchop = P->nrchop; G.npchop = P->npchop; G.nzchop = P->nzchop;
  G.ell = P->ell;
  G.nrdim = nr + std::max(3, P->hyperpow);
  G.npdim = np / 2 + 1;
  G.nzdim = nz;
  G.nrh = nr / 2;
  G.ne = P->nrchop + 14;
  G.chopzl = P->nzchop;
  G.chopzu = nz - P->nzchop + 2;
  G.nph = np / 2;
  G.fsize = (size_t)G.nrdim * G.npdim * G.nzdim;

  std::vector<double> x(nr), w(nr), r(nr), lnx(nr), ak(nz);
  gauss_legendre(-1.0, 1.0, x, w, nr);
  for (int i = 0; i < nr; ++i) lnx[i] = -std::log(1.0 - x[i]);
  for (int i = 0; i < nr; ++i) r[i] = G.ell * std::sqrt((1.0 + x[i]) / (1.0 - x[i]));
  for (int i = -nz; i <= -1; ++i) ak[i + nz] = 2.0 * PI / P->zlen * i;
  for (int i = 0; i <= nz / 2; ++i) ak[i] = 2.0 * PI / P->zlen * i;
  std::vector<double> lognorm = leg_lognorm(G.ne, G.npchop);
  int nlf = G.npchop + G.ne + 2;
  std::vector<double> logfact(nlf);
  for (int m = 0; m < nlf; ++m) logfact[m] = std::lgamma(2 * m + 1.0) - m * std::log(2.0) - std::lgamma(m + 1.0);

  std::vector<double> rinv(nr);
  for (int i = 0; i < nr; ++i) rinv[i] = 1.0 / r[i];
  std::vector<float> w32(nr);
  for (int i = 0; i < nr; ++i) w32[i] = (float)w[i];
  MLG_TRY(upload(&G.w32, w32));
  std::vector<float> ak2f(nz);
  for (int i = 0; i < nz; ++i) ak2f[i] = (float)(ak[i] * ak[i]);
  MLG_TRY(upload(&G.ak2f, ak2f));
  MLG_TRY(upload(&G.x, x)); MLG_TRY(upload(&G.w, w)); MLG_TRY(upload(&G.r, r)); MLG_TRY(upload(&G.rinv, rinv));
  MLG_TRY(upload(&G.lnx, lnx)); MLG_TRY(upload(&G.ak, ak)); MLG_TRY(upload(&G.lognorm, lognorm));
  double* d_logfact = nullptr;
  MLG_TRY(upload(&d_logfact, logfact));

  // P_L^m table on the GPU (:144-145) and the origin / infinity values (:147-150)
  size_t npf = (size_t)G.nrh * G.ne * G.npchop;
  MLG_TRY(dmalloc((void**)&G.pf, npf * sizeof(double)));
  {
    dim3 grid(cdiv(G.nrh, 64), G.npchop);
    k_leg_tbl<<<grid, 64, 0, G.stream>>>(G.x, G.nrh, G.ne, G.npchop, G.lognorm, G.ne, d_logfact, 0, G.pf);
    MLG_LAUNCH();
  }
  std::vector<double> xa(1, -1.0 + 1.0e-15), xb(1, 1.0 - 1.0e-15);
  double *d_xa = nullptr, *d_xb = nullptr;
  MLG_TRY(upload(&d_xa, xa)); MLG_TRY(upload(&d_xb, xb));
  MLG_TRY(dmalloc((void**)&G.at0, G.nrchop * sizeof(double)));
  MLG_TRY(dmalloc((void**)&G.at1, G.nrchop * sizeof(double)));
  k_leg_tbl<<<dim3(1, 1), 32, 0, G.stream>>>(d_xa, 1, G.nrchop, 1, G.lognorm, G.ne, d_logfact, 1, G.at0);
  MLG_LAUNCH();
  k_leg_tbl<<<dim3(1, 1), 32, 0, G.stream>>>(d_xb, 1, G.nrchop, 1, G.lognorm, G.ne, d_logfact, 1, G.at1);
  MLG_LAUNCH();

  // band coefficients
  MLG_TRY(dmalloc((void**)&G.bd2, (size_t)5 * G.ne * G.npchop * sizeof(double)));
  MLG_TRY(dmalloc((void**)&G.bxx, (size_t)3 * G.ne * G.npchop * sizeof(double)));
  k_bands<<<dim3(cdiv(G.ne, 64), G.npchop), 64, 0, G.stream>>>(G.ne, G.npchop, G.ell, G.lognorm, G.bd2, G.bxx);
  MLG_LAUNCH();
  MLG_TRY(dmalloc((void**)&G.bd2f, (size_t)5 * G.ne * G.npchop * sizeof(float)));
  MLG_TRY(dmalloc((void**)&G.bxxf, (size_t)3 * G.ne * G.npchop * sizeof(float)));
  k_to_f32<<<256, 256, 0, G.stream>>>(G.bd2, G.bd2f, (size_t)5 * G.ne * G.npchop); MLG_LAUNCH();
  k_to_f32<<<256, 256, 0, G.stream>>>(G.bxx, G.bxxf, (size_t)3 * G.ne * G.npchop); MLG_LAUNCH();

  // vec2tp matrices
  MLG_TRY(dmalloc((void**)&G.tV, npf * sizeof(double)));
  MLG_TRY(dmalloc((void**)&G.tD, npf * sizeof(double)));
  MLG_TRY(dmalloc((void**)&G.tT, npf * sizeof(double)));
  k_vec2tp_mats<<<dim3(cdiv(G.nrh, 64), G.ne, G.npchop), 64, 0, G.stream>>>(G.nrh, G.ne, G.npchop, G.nrchop, G.pf,
                                                                            G.bxx, G.x, G.w, G.tV, G.tD, G.tT);
  MLG_LAUNCH();

  // FP32 copies for the mixed form
  MLG_TRY(dmalloc((void**)&G.tV32, npf * sizeof(float)));
  MLG_TRY(dmalloc((void**)&G.tD32, npf * sizeof(float)));
  MLG_TRY(dmalloc((void**)&G.tT32, npf * sizeof(float)));
  k_to_f32<<<256, 256, 0, G.stream>>>(G.tV, G.tV32, npf); MLG_LAUNCH();
  k_to_f32<<<256, 256, 0, G.stream>>>(G.tD, G.tD32, npf); MLG_LAUNCH();
  k_to_f32<<<256, 256, 0, G.stream>>>(G.tT, G.tT32, npf); MLG_LAUNCH();

  // FFT twiddles, exp(-2 pi i k / L) as in FFTE's SETTBL0 (fft235.f:205-217)
  auto twid = [](int L, int count) {
    std::vector<double2> t(std::max(count, 1));
    for (int k = 0; k < count; ++k) {
      double a = -2.0 * PI / (double)L * (double)k;
      t[k] = make_double2(std::cos(a), std::sin(a));
    }
    return t;
  };
  auto to32 = [](const std::vector<double2>& t) {
    std::vector<float2> f(t.size());
    for (size_t i = 0; i < t.size(); ++i) f[i] = make_float2((float)t[i].x, (float)t[i].y);
    return f;
  };
  std::vector<double2> tp = twid(std::max(G.nph, 1), std::max(G.nph, 1)), tpr = twid(std::max(np, 1), G.nph + 1),
                       tz = twid(nz, nz);
  MLG_TRY(upload(&G.tw_p, tp));
  MLG_TRY(upload(&G.tw_pr, tpr));
  MLG_TRY(upload(&G.tw_z, tz));
  MLG_TRY(upload(&G.tw_p32, to32(tp)));
  MLG_TRY(upload(&G.tw_pr32, to32(tpr)));
  MLG_TRY(upload(&G.tw_z32, to32(tz)));
  auto todf = [](const std::vector<double2>& t) {   // x = hi + lo, hi = x rounded to FP32
    std::vector<float4> f(t.size());
    for (size_t i = 0; i < t.size(); ++i) {
      const float rh = (float)t[i].x, ih = (float)t[i].y;
      f[i] = make_float4(rh, (float)(t[i].x - (double)rh), ih, (float)(t[i].y - (double)ih));
    }
    return f;
  };
  MLG_TRY(upload(&G.tw_pdf, todf(tp)));
  MLG_TRY(upload(&G.tw_prdf, todf(tpr)));
  MLG_TRY(upload(&G.tw_zdf, todf(tz)));

  MLG_CUDA(cudaStreamSynchronize(G.stream));
  dfree(d_logfact, logfact.size() * sizeof(double));
  dfree(d_xa, sizeof(double));
  dfree(d_xb, sizeof(double));

  MLG_TRY(dmalloc((void**)&G.dscal, DS_COUNT * sizeof(double)));
  MLG_CUDA(cudaMemset(G.dscal, 0, DS_COUNT * sizeof(double)));
  MLG_CUDA(cudaGetDevice(&G.device));
  G.kit_set = true;
  return 0;
}

}  // namespace mlg
