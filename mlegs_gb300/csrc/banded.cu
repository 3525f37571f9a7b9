// banded.cu — banded radial operators and solves per (m, k) column.
//
//   matvec: xxdx (tridiagonal), del2h, del2 (pentadiagonal), mlegs_scalar_ops.f90:418-573, with the
//           bands of mlegs_spectfm_diff.f90:6-152 precomputed once per m (kit.cu); del2 adds -ak^2 on
//           the diagonal per k.  One CTA per (m, k) column stages the column in shared memory and
//           applies the band in place.
//   solve:  ihelm, idel2 (pre/pro ln), ihelmp (:575-1000) through lsolve -> zgbtrf + zgbtrs
//           (mlegs_bndmat_ops.f90:369-457): LU with partial pivoting over kl rows, multipliers by the
//           reciprocal pivot, U of bandwidth kl+ku, one right-hand side.  One thread per system;
//           the factor lives in a scratch band laid out [row][diagonal][system] so that a warp's
//           32 systems touch consecutive addresses.
// Every per-(m,k) loop of the reference visits k = 1..nzc and then k = nzcu..nzdim; when nzc == nzcu
// (nzchop = nz/2+1) the shared slot is processed twice, and so it is here.
#include "common.cuh"

namespace mlg {

__device__ __forceinline__ int k_count(int k0, int nzc, int nzcu, int nzdim) {  // 0-based k
  int kk = k0 + 1;
  return (kk <= min(nzdim, nzc) ? 1 : 0) + (kk >= max(nzcu, 1) ? 1 : 0);
}

// op: 0 = xxdx, 1 = del2h, 2 = del2
// ln handling (column (m=0,k=0) only): the ln terms added after the band product, and ln <- 0.
__global__ void k_band_apply(double2* __restrict__ e, const double* __restrict__ bd2, const double* __restrict__ bxx,
                             const double* __restrict__ ak, double* __restrict__ lnp, const double* __restrict__ lognorm,
                             int op, int nrdim, int npdim, int ne, int nrc, int npc, int nzc, int nzcu, int nzdim,
                             double ell) {
  extern __shared__ double2 col[];
  double2* c0 = col;
  double2* c1 = col + nrdim;
  int m = blockIdx.y, k = blockIdx.x;
  int nn = max(min(nrc, nrc - m), 0);
  int cnt = k_count(k, nzc, nzcu, nzdim);
  double2* g = e + (size_t)nrdim * (m + (size_t)npdim * k);
  bool lnblk = (m == 0 && k == 0);
  double lnin = 0.0;
  if (lnblk) lnin = *lnp;
  if (m < npc && nn > 0 && cnt > 0) {
    for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = g[i];
    __syncthreads();
    double akv = ak[k];
    for (int rep = 0; rep < cnt; ++rep) {
      for (int i = threadIdx.x; i < nn; i += blockDim.x) {
        double2 acc = make_double2(0, 0);
        if (op == 0) {
          const double* b = bxx + 3 * ((size_t)i + (size_t)ne * m);
          if (i - 1 >= 0) { acc.x += b[0] * c0[i - 1].x; acc.y += b[0] * c0[i - 1].y; }
          if (i + 1 < nn) { acc.x += b[2] * c0[i + 1].x; acc.y += b[2] * c0[i + 1].y; }
        } else {
          const double* b = bd2 + 5 * ((size_t)i + (size_t)ne * m);
#pragma unroll
          for (int c = 0; c < 5; ++c) {
            int j = i - 2 + c;
            if (j < 0 || j >= nn) continue;
            double v = b[c];
            if (c == 2 && op == 2) v = v - pow(akv, 2.0);
            acc.x += v * c0[j].x;
            acc.y += v * c0[j].y;
          }
        }
        c1[i] = acc;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < nn; i += blockDim.x) c0[i] = c1[i];
      __syncthreads();
    }
    if (lnblk && threadIdx.x == 0) {
      if (op == 0) {   // r d/dr of the log term (:452-456)
        c0[0].x += 1.0 / exp(lognorm[0]) * lnin;
        if (nn > 1) c0[1].x += 1.0 / exp(lognorm[1]) * lnin;
      } else {         // (:506-511, :561-566)
        double e2 = pow(ell, 2.0);
        c0[0].x += 4.0 / 3.0 / e2 / exp(lognorm[0]) * lnin;
        if (nn > 1) c0[1].x -= 2.0 / 1.0 / e2 / exp(lognorm[1]) * lnin;
        if (nn > 2) c0[2].x += 2.0 / 3.0 / e2 / exp(lognorm[2]) * lnin;
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nn; i += blockDim.x) g[i] = c0[i];
  } else if (lnblk && threadIdx.x == 0) {
    // the (1,1,1) column is not active: the ln terms still land on it
    double e2 = pow(ell, 2.0);
    if (op == 0) {
      g[0].x += 1.0 / exp(lognorm[0]) * lnin;
      g[1].x += 1.0 / exp(lognorm[1]) * lnin;
    } else {
      g[0].x += 4.0 / 3.0 / e2 / exp(lognorm[0]) * lnin;
      g[1].x -= 2.0 / 1.0 / e2 / exp(lognorm[1]) * lnin;
      g[2].x += 2.0 / 3.0 / e2 / exp(lognorm[2]) * lnin;
    }
  }
  if (lnblk && threadIdx.x == 0) *lnp = 0.0;
}

int launch_band_apply(Scalar& s, int op, const ChopIdx& c) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  size_t sm = 2ull * G.nrdim * sizeof(double2);
  if (sm > 48 * 1024) MLG_CUDA(cudaFuncSetAttribute(k_band_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  dim3 grid(G.nzdim, std::max(c.npc, 1));
  kt_begin(2);
  k_band_apply<<<grid, 128, sm, G.stream>>>(s.e, G.bd2, G.bxx, G.ak, s.ln, G.lognorm, op, G.nrdim, G.npdim, G.ne, c.nrc,
                                            c.npc, c.nzc, c.nzcu, G.nzdim, G.ell);
  MLG_LAUNCH();
  kt_end(2, 2.0 * G.fsize * 16);
  return 0;
}

// ------------------------------------------------------------------------------------------------
// banded LU solve, one thread per (m, k) system.
// mode 0: ihelm / idel2 generic:  A = D0(m) - ak^2 I + alpha I             (kl = ku = 2)
// mode 1: idel2_proln on (0,0):   A = D0(0) with the column-1 log-term additions (:705-711)
// mode 2: idel2_preln on (0,0):   rows shifted down, bordered by the ln unknown (:609-625), kl = 3
// mode 3: ihelmp:                 A = D^q + beta D + alpha I, q = power/2   (kl = ku = power)
// flags (per launch): pre-solve ln handling for ihelm/ihelmp, post-solve ln for idel2.
struct SolveArgs {
  double2* e;
  double* ws;           // scratch band [row][W][nsys]
  double* lnp;
  const double* bd2;
  const double* ak;
  const double* lognorm;
  int* status;
  int nrdim, npdim, ne, nrc, npc, nzc, nzcu, nzdim;
  int nsys;             // npc * nzdim
  double alpha, beta, ell, preln;
  int kind;             // 0 ihelm, 1 idel2_proln, 2 idel2_preln, 3 ihelmp
  int power;
};

// entry (i, j) (0-based) of D(m,k) = D0(m) - ak^2 I for an n x n truncation
__device__ __forceinline__ double dmat(const SolveArgs& a, int m, double akv, int n, int i, int j) {
  if (i < 0 || j < 0 || i >= n || j >= n) return 0.0;
  int c = j - i + 2;
  if (c < 0 || c > 4) return 0.0;
  double v = a.bd2[c + 5 * ((size_t)i + (size_t)a.ne * m)];
  if (c == 2) v = v - pow(akv, 2.0);
  return v;
}

__global__ void k_band_solve(SolveArgs a) {
  int sys = blockIdx.x * blockDim.x + threadIdx.x;
  if (sys >= a.nsys) return;
  int m = sys / a.nzdim, k = sys % a.nzdim;
  int cnt = k_count(k, a.nzc, a.nzcu, a.nzdim);
  int nn = max(min(a.nrc, a.nrc - m), 0);
  bool root = (m == 0 && k == 0);
  double e2 = pow(a.ell, 2.0);
  // ln handling before the solves (ihelm :818-824, ihelmp :937-951 is done separately)
  if (root && a.kind == 0) {
    double lnin = *a.lnp;
    double lno = lnin / a.alpha;
    *a.lnp = lno;
    double2* g = a.e;
    g[0].x -= 4.0 / 3.0 / e2 / exp(a.lognorm[0]) * lno;
    g[1].x += 2.0 / 1.0 / e2 / exp(a.lognorm[1]) * lno;
    g[2].x -= 2.0 / 3.0 / e2 / exp(a.lognorm[2]) * lno;
  }
  if (m >= a.npc || nn < 1 || cnt == 0) return;
  bool special = root && (a.kind == 1 || a.kind == 2);
  int kl = 2, ku = 2;
  if (special && a.kind == 2) { kl = 3; ku = 2; }
  if (a.kind == 3) { kl = a.power; ku = a.power; }
  int W = 2 * kl + ku + 1;
  double akv = a.ak[k];
  double2* x = a.e + (size_t)a.nrdim * (m + (size_t)a.npdim * k);
  double alpha = (a.kind == 0 || a.kind == 3) ? a.alpha : 0.0;
  size_t ns = a.nsys;
#define U(i, j) a.ws[((size_t)(i) * W + ((j) - (i) + kl)) * ns + sys]
  for (int rep = 0; rep < cnt; ++rep) {
    // build the band rows (columns i-kl .. i+ku) into the work band
    for (int i = 0; i < nn; ++i) {
      for (int c = 0; c < W; ++c) a.ws[((size_t)i * W + c) * ns + sys] = 0.0;
      if (a.kind == 3) {
        // row i of the truncated power D^q, q = power/2 (the band products of mulrbrb,
        // mlegs_bndmat_ops.f90:251-318, on nn x nn matrices), window i-8 .. i+8
        int q = a.power / 2;
        double rv[17], nv[17];
        int w0 = i - 8;
        for (int u = 0; u < 17; ++u) rv[u] = 0.0;
        for (int jj = max(0, i - 2); jj <= min(nn - 1, i + 2); ++jj) rv[jj - w0] = dmat(a, m, akv, nn, i, jj);
        for (int t = 2; t <= q; ++t) {
          for (int u = 0; u < 17; ++u) nv[u] = 0.0;
          for (int u = 0; u < 17; ++u) {
            int col = w0 + u;
            if (col < 0 || col >= nn) continue;
            for (int jj = max(0, col - 2); jj <= min(nn - 1, col + 2); ++jj) {
              int uu = jj - w0;
              if (uu >= 0 && uu < 17) nv[uu] += rv[u] * dmat(a, m, akv, nn, col, jj);
            }
          }
          for (int u = 0; u < 17; ++u) rv[u] = nv[u];
        }
        for (int j = max(0, i - kl); j <= min(nn - 1, i + ku); ++j) {
          double v = rv[j - w0] + a.beta * dmat(a, m, akv, nn, i, j);
          if (i == j) v += alpha;
          U(i, j) = v;
        }
        continue;
      }
      for (int j = max(0, i - kl); j <= min(nn - 1, i + ku); ++j) {
        double v;
        if (special && a.kind == 1) {
          v = dmat(a, 0, akv, nn, i, j);
          if (j == 0) {
            if (i == 0) v += 4.0 / 3.0 / e2;
            if (i == 1) v -= 2.0 / 1.0 / e2 * exp(a.lognorm[0] - a.lognorm[1]);
            if (i == 2) v += 2.0 / 3.0 / e2 * exp(a.lognorm[0] - a.lognorm[2]);
          }
        } else if (special && a.kind == 2) {
          // del2_pre(2:nn,:) = del2_pre(1:nn-1,:); row 1 = e_1; column-1 additions (:609-617)
          if (i == 0) v = (j == 0) ? 1.0 : 0.0;
          else {
            v = dmat(a, 0, akv, nn, i - 1, j);
            if (j == 0) {
              if (i == 1) v += 4.0 / 3.0 / e2;
              if (i == 2) v -= 2.0 / 1.0 / e2 * exp(a.lognorm[0] - a.lognorm[1]);
              if (i == 3) v += 2.0 / 3.0 / e2 * exp(a.lognorm[0] - a.lognorm[2]);
            }
          }
        } else {
          v = dmat(a, m, akv, nn, i, j);
          if (i == j) v += alpha;
        }
        U(i, j) = v;
      }
    }
    if (special && a.kind == 2 && rep == 0) {
      for (int i = nn - 1; i >= 1; --i) x[i] = x[i - 1];
      x[0] = make_double2(a.preln / exp(a.lognorm[0]), 0.0);
    }
    // factor + forward substitution (gbtrf/gbtrs 'N')
    for (int j = 0; j < nn; ++j) {
      int km = min(kl, nn - 1 - j), p = j;
      double best = fabs(U(j, j));
      for (int i = j + 1; i <= j + km; ++i) {
        double t = fabs(U(i, j));
        if (t > best) { best = t; p = i; }
      }
      if (U(p, j) == 0.0) { atomicExch(a.status, 1); return; }
      int ju = min(nn - 1, j + kl + ku);
      if (p != j) {
        for (int c = j; c <= ju; ++c) { double t = U(p, c); U(p, c) = U(j, c); U(j, c) = t; }
        double2 t = x[p]; x[p] = x[j]; x[j] = t;
      }
      double rp = 1.0 / U(j, j);
      double2 xj = x[j];
      for (int i = j + 1; i <= j + km; ++i) {
        double l = U(i, j) * rp;
        U(i, j) = l;
        for (int c = j + 1; c <= ju; ++c) U(i, c) -= l * U(j, c);
        x[i].x -= l * xj.x;
        x[i].y -= l * xj.y;
      }
    }
    for (int j = nn - 1; j >= 0; --j) {
      double d = U(j, j);
      double2 xj = make_double2(x[j].x / d, x[j].y / d);
      x[j] = xj;
      for (int i = j - 1; i >= max(0, j - kl - ku); --i) {
        double u = U(i, j);
        x[i].x -= xj.x * u;
        x[i].y -= xj.y * u;
      }
    }
  }
#undef U
  if (special) *a.lnp = x[0].x * exp(a.lognorm[0]);
}

// ihelmp's log-term pre-step (mlegs_scalar_ops.f90:937-951): ln <- ln/alpha, then
// e(:nrc,1,1) -= D(0,0)^(q-1) bl2 + beta bl2 with bl2 = (4/3, -2, 2/3)/ell^2/exp(lognorm) * ln.
__global__ void k_ihelmp_pre(double2* __restrict__ e, double* __restrict__ lnp, const double* __restrict__ bd2,
                             const double* __restrict__ ak, const double* __restrict__ lognorm, double* __restrict__ tmp,
                             int nrc, int ne, int power, double alpha, double beta, double ell) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double lno = *lnp / alpha;
  *lnp = lno;
  double e2 = pow(ell, 2.0);
  double* bl = tmp;
  double* bl2 = tmp + nrc;
  double* t = tmp + 2 * nrc;
  for (int i = 0; i < nrc; ++i) bl2[i] = 0.0;
  bl2[0] = 4.0 / 3.0 / e2 / exp(lognorm[0]) * lno;
  if (nrc > 1) bl2[1] = -2.0 / e2 / exp(lognorm[1]) * lno;
  if (nrc > 2) bl2[2] = 2.0 / 3.0 / e2 / exp(lognorm[2]) * lno;
  for (int i = 0; i < nrc; ++i) bl[i] = bl2[i];
  double akv = ak[0];
  for (int n = 1; n <= power / 2 - 1; ++n) {
    for (int i = 0; i < nrc; ++i) {
      double acc = 0.0;
      for (int j = max(0, i - 2); j <= min(nrc - 1, i + 2); ++j) {
        int c = j - i + 2;
        double v = bd2[c + 5 * ((size_t)i + (size_t)ne * 0)];
        if (c == 2) v = v - pow(akv, 2.0);
        acc += v * bl[j];
      }
      t[i] = acc;
    }
    for (int i = 0; i < nrc; ++i) bl[i] = t[i];
  }
  for (int i = 0; i < nrc; ++i) e[i].x -= bl[i] + beta * bl2[i];
}

int launch_ihelmp_pre(Scalar& s, const ChopIdx& c, int power, double alpha, double beta) {
  if (3 * c.nrc > 2 * 4096) return set_error(MLG_ESIZE, "ihelmp: nrc too large for the log-term workspace");
  k_ihelmp_pre<<<1, 32, 0, G.stream>>>(s.e, s.ln, G.bd2, G.ak, G.lognorm, G.dscal + DS_CALC, c.nrc, G.ne, power, alpha,
                                       beta, G.ell);
  MLG_LAUNCH();
  return 0;
}

// kind as in SolveArgs; the band scratch grows to fit (kl, ku)
int launch_band_solve(Scalar& s, int kind, const ChopIdx& c, double alpha, double beta, double preln, int power) {
  if (c.npc > G.npchop) return set_error(MLG_ECHOP, "chop_index: chopping in p beyond the kit's azimuthal modes");
  int kl = 2, ku = 2;
  if (kind == 2) kl = 3;
  if (kind == 3) { kl = power; ku = power; }
  int W = 2 * kl + ku + 1;
  int npc = std::max(c.npc, 1);
  size_t nsys = (size_t)npc * G.nzdim;
  int nnmax = std::max(std::min(c.nrc, G.nrdim), 1);
  size_t need = (size_t)nnmax * W * nsys * sizeof(double);
  if (need > G.band_ws_bytes) {
    if (G.band_ws) dfree(G.band_ws, G.band_ws_bytes);
    G.band_ws = nullptr;
    G.band_ws_bytes = 0;
    MLG_TRY(dmalloc((void**)&G.band_ws, need));
    G.band_ws_bytes = need;
  }
  SolveArgs a;
  a.e = s.e; a.ws = G.band_ws; a.lnp = s.ln; a.bd2 = G.bd2; a.ak = G.ak; a.lognorm = G.lognorm;
  a.status = (int*)(G.dscal + DS_FLAG + 1);
  a.nrdim = G.nrdim; a.npdim = G.npdim; a.ne = G.ne; a.nrc = c.nrc; a.npc = c.npc; a.nzc = c.nzc; a.nzcu = c.nzcu;
  a.nzdim = G.nzdim; a.nsys = (int)nsys; a.alpha = alpha; a.beta = beta; a.ell = G.ell; a.preln = preln;
  a.kind = kind; a.power = power;
  kt_begin(2);
  k_band_solve<<<cdiv(nsys, 64), 64, 0, G.stream>>>(a);
  MLG_LAUNCH();
  kt_end(2, 2.0 * G.fsize * 16);
  return 0;
}

}  // namespace mlg
