// diag.cu — diagnostics on the device: fftreat (mlegs_scalar_ops.f90:1002-1063 with smooth,
// :2149-2175), the vorticity magnitude of save_vort_mag (vortical_flow_3d.f90:411-465) and the
// kinetic-energy spectrum of the velocity field.
#include "common.cuh"

namespace mlg {

int launch_vfft_multi(Scalar* const* s, int n, int dir);
int launch_hfft_multi(Scalar* const* s, const double* const* rs, int n, int dir);
int assign(Scalar& d, const Scalar& s);
int op_delsqp(Scalar& s, bool inverse);
int launch_set_ln(double* ln, double v);
int launch_copy_ln(double* dst, const double* src);

// one smoothing pass of a column segment of ni values (ni >= 3), in the gather form of the reference's
// scatter loop: each output adds its contributions in the loop's order (the end value's fixed weights
// first, then the neighbours i-1, i, i+1 in increasing i), so the sums are the reference's
__device__ __forceinline__ double2 smooth_at(const double2* a, int j, int ni) {   // j 0-based
  auto fw = [&](int i) {   // f of the reference's 1-based row i + 1
    return (1.0 + (double)(ni - (i + 1)) / (ni - 1.0)) * 0.5;
  };
  double2 v = make_double2(0.0, 0.0);
  if (j == 0) v = a[0];
  if (j >= ni - 3) {
    const double fae = j == ni - 3 ? 0.2 : (j == ni - 2 ? 0.3 : 0.5);
    v.x = v.x + a[ni - 1].x * fae;
    v.y = v.y + a[ni - 1].y * fae;
  }
#pragma unroll
  for (int d = -1; d <= 1; ++d) {
    const int i = j + d;   // the source row, 0-based; the loop runs over 1 <= i <= ni - 2
    if (i < 1 || i > ni - 2) continue;
    const double f = fw(i);
    const double c = d == 0 ? f : (1.0 - f) / 2.0;
    v.x = v.x + a[i].x * c;
    v.y = v.y + a[i].y * c;
  }
  return v;
}

// fftreat's middle part on (physical r, Fourier phi, z), one block per (m, k) column of m < npc:
// rows < nr times (1-x)^2, rows from ns0 of m >= 1 zeroed, five smoothing passes over the rows from
// ns (to nrdim), rows < nr divided by (1-x)^2 (each step on the active k only, as the reference)
__global__ void __launch_bounds__(128) k_fftreat_col(double2* __restrict__ e, const double* __restrict__ x, int nr,
                                                     int nrdim, int npdim, int ns, int ns0, int nzc, int nzcu) {
  extern __shared__ __align__(16) double2 ft_col[];   // 2 * (nrdim - ns + 1)
  const int k = blockIdx.x, m = blockIdx.y;
  double2* g = e + (size_t)nrdim * (m + (size_t)npdim * k);
  const bool act = (k + 1) <= nzc || (k + 1) >= nzcu;
  if (act)
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      const double w = (1.0 - x[i]) * (1.0 - x[i]);
      g[i] = make_double2(g[i].x * w, g[i].y * w);
    }
  __syncthreads();
  if (m >= 1)
    for (int i = ns0 + threadIdx.x; i < nrdim; i += blockDim.x) g[i] = make_double2(0.0, 0.0);
  __syncthreads();
  if (act) {
    const int ni = nrdim - ns;   // rows ns..nrdim-1 (0-based)
    double2* a = ft_col;
    double2* b = ft_col + ni;
    for (int j = threadIdx.x; j < ni; j += blockDim.x) a[j] = g[ns + j];
    __syncthreads();
    for (int pass = 0; pass < 5; ++pass) {
      for (int j = threadIdx.x; j < ni; j += blockDim.x) b[j] = smooth_at(a, j, ni);
      __syncthreads();
      double2* t = a; a = b; b = t;
    }
    for (int j = threadIdx.x; j < ni; j += blockDim.x) g[ns + j] = a[j];
    __syncthreads();
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      const double w = (1.0 - x[i]) * (1.0 - x[i]);
      g[i] = make_double2(g[i].x / w, g[i].y / w);
    }
  }
}

int op_fftreat(Scalar& s) {
  if (!s.is("FFF")) MLG_TRY(op_trans(s, "FFF"));
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  const int nr = G.nr, ns = nr * 3 / 4, ns0 = std::min(ns + 4, nr);
  // smooth acts on the rows ns..nrdim (1-based): at least 3 of them
  if (G.nrdim - (ns - 1) < 3) return set_error(MLG_EPARAM, "smooth: the input length must be longer than or equal to 3.");
  TMP(so);
  MLG_TRY(assign(so, s));
  MLG_TRY(launch_set_ln(so.ln, 0.0));
  MLG_TRY(op_delsqp(so, false));
  MLG_TRY(launch_rtrans_bwd(so, true));
  so.set_space("PFF");   // non-standard, as in the reference
  if (c.npc > 0) {
    const int ni = G.nrdim - (ns - 1);
    dim3 grid(G.nzdim, c.npc);
    k_fftreat_col<<<grid, 128, 2 * ni * sizeof(double2), G.stream>>>(so.e, G.x, nr, G.nrdim, G.npdim, ns - 1, ns0 - 1,
                                                                     c.nzc, c.nzcu);
    MLG_LAUNCH();
  }
  so.set_space("FFF");
  MLG_TRY(launch_rtrans_fwd(so));
  MLG_TRY(op_delsqp(so, true));
  MLG_TRY(launch_copy_ln(so.ln, s.ln));
  MLG_TRY(op_zeroat1(so));
  return assign(s, so);
}

// |w| per physical sample: the real and imaginary parts of a slot are two phi samples
__global__ void k_vort_mag(double2* __restrict__ out, const double2* __restrict__ wr, const double2* __restrict__ wp,
                           const double2* __restrict__ wz, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double2 a = wr[i], b = wp[i], c = wz[i];
    out[i] = make_double2(sqrt(a.x * a.x + b.x * b.x + c.x * c.x), sqrt(a.y * a.y + b.y * b.y + c.y * c.y));
  }
}

int op_vort_mag(const Scalar& psi, const Scalar& chi, Scalar& out) {
  if (!psi.is("FFF") || !chi.is("FFF")) return set_error(MLG_ESPACE, "save_vort_mag: psi and chi must be in FFF");
  TMP(wr); TMP(wp); TMP(wz);
  for (Scalar* q : {&wr, &wp, &wz}) q->set_space("PPP");
  MLG_TRY(op_tp2curlvec(psi, chi, wr, wp, wz));
  k_vort_mag<<<nblk(G.fsize), 256, 0, G.stream>>>(out.e, wr.e, wp.e, wz.e, G.fsize);
  MLG_LAUNCH();
  MLG_TRY(launch_set_ln(out.ln, 0.0));
  out.set_space("PPP");
  out.off[0] = out.off[1] = out.off[2] = 0;
  return 0;
}

// E(m, k) = 1/2 c_m sum_i W_i sum_c |v_c(i, m, k)|^2, one block per (m, k), a deterministic tree sum
__global__ void __launch_bounds__(128) k_ke_spectrum(const double2* __restrict__ v0, const double2* __restrict__ v1,
                                                     const double2* __restrict__ v2, const double* __restrict__ x,
                                                     const double* __restrict__ w, const double* __restrict__ r, int nr,
                                                     int nrdim, int npdim, int np, double zlen, double* __restrict__ E) {
  __shared__ double red[128];
  const int m = blockIdx.x, k = blockIdx.y;
  const size_t off = (size_t)nrdim * (m + (size_t)npdim * k);
  double s = 0.0;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    const double W = w[i] * r[i] * r[i] / (1.0 - x[i] * x[i]) * 2.0 * 3.14159265358979323846 * zlen;
    const double2 a = v0[off + i], b = v1[off + i], c = v2[off + i];
    s += W * (a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 64; o; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double cm = (m == 0 || (np % 2 == 0 && m == np / 2)) ? 1.0 : 2.0;
    E[m + (size_t)npdim * k] = 0.5 * cm * red[0];
  }
}

int op_ke_spectrum(const Scalar& psi, const Scalar& chi, double* E_host) {
  if (!psi.is("FFF") || !chi.is("FFF")) return set_error(MLG_ESPACE, "ke_spectrum: psi and chi must be in FFF");
  PrecisionScope fp64(MLG_PLAIN_FP64);   // an energy reduction: FP64 in either form
  TMP(vr); TMP(vp); TMP(vz);
  for (Scalar* q : {&vr, &vp, &vz}) q->set_space("PPP");
  MLG_TRY(op_tp2vec(psi, chi, vr, vp, vz));
  Scalar* v3[3] = {&vr, &vp, &vz};
  if (G.np > 1) MLG_TRY(launch_hfft_multi(v3, nullptr, 3, -1));   // (1/np) sum e^{-2 pi i jm/np}
  if (G.nz > 1) MLG_TRY(launch_vfft_multi(v3, 3, -1));            // (1/nz) sum e^{-2 pi i zk/nz}
  const int nm = std::min(G.npdim, G.np / 2 + 1);
  double* Ed = nullptr;
  const size_t bytes = (size_t)G.npdim * G.nzdim * sizeof(double);
  MLG_TRY(dmalloc((void**)&Ed, bytes));
  MLG_CUDA(cudaMemsetAsync(Ed, 0, bytes, G.stream));
  k_ke_spectrum<<<dim3(nm, G.nzdim), 128, 0, G.stream>>>(vr.e, vp.e, vz.e, G.x, G.w, G.r, G.nr, G.nrdim, G.npdim, G.np,
                                                         G.P.zlen, Ed);
  MLG_LAUNCH();
  int rc = 0;
  if (cudaMemcpyAsync(E_host, Ed, bytes, cudaMemcpyDeviceToHost, G.stream) != cudaSuccess ||
      cudaStreamSynchronize(G.stream) != cudaSuccess)
    rc = set_error(MLG_ECUDA, "ke_spectrum: copy to the host failed");
  dfree(Ed, bytes);
  return rc;
}

}  // namespace mlg

using namespace mlg;

extern "C" {

int mlg_fftreat(mlg_scalar h) {
  if (!G.kit_set) return set_error(MLG_ENOKIT, "transformation kit is not initialized");
  Scalar* s = reinterpret_cast<Scalar*>(h);
  if (!s || !s->e) return set_error(MLG_EHANDLE, "invalid scalar handle");
  return op_fftreat(*s);
}

int mlg_vort_mag(mlg_scalar psi, mlg_scalar chi, mlg_scalar out) {
  if (!G.kit_set) return set_error(MLG_ENOKIT, "transformation kit is not initialized");
  Scalar *p = reinterpret_cast<Scalar*>(psi), *c = reinterpret_cast<Scalar*>(chi), *o = reinterpret_cast<Scalar*>(out);
  if (!p || !c || !o || !p->e || !c->e || !o->e) return set_error(MLG_EHANDLE, "invalid scalar handle");
  if (o->e == p->e || o->e == c->e) return set_error(MLG_EHANDLE, "save_vort_mag: out must not alias psi or chi");
  return op_vort_mag(*p, *c, *o);
}

int mlg_ke_spectrum(mlg_scalar psi, mlg_scalar chi, double* E) {
  if (!G.kit_set) return set_error(MLG_ENOKIT, "transformation kit is not initialized");
  Scalar *p = reinterpret_cast<Scalar*>(psi), *c = reinterpret_cast<Scalar*>(chi);
  if (!p || !c || !p->e || !c->e || !E) return set_error(MLG_EHANDLE, "invalid scalar handle");
  return op_ke_spectrum(*p, *c, E);
}

}  // extern "C"
