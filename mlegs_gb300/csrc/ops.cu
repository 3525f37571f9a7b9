// ops.cu — the scalar operator API of the reference (module mlegs_scalar, mlegs_scalar_ops.f90) on
// device-resident fields, and the 3-D vortex step of src/apps/vortical_flow_3d.f90.  Host code keeps
// the reference's control flow (space state machine, chop offsets, per-routine order of work); all
// field arithmetic runs in the kernels of this file, fft.cu, radial.cu and banded.cu.  The log-term
// coefficient ln of every field lives in device memory, so no step needs a host round trip.
#include "common.cuh"
#include <cmath>
#include <mutex>
#include <algorithm>

namespace mlg {

Ctx G;
static std::string g_err;

int set_error(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int dmalloc(void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(MLG_EALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  G.mem_bytes += (long long)bytes;
  G.mem_high = std::max(G.mem_high, G.mem_bytes);
  return 0;
}
void dfree(void* p, size_t bytes) {
  if (p) cudaFree(p);
  G.mem_bytes -= (long long)bytes;
}

cd* get_buf() {
  if (!G.pool.empty()) {
    cd* b = G.pool.back();
    G.pool.pop_back();
    return b;
  }
  cd* b = nullptr;
  if (dmalloc((void**)&b, G.fsize * sizeof(cd))) return nullptr;
  G.all_bufs.push_back(b);
  return b;
}
void put_buf(cd* b) {
  if (b) G.pool.push_back(b);
}
int pool_reserve(int n) {
  std::vector<cd*> t;
  for (int i = 0; i < n; ++i) {
    cd* b = get_buf();
    if (!b) return MLG_EALLOC;
    t.push_back(b);
  }
  for (cd* b : t) put_buf(b);
  return 0;
}

int side_fork() {
  MLG_CUDA(cudaEventRecord(G.ev_fork, G.stream));
  MLG_CUDA(cudaStreamWaitEvent(G.side, G.ev_fork, 0));
  return 0;
}
int side_join() {
  MLG_CUDA(cudaEventRecord(G.ev_join, G.side));
  MLG_CUDA(cudaStreamWaitEvent(G.stream, G.ev_join, 0));
  return 0;
}

void kt_begin(int kind) {
  if (!G.kt.on) return;
  (void)kind;
  cudaEventRecord(G.ev0, G.stream);
}
void kt_end(int kind, double work) {
  if (!G.kt.on) return;
  cudaEventRecord(G.ev1, G.stream);
  cudaEventSynchronize(G.ev1);
  float ms = 0;
  cudaEventElapsedTime(&ms, G.ev0, G.ev1);
  G.kt.ms[kind] += ms;
  G.kt.n[kind] += 1;
  G.kt.work[kind] += work;
}

int chop_index(const Scalar& s, ChopIdx& c) {
  c.nrc = G.nrchop + s.off[0];
  c.npc = G.npchop + s.off[1];
  c.nzc = G.chopzl + s.off[2];
  c.nzcu = G.chopzu - s.off[2];
  if (c.nrc > G.nrdim) return set_error(MLG_ECHOP, "chop_index: chopping in r too large");
  if (c.npc > G.npdim) return set_error(MLG_ECHOP, "chop_index: chopping in p too large");
  if (2 * s.off[2] > c.nzcu - c.nzc) return set_error(MLG_ECHOP, "chop_index: chopping in z too large");
  if (c.nrc > G.ne) return set_error(MLG_ECHOP, "chop_index: chopping in r beyond the Legendre table");
  return 0;
}

int launch_band_apply(Scalar& s, int op, const ChopIdx& c);
int launch_band_solve(Scalar& s, int kind, const ChopIdx& c, double alpha, double beta, double preln, int power);
int launch_ihelmp_pre(Scalar& s, const ChopIdx& c, int power, double alpha, double beta);

// ------------------------------------------------------------------------------------------------
// pointwise kernels

// chop (mlegs_scalar_ops.f90:6-41) and dealias (:43-70) as masks
// one warp per (m, k) column (8 per block): the column's first zeroed row is worked out once, and
// only the zeroed rows are written (a column that keeps all its rows touches no memory)
// chop (:6-41) and / or dealias (:43-70) of up to six fields with the same chop window and space, one
// warp per column: rows [zf, nrdim) of a column become zero, zf = 0 for a column the dealias band or the
// chop's m / k window removes whole, the chop's nn(m) otherwise
struct MaskSet {
  double2* e[6];
  int n;
  double* lnz[2];   // ln slots set to zero by the launch (or null): a field's ln reset folded into its mask
};
__global__ void __launch_bounds__(256) k_mask(MaskSet fs, int nrdim, int npdim, int nzdim, int chop, int dealias, int f0,
                                              int f1, int f2, int nrc, int npc, int nzc, int nzcu, int pcut, int zcut,
                                              int zupper, int np_gt1, int nz_gt1) {
  const int cf = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  const int ncols = npdim * nzdim;
  if (blockIdx.x == 0 && threadIdx.x < 2 && fs.lnz[threadIdx.x]) *fs.lnz[threadIdx.x] = 0.0;
  if (cf >= fs.n * ncols) return;
  const int f = cf / ncols, col = cf - f * ncols;
  double2* e = fs.e[0];
#pragma unroll
  for (int q = 1; q < 6; ++q)
    if (f == q) e = fs.e[q];
  const int m = col % npdim, k = col / npdim;
  int zf = nrdim;   // rows [zf, nrdim) become zero
  if (chop) {
    if ((f1 && m >= npc) || (f2 && nzc < nzcu && (k + 1) >= nzc + 1 && (k + 1) <= nzcu - 1)) zf = 0;
    else if (f0) zf = (m < npc) ? max(min(nrc, nrc - m), 0) : 0;
  }
  if (dealias && ((np_gt1 && f1 && (m + 1) > pcut) || (nz_gt1 && f2 && (k + 1) > zcut && (k + 1) < zupper))) zf = 0;
  double2* g = e + (size_t)nrdim * col;
  for (int i = zf + lane; i < nrdim; i += 32) g[i] = make_double2(0.0, 0.0);
}

// e(:nr, 1, :) += sgn * ln * lnx (trans :193-195, :219-221)
__global__ void k_ln_adjust(double2* __restrict__ e, const double* __restrict__ lnp, const double* __restrict__ lnx,
                            int nr, int nrdim, int npdim, int nzdim, double sgn) {
  double l = *lnp;
  if (l == 0.0) return;
  size_t n = (size_t)nr * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nr);
    int k = (int)(idx / (unsigned)nr);
    e[i + (size_t)nrdim * npdim * k].x += sgn * l * lnx[i];
  }
}

// one linear combination (LinArgs) over a field
__global__ void k_lincomb(LinArgs a) {
  const bool scaled = a.post != 1.0;   // multiplying by 1 changes nothing: skipped
  GRID_STRIDE(idx, a.n) {
    double2 acc = make_double2(0, 0);
    bool first = true;
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (a.in[t]) {
        double2 v = a.in[t][idx];
        if (first) { acc.x = a.c[t] * v.x; acc.y = a.c[t] * v.y; first = false; }   // 0 + c v, exactly
        else { acc.x += a.c[t] * v.x; acc.y += a.c[t] * v.y; }
      }
    a.out[idx] = scaled ? make_double2(a.post * acc.x, a.post * acc.y) : acc;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && a.lnout) {
    double l = 0.0;
    for (int t = 0; t < 4; ++t)
      if (a.lnin[t]) l += a.lc[t] * *a.lnin[t];
    *a.lnout = a.post * l;
  }
}

// up to four independent linear combinations (no combination reads another one's output) in one
// launch, each exactly as k_lincomb computes it
struct LinSet {
  LinArgs a[4];
  int n;
};
__global__ void k_lincomb_n(LinSet s) {
  const size_t n = s.a[0].n;
  GRID_STRIDE(gidx, n * s.n) {
    const int q = (int)(gidx / n);
    const size_t idx = gidx - (size_t)q * n;
    const LinArgs& a = q == 0 ? s.a[0] : (q == 1 ? s.a[1] : (q == 2 ? s.a[2] : s.a[3]));
    const bool scaled = a.post != 1.0;
    double2 acc = make_double2(0, 0);
    bool first = true;
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (a.in[t]) {
        double2 v = a.in[t][idx];
        if (first) { acc.x = a.c[t] * v.x; acc.y = a.c[t] * v.y; first = false; }
        else { acc.x += a.c[t] * v.x; acc.y += a.c[t] * v.y; }
      }
    a.out[idx] = scaled ? make_double2(a.post * acc.x, a.post * acc.y) : acc;
  }
  if (blockIdx.x == 0 && threadIdx.x < (unsigned)s.n) {
    const LinArgs& a = threadIdx.x == 0 ? s.a[0] : (threadIdx.x == 1 ? s.a[1] : (threadIdx.x == 2 ? s.a[2] : s.a[3]));
    if (a.lnout) {
      double l = 0.0;
      for (int t = 0; t < 4; ++t)
        if (a.lnin[t]) l += a.lc[t] * *a.lnin[t];
      *a.lnout = a.post * l;
    }
  }
}

// calcat (mlegs_scalar_ops.f90:237-309): calc(k) = sum_n e(n, 1, k) * at(n); zeroat1 (:311-325)
// additionally subtracts calc(k)/at1(1) from e(1, 1, k).  One warp per k.
__global__ void k_calcat(double2* __restrict__ e0, double2* __restrict__ e1, const double* __restrict__ at, int nmax,
                         int nrdim, int npdim, int nzdim, double2* __restrict__ out, int zero_mode) {
  // one warp per k of e0 and, when e1 is given, of e1; the values at the point go to out from the last
  // field (what two calls one after the other leave there)
  const int kf = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (kf >= (e1 ? 2 : 1) * nzdim) return;
  const int k = kf < nzdim ? kf : kf - nzdim;
  if (e1 && kf < nzdim) out = nullptr;
  double2* col = (kf < nzdim ? e0 : e1) + (size_t)nrdim * npdim * k;
  double sx = 0, sy = 0;
  for (int n = lane; n < nmax; n += 32) { double2 v = col[n]; sx += v.x * at[n]; sy += v.y * at[n]; }
  for (int o = 16; o; o >>= 1) { sx += __shfl_xor_sync(0xffffffffu, sx, o); sy += __shfl_xor_sync(0xffffffffu, sy, o); }
  if (lane == 0) {
    if (out) out[k] = make_double2(sx, sy);
    if (zero_mode) { col[0].x -= sx / at[0]; col[0].y -= sy / at[0]; }
  }
}

// the projection's log-term bookkeeping in one launch: psi%ln = f Re(calcat1(up)(1)) with f = -1/2
// (:1366-1367, from the calcat output of k = 1), up(:nr,1,1) += psi%ln (1 + x) (:1371-1373) and
// chi%ln = 0 (:1331)
__global__ void k_proj_ln(double2* __restrict__ e, const double2* __restrict__ calc, double f, double* __restrict__ psiln,
                          double* __restrict__ chiln, const double* __restrict__ x, int nr) {
  const double l = f * calc[0].x;
  if (threadIdx.x == 0) { *psiln = l; *chiln = 0.0; }
  for (int i = threadIdx.x; i < nr; i += blockDim.x) e[i].x += l * (1.0 + x[i]);
}

// e(:nr, :, :) *= r (rows scaled by the table passed: r, or 1/r for the division of tp2vec)
__global__ void k_scale_r(double2* __restrict__ e, const double* __restrict__ r, int nr, int nrdim, size_t ncol) {
  size_t n = (size_t)nr * ncol;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nr);
    unsigned c = idx / (unsigned)nr;
    double2* p = e + i + (size_t)nrdim * c;
    double v = r[i];
    p->x *= v; p->y *= v;
  }
}

// vecprod (mlegs_scalar_ops.f90:1264-1306) on the packed reals; everything else zero
// v x u on the packed samples; vzb (optional): a field added to vz first (the background axial flow of
// advection_rhs, vortical_flow_3d.f90:371, with the rounding of that separate addition)
__global__ void k_vecprod(double2* vr, double2* vp, double2* vz, const double2* __restrict__ ur,
                          const double2* __restrict__ up, const double2* __restrict__ uz, const double2* __restrict__ vzb,
                          double2* o_r, double2* o_p, double2* o_z, int nr, int nph, int nrdim, int npdim, int nzdim) {
  size_t n = (size_t)nrdim * npdim * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int m = (int)((idx / (unsigned)nrdim) % (unsigned)npdim);
    double2 o1 = make_double2(0, 0), o2 = o1, o3 = o1;
    if (i < nr && m < nph) {
      double2 A1 = vr[idx], A2 = vp[idx], A3 = vz[idx], B1 = ur[idx], B2 = up[idx], B3 = uz[idx];
      if (vzb) { double2 b = vzb[idx]; A3 = make_double2(A3.x + b.x, A3.y + b.y); }
      o1 = make_double2(A2.x * B3.x - A3.x * B2.x, A2.y * B3.y - A3.y * B2.y);
      o2 = make_double2(A3.x * B1.x - A1.x * B3.x, A3.y * B1.y - A1.y * B3.y);
      o3 = make_double2(A1.x * B2.x - A2.x * B1.x, A1.y * B2.y - A2.y * B1.y);
    }
    o_r[idx] = o1; o_p[idx] = o2; o_z[idx] = o3;   // in place when the outputs are (vr, vp, vz)
  }
}

// svv_filter (mlegs_scalar_ops.f90:72-155).  q = min(1, max(q_r(n), q_p(m), q_z(k))) with cutoff < 1,
// so "q >= cutoff" is "any of the three >= cutoff", and since the filter exp(-s*shape(q)^8) decreases
// in q, its value at the maximum is the minimum of its values at q_r, q_p, q_z: the per-element work
// reduces to 1-D tables (filled once per call) and a min.
__device__ __forceinline__ double svv_qr(int i, int nrchop) {
  return fmin(1.0, (double)max(i, 0) / fmax((double)(nrchop - 1), 1.0));
}
__device__ __forceinline__ double svv_qp(int m, int np) { return fmin(1.0, (double)abs(m) / fmax((double)(np / 2), 1.0)); }
__device__ __forceinline__ double svv_qz(int k, const double* ak, int nak, double kmax) {
  int gk = k + 1;
  double kv = (gk >= 1 && gk <= nak) ? fabs(ak[k]) : 0.0;
  return fmin(1.0, kv / kmax);
}
// per block: the energy of the head and of the tail (q >= cutoff) of the spectrum (:112-117).  The q
// are in [0, 1], so q >= cutoff is compared on the FP64 bit patterns; the sums stay FP64.
// blockIdx.y = field (e0, e1: the two fields of a paired call, or one field twice with gridDim.y = 1)
__global__ void __launch_bounds__(256, 8) k_svv_sums(const double2* __restrict__ e0, const double2* __restrict__ e1,
                                                  int nrdim, int npdim, int nzdim, const double* __restrict__ qt,
                                                  unsigned long long cbits, double* __restrict__ partial) {
  const double2* __restrict__ e = blockIdx.y ? e1 : e0;
  partial += (size_t)blockIdx.y * 2 * gridDim.x;
  // a warp per column (m, k), its lanes over the rows; |e|^2 summed in FP64 into the head (q below the
  // cutoff) and the tail.  q of a row rises with the row (svv_qr), so the rows below the cutoff are
  // the first nc: a column whose m or k is at or above the cutoff goes to the tail whole, any other
  // splits at row nc, and no element needs a predicated FP64 add.
  __shared__ double s0[8], s1[8];
  const unsigned long long* qb = reinterpret_cast<const unsigned long long*>(qt);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int ncol = npdim * nzdim;
  int nc = 0;
  for (int i0 = 0; i0 < nrdim; i0 += 32) {
    const int i = i0 + lane;
    nc += __popc(__ballot_sync(0xffffffffu, i < nrdim && qb[i] < cbits));
  }
  double head = 0, tail = 0;
  for (int c = blockIdx.x * 8 + wib; c < ncol; c += gridDim.x * 8) {
    const int m = c % npdim, k = c / npdim;
    const unsigned long long bm = qb[nrdim + m], bk = qb[nrdim + npdim + k];
    const int split = (bm >= cbits || bk >= cbits) ? 0 : nc;
    const double2* col = e + (size_t)nrdim * c;
    for (int i = lane; i < split; i += 32) {
      const double2 v = col[i];
      head += v.x * v.x + v.y * v.y;
    }
    for (int i = split + lane; i < nrdim; i += 32) {
      const double2 v = col[i];
      tail += v.x * v.x + v.y * v.y;
    }
  }
  for (int o = 16; o; o >>= 1) {
    head += __shfl_xor_sync(0xffffffffu, head, o);
    tail += __shfl_xor_sync(0xffffffffu, tail, o);
  }
  if (lane == 0) { s0[wib] = head; s1[wib] = tail; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double h = 0, t = 0;
    for (int w = 0; w < 8; ++w) { h += s0[w]; t += s1[w]; }
    partial[2 * blockIdx.x] = h;
    partial[2 * blockIdx.x + 1] = t;
  }
}
// gain relaxation and strength (:119-126) and the 1-D factor tables ft[0..nrdim) (n), ft[nrdim..+npdim)
// (m), ft[..+nzdim) (k): exp(-s*shape^8) where q > cutoff, 1 elsewhere.  Every block reduces the
// partial sums (a tree over its threads) and fills its share of the tables; block 0 stores the
// strength in st[0] and the new gain in st[1] (copied to the gain by k_svv_apply: no block may see
// a half-updated gain)
// blockIdx.y = field: its partial sums, gain, st pair and factor tables
__global__ void k_svv_gain(const double* __restrict__ partial, int nb, const double* __restrict__ gain,
                           double* __restrict__ st, double target, double relax, double strength_max,
                           double* __restrict__ ft, int nrdim, int npdim, int nzdim, int nrchop, int np, double kmax,
                           const double* __restrict__ ak, double cutoff) {
  partial += (size_t)blockIdx.y * 2 * nb;
  gain += blockIdx.y;
  st += 2 * blockIdx.y;
  ft += (size_t)blockIdx.y * (nrdim + npdim + nzdim);
  __shared__ double r0[256], r1[256];
  __shared__ double str;
  double h = 0, t = 0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) { h += partial[2 * b]; t += partial[2 * b + 1]; }
  r0[threadIdx.x] = h; r1[threadIdx.x] = t;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if (threadIdx.x < o) { r0[threadIdx.x] += r0[threadIdx.x + o]; r1[threadIdx.x] += r1[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double tail = r1[0], tot = r0[0] + tail;
    double g = *gain, sv = 0.0;
    if (tot > 2.2250738585072014e-308) {
      double ratio = tail / tot;
      double fb = fmin(fmax(ratio / target - 1.0, 0.0), 1.0);
      double rl = fmin(fmax(relax, 0.0), 1.0);
      g = (1.0 - rl) * g + rl * fb;
      sv = fmin(fmax(strength_max, 0.0) * g, 1.0);
    }
    if (blockIdx.x == 0) { st[0] = sv; st[1] = g; }
    str = sv;
  }
  __syncthreads();
  double sv = str;
  int ntot = nrdim + npdim + nzdim;
  for (int tt = blockIdx.x * blockDim.x + threadIdx.x; tt < ntot; tt += gridDim.x * blockDim.x) {
    double q = (tt < nrdim) ? svv_qr(tt, nrchop) : (tt < nrdim + npdim) ? svv_qp(tt - nrdim, np)
                                                                          : svv_qz(tt - nrdim - npdim, ak, nzdim, kmax);
    q = fmin(1.0, q);
    double f = 1.0;
    if (sv > 0.0 && q > cutoff) {
      double shape = (q - cutoff) / (1.0 - cutoff);
      double s2 = shape * shape, s4 = s2 * s2;
      f = exp(-sv * (s4 * s4));
    }
    ft[tt] = f;
  }
}
// q_r, q_p, q_z of every row, azimuthal slot and axial slot (:96-110), filled once
__global__ void k_svv_qtab(double* __restrict__ qt, int nrdim, int npdim, int nzdim, int nrchop, int np, double kmax,
                           const double* __restrict__ ak) {
  int ntot = nrdim + npdim + nzdim;
  for (int t = threadIdx.x; t < ntot; t += blockDim.x)
    qt[t] = (t < nrdim) ? svv_qr(t, nrchop) : (t < nrdim + npdim) ? svv_qp(t - nrdim, np)
                                                                 : svv_qz(t - nrdim - npdim, ak, nzdim, kmax);
}
// blockIdx.y = field, as in k_svv_gain
__global__ void k_svv_apply(double2* __restrict__ e0, double2* __restrict__ e1, int nrdim, int npdim, int nzdim,
                            const double* __restrict__ st, const double* __restrict__ ft, double* __restrict__ gain) {
  double2* __restrict__ e = blockIdx.y ? e1 : e0;
  st += 2 * blockIdx.y;
  ft += (size_t)blockIdx.y * (nrdim + npdim + nzdim);
  gain += blockIdx.y;
  if (blockIdx.x == 0 && threadIdx.x == 0) *gain = st[1];
  if (st[0] <= 0.0) return;
  size_t n = (size_t)nrdim * npdim * nzdim;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int m = (int)((idx / (unsigned)nrdim) % (unsigned)npdim);
    int k = (int)(idx / (unsigned)(nrdim * npdim));
    double f = fmin(ft[i], fmin(ft[nrdim + m], ft[nrdim + npdim + k]));
    if (f != 1.0) {
      double2 v = e[idx];
      e[idx] = make_double2(f * v.x, f * v.y);
    }
  }
}

// delsqp (:327-366) / idelsqp (:368-416), elementwise in place on the active rows of every k;
// the ln-dependent entry (1,1,1) and the (1,1,:) reset are applied by the same thread.
__global__ void k_delsqp(double2* __restrict__ e, const double* __restrict__ lnp, const double* __restrict__ lognorm,
                         int inverse, int nrdim, int npdim, int nzdim, int nrc, int npc, double ell) {
  size_t n = (size_t)nrdim * npdim * nzdim;
  double e2 = ell * ell;
  GRID_STRIDE(idx, n) {
    int i = (int)(idx % (unsigned)nrdim);
    int m = (int)((idx / (unsigned)nrdim) % (unsigned)npdim);
    int nrcs = (m < npc) ? max(min(nrc, nrc - m), 0) : 0;
    double2 v = e[idx];
    if (i < nrcs) {
      int in_ = m + i;
      double dn = (double)in_;
      if (!inverse) {
        v.x = -v.x * dn * (dn + 1.0) / e2;
        v.y = -v.y * dn * (dn + 1.0) / e2;
      } else if (in_ == 0) {
        v = make_double2(0, 0);
      } else {
        v.x = -v.x / (double)in_ / (in_ + 1.0) * e2;
        v.y = -v.y / (double)in_ / (in_ + 1.0) * e2;
      }
    }
    if (!inverse && idx == 0) v = make_double2(*lnp / e2 / exp(lognorm[0]), 0.0);
    if (inverse && i == 0 && m == 0) v = make_double2(0, 0);
    e[idx] = v;
  }
}
__global__ void k_idelsqp_ln(const double2* __restrict__ e, double* __restrict__ lnp, const double* __restrict__ lognorm,
                             double ell) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *lnp = e[0].x * pow(ell, 2.0) * exp(lognorm[0]);
}
__global__ void k_ln_zero(double* __restrict__ lnp) { if (threadIdx.x == 0) *lnp = 0.0; }
__global__ void k_ln_set(double* __restrict__ lnp, double v) { if (threadIdx.x == 0) *lnp = v; }
__global__ void k_ln_set2(double* __restrict__ a, double* __restrict__ b, double v) {
  if (threadIdx.x == 0) *a = v;
  if (threadIdx.x == 1) *b = v;
}
__global__ void k_ln_copy(double* __restrict__ d, const double* __restrict__ s) { if (threadIdx.x == 0) *d = *s; }

// field copy that also carries the ln slot (assignment(=), mlegs_scalar_init.f90:106-140)
__global__ void k_copy_scalar(double2* __restrict__ d, const double2* __restrict__ s, size_t n, double* __restrict__ dln,
                              const double* __restrict__ sln) {
  GRID_STRIDE(idx, n) d[idx] = s[idx];
  if (blockIdx.x == 0 && threadIdx.x == 0) *dln = *sln;
}

// non-finite (inf or NaN) from the exponent bits, on the integer pipe
__device__ __forceinline__ unsigned nonfinite_bits(double x) {
  return (unsigned)((__double2hiint(x) & 0x7FF00000) == 0x7FF00000);
}
__global__ void k_finite(const double2* __restrict__ a, const double2* __restrict__ b, size_t n, int* __restrict__ flag) {
  GRID_STRIDE(idx, n) {
    const double2 u = a[idx], v = b[idx];
    if (nonfinite_bits(u.x) | nonfinite_bits(u.y) | nonfinite_bits(v.x) | nonfinite_bits(v.y)) atomicExch(flag, 1);
  }
}

// ------------------------------------------------------------------------------------------------
// launch helpers
int launch_zero(cd* e) { MLG_CUDA(cudaMemsetAsync(e, 0, G.fsize * sizeof(cd), G.stream)); return 0; }
int launch_copy(cd* d, const cd* s) {
  if (d != s) MLG_CUDA(cudaMemcpyAsync(d, s, G.fsize * sizeof(cd), cudaMemcpyDeviceToDevice, G.stream));
  return 0;
}
int launch_copy_ln(double* d, const double* s) {
  if (d != s) { k_ln_copy<<<1, 32, 0, G.stream>>>(d, s); MLG_LAUNCH(); }
  return 0;
}
int launch_set_ln(double* d, double v) { k_ln_set<<<1, 32, 0, G.stream>>>(d, v); MLG_LAUNCH(); return 0; }
int launch_set_ln2(double* a, double* b, double v) { k_ln_set2<<<1, 32, 0, G.stream>>>(a, b, v); MLG_LAUNCH(); return 0; }
struct LnSet {
  double* p[6];
  int n;
};
__global__ void k_ln_setn(LnSet s, double v) {
  const int t = threadIdx.x;
  double* d = s.p[0];
#pragma unroll
  for (int q = 1; q < 6; ++q)
    if (t == q) d = s.p[q];
  if (t < s.n) *d = v;
}
int launch_set_ln_n(double* const* d, int n, double v) {
  if (n < 1 || n > 6) return set_error(MLG_EPARAM, "set_ln: one to six slots per launch");
  LnSet s{};
  for (int i = 0; i < n; ++i) s.p[i] = d[i];
  s.n = n;
  k_ln_setn<<<1, 32, 0, G.stream>>>(s, v);
  MLG_LAUNCH();
  return 0;
}

int launch_ln_adjust(Scalar& s, double sign) {
  size_t n = (size_t)G.nr * G.nzdim;
  k_ln_adjust<<<nblk(n), 256, 0, G.stream>>>(s.e, s.ln, G.lnx, G.nr, G.nrdim, G.npdim, G.nzdim, sign);
  MLG_LAUNCH();
  return 0;
}

LinArgs lin_args(Scalar& out, std::initializer_list<std::pair<const Scalar*, double>> terms,
                 std::initializer_list<std::pair<const Scalar*, double>> lnterms, double post, bool do_ln) {
  LinArgs a{};
  a.out = out.e;
  a.n = G.fsize;
  a.post = post;
  int t = 0;
  for (auto& p : terms) { a.in[t] = p.first ? p.first->e : nullptr; a.c[t] = p.second; ++t; }
  for (; t < 4; ++t) { a.in[t] = nullptr; a.c[t] = 0; }
  t = 0;
  a.lnout = do_ln ? out.ln : nullptr;
  for (auto& p : lnterms) { a.lnin[t] = p.first ? p.first->ln : nullptr; a.lc[t] = p.second; ++t; }
  for (; t < 4; ++t) { a.lnin[t] = nullptr; a.lc[t] = 0; }
  return a;
}
int lincomb(Scalar& out, std::initializer_list<std::pair<const Scalar*, double>> terms,
            std::initializer_list<std::pair<const Scalar*, double>> lnterms, double post, bool do_ln) {
  LinArgs a = lin_args(out, terms, lnterms, post, do_ln);
  k_lincomb<<<nblk(G.fsize), 256, 0, G.stream>>>(a);
  MLG_LAUNCH();
  return 0;
}
int lincomb_n(std::initializer_list<LinArgs> combos) {
  if (combos.size() < 1 || combos.size() > 4) return set_error(MLG_EPARAM, "lincomb: one to four combinations per launch");
  LinSet s{};
  for (const LinArgs& a : combos) s.a[s.n++] = a;
  k_lincomb_n<<<nblk(G.fsize * s.n), 256, 0, G.stream>>>(s);
  MLG_LAUNCH();
  return 0;
}

// ------------------------------------------------------------------------------------------------
// scalar bookkeeping
static int alloc_slot() {
  if (G.free_slots.empty()) return -1;
  int s = G.free_slots.back();
  G.free_slots.pop_back();
  return s;
}
static void free_slot(int s) { if (s >= 0) G.free_slots.push_back(s); }

int scalar_init(Scalar& s, bool zero_ln) {   // scalar_init (mlegs_scalar_init.f90:6-67): space PPP
  s.e = get_buf();
  if (!s.e) return set_error(MLG_EALLOC, "scalar_init: out of device memory");
  s.slot = alloc_slot();
  if (s.slot < 0) { put_buf(s.e); s.e = nullptr; return set_error(MLG_ESIZE, "scalar_init: too many scalars"); }
  s.ln = G.ln_slots + s.slot;
  s.set_space("PPP");
  s.off[0] = s.off[1] = s.off[2] = 0;
  if (zero_ln) MLG_TRY(launch_set_ln(s.ln, 0.0));
  return 0;
}
void scalar_release(Scalar& s) {
  put_buf(s.e);
  s.e = nullptr;
  free_slot(s.slot);
  s.slot = -1;
  s.ln = nullptr;
}
// scalar_copy (mlegs_scalar_init.f90:106-140)
int assign(Scalar& d, const Scalar& s) {
  if (d.e != s.e) {
    k_copy_scalar<<<nblk(G.fsize), 256, 0, G.stream>>>(d.e, s.e, G.fsize, d.ln, s.ln);
    MLG_LAUNCH();
  } else {
    MLG_TRY(launch_copy_ln(d.ln, s.ln));
  }
  std::memcpy(d.space, s.space, 4);
  for (int i = 0; i < 3; ++i) d.off[i] = s.off[i];
  return 0;
}


// ------------------------------------------------------------------------------------------------
// operators (mlegs_scalar_ops.f90)
static int space_code(const char* sp) {
  if (!std::strncmp(sp, "PPP", 3)) return 0;
  if (!std::strncmp(sp, "PFP", 3)) return 1;
  if (!std::strncmp(sp, "FFP", 3)) return 2;
  if (!std::strncmp(sp, "FFF", 3)) return 3;
  return -1;
}

static int vfft_check(const Scalar& s, int dir) {
  int nzc = G.chopzl + s.off[2], nzcu = G.chopzu - s.off[2];
  if (2 * s.off[2] > nzcu - nzc)
    return set_error(MLG_ECHOP, dir < 0 ? "vertical_fft_forward: chopping in z too large" : "vertical_fft_backward: chopping in z too large");
  return 0;
}
static int vfft_checked(Scalar& s, int dir) {
  MLG_TRY(vfft_check(s, dir));
  return launch_vfft(s, dir);
}

// trans (:157-235)
int ihelm_noalloc(void* e_dev, double* ln, double alpha);

int op_trans(Scalar& s, const char* space) {
  int cur = space_code(s.space);
  if (cur < 0) return set_error(MLG_ESPACE, "trans: scalar space info corrupted (only accepting PPP, PFP, FFP and FFF)");
  int nw = space_code(space);
  if (nw < 0) return set_error(MLG_ESPACE, "trans: only taking PPP, PFP, FFP and FFF for spectral transformation");
  if (cur < nw) {
    while (true) {
      if (cur == 0) { if (G.np > 1) MLG_TRY(launch_hfft(s, -1)); s.set_space("PFP"); }
      if (cur == 1) { MLG_TRY(launch_ln_adjust(s, -1.0)); MLG_TRY(launch_rtrans_fwd(s)); s.set_space("FFP"); }
      if (cur == 2) { if (G.nz > 1) MLG_TRY(vfft_checked(s, -1)); s.set_space("FFF"); }
      if (cur == 3) break;
      cur++;
      if (cur == nw) break;
    }
  }
  if (cur > nw) {
    while (true) {
      if (cur == 3) { if (G.nz > 1) MLG_TRY(vfft_checked(s, +1)); s.set_space("FFP"); }
      if (cur == 2) { MLG_TRY(launch_rtrans_bwd(s, true)); s.set_space("PFP"); }
      if (cur == 1) { if (G.np > 1) MLG_TRY(launch_hfft(s, +1)); s.set_space("PPP"); }
      if (cur == 0) break;
      cur--;
      if (cur == nw) break;
    }
  }
  return 0;
}

// chop and / or dealias of n <= 6 fields (the first field's chop window and space stand for all)
static int mask_launch(Scalar* const* f, int n, bool chop, bool dealias, const ChopIdx& c, double* lnz0 = nullptr,
                       double* lnz1 = nullptr) {
  MaskSet fs{};
  for (int i = 0; i < n; ++i) fs.e[i] = f[i]->e;
  fs.n = n;
  fs.lnz[0] = lnz0;
  fs.lnz[1] = lnz1;
  const Scalar& s = *f[0];
  int pcut = std::max(G.np / 3 + 1, 1), zcut = std::max(G.nz / 3 + 1, 1), zupper = G.nz - zcut + 2;
  k_mask<<<cdiv((long long)n * G.npdim * G.nzdim, 8), 256, 0, G.stream>>>(
      fs, G.nrdim, G.npdim, G.nzdim, chop ? 1 : 0, dealias ? 1 : 0, s.space[0] == 'F', s.space[1] == 'F', s.space[2] == 'F',
      c.nrc, c.npc, c.nzc, c.nzcu, pcut, zcut, zupper, G.np > 1, G.nz > 1);
  MLG_LAUNCH();
  return 0;
}
// fields that one launch can take together: distinct, the same space and chop window
static bool mask_batchable(Scalar* const* f, int n, bool chop, ChopIdx& c) {
  ChopIdx c0{};
  if (chop && chop_index(*f[0], c0)) return false;   // the one-by-one path reports the error
  for (int i = 1; i < n; ++i) {
    if (std::strncmp(f[i]->space, f[0]->space, 3) != 0) return false;
    for (int j = 0; j < i; ++j)
      if (f[i]->e == f[j]->e) return false;
    if (chop) {
      ChopIdx ci;
      if (chop_index(*f[i], ci)) return false;
      if (ci.nrc != c0.nrc || ci.npc != c0.npc || ci.nzc != c0.nzc || ci.nzcu != c0.nzcu) return false;
    }
  }
  c = c0;
  return true;
}
// chop (if chop) and then dealias (if dealias) of each of n <= 6 fields, in one launch where they can
// share it
int op_mask_n(Scalar* const* f, int n, bool chop, bool dealias) {
  if (n < 1 || n > 6) return set_error(MLG_EPARAM, "mask: one to six fields per launch");
  ChopIdx c{};
  if (mask_batchable(f, n, chop, c)) return mask_launch(f, n, chop, dealias, c);
  for (int i = 0; i < n; ++i) {
    ChopIdx ci{};
    if (chop) MLG_TRY(chop_index(*f[i], ci));
    MLG_TRY(mask_launch(&f[i], 1, chop, dealias, ci));
  }
  return 0;
}
int op_chop(Scalar& s) {
  Scalar* f[1] = {&s};
  return op_mask_n(f, 1, true, false);
}
int op_chop2(Scalar& a, Scalar& b) {
  Scalar* f[2] = {&a, &b};
  return op_mask_n(f, 2, true, false);
}
int op_dealias(Scalar& s) {
  Scalar* f[1] = {&s};
  return op_mask_n(f, 1, false, true);
}
int op_dealias2(Scalar& a, Scalar& b) {
  Scalar* f[2] = {&a, &b};
  return op_mask_n(f, 2, false, true);
}
// a%ln = 0, b%ln = 0, then dealias(a), dealias(b): the ln resets ride on the mask launch
static int op_zero_ln_dealias2(Scalar& a, Scalar& b) {
  Scalar* f[2] = {&a, &b};
  ChopIdx c{};
  if (mask_batchable(f, 2, false, c)) return mask_launch(f, 2, false, true, c, a.ln, b.ln);
  MLG_TRY(launch_set_ln2(a.ln, b.ln, 0.0));
  return op_dealias2(a, b);
}

// svv_filter with the gain kept in device memory (gain_dev)
// svv_filter (:72-155) of one field, or of two with their own gains in one set of launches (the psi and
// chi filters of a vortex step: gain_dev[0] and gain_dev[1]); the results are those of separate calls
static int svv_filter_fields(Scalar* const* f, int nf, double* gain_dev) {
  if (!G.P.is_svv) return 0;
  for (int i = 0; i < nf; ++i)
    if (!f[i]->is("FFF")) return set_error(MLG_ESPACE, "svv_filter: scalar must be in FFF space");
  double cutoff = std::min(std::max(G.P.svv_cutoff, 0.0), 0.99);
  double target = std::max(G.P.svv_target, 1.0e-12);
  // kmax = max(maxval(abs(ak)), 1) over the kit's ak (mlegs_spectfm_init.f90:132-134)
  double kmax = 0.0;
  {
    std::vector<double> ak(G.nz);
    for (int i = -G.nz; i <= -1; ++i) ak[i + G.nz] = 2.0 * 3.14159265358979323846 / G.P.zlen * i;
    for (int i = 0; i <= G.nz / 2; ++i) ak[i] = 2.0 * 3.14159265358979323846 / G.P.zlen * i;
    for (double a : ak) kmax = std::max(kmax, std::fabs(a));
    kmax = std::max(kmax, 1.0);
  }
  // scratch: the partial sums [field][NB][2], the factor tables [field][ntab], the q table [ntab]; the
  // strength and new gain of field i at DS_SUM0 + 2 i
  const int NB = 304;
  const int ntab = G.nrdim + G.npdim + G.nzdim;
  double* partial = G.dscal + DS_CALC + 2 * 2048;
  double* ft = partial + 2 * 2 * NB;
  double* qt = ft + 2 * ntab;
  if (DS_CALC + 2 * 2048 + 4 * NB + 3 * ntab > DS_COUNT)
    return set_error(MLG_ESIZE, "svv_filter: grid too large for the filter tables");
  if (!G.svv_q_ready) {
    k_svv_qtab<<<1, 256, 0, G.stream>>>(qt, G.nrdim, G.npdim, G.nzdim, G.nrchop, G.np, kmax, G.ak);
    MLG_LAUNCH();
    G.svv_q_ready = true;
  }
  unsigned long long cbits = 0;
  std::memcpy(&cbits, &cutoff, sizeof(cbits));
  double2* e0 = f[0]->e;
  double2* e1 = f[nf - 1]->e;
  k_svv_sums<<<dim3(NB, nf), 256, 0, G.stream>>>(e0, e1, G.nrdim, G.npdim, G.nzdim, qt, cbits, partial);
  MLG_LAUNCH();
  k_svv_gain<<<dim3(std::max(1, std::min(8, cdiv(ntab, 64))), nf), 256, 0, G.stream>>>(
      partial, NB, gain_dev, G.dscal + DS_SUM0, target, G.P.svv_relax, G.P.svv_strength, ft, G.nrdim, G.npdim, G.nzdim,
      G.nrchop, G.np, kmax, G.ak, cutoff);
  MLG_LAUNCH();
  k_svv_apply<<<dim3(nblk(G.fsize), nf), 256, 0, G.stream>>>(e0, e1, G.nrdim, G.npdim, G.nzdim, G.dscal + DS_SUM0, ft,
                                                              gain_dev);
  MLG_LAUNCH();
  return 0;
}
int op_svv_filter_dev(Scalar& s, double* gain_dev) {
  Scalar* f[1] = {&s};
  return svv_filter_fields(f, 1, gain_dev);
}
int op_svv_filter2_dev(Scalar& a, Scalar& b, double* gains_dev) {
  Scalar* f[2] = {&a, &b};
  return svv_filter_fields(f, 2, gains_dev);
}

// calcat0/1 into dscal[DS_CALC..] (device), optionally zeroat1
int calcat_dev(Scalar& s, const double* at, bool zero_mode) {
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  int nmax = std::min(std::min(G.nrdim, c.nrc), G.nrchop);
  k_calcat<<<cdiv(G.nzdim, 4), 128, 0, G.stream>>>(s.e, nullptr, at, nmax, G.nrdim, G.npdim, G.nzdim,
                                                    (double2*)(G.dscal + DS_CALC), zero_mode ? 1 : 0);
  MLG_LAUNCH();
  return 0;
}

int op_calcat(Scalar& s, int which, double* host_out) {
  if (!s.is("FFF")) {
    TMP(st);
    MLG_TRY(assign(st, s));
    MLG_TRY(op_trans(st, "FFF"));
    MLG_TRY(calcat_dev(st, which ? G.at1 : G.at0, false));
  } else {
    MLG_TRY(calcat_dev(s, which ? G.at1 : G.at0, false));
  }
  if (host_out) {
    MLG_CUDA(cudaMemcpyAsync(host_out, G.dscal + DS_CALC, 2 * G.nz * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
    MLG_CUDA(cudaStreamSynchronize(G.stream));
  }
  return 0;
}

int op_zeroat1(Scalar& s) {
  if (!s.is("FFF")) MLG_TRY(op_trans(s, "FFF"));
  return calcat_dev(s, G.at1, true);
}
int op_zeroat1_2(Scalar& a, Scalar& b) {
  if (!a.is("FFF") || !b.is("FFF") || a.e == b.e) {
    MLG_TRY(op_zeroat1(a));
    return op_zeroat1(b);
  }
  ChopIdx ca, cb;
  MLG_TRY(chop_index(a, ca));
  MLG_TRY(chop_index(b, cb));
  const int na = std::min(std::min(G.nrdim, ca.nrc), G.nrchop), nb = std::min(std::min(G.nrdim, cb.nrc), G.nrchop);
  if (na != nb) {
    MLG_TRY(op_zeroat1(a));
    return op_zeroat1(b);
  }
  k_calcat<<<cdiv(2 * G.nzdim, 4), 128, 0, G.stream>>>(a.e, b.e, G.at1, na, G.nrdim, G.npdim, G.nzdim,
                                                        (double2*)(G.dscal + DS_CALC), 1);
  MLG_LAUNCH();
  return 0;
}

static int require_fff(Scalar& s) {
  if (!s.is("FFF")) MLG_TRY(op_trans(s, "FFF"));
  return 0;
}

int op_delsqp(Scalar& s, bool inverse) {
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  MLG_TRY(require_fff(s));
  if (inverse) { k_idelsqp_ln<<<1, 32, 0, G.stream>>>(s.e, s.ln, G.lognorm, G.ell); MLG_LAUNCH(); }
  k_delsqp<<<nblk(G.fsize), 256, 0, G.stream>>>(s.e, s.ln, G.lognorm, inverse ? 1 : 0, G.nrdim, G.npdim, G.nzdim, c.nrc,
                                                c.npc, G.ell);
  MLG_LAUNCH();
  if (!inverse) { k_ln_zero<<<1, 32, 0, G.stream>>>(s.ln); MLG_LAUNCH(); }
  return 0;
}

int op_band(Scalar& s, int op) {   // xxdx (op 0), del2h (1), del2 (2)
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  MLG_TRY(require_fff(s));
  return launch_band_apply(s, op, c);
}

int op_idel2(Scalar& s, bool pre, double preln) {
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  MLG_TRY(require_fff(s));
  return launch_band_solve(s, pre ? 2 : 1, c, 0.0, 0.0, preln, 0);
}

int op_ihelm(Scalar& s, double alpha) {
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  MLG_TRY(require_fff(s));
  if (std::fabs(alpha) < 5.0e-14)
    return set_error(MLG_EALPHA, "ihelm: alpha equals to zero. Inversion of 0*identity is impossible");
  return launch_band_solve(s, 0, c, alpha, 0.0, 0.0, 0);
}

// helm (:762-789): the reference forms del2(s)+alpha*s in a temporary and never assigns it back,
// so the call leaves s unchanged (it only moves s to FFF first).
int op_helm(Scalar& s, double alpha) {
  (void)alpha;
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  return require_fff(s);
}

int op_helmp(Scalar& s, int power, double alpha, double beta) {
  if (!(power % 2 == 0 && power >= 4)) return set_error(MLG_EPOWER, "helmp: even power greater than or equal to 4");
  if (power > 8) return set_error(MLG_EPOWER, "helmp: power must be less than or equal to 8 (supported power = 4, 6 or 8)");
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  MLG_TRY(require_fff(s));
  TMP(s2);
  MLG_TRY(assign(s2, s));
  MLG_TRY(op_band(s2, 2));
  TMP(sp);
  MLG_TRY(assign(sp, s2));
  for (int n = 1; n <= power / 2 - 1; ++n) MLG_TRY(op_band(sp, 2));
  // so%e = sp%e + beta*s2%e + alpha*s%e; so%ln = alpha*s%ln
  MLG_TRY(lincomb(s, {{&sp, 1.0}, {&s2, beta}, {&s, alpha}}, {{&s, alpha}}));
  return 0;
}

int op_ihelmp(Scalar& s, int power, double alpha, double beta) {
  if (!(power % 2 == 0 && power >= 4)) return set_error(MLG_EPOWER, "ihelmp: even power greater than or equal to 4");
  if (power > 8) return set_error(MLG_EPOWER, "ihelmp: power must be less than or equal to 8 (supported power = 4, 6 or 8)");
  ChopIdx c;
  MLG_TRY(chop_index(s, c));
  MLG_TRY(require_fff(s));
  if (std::fabs(alpha) < 5.0e-14)
    return set_error(MLG_EALPHA, "ihelmp: alpha equals to zero. Inversion of 0*identity is impossible");
  MLG_TRY(launch_ihelmp_pre(s, c, power, alpha, beta));
  return launch_band_solve(s, 3, c, alpha, beta, 0.0, power);
}

// ------------------------------------------------------------------------------------------------
// time steppers (:1065-1262)
static double hsign() { return (((G.P.hyperpow / 2 + 1) % 2) == 0) ? 1.0 : -1.0; }

static int lterm(Scalar& svis) {   // svis <- visc*del2(svis) / hyperviscous operator; ln as the reference
  if (G.P.hyperpow == 0) {
    if (G.P.visc < 5.0e-14) { MLG_TRY(launch_zero(svis.e)); }
    else {
      MLG_TRY(op_band(svis, 2));
      MLG_TRY(lincomb(svis, {{&svis, G.P.visc}}, {}, 1.0, false));
    }
  } else {
    double hv = G.P.hypervisc * hsign();
    MLG_TRY(op_helmp(svis, G.P.hyperpow, 0.0, G.P.visc / hv));
    MLG_TRY(lincomb(svis, {{&svis, hv}}, {}, 1.0, false));
  }
  return 0;
}

static bool fff4(const Scalar& a, const Scalar& b) { return a.is("FFF") && b.is("FFF"); }

int op_fefe(Scalar& s, const Scalar& nl, double dt) {
  if (!fff4(s, nl)) return set_error(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  TMP(svis);
  MLG_TRY(assign(svis, s));
  MLG_TRY(lterm(svis));
  MLG_TRY(lincomb(s, {{&s, 1.0}, {&nl, dt}, {&svis, dt}}, {{&s, 1.0}, {&nl, dt}, {&svis, dt}}));
  return 0;
}

int op_abab(Scalar& s, Scalar& s_p, Scalar& nl, Scalar& nl_p, double dt, bool is2nd) {
  if (!fff4(s, nl) || !fff4(s_p, nl_p)) return set_error(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  TMP(svis);
  MLG_TRY(assign(svis, s));
  MLG_TRY(lterm(svis));
  TMP(svis_p);
  MLG_TRY(assign(svis_p, s_p));
  if (!is2nd) {
    if (G.P.hyperpow == 0) {
      if (G.P.visc < 5.0e-14) { MLG_TRY(launch_zero(svis.e)); }   // (:1135) zeroes svis, not svis_p
      else { MLG_TRY(op_band(svis_p, 2)); MLG_TRY(lincomb(svis_p, {{&svis_p, G.P.visc}}, {}, 1.0, false)); }
    } else {
      double hv = G.P.hypervisc * hsign();
      MLG_TRY(op_helmp(svis_p, G.P.hyperpow, 0.0, G.P.visc / hv));
      MLG_TRY(lincomb(svis_p, {{&svis_p, hv}}, {}, 1.0, false));
    }
  }
  // s = s + dt*(1.5*(nl + svis) - .5*(nl_p + svis_p)), in two passes (four-input combination)
  TMP(acc);
  MLG_TRY(lincomb(acc, {{&nl, 1.5 * dt}, {&svis, 1.5 * dt}, {&nl_p, -.5 * dt}, {&svis_p, -.5 * dt}},
                  {{&nl, 1.5 * dt}, {&svis, 1.5 * dt}, {&nl_p, -.5 * dt}, {&svis_p, -.5 * dt}}));
  MLG_TRY(lincomb(s, {{&s, 1.0}, {&acc, 1.0}}, {{&s, 1.0}, {&acc, 1.0}}));
  MLG_TRY(assign(s_p, s));
  MLG_TRY(assign(nl_p, nl));
  return 0;
}

int op_febe(Scalar& s, const Scalar& nl, double dt) {
  if (!fff4(s, nl)) return set_error(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  if (G.P.hyperpow == 0) {
    if (G.P.visc < 5.0e-14) return set_error(MLG_EINVISCID, "febe: inviscid case and no linear term in rhs. semi-implicit time adv is impossible");
    double a = -1.0 / (dt * G.P.visc);
    // sh = a*(s + dt*nl) (both e and ln), then ihelm(sh, a); s = sh
    MLG_TRY(lincomb(s, {{&s, 1.0}, {&nl, dt}}, {{&s, 1.0}, {&nl, dt}}, a));
    MLG_TRY(op_ihelm(s, a));
  } else {
    double hv = G.P.hypervisc * hsign();
    double a = -1.0 / (dt * hv), b = G.P.visc / hv;
    MLG_TRY(lincomb(s, {{&s, 1.0}, {&nl, dt}}, {{&s, 1.0}, {&nl, dt}}, a));
    MLG_TRY(op_ihelmp(s, G.P.hyperpow, a, b));
  }
  return 0;
}

int op_abcn(Scalar& s, Scalar& s_p, Scalar& nl, Scalar& nl_p, double dt) {
  if (!fff4(s, nl) || !fff4(s_p, nl_p)) return set_error(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  if (G.P.hyperpow == 0 && G.P.visc < 5.0e-14)
    return set_error(MLG_EINVISCID, "abcn: inviscid case and no linear term in rhs. semi-implicit time adv is impossible");
  TMP(svis);
  MLG_TRY(assign(svis, s));
  MLG_TRY(lterm(svis));
  double a;
  if (G.P.hyperpow == 0) a = -2.0 / (dt * G.P.visc);
  else a = -2.0 / (dt * (G.P.hypervisc * hsign()));
  // sh = s + dt*(1.5 nl - .5 nl_p); sh = a*(sh + dt/2*svis)
  MLG_TRY(lincomb(s, {{&s, 1.0}, {&nl, 1.5 * dt}, {&nl_p, -.5 * dt}, {&svis, dt / 2.0}},
                  {{&s, 1.0}, {&nl, 1.5 * dt}, {&nl_p, -.5 * dt}, {&svis, dt / 2.0}}, a));
  if (G.P.hyperpow == 0) MLG_TRY(op_ihelm(s, a));
  else MLG_TRY(op_ihelmp(s, G.P.hyperpow, a, G.P.visc / (G.P.hypervisc * hsign())));
  MLG_TRY(assign(s_p, s));
  MLG_TRY(assign(nl_p, nl));
  return 0;
}

// d = s where s is rewritten in full before it is next read: d takes s's buffer, s keeps d's old one
static int move_into(Scalar& d, Scalar& s) {
  std::swap(d.e, s.e);
  MLG_TRY(launch_copy_ln(d.ln, s.ln));
  std::memcpy(d.space, s.space, 4);
  for (int i = 0; i < 3; ++i) d.off[i] = s.off[i];
  return 0;
}

// abcn of the two fields of a vortex step, (psi, psi_p, nlpsi, nlpsi_p) and (chi, ...): the same
// operations as two abcn calls, with the two Helmholtz solves (same alpha, same chop window) done in
// one substitution pass.  in_step: the caller recomputes nl and ml in full before reading them again,
// so nl_p and ml_p take their buffers instead of copies; write_prev = false leaves s_p and t_p unwritten.
static int op_abcn_pair(Scalar& s, Scalar& s_p, Scalar& nl, Scalar& nl_p, Scalar& t, Scalar& t_p, Scalar& ml,
                        Scalar& ml_p, double dt, bool in_step, bool write_prev) {
  if (G.P.hyperpow != 0) {
    MLG_TRY(op_abcn(s, s_p, nl, nl_p, dt));
    return op_abcn(t, t_p, ml, ml_p, dt);
  }
  if (!fff4(s, nl) || !fff4(s_p, nl_p) || !fff4(t, ml) || !fff4(t_p, ml_p))
    return set_error(MLG_ESPACE, "fefe: all input scalars must be in FFF for time stepping");
  if (G.P.visc < 5.0e-14)
    return set_error(MLG_EINVISCID, "abcn: inviscid case and no linear term in rhs. semi-implicit time adv is impossible");
  double a = -2.0 / (dt * G.P.visc);
  if (std::fabs(a) < 5.0e-14) return set_error(MLG_EALPHA, "ihelm: alpha equals to zero. Inversion of 0*identity is impossible");
  MLG_TRY(launch_abcn_rhs(s, nl, nl_p, dt, a));
  MLG_TRY(launch_abcn_rhs(t, ml, ml_p, dt, a));
  ChopIdx c1, c2;
  MLG_TRY(chop_index(s, c1));
  MLG_TRY(chop_index(t, c2));
  if (c1.nrc == c2.nrc && c1.npc == c2.npc && c1.nzc == c2.nzc && c1.nzcu == c2.nzcu) {
    MLG_TRY(launch_ihelm_pair(s, t, c1, a));
  } else {
    MLG_TRY(launch_band_solve(s, 0, c1, a, 0.0, 0.0, 0));
    MLG_TRY(launch_band_solve(t, 0, c2, a, 0.0, 0.0, 0));
  }
  if (write_prev) { MLG_TRY(assign(s_p, s)); MLG_TRY(assign(t_p, t)); }
  if (in_step) {
    MLG_TRY(move_into(nl_p, nl)); MLG_TRY(move_into(ml_p, ml));
  } else {
    MLG_TRY(assign(nl_p, nl)); MLG_TRY(assign(ml_p, ml));
  }
  return 0;
}

// ------------------------------------------------------------------------------------------------
// vector fields (:1264-1560)
// (vr, vp, vz) x (ur, up, uz), vz plus the background vzb when given, into out (or in place)
static int vecprod_bg(Scalar& vr, Scalar& vp, Scalar& vz, const Scalar& ur, const Scalar& up, const Scalar& uz,
                      const Scalar* vzb, Scalar* const* out = nullptr) {
  for (const Scalar* q : {(const Scalar*)&vr, (const Scalar*)&vp, (const Scalar*)&vz, &ur, &up, &uz})
    if (!q->is("PPP")) return set_error(MLG_ESPACE, "vector_product: to compute v x u, all inputs must be in PPP");
  Scalar* o[3] = {&vr, &vp, &vz};
  if (out) for (int i = 0; i < 3; ++i) o[i] = out[i];
  k_vecprod<<<nblk(G.fsize), 256, 0, G.stream>>>(vr.e, vp.e, vz.e, ur.e, up.e, uz.e, vzb ? vzb->e : nullptr, o[0]->e,
                                                 o[1]->e, o[2]->e, G.nr, G.np / 2, G.nrdim, G.npdim, G.nzdim);
  MLG_LAUNCH();
  double* lns[3] = {o[0]->ln, o[1]->ln, o[2]->ln};
  MLG_TRY(launch_set_ln_n(lns, 3, 0.0));
  for (Scalar* q : o) { q->set_space("PPP"); q->off[0] = q->off[1] = q->off[2] = 0; }
  return 0;
}
int op_vecprod(Scalar& vr, Scalar& vp, Scalar& vz, const Scalar& ur, const Scalar& up, const Scalar& uz) {
  return vecprod_bg(vr, vp, vz, ur, up, uz, nullptr);
}

int scale_r(Scalar& s, int mode) {
  size_t ncol = (size_t)G.npdim * G.nzdim;
  k_scale_r<<<nblk((size_t)G.nr * ncol), 256, 0, G.stream>>>(s.e, mode == 0 ? G.r : G.rinv, G.nr, G.nrdim, ncol);
  MLG_LAUNCH();
  return 0;
}


// vector_projection on (ur, up, uz) PPP fields that it may overwrite (the caller's copies or its own
// temporaries): r*ur, r*up enter the φ transforms (scale_r folded into them)
static int vec2tp_core(Scalar& ur, Scalar& up, Scalar& uz, Scalar& psi, Scalar& chi) {
  // the three components stage by stage, each stage one launch over the three: phi forward (ur and up
  // times r first), then up's radial forward (op_trans's PFP -> FFP step), then z forward
  Scalar* u3[3] = {&ur, &uz, &up};   // up last: its radial transform follows while it is in L2
  if (G.nz > 1)
    for (Scalar* q : u3) MLG_TRY(vfft_check(*q, -1));
  if (G.np > 1) {
    const double* rs[3] = {G.r, nullptr, G.r};
    MLG_TRY(launch_hfft_multi(u3, rs, 3, -1));
  } else {
    MLG_TRY(scale_r(ur, 0));
    MLG_TRY(scale_r(up, 0));
  }
  for (Scalar* q : u3) q->set_space("PFP");
  MLG_TRY(launch_ln_adjust(up, -1.0));
  MLG_TRY(launch_rtrans_fwd(up));
  up.set_space("FFP");
  if (G.nz > 1) MLG_TRY(launch_vfft_multi(u3, 3, -1));
  ur.set_space("PFF");
  up.set_space("FFF");
  uz.set_space("PFF");
  MLG_TRY(calcat_dev(up, G.at1, false));
  MLG_TRY(launch_rtrans_bwd(up, false));   // reads neither psi%ln nor the calcat1 values
  up.set_space("PFF");
  // psi%ln = -calcat1(up)/2, up(:nr,1,1) += psi%ln (1 + x), chi%ln = 0 (:1331) in one launch; psi%e = 0
  // and chi%e = 0 (:1330-1331) are the zeros written by the contraction below
  k_proj_ln<<<1, 256, 0, G.stream>>>(up.e, (const double2*)(G.dscal + DS_CALC), -1.0 / 2.0, psi.ln, chi.ln, G.x, G.nr);
  MLG_LAUNCH();
  MLG_TRY(launch_vec2tp_contract(ur.e, up.e, uz.e, psi.e, chi.e, 3));
  MLG_TRY(op_idel2(chi, false, 0.0));
  psi.off[0] = psi.off[1] = psi.off[2] = 0;
  chi.off[0] = chi.off[1] = chi.off[2] = 0;
  MLG_TRY(op_chop2(psi, chi));
  MLG_TRY(op_zeroat1_2(psi, chi));
  return 0;
}

static int vec2tp_check(const Scalar& vr, const Scalar& vp, const Scalar& vz, const Scalar& psi, const Scalar& chi) {
  if (!vr.is("PPP") || !vp.is("PPP") || !vz.is("PPP")) return set_error(MLG_ESPACE, "vector_projection: vr must be in PPP");
  if (!psi.is("FFF")) return set_error(MLG_ESPACE, "vector_projection: psi must be in FFF");
  if (!chi.is("FFF")) return set_error(MLG_ESPACE, "vector_projection: chi must be in FFF");
  return 0;
}

int op_vec2tp(const Scalar& vr, const Scalar& vp, const Scalar& vz, Scalar& psi, Scalar& chi) {
  MLG_TRY(vec2tp_check(vr, vp, vz, psi, chi));
  TMP(ur); TMP(up); TMP(uz);
  MLG_TRY(assign(ur, vr)); MLG_TRY(assign(up, vp)); MLG_TRY(assign(uz, vz));
  return vec2tp_core(ur, up, uz, psi, chi);
}

// vector_reconstruction up to its transforms: (ur, up, uz) in FFF from (psi, chi), none of them
// aliasing psi or chi (they are the workspace: the same steps as copying chi / psi into temporaries and
// the temporaries into the outputs)
static int tp2vec_spec(const Scalar& psi, const Scalar& chi, Scalar& ur, Scalar& up, Scalar& uz) {
  for (Scalar* q : {&ur, &up, &uz}) { q->set_space("FFF"); q->off[0] = 3; q->off[1] = q->off[2] = 0; }
  ChopIdx c, c0;
  MLG_TRY(chop_index(ur, c));
  for (Scalar* q : {&ur, &up, &uz}) q->off[0] = 0;
  MLG_TRY(chop_index(ur, c0));   // the chop after the products (offsets 0), folded into their kernels
  // -del2h chi on the side stream beside r d/dr chi, r d/dr psi and their mix (the two read psi and chi
  // and write different fields)
  MLG_TRY(side_fork());
  MLG_TRY(launch_band_apply_to(uz, chi, 1, c, -1.0, post_chop(c0), G.side));
  MLG_TRY(launch_tp2vec_uv(ur, up, psi, chi, c, post_chop(c0)));
  MLG_TRY(side_join());
  return 0;
}

// FFF -> PPP of n fields (the components of one or two vector fields), stage by stage, each stage one
// launch over all of them: z backward, radial backward, phi backward, the rows of the fields with
// by_r[i] divided by r (scale_r folded into the last transform)
static int to_ppp_batch(Scalar* const* f, const bool* by_r, int n) {
  for (int i = 0; i < n; ++i) {
    if (!f[i]->is("FFF")) return set_error(MLG_ESPACE, "trans: batched backward transforms start from FFF");
    if (G.nz > 1) MLG_TRY(vfft_check(*f[i], +1));
  }
  if (G.nz > 1) MLG_TRY(launch_vfft_multi(f, n, +1));
  for (int i = 0; i < n; ++i) f[i]->set_space("FFP");
  MLG_TRY(launch_rtrans_bwd_multi(f, n, true));   // one launch over the n fields
  for (int i = 0; i < n; ++i) f[i]->set_space("PFP");
  if (G.np > 1) {
    const double* rs[6];
    for (int i = 0; i < n; ++i) rs[i] = by_r[i] ? G.rinv : nullptr;
    MLG_TRY(launch_hfft_multi(f, rs, n, +1));
  } else {
    for (int i = 0; i < n; ++i)
      if (by_r[i]) MLG_TRY(scale_r(*f[i], 1));
  }
  for (int i = 0; i < n; ++i) f[i]->set_space("PPP");
  return 0;
}

// vector_reconstruction into (ur, up, uz)
static int tp2vec_into(const Scalar& psi, const Scalar& chi, Scalar& ur, Scalar& up, Scalar& uz) {
  MLG_TRY(tp2vec_spec(psi, chi, ur, up, uz));
  Scalar* f[3] = {&ur, &up, &uz};
  const bool by_r[3] = {true, true, false};
  return to_ppp_batch(f, by_r, 3);
}

static bool aliases(const Scalar& a, const Scalar& b) { return a.e == b.e; }

int op_tp2vec(const Scalar& psi, const Scalar& chi, Scalar& vr, Scalar& vp, Scalar& vz) {
  if (!psi.is("FFF") || !chi.is("FFF")) return set_error(MLG_ESPACE, "vector_projection: psi must be in FFF");
  if (!vr.is("PPP") || !vp.is("PPP") || !vz.is("PPP")) return set_error(MLG_ESPACE, "vector_projection: vr must be in PPP");
  bool alias = false;
  for (const Scalar* o : {&vr, &vp, &vz})
    for (const Scalar* i : {&psi, &chi}) alias = alias || aliases(*o, *i);
  alias = alias || aliases(vr, vp) || aliases(vr, vz) || aliases(vp, vz);
  if (!alias) return tp2vec_into(psi, chi, vr, vp, vz);
  TMP(ur); TMP(up); TMP(uz);
  MLG_TRY(tp2vec_into(psi, chi, ur, up, uz));
  MLG_TRY(assign(vr, ur)); MLG_TRY(assign(vp, up)); MLG_TRY(assign(vz, uz));
  return 0;
}

int op_tp2curlvec(const Scalar& psi, const Scalar& chi, Scalar& wr, Scalar& wp, Scalar& wz) {
  TMP(md);
  md.set_space("FFF");
  md.off[0] = chi.off[0]; md.off[1] = chi.off[1]; md.off[2] = chi.off[2];
  ChopIdx c;
  MLG_TRY(chop_index(md, c));
  MLG_TRY(launch_band_apply_to(md, chi, 2, c, -1.0));   // md = -del2 chi
  return op_tp2vec(md, psi, wr, wp, wz);
}

// advection_rhs (vortical_flow_3d.f90:353-395)
int op_advection_rhs(Scalar& psi, Scalar& chi, Scalar& nlpsi, Scalar& nlchi, const Scalar& uz, Scalar* const* keep,
                     bool dealiased) {
  if (!psi.is("FFF") || !chi.is("FFF") || !nlpsi.is("FFF") || !nlchi.is("FFF") || !uz.is("PPP"))
    return set_error(MLG_ESPACE, "advection_rhs: psi, chi, nlpsi, nlchi must be in FFF and uz in PPP");
  if (!dealiased) MLG_TRY(op_dealias2(psi, chi));
  TMP(vr_t); TMP(vp_t); TMP(vz_t); TMP(wr_t); TMP(wp_t); TMP(wz_t);
  Scalar* vw[6] = {&vr_t, &vp_t, &vz_t, &wr_t, &wp_t, &wz_t};
  if (keep) for (int i = 0; i < 6; ++i) vw[i] = keep[i];
  for (Scalar* q : vw) q->set_space("PPP");
  Scalar &vr = *vw[0], &vp = *vw[1], &vz = *vw[2], &wr = *vw[3], &wp = *vw[4], &wz = *vw[5];
  // v and w, each with its three transforms to PPP batched (three fields, 78 MB at 192x128x128, stay
  // in L2 from one stage to the next; six would not).  w = tp2vec(-del2 chi, psi) (tp2curlvec): the
  // -del2 chi starts on the side stream beside v's kernels (the side stream's next join orders it)
  TMP(md);
  md.set_space("FFF");
  md.off[0] = chi.off[0]; md.off[1] = chi.off[1]; md.off[2] = chi.off[2];
  ChopIdx cmd;
  MLG_TRY(chop_index(md, cmd));
  MLG_TRY(side_fork());
  MLG_TRY(launch_band_apply_to(md, chi, 2, cmd, -1.0, PostChop{0, 0, 0, 0, 0}, G.side));   // md = -del2 chi
  MLG_TRY(tp2vec_into(psi, chi, vr, vp, vz));
  MLG_TRY(side_join());
  MLG_TRY(op_tp2vec(md, psi, wr, wp, wz));
  // (vz + uz) with the background flow; in place, or into the temporaries when v and w are kept
  Scalar* prod[3] = {&vr_t, &vp_t, &vz_t};
  MLG_TRY(vecprod_bg(vr, vp, vz, wr, wp, wz, &uz, keep ? prod : nullptr));
  MLG_TRY(vec2tp_core(vr_t, vp_t, vz_t, nlpsi, nlchi));
  MLG_TRY(op_zero_ln_dealias2(nlpsi, nlchi));   // ln = 0, then dealias
  return 0;
}

// main-loop step (vortical_flow_3d.f90:168-180) with the gains in device memory
int op_vortex_step_dev(Scalar& psi, Scalar& chi, Scalar& nlpsi, Scalar& nlchi, Scalar& psip, Scalar& chip, Scalar& nlpsip,
                       Scalar& nlchip, const Scalar& uz, double dt, double* gains_dev, Scalar* const* keep,
                       bool write_prev) {
  for (Scalar* q : {&psi, &chi, &nlpsi, &nlchi, &psip, &chip, &nlpsip, &nlchip}) MLG_TRY(op_trans(*q, "FFF"));
  // nlpsi and nlchi are recomputed in full by the advection below
  MLG_TRY(op_abcn_pair(psi, psip, nlpsi, nlpsip, chi, chip, nlchi, nlchip, dt, true, write_prev));
  MLG_TRY(op_dealias2(psi, chi));
  MLG_TRY(op_svv_filter2_dev(psi, chi, gains_dev));
  MLG_TRY(op_zeroat1_2(psi, chi));
  // advection_rhs's own dealias of psi and chi (vortical_flow_3d.f90:368) finds them dealiased
  // already: the SVV gain and zeroat1 leave a zero coefficient zero, so it is skipped here
  // check_stability's finiteness test of psi and chi, final from here on, on the side stream beside the
  // advection (which reads them only); joined before the step ends
  MLG_TRY(side_fork());
  k_finite<<<nblk(G.fsize), 256, 0, G.side>>>(psi.e, chi.e, G.fsize, (int*)(G.dscal + DS_FLAG));
  MLG_LAUNCH();
  MLG_TRY(op_advection_rhs(psi, chi, nlpsi, nlchi, uz, keep, true));
  MLG_TRY(side_join());
  return 0;
}

}  // namespace mlg

// =================================================================================================
// C ABI
using namespace mlg;

// The error words at DS_FLAG + 1 (w[0]: a banded factorisation met a zero pivot; w[1]: a bounded
// device-side wait of a tensor-core kernel ran out), read by the caller after a stream sync.  Clears
// them and returns the status they stand for; a timeout wins, since the results of that launch are void.
static int device_status(const int* w) {
  if (!w[0] && !w[1]) return 0;
  MLG_CUDA(cudaMemsetAsync(G.dscal + DS_FLAG + 1, 0, sizeof(double), G.stream));
  MLG_CUDA(cudaStreamSynchronize(G.stream));
  if (w[1]) return set_error(MLG_ETIMEOUT, "a bounded device-side wait ran out: the results of the last calls are void");
  return set_error(MLG_ESINGULAR, "lurc: lu factorization resulted in failure");
}

static int need_kit() { return G.kit_set ? 0 : set_error(MLG_ENOKIT, "transformation kit is not initialized"); }
#define NEED_KIT() MLG_TRY(need_kit())
#define SC(p) if (!(p) || !(p)->e) return set_error(MLG_EHANDLE, "invalid scalar handle")
static Scalar* S(mlg_scalar h) { return reinterpret_cast<Scalar*>(h); }

extern "C" {

void mlg_params_default(mlg_params* p) {
  p->nr = 256; p->np = 128; p->nz = 128; p->nrchop = 256; p->npchop = 65; p->nzchop = 65;
  p->ell = 4.0; p->zlen = 2.0 * 3.14159265358979323846; p->visc = 1.0e-3; p->hyperpow = 0; p->hypervisc = 0.0;
  p->is_svv = 1; p->svv_cutoff = 0.75; p->svv_target = 2.0e-2; p->svv_strength = 0.12; p->svv_relax = 0.25;
}

const char* mlg_last_error(void) { return g_err.c_str(); }

int mlg_init(const mlg_params* p) {
  if (!p) return set_error(MLG_EHANDLE, "mlg_init: null parameters");
  if (!G.ev0) { cudaEventCreate(&G.ev0); cudaEventCreate(&G.ev1); }
  if (!G.side) {
    MLG_CUDA(cudaStreamCreateWithFlags(&G.side, cudaStreamNonBlocking));
    MLG_CUDA(cudaEventCreateWithFlags(&G.ev_fork, cudaEventDisableTiming));
    MLG_CUDA(cudaEventCreateWithFlags(&G.ev_join, cudaEventDisableTiming));
  }
  int rc = kit_build(p);
  if (rc) return rc;
  G.n_slots = 4096;
  MLG_TRY(dmalloc((void**)&G.ln_slots, G.n_slots * sizeof(double)));
  MLG_CUDA(cudaMemset(G.ln_slots, 0, G.n_slots * sizeof(double)));
  G.free_slots.clear();
  for (int i = G.n_slots - 1; i >= 0; --i) G.free_slots.push_back(i);
  return 0;
}

int mlg_finalize(void) {
  if (!G.kit_set) return 0;
  cudaStreamSynchronize(G.stream);
  lu_cache_clear();
  xs_free();
  xv_free();
  for (cd* b : G.all_bufs) cudaFree(b);
  void* arrs[] = {G.x, G.w, G.w32, G.r, G.rinv, G.lnx, G.ak, G.lognorm, G.pf, G.at0, G.at1, G.bd2, G.bxx, G.bd2f, G.bxxf, G.ak2f, G.tV, G.tD, G.tT,
                  G.tV32, G.tD32, G.tT32, G.tw_p, G.tw_z, G.tw_pr, G.tw_p32, G.tw_z32, G.tw_pr32, G.tw_pdf, G.tw_zdf, G.tw_prdf, G.ln_slots, G.dscal, G.band_ws};
  for (void* a : arrs) if (a) cudaFree(a);
  cudaStream_t st = G.stream;
  cudaEvent_t e0 = G.ev0, e1 = G.ev1, ef = G.ev_fork, ej = G.ev_join;
  cudaStream_t side = G.side, cap = G.cap;
  G = Ctx();
  G.stream = st;
  G.ev0 = e0; G.ev1 = e1; G.ev_fork = ef; G.ev_join = ej; G.side = side; G.cap = cap;
  return 0;
}

int mlg_kit_dims(int* d) {
  NEED_KIT();
  d[0] = G.nrdim; d[1] = G.npdim; d[2] = G.nzdim; d[3] = G.chopzl; d[4] = G.chopzu; d[5] = G.nrh; d[6] = G.ne;
  d[7] = G.npchop; d[8] = G.nr;
  return 0;
}

int mlg_kit_get(const char* name, double* out, long long count) {
  NEED_KIT();
  std::string n(name ? name : "");
  const double* src = nullptr;
  long long cnt = 0;
  if (n == "x") { src = G.x; cnt = G.nr; } else if (n == "w") { src = G.w; cnt = G.nr; }
  else if (n == "r") { src = G.r; cnt = G.nr; } else if (n == "ln") { src = G.lnx; cnt = G.nr; }
  else if (n == "ak") { src = G.ak; cnt = G.nz; }
  else if (n == "lognorm") { src = G.lognorm; cnt = (long long)G.ne * G.npchop; }
  else if (n == "pf") { src = G.pf; cnt = (long long)G.nrh * G.ne * G.npchop; }
  else if (n == "at0") { src = G.at0; cnt = G.nrchop; } else if (n == "at1") { src = G.at1; cnt = G.nrchop; }
  if (!src) return set_error(MLG_EHANDLE, "mlg_kit_get: unknown array name");
  if (count < cnt) return set_error(MLG_ESIZE, "mlg_kit_get: output buffer too small");
  MLG_CUDA(cudaMemcpyAsync(out, src, cnt * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
  MLG_CUDA(cudaStreamSynchronize(G.stream));
  return 0;
}

int mlg_set_precision(int mode) {
  if (mode != MLG_PLAIN_FP64 && mode != MLG_MIXED) return set_error(MLG_EPARAM, "mlg_set_precision: unknown mode");
  G.precision = mode;
  return 0;
}
int mlg_get_precision(int* mode) { *mode = G.precision; return 0; }
int mlg_set_stream(void* stream) { G.stream = (cudaStream_t)stream; return 0; }
int mlg_sync(void) {
  MLG_CUDA(cudaStreamSynchronize(G.stream));
  if (G.kit_set) {
    int w[2] = {0, 0};
    MLG_CUDA(cudaMemcpyAsync(w, G.dscal + DS_FLAG + 1, sizeof(w), cudaMemcpyDeviceToHost, G.stream));
    MLG_CUDA(cudaStreamSynchronize(G.stream));
    return device_status(w);
  }
  return 0;
}
long long mlg_mem_bytes(void) { return G.mem_bytes; }
long long mlg_mem_high_water(void) { return G.mem_high; }
long long mlg_launch_count(void) { return G.launches; }

int mlg_scalar_alloc(mlg_scalar* out) {
  NEED_KIT();
  Scalar* s = new Scalar;
  int rc = scalar_init(*s);
  if (rc) { delete s; return rc; }
  MLG_CUDA(cudaMemsetAsync(s->e, 0, G.fsize * sizeof(cd), G.stream));
  *out = reinterpret_cast<mlg_scalar>(s);
  return 0;
}
int mlg_scalar_free(mlg_scalar h) {
  Scalar* s = S(h);
  if (!s) return 0;
  if (G.kit_set && s->e) scalar_release(*s);
  delete s;
  return 0;
}
static int set_space_checked(Scalar& s, const char* sp) {
  if (!sp || space_code(sp) < 0) return set_error(MLG_ESPACE, "space must be PPP, PFP, FFP or FFF");
  s.set_space(sp);
  return 0;
}
int mlg_scalar_upload(mlg_scalar h, const double* e, double ln, const char* space) {
  NEED_KIT(); Scalar* s = S(h); SC(s);
  MLG_TRY(set_space_checked(*s, space));
  MLG_CUDA(cudaMemcpyAsync(s->e, e, G.fsize * sizeof(cd), cudaMemcpyHostToDevice, G.stream));
  MLG_TRY(launch_set_ln(s->ln, ln));
  return 0;
}
int mlg_scalar_upload_device(mlg_scalar h, const void* e, double ln, const char* space) {
  NEED_KIT(); Scalar* s = S(h); SC(s);
  MLG_TRY(set_space_checked(*s, space));
  MLG_CUDA(cudaMemcpyAsync(s->e, e, G.fsize * sizeof(cd), cudaMemcpyDeviceToDevice, G.stream));
  MLG_TRY(launch_set_ln(s->ln, ln));
  return 0;
}
int mlg_scalar_download(mlg_scalar h, double* e, double* ln, char* space4) {
  NEED_KIT(); Scalar* s = S(h); SC(s);
  if (e) MLG_CUDA(cudaMemcpyAsync(e, s->e, G.fsize * sizeof(cd), cudaMemcpyDeviceToHost, G.stream));
  if (ln) MLG_CUDA(cudaMemcpyAsync(ln, s->ln, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
  MLG_CUDA(cudaStreamSynchronize(G.stream));
  if (space4) { std::memcpy(space4, s->space, 4); }
  return 0;
}
int mlg_scalar_download_device(mlg_scalar h, void* e, double* ln, char* space4) {
  NEED_KIT(); Scalar* s = S(h); SC(s);
  if (e) MLG_CUDA(cudaMemcpyAsync(e, s->e, G.fsize * sizeof(cd), cudaMemcpyDeviceToDevice, G.stream));
  if (ln) {
    MLG_CUDA(cudaMemcpyAsync(ln, s->ln, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
    MLG_CUDA(cudaStreamSynchronize(G.stream));
  }
  if (space4) { std::memcpy(space4, s->space, 4); }
  return 0;
}
int mlg_scalar_copy(mlg_scalar d, mlg_scalar s) {
  NEED_KIT(); SC(S(d)); SC(S(s));
  return assign(*S(d), *S(s));
}
int mlg_scalar_chop_offset(mlg_scalar h, int a, int b, int c) {
  Scalar* s = S(h); SC(s);
  s->off[0] = a; s->off[1] = b; s->off[2] = c;
  return 0;
}
int mlg_scalar_get_meta(mlg_scalar h, double* ln, char* space4, int* offs) {
  NEED_KIT(); Scalar* s = S(h); SC(s);
  if (ln) {
    MLG_CUDA(cudaMemcpyAsync(ln, s->ln, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
    MLG_CUDA(cudaStreamSynchronize(G.stream));
  }
  if (space4) std::memcpy(space4, s->space, 4);
  if (offs) for (int i = 0; i < 3; ++i) offs[i] = s->off[i];
  return 0;
}
int mlg_scalar_set_ln(mlg_scalar h, double ln) { NEED_KIT(); Scalar* s = S(h); SC(s); return launch_set_ln(s->ln, ln); }
int mlg_scalar_set_space(mlg_scalar h, const char* sp) { Scalar* s = S(h); SC(s); return set_space_checked(*s, sp); }
int mlg_scalar_axpby(mlg_scalar d, double a, mlg_scalar x, double b, mlg_scalar y) {
  NEED_KIT(); SC(S(d)); SC(S(x));
  if (y) { SC(S(y)); return lincomb(*S(d), {{S(x), a}, {S(y), b}}, {}, 1.0, false); }
  return lincomb(*S(d), {{S(x), a}}, {}, 1.0, false);
}
void* mlg_scalar_device_ptr(mlg_scalar h) { Scalar* s = S(h); return s ? (void*)s->e : nullptr; }

#define OP1(name, call) int name(mlg_scalar h) { NEED_KIT(); Scalar* s = S(h); SC(s); return call; }
OP1(mlg_chop, op_chop(*s))
OP1(mlg_dealias, op_dealias(*s))
OP1(mlg_zeroat1, op_zeroat1(*s))
OP1(mlg_delsqp, op_delsqp(*s, false))
OP1(mlg_idelsqp, op_delsqp(*s, true))
OP1(mlg_xxdx, op_band(*s, 0))
OP1(mlg_del2h, op_band(*s, 1))
OP1(mlg_del2, op_band(*s, 2))
OP1(mlg_idel2_proln, op_idel2(*s, false, 0.0))

int mlg_trans(mlg_scalar h, const char* space) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_trans(*s, space ? space : ""); }
int mlg_svv_filter(mlg_scalar h, double* gain) {
  NEED_KIT(); Scalar* s = S(h); SC(s);
  if (!gain) return set_error(MLG_EHANDLE, "svv_filter: null gain");
  double* gd = G.dscal + DS_GAIN0 + 2;
  MLG_CUDA(cudaMemcpyAsync(gd, gain, sizeof(double), cudaMemcpyHostToDevice, G.stream));
  MLG_TRY(op_svv_filter_dev(*s, gd));
  MLG_CUDA(cudaMemcpyAsync(gain, gd, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
  MLG_CUDA(cudaStreamSynchronize(G.stream));
  return 0;
}
int mlg_calcat0(mlg_scalar h, double* out) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_calcat(*s, 0, out); }
int mlg_calcat1(mlg_scalar h, double* out) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_calcat(*s, 1, out); }
int mlg_idel2_preln(mlg_scalar h, double preln) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_idel2(*s, true, preln); }
int mlg_helm(mlg_scalar h, double a) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_helm(*s, a); }
int mlg_ihelm(mlg_scalar h, double a) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_ihelm(*s, a); }
int mlg_ihelm_noalloc(void* e_dev, double* ln, double alpha) {
  NEED_KIT();
  if (!e_dev || !ln) return set_error(MLG_EHANDLE, "ihelm_noalloc: null field or ln");
  return ihelm_noalloc(e_dev, ln, alpha);
}
int mlg_helmp(mlg_scalar h, int p, double a, double b) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_helmp(*s, p, a, b); }
int mlg_ihelmp(mlg_scalar h, int p, double a, double b) { NEED_KIT(); Scalar* s = S(h); SC(s); return op_ihelmp(*s, p, a, b); }

int mlg_fefe(mlg_scalar h, mlg_scalar nl, double dt) { NEED_KIT(); SC(S(h)); SC(S(nl)); return op_fefe(*S(h), *S(nl), dt); }
int mlg_febe(mlg_scalar h, mlg_scalar nl, double dt) { NEED_KIT(); SC(S(h)); SC(S(nl)); return op_febe(*S(h), *S(nl), dt); }
int mlg_abab(mlg_scalar h, mlg_scalar hp, mlg_scalar nl, mlg_scalar nlp, double dt, int is2nd) {
  NEED_KIT(); SC(S(h)); SC(S(hp)); SC(S(nl)); SC(S(nlp));
  return op_abab(*S(h), *S(hp), *S(nl), *S(nlp), dt, is2nd != 0);
}
int mlg_abcn(mlg_scalar h, mlg_scalar hp, mlg_scalar nl, mlg_scalar nlp, double dt) {
  NEED_KIT(); SC(S(h)); SC(S(hp)); SC(S(nl)); SC(S(nlp));
  return op_abcn(*S(h), *S(hp), *S(nl), *S(nlp), dt);
}
int mlg_vecprod(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e, mlg_scalar f) {
  NEED_KIT(); SC(S(a)); SC(S(b)); SC(S(c)); SC(S(d)); SC(S(e)); SC(S(f));
  return op_vecprod(*S(a), *S(b), *S(c), *S(d), *S(e), *S(f));
}
int mlg_vec2tp(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e) {
  NEED_KIT(); SC(S(a)); SC(S(b)); SC(S(c)); SC(S(d)); SC(S(e));
  return op_vec2tp(*S(a), *S(b), *S(c), *S(d), *S(e));
}
int mlg_tp2vec(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e) {
  NEED_KIT(); SC(S(a)); SC(S(b)); SC(S(c)); SC(S(d)); SC(S(e));
  return op_tp2vec(*S(a), *S(b), *S(c), *S(d), *S(e));
}
int mlg_tp2curlvec(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e) {
  NEED_KIT(); SC(S(a)); SC(S(b)); SC(S(c)); SC(S(d)); SC(S(e));
  return op_tp2curlvec(*S(a), *S(b), *S(c), *S(d), *S(e));
}
int mlg_advection_rhs(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e) {
  NEED_KIT(); SC(S(a)); SC(S(b)); SC(S(c)); SC(S(d)); SC(S(e));
  return op_advection_rhs(*S(a), *S(b), *S(c), *S(d), *S(e));
}

static int vortex_loop(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e, mlg_scalar f, mlg_scalar g,
                       mlg_scalar h, mlg_scalar u, double dt, int nsteps, double* gains) {
  NEED_KIT();
  for (mlg_scalar q : {a, b, c, d, e, f, g, h, u}) SC(S(q));
  if (!gains) return set_error(MLG_EHANDLE, "vortex step: null gains");
  double* gd = G.dscal + DS_GAIN0;
  MLG_CUDA(cudaMemcpyAsync(gd, gains, 2 * sizeof(double), cudaMemcpyHostToDevice, G.stream));
  MLG_CUDA(cudaMemsetAsync(G.dscal + DS_FLAG, 0, sizeof(double), G.stream));
  auto step = [&](bool last) {   // psip and chip are read by no step: written by the last
    return op_vortex_step_dev(*S(a), *S(b), *S(c), *S(d), *S(e), *S(f), *S(g), *S(h), *S(u), dt, gd, nullptr, last);
  };
  cudaGraphExec_t gexec = nullptr;
  if (nsteps >= 4 && !G.kt.on) {
    // The interior steps replay one CUDA graph of two steps: the first step runs as launched (it fills
    // the factor, table and buffer caches, so that the captured steps allocate nothing), the next two
    // are captured on a stream of the library's own (capture cannot run on the legacy default stream),
    // and the graph then runs them in pairs; an odd interior step and the last step (which writes psip
    // and chip) run as launched.  A step hands nlpsi's and nlchi's buffers to nlpsi_p and nlchi_p, so
    // two steps leave every field in its own buffer again: a replay of the pair is the two steps
    // themselves, on the same buffers.
    MLG_TRY(step(false));
    if (!G.cap) MLG_CUDA(cudaStreamCreateWithFlags(&G.cap, cudaStreamNonBlocking));
    const cudaStream_t orig = G.stream;
    const long long l0 = G.launches;
    G.stream = G.cap;
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(G.cap, cudaStreamCaptureModeRelaxed);
    int rc = ce == cudaSuccess ? step(false) : 0;
    if (ce == cudaSuccess && rc == 0) rc = step(false);
    if (ce == cudaSuccess) ce = cudaStreamEndCapture(G.cap, &graph);
    G.stream = orig;
    const long long nl = G.launches - l0;
    G.launches = l0;
    if (rc == 0 && ce == cudaSuccess) ce = cudaGraphInstantiate(&gexec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc) return rc;
    if (ce != cudaSuccess) {
      cudaGetLastError();
      return set_error(MLG_ECUDA, std::string("vortex run: graph capture: ") + cudaGetErrorString(ce));
    }
    const int interior = nsteps - 2;
    for (int t = 0; t + 1 < interior; t += 2) {
      ce = cudaGraphLaunch(gexec, G.stream);
      if (ce != cudaSuccess) break;
      G.launches += nl;
    }
    if (ce == cudaSuccess) {
      int rc2 = (interior & 1) ? step(false) : 0;
      if (rc2 == 0) rc2 = step(true);
      if (rc2) { cudaStreamSynchronize(G.stream); cudaGraphExecDestroy(gexec); return rc2; }
    }
    cudaStreamSynchronize(G.stream);
    cudaGraphExecDestroy(gexec);
    if (ce != cudaSuccess) {
      cudaGetLastError();
      return set_error(MLG_ECUDA, std::string("vortex run: graph launch: ") + cudaGetErrorString(ce));
    }
  } else {
    for (int t = 0; t < nsteps; ++t) MLG_TRY(step(t == nsteps - 1));
  }
  MLG_CUDA(cudaMemcpyAsync(gains, gd, 2 * sizeof(double), cudaMemcpyDeviceToHost, G.stream));
  int w[4] = {0, 0, 0, 0};   // DS_FLAG: non-finite flag, unused; DS_FLAG + 1: singular-LU flag, timeout flag
  MLG_CUDA(cudaMemcpyAsync(w, G.dscal + DS_FLAG, sizeof(w), cudaMemcpyDeviceToHost, G.stream));
  MLG_CUDA(cudaStreamSynchronize(G.stream));
  MLG_TRY(device_status(w + 2));
  if (w[0]) return set_error(MLG_ENONFINITE, "ERROR: non-finite vortex state");
  return 0;
}
int mlg_vortex_step(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e, mlg_scalar f, mlg_scalar g,
                    mlg_scalar h, mlg_scalar u, double dt, double* gains) {
  return vortex_loop(a, b, c, d, e, f, g, h, u, dt, 1, gains);
}
int mlg_vortex_run(mlg_scalar a, mlg_scalar b, mlg_scalar c, mlg_scalar d, mlg_scalar e, mlg_scalar f, mlg_scalar g,
                   mlg_scalar h, mlg_scalar u, double dt, int nsteps, double* gains) {
  return vortex_loop(a, b, c, d, e, f, g, h, u, dt, nsteps, gains);
}

int mlg_selftest_bounded_wait(long long limit_clocks, int arrive) {
  NEED_KIT();
  return wait_selftest(limit_clocks, arrive);
}

int mlg_kernel_timing(int enable) {
  G.kt.on = enable != 0;
  for (int i = 0; i < KT_N; ++i) { G.kt.ms[i] = 0; G.kt.n[i] = 0; G.kt.work[i] = 0; }
  return 0;
}
int mlg_kernel_timing_read(int kind, double* ms, long long* n, double* work) {
  if (kind < 0 || kind >= KT_N) return set_error(MLG_EPARAM, "mlg_kernel_timing_read: kind 0..5");
  if (ms) *ms = G.kt.ms[kind];
  if (n) *n = G.kt.n[kind];
  if (work) *work = G.kt.work[kind];
  return 0;
}

}  // extern "C"
