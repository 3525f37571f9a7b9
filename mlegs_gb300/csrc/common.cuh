// common.cuh — shared state, error handling and small device helpers of the GB300 library.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <initializer_list>
#include <utility>
#include <algorithm>
#include <vector>
#include "../../include/mlegs_gb300.h"

namespace mlg {

typedef double2 cd;   // complex128 as stored in a field (re, im)

// ---------------------------------------------------------------------------------------------
// errors: every C-ABI call returns a status; the message is kept for mlg_last_error()
int set_error(int code, const std::string& msg);
#define MLG_TRY(x) do { int _rc = (x); if (_rc) return _rc; } while (0)
#define MLG_CUDA(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) \
    return ::mlg::set_error(MLG_ECUDA, std::string(#x) + ": " + cudaGetErrorString(_e)); } while (0)
#define MLG_LAUNCH() do { ++::mlg::G.launches; cudaError_t _e = cudaGetLastError(); if (_e != cudaSuccess) \
    return ::mlg::set_error(MLG_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(_e)); } while (0)

// ---------------------------------------------------------------------------------------------
// a field ("scalar"): device complex128 array (nrdim, npdim, nzdim), Fortran order
struct Scalar {
  cd* e = nullptr;        // device data
  double* ln = nullptr;   // device slot holding the log-term coefficient (ln of type(scalar))
  char space[4] = {'P', 'P', 'P', 0};
  int off[3] = {0, 0, 0};
  int slot = -1;          // index of the ln slot
  bool is(const char* s) const { return std::strncmp(space, s, 3) == 0; }
  void set_space(const char* s) { std::memcpy(space, s, 3); space[3] = 0; }
};

// chop_index (mlegs_scalar_ops.f90:2012-2063) on one process
struct ChopIdx { int nrc, npc, nzc, nzcu; };
// chop (mlegs_scalar_ops.f90:6-41) of an FFF field folded into a kernel's output: on == 0 leaves the
// output as it is; else column (m, k) keeps only its rows below chop_from(m, k)
struct PostChop { int on, nrc, npc, nzc, nzcu; };
__host__ __device__ inline int chop_from(const PostChop& p, int m, int k, int nrdim) {
  if (!p.on) return nrdim;
  if (m >= p.npc || (p.nzc < p.nzcu && k + 1 >= p.nzc + 1 && k + 1 <= p.nzcu - 1)) return 0;
  int n = p.nrc - m;
  return n < 0 ? 0 : (n < p.nrc ? n : p.nrc);
}
inline PostChop post_chop(const ChopIdx& c) { return PostChop{1, c.nrc, c.npc, c.nzc, c.nzcu}; }

// kernel-time accounting per kernel class (mlg_kernel_timing)
enum { KT_RFWD = 0, KT_FFT = 1, KT_BAND = 2, KT_RBWD = 3, KT_V2TP = 4, KT_SOLVE = 5, KT_N = 6 };
struct KTimer {
  bool on = false;
  double ms[KT_N] = {0, 0, 0, 0, 0, 0};
  long long n[KT_N] = {0, 0, 0, 0, 0, 0};
  double work[KT_N] = {0, 0, 0, 0, 0, 0};
};

struct Ctx {
  bool kit_set = false;
  mlg_params P{};
  int nr = 0, np = 0, nz = 0, nrchop = 0, npchop = 0, nzchop = 0;
  int nrdim = 0, npdim = 0, nzdim = 0, nrh = 0, ne = 0, chopzl = 0, chopzu = 0, nph = 0;
  size_t fsize = 0;       // complex entries per field
  double ell = 0;
  int precision = MLG_PLAIN_FP64;
  cudaStream_t stream = 0;
  int device = -1;        // the CUDA device that was current when the kit was built

  // kit arrays on the device
  double *x = nullptr, *w = nullptr, *r = nullptr, *rinv = nullptr, *lnx = nullptr, *ak = nullptr;
  float* w32 = nullptr;        // FP32 quadrature weights (mixed form)
  bool svv_q_ready = false;
  double *lognorm = nullptr;   // (ne, npchop)
  double *pf = nullptr;        // (nrh, ne, npchop): P_L^m(x_i) normalised, reference layout
  double *at0 = nullptr, *at1 = nullptr;   // (nrchop)
  double *bd2 = nullptr;       // del2 bands without the -k^2 term: (5, ne, npchop)
  double *bxx = nullptr;       // xxdx bands: (3, ne+1, npchop)
  float *bd2f = nullptr, *bxxf = nullptr, *ak2f = nullptr;   // FP32 bands and ak^2 (the mixed form's m >= 1 stencils)
  double *tV = nullptr, *tD = nullptr, *tT = nullptr;   // vec2tp matrices (nrh, ne, npchop)
  float *tV32 = nullptr, *tD32 = nullptr, *tT32 = nullptr;   // FP32 copies (the mixed form's adjoint)
  double2 *tw_p = nullptr, *tw_z = nullptr;  // FFT twiddles exp(-2 pi i k/L): L = np/2 (phi), nz (z)
  double2 *tw_pr = nullptr;    // real-FFT post-processing twiddles exp(-2 pi i k/np), k < np/2+1
  float2 *tw_p32 = nullptr, *tw_z32 = nullptr, *tw_pr32 = nullptr;   // FP32 copies for the mixed form
  float4 *tw_pdf = nullptr, *tw_zdf = nullptr, *tw_prdf = nullptr;   // double-float copies (re hi, re lo, im hi, im lo)

  // ln slots of all scalars (device), and per-step scalars (svv gains, flags, scratch reductions)
  double* ln_slots = nullptr;  int n_slots = 0;  std::vector<int> free_slots;
  double* dscal = nullptr;     // misc device scalars (see DS_* below)

  // banded-solve scratch: LU work band (7 or more rows) per (m, k) system
  double* band_ws = nullptr;   size_t band_ws_bytes = 0;

  // pool of field-sized device buffers for out-of-place steps and temporaries
  std::vector<cd*> pool;
  std::vector<cd*> all_bufs;

  long long mem_bytes = 0, mem_high = 0;
  long long launches = 0;     // kernels launched by the library since mlg_init
  KTimer kt;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // side stream for work that runs beside the work stream (the mixed form's m = 0 plane), forked and
  // joined with events so that callers only ever see the work stream
  cudaStream_t side = nullptr;
  cudaStream_t cap = nullptr;   // the stream a vortex run's interior step is captured on (a CUDA graph)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};
extern Ctx G;

// indices into G.dscal
enum { DS_SUM0 = 0, DS_SUM1 = 1, DS_GAIN0 = 4, DS_GAIN1 = 5, DS_FLAG = 8, DS_CALC = 16, DS_COUNT = 16 + 3 * 4096 };

// device memory accounting
int dmalloc(void** p, size_t bytes);
void dfree(void* p, size_t bytes);
cd* get_buf();
void put_buf(cd* b);
int pool_reserve(int n);

// side stream: fork makes it wait for everything enqueued on the work stream so far; join makes the
// work stream wait for everything enqueued on it so far
int side_fork();
int side_join();

// kernel timing helpers
void kt_begin(int kind);
void kt_end(int kind, double work);

// host-side chop_index
int chop_index(const Scalar& s, ChopIdx& c);

// kernels (host launchers), defined in the .cu files
int kit_build(const mlg_params* p);
int kit_free();
int launch_hfft(Scalar& s, int dir);             // dir -1 forward (1/np), +1 backward
int launch_hfft_rs(Scalar& s, int dir, const double* rs);   // with the rows times rs (before fwd / after bwd)
int launch_vfft(Scalar& s, int dir);             // dir -1 forward (1/nz), +1 backward
int launch_vfft_buf(cd* e, int dir);
int launch_vfft_scaled(cd* e, int dir, double scale);
int launch_hfft_fwd_scaled(cd* e, double scale);
int launch_hfft_bwd_buf(cd* e);
int launch_vfft_multi(Scalar* const* s, int n, int dir);   // n <= 6 fields in one pass
// the adjoint's FFTs of n <= 6 buffers in one pass
int launch_vfft_scaled_n(cd* const* e, int n, int dir, double scale);
int launch_hfft_fwd_scaled_n(cd* const* e, int n, double scale);
int launch_hfft_bwd_buf_n(cd* const* e, int n);
int launch_hfft_multi(Scalar* const* s, const double* const* rs, int n, int dir);
int launch_rtrans_fwd(Scalar& s);
int launch_rtrans_bwd(Scalar& s, bool add_ln);
int launch_rtrans_bwd_multi(Scalar* const* f, int n, bool add_ln);   // n <= 3 fields, one launch
int launch_rtrans_fwd_multi(Scalar* const* f, int n);                // n <= 3 fields, one launch
int launch_ln_adjust(Scalar& s, double sign);    // e(:nr,1,:) += sign * ln * lnx
void lu_cache_clear();
// the bounded-wait path of the tensor-core kernels on its own (xs_radial.cu)
int wait_selftest(long long limit, int arrive);
// exact-slice radial contractions on the tensor cores (xs_radial.cu): mode 0 forward, 1 backward, for
// m0 <= m < npc; plain: FP64-grade digits, else the mixed form's
bool xs_supported(int mode, int nrc, bool plain);
int xs_rtrans(int mode, const cd* in, cd* out, int nrc, int npc, int m0, const double* lnp, bool add_ln, bool plain);
int xs_rtrans_multi(int mode, const cd* const* in, cd* const* out, int nf, int nrc, int npc, int m0,
                    const double* const* lnp, bool add_ln, bool plain);
void xs_free();
// the mixed form's projection contraction as exact slices (xs_vec2tp.cu): psi, chi rows of
// m0 <= m < npc written
bool xv_supported();
int xv_contract(const cd* ur, const cd* up, const cd* uz, cd* psi, cd* chi, int nrc, int npc, int m0);
void xv_free();
int launch_vec2tp_contract(const cd* ur, const cd* up, const cd* uz, cd* psi, cd* chi, int nrc_off);
// zeros to the rows of a mixed-form contraction's output that its kernels leave unwritten (radial.cu)
int launch_zero_tails(cd* out, int mode, int nrc, int npc, int nzc, int nzcu);
int launch_zero_tails_n(cd* const* out, int n, int mode, int nrc, int npc, int nzc, int nzcu, cudaStream_t st = nullptr);

// pointwise
int launch_zero(cd* e);
int launch_copy(cd* dst, const cd* src);
int launch_copy_ln(double* dst, const double* src);
int launch_set_ln(double* dst, double v);
int launch_set_ln2(double* d1, double* d2, double v);
int launch_set_ln_n(double* const* d, int n, double v);   // n <= 6 slots

// grid-stride loop over n elements (32-bit indices: a field has < 2^32 entries)
#define GRID_STRIDE(i, n) for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < (unsigned)(n); i += gridDim.x * blockDim.x)
static inline int nblk(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

// scalar bookkeeping and operators shared by ops.cu and adjoint.cu
int scalar_init(Scalar& s, bool zero_ln = true);
void scalar_release(Scalar& s);
int assign(Scalar& d, const Scalar& s);   // e, ln, space, offsets
// one linear combination for k_lincomb: out = c0*a + c1*b + c2*c + c3*d (null inputs skipped), times
// post; ln likewise with separate coefficients
struct LinArgs {
  double2* out;
  const double2* in[4];
  double c[4];
  double* lnout;
  const double* lnin[4];
  double lc[4];
  double post;     // overall multiplier applied after the sum (e and ln)
  size_t n;
};
LinArgs lin_args(Scalar& out, std::initializer_list<std::pair<const Scalar*, double>> terms,
                 std::initializer_list<std::pair<const Scalar*, double>> lnterms, double post = 1.0, bool do_ln = true);
// up to four independent combinations (none reads another one's output) in one launch
int lincomb_n(std::initializer_list<LinArgs> combos);
// out = post * sum c_i in_i (e), ln likewise from lnterms unless do_ln is false
int lincomb(Scalar& out, std::initializer_list<std::pair<const Scalar*, double>> terms,
            std::initializer_list<std::pair<const Scalar*, double>> lnterms, double post = 1.0, bool do_ln = true);
struct Tmp {
  Scalar s;
  int rc = 0;
  Tmp() { rc = scalar_init(s, false); }   // every temporary is assigned (e and ln) before it is read
  ~Tmp() { if (s.e) scalar_release(s); }
};
#define TMP(name) Tmp name##_t; if (name##_t.rc) return name##_t.rc; Scalar& name = name##_t.s
// restores the precision form on scope exit
struct PrecisionScope {
  int saved;
  explicit PrecisionScope(int mode) : saved(G.precision) { G.precision = mode; }
  ~PrecisionScope() { G.precision = saved; }
};
int calcat_dev(Scalar& s, const double* at, bool zero_mode);
int scale_r(Scalar& s, int mode);   // rows i < nr times r_i (mode 0) or 1/r_i (mode 1)
int op_trans(Scalar& s, const char* space);
int op_chop(Scalar& s);
int op_dealias(Scalar& s);
int op_zeroat1(Scalar& s);
// the same operators on two fields in one launch where their chop and spaces agree (else one by one)
int op_chop2(Scalar& a, Scalar& b);
// chop (if chop) and then dealias (if dealias) of each of n <= 6 fields
int op_mask_n(Scalar* const* f, int n, bool chop, bool dealias);
int op_dealias2(Scalar& a, Scalar& b);
int op_zeroat1_2(Scalar& a, Scalar& b);
int op_band(Scalar& s, int op);
int op_tp2vec(const Scalar& psi, const Scalar& chi, Scalar& vr, Scalar& vp, Scalar& vz);
int op_tp2curlvec(const Scalar& psi, const Scalar& chi, Scalar& wr, Scalar& wp, Scalar& wz);
int op_vecprod(Scalar& vr, Scalar& vp, Scalar& vz, const Scalar& ur, const Scalar& up, const Scalar& uz);
int op_vec2tp(const Scalar& vr, const Scalar& vp, const Scalar& vz, Scalar& psi, Scalar& chi);
// keep (optional): six scalars that receive the velocity and vorticity (vr, vp, vz, wr, wp, wz, in PPP,
// vz without the background) the nonlinear term was formed from
// dealiased: psi and chi are dealiased already (the vortex step's own dealias ran just before), so the
// routine's first dealias is skipped
int op_advection_rhs(Scalar& psi, Scalar& chi, Scalar& nlpsi, Scalar& nlchi, const Scalar& uz,
                     Scalar* const* keep = nullptr, bool dealiased = false);
// write_prev = false leaves psip and chip unwritten: for every step of a run but its last, whose
// psip and chip no later step reads
int op_vortex_step_dev(Scalar& psi, Scalar& chi, Scalar& nlpsi, Scalar& nlchi, Scalar& psip, Scalar& chip, Scalar& nlpsip,
                       Scalar& nlchip, const Scalar& uz, double dt, double* gains_dev, Scalar* const* keep = nullptr,
                       bool write_prev = true);
int launch_band_apply(Scalar& s, int op, const ChopIdx& c);
int launch_band_apply_to(Scalar& dst, const Scalar& src, int op, const ChopIdx& c, double scale,
                         PostChop pc = PostChop{0, 0, 0, 0, 0}, cudaStream_t st = nullptr);
int launch_tp2vec_uv(Scalar& ur, Scalar& up, const Scalar& psi, const Scalar& chi, const ChopIdx& c,
                     PostChop pc = PostChop{0, 0, 0, 0, 0});
int launch_band_apply_T(Scalar& s, int op, const ChopIdx& c);
int launch_band_solve(Scalar& s, int kind, const ChopIdx& c, double alpha, double beta, double preln, int power);
int launch_band_solve_T(Scalar& s, int kind, const ChopIdx& c, double alpha);
int launch_band_solve_T_pair(Scalar& s1, Scalar& s2, const ChopIdx& c, double alpha);
int launch_ihelm_pair(Scalar& s1, Scalar& s2, const ChopIdx& c, double alpha);
int launch_abcn_rhs(Scalar& s, const Scalar& nl, const Scalar& nl_p, double dt, double a);

}  // namespace mlg

// ---------------------------------------------------------------------------------------------
// device helpers
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ float2 caddf(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csubf(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// FP64 <-> FP32 conversions on the integer pipe.  On GB300 the FP64 pipe runs ~1.3 ops per clock
// per SM, and cvt.f32.f64 / cvt.f64.f32 execute there; the mixed form converts every field element
// it touches, so doing it with integer ops keeps those kernels off the FP64 pipe.
// Round to nearest even; magnitudes below 2^-126 become signed zero; inf and NaN are kept.
__device__ __forceinline__ float d2f_fast(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  unsigned sign = hi & 0x80000000u;
  int e = (int)((hi >> 20) & 0x7FFu);
  unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  unsigned rest = lo & 0x1FFFFFFFu;
  int e32 = e - 1023 + 127;
  if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (((hi & 0xFFFFFu) | lo) ? 0x400000u : 0u));
  if (e32 <= 0) return __uint_as_float(sign);
  if (e32 >= 255) return __uint_as_float(sign | 0x7F800000u);
  unsigned r = sign | ((unsigned)e32 << 23) | m;
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) r += 1u;   // carries into the exponent
  return __uint_as_float(r);
}
__device__ __forceinline__ double f2d_fast(float y) {   // exact (FP32 subnormals become zero)
  unsigned f = __float_as_uint(y);
  unsigned sign = f & 0x80000000u;
  unsigned e = (f >> 23) & 0xFFu;
  unsigned m = f & 0x7FFFFFu;
  if (e == 0u) return __hiloint2double((int)sign, 0);
  unsigned hi = (e == 255u) ? (sign | 0x7FF00000u | (m >> 3)) : (sign | ((e + 896u) << 20) | (m >> 3));
  return __hiloint2double((int)hi, (int)(m << 29));
}
__device__ __forceinline__ float2 ld_c32(const double2* p) { double2 v = *p; return make_float2(d2f_fast(v.x), d2f_fast(v.y)); }
__device__ __forceinline__ void st_c32(double2* p, float2 v) { *p = make_double2(f2d_fast(v.x), f2d_fast(v.y)); }

static inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }
