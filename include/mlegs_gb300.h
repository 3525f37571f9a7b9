/*
 * mlegs_gb300.h — C ABI of the GB300 (sm_103a) implementation of the MLegS spectral hot path.
 *
 * Every entry point replaces one routine of the reference's Fortran operator API
 * (module mlegs_scalar, src/modules/mlegs_scalar.f90:95-450, and the kit initialiser
 * tfm_kit_init, src/submodules/mlegs_spectfm_init.f90:6-154).  The Fortran side binds these
 * through ISO_C_BINDING (interface module include/mlegs_gb300_iface.f90); Python binds them
 * through ctypes (mlegs_gb300/kit.py).
 *
 * Conventions
 *  - A field ("scalar") is an opaque handle owning a device-resident complex128 array of
 *    (nrdim, npdim, nzdim) in Fortran (column-major, r fastest) order, exactly the layout of
 *    the reference's scalar%e (mlegs_scalar.f90:25), plus ln, the three chop offsets and
 *    the space tag ("PPP", "PFP", "FFP", "FFF").
 *  - Every call returns an int status: MLG_OK (0) or one of the MLG_E* codes below, which
 *    stand for the reference's `stop` messages; mlg_last_error() gives the message text.
 *  - All work is enqueued on one CUDA stream (mlg_set_stream); calls return once enqueued,
 *    except those that hand a value back to the host (downloads, calcat0/1, svv_filter's
 *    gain), which synchronise that stream first.  Inside a call the library also runs work on
 *    a side stream of its own (forked from and joined back into the caller's stream with
 *    events before the call returns), so stream order with the caller's work is kept.
 *  - One transform kit per process, as in the reference (mlegs_spectfm_init.f90:15-16).
 */
#ifndef MLEGS_GB300_H
#define MLEGS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define MLG_OK              0
#define MLG_EPARAM          1   /* invalid kit parameter (tfm_kit_init stop messages, :35-62)      */
#define MLG_ENOKIT          2   /* kit not initialised / already initialised (:15, scalar ops :46)  */
#define MLG_ESPACE          3   /* wrong space tag for the operation (e.g. ops :80, :1069, :1270)   */
#define MLG_ECHOP           4   /* chopping offset too large (chop_index :2053-2055)                */
#define MLG_EALPHA          5   /* alpha == 0 in ihelm/ihelmp (:809-811, :928-931)                  */
#define MLG_EPOWER          6   /* helmp/ihelmp power not 4, 6 or 8 (:865-866, :917-918)            */
#define MLG_EINVISCID       7   /* febe/abcn with zero viscosity (:1174, :1234)                     */
#define MLG_ENONFINITE      8   /* non-finite vortex state (vortical_flow_3d.f90:397-409)           */
#define MLG_ECUDA           9   /* CUDA runtime error                                               */
#define MLG_EALLOC         10   /* device allocation failure                                        */
#define MLG_EHANDLE        11   /* invalid scalar handle / argument                                 */
#define MLG_ESINGULAR      12   /* singular banded system (lurc: lu factorization failure, bndmat_ops :396-399) */
#define MLG_ETIMEOUT       13   /* a bounded device-side wait ran out                               */
#define MLG_ESIZE          14   /* size beyond a fixed capacity                                     */

/* Precision forms. */
#define MLG_PLAIN_FP64      0   /* all-FP64: the drop-in form                                       */
#define MLG_MIXED           1   /* 42-bit sliced tensor-core Legendre contractions, FP32 FFTs       */

/* Kit parameters: the module globals of mlegs_base (src/modules/mlegs_base.f90:7-41). */
typedef struct mlg_params {
    int    nr, np, nz;                 /* collocation points (nr even; np, nz even 2^p3^q5^r or 1) */
    int    nrchop, npchop, nzchop;     /* spectral truncation                                      */
    double ell;                        /* Legendre map parameter                                   */
    double zlen;                       /* axial period                                             */
    double visc;                       /* viscosity                                                */
    int    hyperpow;                   /* hyperviscosity power (0, 4, 6, 8)                        */
    double hypervisc;                  /* hyperviscosity                                           */
    int    is_svv;                     /* spectral-vanishing-viscosity filter on/off               */
    double svv_cutoff, svv_target, svv_strength, svv_relax;
} mlg_params;

/* Fills p with the reference defaults (mlegs_base.f90:7-41). */
void mlg_params_default(mlg_params* p);

typedef struct mlg_scalar_s* mlg_scalar;

/* ---- kit ------------------------------------------------------------------------------- */
/* tfm%init() (mlegs_spectfm_init.f90:6-154): Gauss-Legendre nodes, map, lognorm and the
 * P_L^m table, generated on the GPU. */
int mlg_init(const mlg_params* p);
int mlg_finalize(void);
/* dims[0..8] = nrdim, npdim, nzdim, chopzl, chopzu, nrh(=nr/2), ne(=nrchop+14), npchop, nr */
int mlg_kit_dims(int* dims);
/* Copies a kit array to host memory: "x","w","r","ln","ak","lognorm","pf","at0","at1". */
int mlg_kit_get(const char* name, double* out, long long count);
/* Selects MLG_PLAIN_FP64 or MLG_MIXED for the transforms and contractions that follow. */
int mlg_set_precision(int mode);
int mlg_get_precision(int* mode);
/* Work stream (a cudaStream_t passed as void*); NULL selects the legacy default stream. */
int mlg_set_stream(void* stream);
int mlg_sync(void);
const char* mlg_last_error(void);
/* Bytes of device memory currently held by the library (fields, tables, workspaces). */
long long mlg_mem_bytes(void);
long long mlg_mem_high_water(void);
/* Number of kernels the library has launched since mlg_init. */
long long mlg_launch_count(void);

/* ---- scalar container: type(scalar) (mlegs_scalar.f90:15-49, mlegs_scalar_init.f90) ------ */
int mlg_scalar_alloc(mlg_scalar* s);               /* scalar_init: space 'PPP', ln 0, offsets 0 */
int mlg_scalar_free(mlg_scalar s);                 /* scalar_dealloc                            */
/* e: host complex128 (re,im interleaved) array of nrdim*npdim*nzdim, Fortran order. */
int mlg_scalar_upload(mlg_scalar s, const double* e, double ln, const char* space);
int mlg_scalar_download(mlg_scalar s, double* e, double* ln, char* space4);
/* Same as upload/download, with a device pointer to nrdim*npdim*nzdim complex128 values. */
int mlg_scalar_upload_device(mlg_scalar s, const void* dev_e, double ln, const char* space);
int mlg_scalar_download_device(mlg_scalar s, void* dev_e, double* ln, char* space4);
int mlg_scalar_copy(mlg_scalar dst, mlg_scalar src);            /* assignment(=) :106-140 */
int mlg_scalar_chop_offset(mlg_scalar s, int iof1, int iof2, int iof3); /* :84-103 */
int mlg_scalar_get_meta(mlg_scalar s, double* ln, char* space4, int* offsets3);
int mlg_scalar_set_ln(mlg_scalar s, double ln);
int mlg_scalar_set_space(mlg_scalar s, const char* space);
/* dst%e = a*x%e + b*y%e (y may be NULL), ln and tags of dst unchanged: the device-side form of the
 * apps' direct array arithmetic on s%e (e.g. the Richardson step, vortical_flow_3d.f90:136-137). */
int mlg_scalar_axpby(mlg_scalar dst, double a, mlg_scalar x, double b, mlg_scalar y);
/* Raw device pointer of the field (for interop).  Valid until the scalar is freed or passed to a
 * call that transforms it (trans, and the operators that move it between spaces): a radial transform
 * writes into a fresh buffer and the scalar takes it.  Query it again after such calls. */
void* mlg_scalar_device_ptr(mlg_scalar s);

/* ---- transforms and masks (mlegs_scalar_ops.f90) -------------------------------------- */
int mlg_trans(mlg_scalar s, const char* space);             /* trans      :157-235 */
int mlg_chop(mlg_scalar s);                                 /* chop       :6-41    */
int mlg_dealias(mlg_scalar s);                              /* dealias    :43-70   */
int mlg_svv_filter(mlg_scalar s, double* gain);             /* svv_filter :72-155  */
int mlg_calcat0(mlg_scalar s, double* out_c);               /* calcat0    :237-272 (nz complex) */
int mlg_calcat1(mlg_scalar s, double* out_c);               /* calcat1    :274-309 */
int mlg_zeroat1(mlg_scalar s);                              /* zeroat1    :311-325 */

/* ---- banded spectral operators and solves ---------------------------------------------- */
int mlg_delsqp(mlg_scalar s);                               /* :327-366  */
int mlg_idelsqp(mlg_scalar s);                              /* :368-416  */
int mlg_xxdx(mlg_scalar s);                                 /* :418-463  */
int mlg_del2h(mlg_scalar s);                                /* :465-518  */
int mlg_del2(mlg_scalar s);                                 /* :520-573  */
int mlg_idel2_preln(mlg_scalar s, double preln);            /* :575-669  */
int mlg_idel2_proln(mlg_scalar s);                          /* :671-760  */
int mlg_helm(mlg_scalar s, double alpha);                   /* :762-789  */
int mlg_ihelm(mlg_scalar s, double alpha);                  /* :791-854  */
/* ihelm without any device allocation; no counterpart in the reference.  For callers whose host
 * owns all device memory (a fixed arena or its own allocator) or that forbid allocation inside
 * their step loop.  e_dev: caller-owned device field (nrdim, npdim, nzdim) complex128 in FFF space
 * with zero chop offsets, solved in place; *ln: the field's ln on input, ln/alpha on output.  The
 * only workspace is a fixed 16 MiB device array inside the library (held by every GPU that loads
 * it); radial systems are processed in batches that fit it, and a single system that does not fit
 * is rejected with MLG_ESIZE.  The first call with a given device current looks up that array's
 * device address; make that call before any stream capture.  Calls that overlap on the GPU share
 * the array and race. */
int mlg_ihelm_noalloc(void* e_dev, double* ln, double alpha);
int mlg_helmp(mlg_scalar s, int power, double alpha, double beta);   /* :856-903  */
int mlg_ihelmp(mlg_scalar s, int power, double alpha, double beta);  /* :905-1000 */

/* ---- time steppers ---------------------------------------------------------------------- */
int mlg_fefe(mlg_scalar s, mlg_scalar nl, double dt);                                  /* :1065-1094 */
int mlg_abab(mlg_scalar s, mlg_scalar s_p, mlg_scalar nl, mlg_scalar nl_p, double dt,
             int is_2nd_svis_p);                                                       /* :1096-1155 */
int mlg_febe(mlg_scalar s, mlg_scalar nl, double dt);                                  /* :1157-1198 */
int mlg_abcn(mlg_scalar s, mlg_scalar s_p, mlg_scalar nl, mlg_scalar nl_p, double dt); /* :1200-1262 */

/* ---- vector fields in toroidal/poloidal form ------------------------------------------- */
int mlg_vecprod(mlg_scalar vr, mlg_scalar vp, mlg_scalar vz,
                mlg_scalar ur, mlg_scalar up, mlg_scalar uz);                          /* :1264-1306 */
int mlg_vec2tp(mlg_scalar vr, mlg_scalar vp, mlg_scalar vz, mlg_scalar psi, mlg_scalar chi); /* :1308-1453 */
int mlg_tp2vec(mlg_scalar psi, mlg_scalar chi, mlg_scalar vr, mlg_scalar vp, mlg_scalar vz); /* :1455-1545 */
int mlg_tp2curlvec(mlg_scalar psi, mlg_scalar chi, mlg_scalar wr, mlg_scalar wp, mlg_scalar wz); /* :1547-1560 */

/* ---- 3-D vortex driver (src/apps/vortical_flow_3d.f90) ------------------------------------ */
/* advection_rhs (:353-395): nlpsi, nlchi <- TP projection of -(curl V) x (V + uz e_z). */
int mlg_advection_rhs(mlg_scalar psi, mlg_scalar chi, mlg_scalar nlpsi, mlg_scalar nlchi,
                      mlg_scalar uz);
/* One main-loop step (:168-180): abcn(psi), abcn(chi), dealias, svv_filter (gains updated in
 * gains[0..1]), zeroat1, advection_rhs, check_stability. */
int mlg_vortex_step(mlg_scalar psi, mlg_scalar chi, mlg_scalar nlpsi, mlg_scalar nlchi,
                    mlg_scalar psi_p, mlg_scalar chi_p, mlg_scalar nlpsi_p, mlg_scalar nlchi_p,
                    mlg_scalar uz, double dt, double* gains);
/* nsteps of mlg_vortex_step with the SVV gains and the finiteness flag kept on the device
 * (no host synchronisation inside the loop; gains copied back at the end).  The eight fields end
 * as after nsteps calls of mlg_vortex_step.  Both calls hand nlpsi's and nlchi's buffers to nlpsi_p
 * and nlchi_p each step (the step recomputes nlpsi and nlchi), so the device pointers of those four
 * scalars change; a run writes psi_p and chi_p on its last step only.  With nsteps >= 4 the interior
 * steps replay a CUDA graph of two steps (same kernels, same buffers, same bytes). */
int mlg_vortex_run(mlg_scalar psi, mlg_scalar chi, mlg_scalar nlpsi, mlg_scalar nlchi,
                   mlg_scalar psi_p, mlg_scalar chi_p, mlg_scalar nlpsi_p, mlg_scalar nlchi_p,
                   mlg_scalar uz, double dt, int nsteps, double* gains);

/* ---- adjoint (no counterpart in the reference) ------------------------------------------- */
/* Inner product for every adjoint below: <a, b> = sum over the whole stored array of
 * Re(conj(a.e) b.e) + a.ln * b.ln.  Each mlg_adj_* applies the exact transpose of the named forward
 * entry point (as implemented here) in place on an adjoint variable.  Requires is_svv = 0 and
 * hyperpow = 0 (MLG_EPARAM otherwise). */
/* The gradient of J = 1/2 sum W |u'|^2 at step nsteps of the vortex step sequence started from
 * (psi0, chi0) [psi <- psi0, nl <- advection_rhs, nl_p <- nl, then mlg_vortex_step nsteps times],
 * u' the velocity without the (m = 0, k = 0) column and ln, W the volume quadrature weights
 * w_i r_i^2/(1-x_i^2) (2 pi/np)(zlen/nz).  The forward state is kept every k_ckpt steps and each
 * segment recomputed on the way back.  The gradient is with respect to the active coefficients (those
 * that chop and dealias keep, which is where the step keeps its state); it is zero elsewhere.
 * grad_psi/grad_chi NULL: J only.  psi0, chi0 unchanged. */
int mlg_adjoint_run(mlg_scalar psi0, mlg_scalar chi0, mlg_scalar uz, double dt, int nsteps, int k_ckpt,
                    mlg_scalar grad_psi, mlg_scalar grad_chi, double* J);
/* One step: state = (psi, chi, nlpsi, nlchi, nlpsi_p, nlchi_p) at the step's start (unchanged);
 * adj = the adjoint of the state at its end, replaced by the adjoint at its start. */
int mlg_adj_vortex_step(const mlg_scalar* state, mlg_scalar uz, double dt, const mlg_scalar* adj);
int mlg_adj_trans(mlg_scalar s, const char* forward_from_space);  /* s.space: the forward's target */
int mlg_adj_band(mlg_scalar s, int op);          /* op 0 xxdx, 1 del2h, 2 del2 */
int mlg_adj_ihelm(mlg_scalar s, double alpha);
int mlg_adj_idel2_proln(mlg_scalar s);
int mlg_adj_zeroat1(mlg_scalar s);
int mlg_adj_tp2vec(mlg_scalar vr_bar, mlg_scalar vp_bar, mlg_scalar vz_bar, mlg_scalar psi_bar, mlg_scalar chi_bar);
int mlg_adj_tp2curlvec(mlg_scalar wr_bar, mlg_scalar wp_bar, mlg_scalar wz_bar, mlg_scalar psi_bar, mlg_scalar chi_bar);
int mlg_adj_vec2tp(mlg_scalar psi_bar, mlg_scalar chi_bar, mlg_scalar vr_bar, mlg_scalar vp_bar, mlg_scalar vz_bar);
/* advection_rhs linearised at (psi, chi) (not modified): (nlpsi_bar, nlchi_bar) -> (psi_bar, chi_bar) */
int mlg_adj_advection(mlg_scalar psi, mlg_scalar chi, mlg_scalar uz, mlg_scalar nlpsi_bar, mlg_scalar nlchi_bar,
                      mlg_scalar psi_bar, mlg_scalar chi_bar);

/* ---- field I/O (src/submodules/mlegs_scalar_io.f90) ---------------------------------------- */
/* msave (:6-103): the field, ln, chop offsets and space tag to the file fn.
 *  is_binary != 0: stream-access unformatted -- the three sizes as int32, the complex128 array in
 *    Fortran order, ln as float64, the three chop offsets as int32, the 3-character space tag;
 *  is_binary == 0: formatted -- the sizes as '(3(1X,I10))', then for each z and each radial row one
 *    line of 2*npdim values (re, im) as '1PE24.15E3', a blank line between z blocks, then a line with
 *    ln and the offsets and a line with the space tag.
 *  is_global != 0: one file fn with the global layout above; is_global == 0: the per-rank form, file
 *    fn_0, whose header holds the global size, local size and local start (one process: the whole
 *    array).  The reference's optional arguments default to formatted and global. */
int mlg_msave(mlg_scalar s, const char* fn, int is_binary, int is_global);
/* mload (:105-249): the inverse of mlg_msave into s (device).  The stored sizes must equal
 * (nrdim, npdim, nzdim) (MLG_ESIZE, the reference's 'size inconsistency'); a file that cannot be
 * opened or parsed gives MLG_EPARAM. */
int mlg_mload(mlg_scalar s, const char* fn, int is_binary, int is_global);

/* ---- diagnostics ------------------------------------------------------------------------- */
/* fftreat (mlegs_scalar_ops.f90:1002-1063): delsqp, to (physical r, Fourier phi, z), the rows times
 * (1-x)^2, rows from 3nr/4+4 of m >= 1 zeroed, five passes of smooth over the rows from 3nr/4,
 * divided by (1-x)^2, back, idelsqp (ln kept), zeroat1; in place on an FFF field. */
int mlg_fftreat(mlg_scalar s);
/* The field of save_vort_mag (src/apps/vortical_flow_3d.f90:411-465), without the file: out (PPP,
 * ln 0) <- |curl v| of the velocity of (psi, chi) per physical sample (the real and imaginary parts
 * of each slot are the two packed phi samples).  psi, chi: FFF, unchanged. */
int mlg_vort_mag(mlg_scalar psi, mlg_scalar chi, mlg_scalar out);
/* Kinetic-energy spectrum of the velocity v of (psi, chi): E[m + npdim*k] = 1/2 sum_i W_i c_m
 * sum_{v_r, v_phi, v_z} |v_hat(i, m, k)|^2, v_hat the phi (1/np) and z (1/nz) Fourier coefficients of
 * the physical samples, W_i = w_i r_i^2/(1-x_i^2) 2 pi zlen, c_m = 1 for m = 0 and m = np/2, else 2:
 * sum over (m, k) is the kinetic energy.  Computed in FP64 in either precision form. */
int mlg_ke_spectrum(mlg_scalar psi, mlg_scalar chi, double* E);

/* ---- parameter file: read_input (src/submodules/mlegs_misc_io.f90:307-388) ---------------- */
/* The time-stepping and output settings of the input file besides the kit parameters. */
typedef struct mlg_run_params {
    double dt, ti, totaltime;
    int    ni, totaln;
    int    isfldsav, fldsavintvl;
    int    islogsav, logsavintvl;
    char   flddir[260];                /* with a trailing '/'                                      */
    char   logdir[260];
} mlg_run_params;
/* Reads fn in the reference's layout (a comment line before each group of values; the optional SVV
 * line at the end) into p (the reference defaults for anything the file leaves out) and run, and
 * checks it as read_input does (MLG_EPARAM with the reference's message).  make_dirs != 0 creates
 * flddir and logdir (mkdir -p) as the reference does. */
int mlg_read_input(const char* fn, mlg_params* p, mlg_run_params* run, int make_dirs);

/* ---- diagnostics of the bounded device waits (no counterpart in the reference) ------------ */
/* Every wait of a tensor-core kernel on an mbarrier gives up after about a second of SM clock, sets a
 * timeout word in device memory and lets the kernel return; the next mlg_sync (or vortex step/run)
 * then returns MLG_ETIMEOUT.  This call enqueues one thread that takes that same path on an mbarrier:
 * arrive = 0, nothing arrives and the wait runs out after limit_clocks (0 .. 2e9); arrive = 1, the
 * thread arrives first and the wait succeeds.  It lets a host check, without any fault, that a wait
 * that runs out reaches it as MLG_ETIMEOUT. */
int mlg_selftest_bounded_wait(long long limit_clocks, int arrive);

/* ---- kernel timing (CUDA events around each launch of one kernel class) ----------------- */
/* kind: 0 = forward radial Legendre contraction, 1 = FFTs, 2 = banded operators (applies and the
 *       fused abcn right-hand side), 3 = backward radial contraction, 4 = vec2tp projection
 *       contraction, 5 = banded solves (substitutions with cached factors).  work = flops for the
 *       contractions, algorithmic bytes (each field read and written once, tables and factors read
 *       once) for the others. */
int mlg_kernel_timing(int enable);
int mlg_kernel_timing_read(int kind, double* total_ms, long long* launches, double* flops_or_bytes);

#ifdef __cplusplus
}
#endif
#endif /* MLEGS_GB300_H */
