! mlegs_gb300_iface.f90 — ISO_C_BINDING interface of the GB300 library for the MLegS Fortran host.
!
! Binds every entry point of include/mlegs_gb300.h, and wraps them in a module `mlegs_scalar_gpu`
! whose procedure names and argument meaning follow the reference's `module mlegs_scalar`
! (src/modules/mlegs_scalar.f90:95-450): a Fortran app switches by replacing
!   use mlegs_scalar            ->   use mlegs_scalar_gpu
!   type(scalar) :: s           ->   type(scalar_gpu) :: s
! and keeps its calls (call trans(s, 'FFF', tfm), call ihelm(s, alpha, tfm), ...).  The kit argument
! is accepted and ignored: the GPU kit is the process singleton created by gpu_kit_init.
! A non-zero status stops the program with the library's message, as the reference's `stop` does.
! Beyond the reference's routines the wrapper module exposes the 3-D vortex step and run
! (src/apps/vortical_flow_3d.f90:160-206), the adjoint (no counterpart in the reference), the
! device-side linear combination the apps write as array arithmetic on s%e (:136-137), read_input
! (src/submodules/mlegs_misc_io.f90:307-388) and the stream, precision and sync controls.
module mlegs_gb300_c
  use iso_c_binding
  implicit none

  type, bind(c) :: mlg_params
    integer(c_int) :: nr, np, nz, nrchop, npchop, nzchop
    real(c_double) :: ell, zlen, visc
    integer(c_int) :: hyperpow
    real(c_double) :: hypervisc
    integer(c_int) :: is_svv
    real(c_double) :: svv_cutoff, svv_target, svv_strength, svv_relax
  end type

  type, bind(c) :: mlg_run_params
    real(c_double) :: dt, ti, totaltime
    integer(c_int) :: ni, totaln
    integer(c_int) :: isfldsav, fldsavintvl
    integer(c_int) :: islogsav, logsavintvl
    character(kind=c_char) :: flddir(260)
    character(kind=c_char) :: logdir(260)
  end type

  integer(c_int), parameter :: MLG_PLAIN_FP64 = 0, MLG_MIXED = 1

  interface
    ! ---- kit, precision, stream ----
    subroutine mlg_params_default(p) bind(c, name='mlg_params_default')
      import :: mlg_params
      type(mlg_params), intent(out) :: p
    end subroutine
    integer(c_int) function mlg_init(p) bind(c, name='mlg_init')
      import :: c_int, mlg_params
      type(mlg_params), intent(in) :: p
    end function
    integer(c_int) function mlg_finalize() bind(c, name='mlg_finalize')
      import :: c_int
    end function
    integer(c_int) function mlg_kit_dims(d) bind(c, name='mlg_kit_dims')
      import :: c_int
      integer(c_int), intent(out) :: d(9)
    end function
    integer(c_int) function mlg_kit_get(name, out, count) bind(c, name='mlg_kit_get')
      import :: c_int, c_char, c_double, c_long_long
      character(kind=c_char), intent(in) :: name(*)
      real(c_double), intent(out) :: out(*)
      integer(c_long_long), value :: count
    end function
    integer(c_int) function mlg_set_precision(mode) bind(c, name='mlg_set_precision')
      import :: c_int
      integer(c_int), value :: mode
    end function
    integer(c_int) function mlg_get_precision(mode) bind(c, name='mlg_get_precision')
      import :: c_int
      integer(c_int), intent(out) :: mode
    end function
    integer(c_int) function mlg_set_stream(stream) bind(c, name='mlg_set_stream')
      import :: c_int, c_ptr
      type(c_ptr), value :: stream
    end function
    integer(c_int) function mlg_sync() bind(c, name='mlg_sync')
      import :: c_int
    end function
    type(c_ptr) function mlg_last_error() bind(c, name='mlg_last_error')
      import :: c_ptr
    end function
    integer(c_long_long) function mlg_mem_bytes() bind(c, name='mlg_mem_bytes')
      import :: c_long_long
    end function
    integer(c_long_long) function mlg_mem_high_water() bind(c, name='mlg_mem_high_water')
      import :: c_long_long
    end function
    integer(c_long_long) function mlg_launch_count() bind(c, name='mlg_launch_count')
      import :: c_long_long
    end function

    ! ---- scalar container ----
    integer(c_int) function mlg_scalar_alloc(s) bind(c, name='mlg_scalar_alloc')
      import :: c_int, c_ptr
      type(c_ptr), intent(out) :: s
    end function
    integer(c_int) function mlg_scalar_free(s) bind(c, name='mlg_scalar_free')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_scalar_upload(s, e, ln, space) bind(c, name='mlg_scalar_upload')
      import :: c_int, c_ptr, c_double, c_double_complex, c_char
      type(c_ptr), value :: s
      complex(c_double_complex), intent(in) :: e(*)
      real(c_double), value :: ln
      character(kind=c_char), intent(in) :: space(*)
    end function
    integer(c_int) function mlg_scalar_download(s, e, ln, space4) bind(c, name='mlg_scalar_download')
      import :: c_int, c_ptr, c_double, c_double_complex, c_char
      type(c_ptr), value :: s
      complex(c_double_complex), intent(out) :: e(*)
      real(c_double), intent(out) :: ln
      character(kind=c_char), intent(out) :: space4(4)
    end function
    integer(c_int) function mlg_scalar_upload_device(s, dev_e, ln, space) bind(c, name='mlg_scalar_upload_device')
      import :: c_int, c_ptr, c_double, c_char
      type(c_ptr), value :: s, dev_e
      real(c_double), value :: ln
      character(kind=c_char), intent(in) :: space(*)
    end function
    integer(c_int) function mlg_scalar_download_device(s, dev_e, ln, space4) bind(c, name='mlg_scalar_download_device')
      import :: c_int, c_ptr, c_double, c_char
      type(c_ptr), value :: s, dev_e
      real(c_double), intent(out) :: ln
      character(kind=c_char), intent(out) :: space4(4)
    end function
    integer(c_int) function mlg_scalar_copy(d, s) bind(c, name='mlg_scalar_copy')
      import :: c_int, c_ptr
      type(c_ptr), value :: d, s
    end function
    integer(c_int) function mlg_scalar_chop_offset(s, a, b, c) bind(c, name='mlg_scalar_chop_offset')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
      integer(c_int), value :: a, b, c
    end function
    integer(c_int) function mlg_scalar_get_meta(s, ln, space4, offsets3) bind(c, name='mlg_scalar_get_meta')
      import :: c_int, c_ptr, c_double, c_char
      type(c_ptr), value :: s
      real(c_double), intent(out) :: ln
      character(kind=c_char), intent(out) :: space4(4)
      integer(c_int), intent(out) :: offsets3(3)
    end function
    integer(c_int) function mlg_scalar_set_ln(s, ln) bind(c, name='mlg_scalar_set_ln')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      real(c_double), value :: ln
    end function
    integer(c_int) function mlg_scalar_set_space(s, space) bind(c, name='mlg_scalar_set_space')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: s
      character(kind=c_char), intent(in) :: space(*)
    end function
    integer(c_int) function mlg_scalar_axpby(d, a, x, b, y) bind(c, name='mlg_scalar_axpby')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: d, x, y
      real(c_double), value :: a, b
    end function
    type(c_ptr) function mlg_scalar_device_ptr(s) bind(c, name='mlg_scalar_device_ptr')
      import :: c_ptr
      type(c_ptr), value :: s
    end function

    ! ---- transforms and masks ----
    integer(c_int) function mlg_trans(s, space) bind(c, name='mlg_trans')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: s
      character(kind=c_char), intent(in) :: space(*)
    end function
    integer(c_int) function mlg_chop(s) bind(c, name='mlg_chop')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_dealias(s) bind(c, name='mlg_dealias')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_svv_filter(s, gain) bind(c, name='mlg_svv_filter')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      real(c_double), intent(inout) :: gain
    end function
    integer(c_int) function mlg_calcat0(s, out) bind(c, name='mlg_calcat0')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: s
      complex(c_double_complex), intent(out) :: out(*)
    end function
    integer(c_int) function mlg_calcat1(s, out) bind(c, name='mlg_calcat1')
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: s
      complex(c_double_complex), intent(out) :: out(*)
    end function
    integer(c_int) function mlg_zeroat1(s) bind(c, name='mlg_zeroat1')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function

    ! ---- banded operators and solves ----
    integer(c_int) function mlg_delsqp(s) bind(c, name='mlg_delsqp')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_idelsqp(s) bind(c, name='mlg_idelsqp')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_xxdx(s) bind(c, name='mlg_xxdx')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_del2h(s) bind(c, name='mlg_del2h')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_del2(s) bind(c, name='mlg_del2')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_idel2_preln(s, preln) bind(c, name='mlg_idel2_preln')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      real(c_double), value :: preln
    end function
    integer(c_int) function mlg_idel2_proln(s) bind(c, name='mlg_idel2_proln')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_helm(s, alpha) bind(c, name='mlg_helm')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      real(c_double), value :: alpha
    end function
    integer(c_int) function mlg_ihelm(s, alpha) bind(c, name='mlg_ihelm')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      real(c_double), value :: alpha
    end function
    integer(c_int) function mlg_ihelm_noalloc(e_dev, ln, alpha) bind(c, name='mlg_ihelm_noalloc')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: e_dev
      real(c_double), intent(inout) :: ln
      real(c_double), value :: alpha
    end function
    integer(c_int) function mlg_helmp(s, power, alpha, beta) bind(c, name='mlg_helmp')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      integer(c_int), value :: power
      real(c_double), value :: alpha, beta
    end function
    integer(c_int) function mlg_ihelmp(s, power, alpha, beta) bind(c, name='mlg_ihelmp')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      integer(c_int), value :: power
      real(c_double), value :: alpha, beta
    end function

    ! ---- time steppers ----
    integer(c_int) function mlg_fefe(s, nl, dt) bind(c, name='mlg_fefe')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s, nl
      real(c_double), value :: dt
    end function
    integer(c_int) function mlg_febe(s, nl, dt) bind(c, name='mlg_febe')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s, nl
      real(c_double), value :: dt
    end function
    integer(c_int) function mlg_abab(s, sp, nl, nlp, dt, is2nd) bind(c, name='mlg_abab')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s, sp, nl, nlp
      real(c_double), value :: dt
      integer(c_int), value :: is2nd
    end function
    integer(c_int) function mlg_abcn(s, sp, nl, nlp, dt) bind(c, name='mlg_abcn')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s, sp, nl, nlp
      real(c_double), value :: dt
    end function

    ! ---- vector fields ----
    integer(c_int) function mlg_vecprod(vr, vp, vz, ur, up, uz) bind(c, name='mlg_vecprod')
      import :: c_int, c_ptr
      type(c_ptr), value :: vr, vp, vz, ur, up, uz
    end function
    integer(c_int) function mlg_vec2tp(vr, vp, vz, psi, chi) bind(c, name='mlg_vec2tp')
      import :: c_int, c_ptr
      type(c_ptr), value :: vr, vp, vz, psi, chi
    end function
    integer(c_int) function mlg_tp2vec(psi, chi, vr, vp, vz) bind(c, name='mlg_tp2vec')
      import :: c_int, c_ptr
      type(c_ptr), value :: psi, chi, vr, vp, vz
    end function
    integer(c_int) function mlg_tp2curlvec(psi, chi, wr, wp, wz) bind(c, name='mlg_tp2curlvec')
      import :: c_int, c_ptr
      type(c_ptr), value :: psi, chi, wr, wp, wz
    end function

    ! ---- 3-D vortex driver ----
    integer(c_int) function mlg_advection_rhs(psi, chi, nlpsi, nlchi, uz) bind(c, name='mlg_advection_rhs')
      import :: c_int, c_ptr
      type(c_ptr), value :: psi, chi, nlpsi, nlchi, uz
    end function
    integer(c_int) function mlg_vortex_step(psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz, dt, gains) &
        bind(c, name='mlg_vortex_step')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz
      real(c_double), value :: dt
      real(c_double), intent(inout) :: gains(2)
    end function
    integer(c_int) function mlg_vortex_run(psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz, dt, nsteps, &
        gains) bind(c, name='mlg_vortex_run')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz
      real(c_double), value :: dt
      integer(c_int), value :: nsteps
      real(c_double), intent(inout) :: gains(2)
    end function

    ! ---- adjoint (no counterpart in the reference) ----
    integer(c_int) function mlg_adjoint_run(psi0, chi0, uz, dt, nsteps, k_ckpt, grad_psi, grad_chi, j) &
        bind(c, name='mlg_adjoint_run')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: psi0, chi0, uz, grad_psi, grad_chi
      real(c_double), value :: dt
      integer(c_int), value :: nsteps, k_ckpt
      real(c_double), intent(out) :: j
    end function
    integer(c_int) function mlg_adj_vortex_step(state, uz, dt, adj) bind(c, name='mlg_adj_vortex_step')
      import :: c_int, c_ptr, c_double
      type(c_ptr), intent(in) :: state(6), adj(6)
      type(c_ptr), value :: uz
      real(c_double), value :: dt
    end function
    integer(c_int) function mlg_adj_trans(s, forward_from_space) bind(c, name='mlg_adj_trans')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: s
      character(kind=c_char), intent(in) :: forward_from_space(*)
    end function
    integer(c_int) function mlg_adj_band(s, op) bind(c, name='mlg_adj_band')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
      integer(c_int), value :: op
    end function
    integer(c_int) function mlg_adj_ihelm(s, alpha) bind(c, name='mlg_adj_ihelm')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: s
      real(c_double), value :: alpha
    end function
    integer(c_int) function mlg_adj_idel2_proln(s) bind(c, name='mlg_adj_idel2_proln')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_adj_zeroat1(s) bind(c, name='mlg_adj_zeroat1')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_adj_tp2vec(vr_bar, vp_bar, vz_bar, psi_bar, chi_bar) bind(c, name='mlg_adj_tp2vec')
      import :: c_int, c_ptr
      type(c_ptr), value :: vr_bar, vp_bar, vz_bar, psi_bar, chi_bar
    end function
    integer(c_int) function mlg_adj_tp2curlvec(wr_bar, wp_bar, wz_bar, psi_bar, chi_bar) bind(c, name='mlg_adj_tp2curlvec')
      import :: c_int, c_ptr
      type(c_ptr), value :: wr_bar, wp_bar, wz_bar, psi_bar, chi_bar
    end function
    integer(c_int) function mlg_adj_vec2tp(psi_bar, chi_bar, vr_bar, vp_bar, vz_bar) bind(c, name='mlg_adj_vec2tp')
      import :: c_int, c_ptr
      type(c_ptr), value :: psi_bar, chi_bar, vr_bar, vp_bar, vz_bar
    end function
    integer(c_int) function mlg_adj_advection(psi, chi, uz, nlpsi_bar, nlchi_bar, psi_bar, chi_bar) &
        bind(c, name='mlg_adj_advection')
      import :: c_int, c_ptr
      type(c_ptr), value :: psi, chi, uz, nlpsi_bar, nlchi_bar, psi_bar, chi_bar
    end function

    ! ---- field I/O, diagnostics, parameter file ----
    integer(c_int) function mlg_msave(s, fn, is_binary, is_global) bind(c, name='mlg_msave')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: s
      character(kind=c_char), intent(in) :: fn(*)
      integer(c_int), value :: is_binary, is_global
    end function
    integer(c_int) function mlg_mload(s, fn, is_binary, is_global) bind(c, name='mlg_mload')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: s
      character(kind=c_char), intent(in) :: fn(*)
      integer(c_int), value :: is_binary, is_global
    end function
    integer(c_int) function mlg_fftreat(s) bind(c, name='mlg_fftreat')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
    end function
    integer(c_int) function mlg_vort_mag(psi, chi, out) bind(c, name='mlg_vort_mag')
      import :: c_int, c_ptr
      type(c_ptr), value :: psi, chi, out
    end function
    integer(c_int) function mlg_ke_spectrum(psi, chi, e) bind(c, name='mlg_ke_spectrum')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: psi, chi
      real(c_double), intent(out) :: e(*)
    end function
    integer(c_int) function mlg_read_input(fn, p, run, make_dirs) bind(c, name='mlg_read_input')
      import :: c_int, c_char, mlg_params, mlg_run_params
      character(kind=c_char), intent(in) :: fn(*)
      type(mlg_params), intent(out) :: p
      type(mlg_run_params), intent(out) :: run
      integer(c_int), value :: make_dirs
    end function

    ! ---- diagnostics of the bounded device waits, kernel timing ----
    integer(c_int) function mlg_selftest_bounded_wait(limit_clocks, arrive) bind(c, name='mlg_selftest_bounded_wait')
      import :: c_int, c_long_long
      integer(c_long_long), value :: limit_clocks
      integer(c_int), value :: arrive
    end function
    integer(c_int) function mlg_kernel_timing(enable) bind(c, name='mlg_kernel_timing')
      import :: c_int
      integer(c_int), value :: enable
    end function
    integer(c_int) function mlg_kernel_timing_read(kind, total_ms, launches, work) bind(c, name='mlg_kernel_timing_read')
      import :: c_int, c_double, c_long_long
      integer(c_int), value :: kind
      real(c_double), intent(out) :: total_ms, work
      integer(c_long_long), intent(out) :: launches
    end function
  end interface
end module

module mlegs_scalar_gpu
  ! the reference's operator names over device-resident fields
  use iso_c_binding
  use mlegs_gb300_c
  implicit none
  private

  type, public :: scalar_gpu
    type(c_ptr) :: h = c_null_ptr
  end type

  public :: MLG_PLAIN_FP64, MLG_MIXED, mlg_params, mlg_run_params
  public :: gpu_kit_init, gpu_kit_finalize, set_precision, set_stream, gpu_sync, read_input
  public :: scalar_init, scalar_free, upload, download, copy, chop_offset, set_ln, set_space, axpby
  public :: trans, chop, dealias, svv_filter, calcat0, calcat1, zeroat1, delsqp, idelsqp, xxdx, del2h, del2
  public :: idel2, helm, ihelm, helmp, ihelmp, fefe, abab, febe, abcn, vecprod, vec2tp, tp2vec, tp2curlvec
  public :: advection_rhs, vortex_step, vortex_run, adjoint_run
  public :: msave, mload, fftreat, vort_mag, ke_spectrum

  interface idel2
    module procedure idel2_preln, idel2_proln
  end interface

contains

  subroutine check(rc)
    integer(c_int), intent(in) :: rc
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == 0) return
    call c_f_pointer(mlg_last_error(), msg, [512])
    n = 0
    do while (n < 512)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    enddo
    write(*,*) 'mlegs_gb300: ', msg(1:n)
    stop
  end subroutine

  ! ---- kit, precision, stream ----
  subroutine gpu_kit_init(nr, np, nz, nrchop, npchop, nzchop, ell, zlen, visc, hyperpow, hypervisc, is_svv, &
                          svv_cutoff, svv_target, svv_strength, svv_relax)
    integer, intent(in) :: nr, np, nz, nrchop, npchop, nzchop, hyperpow
    real(c_double), intent(in) :: ell, zlen, visc, hypervisc, svv_cutoff, svv_target, svv_strength, svv_relax
    logical, intent(in) :: is_svv
    type(mlg_params) :: p
    p = mlg_params(nr, np, nz, nrchop, npchop, nzchop, ell, zlen, visc, hyperpow, hypervisc, &
                   merge(1, 0, is_svv), svv_cutoff, svv_target, svv_strength, svv_relax)
    call check(mlg_init(p))
  end subroutine
  subroutine gpu_kit_finalize()
    call check(mlg_finalize())
  end subroutine
  ! MLG_PLAIN_FP64 (the drop-in) or MLG_MIXED, for the calls that follow
  subroutine set_precision(mode)
    integer(c_int), intent(in) :: mode
    call check(mlg_set_precision(mode))
  end subroutine
  ! a cudaStream_t as c_ptr (c_null_ptr: the legacy default stream)
  subroutine set_stream(stream)
    type(c_ptr), intent(in) :: stream
    call check(mlg_set_stream(stream))
  end subroutine
  ! waits for the enqueued work; stops on a device-side error (singular band, a wait that ran out)
  subroutine gpu_sync()
    call check(mlg_sync())
  end subroutine
  ! read_input (mlegs_misc_io.f90:307-388) for hosts that do not keep their own
  subroutine read_input(fn, p, run, make_dirs)
    character(len=*), intent(in) :: fn
    type(mlg_params), intent(out) :: p
    type(mlg_run_params), intent(out) :: run
    logical, intent(in) :: make_dirs
    call check(mlg_read_input(trim(fn) // c_null_char, p, run, merge(1, 0, make_dirs)))
  end subroutine

  ! ---- scalar container ----
  subroutine scalar_init(s)
    type(scalar_gpu), intent(inout) :: s
    call check(mlg_scalar_alloc(s%h))
  end subroutine
  subroutine scalar_free(s)
    type(scalar_gpu), intent(inout) :: s
    call check(mlg_scalar_free(s%h))
    s%h = c_null_ptr
  end subroutine
  subroutine upload(s, e, ln, space)
    type(scalar_gpu), intent(inout) :: s
    complex(c_double_complex), intent(in) :: e(:,:,:)
    real(c_double), intent(in) :: ln
    character(len=3), intent(in) :: space
    call check(mlg_scalar_upload(s%h, e, ln, space // c_null_char))
  end subroutine
  subroutine download(s, e, ln)
    type(scalar_gpu), intent(inout) :: s
    complex(c_double_complex), intent(out) :: e(:,:,:)
    real(c_double), intent(out) :: ln
    character(kind=c_char) :: sp(4)
    call check(mlg_scalar_download(s%h, e, ln, sp))
  end subroutine
  ! d = s (assignment(=), mlegs_scalar_init.f90:106-140)
  subroutine copy(d, s)
    type(scalar_gpu), intent(inout) :: d
    type(scalar_gpu), intent(in) :: s
    call check(mlg_scalar_copy(d%h, s%h))
  end subroutine
  subroutine chop_offset(s, iof1, iof2, iof3)
    type(scalar_gpu) :: s; integer, intent(in) :: iof1, iof2, iof3
    call check(mlg_scalar_chop_offset(s%h, iof1, iof2, iof3))
  end subroutine
  subroutine set_ln(s, ln)
    type(scalar_gpu) :: s; real(c_double), intent(in) :: ln
    call check(mlg_scalar_set_ln(s%h, ln))
  end subroutine
  subroutine set_space(s, space)
    type(scalar_gpu) :: s; character(len=3), intent(in) :: space
    call check(mlg_scalar_set_space(s%h, space // c_null_char))
  end subroutine
  ! d%e = a*x%e + b*y%e on the device (the apps' array arithmetic on s%e, e.g. the Richardson start
  ! psi%e = 2*psi%e - psi_rich%e, vortical_flow_3d.f90:136-137); y may be omitted
  subroutine axpby(d, a, x, b, y)
    type(scalar_gpu) :: d, x; real(c_double), intent(in) :: a; real(c_double), intent(in), optional :: b
    type(scalar_gpu), optional :: y
    real(c_double) :: bb
    type(c_ptr) :: yh
    bb = 0.d0; yh = c_null_ptr
    if (present(b)) bb = b
    if (present(y)) yh = y%h
    call check(mlg_scalar_axpby(d%h, a, x%h, bb, yh))
  end subroutine

  ! ---- operators ----
  subroutine trans(s, space, tfm)
    type(scalar_gpu), intent(inout) :: s
    character(len=3), intent(in) :: space
    class(*), intent(in) :: tfm
    call check(mlg_trans(s%h, space // c_null_char))
  end subroutine
  subroutine chop(s, tfm);       type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_chop(s%h));     end subroutine
  subroutine dealias(s, tfm);    type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_dealias(s%h));  end subroutine
  subroutine zeroat1(s, tfm);    type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_zeroat1(s%h));  end subroutine
  subroutine delsqp(s, tfm);     type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_delsqp(s%h));   end subroutine
  subroutine idelsqp(s, tfm);    type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_idelsqp(s%h));  end subroutine
  subroutine xxdx(s, tfm);       type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_xxdx(s%h));     end subroutine
  subroutine del2h(s, tfm);      type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_del2h(s%h));    end subroutine
  subroutine del2(s, tfm);       type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_del2(s%h));     end subroutine
  subroutine idel2_proln(s, tfm); type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_idel2_proln(s%h)); end subroutine
  subroutine idel2_preln(s, tfm, preln)
    type(scalar_gpu) :: s; class(*) :: tfm; real(c_double) :: preln
    call check(mlg_idel2_preln(s%h, preln))
  end subroutine
  subroutine svv_filter(s, tfm, gain)
    type(scalar_gpu) :: s; class(*) :: tfm; real(c_double), intent(inout) :: gain
    call check(mlg_svv_filter(s%h, gain))
  end subroutine
  ! calcat0 / calcat1 (mlegs_scalar_ops.f90:237-309): the value at r = 0 / r = infinity per k
  subroutine calcat0(s, calc, tfm)
    type(scalar_gpu) :: s; complex(c_double_complex), intent(out) :: calc(:); class(*) :: tfm
    call check(mlg_calcat0(s%h, calc))
  end subroutine
  subroutine calcat1(s, calc, tfm)
    type(scalar_gpu) :: s; complex(c_double_complex), intent(out) :: calc(:); class(*) :: tfm
    call check(mlg_calcat1(s%h, calc))
  end subroutine
  subroutine helm(s, alpha, tfm);  type(scalar_gpu) :: s; real(c_double) :: alpha; class(*) :: tfm
    call check(mlg_helm(s%h, alpha)); end subroutine
  subroutine ihelm(s, alpha, tfm); type(scalar_gpu) :: s; real(c_double) :: alpha; class(*) :: tfm
    call check(mlg_ihelm(s%h, alpha)); end subroutine
  subroutine helmp(s, power, alpha, beta, tfm)
    type(scalar_gpu) :: s; integer :: power; real(c_double) :: alpha, beta; class(*) :: tfm
    call check(mlg_helmp(s%h, power, alpha, beta))
  end subroutine
  subroutine ihelmp(s, power, alpha, beta, tfm)
    type(scalar_gpu) :: s; integer :: power; real(c_double) :: alpha, beta; class(*) :: tfm
    call check(mlg_ihelmp(s%h, power, alpha, beta))
  end subroutine
  subroutine fefe(s, nl, dt, tfm); type(scalar_gpu) :: s, nl; real(c_double) :: dt; class(*) :: tfm
    call check(mlg_fefe(s%h, nl%h, dt)); end subroutine
  subroutine febe(s, nl, dt, tfm); type(scalar_gpu) :: s, nl; real(c_double) :: dt; class(*) :: tfm
    call check(mlg_febe(s%h, nl%h, dt)); end subroutine
  subroutine abab(s, sp, nl, nlp, dt, tfm, is_2nd_svis_p)
    type(scalar_gpu) :: s, sp, nl, nlp; real(c_double) :: dt; class(*) :: tfm; logical, optional :: is_2nd_svis_p
    integer(c_int) :: f
    f = 0
    if (present(is_2nd_svis_p)) f = merge(1, 0, is_2nd_svis_p)
    call check(mlg_abab(s%h, sp%h, nl%h, nlp%h, dt, f))
  end subroutine
  subroutine abcn(s, sp, nl, nlp, dt, tfm)
    type(scalar_gpu) :: s, sp, nl, nlp; real(c_double) :: dt; class(*) :: tfm
    call check(mlg_abcn(s%h, sp%h, nl%h, nlp%h, dt))
  end subroutine
  subroutine vecprod(vr, vp, vz, ur, up, uz, tfm)
    type(scalar_gpu) :: vr, vp, vz, ur, up, uz; class(*) :: tfm
    call check(mlg_vecprod(vr%h, vp%h, vz%h, ur%h, up%h, uz%h))
  end subroutine
  subroutine vec2tp(vr, vp, vz, psi, chi, tfm)
    type(scalar_gpu) :: vr, vp, vz, psi, chi; class(*) :: tfm
    call check(mlg_vec2tp(vr%h, vp%h, vz%h, psi%h, chi%h))
  end subroutine
  subroutine tp2vec(psi, chi, vr, vp, vz, tfm)
    type(scalar_gpu) :: psi, chi, vr, vp, vz; class(*) :: tfm
    call check(mlg_tp2vec(psi%h, chi%h, vr%h, vp%h, vz%h))
  end subroutine
  subroutine tp2curlvec(psi, chi, wr, wp, wz, tfm)
    type(scalar_gpu) :: psi, chi, wr, wp, wz; class(*) :: tfm
    call check(mlg_tp2curlvec(psi%h, chi%h, wr%h, wp%h, wz%h))
  end subroutine

  ! ---- the 3-D vortex app (vortical_flow_3d.f90) ----
  ! advection_rhs (:353-395); uz is the background axial flow (PPP)
  subroutine advection_rhs(psi, chi, nlpsi, nlchi, uz)
    type(scalar_gpu) :: psi, chi, nlpsi, nlchi, uz
    call check(mlg_advection_rhs(psi%h, chi%h, nlpsi%h, nlchi%h, uz%h))
  end subroutine
  ! one main-loop step (:168-180); gains(2): the SVV gains of psi and chi, updated
  subroutine vortex_step(psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz, dt, gains)
    type(scalar_gpu) :: psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz
    real(c_double), intent(in) :: dt
    real(c_double), intent(inout) :: gains(2)
    call check(mlg_vortex_step(psi%h, chi%h, nlpsi%h, nlchi%h, psi_p%h, chi_p%h, nlpsi_p%h, nlchi_p%h, uz%h, dt, gains))
  end subroutine
  ! nsteps main-loop steps without a host round trip (the state ends as after nsteps vortex_step calls)
  subroutine vortex_run(psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz, dt, nsteps, gains)
    type(scalar_gpu) :: psi, chi, nlpsi, nlchi, psi_p, chi_p, nlpsi_p, nlchi_p, uz
    real(c_double), intent(in) :: dt
    integer, intent(in) :: nsteps
    real(c_double), intent(inout) :: gains(2)
    call check(mlg_vortex_run(psi%h, chi%h, nlpsi%h, nlchi%h, psi_p%h, chi_p%h, nlpsi_p%h, nlchi_p%h, uz%h, dt, &
                              nsteps, gains))
  end subroutine
  ! the adjoint: J (final perturbation kinetic energy after nsteps) and, when grad_psi / grad_chi are
  ! present, dJ/d(psi0, chi0) written into them; checkpoint every k_ckpt steps, segments recomputed
  subroutine adjoint_run(psi0, chi0, uz, dt, nsteps, k_ckpt, j, grad_psi, grad_chi)
    type(scalar_gpu) :: psi0, chi0, uz
    real(c_double), intent(in) :: dt
    integer, intent(in) :: nsteps, k_ckpt
    real(c_double), intent(out) :: j
    type(scalar_gpu), optional :: grad_psi, grad_chi
    type(c_ptr) :: gp, gc
    gp = c_null_ptr; gc = c_null_ptr
    if (present(grad_psi)) gp = grad_psi%h
    if (present(grad_chi)) gc = grad_chi%h
    call check(mlg_adjoint_run(psi0%h, chi0%h, uz%h, dt, nsteps, k_ckpt, gp, gc, j))
  end subroutine

  ! ---- field I/O and diagnostics ----
  ! msave / mload (mlegs_scalar_io.f90): formatted and global unless told otherwise
  subroutine msave(s, fn, is_binary, is_global)
    type(scalar_gpu) :: s; character(len=*), intent(in) :: fn; logical, optional :: is_binary, is_global
    integer(c_int) :: b, g
    b = 0; g = 1
    if (present(is_binary)) b = merge(1, 0, is_binary)
    if (present(is_global)) g = merge(1, 0, is_global)
    call check(mlg_msave(s%h, trim(fn) // c_null_char, b, g))
  end subroutine
  subroutine mload(s, fn, is_binary, is_global)
    type(scalar_gpu) :: s; character(len=*), intent(in) :: fn; logical, optional :: is_binary, is_global
    integer(c_int) :: b, g
    b = 0; g = 1
    if (present(is_binary)) b = merge(1, 0, is_binary)
    if (present(is_global)) g = merge(1, 0, is_global)
    call check(mlg_mload(s%h, trim(fn) // c_null_char, b, g))
  end subroutine
  subroutine fftreat(s, tfm); type(scalar_gpu) :: s; class(*) :: tfm; call check(mlg_fftreat(s%h)); end subroutine
  ! the field save_vort_mag saves (vortical_flow_3d.f90:411-465), into out (PPP)
  subroutine vort_mag(psi, chi, out)
    type(scalar_gpu) :: psi, chi, out
    call check(mlg_vort_mag(psi%h, chi%h, out%h))
  end subroutine
  ! kinetic-energy spectrum e(m + 1, k + 1), m < npdim, k < nzdim
  subroutine ke_spectrum(psi, chi, e)
    type(scalar_gpu) :: psi, chi
    real(c_double), intent(out) :: e(:,:)
    call check(mlg_ke_spectrum(psi%h, chi%h, e))
  end subroutine
end module
