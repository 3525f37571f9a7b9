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

  interface
    integer(c_int) function mlg_init(p) bind(c, name='mlg_init')
      import :: c_int, mlg_params
      type(mlg_params), intent(in) :: p
    end function
    integer(c_int) function mlg_finalize() bind(c, name='mlg_finalize')
      import :: c_int
    end function
    type(c_ptr) function mlg_last_error() bind(c, name='mlg_last_error')
      import :: c_ptr
    end function
    integer(c_int) function mlg_kit_dims(d) bind(c, name='mlg_kit_dims')
      import :: c_int
      integer(c_int), intent(out) :: d(9)
    end function
    integer(c_int) function mlg_set_precision(mode) bind(c, name='mlg_set_precision')
      import :: c_int
      integer(c_int), value :: mode
    end function
    integer(c_int) function mlg_sync() bind(c, name='mlg_sync')
      import :: c_int
    end function
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
    integer(c_int) function mlg_scalar_copy(d, s) bind(c, name='mlg_scalar_copy')
      import :: c_int, c_ptr
      type(c_ptr), value :: d, s
    end function
    integer(c_int) function mlg_scalar_chop_offset(s, a, b, c) bind(c, name='mlg_scalar_chop_offset')
      import :: c_int, c_ptr
      type(c_ptr), value :: s
      integer(c_int), value :: a, b, c
    end function
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

  public :: gpu_kit_init, scalar_init, upload, download
  public :: trans, chop, dealias, svv_filter, zeroat1, delsqp, idelsqp, xxdx, del2h, del2
  public :: idel2, helm, ihelm, helmp, ihelmp, fefe, abab, febe, abcn, vecprod, vec2tp, tp2vec, tp2curlvec

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

  subroutine scalar_init(s)
    type(scalar_gpu), intent(inout) :: s
    call check(mlg_scalar_alloc(s%h))
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
end module
