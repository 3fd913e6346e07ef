! he4g_c.f90 -- ISO_C_BINDING interface of include/he4g.h for the Fortran
! driver DFT4He3d.f90 (the reference's host program). Built with the driver
! (makefile:15-20), linked against 4hetddft-isotropic_gb300/he4gpu/_lib/libhe4g.so.
! The bind(C) types mirror the C structs field for field;
! tests/test_fortran_binding.py checks that against the header.
module he4g_c
  use iso_c_binding
  implicit none
  type, bind(C) :: he4g_config
    integer(c_int32_t) :: nx, ny, nz, npd, icon, core, lsolid, lrk, precision, npot
    real(c_double) :: xmax, ymax, zmax, deltat
    real(c_double) :: cp4, cpp4, h2o2m4, alphas, l_alpha, den0s, c_solid, beta_solid, den_m
    real(c_double) :: eps4, sigma4, h4, hcg
    real(c_double) :: lambdah, txmean, txsurf, tymean, tysurf, tzmean, tzsurf
    real(c_double) :: mimpur, delinter
  end type
  type, bind(C) :: he4g_energies
    real(c_double) :: etot4, ekin4, elj4, ecor4, ealphas, esolid, eext, ekinx, eHeX, eimpu, etot
  end type
  type(c_ptr), save :: he4g_run = c_null_ptr
  ! loop cadence of the driver, read from its namelist echo (DFT4He3d.f90:195-196):
  ! the wrappers copy psi and den back only on the steps where the driver reads them
  logical, save :: he4g_lazy = .false.
  integer(c_int), save :: he4g_iter0 = 0, he4g_niter = 0, he4g_pener = 1, he4g_pcurr = 1
  integer, save :: he4g_k = 0                ! steps taken through the wrappers (iteraux)
  logical, save :: he4g_loop_state_sent = .false.
  interface
    integer(c_int) function he4g_create(cfg, fvlj4, wcgk, kalfs, potion, out) bind(C, name="he4g_create")
      import
      type(he4g_config), intent(in) :: cfg
      real(c_double), intent(in) :: fvlj4(*), wcgk(*), kalfs(*), potion(*)   ! kalfs: read for core OTC only
      type(c_ptr), intent(out) :: out
    end function
    integer(c_int) function he4g_set_state(run, psi, rimp, vimp) bind(C, name="he4g_set_state")
      import
      type(c_ptr), value :: run
      complex(c_double_complex), intent(in) :: psi(*)
      real(c_double), intent(in) :: rimp(3), vimp(3)
    end function
    integer(c_int) function he4g_potenimp(run, rimp) bind(C, name="he4g_potenimp")
      import
      type(c_ptr), value :: run
      real(c_double), intent(in) :: rimp(3)
    end function
    integer(c_int) function he4g_poten(run) bind(C, name="he4g_poten")
      import
      type(c_ptr), value :: run
    end function
    integer(c_int) function he4g_forceimp(run, rimp, f) bind(C, name="he4g_forceimp")
      import
      type(c_ptr), value :: run
      real(c_double), intent(in) :: rimp(3)
      real(c_double), intent(out) :: f(3)
    end function
    integer(c_int) function he4g_steprk(run, deltat) bind(C, name="he4g_steprk")
      import
      type(c_ptr), value :: run
      real(c_double), value :: deltat
    end function
    integer(c_int) function he4g_steppc(run, deltat, errhe, errimp) bind(C, name="he4g_steppc")
      import
      type(c_ptr), value :: run
      real(c_double), value :: deltat
      real(c_double), intent(out) :: errhe, errimp
    end function
    integer(c_int) function he4g_energy(run, e) bind(C, name="he4g_energy")
      import
      type(c_ptr), value :: run
      type(he4g_energies), intent(out) :: e
    end function
    integer(c_int) function he4g_set_impurity(run, r, v, a) bind(C, name="he4g_set_impurity")
      import
      type(c_ptr), value :: run
      real(c_double), intent(in) :: r(3), v(3), a(3)
    end function
    integer(c_int) function he4g_get_impurity(run, r, v, a) bind(C, name="he4g_get_impurity")
      import
      type(c_ptr), value :: run
      real(c_double), intent(out) :: r(3), v(3), a(3)
    end function
    integer(c_int) function he4g_get_psi(run, psi) bind(C, name="he4g_get_psi")
      import
      type(c_ptr), value :: run
      complex(c_double_complex), intent(out) :: psi(*)
    end function
    ! psi into pinned host memory without waiting (the copy overlaps the next
    ! steps); psi must not be touched before he4g_wait_psi returns
    integer(c_int) function he4g_get_psi_async(run, psi) bind(C, name="he4g_get_psi_async")
      import
      type(c_ptr), value :: run
      complex(c_double_complex), intent(inout) :: psi(*)
    end function
    integer(c_int) function he4g_wait_psi(run) bind(C, name="he4g_wait_psi")
      import
      type(c_ptr), value :: run
    end function
    integer(c_int) function he4g_get_den(run, den) bind(C, name="he4g_get_den")
      import
      type(c_ptr), value :: run
      real(c_double), intent(out) :: den(*)
    end function
    integer(c_int) function he4g_get_field(run, which, out) bind(C, name="he4g_get_field")
      import
      type(c_ptr), value :: run
      integer(c_int), value :: which
      real(c_double), intent(out) :: out(*)
    end function
    ! the driver's absorber array timec (grid module, modules.f90:101)
    integer(c_int) function he4g_set_timec(run, timec) bind(C, name="he4g_set_timec")
      import
      type(c_ptr), value :: run
      complex(c_double_complex), intent(in) :: timec(*)
    end function
    ! the driver's external potential uext (field module, modules.f90:54)
    integer(c_int) function he4g_set_uext(run, uext) bind(C, name="he4g_set_uext")
      import
      type(c_ptr), value :: run
      real(c_double), intent(in) :: uext(*)
    end function
    integer(c_int) function he4g_read_namelist_int(path, name, val) bind(C, name="he4g_read_namelist_int")
      import
      character(kind=c_char), intent(in) :: path(*), name(*)
      integer(c_int), intent(out) :: val
    end function
    type(c_ptr) function he4g_last_error(run) bind(C, name="he4g_last_error")
      import
      type(c_ptr), value :: run
    end function
  end interface
contains
  ! iter = iter0 + iteraux (DFT4He3d.f90:833-836): psi is read by the driver
  ! every pener iterations (angular momentum, :869-926), every pcurr
  ! (printoutc, :972-994) and after the last one (:1006-1010)
  logical function he4g_psi_wanted()
    he4g_psi_wanted = .not. he4g_lazy
    if (he4g_lazy) he4g_psi_wanted = mod(he4g_iter0 + he4g_k, he4g_pener) == 0 .or. &
        (he4g_pcurr > 0 .and. mod(he4g_k, max(he4g_pcurr, 1)) == 0) .or. he4g_iter0 + he4g_k >= he4g_niter
  end function
  ! den is read every pener iterations, after poten (:869, r_cm :875)
  logical function he4g_den_wanted()
    he4g_den_wanted = .not. he4g_lazy
    if (he4g_lazy) he4g_den_wanted = he4g_k > 0 .and. mod(he4g_iter0 + he4g_k, he4g_pener) == 0
  end function
  subroutine he4g_read_cadence()
    character(*), parameter :: f = 'DFT4He3d.namelist.read'
    logical :: op
    integer :: u
    inquire(file=f, opened=op, number=u)
    if (op) flush(u)                         ! the driver leaves the unit open
    he4g_lazy = he4g_read_namelist_int(f//c_null_char, 'iter0'//c_null_char, he4g_iter0) == 0 .and. &
                he4g_read_namelist_int(f//c_null_char, 'niter'//c_null_char, he4g_niter) == 0 .and. &
                he4g_read_namelist_int(f//c_null_char, 'pener'//c_null_char, he4g_pener) == 0 .and. &
                he4g_read_namelist_int(f//c_null_char, 'pcurr'//c_null_char, he4g_pcurr) == 0
    if (he4g_lazy) he4g_lazy = he4g_pener > 0
    if (.not. he4g_lazy) write(0,'(A)') 'he4g: no loop cadence in '//f//'; psi and den are copied every step'
  end subroutine
  subroutine he4g_check(rc, where)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: where
    if (rc /= 0) then
      write(0,'("he4g error ",I4," in ",A)') rc, where
      stop 'GPU time step failed'          ! the reference STOPs too (steprk.f90:91)
    end if
  end subroutine
end module he4g_c
