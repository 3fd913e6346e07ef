! he4g_wrappers.f90 -- replacements for steprk.f90, steppc.f90, poten.f90,
! potenimp.f90 and energy.f90 with the reference routine names and argument
! lists, so that DFT4He3d.f90 compiles unchanged against the GPU time step.
! They read module variables of modules.f90 only (no driver locals): the
! absorber comes from the grid module's timec array, the surface potential
! from the field module's uext, and the loop cadence from the namelist echo
! the driver writes itself. The fields stay on the GPU; psi and den are
! copied back only on the steps where the driver reads them.
subroutine he4g_ensure_run()
  use he4g_c
  use grid, only: nx, ny, nz, xmax, ymax, zmax
  use he4, only: lsolid, cp4, cpp4, h2o2m4, alphas, l, den0s, C, beta, den_m
  use lenard4, only: core4, eps4, sigma4, h4, fvlj4
  use rho, only: psi, wcgk
  use classicimp, only: rimp, vimp, mAg_u, mp_u
  use interpol, only: npot, DelInter, potion
  use alphasterm, only: kalfs
  implicit none
  type(he4g_config) :: cfg                   ! not "c": the he4 module's C is use-associated
  if (c_associated(he4g_run)) return
  cfg%nx = nx; cfg%ny = ny; cfg%nz = nz; cfg%npd = 13; cfg%icon = 13; cfg%precision = 0
  cfg%core = merge(1, 0, core4 == 'OTC'); cfg%lsolid = merge(1, 0, lsolid); cfg%lrk = 0
  cfg%npot = npot; cfg%delinter = DelInter
  cfg%xmax = xmax; cfg%ymax = ymax; cfg%zmax = zmax; cfg%deltat = 0.d0
  cfg%cp4 = cp4; cfg%cpp4 = cpp4; cfg%h2o2m4 = h2o2m4; cfg%alphas = alphas; cfg%l_alpha = l
  cfg%den0s = den0s; cfg%c_solid = C; cfg%beta_solid = beta; cfg%den_m = den_m
  cfg%eps4 = eps4; cfg%sigma4 = sigma4; cfg%h4 = h4; cfg%hcg = merge(1.065d0*h4, h4, lsolid)
  ! no absorber until the driver has built timec (DFT4He3d.f90:689-699, after
  ! the first poten): the first step sends the array itself (he4g_set_timec)
  cfg%lambdah = 0.d0; cfg%txmean = 1.d3; cfg%txsurf = 1.d0; cfg%tymean = 1.d3; cfg%tysurf = 1.d0
  cfg%tzmean = 1.d3; cfg%tzsurf = 1.d0
  cfg%mimpur = mAg_u / mp_u
  if (core4 == 'OTC') then
    call he4g_check(he4g_create(cfg, fvlj4, wcgk, kalfs, potion, he4g_run), 'create')
  else                                       ! kalfs is not allocated; the library ignores it for OT
    call he4g_check(he4g_create(cfg, fvlj4, wcgk, fvlj4, potion, he4g_run), 'create')
  end if
  call he4g_check(he4g_set_state(he4g_run, psi, rimp, vimp), 'set_state')
  call he4g_read_cadence()
end subroutine

! before the first step: the arrays the driver builds after its first
! potential evaluation (timec :689-699, uext :760-784)
subroutine he4g_send_loop_state()
  use he4g_c
  use grid, only: timec
  use field, only: uext
  implicit none
  if (he4g_loop_state_sent) return
  call he4g_check(he4g_set_timec(he4g_run, timec), 'set_timec')
  call he4g_check(he4g_set_uext(he4g_run, uext), 'set_uext')
  he4g_loop_state_sent = .true.
end subroutine

subroutine potenimp(rimp_in)
  use he4g_c
  use classicimp, only: uimp
  implicit none
  real(8), intent(in) :: rimp_in(3)
  call he4g_ensure_run()
  call he4g_check(he4g_potenimp(he4g_run, rimp_in), 'potenimp')
  ! before the loop the driver writes uimp out (respar, DFT4He3d.f90:646)
  if (he4g_k == 0) call he4g_check(he4g_get_field(he4g_run, 3, uimp), 'get_field uimp')
end subroutine

subroutine poten()
  use he4g_c
  use rho, only: den
  implicit none
  call he4g_check(he4g_poten(he4g_run), 'poten')
  if (he4g_den_wanted()) call he4g_check(he4g_get_den(he4g_run, den), 'get_den')
end subroutine

subroutine forceimp(rimp_in, F)
  use he4g_c
  implicit none
  real(8), intent(in) :: rimp_in(3)
  real(8), intent(out) :: F(3)
  call he4g_check(he4g_forceimp(he4g_run, rimp_in, F), 'forceimp')
end subroutine

subroutine steprk(deltat)
  use he4g_c
  use classicimp, only: rimp, vimp, aimp
  use rho, only: psi
  implicit none
  real(8) :: deltat
  call he4g_send_loop_state()
  call he4g_check(he4g_set_impurity(he4g_run, rimp, vimp, aimp), 'set_impurity')
  call he4g_check(he4g_steprk(he4g_run, deltat), 'steprk')
  call he4g_check(he4g_get_impurity(he4g_run, rimp, vimp, aimp), 'get_impurity')
  he4g_k = he4g_k + 1
  if (he4g_psi_wanted()) call he4g_check(he4g_get_psi(he4g_run, psi), 'get_psi')
end subroutine

subroutine steppc(deltat, errHe, errimp)
  use he4g_c
  use classicimp, only: rimp, vimp, aimp
  use rho, only: psi
  implicit none
  real(8) :: deltat, errHe, errimp
  call he4g_send_loop_state()
  call he4g_check(he4g_set_impurity(he4g_run, rimp, vimp, aimp), 'set_impurity')
  call he4g_check(he4g_steppc(he4g_run, deltat, errHe, errimp), 'steppc')
  call he4g_check(he4g_get_impurity(he4g_run, rimp, vimp, aimp), 'get_impurity')
  he4g_k = he4g_k + 1
  if (he4g_psi_wanted()) call he4g_check(he4g_get_psi(he4g_run, psi), 'get_psi')
end subroutine

subroutine energy()
  use he4g_c
  use energies, only: etot4, ekin4, elj4, ecor4, ealphas, esolid, ekinx, eHeX, eimpu, etot
  implicit none
  type(he4g_energies) :: e
  call he4g_check(he4g_energy(he4g_run, e), 'energy')
  etot4 = e%etot4; ekin4 = e%ekin4; elj4 = e%elj4; ecor4 = e%ecor4; ealphas = e%ealphas
  esolid = e%esolid; ekinx = e%ekinx; eHeX = e%eHeX; eimpu = e%eimpu; etot = e%etot
end subroutine
