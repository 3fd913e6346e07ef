! he4g_wrappers.f90 -- replacements for steprk.f90, steppc.f90, poten.f90,
! potenimp.f90 and energy.f90 with the reference routine names and argument
! lists, so that DFT4He3d.f90 compiles unchanged against the GPU time step.
! The fields stay on the GPU; the wrappers synchronise the module variables
! the driver reads (modules.f90) where it reads them.
subroutine he4g_ensure_run()
  use he4g_c; use grid; use he4; use lenard4; use rho; use classicimp; use interpol
  use alphasterm, only: kalfs
  implicit none
  type(he4g_config) :: c
  if (c_associated(he4g_run)) return
  c%nx = nx; c%ny = ny; c%nz = nz; c%npd = 13; c%icon = 13; c%precision = 0
  c%core = merge(1, 0, core4 == 'OTC'); c%lsolid = merge(1, 0, lsolid); c%lrk = 0
  c%npot = npot; c%delinter = DelInter
  c%xmax = xmax; c%ymax = ymax; c%zmax = zmax; c%deltat = 0.d0
  c%cp4 = cp4; c%cpp4 = cpp4; c%h2o2m4 = h2o2m4; c%alphas = alphas; c%l_alpha = l; c%den0s = den0s
  c%c_solid = C; c%beta_solid = beta; c%den_m = den_m
  c%eps4 = eps4; c%sigma4 = sigma4; c%h4 = h4; c%hcg = merge(1.065d0*h4, h4, lsolid)
  c%lambdah = Lambdah; c%txmean = txmean; c%txsurf = txsurf      ! driver locals: pass them
  c%tymean = tymean; c%tysurf = tysurf; c%tzmean = tzmean; c%tzsurf = tzsurf  ! via a module
  c%mimpur = mAg_u / mp_u
  if (core4 == 'OTC') then
    call he4g_check(he4g_create(c, fvlj4, wcgk, c_loc(kalfs), potion, he4g_run), 'create')
  else
    call he4g_check(he4g_create(c, fvlj4, wcgk, c_null_ptr, potion, he4g_run), 'create')
  end if
  call he4g_check(he4g_set_state(he4g_run, psi, rimp, vimp), 'set_state')
end subroutine

subroutine potenimp(rimp_in)
  use he4g_c; implicit none
  real(8), intent(in) :: rimp_in(3)
  call he4g_ensure_run()
  call he4g_check(he4g_potenimp(he4g_run, rimp_in), 'potenimp')
end subroutine

subroutine poten()
  use he4g_c; use rho, only: den, dencg; use lenard4, only: delj4; use field, only: pot4
  implicit none
  call he4g_check(he4g_poten(he4g_run), 'poten')
  ! module arrays the driver reads (den at DFT4He3d.f90:869; pot4/delj4/dencg only in energy)
  call he4g_check(he4g_get_den(he4g_run, den), 'get_den')
end subroutine

subroutine forceimp(rimp_in, F)
  use he4g_c; implicit none
  real(8), intent(in) :: rimp_in(3)
  real(8), intent(out) :: F(3)
  call he4g_check(he4g_forceimp(he4g_run, rimp_in, F), 'forceimp')
end subroutine

subroutine steprk(deltat)
  use he4g_c; use classicimp, only: rimp, vimp, aimp; use rho, only: psi
  implicit none
  real(8) :: deltat
  call he4g_check(he4g_set_impurity(he4g_run, rimp, vimp, aimp), 'set_impurity')
  call he4g_check(he4g_steprk(he4g_run, deltat), 'steprk')
  call he4g_check(he4g_get_impurity(he4g_run, rimp, vimp, aimp), 'get_impurity')
  call he4g_check(he4g_get_psi(he4g_run, psi), 'get_psi')
end subroutine

subroutine steppc(deltat, errHe, errimp)
  use he4g_c; use classicimp, only: rimp, vimp, aimp; use rho, only: psi
  implicit none
  real(8) :: deltat, errHe, errimp
  call he4g_check(he4g_set_impurity(he4g_run, rimp, vimp, aimp), 'set_impurity')
  call he4g_check(he4g_steppc(he4g_run, deltat, errHe, errimp), 'steppc')
  call he4g_check(he4g_get_impurity(he4g_run, rimp, vimp, aimp), 'get_impurity')
  call he4g_check(he4g_get_psi(he4g_run, psi), 'get_psi')
end subroutine

subroutine energy()
  use he4g_c; use energies; implicit none
  type(he4g_energies) :: e
  call he4g_check(he4g_energy(he4g_run, e), 'energy')
  etot4 = e%etot4; ekin4 = e%ekin4; elj4 = e%elj4; ecor4 = e%ecor4; ealphas = e%ealphas
  esolid = e%esolid; ekinx = e%ekinx; eHeX = e%eHeX; eimpu = e%eimpu; etot = e%etot
end subroutine
