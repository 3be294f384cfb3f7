!===================================================================================================
! fsibe_iso_c.f90 -- ISO_C_BINDING layer that lets the reference's Fortran driver (dns.f90,
! time_step.f90) call the GB300 library through include/fsibe.h.
!
! The module keeps one device context (the reference is one run per process) built from the
! share_vars globals, and provides subroutines with the reference's names and argument lists
! whose bodies call the C ABI.  Non-zero statuses map onto the reference's behaviour: `stop`
! for hard errors, continue_timestep = .false. for the emergency brake.
!
! Compile with the reference sources (gfortran -fdefault-real-8 ... fsibe_iso_c.f90) and link
! fsibe_2d_gb300/_lib/libfsibe_gb300.so.
!===================================================================================================
module fsibe_iso_c
  use iso_c_binding
  implicit none

  type, bind(C) :: fsibe_params_t
    integer(c_int32_t) :: nx, ny, ns, precision
    real(c_double) :: xl, yl, nu, eps, cfl, dt_fixed, time_end, eta, mue, t_release, tau
    real(c_double) :: angle_beam, grav, sigma
    integer(c_int32_t) :: iImpulse, time_method_solid, iFLUSI, iMotion, iViscous, iSaveBeam
    integer(c_int32_t) :: iBeam, iSharpTrailing, iMeanVelocity, idealis
    real(c_double) :: T_fullspeed, theta_inf, x0, y0, length, t_beam, N_smooth, newton_tol
    integer(c_int32_t) :: newton_maxit, reserved
    integer(c_int32_t) :: iWalls, iCylinder, iSponge, reserved2
    real(c_double) :: h_channel, R_cylinder, SpongeSize, eps_sponge
  end type

  type, bind(C) :: fsibe_scalars_t
    real(c_double) :: time, dt0, dt1, u_max, mean_ux, mean_uy
    real(c_double) :: vor_rms, kinetic, dissipation, porous_diss, inflow_solid, inflow_mean
    real(c_double) :: force(2), force_unst(2), force_press(2), inertial_force(2)
    real(c_double) :: e_kinetic, e_elastic, e_pot
    real(c_double) :: beam_data(21)
    integer(c_int32_t) :: newton_iters, status, step, reserved
  end type

  integer(c_int), parameter :: FSIBE_OK = 0, FSIBE_ERR_BRAKE = 10

  interface
    integer(c_int) function fsibe_create(p, ctx) bind(C, name="fsibe_create")
      import :: c_int, c_ptr, fsibe_params_t
      type(fsibe_params_t), intent(in) :: p
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function fsibe_destroy(ctx) bind(C, name="fsibe_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function fsibe_fft_forward(ctx, f, fk) bind(C, name="fsibe_fft_forward")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: f(*)
      real(c_double), intent(out) :: fk(*)
    end function
    integer(c_int) function fsibe_fft_inverse(ctx, fk, f) bind(C, name="fsibe_fft_inverse")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: fk(*)
      real(c_double), intent(out) :: f(*)
    end function
    integer(c_int) function fsibe_poisson(ctx, f, ans) bind(C, name="fsibe_poisson")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: f(*)
      real(c_double), intent(out) :: ans(*)
    end function
    integer(c_int) function fsibe_vis(ctx, dt, work) bind(C, name="fsibe_vis")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: dt
      real(c_double), intent(out) :: work(*)
    end function
    integer(c_int) function fsibe_init_fields(ctx, vort) bind(C, name="fsibe_init_fields")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: vort(*)
    end function
    integer(c_int) function fsibe_create_mask(ctx, time) bind(C, name="fsibe_create_mask")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: time
    end function
    integer(c_int) function fsibe_fluid_step(ctx, explicit_step) bind(C, name="fsibe_fluid_step")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: explicit_step
    end function
    integer(c_int) function fsibe_get_forces(ctx, time) bind(C, name="fsibe_get_forces")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: time
    end function
    integer(c_int) function fsibe_solid_step(ctx, time) bind(C, name="fsibe_solid_step")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: time
    end function
    integer(c_int) function fsibe_advance(ctx) bind(C, name="fsibe_advance")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function fsibe_write_backup(ctx, path) bind(C, name="fsibe_write_backup")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
    end function
    integer(c_int) function fsibe_read_backup(ctx, path) bind(C, name="fsibe_read_backup")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
    end function
    integer(c_int) function fsibe_run(ctx, nsteps, rows) bind(C, name="fsibe_run")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nsteps
      real(c_double), intent(out) :: rows(*)
    end function
    integer(c_int) function fsibe_download_vort(ctx, vort) bind(C, name="fsibe_download_vort")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: vort(*)
    end function
    integer(c_int) function fsibe_download_u(ctx, u) bind(C, name="fsibe_download_u")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: u(*)
    end function
    integer(c_int) function fsibe_download_press(ctx, p) bind(C, name="fsibe_download_press")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: p(*)
    end function
    integer(c_int) function fsibe_get_scalars(ctx, s) bind(C, name="fsibe_get_scalars")
      import :: c_int, c_ptr, fsibe_scalars_t
      type(c_ptr), value :: ctx
      type(fsibe_scalars_t), intent(out) :: s
    end function
  end interface

  type(c_ptr), save :: gctx = c_null_ptr

contains

  ! Build the context from the share_vars globals (after params() ran).
  subroutine fsibe_start()
    use share_vars
    type(fsibe_params_t) :: p
    integer(c_int) :: st
    p%nx = nx; p%ny = ny; p%ns = ns; p%precision = 0
    p%xl = xl; p%yl = yl; p%nu = nu; p%eps = eps; p%cfl = cfl; p%dt_fixed = dt_fixed
    p%time_end = Time_end; p%eta = eta; p%mue = mue; p%t_release = T_release; p%tau = tau
    p%angle_beam = AngleBeam; p%grav = grav; p%sigma = sigma
    p%iImpulse = iImpulse; p%time_method_solid = TimeMethodSolid; p%iFLUSI = iFLUSI
    p%iMotion = iMotion; p%iViscous = iViscous; p%iSaveBeam = iSaveBeam; p%iBeam = iBeam
    p%iSharpTrailing = iSharpTrailing; p%iMeanVelocity = iMeanVelocity; p%idealis = idealis
    p%T_fullspeed = T_fullspeed; p%theta_inf = theta_inf; p%x0 = x0; p%y0 = y0
    p%length = length; p%t_beam = t_beam; p%N_smooth = N_smooth
    p%newton_tol = 1.0d-7; p%newton_maxit = 50; p%reserved = 0
    p%iWalls = iWalls; p%iCylinder = iCylinder; p%iSponge = iSponge; p%reserved2 = 0
    p%h_channel = h_channel; p%R_cylinder = R_cylinder; p%SpongeSize = SpongeSize; p%eps_sponge = eps_sponge
    st = fsibe_create(p, gctx)
    call fsibe_check(st, "fsibe_create")
  end subroutine

  subroutine fsibe_stop()
    integer(c_int) :: st
    st = fsibe_destroy(gctx)
    gctx = c_null_ptr
  end subroutine

  ! status -> reference behaviour
  subroutine fsibe_check(st, where)
    use share_vars
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    if (st == FSIBE_OK) return
    if (st == FSIBE_ERR_BRAKE) then
      continue_timestep = .false.
      return
    endif
    write (*,*) "!!! ", where, " failed with status ", st
    stop
  end subroutine

  ! coftxy / cofitxy / poisson / vis with the reference's argument lists
  subroutine coftxy_gb300(f, fk)
    use share_vars
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(in) :: f
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(out) :: fk
    call fsibe_check(fsibe_fft_forward(gctx, f, fk), "coftxy")
  end subroutine

  subroutine cofitxy_gb300(fk, f)
    use share_vars
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(in) :: fk
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(out) :: f
    call fsibe_check(fsibe_fft_inverse(gctx, fk, f), "cofitxy")
  end subroutine

  subroutine poisson_gb300(f, ans)
    use share_vars
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(in) :: f
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(out) :: ans
    call fsibe_check(fsibe_poisson(gctx, f, ans), "poisson")
  end subroutine

  subroutine vis_gb300(dt, work)
    use share_vars
    real(kind=pr), intent(in) :: dt
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(out) :: work
    call fsibe_check(fsibe_vis(gctx, dt, work), "vis")
  end subroutine

  ! init_fields with inicond = 111 (init_fields.f90:110-130): vort read from inicond_file
  subroutine init_fields_gb300(vort)
    use share_vars
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(in) :: vort
    call fsibe_check(fsibe_init_fields(gctx, vort), "init_fields")
  end subroutine

  ! MakeRuntimeBackup (save_fields.f90:109-152): the same file, written from the device state;
  ! nbackup alternates between 0 and 1 as in the reference
  subroutine makeruntimebackup_gb300(nbackup)
    use share_vars
    integer, intent(inout) :: nbackup
    character(len=1) :: name1
    write (name1, '(I1)') nbackup
    call fsibe_check(fsibe_write_backup(gctx, trim(dir_name)//'/runtime_backup'//name1//'.in'//c_null_char), &
                     "MakeRuntimeBackup")
    nbackup = 1 - nbackup
  end subroutine

  ! inicond = 2: resume from runtime_backup<ibackup>.in (the caller picks the later file, as
  ! init_fields.f90:44-92 does); replaces init_fields + init_beams + create_mask
  subroutine resume_gb300(ibackup)
    use share_vars
    integer, intent(in) :: ibackup
    character(len=1) :: name1
    write (name1, '(I1)') ibackup
    call fsibe_check(fsibe_read_backup(gctx, trim(dir_name)//'/runtime_backup'//name1//'.in'//c_null_char), &
                     "init_fields (inicond=2)")
  end subroutine

  subroutine create_mask_gb300(time)
    real(c_double), intent(in) :: time
    call fsibe_check(fsibe_create_mask(gctx, time), "create_mask")
  end subroutine

  ! EvolveFluidExplicit (explicit=1) / EvolveFluidAB2 (explicit=0), both ending with pressure()
  subroutine evolve_fluid_gb300(explicit_step)
    integer, intent(in) :: explicit_step
    call fsibe_check(fsibe_fluid_step(gctx, int(explicit_step, c_int)), "EvolveFluid")
  end subroutine

  subroutine getforces_gb300(time)
    real(c_double), intent(in) :: time
    call fsibe_check(fsibe_get_forces(gctx, time), "GetForces")
  end subroutine

  subroutine solidsolverwrapper_gb300(time)
    real(c_double), intent(in) :: time
    call fsibe_check(fsibe_solid_step(gctx, time), "SolidSolverWrapper")
  end subroutine

  ! The body of time_step.f90's loop for nsteps steps; beam_data rows returned in rows(21,nsteps)
  subroutine time_step_gb300(nsteps, rows)
    integer, intent(in) :: nsteps
    real(c_double), intent(out) :: rows(21, nsteps)
    call fsibe_check(fsibe_run(gctx, int(nsteps, c_int), rows), "time_step")
  end subroutine

end module fsibe_iso_c
