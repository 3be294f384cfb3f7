!===================================================================================================
! fsibe_reference_api.f90 -- the reference's own routine names and argument lists over the GB300
! library, so that time_step.f90 keeps every call of its hot loop and needs one line more:
!
!     use fsibe_reference_api
!
! at the top of subroutine time_step.  Inside that scope the names below resolve to these module
! procedures instead of the reference's external ones (create_mask.f90:2, NavierStokes.f90:422,463,
! BeamForces.f90:6, SolidSolver.f90:13,874), which stay linked and unused.
!
! The device holds the run's state.  The host arguments keep their meaning where the
! reference's own code reads them:
!   * dt1 (intent inout of EvolveFluid*): the step cal_nlk chose (NavierStokes.f90:60-78), read
!     back after every fluid step;
!   * beams(1): pressure_new / tau_new after every GetForces, the positions, angles, velocities,
!     forces and energies after every SolidSolverWrapper (a few KB a step), so SaveBeamData and
!     the brake test see the reference's values;
!   * vortk(:,:,n0), u, press: copied back only by fsibe_sync_fields (fields are MB; call it
!     before save_fields / SaveField);
!   * mask, nlk, workvis: not maintained on the host.
! Start: the first EvolveFluidExplicit builds the device run from the share_vars globals and
! vortk(:,:,n0) (inicond = 111, init_fields.f90:110-130, after the reference's init_fields ran);
! a resumed run (inicond = 2, no start-up step) is built by the first EvolveFluidAB2 from the
! later of dir_name/runtime_backup{0,1}.in, the file init_fields.f90:44-92 read.
! Time levels: time_step.f90 swaps n0/n1, adds dt1 to time and copies the beam loads on its own
! variables (:152-159, :222-228); the next call whose time is ahead of the device's advances
! the device the same way (fsibe_advance).
! Statuses map as in fsibe_iso_c: `stop` on hard errors, continue_timestep = .false. on the
! emergency brake.
!===================================================================================================
module fsibe_reference_api
  use iso_c_binding
  use fsibe_iso_c
  implicit none
  private
  public :: create_mask, EvolveFluidExplicit, EvolveFluidAB2, GetForces, GravityImpulse, &
            SolidSolverWrapper, fsibe_sync_fields, ComputePressureSnapshot

  interface
    integer(c_int) function fsibe_download_beam(ctx, beam, po, pn, to, tn) bind(C, name="fsibe_download_beam")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: beam(*), po(*), pn(*), to(*), tn(*)
    end function
    integer(c_int) function fsibe_download_vortk(ctx, v) bind(C, name="fsibe_download_vortk")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: v(*)
    end function
    integer(c_int) function fsibe_pressure_snapshot(ctx, time, p) bind(C, name="fsibe_pressure_snapshot")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: time
      real(c_double), intent(out) :: p(*)
    end function
  end interface

  logical, save :: started = .false.

contains

  ! build the device run from the host's initial vorticity (inicond = 111)
  subroutine start_from_vortk(vortk_n0)
    use share_vars
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(in) :: vortk_n0
    real(kind=pr), allocatable :: vort(:,:)
    call fsibe_start()
    allocate(vort(0:nx-1,0:ny-1))
    call fsibe_check(fsibe_fft_inverse(gctx, vortk_n0, vort), "cofitxy")
    call fsibe_check(fsibe_init_fields(gctx, vort), "init_fields")
    deallocate(vort)
    started = .true.
  end subroutine

  ! build the device run from the later runtime backup (inicond = 2)
  subroutine start_from_backup()
    use share_vars
    real(kind=pr) :: t0, t1
    integer :: pick
    t0 = backup_time(trim(dir_name)//'/runtime_backup0.in')
    t1 = backup_time(trim(dir_name)//'/runtime_backup1.in')
    pick = 0
    if (t1 > t0) pick = 1
    call fsibe_start()
    call resume_gb300(pick)
    started = .true.
  end subroutine

  ! the first record of a runtime backup (its time); -1 when the file cannot be read
  real(kind=pr) function backup_time(path)
    use share_vars, only: pr
    character(len=*), intent(in) :: path
    integer :: ios
    backup_time = -1.0_pr
    open (21, file=path, form='unformatted', status='old', action='read', iostat=ios)
    if (ios /= 0) return
    read (21, iostat=ios) backup_time
    if (ios /= 0) backup_time = -1.0_pr
    close (21)
  end function

  ! the host finished a time step on its own variables: the device does the same
  subroutine sync_time(time)
    use share_vars, only: pr
    real(kind=pr), intent(in) :: time
    type(fsibe_scalars_t) :: s
    call fsibe_check(fsibe_get_scalars(gctx, s), "get_scalars")
    if (time > s%time + 0.5_pr * s%dt1) call fsibe_check(fsibe_advance(gctx), "advance")
  end subroutine

  ! create_mask.f90:2-218 (the beam's mask, drawn on the device from the device's beam)
  subroutine create_mask(time, beams)
    use share_vars
    real(kind=pr), intent(in) :: time
    type(solid), dimension(1:iBeam), intent(inout) :: beams
    if (.not. started) return     ! the start-up mask is drawn when the device run starts
    call sync_time(time)
    call fsibe_check(fsibe_create_mask(gctx, time), "create_mask")
  end subroutine

  ! NavierStokes.f90:422-459
  subroutine EvolveFluidExplicit(time, dt1, n0, n1, beams, vortk, workvis, nlk, u, press)
    use share_vars
    real(kind=pr), intent(inout) :: time, dt1
    integer, intent(in) :: n0, n1
    type(solid), dimension(1:iBeam), intent(inout) :: beams
    real(kind=pr), dimension(0:nx-1,0:ny-1,0:1), intent(inout) :: vortk, workvis, nlk
    real(kind=pr), dimension(0:nx-1,0:ny-1,1:2), intent(inout) :: u
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(inout) :: press
    type(fsibe_scalars_t) :: s
    if (.not. started) call start_from_vortk(vortk(:,:,n0))
    call sync_time(time)
    call fsibe_check(fsibe_fluid_step(gctx, 1_c_int), "EvolveFluidExplicit")
    call fsibe_check(fsibe_get_scalars(gctx, s), "get_scalars")
    dt1 = s%dt1
  end subroutine

  ! NavierStokes.f90:463-508
  subroutine EvolveFluidAB2(time, dt0, dt1, n0, n1, beams, vortk, workvis, nlk, u, press)
    use share_vars
    real(kind=pr), intent(inout) :: time, dt0, dt1
    integer, intent(in) :: n0, n1
    type(solid), dimension(1:iBeam), intent(inout) :: beams
    real(kind=pr), dimension(0:nx-1,0:ny-1,0:1), intent(inout) :: vortk, workvis, nlk
    real(kind=pr), dimension(0:nx-1,0:ny-1,1:2), intent(inout) :: u
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(inout) :: press
    type(fsibe_scalars_t) :: s
    if (.not. started) call start_from_backup()
    call sync_time(time)
    call fsibe_check(fsibe_fluid_step(gctx, 0_c_int), "EvolveFluidAB2")
    call fsibe_check(fsibe_get_scalars(gctx, s), "get_scalars")
    dt1 = s%dt1
  end subroutine

  ! BeamForces.f90:6-51 with SPL = 3 ("new" is the time level the hot loop asks for)
  subroutine GetForces(time, beams, press, u, timelevel)
    use share_vars
    real(kind=pr), intent(in) :: time
    type(solid), dimension(1:iBeam), intent(inout) :: beams
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(in) :: press
    real(kind=pr), dimension(0:nx-1,0:ny-1,1:2), intent(in) :: u
    character(len=*), intent(in) :: timelevel
    type(fsibe_scalars_t) :: s
    real(kind=pr), allocatable :: b(:,:), po(:), to(:)
    if (timelevel /= "new") then
      write (*,*) "!!! GetForces: only the 'new' time level runs on the device"
      stop
    endif
    call fsibe_check(fsibe_get_forces(gctx, time), "GetForces")
    allocate(b(0:ns-1,1:6), po(0:ns-1), to(0:ns-1))
    call fsibe_check(fsibe_download_beam(gctx, b, po, beams(1)%pressure_new, to, beams(1)%tau_new), "GetForces")
    call fsibe_check(fsibe_get_scalars(gctx, s), "get_scalars")
    beams(1)%Force = s%force
    beams(1)%Force_unst = s%force_unst
    beams(1)%Force_press = s%force_press
    deallocate(b, po, to)
  end subroutine

  ! SolidSolver.f90:874-911: applied by the device inside SolidSolverWrapper
  subroutine GravityImpulse(time)
    use share_vars, only: pr
    real(kind=pr), intent(in) :: time
  end subroutine

  ! SolidSolver.f90:13-44 (with GravityImpulse): the beam Newton step on the device, then the
  ! beam state, forces and energies into beams(1)
  subroutine SolidSolverWrapper(time, dt, beams)
    use share_vars
    real(kind=pr), intent(in) :: time, dt
    type(solid), dimension(1:iBeam), intent(inout) :: beams
    type(fsibe_scalars_t) :: s
    real(kind=pr), allocatable :: b(:,:)
    call fsibe_check(fsibe_solid_step(gctx, time), "SolidSolverWrapper")
    allocate(b(0:ns-1,1:6))
    call fsibe_check(fsibe_download_beam(gctx, b, beams(1)%pressure_old, beams(1)%pressure_new, &
                                         beams(1)%tau_old, beams(1)%tau_new), "SolidSolverWrapper")
    beams(1)%x = b(:,1); beams(1)%y = b(:,2); beams(1)%vx = b(:,3); beams(1)%vy = b(:,4)
    beams(1)%theta = b(:,5); beams(1)%theta_dot = b(:,6)
    call fsibe_check(fsibe_get_scalars(gctx, s), "get_scalars")
    beams(1)%Inertial_Force = s%inertial_force
    beams(1)%E_kinetic = s%e_kinetic
    beams(1)%E_elastic = s%e_elastic
    beams(1)%E_pot = s%e_pot
    deallocate(b)
  end subroutine

  ! the device's vorticity (packed, into vortk(:,:,n0)), velocity and pressure, for the
  ! reference's field output
  subroutine fsibe_sync_fields(n0, vortk, u, press)
    use share_vars
    integer, intent(in) :: n0
    real(kind=pr), dimension(0:nx-1,0:ny-1,0:1), intent(inout) :: vortk
    real(kind=pr), dimension(0:nx-1,0:ny-1,1:2), intent(out) :: u
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(out) :: press
    call fsibe_check(fsibe_download_vortk(gctx, vortk(:,:,n0)), "download_vortk")
    call fsibe_check(fsibe_download_u(gctx, u), "download_u")
    call fsibe_check(fsibe_download_press(gctx, press), "download_press")
  end subroutine

  ! ComputePressureSnapshot (NavierStokes.f90:598-665): the static pressure of the run's current
  ! vorticity with the velocity at `time` and the current mask.  vortk must be the run's
  ! current vorticity (the device's copy is the one used).
  subroutine ComputePressureSnapshot(time, vortk, press)
    use share_vars
    real(kind=pr), intent(in) :: time
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(in) :: vortk
    real(kind=pr), dimension(0:nx-1,0:ny-1), intent(out) :: press
    call fsibe_check(fsibe_pressure_snapshot(gctx, time, press), "pressure_snapshot")
  end subroutine

end module fsibe_reference_api
