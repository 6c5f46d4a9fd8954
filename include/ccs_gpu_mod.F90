! ccs_gpu_mod.F90 -- Fortran 2003 (ISO_C_BINDING) binding of include/ccs_gpu.h for the
! reference driver of DwyaneChou/Conformal_Cubed_Sphere.
!
! Two modules:
!   ccs_gpu_mod         the C ABI itself: constants, the three view types and the
!                       entry points a Fortran driver calls (needs iso_c_binding only)
!   ccs_gpu_driver_mod  helpers over the reference's own modules (parameters_mod,
!                       constants_mod, mesh_mod, stat_mod): the handle set-up from
!                       read_mesh's arrays, a stat_field view and a status check that
!                       stops like io_mod.F90:604-612 does
!
! Add this file to dynamic_core/CMakeLists.txt's source_files (after stat_mod.F90)
! and link libccs_gpu.so; the reference builds with -fdefault-real-8, so its `real`
! is c_double.  The call site it serves is the time loop of ccsm.F90:50-67.
module ccs_gpu_mod
  use, intrinsic :: iso_c_binding
  implicit none

  ! status codes
  integer(c_int), parameter :: CCS_OK = 0, CCS_ERR_ARG = 1, CCS_ERR_CUDA = 2, CCS_ERR_NAN = 3, &
                               CCS_ERR_TIMEOUT = 4, CCS_ERR_UNSUPPORTED = 5, CCS_ERR_MESH = 6, &
                               CCS_ERR_NOMEM = 7, CCS_ERR_NODEVICE = 8, CCS_ERR_TOO_LARGE = 9, &
                               CCS_ERR_IO = 10
  ! integral_scheme (parameters_mod.F90:402-408), arithmetic lane, E-flux option
  integer(c_int), parameter :: CCS_RK4 = 0, CCS_RK3_TVD = 1
  integer(c_int), parameter :: CCS_FP64 = 0, CCS_MIXED = 1
  integer(c_int), parameter :: CCS_EDISS_ZERO = 0, CCS_EDISS_RECONSTRUCT = 1
  ! spatial operator (the reference picks one spatial_operators_mod at build time)
  integer(c_int), parameter :: CCS_OP_WENO = 0, CCS_OP_CENTRAL2 = 2, CCS_OP_CENTRAL4 = 4, CCS_OP_CENTRAL6 = 6

  ! ccs_config
  type, bind(C) :: ccs_config
    integer(c_int) :: N
    integer(c_int) :: halo
    integer(c_int) :: scheme
    integer(c_int) :: precision
    integer(c_int) :: e_dissipation
    integer(c_int) :: device
    real(c_double) :: dx
    real(c_double) :: dy
    real(c_double) :: dt
    real(c_double) :: radius
    real(c_double) :: gravity
    real(c_double) :: omega
    real(c_double) :: phi_mean
  end type ccs_config

  ! ccs_mesh_view: mesh_mod.F90:17-33 after read_mesh
  type, bind(C) :: ccs_mesh_view
    type(c_ptr) :: sqrtG
    type(c_ptr) :: matrixG
    type(c_ptr) :: matrixIG
    type(c_ptr) :: matrixA
    type(c_ptr) :: matrixIA
    type(c_ptr) :: f
    type(c_ptr) :: phis
  end type ccs_mesh_view

  ! ccs_state_view: stat_field, stat_mod.F90:7-17
  type, bind(C) :: ccs_state_view
    type(c_ptr) :: phiG
    type(c_ptr) :: u
    type(c_ptr) :: v
    type(c_ptr) :: phi
    type(c_ptr) :: uC
    type(c_ptr) :: vC
    type(c_ptr) :: zonal_wind
    type(c_ptr) :: meridional_wind
    type(c_ptr) :: phit
  end type ccs_state_view

  interface
    ! read_mesh + initStat / initTend on the device side
    integer(c_int) function ccs_init(cfg, mesh, h) bind(C, name='ccs_init')
      import :: c_int, c_ptr, ccs_config, ccs_mesh_view
      type(ccs_config), intent(in) :: cfg
      type(ccs_mesh_view), intent(in) :: mesh
      type(c_ptr), intent(out) :: h
    end function ccs_init

    integer(c_int) function ccs_init_shared(cfg, mesh_owner, h) bind(C, name='ccs_init_shared')
      import :: c_int, c_ptr, ccs_config
      type(ccs_config), intent(in) :: cfg
      type(c_ptr), value :: mesh_owner
      type(c_ptr), intent(out) :: h
    end function ccs_init_shared

    subroutine ccs_destroy(h) bind(C, name='ccs_destroy')
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine ccs_destroy

    ! stat(old) in and out
    integer(c_int) function ccs_set_state(h, s) bind(C, name='ccs_set_state')
      import :: c_int, c_ptr, ccs_state_view
      type(c_ptr), value :: h
      type(ccs_state_view), intent(in) :: s
    end function ccs_set_state

    integer(c_int) function ccs_get_state(h, s) bind(C, name='ccs_get_state')
      import :: c_int, c_ptr, ccs_state_view
      type(c_ptr), value :: h
      type(ccs_state_view), intent(in) :: s
    end function ccs_get_state

    integer(c_int) function ccs_set_state_async(h, s) bind(C, name='ccs_set_state_async')
      import :: c_int, c_ptr, ccs_state_view
      type(c_ptr), value :: h
      type(ccs_state_view), intent(in) :: s
    end function ccs_set_state_async

    integer(c_int) function ccs_get_state_async(h, s) bind(C, name='ccs_get_state_async')
      import :: c_int, c_ptr, ccs_state_view
      type(c_ptr), value :: h
      type(ccs_state_view), intent(in) :: s
    end function ccs_get_state_async

    ! RK4 / RK3_TVD + copyStat, nsteps times (ccsm.F90:50-67)
    integer(c_int) function ccs_step(h, nsteps) bind(C, name='ccs_step')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function ccs_step

    integer(c_int) function ccs_step_async(h, nsteps) bind(C, name='ccs_step_async')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function ccs_step_async

    integer(c_int) function ccs_sync(h) bind(C, name='ccs_sync')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function ccs_sync

    integer(c_int) function ccs_set_operator(h, op) bind(C, name='ccs_set_operator')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: op
    end function ccs_set_operator

    ! chosen / times_us: c_loc of an integer(c_int) / real(c_double) array, or c_null_ptr
    integer(c_int) function ccs_autotune(h, reps, force, chosen, times_us) bind(C, name='ccs_autotune')
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: reps, force
      type(c_ptr), value :: chosen, times_us
    end function ccs_autotune

    ! spatial_operator(stat(old), tend) (spatial_operators_mod.F90:13-181)
    integer(c_int) function ccs_spatial_operator(h, tend_phiG, tend_u, tend_v) bind(C, name='ccs_spatial_operator')
      import :: c_int, c_ptr
      type(c_ptr), value :: h, tend_phiG, tend_u, tend_v
    end function ccs_spatial_operator

    integer(c_int) function ccs_check_state(h, bad_cells) bind(C, name='ccs_check_state')
      import :: c_int, c_int64_t, c_ptr
      type(c_ptr), value :: h
      integer(c_int64_t), intent(out) :: bad_cells
    end function ccs_check_state

    integer(c_int) function ccs_courant(h, courant) bind(C, name='ccs_courant')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(out) :: courant
    end function ccs_courant

    ! calc_total_mass / calc_total_energy (diag_mod.F90:10-53) on the device
    integer(c_int) function ccs_diag(h, total_mass, total_energy) bind(C, name='ccs_diag')
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(out) :: total_mass, total_energy
    end function ccs_diag

    ! ensembles: members(1:n) are handles
    integer(c_int) function ccs_batch_create(members, n, b) bind(C, name='ccs_batch_create')
      import :: c_int, c_ptr
      type(c_ptr), intent(in) :: members(*)
      integer(c_int), value :: n
      type(c_ptr), intent(out) :: b
    end function ccs_batch_create

    integer(c_int) function ccs_batch_step(b, nsteps) bind(C, name='ccs_batch_step')
      import :: c_int, c_ptr
      type(c_ptr), value :: b
      integer(c_int), value :: nsteps
    end function ccs_batch_step

    subroutine ccs_batch_destroy(b) bind(C, name='ccs_batch_destroy')
      import :: c_ptr
      type(c_ptr), value :: b
    end subroutine ccs_batch_destroy

    ! restart files (the eight stat fields in the reference layout)
    integer(c_int) function ccs_state_write(path, N, halo, s) bind(C, name='ccs_state_write')
      import :: c_int, c_char, ccs_state_view
      character(kind=c_char), dimension(*), intent(in) :: path
      integer(c_int), value :: N, halo
      type(ccs_state_view), intent(in) :: s
    end function ccs_state_write

    integer(c_int) function ccs_state_read(path, N, halo, s) bind(C, name='ccs_state_read')
      import :: c_int, c_char, ccs_state_view
      character(kind=c_char), dimension(*), intent(in) :: path
      integer(c_int), value :: N, halo
      type(ccs_state_view), intent(in) :: s
    end function ccs_state_read

    ! C strings (const char *): convert with c_f_pointer
    type(c_ptr) function ccs_strerror(status) bind(C, name='ccs_strerror')
      import :: c_int, c_ptr
      integer(c_int), value :: status
    end function ccs_strerror

    type(c_ptr) function ccs_last_error(h) bind(C, name='ccs_last_error')
      import :: c_ptr
      type(c_ptr), value :: h
    end function ccs_last_error

    integer(c_int) function ccs_abi_version() bind(C, name='ccs_abi_version')
      import :: c_int
    end function ccs_abi_version
  end interface
end module ccs_gpu_mod


module ccs_gpu_driver_mod
  use, intrinsic :: iso_c_binding
  use ccs_gpu_mod
  implicit none

contains

  ! The handle of the run: the configuration from parameters_mod / constants_mod and
  ! the metric arrays read_mesh derived (io_mod.F90:15-307).  mesh_mod.F90:50
  ! declares `mesh` with the target attribute, so c_loc of its components is valid.
  subroutine ccs_gpu_init(h, precision)
    use parameters_mod, only: ite, xhalo, integral_scheme, dx, dy, dt
    use constants_mod, only: radius, gravity, Omega
    use mesh_mod, only: mesh
    type(c_ptr), intent(out) :: h
    integer(c_int), intent(in), optional :: precision
    type(ccs_config) :: cfg
    type(ccs_mesh_view) :: mv
    integer(c_int) :: lane, scheme

    lane = CCS_FP64
    if (present(precision)) lane = precision
    scheme = CCS_RK4
    if (trim(adjustl(integral_scheme)) == 'RK3_TVD') scheme = CCS_RK3_TVD
    cfg = ccs_config(int(ite, c_int), int(xhalo, c_int), scheme, lane, CCS_EDISS_ZERO, 0_c_int, &
                     real(dx, c_double), real(dy, c_double), real(dt, c_double), real(radius, c_double), &
                     real(gravity, c_double), real(Omega, c_double), 0._c_double)
    mv = ccs_mesh_view(c_loc(mesh%sqrtG), c_loc(mesh%matrixG), c_loc(mesh%matrixIG), c_loc(mesh%matrixA), &
                       c_loc(mesh%matrixIA), c_loc(mesh%f), c_loc(mesh%phis))
    call ccs_gpu_check(ccs_init(cfg, mv, h), 'ccs_init')
  end subroutine ccs_gpu_init

  ! A view of one stat_field (stat_mod.F90:19 declares `stat` with the target
  ! attribute).
  function state_view(s) result(v)
    use stat_mod, only: stat_field
    type(stat_field), target, intent(in) :: s
    type(ccs_state_view) :: v
    v = ccs_state_view(c_loc(s%phiG), c_loc(s%u), c_loc(s%v), c_loc(s%phi), c_loc(s%uC), c_loc(s%vC), &
                       c_loc(s%zonal_wind), c_loc(s%meridional_wind), c_loc(s%phit))
  end function state_view

  ! Stops with the library's message on a non-zero status, as the reference stops
  ! on its own errors (io_mod.F90:604-612).
  subroutine ccs_gpu_check(status, where)
    integer(c_int), intent(in) :: status
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    integer :: n

    if (status == CCS_OK) return
    call c_f_pointer(ccs_strerror(status), msg, [256])
    n = 0
    do while (n < 256)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    enddo
    print *, trim(where), ' failed: ', msg(1:n)
    stop 'ccs_gpu error'
  end subroutine ccs_gpu_check
end module ccs_gpu_driver_mod
