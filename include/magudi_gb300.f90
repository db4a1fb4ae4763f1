! magudi_gb300.f90 -- ISO_C_BINDING interface of the C ABI in magudi_gb300.h
! for Fortran callers (magudi's Region/Solver code). Standard Fortran 2008,
! no dependency on magudi's own modules; RegionGB300.f90 shows the calls
! that replace t_Region%computeRhs and t_Solver%runForward/runAdjoint.
!
! The derived types mirror the C structs field for field and in the same
! order (bind(C) gives them the C layout); the parameters mirror the header's
! enums. Every function returns the C status: 0 success, MGD_SOLUTION_LIMITS
! for a run that stopped at a solution-limit violation (cost = HUGE), any
! other positive value an error whose text mgdLastError returns.
module MagudiGB300

  use, intrinsic :: iso_c_binding

  implicit none
  public

  ! include/Region.f90:9-11
  integer(c_int), parameter :: MGD_FORWARD = 1, MGD_ADJOINT = -1, MGD_LINEARIZED = 0

  integer(c_int), parameter :: MGD_PERIODIC_NONE = 0, MGD_PERIODIC_PLANE = 1, MGD_PERIODIC_OVERLAP = 2

  integer(c_int), parameter :: MGD_PATCH_SAT_FAR_FIELD = 1, MGD_PATCH_SPONGE = 2, MGD_PATCH_ACTUATOR = 3, &
       MGD_PATCH_COST_TARGET = 4, MGD_PATCH_SLIP_WALL = 5, MGD_PATCH_ISOTHERMAL_WALL = 6,                   &
       MGD_PATCH_ADIABATIC_WALL = 7, MGD_PATCH_BLOCK_INTERFACE = 8, MGD_PATCH_SOLENOIDAL_EXCITATION = 9

  integer(c_int), parameter :: MGD_FIELD_CONSERVED = 0, MGD_FIELD_ADJOINT = 1, MGD_FIELD_TARGET = 2,       &
       MGD_FIELD_RHS = 3, MGD_FIELD_CONTROL_MOLLIFIER = 4, MGD_FIELD_TARGET_MOLLIFIER = 5,                 &
       MGD_FIELD_MEAN_PRESSURE = 6, MGD_FIELD_METRICS = 7, MGD_FIELD_JACOBIAN = 8, MGD_FIELD_NORM = 9,     &
       MGD_FIELD_PRESSURE = 10, MGD_FIELD_TEMPERATURE = 11, MGD_FIELD_ARC_LENGTHS = 12

  integer(c_int), parameter :: MGD_SBP_48 = 0, MGD_SBP_12 = 1, MGD_SBP_24 = 2, MGD_SBP_36 = 3

  integer(c_int), parameter :: MGD_FUNCTIONAL_SOUND = 0, MGD_FUNCTIONAL_TERMINAL_KINETIC_ENERGY = 1

  integer(c_int), parameter :: MGD_SOLUTION_LIMITS = 2

  integer, parameter :: MGD_NAME_LEN = 64

  type, bind(C) :: mgd_options
     integer(c_int) :: n_dimensions
     integer(c_int) :: viscous
     integer(c_int) :: dissipation
     integer(c_int) :: composite_dissipation
     integer(c_int) :: curvilinear
     integer(c_int) :: use_constant_cfl
     integer(c_int) :: enable_controller
     integer(c_int) :: enable_functional
     integer(c_int) :: controller_switch
     integer(c_int) :: adjoint_forcing_switch
     real(c_double) :: ratio_of_specific_heats
     real(c_double) :: reynolds_number
     real(c_double) :: prandtl_number
     real(c_double) :: viscosity_power_law_exponent
     real(c_double) :: bulk_viscosity_ratio
     real(c_double) :: dissipation_amount
     real(c_double) :: time_step_size
     real(c_double) :: cfl
     integer(c_int) :: functional_type
     integer(c_int) :: enable_solution_limits
     real(c_double) :: minimum_density
     real(c_double) :: maximum_density
     real(c_double) :: minimum_temperature
     real(c_double) :: maximum_temperature
     integer(c_int) :: discretization_scheme
  end type mgd_options

  type, bind(C) :: mgd_block_desc
     integer(c_int) :: grid_size(3)
     integer(c_int) :: periodicity_type(3)
     real(c_double) :: periodic_length(3)
  end type mgd_block_desc

  type, bind(C) :: mgd_patch_desc
     character(kind=c_char) :: name(MGD_NAME_LEN)
     integer(c_int) :: type
     integer(c_int) :: grid_index
     integer(c_int) :: normal_direction
     integer(c_int) :: extent(6)
     real(c_double) :: inviscid_penalty_amount
     real(c_double) :: viscous_penalty_amount
     real(c_double) :: sponge_amount
     integer(c_int) :: sponge_exponent
     real(c_double) :: wall_temperature
     character(kind=c_char) :: conforms_with(MGD_NAME_LEN)
     integer(c_int) :: interface_index(3)
     integer(c_int) :: n_modes
     real(c_double) :: origin(2)
     real(c_double) :: velocity(2)
     real(c_double) :: amplitude
     real(c_double) :: radius
     type(c_ptr) :: angular_frequencies
     type(c_ptr) :: phases
  end type mgd_patch_desc

  type, bind(C) :: mgd_acoustic_source
     real(c_double) :: location(3)
     real(c_double) :: amplitude
     real(c_double) :: frequency
     real(c_double) :: radius
     real(c_double) :: phase
  end type mgd_acoustic_source

  interface

     type(c_ptr) function mgd_last_error(ctx) bind(C, name="mgd_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function mgd_last_error

     integer(c_int) function mgd_create(options, ctx) bind(C, name="mgd_create")
       import :: c_int, c_ptr, mgd_options
       type(mgd_options), intent(in) :: options
       type(c_ptr), intent(out) :: ctx
     end function mgd_create

     integer(c_int) function mgd_destroy(ctx) bind(C, name="mgd_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function mgd_destroy

     integer(c_int) function mgd_add_block(ctx, block, coordinates, iblank) bind(C, name="mgd_add_block")
       import :: c_int, c_ptr, mgd_block_desc
       type(c_ptr), value :: ctx
       type(mgd_block_desc), intent(in) :: block
       type(c_ptr), value :: coordinates, iblank
     end function mgd_add_block

     integer(c_int) function mgd_add_patch(ctx, patch) bind(C, name="mgd_add_patch")
       import :: c_int, c_ptr, mgd_patch_desc
       type(c_ptr), value :: ctx
       type(mgd_patch_desc), intent(in) :: patch
     end function mgd_add_patch

     integer(c_int) function mgd_add_acoustic_source(ctx, source) bind(C, name="mgd_add_acoustic_source")
       import :: c_int, c_ptr, mgd_acoustic_source
       type(c_ptr), value :: ctx
       type(mgd_acoustic_source), intent(in) :: source
     end function mgd_add_acoustic_source

     integer(c_int) function mgd_set_field(ctx, block, field, array) bind(C, name="mgd_set_field")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, array
       integer(c_int), value :: block, field
     end function mgd_set_field

     integer(c_int) function mgd_get_field(ctx, block, field, array) bind(C, name="mgd_get_field")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, array
       integer(c_int), value :: block, field
     end function mgd_get_field

     integer(c_int) function mgd_finalize_setup(ctx) bind(C, name="mgd_finalize_setup")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function mgd_finalize_setup

     integer(c_int) function mgd_update_state(ctx) bind(C, name="mgd_update_state")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function mgd_update_state

     integer(c_int) function mgd_compute_rhs(ctx, mode, time, factor) bind(C, name="mgd_compute_rhs")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: mode
       real(c_double), value :: time, factor
     end function mgd_compute_rhs

     integer(c_int) function mgd_update_adjoint_forcing(ctx, no_adjoint_forcing) &
          bind(C, name="mgd_update_adjoint_forcing")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: no_adjoint_forcing
     end function mgd_update_adjoint_forcing

     integer(c_int) function mgd_compute_functional(ctx, value) bind(C, name="mgd_compute_functional")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: value
     end function mgd_compute_functional

     integer(c_int) function mgd_compute_sensitivity(ctx, value) bind(C, name="mgd_compute_sensitivity")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: value
     end function mgd_compute_sensitivity

     integer(c_int) function mgd_rk4_substep(ctx, mode, time, dt, stage) bind(C, name="mgd_rk4_substep")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: mode, stage
       real(c_double), intent(inout) :: time
       real(c_double), value :: dt
     end function mgd_rk4_substep

     integer(c_int) function mgd_set_control_forcing(ctx, host, n_entries) bind(C, name="mgd_set_control_forcing")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: ctx, host
       integer(c_long_long), value :: n_entries
     end function mgd_set_control_forcing

     integer(c_int) function mgd_actuator_patch_size(ctx, n_points) bind(C, name="mgd_actuator_patch_size")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: ctx
       integer(c_long_long), intent(out) :: n_points
     end function mgd_actuator_patch_size

     integer(c_int) function mgd_run_forward(ctx, n_steps, save_interval, t0, cost) bind(C, name="mgd_run_forward")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: n_steps, save_interval
       real(c_double), value :: t0
       real(c_double), intent(out) :: cost
     end function mgd_run_forward

     integer(c_int) function mgd_time_step_size(ctx, dt) bind(C, name="mgd_time_step_size")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: dt
     end function mgd_time_step_size

     integer(c_int) function mgd_run_adjoint(ctx, sensitivity) bind(C, name="mgd_run_adjoint")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: sensitivity
     end function mgd_run_adjoint

     integer(c_int) function mgd_check_solution_limits(ctx, within) bind(C, name="mgd_check_solution_limits")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: within
     end function mgd_check_solution_limits

     integer(c_int) function mgd_run_linearized(ctx, delta_forcing, n_entries, delta_cost) &
          bind(C, name="mgd_run_linearized")
       import :: c_int, c_ptr, c_long_long, c_double
       type(c_ptr), value :: ctx, delta_forcing
       integer(c_long_long), value :: n_entries
       real(c_double), intent(out) :: delta_cost
     end function mgd_run_linearized

     integer(c_int) function mgd_set_patch_control_forcing(ctx, forcing) &
          bind(C, name="mgd_set_patch_control_forcing")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, forcing
     end function mgd_set_patch_control_forcing

     integer(c_int) function mgd_set_trajectory_storage(ctx, enable, max_bytes) &
          bind(C, name="mgd_set_trajectory_storage")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: enable
       real(c_double), value :: max_bytes
     end function mgd_set_trajectory_storage

     integer(c_int) function mgd_set_adjoint_nonzero_initial_condition(ctx, enable) &
          bind(C, name="mgd_set_adjoint_nonzero_initial_condition")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: enable
     end function mgd_set_adjoint_nonzero_initial_condition

     integer(c_int) function mgd_get_gradient(ctx, host, n_entries) bind(C, name="mgd_get_gradient")
       import :: c_int, c_ptr, c_long_long
       type(c_ptr), value :: ctx, host
       integer(c_long_long), value :: n_entries
     end function mgd_get_gradient

     integer(c_int) function mgd_tune_run(ctx, n_steps, save_interval, with_adjoint, best_ms) &
          bind(C, name="mgd_tune_run")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: n_steps, save_interval, with_adjoint
       real(c_double), intent(out) :: best_ms
     end function mgd_tune_run

     integer(c_int) function mgd_save_solution(ctx, filename, field, timestep, time) &
          bind(C, name="mgd_save_solution")
       import :: c_int, c_ptr, c_char, c_double
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: filename(*)
       integer(c_int), value :: field, timestep
       real(c_double), value :: time
     end function mgd_save_solution

     integer(c_int) function mgd_wait_io(ctx) bind(C, name="mgd_wait_io")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function mgd_wait_io

     ! the actuator streams and ZAXPY of magudi's optimisation drivers
     ! (.gradient_<patch>.dat / .control_forcing_<patch>.dat, bin/ZAXPY.f90)
     integer(c_int) function mgd_save_gradient(ctx, prefix, n_entries) bind(C, name="mgd_save_gradient")
       import :: c_int, c_ptr, c_char, c_long_long
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: prefix(*)
       integer(c_long_long), value :: n_entries
     end function mgd_save_gradient

     integer(c_int) function mgd_load_control_forcing(ctx, prefix, n_entries) &
          bind(C, name="mgd_load_control_forcing")
       import :: c_int, c_ptr, c_char, c_long_long
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: prefix(*)
       integer(c_long_long), value :: n_entries
     end function mgd_load_control_forcing

     integer(c_int) function mgd_control_zaxpy(ctx, a, accumulate) bind(C, name="mgd_control_zaxpy")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: a
       integer(c_int), value :: accumulate
     end function mgd_control_zaxpy

     ! the step sizes of the last forward run, one per step (the adjoint run uses the same)
     integer(c_int) function mgd_get_step_sizes(ctx, host, n_steps) bind(C, name="mgd_get_step_sizes")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, host
       integer(c_int), value :: n_steps
     end function mgd_get_step_sizes

     ! the actuator patches' quadrature weights H*det (mgd_actuator_patch_size entries, 0 on holes)
     integer(c_int) function mgd_actuator_weights(ctx, out) bind(C, name="mgd_actuator_weights")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, out
     end function mgd_actuator_weights

     ! forward RHS of device arrays q and rhs without any device allocation
     integer(c_int) function mgd_forward_rhs_noalloc(ctx, q, time, rhs) bind(C, name="mgd_forward_rhs_noalloc")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx, q, rhs
       real(c_double), value :: time
     end function mgd_forward_rhs_noalloc

     integer(c_size_t) function c_strlen(s) bind(C, name="strlen")
       import :: c_size_t, c_ptr
       type(c_ptr), value :: s
     end function c_strlen

  end interface

contains

  ! The text of mgd_last_error(ctx) as a Fortran string.
  function mgdLastError(ctx) result(message)
    type(c_ptr), intent(in) :: ctx
    character(len=:), allocatable :: message
    type(c_ptr) :: p
    character(kind=c_char), pointer :: chars(:)
    integer :: i, n
    p = mgd_last_error(ctx)
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: message)
    do i = 1, n
       message(i:i) = chars(i)
    end do
  end function mgdLastError

  ! A Fortran string into a NUL-padded C name field.
  subroutine mgdSetName(field, name)
    character(kind=c_char), intent(out) :: field(MGD_NAME_LEN)
    character(len=*), intent(in) :: name
    integer :: i
    field = c_null_char
    do i = 1, min(len_trim(name), MGD_NAME_LEN - 1)
       field(i) = name(i:i)
    end do
  end subroutine mgdSetName

end module MagudiGB300
