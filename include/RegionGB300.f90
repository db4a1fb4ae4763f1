! RegionGB300.f90 -- the magudi-side seam of the GB300 library: a module a
! maintainer adds to magudi's src/ (it uses magudi's own types, so it
! compiles inside the magudi tree, with MagudiGB300 from magudi_gb300.f90).
!
!   setupRegionGB300   after Region%setup and Solver%setup: fills mgd_options
!                      from region%simulationFlags / solverOptions, adds every
!                      grid (coordinates, iblank, periodicity), every bc.dat
!                      patch with the patches/<name>/... amounts of magudi.inp,
!                      the acoustic sources and the target state and
!                      mollifier arrays, then finalizes the context (the
!                      functional's mean pressure goes in the same way, with
!                      MGD_FIELD_MEAN_PRESSURE).
!   computeRhsGB300    the body of t_Region%computeRhs (include/Region.f90:184,
!                      src/RegionImpl.f90:1877-2027) for one process holding
!                      every block: the states go to the device, the library
!                      computes the RHS of every block (fluxes, dissipation,
!                      SATs, sponges, sources, interfaces) and it comes back
!                      into state%rightHandSide.
!   runForwardGB300 / runAdjointGB300
!                      Solver%runForward / runAdjoint (src/SolverImpl.f90:672,
!                      :914) with the checkpoints on the device; a
!                      solution-limit stop returns HUGE as the reference does.
!
! The call site in src/RegionImpl.f90 becomes
!     subroutine computeRhs(this, mode, timeStep, stage)
!       ...
!       call computeRhsGB300(this, mode)
!     end subroutine computeRhs
! and magudi.inp and bc.dat keep their meaning: nothing else reads them.
module RegionGB300

  use, intrinsic :: iso_c_binding
  use MagudiGB300

  implicit none
  private

  ! One context per process: every block of the region lives on one GPU.
  type(c_ptr), save :: gb300Context = c_null_ptr

  public :: setupRegionGB300, computeRhsGB300, runForwardGB300, runAdjointGB300, cleanupRegionGB300

contains

  subroutine check(status)
    use ErrorHandler, only : gracefulExit
    use MPI, only : MPI_COMM_WORLD
    integer(c_int), intent(in) :: status
    if (status /= 0_c_int) call gracefulExit(MPI_COMM_WORLD, mgdLastError(gb300Context))
  end subroutine check

  integer(c_int) function flag(value)
    logical, intent(in) :: value
    flag = merge(1_c_int, 0_c_int, value)
  end function flag

  integer(c_int) function schemeOf(name)
    character(len=*), intent(in) :: name
    select case (trim(name))
    case ("SBP 1-2")
       schemeOf = MGD_SBP_12
    case ("SBP 2-4")
       schemeOf = MGD_SBP_24
    case ("SBP 3-6")
       schemeOf = MGD_SBP_36
    case default
       schemeOf = MGD_SBP_48
    end select
  end function schemeOf

  integer(c_int) function patchTypeOf(name)
    character(len=*), intent(in) :: name
    select case (trim(name))
    case ("SAT_FAR_FIELD")
       patchTypeOf = MGD_PATCH_SAT_FAR_FIELD
    case ("SPONGE")
       patchTypeOf = MGD_PATCH_SPONGE
    case ("ACTUATOR")
       patchTypeOf = MGD_PATCH_ACTUATOR
    case ("COST_TARGET")
       patchTypeOf = MGD_PATCH_COST_TARGET
    case ("SAT_SLIP_WALL")
       patchTypeOf = MGD_PATCH_SLIP_WALL
    case ("SAT_ISOTHERMAL_WALL")
       patchTypeOf = MGD_PATCH_ISOTHERMAL_WALL
    case ("SAT_ADIABATIC_WALL")
       patchTypeOf = MGD_PATCH_ADIABATIC_WALL
    case ("SAT_BLOCK_INTERFACE")
       patchTypeOf = MGD_PATCH_BLOCK_INTERFACE
    case ("SOLENOIDAL_EXCITATION")
       patchTypeOf = MGD_PATCH_SOLENOIDAL_EXCITATION
    case default
       patchTypeOf = 0
    end select
  end function patchTypeOf

  subroutine setupRegionGB300(region)

    use Region_mod, only : t_Region
    use InputHelper, only : getOption
    use ErrorHandler, only : gracefulExit

    type(t_Region), intent(inout), target :: region

    integer, parameter :: wp = kind(0.0d0)
    type(mgd_options) :: o
    type(mgd_block_desc) :: b
    type(mgd_patch_desc) :: p
    type(mgd_acoustic_source) :: s
    integer :: i, nDimensions
    character(len=256) :: key
    integer(c_int), allocatable, target :: iblank(:)

    nDimensions = size(region%globalGridSizes, 1)
    o%n_dimensions = nDimensions
    o%viscous = flag(region%simulationFlags%viscosityOn)
    o%dissipation = flag(region%simulationFlags%dissipationOn)
    o%composite_dissipation = flag(region%simulationFlags%compositeDissipation)
    o%curvilinear = flag(region%simulationFlags%isDomainCurvilinear)
    o%use_constant_cfl = flag(region%simulationFlags%useConstantCfl)
    o%enable_controller = flag(region%simulationFlags%enableController)
    o%enable_functional = flag(region%simulationFlags%enableFunctional)
    o%controller_switch = flag(getOption("controller_switch", .false.))
    o%adjoint_forcing_switch = flag(region%simulationFlags%adjointForcingSwitch)
    o%ratio_of_specific_heats = region%solverOptions%ratioOfSpecificHeats
    ! the library takes Re and Pr; solverOptions holds their inverses
    o%reynolds_number = 0.0_wp
    o%prandtl_number = 0.0_wp
    if (region%solverOptions%reynoldsNumberInverse > 0.0_wp)                                 &
         o%reynolds_number = 1.0_wp / region%solverOptions%reynoldsNumberInverse
    if (region%solverOptions%prandtlNumberInverse > 0.0_wp)                                  &
         o%prandtl_number = 1.0_wp / region%solverOptions%prandtlNumberInverse
    o%viscosity_power_law_exponent = region%solverOptions%powerLawExponent
    o%bulk_viscosity_ratio = region%solverOptions%bulkViscosityRatio
    o%dissipation_amount = region%solverOptions%dissipationAmount
    o%time_step_size = region%solverOptions%timeStepSize
    o%cfl = region%solverOptions%cfl
    o%functional_type = MGD_FUNCTIONAL_SOUND
    o%enable_solution_limits = flag(region%simulationFlags%enableSolutionLimits)
    o%minimum_density = region%solverOptions%densityRange(1)
    o%maximum_density = region%solverOptions%densityRange(2)
    o%minimum_temperature = region%solverOptions%temperatureRange(1)
    o%maximum_temperature = region%solverOptions%temperatureRange(2)
    o%discretization_scheme = schemeOf(region%solverOptions%discretizationType)
    call check(mgd_create(o, gb300Context))

    do i = 1, size(region%grids)
       if (any(region%grids(i)%localSize /= region%grids(i)%globalSize))                      &
            call gracefulExit(region%comm, "the GB300 library holds whole blocks: run on one process")
       b%grid_size = 1
       b%grid_size(1:nDimensions) = region%grids(i)%globalSize(1:nDimensions)
       b%periodicity_type = region%grids(i)%periodicityType
       b%periodic_length = region%grids(i)%periodicLength
       allocate(iblank(size(region%grids(i)%iblank)))
       iblank = region%grids(i)%iblank
       call check(mgd_add_block(gb300Context, b, c_loc(region%grids(i)%coordinates), c_loc(iblank)))
       deallocate(iblank)
    end do

    do i = 1, size(region%patchData)
       associate (d => region%patchData(i))
         call mgdSetName(p%name, d%name)
         p%type = patchTypeOf(d%patchType)
         if (p%type == 0) call gracefulExit(region%comm, "patch type " // trim(d%patchType) //     &
              " is not on the GB300 path")
         p%grid_index = d%gridIndex
         p%normal_direction = d%normalDirection
         p%extent = [d%iMin, d%iMax, d%jMin, d%jMax, d%kMin, d%kMax]
         key = "patches/" // trim(d%name) // "/"
         p%inviscid_penalty_amount = getOption(trim(key) // "inviscid_penalty_amount",              &
              getOption("defaults/inviscid_penalty_amount", 1.0_wp))
         p%viscous_penalty_amount = getOption(trim(key) // "viscous_penalty_amount",                &
              getOption("defaults/viscous_penalty_amount", 1.0_wp))
         p%sponge_amount = getOption(trim(key) // "sponge_amount", getOption("defaults/sponge_amount", 1.0_wp))
         p%sponge_exponent = getOption(trim(key) // "sponge_exponent", getOption("defaults/sponge_exponent", 2))
         p%wall_temperature = 0.0_wp
         call mgdSetName(p%conforms_with, getOption(trim(key) // "conforms_with", ""))
         p%interface_index = [getOption(trim(key) // "interface_index1", 0),                      &
              getOption(trim(key) // "interface_index2", 0), getOption(trim(key) // "interface_index3", 0)]
         ! SOLENOIDAL_EXCITATION rows also pass c_loc of the patch object's
         ! angularFrequencies and phases after its setup (see magudi_gb300.h)
         p%n_modes = 0
         p%angular_frequencies = c_null_ptr
         p%phases = c_null_ptr
         call check(mgd_add_patch(gb300Context, p))
       end associate
    end do

    if (allocated(region%states(1)%acousticSources)) then
       do i = 1, size(region%states(1)%acousticSources)
          associate (a => region%states(1)%acousticSources(i))
            s%location = a%location
            s%amplitude = a%amplitude
            s%frequency = a%angularFrequency / (2.0_wp * 4.0_wp * atan(1.0_wp))
            s%radius = sqrt(9.0_wp / (2.0_wp * a%gaussianFactor))
            s%phase = a%phase
            call check(mgd_add_acoustic_source(gb300Context, s))
          end associate
       end do
    end if

    do i = 1, size(region%grids)
       call check(mgd_set_field(gb300Context, i, MGD_FIELD_TARGET, c_loc(region%states(i)%targetState)))
       if (allocated(region%grids(i)%controlMollifier))                                    &
            call check(mgd_set_field(gb300Context, i, MGD_FIELD_CONTROL_MOLLIFIER,            &
            c_loc(region%grids(i)%controlMollifier)))
       if (allocated(region%grids(i)%targetMollifier))                                     &
            call check(mgd_set_field(gb300Context, i, MGD_FIELD_TARGET_MOLLIFIER,             &
            c_loc(region%grids(i)%targetMollifier)))
    end do
    call check(mgd_finalize_setup(gb300Context))

  end subroutine setupRegionGB300

  ! t_Region%computeRhs for mode FORWARD, ADJOINT or LINEARIZED.
  subroutine computeRhsGB300(region, mode)

    use Region_mod, only : t_Region
    use Region_enum, only : FORWARD

    type(t_Region), intent(inout), target :: region
    integer, intent(in) :: mode

    integer :: i

    do i = 1, size(region%states)
       call check(mgd_set_field(gb300Context, i, MGD_FIELD_CONSERVED,                            &
            c_loc(region%states(i)%conservedVariables)))
       if (mode /= FORWARD) call check(mgd_set_field(gb300Context, i, MGD_FIELD_ADJOINT,           &
            c_loc(region%states(i)%adjointVariables)))
    end do
    call check(mgd_update_state(gb300Context))
    call check(mgd_compute_rhs(gb300Context, int(mode, c_int), region%states(1)%time,             &
         region%states(1)%adjointForcingFactor))
    do i = 1, size(region%states)
       call check(mgd_get_field(gb300Context, i, MGD_FIELD_RHS, c_loc(region%states(i)%rightHandSide)))
    end do

  end subroutine computeRhsGB300

  ! Solver%runForward from the current conserved variables: the whole run on
  ! the device, checkpoints every saveInterval steps kept there.
  function runForwardGB300(region, nTimesteps, saveInterval, time) result(costFunctional)

    use Region_mod, only : t_Region

    type(t_Region), intent(inout), target :: region
    integer, intent(in) :: nTimesteps, saveInterval
    real(kind(0.0d0)), intent(in) :: time
    real(kind(0.0d0)) :: costFunctional

    integer :: i, status
    real(c_double) :: cost

    do i = 1, size(region%states)
       call check(mgd_set_field(gb300Context, i, MGD_FIELD_CONSERVED,                            &
            c_loc(region%states(i)%conservedVariables)))
    end do
    status = mgd_run_forward(gb300Context, int(nTimesteps, c_int), int(saveInterval, c_int), time, cost)
    ! src/SolverImpl.f90:813-818: a solution-limit stop is HUGE, not an error
    if (status /= MGD_SOLUTION_LIMITS) call check(status)
    costFunctional = cost
    do i = 1, size(region%states)
       call check(mgd_get_field(gb300Context, i, MGD_FIELD_CONSERVED,                            &
            c_loc(region%states(i)%conservedVariables)))
    end do

  end function runForwardGB300

  ! Solver%runAdjoint over the horizon of the preceding runForwardGB300.
  function runAdjointGB300(region) result(costSensitivity)

    use Region_mod, only : t_Region

    type(t_Region), intent(inout), target :: region
    real(kind(0.0d0)) :: costSensitivity

    integer :: i, status
    real(c_double) :: sensitivity

    status = mgd_run_adjoint(gb300Context, sensitivity)
    if (status /= MGD_SOLUTION_LIMITS) call check(status)
    costSensitivity = sensitivity
    do i = 1, size(region%states)
       call check(mgd_get_field(gb300Context, i, MGD_FIELD_ADJOINT,                              &
            c_loc(region%states(i)%adjointVariables)))
    end do

  end function runAdjointGB300

  subroutine cleanupRegionGB300()
    if (c_associated(gb300Context)) call check(mgd_destroy(gb300Context))
    gb300Context = c_null_ptr
  end subroutine cleanupRegionGB300

end module RegionGB300
