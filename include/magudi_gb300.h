/*
 * magudi_gb300.h -- C ABI of the GB300 (sm_103a) implementation of magudi's
 * forward and discrete-adjoint compressible Navier-Stokes right-hand side,
 * its RK4 stage updates, the acoustic-noise functional, the thermal-actuator
 * gradient and uniform checkpointing.
 *
 * Every entry point is plain C: pointers, sizes and status codes. Status 0 is
 * success; a positive value is an error whose text mgd_last_error() returns.
 * Arrays use magudi's Fortran column-major layout x(nGridPoints, nComponents):
 * component c of grid point p = i + Nx*(j + Ny*k) (0-based) sits at
 * x[p + nGridPoints*c]. A Fortran caller therefore passes c_loc(array) with no
 * copy. One context owns one region (a set of blocks on one GPU) and one CUDA
 * stream; calls on one context must come from one host thread at a time.
 *
 * The reference interface each call replaces is named beside it
 * (paths relative to the magudi source tree).
 */
#ifndef MAGUDI_GB300_H
#define MAGUDI_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define MGD_MAX_BLOCKS 8
#define MGD_MAX_PATCHES 64
#define MGD_MAX_SOURCES 8
#define MGD_NAME_LEN 64

/* include/Region.f90:9-11 (FORWARD = +1, ADJOINT = -1, LINEARIZED = 0). */
enum { MGD_FORWARD = 1, MGD_ADJOINT = -1, MGD_LINEARIZED = 0 };

/* src/GridImpl.f90:202-210 periodicity types. */
enum { MGD_PERIODIC_NONE = 0, MGD_PERIODIC_PLANE = 1, MGD_PERIODIC_OVERLAP = 2 };

/* Patch types of src/PatchFactoryImpl.f90:43-84 that this library implements. */
enum {
  MGD_PATCH_SAT_FAR_FIELD = 1,
  MGD_PATCH_SPONGE = 2,
  MGD_PATCH_ACTUATOR = 3,
  MGD_PATCH_COST_TARGET = 4,
  MGD_PATCH_SLIP_WALL = 5,         /* SAT_SLIP_WALL: t_ImpenetrableWall */
  MGD_PATCH_ISOTHERMAL_WALL = 6,   /* SAT_ISOTHERMAL_WALL */
  MGD_PATCH_ADIABATIC_WALL = 7,    /* SAT_ADIABATIC_WALL */
  MGD_PATCH_BLOCK_INTERFACE = 8,   /* SAT_BLOCK_INTERFACE */
  MGD_PATCH_SOLENOIDAL_EXCITATION = 9 /* SOLENOIDAL_EXCITATION */
};

/* Fields that mgd_set_field / mgd_get_field move between host and device. */
enum {
  MGD_FIELD_CONSERVED = 0,         /* state%conservedVariables (N, nU)   */
  MGD_FIELD_ADJOINT = 1,           /* state%adjointVariables   (N, nU)   */
  MGD_FIELD_TARGET = 2,            /* state%targetState        (N, nU)   */
  MGD_FIELD_RHS = 3,               /* state%rightHandSide      (N, nU)   */
  MGD_FIELD_CONTROL_MOLLIFIER = 4, /* grid%controlMollifier    (N, 1)    */
  MGD_FIELD_TARGET_MOLLIFIER = 5,  /* grid%targetMollifier     (N, 1)    */
  MGD_FIELD_MEAN_PRESSURE = 6,     /* AcousticNoise meanPressure (N, 1)  */
  MGD_FIELD_METRICS = 7,           /* grid%metrics   (N, nD*nD)  read-only */
  MGD_FIELD_JACOBIAN = 8,          /* grid%jacobian  (N, 1) = 1/det      */
  MGD_FIELD_NORM = 9,              /* grid%norm      (N, 1) = H*det      */
  MGD_FIELD_PRESSURE = 10,         /* state%pressure (N, 1)  read-only   */
  MGD_FIELD_TEMPERATURE = 11,      /* state%temperature (N, 1) read-only */
  MGD_FIELD_ARC_LENGTHS = 12       /* grid%arcLengths (N, nD) read-only  */
};

/* Region-wide options: the keys of magudi.inp that parameterize the hot path
 * (src/SimulationFlagsImpl.f90:24-45, src/SolverOptionsImpl.f90:46-135). */
typedef struct {
  int n_dimensions;                  /* 2 or 3 */
  int viscous;                       /* include_viscous_terms */
  int dissipation;                   /* add_dissipation */
  int composite_dissipation;         /* composite_dissipation */
  int curvilinear;                   /* curvilinear_domain */
  int use_constant_cfl;              /* use_constant_CFL_mode */
  int enable_controller;             /* enable_controller */
  int enable_functional;             /* enable_functional */
  int controller_switch;             /* controller_switch: add the control forcing */
  int adjoint_forcing_switch;        /* adjoint_forcing_switch */
  double ratio_of_specific_heats;    /* ratio_of_specific_heats */
  double reynolds_number;            /* Reynolds_number */
  double prandtl_number;             /* Prandtl_number */
  double viscosity_power_law_exponent;
  double bulk_viscosity_ratio;
  double dissipation_amount;
  double time_step_size;
  double cfl;
  int functional_type;               /* MGD_FUNCTIONAL_*: which cost functional J is */
  /* Solution limits (enable_solution_limits, minimum_density,
   * maximum_density, minimum_temperature, maximum_temperature;
   * src/SimulationFlagsImpl.f90:34, src/SolverOptionsImpl.f90:73-78): with
   * the flag set, a forward run checks the density and the temperature of
   * every grid point at the start of every RK stage, as
   * checkSolutionLimits (src/SolverImpl.f90:189-304) does, and stops at the
   * first stage whose state lies outside the open ranges (non-finite values
   * count as outside); see MGD_SOLUTION_LIMITS. */
  int enable_solution_limits;
  double minimum_density;
  double maximum_density;
  double minimum_temperature;
  double maximum_temperature;
  int discretization_scheme;         /* MGD_SBP_*: defaults/discretization_scheme */
} mgd_options;

/* Status of mgd_run_forward / mgd_run_adjoint when the solution left the
 * limits (not a failure of the call): the run stopped as Solver%runForward
 * does on a checkSolutionLimits violation (src/SolverImpl.f90:813-818,
 * 1193-1198) and its cost (or sensitivity) is HUGE (DBL_MAX). The
 * conserved variables are left at the violating state (the state the
 * reference saves as "<prefix>-crashed.q"), and mgd_last_error names the
 * quantity, block, grid point, value, step and stage. An mgd_run_adjoint
 * after such a run returns the same status with a HUGE sensitivity. */
#define MGD_SOLUTION_LIMITS 2

/* defaults/discretization_scheme (src/StencilOperatorImpl.f90:1164-1960):
 * the SBP first derivative with its composite and non-composite artificial
 * dissipation. SBP 1-2 has no non-composite dissipation. */
enum {
  MGD_SBP_48 = 0, /* "SBP 4-8" */
  MGD_SBP_12 = 1, /* "SBP 1-2" */
  MGD_SBP_24 = 2, /* "SBP 2-4" */
  MGD_SBP_36 = 3  /* "SBP 3-6" */
};

/* Cost functionals. SOUND is the reference's acoustic-noise functional
 * (functional_type = "SOUND", src/AcousticNoiseImpl.f90), integrated in time
 * over the cost-target patches. TERMINAL_KINETIC_ENERGY (no reference
 * counterpart) is the kinetic energy sum H det rho |u|^2 / 2 over the whole
 * grid at the final step; its adjoint starts from lambda(T) = H^-1 dJ/dq(T)
 * and has no forcing during the run. */
enum {
  MGD_FUNCTIONAL_SOUND = 0,
  MGD_FUNCTIONAL_TERMINAL_KINETIC_ENERGY = 1
};

/* One block of the region: its size and periodicity (grid00N/dirM/...). */
typedef struct {
  int grid_size[3];                  /* 1 for unused dimensions */
  int periodicity_type[3];           /* MGD_PERIODIC_* */
  double periodic_length[3];
} mgd_block_desc;

/* One row of bc.dat plus the patch options read from magudi.inp
 * (src/RegionImpl.f90:175-337, src/PatchDescriptorImpl.f90:40-100). */
typedef struct {
  char name[MGD_NAME_LEN];
  int type;                          /* MGD_PATCH_* */
  int grid_index;                    /* 1-based block index */
  int normal_direction;              /* +-1..3, 0 */
  int extent[6];                     /* iMin iMax jMin jMax kMin kMax as in bc.dat */
  double inviscid_penalty_amount;    /* patches/<name>/inviscid_penalty_amount */
  double viscous_penalty_amount;     /* patches/<name>/viscous_penalty_amount
                                        (viscous_penalty_amount1 for isothermal walls) */
  double sponge_amount;              /* patches/<name>/sponge_amount */
  int sponge_exponent;               /* patches/<name>/sponge_exponent */
  double wall_temperature;           /* isothermal walls: patches/<name>/temperature, or
                                        <= 0 for the target state's temperature
                                        (use_target_state, src/PatchFactoryImpl.f90:512-538) */
  char conforms_with[MGD_NAME_LEN];  /* block interfaces: patches/<name>/conforms_with */
  int interface_index[3];            /* patches/<name>/interface_index1..3 (0 = default 1,2,3)
                                        (src/InterfaceHelperImpl.f90:3-113) */
  /* Solenoidal excitation (src/SolenoidalExcitationPatchImpl.f90:3-120):
     patches/<name>/number_of_modes, origin_x/y, velocity_x/y, amplitude and
     radius, and the modes the reference draws at setup: angular_frequencies
     (n_modes) and phases (n_modes x 3, mode index fastest), already scaled
     as its setup scales them (2 pi frequency (l + r_l - 1/2) / (n_modes / 2)
     and 2 pi r). The arrays are copied by mgd_add_patch. */
  int n_modes;
  double origin[2];
  double velocity[2];
  double amplitude;
  double radius;
  const double* angular_frequencies;
  const double* phases;
} mgd_patch_desc;

/* acoustic_sourceNN/... (src/AcousticSourceImpl.f90:3-32). */
typedef struct {
  double location[3];
  double amplitude;
  double frequency;
  double radius;
  double phase;
} mgd_acoustic_source;

typedef struct mgd_ctx mgd_ctx;

/* Text of the last error on ctx (or of the last failed mgd_create when ctx is
 * NULL). Replaces gracefulExit's message, src/ErrorHandlerImpl.f90:162. */
const char* mgd_last_error(const mgd_ctx* ctx);

/* Region%setup + Solver%setup options (src/RegionImpl.f90:1225,
 * src/SolverImpl.f90:445). Creates a context on the current CUDA device. */
int mgd_create(const mgd_options* options, mgd_ctx** out);
int mgd_destroy(mgd_ctx* ctx);

/* Grid%setup + Grid%update (src/GridImpl.f90:487-1066): adds block
 * number (count of earlier calls + 1) with its coordinates (N, nD) and iblank
 * (N); metrics, 1/det, H*det and arc lengths are computed on the device.
 * Each direction needs at least 25 points when it is not periodic (the
 * operators' closure windows), 4 when PLANE-periodic and 5 when
 * OVERLAP-periodic (the stencils reach 4 points to either side and wrap
 * once); smaller blocks are refused with an error. */
int mgd_add_block(mgd_ctx* ctx, const mgd_block_desc* block,
                  const double* coordinates, const int* iblank);

/* Region%readBoundaryConditions (src/RegionImpl.f90:175) for one bc.dat row. */
int mgd_add_patch(mgd_ctx* ctx, const mgd_patch_desc* patch);

/* State%setup acoustic sources (src/StateImpl.f90:135-150). */
int mgd_add_acoustic_source(mgd_ctx* ctx, const mgd_acoustic_source* source);

/* Region%loadData / saveData for one field of one block (src/RegionImpl.f90:1489).
 * The pointer may be host or device memory (unified addressing). */
int mgd_set_field(mgd_ctx* ctx, int block, int field, const double* host);
int mgd_get_field(mgd_ctx* ctx, int block, int field, double* host);

/* The rest of Solver%setup: computeSpongeStrengths (src/PatchFactoryImpl.f90:161),
 * updatePatchFactories (:446), mollifier normalization
 * (src/RegionImpl.f90:459-603) and the time-invariant far-field SAT matrices.
 * Call once after blocks, patches, target state and mollifiers are set. */
int mgd_finalize_setup(mgd_ctx* ctx);

/* State%update on every block (src/StateImpl.f90:466-537). */
int mgd_update_state(mgd_ctx* ctx);

/* Region%computeRhs (src/RegionImpl.f90:1877-2027). mode = MGD_FORWARD,
 * MGD_ADJOINT or MGD_LINEARIZED; time is state%time; adjoint_forcing_factor is
 * state%adjointForcingFactor. MGD_LINEARIZED (computeRhsLinearized,
 * src/RhsHelperImpl.f90:598-829) is the tangent RHS of the perturbation held
 * in MGD_FIELD_ADJOINT (the reference keeps it in adjointVariables) about the
 * current conserved state; it covers far-field, wall, sponge, actuator and
 * cost-target patches and refuses block interfaces and excitations. The result stays on the device
 * (read it with mgd_get_field(..., MGD_FIELD_RHS, ...)). */
int mgd_compute_rhs(mgd_ctx* ctx, int mode, double time, double adjoint_forcing_factor);

/* Functional%updateAdjointForcing (src/FunctionalImpl.f90:26-72). */
int mgd_update_adjoint_forcing(mgd_ctx* ctx, int no_adjoint_forcing);

/* AcousticNoise%compute (src/AcousticNoiseImpl.f90:123-206). */
int mgd_compute_functional(mgd_ctx* ctx, double* value);

/* ThermalActuator%computeSensitivity (src/ThermalActuatorImpl.f90:83-159). */
int mgd_compute_sensitivity(mgd_ctx* ctx, double* value);

/* RK4Integrator%substepForward / substepAdjoint / substepLinearized
 * (src/RK4IntegratorImpl.f90:65-380), followed for the forward mode by
 * State%update as Solver%runForward does (src/SolverImpl.f90:827-834).
 * *time is advanced (forward) or retreated (adjoint) as the reference does. */
int mgd_rk4_substep(mgd_ctx* ctx, int mode, double* time, double dt, int stage);

/* Control forcing for controller_switch = true, in the order the reference
 * reads it from <prefix>.control_forcing_<patch>.dat: entry e (0-based) holds
 * the actuator-patch values of the (e)-th stage counted backwards from the
 * last stage of the run, nPatchPoints doubles each
 * (src/ThermalActuatorImpl.f90:161-233, src/ActuatorPatchImpl.f90:226). */
int mgd_set_control_forcing(mgd_ctx* ctx, const double* host, long long n_entries);
/* (The forcing and gradient buffers of mgd_set_control_forcing and
 * mgd_get_gradient may be host or device memory.) */

/* Number of actuator-patch points (the length of one forcing/gradient entry). */
int mgd_actuator_patch_size(mgd_ctx* ctx, long long* n_points);

/* Quadrature weight H*det of each actuator-patch point in patch order, 0 on
 * holes (computeQuadratureOnPatches, src/PatchFactoryImpl.f90:376-444):
 * the weights with which ThermalActuator%computeSensitivity sums the
 * gradient (src/ThermalActuatorImpl.f90:83-159). out: host or device memory. */
int mgd_actuator_weights(mgd_ctx* ctx, double* out);

/* Solver%runForward (src/SolverImpl.f90:672-912) from the current conserved
 * variables at time t0 for n_steps RK4 steps; keeps a snapshot every
 * save_interval steps in device memory for a following mgd_run_adjoint.
 * The step size is time_step_size, or in constant-CFL mode the step size of
 * the state at the start of each step (src/SolverImpl.f90:809), evaluated on
 * the device. *cost = the time-integrated functional. */
int mgd_run_forward(mgd_ctx* ctx, int n_steps, int save_interval, double t0, double* cost);

/* Region%getTimeStepSize (src/RegionImpl.f90:1842-1875 with
 * computeTimeStepSize, src/CNSHelperImpl.f90:913-982): time_step_size, or in
 * constant-CFL mode the minimum over the grid of the advective and viscous
 * CFL bounds of the current conserved variables. */
int mgd_time_step_size(mgd_ctx* ctx, double* dt);

/* Step sizes of the steps of the last mgd_run_forward (n_steps doubles);
 * the adjoint run uses the same ones. */
int mgd_get_step_sizes(mgd_ctx* ctx, double* host, int n_steps);

/* Solver%runAdjoint (src/SolverImpl.f90:914-1245) over the horizon of the
 * preceding mgd_run_forward, with UniformCheckpointer recomputation
 * (src/UniformCheckpointerImpl.f90:80-208) from the device snapshots.
 * *sensitivity = the time-integrated cost sensitivity (Grad0). */
int mgd_run_adjoint(mgd_ctx* ctx, double* sensitivity);

/* checkSolutionLimits (src/SolverImpl.f90:189-304) for hosts that drive the
 * per-call entry points: *within = 1 when the density and the temperature of
 * every grid point of every block lie strictly inside the ranges set in
 * the options struct (the primitive variables must be current: see mgd_update_state),
 * else 0 with the reference's message in mgd_last_error. Needs
 * enable_solution_limits. */
int mgd_check_solution_limits(mgd_ctx* ctx, int* within);

/* Solver%runLinearized (src/SolverImpl.f90:1300-1450) over the steps of the
 * last mgd_run_forward: the perturbation held in MGD_FIELD_ADJOINT (the
 * linearized initial condition) advances with substepLinearizedRK4 along the
 * checkpointed forward trajectory, with the forward run's step sizes; the
 * final perturbation is left in MGD_FIELD_ADJOINT and the conserved state of
 * the final step is kept. delta_forcing (host or device, may be NULL) is a
 * control perturbation of n_entries entries in the control-forcing layout,
 * added by the actuators as the reference's deltaControlForcing
 * (src/ActuatorPatchImpl.f90:162-170). *delta_cost (may be NULL) receives the
 * tangent of the time-integrated SOUND functional: with a zero initial
 * perturbation, the directional derivative of J along delta_forcing, the
 * forward-mode counterpart of mgd_run_adjoint's gradient. Multi-block
 * regions carry the block-interface SATs; the patch types of MGD_LINEARIZED. */
int mgd_run_linearized(mgd_ctx* ctx, const double* delta_forcing, long long n_entries, double* delta_cost);

/* The actuator patches' controlForcing for the per-call forward RHS
 * (mgd_compute_rhs, mgd_rk4_substep, MGD_FORWARD): nPatchPoints values per
 * actuator patch, concatenated in patch order (mgd_actuator_patch_size), as
 * the controller's updateForcing fills them for the coming stage
 * (src/ThermalActuatorImpl.f90:161-233); the RHS adds control mollifier x
 * forcing to the energy equation (src/ActuatorPatchImpl.f90:108-181) while
 * controller_switch is on. Host or device pointer; NULL clears it. The
 * checkpointed runs take their forcing from mgd_set_control_forcing instead. */
int mgd_set_patch_control_forcing(mgd_ctx* ctx, const double* forcing);

/* Resident trajectory (no reference counterpart; the reference always
 * recomputes checkpoint segments, src/SolverImpl.f90:1027-1245 with
 * UniformCheckpointer): with enable != 0, mgd_run_forward also stores every
 * RK stage's state, primitives, stress and heat flux of every block on the
 * device when the 4 x n_steps stage slots of all blocks fit in max_bytes
 * (<= 0: half of the free device memory), and the following mgd_run_adjoint
 * reads them instead of recomputing the segments between checkpoints. The
 * results are identical either way. mgd_run_linearized reads the same slots
 * and leaves them for a later mgd_run_adjoint. Runs that do not fit
 * recompute as usual. Off by default: a forward-only user would hold the
 * slots for nothing. */
int mgd_set_trajectory_storage(mgd_ctx* ctx, int enable, double max_bytes);

/* adjoint_nonzero_initial_condition (src/SolverImpl.f90:1027-1102, set per
 * segment by bin/msadjoint.f90:141-400): when enabled, mgd_run_adjoint starts
 * from the adjoint field the context holds (loaded with mgd_set_field(...,
 * MGD_FIELD_ADJOINT, ...)) instead of zero, and adds the final step's
 * cost-target forcing (or the terminal functional's gradient) to it, as
 * loadInitialCondition(ADJOINT) does with a restart file
 * (src/SolverImpl.f90:368-427). Stays as set until changed; off at creation. */
int mgd_set_adjoint_nonzero_initial_condition(mgd_ctx* ctx, int enable);

/* The gradient vector of the last mgd_run_adjoint, in the order the reference
 * writes <prefix>.gradient_<patch>.dat (ThermalActuator%updateGradient,
 * src/ThermalActuatorImpl.f90:383-443): 4*n_steps entries of nPatchPoints. */
int mgd_get_gradient(mgd_ctx* ctx, double* host, long long n_entries);

/* Batched forward runs. The reference runs its gradient-accuracy sweep as one
 * ./forward process per control amplitude after ./zaxpy (README.md:118-165,
 * bin/ZAXPY.f90); a batch runs many such forward solves at once. A batch
 * groups finalized single-block contexts on one device whose options agree
 * except for the grids (constant time_step_size). mgd_batch_run_forward
 * advances every instance n_steps RK4 steps from its current conserved
 * variables and control forcing (Solver%runForward, src/SolverImpl.f90:672-912,
 * without snapshots); each stage kernel is one launch for the whole batch and
 * each step is one CUDA graph. costs[i] receives instance i's functional;
 * the final states stay in the instances. Tile shapes are chosen per grid
 * size by timing candidate shapes at mgd_batch_create. */
typedef struct mgd_batch mgd_batch;
int mgd_batch_create(mgd_ctx* const* instances, int n_instances, mgd_batch** batch);
int mgd_batch_run_forward(mgd_batch* batch, int n_steps, double t0, double* costs);
int mgd_batch_destroy(mgd_batch* batch);
const char* mgd_batch_last_error(const mgd_batch* batch);
/* How a batch runs (no reference counterpart): mode 1 (the default) runs
 * all steps of mgd_batch_run_forward as one persistent cooperative launch,
 * captured in a CUDA graph, whose CTAs draw (instance, stage phase, tile)
 * units from a device work queue, each unit waiting only for its own
 * instance's previous phase; mode 0 launches one graph of batched stage
 * kernels per step; other values only report. Returns the mode in effect.
 * Both give the same costs, bit for bit. */
int mgd_batch_persistent(mgd_batch* batch, int mode);
/* CTAs of the persistent launch (co-resident on the device). */
int mgd_batch_persistent_grid(mgd_batch* batch);
long long mgd_batch_kernel_launches(mgd_batch* batch, int reset);

/* ---- files around the hot path (host code; no GPU needed) ---- */

/* PLOT3D whole-format multi-block files as magudi writes them
 * (write_skeleton, src/PLOT3DFormat.c:208-292; plot3dWriteSingleGrid /
 * plot3dWriteSingleSolution, src/PLOT3DHelperImpl.f90:554-784): 4-byte
 * record markers, native byte order. Grid: x, y, z and iblank of each block
 * (z = 0 in 2D). Solution: a 4-double auxiliary header per block
 * (timestep, 0, 0, time) and 5 component slots, components 1..n-1 in slots
 * 1..n-1 and the last (energy) in slot 5. grid_sizes: 3 per grid; arrays are
 * component-major (N per component) per grid. */
int mgd_plot3d_write_grid(const char* filename, int n_grids, const int* grid_sizes, int n_dimensions,
                          const double* const* coordinates, const int* const* iblank);
int mgd_plot3d_write_solution(const char* filename, int n_grids, const int* grid_sizes, int n_components,
                              const double* const* q, const double* aux);
int mgd_plot3d_read_solution(const char* filename, int n_grids, const int* grid_sizes, int n_components,
                             double* const* q, double* aux);

/* Actuator-patch control forcing / gradient streams (the .dat files of
 * src/ActuatorPatchImpl.f90:226-458): raw native doubles, one patch's points
 * per entry, entries in file order. The entries are read from / written to
 * entries[e * stride + offset + 0 .. points_per_entry - 1]. */
int mgd_write_patch_stream(const char* filename, const double* entries, long long n_entries,
                           long long points_per_entry, long long stride, long long offset);
int mgd_read_patch_stream(const char* filename, double* entries, long long n_entries, long long points_per_entry,
                          long long stride, long long offset);

/* State%saveData for one field (MGD_FIELD_CONSERVED or MGD_FIELD_ADJOINT) of
 * every block as a PLOT3D solution file (src/StateImpl.f90:340-380): the
 * device-to-host copy is ordered on the context stream and the file is
 * written by a host thread while later work runs; mgd_wait_io joins it. */
int mgd_save_solution(mgd_ctx* ctx, const char* filename, int field, int timestep, double time);
int mgd_wait_io(mgd_ctx* ctx);
/* Region%loadData of one field from a PLOT3D solution file; *time receives
 * the file's time. */
int mgd_load_solution(mgd_ctx* ctx, const char* filename, int field, double* time);
/* The grid of every block as a PLOT3D grid file. */
int mgd_save_grid(mgd_ctx* ctx, const char* filename);
/* <prefix>.gradient_<patch>.dat for every actuator patch, from the gradient
 * of the last adjoint run; <prefix>.control_forcing_<patch>.dat read into
 * the control forcing (src/ActuatorPatchImpl.f90:226-458). */
int mgd_save_gradient(mgd_ctx* ctx, const char* prefix, long long n_entries);
int mgd_load_control_forcing(mgd_ctx* ctx, const char* prefix, long long n_entries);
/* ZAXPY on the device (bin/ZAXPY.f90, ControlSpaceAdvancer): control
 * forcing = a * gradient (+ the current forcing when accumulate != 0), over
 * the 4 * n_steps entries of the last run, with no host round trip. */
int mgd_control_zaxpy(mgd_ctx* ctx, double a, int accumulate);

/* Measurement hook (no reference counterpart): times each kernel of one RK
 * stage separately with CUDA events on the context stream, reps launches
 * back to back without programmatic dependent launch, and writes the mean
 * milliseconds per launch. Forward (MGD_FORWARD) gives 5 durations
 * [gradient/flux, dissipation, divergence+RK, primitives, functional],
 * adjoint 6 [core, dissipation, diffusion, assembly+RK,
 * gradient/sensitivity, wall and far-field SAT vectors]; *n_kernels is the
 * count, avg_ms must hold 6. Needs a preceding mgd_run_forward; leaves the
 * state changed. */
int mgd_profile_stage_kernels(mgd_ctx* ctx, int mode, int reps, double* avg_ms, int* n_kernels);

/* Self-test (no reference counterpart): evaluates x[i]^e on the current
 * device with the library's table-driven power function (fast) and with
 * CUDA's pow (ref), for checking the viscosity law's error bound. */
int mgd_selftest_pow(const double* x, int n, double e, double* fast, double* ref);

/* Self-test of the bounded wait of the persistent batched kernel (no
 * reference counterpart), used as a grid barrier: a cooperative launch of
 * n_blocks CTAs meets `rounds` times at a barrier that expects `expected`
 * arrivals; after each
 * meeting CTA 0 sums stamps the others wrote before it, into *checksum
 * (rounds (rounds + 1) / 2 * n_blocks (n_blocks + 1) / 2 when every round
 * completes). A wait gives up after `limit` polls of about 100 ns: with
 * expected > n_blocks no round completes and *status = 1 (0 otherwise);
 * the kernel then returns and the context stays usable. */
int mgd_selftest_grid_barrier(int n_blocks, int expected, int rounds, long long limit, int* status,
                              long long* checksum);

/* FP64 throughput probe (no reference counterpart): one CTA of
 * warps_per_sm (1..32) warps on every SM of the current device, each thread
 * running four independent DFMA chains; *lane_ops_per_clock receives the
 * DFMA lane-operations per clock per SM at the device's maximum clock. On
 * GB300 it rises by about 0.49 per warp up to 4 warps and stays near 1.97
 * beyond: each of the 4 sub-partitions has its own FP64 pipe, which a
 * warp-wide DFMA holds for about 64 cycles. */
int mgd_selftest_fp64_rate(int warps_per_sm, double* lane_ops_per_clock);

/* Forward RHS without any device allocation (no counterpart in the
 * reference). For callers that must not allocate device memory when they
 * evaluate an RHS -- a host that reserved its device-memory budget up front
 * with its own pool, or a loop that cannot take cudaMalloc's implicit device
 * synchronisation. q (N, nU) and rhs (N, nU) are the caller's device
 * buffers; time is state%time. Grid and patch data come from the context,
 * which must have been finalized; all intermediates live in one fixed
 * 16 MiB array in device memory that every GPU loading the library holds
 * until exit, so blocks above about 100k points (2D) / 55k points (3D) are
 * rejected with an error. The first call on a device looks up that array's
 * device address, so make it before any stream capture. Calls share the
 * array: calls that overlap on the GPU (from different contexts or host
 * threads) race and must be serialised by the caller. Like mgd_compute_rhs
 * it adds the actuators' forcing set by mgd_set_patch_control_forcing when
 * the controller is on, and it refuses regions of several blocks and blocks
 * with block-interface patches. Ordering: the kernels run on the context's
 * own stream, which does not wait for the caller's streams, so q must be
 * complete on the device when the call is made (synchronise the stream that
 * wrote it); rhs is complete when the call returns. The call also uses the
 * context's launch counters and per-call step counters, so it must not
 * overlap any other call on the same context; it leaves the context's
 * state, run checkpoints and gradient untouched. */
int mgd_forward_rhs_noalloc(mgd_ctx* ctx, const double* q, double time, double* rhs);

/* CUDA stream the context launches on (cudaStream_t as void*). */
void* mgd_stream(mgd_ctx* ctx);

/* Counts kernel launches made by the context since the last reset. */
long long mgd_kernel_launches(mgd_ctx* ctx, int reset);

/* Measurement and test hook (no reference counterpart): the form of the
 * gradient/flux kernel of 2D blocks that the setup's autotuner chose, one
 * thread per point (1) or two adjacent threads per point, one per axis (2).
 * lanes = 1 or 2 sets that form for every block of the context from the next
 * launch on; lanes = 0 only reports it. Returns the form in effect (3D blocks
 * always use 1), or -1 for other values of lanes. */
int mgd_gradient_lanes(mgd_ctx* ctx, int lanes);

/* Measurement and test hook (no reference counterpart): the form of the
 * adjoint core of 2D blocks, one thread per point (1) or one per point and
 * axis (2, the axes' shares summed in shared memory). Only mgd_tune_run
 * chooses the second form. lanes = 1 or 2 sets it for every block of the
 * context, 0 only reports it; returns the form in effect (3D: 1), or -1. */
int mgd_adjoint_core_lanes(mgd_ctx* ctx, int lanes);

/* Measurement and test hook (no reference counterpart): the form of the
 * composite dissipation of 3D blocks that are PLANE-periodic along all axes
 * (and whose sizes are multiples of 32 x 8 x 16): operands staged in shared
 * memory by the tensor memory accelerator (1) or read through the L1 cache
 * (0, the default: the kernel is FP64-bound and measured faster that way).
 * mode = 0 or 1 sets it, -1 only reports it; returns the setting in effect,
 * or -1. Both forms give the same results to rounding. */
int mgd_dissipation_tma(mgd_ctx* ctx, int mode);

/* Run-level autotuner (no reference counterpart): chooses the thread-block
 * tiles of the six stage kernels (and the 2D gradient/flux form) by timing
 * whole checkpointed runs, mgd_run_forward(n_steps, save_interval) followed
 * by mgd_run_adjoint when with_adjoint != 0, from the context's current state:
 * coordinate descent over the kernels, two passes, fastest of two runs per
 * candidate. Inside a run the stage kernels share the SMs with the side-stream
 * dissipation and the concurrent checkpoint recomputation, so the tiles that
 * finish a run first differ from those of the setup's per-kernel timings.
 * Every block gets the same tiles. The state and adjoint fields are restored
 * afterwards, the chosen tiles also go to later contexts of the process with
 * the same grid and physics, and *best_ms (may be NULL) receives the tuned
 * run's wall time. Call it before the runs: it discards the last run's
 * trajectory (a following mgd_run_adjoint needs a new mgd_run_forward). */
int mgd_tune_run(mgd_ctx* ctx, int n_steps, int save_interval, int with_adjoint, double* best_ms);

/* Measurement and test hook (no reference counterpart): the thread-block
 * tile (points per CTA along each axis) of one stage kernel, 0 gradient/flux,
 * 1 dissipation, 2 divergence + RK update, 3 adjoint core, 4 adjoint
 * diffusion, 5 adjoint assembly + RK update. set != 0 gives every block of
 * the context that tile from the next launch on (tile[0..2] >= 1 with a
 * product of at most 256); set = 0 writes the current tile to tile[0..2]. */
int mgd_stage_tile(mgd_ctx* ctx, int kernel, int* tile, int set);

#ifdef __cplusplus
}
#endif

#endif /* MAGUDI_GB300_H */
