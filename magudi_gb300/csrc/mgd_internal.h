// mgd_internal.h -- device-resident region state of one context and the
// launchers of the kernels in mgd_kernels.cu.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <thread>
#include <vector>

#include "../../include/magudi_gb300.h"
#include "mgd_device.cuh"

namespace mgd {

// Component offsets inside the primitive-variable array `prim` (N x nPrim):
// v = 1/rho, u_1..u_nD, p, T, mu, lambda (second coefficient), k.
struct PrimLayout {
  int nD;
  __host__ __device__ int v() const { return 0; }
  __host__ __device__ int u(int d) const { return 1 + d; }
  __host__ __device__ int p() const { return 1 + nD; }
  __host__ __device__ int T() const { return 2 + nD; }
  __host__ __device__ int mu() const { return 3 + nD; }
  __host__ __device__ int la() const { return 4 + nD; }
  __host__ __device__ int k() const { return 5 + nD; }
  __host__ __device__ int count() const { return 6 + nD; }
};

// Boundary SAT entry: one (far-field or wall patch, point) pair.
enum { SAT_FAR_FIELD = 0, SAT_WALL = 1, SAT_ISOTHERMAL_WALL = 2, SAT_INTERFACE = 3 };
struct FarFieldEntries {
  int n = 0;
  int* point = nullptr;      // grid point
  int* normalDir = nullptr;  // 1-based normal direction (unsigned)
  int* kind = nullptr;       // SAT_FAR_FIELD, SAT_WALL (slip or adiabatic), SAT_ISOTHERMAL_WALL
  double* wallInv = nullptr;   // walls: signed inviscid penalty / H0 * jacobian
  double* wallVisc = nullptr;  // isothermal walls: viscous penalty / H0 / Re * jacobian (0 if inviscid)
  double* wallT = nullptr;     // isothermal walls: wall temperature
  // block interfaces (kind SAT_INTERFACE)
  int* partnerBlock = nullptr;   // 0-based block of the conforming point
  int* partnerPoint = nullptr;   // its grid point
  int* partnerEntry = nullptr;   // its SAT entry
  int* dirL = nullptr;           // signed normal direction of this side
  int* dirR = nullptr;           // and of the partner
  double* metricsR = nullptr;    // nD: the partner's normal metric row
  double* ifInv = nullptr;       // 2: inviscid penalty of this side and of the partner (signed, / H0)
  double* ifVis = nullptr;       // 2: viscous penalty of this side and of the partner (signed, / H0)
  double* ifVisc = nullptr;      // nU: sum_j F_v(:, j) m_L,j of this side (component 0 zero)
  double* ifAd = nullptr;        // nD x (nU-1): interface terms of the adjoint viscous diffusion
  int* ifList = nullptr;         // the block's interface entries, ascending
  double* M = nullptr;       // nU*nU: inviscidPenaltyAmount * jacobian * A+(target), column-major
  double* sigV = nullptr;    // viscousPenaltyAmount * jacobian
  double* sigVRaw = nullptr; // viscousPenaltyAmount
  double* visc = nullptr;    // nU: SAT vector of the entry at the current stage (forward or adjoint)
  double* viscT = nullptr;   // nU: the same for the target state
};

// Plain-old-data view of a block that kernels receive by value.
struct BlockView {
  int nD, nU;
  long long N;
  int gs[3];
  Axis ax[3];
  int curvilinear;
  // grid
  const double* metrics;
  const double* jac;
  const double* arcA;   // nD components: -dissipationAmount * arcLength_i
  const int* iblank;
  // state
  double* q;
  double* lam;
  const double* qt;
  double* rhs;
  double* b1;
  double* b2;
  double* prim;
  double* tau;
  double* hf;
  double* fhat;   // nD x nU
  double* dq;     // nD x nU (composite dissipation: nU, already scaled)
  double* rcore;  // nU
  double* ad;     // nD x (nU-1)
  double* t2;     // nU-1: divergence of the adjoint viscous diffusion
  double* adjF;   // nU: stored cost-target adjoint forcing (per-call API path)
  // patches
  const double* sponge;   // summed sponge strength
  const double* mc;       // control mollifier (normalized)
  const double* mt;       // target mollifier (normalized)
  const double* meanP;
  const double* wT;       // cost-target quadrature weight: mask * norm
  const double* wA;       // actuator quadrature weight: mask * norm
  const double* tgtCount; // number of cost-target patches holding the point (0 if hole)
  const int* actIdx;      // actuator-patch point index, -1 if none
  const int* ffOfPoint;   // 3 far-field entry indices per point, -1 if none
  const double* srcG;     // nSources x N: exp(-gaussianFactor r^2), 0 on holes
  int nSources;
  const int* tgtPts;      // points with a cost-target quadrature weight
  int nTgt;
  const int* actPts;      // grid point of each actuator-patch point, patch order
  int nAct;
  FarFieldEntries ff;
  // solenoidal excitation: entry of each point (null when the block has none)
  // and 3 values per entry for the current stage, written by kExcitation:
  // forward (f_x, f_y, u . f), adjoint (its terms for components 0, 1, 2)
  const int* excIdx;
  double* excF;
};

// Arrays of every block of a context that the block-interface kernels read
// across blocks.
struct BlockRefs {
  const double* q[MGD_MAX_BLOCKS];
  const double* lam[MGD_MAX_BLOCKS];
  const double* ifVisc[MGD_MAX_BLOCKS];
  long long N[MGD_MAX_BLOCKS];
  const double* stage[MGD_MAX_BLOCKS];  // stage buffers of a run (slots of all blocks share counters)
  long long slotStride[MGD_MAX_BLOCKS];
};

// Thread-block tiling of a block's points: blocks of t[0] x t[1] x t[2]
// threads cover n[0] x n[1] x n[2] tiles of the grid.
// Thread-block tiling of a block's grid: t[] points per CTA along each axis,
// n[] CTAs along each axis. div[] holds the divisors t[0], t[0] t[1], n[0],
// n[0] n[1] of the kernels' index decomposition with their reciprocals
// rcp[] = floor(2^64 / d) + 1 (0 for d = 1), so that a kernel divides by
// multiply-high instead of an integer division sequence.
struct Tile {
  int t[3];
  int n[3];
  unsigned div[4];
  unsigned long long rcp[4];
  __host__ __device__ int threads() const { return t[0] * t[1] * t[2]; }
  __host__ __device__ int blocks() const { return n[0] * n[1] * n[2]; }
};

// Constants of the physics and of the run.
struct Physics {
  double g, gm1, gOverGm1, reInv, prInv, powerLawExponent, laFactor;
  // 1/(g-1), (g-2)/(g-1) and 1/g, so that the adjoint core multiplies
  // instead of dividing per point
  double invGm1, gm2OverGm1, invG;
  double dissipationAmount;
  int viscous, dissipation, composite;
  int powerLaw;  // powerLawExponent > 0: mu follows the power law of T
};

struct RunScalars {
  // device pointers read by the kernels of a captured step
  const int* step;        // 1-based forward step of the current RK step
  const int* segBase;     // first step of the checkpoint segment minus 1
  const double* amp;      // source amplitudes per (step-1)*4 + stage-1, nSources each
  const double* forcing;  // control forcing entries, P each (file order)
  const double* apiForcing;  // per-call path: the actuator patches' current forcing (P values), or null
  long long nForcingEntries;
  int nSteps;
  long long P;            // actuator-patch points
  double* gradient;       // gradient entries, P each (file order)
  double* partials;       // block partial sums per stage slot
  int nPartialBlocks;
  double* stageBuf;       // stage inputs of the current segment (4*S slots)
  long long slotStride;   // doubles per stage slot
  int slotFull;           // slots hold q, primitives, stress and heat flux (else q only)
  double dt, h6, h3, h2;   // step size and dt/6, dt/3, dt/2 when rk is null
  const double* rk;        // per step (indexed by step - 1): dt, dt/6, dt/3, dt/2; or null
  int adjointForcingSwitch;
  const double* stageTime; // time of each forward stage, (step-1)*4 + stage-1
  // solution limits of a forward run (null when off): the key of the first
  // violation, all ones while there is none; the RK update kernels leave the
  // state unchanged once it is set, so the run ends on the violating state
  const unsigned long long* limitKey;
};

// Open ranges of checkSolutionLimits (src/SolverImpl.f90:189-304).
struct SolutionLimits {
  double rhoMin, rhoMax, TMin, TMax;
};
// Key of a solution-limit violation: the earliest forward stage first, then
// the block, density before temperature, the lowest grid point.
__host__ __device__ inline unsigned long long limitKeyOf(long long ordinal, int block, int quantity, long long p) {
  return ((unsigned long long)ordinal << 36) | ((unsigned long long)block << 33) |
         ((unsigned long long)quantity << 32) | (unsigned long long)p;
}
constexpr unsigned long long kNoLimitViolation = ~0ULL;

// RK4 coefficients of the current step of a run (or of the per-call step).
struct RkCoeffs {
  double dt, h6, h3, h2;
};
__device__ __forceinline__ RkCoeffs rkCoeffs(const RunScalars& rs) {
  if (!rs.rk) return {rs.dt, rs.h6, rs.h3, rs.h2};
  const double* k = rs.rk + 4LL * (*rs.step - 1);
  return {k[0], k[1], k[2], k[3]};
}
inline void setStepSize(RunScalars& rs, double dt) {
  rs.dt = dt;
  rs.h6 = dt / 6.0;
  rs.h3 = dt / 3.0;
  rs.h2 = dt / 2.0;
}

// One solenoidal-excitation patch of a block: its entries (non-hole patch
// points, entry index off..off+nE-1 of the block) with the time-invariant
// part of the forcing (setupSolenoidalExcitationPatch,
// src/SolenoidalExcitationPatchImpl.f90:93-130): strength, offsets from the
// origin and the spatial functions sin/cos(w (x - x0) + phi_1),
// sin/cos(w (y - y0) + phi_2) of every mode (entry fastest).
struct ExcPatch {
  int nE = 0, off = 0, nModes = 0;
  double g = 0, speed[2] = {0, 0};
  const double* omega = nullptr;  // nModes
  const double* S = nullptr;      // nE
  const double* dx = nullptr;     // nE
  const double* dy = nullptr;     // nE
  const double* cache = nullptr;  // 4 * nModes * nE
  const int* point = nullptr;     // grid point of each entry
};

struct DevBlock {
  mgd_block_desc desc;
  BlockView v;
  std::vector<ExcPatch> exc;
  // tile shapes of the stage kernels, chosen by the autotuner
  Tile tGrad{}, tDiss{}, tRhs{}, tAdjA{}, tAdjD{}, tAdjB{};
  int gradLanes = 1;  // 2D: kGradFlux with one lane per point (1) or two, one per direction (2)
  int coreLanes = 1;  // 2D: kAdjointCore (1) or kAdjointCoreSplit, one thread per point and direction (2)
  std::vector<void*> allocations;
  int nStagePartialBlocks = 0;
  int nInterfaceEntries = 0;
  // buffers of multi-block checkpointed runs
  double* runSnap = nullptr;
  long long runSnapCap = 0;
  double* runStage = nullptr;
  long long runStageCap = 0;
  double* runPartials = nullptr;
  long long runPartialCap = 0;
  std::vector<double> hostIfaceInv, hostIfaceVis;  // own interface penalties per SAT entry
  std::vector<int> hostFfPoint, hostFfSigned;
  // host copies kept for setup
  std::vector<double> hostCoords;
  std::vector<int> hostIblank;
  std::vector<double> hostNorm;        // H * det
  std::vector<double> hostMetricsArc;  // arc lengths of the metrics per direction
  std::vector<double> hostJmi;         // coordinate derivatives d x_c / d xi_d (unmasked)
  // ffOfPoint etc. are built on the host at finalize
};

// A main stream, a side stream for the concurrent branch of a stage, and the
// fork/join events between them.
struct Lanes {
  cudaStream_t main, side;
  cudaEvent_t fork, join;
};

struct Context {
  mgd_options opts;
  Physics phys;
  int nD = 2, nU = 4;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;          // second stream for concurrent graph branches
  cudaEvent_t evFork[8] = {}, evJoin[8] = {};
  // one stream per block of a region (created at the first region run), on
  // which the blocks' stage kernels run concurrently between fork and join
  cudaStream_t blockStreams[MGD_MAX_BLOCKS] = {};
  cudaEvent_t evBlockFork = nullptr, evBlockJoin[MGD_MAX_BLOCKS] = {};
  // the second set, for the recomputation lane of a region's adjoint run
  cudaStream_t blockStreams2[MGD_MAX_BLOCKS] = {};
  cudaEvent_t evBlockFork2 = nullptr, evBlockJoin2[MGD_MAX_BLOCKS] = {};
  // the recomputation lane's own forward work arrays of every block of a
  // region (state, primitives, fluxes, dissipation, RK buffers, SAT vectors,
  // interface fluxes, excitation values)
  std::vector<BlockView> regionShadow;
  // lanes of the checkpoint recomputation, which runs beside the adjoint
  cudaStream_t stream2 = nullptr, side2 = nullptr;
  cudaEvent_t evRecDone[2] = {}, evAdjDone[2] = {};
  int device = 0;
  std::string error;
  std::vector<DevBlock> blocks;
  std::vector<mgd_patch_desc> patches;
  std::vector<std::vector<double>> patchOmega, patchPhases;  // solenoidal-excitation modes per patch
  std::vector<mgd_acoustic_source> sources;
  bool finalized = false;
  bool hasInterfaces = false;
  bool adjointNonzeroIC = false;   // adjoint_nonzero_initial_condition
  std::vector<std::vector<int>> ifacePointEntry;  // per patch: SAT entry of each interface patch point
  long long launches = 0;
  long long actuatorPoints = 0;
  // device scalars: [0] step, [1] segBase, [2] api step (always 1), [3] api segBase,
  // [4] step and [5] segBase of the checkpoint recomputation
  int* dCounters = nullptr;
  double* dApiAmp = nullptr;
  double* dApiTime = nullptr;       // stage time of the per-call path
  double* dStageTime = nullptr;     // time of every forward stage of the run
  long long stageTimeCapacity = 0;
  double* dAmp = nullptr;           // per-stage source amplitudes of the run
  long long ampCapacity = 0;
  double* dForcing = nullptr;       // control forcing entries
  double* dDeltaForcing = nullptr;  // control perturbation of a tangent run
  double* dApiForcing = nullptr;    // actuator forcing of the per-call RHS (P values), set or not
  bool apiForcingSet = false;
  long long deltaForcingCapacity = 0;
  long long nForcingEntries = 0;
  long long forcingCapacity = 0;
  std::vector<double> actuatorWeights;  // quadrature weight of each actuator-patch point
  double* dGradient = nullptr;      // gradient entries
  long long gradientCapacity = 0;
  double* dPartials = nullptr;      // stage partial sums
  long long partialCapacity = 0;
  double* dStageValues = nullptr;   // per-stage reduced values
  long long stageValueCapacity = 0;
  // checkpoints of the last forward run
  int runSteps = 0, saveInterval = 0;
  double runT0 = 0.0;
  std::vector<double> stageTimes;   // time of every forward stage of the run
  double* dSnapshots = nullptr;     // (nSnap) x nU x N per block (single block supported)
  long long snapshotCapacity = 0;
  double* dStageBuf = nullptr;       // two halves of 4*S slots (ping-pong between segments)
  long long stageBufCapacity = 0;
  long long stageHalf = 0;          // doubles per half
  int stageHalves = 1;
  // forward work arrays of the recomputation (q, prim, fhat, dq, b1, b2, SAT vectors)
  std::vector<void*> shadowAllocations;
  BlockView shadow{};
  bool shadowReady = false;
  long long slotStride = 0;         // doubles per stage slot of dStageBuf
  int slotFull = 0;                 // slots also hold primitives, stress and heat flux
  // Resident trajectory: the forward run stores every stage's slot (4 T full
  // slots in dStageBuf) when enabled and within the byte budget (<= 0: half
  // the free device memory); trajectorySteps = T while those slots are intact
  int trajectoryStorage = 0;
  double trajectoryMaxBytes = 0.0;
  int trajectorySteps = 0;
  // RK4 coefficients per step of the last run (dt, dt/6, dt/3, dt/2), their
  // step sizes on the host, constant-CFL reduction scratch and run time
  double* dStepDt = nullptr;
  long long stepDtCapacity = 0;
  std::vector<double> stepDt;
  double* dDtPartials = nullptr;
  long long dtPartialCapacity = 0;
  double* dTime = nullptr;
  double* dNorm = nullptr;          // H det per point (terminal functional)
  // solution limits: device key of the first violation of the current run,
  // and whether the last forward run stopped at one
  unsigned long long* dLimitKey = nullptr;
  // composite dissipation of fully periodic 3D blocks staged by the tensor
  // memory accelerator (off by default: the FP64-bound kernel measured 2%
  // slower staged than through L1); its kernel's error word (a bounded wait
  // ran out) and whether such a kernel was launched since the last check
  bool useTmaDissipation = false;
  int* dKernelError = nullptr;
  bool tmaLaunched = false;
  bool limitViolated = false;
  std::string limitMessage;
  cudaGraphExec_t gForward = nullptr, gRecomputeH[2] = {}, gAdjointH[2] = {};
  // asynchronous solution files: pinned staging, copy stream, writer thread
  cudaStream_t ioStream = nullptr;
  cudaEvent_t ioCopied = nullptr;
  double* ioStaging = nullptr;
  size_t ioStagingBytes = 0;
  std::thread ioThread;
  int ioStatus = 0;
  long long nodesForward = 0, nodesRecompute = 0, nodesAdjoint = 0;
};

// One instance of a batched launch: its block, run scalars and tile shapes.
// All instances of a batch share the physics and the thread count of each
// kernel; grid sizes, tiles, states and controls differ.
struct BatchEntry {
  BlockView v;
  RunScalars rs;
  Tile tGrad, tDiss, tRhs;
  int controller;
};

// Work of the persistent batched run (one launch for all steps), three
// rounds per RK stage: round A units {kind, instance, tile, component} (kind
// 0 gradient/flux tile, 1 dissipation tile and component, 2 functional
// reduction block), round B units {instance, tile, component} (divergence and
// RK update), round C units {instance, block of kBatchThreads points}
// (primitives); counts[i] = {A, B, C units} of instance i. work = the next
// unit of the run's global order, done[i] = units of instance i completed
// (both zeroed before a launch); status = 0, or 1 when a wait ran out of its
// spin limit (the kernel then returns early and the host reports the error).
struct PersistentPlan {
  const int4* unitsA = nullptr;
  int nA = 0;
  const int4* unitsB = nullptr;
  int nB = 0;
  const int2* unitsC = nullptr;
  int nC = 0;
  const int4* counts = nullptr;
  unsigned long long* work = nullptr;
  unsigned long long* done = nullptr;
  int* status = nullptr;
  long long spinLimit = 0;
};

// Block maps of a batched launch: entry k of a map is (instance, block within
// the instance) for thread block k.
enum BatchKernel { BK_GRAD = 0, BK_DISS, BK_RHS, BK_PRIMS, BK_FUNC, BK_COUNT };
struct BatchLaunch {
  const BatchEntry* entries = nullptr;
  const int2* map[BK_COUNT] = {};
  int blocks[BK_COUNT] = {};
  int threads[BK_COUNT] = {};
};

// ----- stage orchestration (mgd_api.cu) -----
void forwardStage(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, bool api, bool controller, bool store,
                  bool functional, const Lanes* lanes = nullptr);
void adjointStage(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, int stage, double apiFactor, bool api,
                  bool fromSlot, bool record, const Lanes* lanes = nullptr);

// The per-call forward RHS adds the actuators' forcing (perCallController)
// from perCallForcing (null until the caller set a forcing); both as
// mgd_compute_rhs uses them. singleBlockRegion: one block and no
// block-interface patch.
bool perCallController(const Context& c);
const double* perCallForcing(const Context& c);
bool singleBlockRegion(const Context& c);
// Reads the solution-limit key of the last check: MGD_SOLUTION_LIMITS with
// *value = HUGE and the reference's message in c.error after a violation
// (perCall: no step and stage in the message), 0 otherwise.
int limitOutcome(Context& c, double* value, bool perCall);

int prepareForwardRun(Context& c, int n_steps, int save_interval, double t0, bool snapshots);
int finishForwardRun(Context& c, double* cost);
RunScalars runScalarsOf(Context& c);
int autotuneTile(Context& c, DevBlock& b, int kernel, const int (*cands)[3], int nCands, Tile* best);

// ----- launchers (mgd_kernels.cu) -----
// Programmatic dependent launch for the launches that follow on this thread.
void setProgrammaticLaunch(bool on);
// Launch priority for the launches that follow on this thread (on = false:
// each launch takes its stream's priority).
void setLaunchPriority(bool on, int priority);
// Every launcher takes the stream it launches on; the context stream when 0.
void uploadOperatorTables();
// Primitive variables of qSrc (or, when stage > 0, of the stage-buffer slot
// of the current step and stage); copyToQ also stores that state as q.
void launchPrims(Context& c, DevBlock& b, const double* qSrc, bool copyToQ, const RunScalars* rs = nullptr,
                 int stage = 0, cudaStream_t s = 0);
// Gradients, stress, heat flux and contravariant fluxes (flags GF_*).
void launchGradFlux(Context& c, DevBlock& b, bool writeFlux, bool writeStress, const RunScalars* rs, int stage,
                    bool storeStage, cudaStream_t s = 0);
// checkSolutionLimits of block b's current state (q and its primitives) at
// the start of RK stage `stage` of the step *step (ordinal 0 when step is
// null): atomically lowers *key to the key of the first violating point.
void launchSolutionLimits(Context& c, DevBlock& b, int blockIndex, const int* step, int stage,
                          unsigned long long* key, cudaStream_t s = 0);
// Artificial dissipation of src (q forward, lambda adjoint) into b.v.dq,
// scaled by sign (+1 forward, -1 adjoint).
void launchDissipation(Context& c, DevBlock& b, const double* src, double sign, cudaStream_t s = 0);
// Flux divergence, dissipation, 1/det, SATs, sources, then the RK4 forward
// update of rkStage (or, for rkStage = 0, the RHS into b.v.rhs).
void launchForwardDivergence(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, bool api, bool controller,
                             cudaStream_t s = 0);
// Linearized RHS (rkStage 0, into b.v.rhs) or one linearized RK stage of the
// perturbation in b.v.lam about a forward state: the block's current state
// (primitives, stress and heat flux current), or with fromSlot the full stage
// slot of (step, stage) of a run; the dissipation of lambda already in
// b.v.dq. factor scales the stored cost-target adjoint forcing as the
// reference's LINEARIZED mode adds it.
void launchLinearized(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, double factor, int stage = 1,
                      bool fromSlot = false, bool controller = false, cudaStream_t s = 0);
// The two halves of launchLinearized for multi-block regions, whose interface
// SATs (launchInterfaceSatLinearized) go between them.
void launchLinearizedFlux(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot, cudaStream_t s = 0);
void launchLinearizedDivergence(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, double factor, int stage,
                                bool controller, cudaStream_t s = 0);
void launchInterfaceSatLinearized(Context& c, DevBlock& b, const BlockRefs& r, const RunScalars* rs = nullptr,
                                  int stage = 1, bool fromSlot = false, cudaStream_t s = 0);
// Tangent of the functional at the forward state of (step, stage) along lambda,
// into the partial sums of the stage before.
void launchFunctionalTangent(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot,
                             cudaStream_t s = 0);
// Functional partial sums of the state just produced (stage slot of step/stage).
void launchFunctional(Context& c, DevBlock& b, const RunScalars& rs, int stage, cudaStream_t s = 0);
// Adjoint: inviscid/viscous Jacobian-transpose products and viscous diffusion.
void launchAdjointCore(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot, cudaStream_t s = 0);
// Solenoidal-excitation values of the stage into b.v.excF (forward: the
// forcing and u . f of the current state; adjoint: the transpose terms of the
// forward state of the stage, with lambda before the stage update).
void launchExcitation(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool adjoint, bool fromSlot,
                      cudaStream_t s = 0);
// Adjoint: divergence of the viscous diffusion (per component).
// The adjoint SAT vectors of the block's wall and far-field entries; they
// run beside the adjoint core and must complete before the assembly.
void launchAdjointSatVectors(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot,
                             cudaStream_t s = 0);
void launchAdjointDiffusion(Context& c, DevBlock& b, cudaStream_t s = 0);
// Adjoint: final assembly, SATs, cost-target forcing and the RK4 adjoint update.
void launchAdjointAssemble(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, int stage, double apiFactor,
                           bool api, bool fromSlot, cudaStream_t s = 0);
// Gradient entry and sensitivity partial sums of the adjoint state at a stage.
void launchGradientSensitivity(Context& c, DevBlock& b, const RunScalars& rs, int stage, cudaStream_t s = 0);
void launchAdjointInitial(Context& c, DevBlock& b, double factor);
// Functional%updateAdjointForcing for the per-call API: stores the forcing of
// the current state (or zeros) in adjF.
void launchStoreAdjointForcing(Context& c, DevBlock& b, bool zero);
void launchSnapshot(Context& c, DevBlock& b, double* snapshots, int saveInterval, bool initial, cudaStream_t s = 0);
void launchStepAdvance(Context& c, int delta, cudaStream_t s = 0);
void launchReducePartials(Context& c, const double* partials, int stride, int count, int nSlots, double* out);
// Constant-CFL step size of the current primitives: with step == null writes
// the step size to dtOut[0]; otherwise writes dt, dt/6, dt/3, dt/2 to
// dtOut[4 (*step - 1) + 0..3], advances *time over the step's four stages and
// stores the stages' source amplitudes in amp.
void launchTimeStep(Context& c, DevBlock& b, double* partials, double* dtOut, const int* step, double* time,
                    double* stageTime, double* amp, cudaStream_t s = 0);
int timeStepBlocks(const DevBlock& b);
void launchTimeStepRegion(Context& c, double* partials, double* dtOut, const int* step, double* time,
                          double* stageTime, double* amp, cudaStream_t s = 0);
void launchAxpy(Context& c, double* z, const double* x, double a, long long n, bool accumulate);
// Block-interface SAT vectors of block b's interface entries (forward; adjoint
// with the interface terms of the adjoint viscous diffusion).
void launchInterfaceSat(Context& c, DevBlock& b, const BlockRefs& r, cudaStream_t s = 0);
void launchInterfaceSatAdjoint(Context& c, DevBlock& b, const BlockRefs& r, const RunScalars* rs = nullptr,
                               int stage = 1, bool fromSlot = false, cudaStream_t s = 0);
// Terminal kinetic energy of the current state into out[0] (norm = H det per point).
void launchKineticEnergy(Context& c, DevBlock& b, const double* norm, double* partials, double* out);
void launchKineticEnergyAdjointInitial(Context& c, DevBlock& b);
void launchCoordinateDerivative(Context& c, DevBlock& b, int dir, double* out);
void launchApplyD1(Context& c, DevBlock& b, int dir, const double* in, double* out, int ncomp);
void launchFarFieldMatricesWith(Context& c, DevBlock& b, const double* sigInv, const int* signedNormal);
void launchFarFieldTargetVisc(Context& c, DevBlock& b);
// Batched forward stage over all instances of a batch (same kernels as
// forwardStage, one launch per kernel for the whole batch).
void launchBatchGradFlux(Context& c, const BatchLaunch& L, int stage, cudaStream_t s);
void launchBatchDissipation(Context& c, const BatchLaunch& L, cudaStream_t s);
void launchBatchForwardDivergence(Context& c, const BatchLaunch& L, int rkStage, cudaStream_t s);
void launchBatchPrims(Context& c, const BatchLaunch& L, cudaStream_t s);
void launchBatchFunctional(Context& c, const BatchLaunch& L, int stage, cudaStream_t s);
void launchStepAdvanceOn(int* counters, int delta, cudaStream_t s);
// The whole batched forward run (n_steps RK4 steps of every instance) as one
// cooperative launch of a persistent kernel with grid barriers between the
// stage phases, on stream s; `grid` CTAs (at most the co-resident number,
// persistentGridSize). Returns the launch status.
cudaError_t launchBatchPersistent(Context& c, const BatchEntry* entries, const PersistentPlan& plan, int nSteps,
                                  int functional, int grid, cudaStream_t s);
int persistentGridSize(const Context& c);
// Grid-barrier self-test (see mgd_selftest_grid_barrier); 0 or a CUDA error.
int selftestFp64Rate(int warpsPerSm, double* laneOpsPerClock);
int selftestGridBarrier(int nBlocks, unsigned int expected, int rounds, long long limit, int* status,
                        long long* sum);
void launchSetCounters(int* counters, int step, int segBase, cudaStream_t s);
constexpr int kBatchThreads = 128;
// Grids of up to this many points (all blocks of a region) recompute the
// checkpoint segments on a second lane beside the adjoint; larger grids fill
// the GPU with either lane alone and recompute each segment in line.
#ifndef MGD_TWO_LANE_MAX_POINTS
#define MGD_TWO_LANE_MAX_POINTS (1LL << 21)
#endif
// Resident CTAs per SM that the persistent batched kernel is compiled for,
// 2D and 3D (its register budget is 65536 / (128 x this)). One kernel holds
// the register budget of its largest phase (the gradient/flux tiles) in
// every phase; at 64 2D monopole instances 12 CTAs per SM (40 registers, the
// flux phase spilling to L1) ran faster than 6, 8, 10 or 16. The 3D flux
// tiles need about twice the registers.
#ifndef MGD_PERSISTENT_MIN_BLOCKS
#define MGD_PERSISTENT_MIN_BLOCKS 12
#endif
#ifndef MGD_PERSISTENT_MIN_BLOCKS_3D
#define MGD_PERSISTENT_MIN_BLOCKS_3D 6
#endif
constexpr int persistentMinBlocks(int nD) { return nD == 2 ? MGD_PERSISTENT_MIN_BLOCKS : MGD_PERSISTENT_MIN_BLOCKS_3D; }
// Consecutive units the persistent batched kernel's CTAs draw at a time
// (2: fewer draws and acquires than 1, a shorter tail than 4 or 8).
#ifndef MGD_PERSISTENT_CHUNK
#define MGD_PERSISTENT_CHUNK 2
#endif
constexpr int kMaxExcitationModes = 256;  // modes of one solenoidal-excitation patch

// Blocks of the fixed-layout reductions (functional, sensitivity).
int reductionBlocks(const DevBlock& b);
void launchPowSelfTest(const double* x, int n, double e, double* fast, double* ref);
Tile makeTile(const DevBlock& b, int tx, int ty, int tz);

}  // namespace mgd

// The opaque handle of the C ABI.
struct mgd_ctx {
  mgd::Context c;
};
