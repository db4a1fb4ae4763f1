// mgd_batch.cu -- batched forward runs: many independent regions (contexts)
// of possibly different grid sizes advance together, each stage kernel
// launched once for the whole batch (block maps route every thread block to
// its instance), one CUDA graph per RK4 step replayed n_steps times.
//
// The reference runs its gradient-accuracy sweep as one ./forward process per
// control amplitude after ./zaxpy (README.md:118-165, bin/ZAXPY.f90); a batch
// runs all amplitudes (or any ensemble of controls and grids) in one go.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "mgd_internal.h"

using namespace mgd;

struct mgd_batch {
  std::vector<mgd_ctx*> inst;
  std::string error;
  int device = 0;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  BatchEntry* dEntries = nullptr;
  int2* dMap[BK_COUNT] = {};
  BatchLaunch L;
  std::vector<std::array<Tile, 3>> tiles;  // per instance: grad, diss, rhs
  int* dCounters = nullptr;
  cudaGraphExec_t graph = nullptr;
  long long nodes = 0, launches = 0;
  // persistent run: one cooperative launch of all steps (default), captured
  // in a graph per step count
  bool persistent = true;
  int4* dUnitsA = nullptr;
  int4* dUnitsB = nullptr;
  int4* dCounts = nullptr;              // per instance {round A, B, C units}
  unsigned long long* dQueue = nullptr;  // {next unit, done[instance]...}
  int* dStatus = nullptr;
  PersistentPlan plan;
  int persistentGrid = 0;
  cudaGraphExec_t graphP = nullptr;
  int graphPSteps = 0;
  bool graphPCaptured = false;
};

static int bfail(mgd_batch* b, const std::string& m) {
  b->error = m;
  return 1;
}

#define BATCH_TRY(b, call)                                                          \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) return bfail(b, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static std::string g_batchCreateError;

// Options that must agree across the instances of a batch (everything but the
// grids, patches, states and controls).
static bool sameOptions(const mgd_options& a, const mgd_options& b) {
  return a.n_dimensions == b.n_dimensions && a.viscous == b.viscous && a.dissipation == b.dissipation &&
         a.composite_dissipation == b.composite_dissipation && a.curvilinear == b.curvilinear &&
         a.use_constant_cfl == b.use_constant_cfl && a.enable_functional == b.enable_functional &&
         a.ratio_of_specific_heats == b.ratio_of_specific_heats && a.reynolds_number == b.reynolds_number &&
         a.prandtl_number == b.prandtl_number && a.viscosity_power_law_exponent == b.viscosity_power_law_exponent &&
         a.bulk_viscosity_ratio == b.bulk_viscosity_ratio && a.dissipation_amount == b.dissipation_amount &&
         a.time_step_size == b.time_step_size;
}

static void destroyBatch(mgd_batch* b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graphP) cudaGraphExecDestroy(b->graphP);
  cudaFree(b->dUnitsA);
  cudaFree(b->dUnitsB);
  cudaFree(b->dCounts);
  cudaFree(b->dQueue);
  cudaFree(b->dStatus);
  cudaFree(b->dEntries);
  for (int k = 0; k < BK_COUNT; ++k) cudaFree(b->dMap[k]);
  cudaFree(b->dCounters);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char* mgd_batch_last_error(const mgd_batch* batch) {
  return batch ? batch->error.c_str() : g_batchCreateError.c_str();
}

int mgd_batch_create(mgd_ctx* const* instances, int n_instances, mgd_batch** out) {
  *out = nullptr;
  if (!instances || n_instances < 1) {
    g_batchCreateError = "a batch needs at least one instance";
    return 1;
  }
  for (int i = 0; i < n_instances; ++i) {
    if (!instances[i] || !instances[i]->c.finalized || instances[i]->c.blocks.size() != 1) {
      g_batchCreateError = "every instance must be a finalized single-block context";
      return 1;
    }
    const Context& c = instances[i]->c;
    if (!sameOptions(c.opts, instances[0]->c.opts) || c.device != instances[0]->c.device) {
      g_batchCreateError = "instances of a batch must share their options (except the grids) and the device";
      return 1;
    }
    if (c.opts.use_constant_cfl) {
      g_batchCreateError = "batched runs use a constant time_step_size";
      return 1;
    }
    if (!c.blocks[0].exc.empty()) {
      g_batchCreateError = "batched runs do not take solenoidal-excitation patches";
      return 1;
    }
    if (c.opts.enable_solution_limits) {
      g_batchCreateError = "batched runs do not check solution limits; run the instance with mgd_run_forward";
      return 1;
    }
  }
  mgd_batch* b = new mgd_batch();
  b->inst.assign(instances, instances + n_instances);
  Context& c0 = b->inst[0]->c;
  b->device = c0.device;
  cudaSetDevice(b->device);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess) {
    g_batchCreateError = "stream or event creation failed";
    destroyBatch(b);
    return 1;
  }
  // tile shapes per grid size, among shapes of kBatchThreads threads
  static const int cand2[][3] = {{128, 1, 1}, {64, 2, 1}, {32, 4, 1}, {16, 8, 1}};
  static const int cand3[][3] = {{128, 1, 1}, {64, 2, 1}, {32, 4, 1}, {32, 2, 2}, {16, 8, 1}, {16, 4, 2}, {8, 4, 4}};
  const bool twoD = c0.nD == 2;
  const int (*cands)[3] = twoD ? cand2 : cand3;
  const int nCands = twoD ? 4 : 7;
  std::map<std::tuple<int, int, int>, std::array<Tile, 3>> chosen;
  b->tiles.resize(n_instances);
  for (int i = 0; i < n_instances; ++i) {
    Context& c = b->inst[i]->c;
    DevBlock& blk = c.blocks[0];
    const auto key = std::make_tuple(blk.v.gs[0], blk.v.gs[1], blk.v.gs[2]);
    auto it = chosen.find(key);
    if (it == chosen.end()) {
      std::array<Tile, 3> t;
      for (int k = 0; k < 3; ++k) {
        t[k] = makeTile(blk, cands[0][0], cands[0][1], cands[0][2]);
        if (k == BK_DISS && !c.phys.dissipation) continue;
        if (autotuneTile(c, blk, k, cands, nCands, &t[k])) {
          g_batchCreateError = "autotune failed: " + c.error;
          destroyBatch(b);
          return 1;
        }
      }
      it = chosen.emplace(key, t).first;
    }
    b->tiles[i] = it->second;
  }
  // block maps
  std::vector<int2> maps[BK_COUNT];
  for (int i = 0; i < n_instances; ++i) {
    const DevBlock& blk = b->inst[i]->c.blocks[0];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < b->tiles[i][k].blocks(); ++j) maps[k].push_back(make_int2(i, j));
    const int nPrims = (int)((blk.v.N + 127) / 128);
    for (int j = 0; j < nPrims; ++j) maps[BK_PRIMS].push_back(make_int2(i, j));
    for (int j = 0; j < reductionBlocks(blk); ++j) maps[BK_FUNC].push_back(make_int2(i, j));
  }
  for (int k = 0; k < BK_COUNT; ++k) {
    if (cudaMalloc((void**)&b->dMap[k], maps[k].size() * sizeof(int2)) != cudaSuccess ||
        cudaMemcpy(b->dMap[k], maps[k].data(), maps[k].size() * sizeof(int2), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      g_batchCreateError = "device allocation failed for the block maps";
      destroyBatch(b);
      return 1;
    }
    b->L.map[k] = b->dMap[k];
    b->L.blocks[k] = (int)maps[k].size();
  }
  b->L.threads[BK_GRAD] = b->L.threads[BK_DISS] = b->L.threads[BK_RHS] = kBatchThreads;
  b->L.threads[BK_PRIMS] = b->L.threads[BK_FUNC] = 128;
  if (cudaMalloc((void**)&b->dEntries, n_instances * sizeof(BatchEntry)) != cudaSuccess ||
      cudaMalloc((void**)&b->dCounters, 2 * sizeof(int)) != cudaSuccess) {
    g_batchCreateError = "device allocation failed for the batch entries";
    destroyBatch(b);
    return 1;
  }
  b->L.entries = b->dEntries;
  // work of the persistent run: round A = gradient/flux tiles, dissipation
  // (tile, component) pairs, functional blocks (heaviest first); round B =
  // divergence (tile, component) pairs (the BK_RHS map with the components);
  // round C = blocks of points for the primitives (the BK_PRIMS map)
  {
    std::vector<int4> unitsA, unitsB;
    std::vector<int4> counts(n_instances, make_int4(0, 0, 0, 0));
    const int nU = c0.nU;
    for (int i = 0; i < n_instances; ++i)
      for (int j = 0; j < b->tiles[i][BK_GRAD].blocks(); ++j) unitsA.push_back(make_int4(0, i, j, 0));
    if (c0.phys.dissipation)
      for (int i = 0; i < n_instances; ++i)
        for (int j = 0; j < b->tiles[i][BK_DISS].blocks(); ++j)
          for (int cc = 0; cc < nU; ++cc) unitsA.push_back(make_int4(1, i, j, cc));
    for (int i = 0; i < n_instances; ++i)
      for (int j = 0; j < reductionBlocks(b->inst[i]->c.blocks[0]); ++j) unitsA.push_back(make_int4(2, i, j, 0));
    for (int cc = 0; cc < nU; ++cc)
      for (const int2& m : maps[BK_RHS]) unitsB.push_back(make_int4(m.x, m.y, cc, 0));
    for (const int4& u : unitsA) counts[u.y].x += 1;
    for (const int4& u : unitsB) counts[u.x].y += 1;
    for (const int2& m : maps[BK_PRIMS]) counts[m.x].z += 1;
    if (cudaMalloc((void**)&b->dUnitsA, unitsA.size() * sizeof(int4)) != cudaSuccess ||
        cudaMemcpy(b->dUnitsA, unitsA.data(), unitsA.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc((void**)&b->dUnitsB, unitsB.size() * sizeof(int4)) != cudaSuccess ||
        cudaMemcpy(b->dUnitsB, unitsB.data(), unitsB.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc((void**)&b->dCounts, counts.size() * sizeof(int4)) != cudaSuccess ||
        cudaMemcpy(b->dCounts, counts.data(), counts.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc((void**)&b->dQueue, (1 + (size_t)n_instances) * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc((void**)&b->dStatus, sizeof(int)) != cudaSuccess) {
      g_batchCreateError = "device allocation failed for the persistent run";
      destroyBatch(b);
      return 1;
    }
    b->plan.unitsA = b->dUnitsA;
    b->plan.nA = (int)unitsA.size();
    b->plan.unitsB = b->dUnitsB;
    b->plan.nB = (int)unitsB.size();
    b->plan.unitsC = b->dMap[BK_PRIMS];
    b->plan.nC = b->L.blocks[BK_PRIMS];
    b->plan.counts = b->dCounts;
    b->plan.work = b->dQueue;
    b->plan.done = b->dQueue + 1;
    b->plan.status = b->dStatus;
    // about 100 ns per poll: a wait gives up after about a second (a unit
    // waits at most for the units of one round of its instance, milliseconds)
    b->plan.spinLimit = 1LL << 23;
    b->persistentGrid = std::min(persistentGridSize(c0), std::max(b->plan.nA, b->plan.nB));
    if (b->persistentGrid < 1) b->persistent = false;
  }
  *out = b;
  return 0;
}

int mgd_batch_persistent(mgd_batch* batch, int mode) {
  if (!batch) return -1;
  if (mode == 0 || mode == 1) batch->persistent = mode == 1 && batch->persistentGrid > 0;
  return batch->persistent ? 1 : 0;
}

int mgd_batch_persistent_grid(mgd_batch* batch) { return batch ? batch->persistentGrid : 0; }

// The persistent run: work queue and status reset, then one cooperative launch
// of every step, captured once per step count in a graph (launched directly
// when the capture is refused).
static int runPersistent(mgd_batch* b, int n_steps, bool functional) {
  Context& c0 = b->inst[0]->c;
  BATCH_TRY(b, cudaMemsetAsync(b->dQueue, 0, (1 + b->inst.size()) * sizeof(unsigned long long), b->stream));
  BATCH_TRY(b, cudaMemsetAsync(b->dStatus, 0, sizeof(int), b->stream));
  if (!b->graphP || b->graphPSteps != n_steps) {
    if (b->graphP) cudaGraphExecDestroy(b->graphP);
    b->graphP = nullptr;
    b->graphPCaptured = false;
    cudaGraph_t g = nullptr;
    const long long before = c0.launches;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const cudaError_t le = launchBatchPersistent(c0, b->dEntries, b->plan, n_steps, functional, b->persistentGrid,
                                                   b->stream);
      const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
      if (le == cudaSuccess && ce == cudaSuccess && g && cudaGraphInstantiate(&b->graphP, g, 0) == cudaSuccess)
        b->graphPCaptured = true;
      if (g) cudaGraphDestroy(g);
    }
    c0.launches = before;
    cudaGetLastError();
    b->graphPSteps = n_steps;
  }
  if (b->graphPCaptured) {
    BATCH_TRY(b, cudaGraphLaunch(b->graphP, b->stream));
  } else {
    BATCH_TRY(b, launchBatchPersistent(c0, b->dEntries, b->plan, n_steps, functional, b->persistentGrid, b->stream));
  }
  b->launches += 1;
  BATCH_TRY(b, cudaStreamSynchronize(b->stream));
  BATCH_TRY(b, cudaGetLastError());
  int status = 0;
  BATCH_TRY(b, cudaMemcpy(&status, b->dStatus, sizeof(int), cudaMemcpyDeviceToHost));
  if (status) return bfail(b, "persistent batched run: a wait for a unit's inputs ran out of its spin limit");
  return 0;
}

int mgd_batch_destroy(mgd_batch* batch) {
  if (batch) destroyBatch(batch);
  return 0;
}

long long mgd_batch_kernel_launches(mgd_batch* batch, int reset) {
  const long long n = batch->launches;
  if (reset) batch->launches = 0;
  return n;
}

int mgd_batch_run_forward(mgd_batch* b, int n_steps, double t0, double* costs) {
  if (n_steps < 1) return bfail(b, "n_steps must be >= 1");
  const int n = (int)b->inst.size();
  std::vector<BatchEntry> entries(n);
  for (int i = 0; i < n; ++i) {
    Context& c = b->inst[i]->c;
    if (prepareForwardRun(c, n_steps, n_steps, t0, false)) return bfail(b, "instance " + std::to_string(i) + ": " + c.error);
    BatchEntry& e = entries[i];
    std::memset(&e, 0, sizeof e);
    e.v = c.blocks[0].v;
    e.rs = runScalarsOf(c);
    e.rs.step = b->dCounters;
    e.rs.segBase = b->dCounters + 1;
    e.tGrad = b->tiles[i][BK_GRAD];
    e.tDiss = b->tiles[i][BK_DISS];
    e.tRhs = b->tiles[i][BK_RHS];
    e.controller = (c.opts.enable_controller && c.opts.controller_switch && c.dForcing) ? 1 : 0;
  }
  for (int i = 0; i < n; ++i) BATCH_TRY(b, cudaStreamSynchronize(b->inst[i]->c.stream));
  BATCH_TRY(b, cudaMemcpyAsync(b->dEntries, entries.data(), n * sizeof(BatchEntry), cudaMemcpyHostToDevice,
                               b->stream));
  const int init[2] = {1, 0};
  BATCH_TRY(b, cudaMemcpyAsync(b->dCounters, init, sizeof init, cudaMemcpyHostToDevice, b->stream));
  Context& c0 = b->inst[0]->c;
  const bool functional = c0.opts.enable_functional != 0;
  if (b->persistent) {
    if (runPersistent(b, n_steps, functional)) return 1;
    for (int i = 0; i < n; ++i) {
      Context& c = b->inst[i]->c;
      if (finishForwardRun(c, &costs[i])) return bfail(b, "instance " + std::to_string(i) + ": " + c.error);
    }
    return 0;
  }
  if (!b->graph) {
    const long long before = c0.launches;
    cudaGraph_t g = nullptr;
    BATCH_TRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 1; i <= 4; ++i) {
      const bool diss = c0.phys.dissipation != 0;
      if (diss) {
        cudaEventRecord(b->fork, b->stream);
        cudaStreamWaitEvent(b->side, b->fork, 0);
        launchBatchDissipation(c0, b->L, b->side);
        cudaEventRecord(b->join, b->side);
      }
      launchBatchGradFlux(c0, b->L, i, b->stream);
      if (diss) cudaStreamWaitEvent(b->stream, b->join, 0);
      launchBatchForwardDivergence(c0, b->L, i, b->stream);
      launchBatchPrims(c0, b->L, b->stream);
      if (functional) launchBatchFunctional(c0, b->L, i, b->stream);
    }
    launchStepAdvanceOn(b->dCounters, 1, b->stream);
    BATCH_TRY(b, cudaStreamEndCapture(b->stream, &g));
    b->nodes = c0.launches - before + 1;
    c0.launches = before;
    const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return bfail(b, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ei));
  }
  for (int s = 0; s < n_steps; ++s) BATCH_TRY(b, cudaGraphLaunch(b->graph, b->stream));
  b->launches += (long long)n_steps * b->nodes;
  BATCH_TRY(b, cudaStreamSynchronize(b->stream));
  BATCH_TRY(b, cudaGetLastError());
  for (int i = 0; i < n; ++i) {
    Context& c = b->inst[i]->c;
    if (finishForwardRun(c, &costs[i])) return bfail(b, "instance " + std::to_string(i) + ": " + c.error);
  }
  return 0;
}
