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
  *out = b;
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
