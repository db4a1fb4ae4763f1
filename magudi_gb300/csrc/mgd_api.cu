// mgd_api.cu -- the C ABI of include/magudi_gb300.h: context lifetime,
// one-time setup (grid metrics, patches, SAT matrices, mollifier
// normalization), RHS and RK4 substep calls, and the graph-captured forward
// and adjoint runs with device-resident uniform checkpointing.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <array>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <limits>
#include <cstring>
#include <string>
#include <vector>

#include "mgd_internal.h"
#include "sbp_tables.h"

using namespace mgd;


static std::string g_createError;

#define CUDA_TRY(ctx, call)                                                        \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      (ctx).error = std::string(#call) + ": " + cudaGetErrorString(e_);            \
      return 1;                                                                    \
    }                                                                              \
  } while (0)

static int fail(Context& c, const std::string& msg) {
  c.error = msg;
  return 1;
}

template <class T>
static cudaError_t devAlloc(DevBlock& b, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e == cudaSuccess) {
    b.allocations.push_back((void*)*p);
    cudaMemset(*p, 0, count * sizeof(T));
  }
  return e;
}

static void freeBlock(DevBlock& b) {
  for (void* p : b.allocations) cudaFree(p);
  b.allocations.clear();
}

static int checkLaunch(Context& c) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(c, std::string("kernel launch: ") + cudaGetErrorString(e));
  if (c.tmaLaunched) {
    // a kernel that waits on tensor-memory-accelerator copies records a wait
    // that ran out in the error word
    c.tmaLaunched = false;
    int flag = 0;
    e = cudaMemcpyAsync(&flag, c.dKernelError, sizeof flag, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return fail(c, std::string("kernel error word: ") + cudaGetErrorString(e));
    if (flag) {
      cudaMemsetAsync(c.dKernelError, 0, sizeof(int), c.stream);
      return fail(c, "a wait for a tensor-memory-accelerator copy ran out of its poll limit");
    }
  }
  return 0;
}

static int ncompOf(const Context& c, int field) {
  switch (field) {
    case MGD_FIELD_CONSERVED: case MGD_FIELD_ADJOINT: case MGD_FIELD_TARGET: case MGD_FIELD_RHS:
      return c.nU;
    case MGD_FIELD_METRICS: return c.nD * c.nD;
    case MGD_FIELD_ARC_LENGTHS: return c.nD;
    default: return 1;
  }
}

// Definitions below take C linkage from their declarations in magudi_gb300.h.

const char* mgd_last_error(const mgd_ctx* ctx) {
  return ctx ? ctx->c.error.c_str() : g_createError.c_str();
}

int mgd_create(const mgd_options* o, mgd_ctx** out) {
  *out = nullptr;
  if (!o || (o->n_dimensions != 2 && o->n_dimensions != 3)) {
    g_createError = "n_dimensions must be 2 or 3";
    return 1;
  }
  if (o->discretization_scheme < MGD_SBP_48 || o->discretization_scheme > MGD_SBP_36) {
    g_createError = "discretization_scheme must be one of MGD_SBP_48, MGD_SBP_12, MGD_SBP_24, MGD_SBP_36";
    return 1;
  }
  if (o->discretization_scheme == MGD_SBP_12 && o->dissipation && !o->composite_dissipation) {
    g_createError = "SBP 1-2 has no non-composite dissipation operator";
    return 1;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    g_createError = "no CUDA device available";
    return 1;
  }
  mgd_ctx* h = new mgd_ctx();
  Context& c = h->c;
  c.opts = *o;
  c.nD = o->n_dimensions;
  c.nU = c.nD + 2;
  cudaGetDevice(&c.device);
  // src/SolverOptionsImpl.f90:46-71
  Physics& P = c.phys;
  P.g = o->ratio_of_specific_heats;
  P.gm1 = P.g - 1.0;
  P.gOverGm1 = P.g / P.gm1;
  P.invGm1 = 1.0 / P.gm1;
  P.gm2OverGm1 = (P.g - 2.0) / P.gm1;
  P.invG = 1.0 / P.g;
  P.viscous = o->viscous;
  P.dissipation = o->dissipation;
  P.composite = o->composite_dissipation;
  P.dissipationAmount = o->dissipation_amount;
  P.reInv = 0.0; P.prInv = 0.0; P.powerLawExponent = 0.0; P.laFactor = 0.0;
  if (o->viscous) {
    const double re = std::max(0.0, o->reynolds_number), pr = std::max(0.0, o->prandtl_number);
    if (re <= 0.0 || pr <= 0.0) {
      P.reInv = re; P.prInv = pr;
      P.laFactor = (0.0 - 2.0 / 3.0);
    } else {
      P.reInv = 1.0 / re; P.prInv = 1.0 / pr;
      P.powerLawExponent = o->viscosity_power_law_exponent;
      P.laFactor = o->bulk_viscosity_ratio - 2.0 / 3.0;
    }
  }
  P.powerLaw = P.powerLawExponent > 0.0 ? 1 : 0;
  if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
    g_createError = "cudaStreamCreate failed";
    delete h;
    return 1;
  }
  if (cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c.stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c.side2, cudaStreamNonBlocking) != cudaSuccess) {
    g_createError = "cudaStreamCreate failed";
    cudaStreamDestroy(c.stream);
    delete h;
    return 1;
  }
  for (int k = 0; k < 8; ++k) {
    cudaEventCreateWithFlags(&c.evFork[k], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c.evJoin[k], cudaEventDisableTiming);
  }
  for (int k = 0; k < 2; ++k) {
    cudaEventCreateWithFlags(&c.evRecDone[k], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c.evAdjDone[k], cudaEventDisableTiming);
  }
  uploadOperatorTables();
  cudaMalloc((void**)&c.dCounters, 8 * sizeof(int));
  const int init[8] = {1, 0, 1, 0, 1, 0, 0, 0};
  cudaMemcpy(c.dCounters, init, sizeof init, cudaMemcpyHostToDevice);
  cudaMalloc((void**)&c.dApiAmp, MGD_MAX_SOURCES * sizeof(double));
  cudaMemset(c.dApiAmp, 0, MGD_MAX_SOURCES * sizeof(double));
  cudaMalloc((void**)&c.dApiTime, sizeof(double));
  cudaMemset(c.dApiTime, 0, sizeof(double));
  cudaMalloc((void**)&c.dLimitKey, sizeof(unsigned long long));
  cudaMemset(c.dLimitKey, 0xFF, sizeof(unsigned long long));
  cudaMalloc((void**)&c.dKernelError, sizeof(int));
  cudaMemset(c.dKernelError, 0, sizeof(int));
  if (cudaGetLastError() != cudaSuccess) {
    g_createError = "device allocation failed";
    delete h;
    return 1;
  }
  *out = h;
  return 0;
}

int mgd_destroy(mgd_ctx* h) {
  if (!h) return 0;
  Context& c = h->c;
  if (c.ioThread.joinable()) c.ioThread.join();
  if (c.ioStaging) cudaFreeHost(c.ioStaging);
  if (c.ioStream) cudaStreamDestroy(c.ioStream);
  if (c.ioCopied) cudaEventDestroy(c.ioCopied);
  cudaStreamSynchronize(c.stream);
  for (DevBlock& b : c.blocks) {
    freeBlock(b);
    cudaFree(b.runSnap);
    cudaFree(b.runStage);
    cudaFree(b.runPartials);
  }
  cudaFree(c.dLimitKey);
  cudaFree(c.dKernelError);
  cudaFree(c.dCounters); cudaFree(c.dApiAmp); cudaFree(c.dAmp); cudaFree(c.dForcing);
  cudaFree(c.dApiTime); cudaFree(c.dStageTime); cudaFree(c.dDeltaForcing); cudaFree(c.dApiForcing);
  cudaFree(c.dGradient); cudaFree(c.dPartials); cudaFree(c.dStageValues);
  cudaFree(c.dSnapshots); cudaFree(c.dStageBuf);
  cudaFree(c.dStepDt); cudaFree(c.dDtPartials); cudaFree(c.dTime); cudaFree(c.dNorm);
  if (c.gForward) cudaGraphExecDestroy(c.gForward);
  for (int k = 0; k < 2; ++k) {
    if (c.gRecomputeH[k]) cudaGraphExecDestroy(c.gRecomputeH[k]);
    if (c.gAdjointH[k]) cudaGraphExecDestroy(c.gAdjointH[k]);
    cudaEventDestroy(c.evRecDone[k]);
    cudaEventDestroy(c.evAdjDone[k]);
  }
  for (void* p : c.shadowAllocations) cudaFree(p);
  if (c.stream2) cudaStreamDestroy(c.stream2);
  if (c.side2) cudaStreamDestroy(c.side2);
  for (int k = 0; k < MGD_MAX_BLOCKS; ++k) {
    if (c.blockStreams[k]) cudaStreamDestroy(c.blockStreams[k]);
    if (c.evBlockJoin[k]) cudaEventDestroy(c.evBlockJoin[k]);
    if (c.blockStreams2[k]) cudaStreamDestroy(c.blockStreams2[k]);
    if (c.evBlockJoin2[k]) cudaEventDestroy(c.evBlockJoin2[k]);
  }
  if (c.evBlockFork) cudaEventDestroy(c.evBlockFork);
  if (c.evBlockFork2) cudaEventDestroy(c.evBlockFork2);
  for (int k = 0; k < 8; ++k) {
    cudaEventDestroy(c.evFork[k]);
    cudaEventDestroy(c.evJoin[k]);
  }
  cudaStreamDestroy(c.side);
  cudaStreamDestroy(c.stream);
  delete h;
  return 0;
}

void* mgd_stream(mgd_ctx* h) { return h ? (void*)h->c.stream : nullptr; }

long long mgd_kernel_launches(mgd_ctx* h, int reset) {
  const long long n = h->c.launches;
  if (reset) h->c.launches = 0;
  return n;
}

int mgd_set_trajectory_storage(mgd_ctx* h, int enable, double max_bytes) {
  Context& c = h->c;
  c.trajectoryStorage = enable != 0;
  c.trajectoryMaxBytes = max_bytes;
  if (!enable) c.trajectorySteps = 0;
  return 0;
}

int mgd_stage_tile(mgd_ctx* h, int kernel, int* tile, int set) {
  Context& c = h->c;
  if (kernel < 0 || kernel > 5 || !tile) return fail(c, "mgd_stage_tile: kernel must be 0..5 and tile non-null");
  if (c.blocks.empty()) return fail(c, "mgd_stage_tile: no blocks");
  auto slot = [&](DevBlock& b) -> Tile& {
    Tile* s[6] = {&b.tGrad, &b.tDiss, &b.tRhs, &b.tAdjA, &b.tAdjD, &b.tAdjB};
    return *s[kernel];
  };
  if (!set) {
    const Tile& t = slot(c.blocks[0]);
    for (int d = 0; d < 3; ++d) tile[d] = t.t[d];
    return 0;
  }
  if (tile[0] < 1 || tile[1] < 1 || tile[2] < 1 || (long long)tile[0] * tile[1] * tile[2] > 256)
    return fail(c, "mgd_stage_tile: tile extents must be >= 1 with at most 256 threads");
  for (auto& b : c.blocks) slot(b) = makeTile(b, tile[0], tile[1], tile[2]);
  return 0;
}

int mgd_adjoint_core_lanes(mgd_ctx* h, int lanes) {
  Context& c = h->c;
  if (lanes < 0 || lanes > 2) {
    fail(c, "mgd_adjoint_core_lanes: lanes must be 0, 1 or 2");
    return -1;
  }
  if (lanes > 0 && c.nD == 2)
    for (auto& b : c.blocks) b.coreLanes = lanes;
  return c.nD == 2 && !c.blocks.empty() ? c.blocks[0].coreLanes : 1;
}

int mgd_dissipation_tma(mgd_ctx* h, int mode) {
  Context& c = h->c;
  if (mode < -1 || mode > 1) {
    fail(c, "mgd_dissipation_tma: mode must be -1, 0 or 1");
    return -1;
  }
  if (mode >= 0) c.useTmaDissipation = mode == 1;
  return c.useTmaDissipation ? 1 : 0;
}

int mgd_gradient_lanes(mgd_ctx* h, int lanes) {
  Context& c = h->c;
  if (lanes < 0 || lanes > 2) {
    fail(c, "mgd_gradient_lanes: lanes must be 0, 1 or 2");
    return -1;
  }
  if (lanes > 0 && c.nD == 2)
    for (auto& b : c.blocks) b.gradLanes = lanes;
  return c.nD == 2 && !c.blocks.empty() ? c.blocks[0].gradLanes : 1;
}

// Grid%update (src/GridImpl.f90:746-1066) from device coordinate derivatives.
static int computeMetrics(Context& c, DevBlock& b) {
  const int nD = c.nD;
  const long long N = b.v.N;
  double* dJmi = nullptr;
  CUDA_TRY(c, cudaMalloc((void**)&dJmi, (size_t)N * nD * nD * sizeof(double)));
  // coordinates staged in q
  CUDA_TRY(c, cudaMemcpyAsync(b.v.q, b.hostCoords.data(), (size_t)N * nD * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  for (int d = 0; d < nD; ++d) launchCoordinateDerivative(c, b, d, dJmi + (size_t)N * nD * d);
  if (checkLaunch(c)) { cudaFree(dJmi); return 1; }
  std::vector<double> jmi((size_t)N * nD * nD);
  CUDA_TRY(c, cudaMemcpyAsync(jmi.data(), dJmi, jmi.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  b.hostJmi = jmi;
  for (int i = 0; i < nD * nD; ++i)
    for (long long p = 0; p < N; ++p)
      if (b.hostIblank[p] == 0) jmi[(size_t)N * i + p] = 0.0;
  auto J = [&](int k, long long p) { return jmi[(size_t)N * (k - 1) + p]; };
  std::vector<double> det(N), metrics((size_t)N * nD * nD, 0.0), arc((size_t)N * nD, 0.0);
  auto M = [&](int k, long long p) -> double& { return metrics[(size_t)N * (k - 1) + p]; };
  const bool curv = c.opts.curvilinear != 0;
  if (nD == 2) {
    for (long long p = 0; p < N; ++p) {
      if (curv) {
        det[p] = J(1, p) * J(4, p) - J(2, p) * J(3, p);
        M(1, p) = J(4, p); M(2, p) = -J(3, p); M(3, p) = -J(2, p); M(4, p) = J(1, p);
        arc[p] = std::sqrt(M(1, p) * M(1, p) + M(2, p) * M(2, p));
        arc[N + p] = std::sqrt(M(3, p) * M(3, p) + M(4, p) * M(4, p));
      } else {
        det[p] = J(1, p) * J(4, p);
        M(1, p) = J(4, p); M(4, p) = J(1, p);
        arc[p] = std::fabs(M(1, p));
        arc[N + p] = std::fabs(M(4, p));
      }
    }
  } else {
    bool plane = false;
    for (int d = 0; d < 3; ++d) plane = plane || b.desc.periodicity_type[d] == MGD_PERIODIC_PLANE;
    for (long long p = 0; p < N; ++p)
      det[p] = curv ? J(1, p) * (J(5, p) * J(9, p) - J(8, p) * J(6, p)) +
                          J(4, p) * (J(8, p) * J(3, p) - J(2, p) * J(9, p)) +
                          J(7, p) * (J(2, p) * J(6, p) - J(5, p) * J(3, p))
                    : J(1, p) * J(5, p) * J(9, p);
    if (plane) {
      for (long long p = 0; p < N; ++p) {
        if (curv) {
          M(1, p) = J(5, p) * J(9, p) - J(8, p) * J(6, p);
          M(2, p) = J(7, p) * J(6, p) - J(4, p) * J(9, p);
          M(3, p) = J(4, p) * J(8, p) - J(7, p) * J(5, p);
          M(4, p) = J(8, p) * J(3, p) - J(2, p) * J(9, p);
          M(5, p) = J(1, p) * J(9, p) - J(7, p) * J(3, p);
          M(6, p) = J(7, p) * J(2, p) - J(1, p) * J(8, p);
          M(7, p) = J(2, p) * J(6, p) - J(5, p) * J(3, p);
          M(8, p) = J(4, p) * J(3, p) - J(1, p) * J(6, p);
          M(9, p) = J(1, p) * J(5, p) - J(4, p) * J(2, p);
        } else {
          M(1, p) = J(5, p) * J(9, p);
          M(5, p) = J(1, p) * J(9, p);
          M(9, p) = J(1, p) * J(5, p);
        }
      }
    } else {
      // conservative form: metric = D_a(jmi * coordinate) - D_b(jmi * coordinate)
      struct Term { int metric, ja, ca, da, jb, cb, db; bool cartesian; };
      const Term terms[9] = {{1, 5, 3, 3, 8, 3, 2, true},  {2, 6, 1, 3, 9, 1, 2, false},
                             {3, 4, 2, 3, 7, 2, 2, false}, {4, 8, 3, 1, 2, 3, 3, false},
                             {5, 9, 1, 1, 3, 1, 3, true},  {6, 7, 2, 1, 1, 2, 3, false},
                             {7, 2, 3, 2, 5, 3, 1, false}, {8, 3, 1, 2, 6, 1, 1, false},
                             {9, 1, 2, 2, 4, 2, 1, true}};
      std::vector<double> F(N), G(N);
      double* dF = dJmi;  // reuse as scratch (jmi already on the host)
      auto derivOfProduct = [&](int ja, int ca, int da) -> int {
        for (long long p = 0; p < N; ++p) F[p] = J(ja, p) * b.hostCoords[(size_t)N * (ca - 1) + p];
        CUDA_TRY(c, cudaMemcpyAsync(dF, F.data(), N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        launchApplyD1(c, b, da - 1, dF, dF + N, 1);
        CUDA_TRY(c, cudaMemcpyAsync(G.data(), dF + N, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CUDA_TRY(c, cudaStreamSynchronize(c.stream));
        return 0;
      };
      for (const Term& t : terms) {
        if (!t.cartesian && !curv) continue;
        if (derivOfProduct(t.ja, t.ca, t.da)) { cudaFree(dJmi); return 1; }
        for (long long p = 0; p < N; ++p) M(t.metric, p) = G[p];
        if (curv) {
          if (derivOfProduct(t.jb, t.cb, t.db)) { cudaFree(dJmi); return 1; }
          for (long long p = 0; p < N; ++p) M(t.metric, p) = M(t.metric, p) - G[p];
        }
      }
      for (int i = 1; i <= 9; ++i)
        for (long long p = 0; p < N; ++p)
          if (b.hostIblank[p] == 0) M(i, p) = 0.0;
    }
    for (long long p = 0; p < N; ++p)
      for (int d = 0; d < 3; ++d)
        arc[N * d + p] = curv ? std::sqrt(M(3 * d + 1, p) * M(3 * d + 1, p) + M(3 * d + 2, p) * M(3 * d + 2, p) +
                                          M(3 * d + 3, p) * M(3 * d + 3, p))
                              : std::fabs(M(4 * d + 1, p));
  }
  cudaFree(dJmi);
  for (long long p = 0; p < N; ++p)
    if (b.hostIblank[p] == 0) det[p] = 1.0;
  for (long long p = 0; p < N; ++p)
    if (!(det[p] > 0.0)) {
      char msg[128];
      std::snprintf(msg, sizeof msg, "Jacobian at point %lld is non-positive!", p);
      return fail(c, msg);
    }
  // norm = H (per non-periodic direction) * det, jacobian = 1/det
  const HostOp d1 = schemeOps(c.opts.discretization_scheme).d1;
  const int nn = (int)d1.norm.size();
  std::vector<double> norm(N, 1.0), jac(N), arcA((size_t)N * nD);
  for (int d = 0; d < nD; ++d) {
    if (b.desc.periodicity_type[d] != MGD_PERIODIC_NONE) continue;
    const int n = b.v.gs[d];
    const long long st = b.v.ax[d].stride;
    for (long long p = 0; p < N; ++p) {
      const int i = (int)((p / st) % n);
      if (i < nn) norm[p] = d1.norm[i] * norm[p];
      else if (i >= n - nn) norm[p] = d1.norm[n - 1 - i] * norm[p];
    }
  }
  for (long long p = 0; p < N; ++p) {
    norm[p] = norm[p] * det[p];
    jac[p] = 1.0 / det[p];
  }
  for (long long k = 0; k < (long long)arc.size(); ++k) arcA[k] = -c.opts.dissipation_amount * arc[k];
  CUDA_TRY(c, cudaMemcpyAsync((void*)b.v.metrics, metrics.data(), metrics.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  CUDA_TRY(c, cudaMemcpyAsync((void*)b.v.jac, jac.data(), N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  CUDA_TRY(c, cudaMemcpyAsync((void*)b.v.arcA, arcA.data(), arcA.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  // keep host copies needed by finalize (norm, arc lengths along each direction of x)
  b.hostNorm = norm;
  b.hostMetricsArc = arc;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

int mgd_add_block(mgd_ctx* h, const mgd_block_desc* desc, const double* coordinates, const int* iblank) {
  Context& c = h->c;
  if (c.finalized) return fail(c, "mgd_add_block after mgd_finalize_setup");
  if ((int)c.blocks.size() >= MGD_MAX_BLOCKS) return fail(c, "too many blocks");
  DevBlock b;
  b.desc = *desc;
  BlockView& v = b.v;
  std::memset(&v, 0, sizeof v);
  v.nD = c.nD;
  v.nU = c.nU;
  for (int i = 0; i < 3; ++i) v.gs[i] = i < c.nD ? desc->grid_size[i] : 1;
  for (int i = 0; i < c.nD; ++i) {
    const int per = desc->periodicity_type[i];
    if (per != MGD_PERIODIC_NONE && per != MGD_PERIODIC_PLANE && per != MGD_PERIODIC_OVERLAP)
      return fail(c, "periodicity_type must be MGD_PERIODIC_NONE, _PLANE or _OVERLAP");
    if (v.gs[i] < 2 * 12 + 1 && per == MGD_PERIODIC_NONE)
      return fail(c, "each non-periodic direction needs at least 25 points (the closure windows of the kernels' "
                     "operator tables)");
    // a stencil tap i +- 4 wraps once: PLANE needs a period of at least 4
    // points, OVERLAP (period n - 1) at least 5 points
    if ((per == MGD_PERIODIC_PLANE && v.gs[i] < 4) || (per == MGD_PERIODIC_OVERLAP && v.gs[i] < 5))
      return fail(c, "a PLANE-periodic direction needs at least 4 points and an OVERLAP-periodic one at least 5 "
                     "(the stencils reach 4 points to either side)");
  }
  v.N = (long long)v.gs[0] * v.gs[1] * v.gs[2];
  for (int i = 0; i < 3; ++i) {
    v.ax[i].n = v.gs[i];
    v.ax[i].per = i < c.nD ? desc->periodicity_type[i] : MGD_PERIODIC_NONE;
    v.ax[i].stride = i == 0 ? 1 : (i == 1 ? v.gs[0] : (long long)v.gs[0] * v.gs[1]);
    v.ax[i].scheme = c.opts.discretization_scheme;
  }
  v.curvilinear = c.opts.curvilinear;
  b.tGrad = b.tDiss = b.tRhs = b.tAdjA = b.tAdjD = b.tAdjB = c.nD == 2 ? makeTile(b, 32, 4, 1) : makeTile(b, 32, 2, 2);
  const long long N = v.N;
  const int nD = c.nD, nU = c.nU;
  PrimLayout L{nD};
  double *metrics, *jac, *arcA;
  int* ib;
  double *qt, *sponge, *mc, *mt, *meanP, *wT, *wA, *tgt, *srcG;
  int *actIdx, *ffOf;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (x != cudaSuccess) e = x; };
  chk(devAlloc(b, &metrics, N * nD * nD));
  chk(devAlloc(b, &jac, N));
  chk(devAlloc(b, &arcA, N * nD));
  chk(devAlloc(b, &ib, N));
  chk(devAlloc(b, &v.q, N * nU));
  chk(devAlloc(b, &v.lam, N * nU));
  chk(devAlloc(b, &qt, N * nU));
  chk(devAlloc(b, &v.rhs, N * nU));
  chk(devAlloc(b, &v.b1, N * nU));
  chk(devAlloc(b, &v.b2, N * nU));
  chk(devAlloc(b, &v.prim, N * L.count()));
  chk(devAlloc(b, &v.tau, N * nD * nD));
  chk(devAlloc(b, &v.hf, N * nD));
  chk(devAlloc(b, &v.fhat, N * nD * nU));
  chk(devAlloc(b, &v.dq, N * nD * nU));
  chk(devAlloc(b, &v.rcore, N * nU));
  chk(devAlloc(b, &v.ad, N * nD * (nU - 1)));
  chk(devAlloc(b, &v.t2, N * (nU - 1)));
  chk(devAlloc(b, &v.adjF, N * nU));
  chk(devAlloc(b, &sponge, N));
  chk(devAlloc(b, &mc, N));
  chk(devAlloc(b, &mt, N));
  chk(devAlloc(b, &meanP, N));
  chk(devAlloc(b, &wT, N));
  chk(devAlloc(b, &wA, N));
  chk(devAlloc(b, &tgt, N));
  chk(devAlloc(b, &actIdx, N));
  chk(devAlloc(b, &ffOf, 3 * N));
  chk(devAlloc(b, &srcG, N * MGD_MAX_SOURCES));
  if (e != cudaSuccess) {
    freeBlock(b);
    return fail(c, std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  v.metrics = metrics; v.jac = jac; v.arcA = arcA; v.iblank = ib; v.qt = qt;
  v.sponge = sponge; v.mc = mc; v.mt = mt; v.meanP = meanP; v.wT = wT; v.wA = wA;
  v.tgtCount = tgt; v.actIdx = actIdx; v.ffOfPoint = ffOf; v.srcG = srcG;
  b.hostCoords.assign(coordinates, coordinates + (size_t)N * nD);
  b.hostIblank.assign(iblank, iblank + N);
  // defaults: quiescent target (State%makeQuiescent), unit mollifiers, p = 1/gamma
  std::vector<double> tmp((size_t)N * nU, 0.0);
  for (long long p = 0; p < N; ++p) {
    tmp[p] = 1.0;
    tmp[(size_t)N * (nD + 1) + p] = 1.0 / c.phys.g / (c.phys.g - 1.0);
  }
  CUDA_TRY(c, cudaMemcpy(qt, tmp.data(), tmp.size() * sizeof(double), cudaMemcpyHostToDevice));
  std::vector<double> ones(N, 1.0), pm(N, 1.0 / c.phys.g);
  CUDA_TRY(c, cudaMemcpy(mc, ones.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(mt, ones.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(meanP, pm.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(ib, iblank, N * sizeof(int), cudaMemcpyHostToDevice));
  std::vector<int> neg(3 * N, -1);
  CUDA_TRY(c, cudaMemcpy(actIdx, neg.data(), N * sizeof(int), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(ffOf, neg.data(), 3 * N * sizeof(int), cudaMemcpyHostToDevice));
  c.blocks.push_back(std::move(b));
  if (computeMetrics(c, c.blocks.back())) {
    freeBlock(c.blocks.back());
    c.blocks.pop_back();
    return 1;
  }
  return 0;
}

int mgd_add_patch(mgd_ctx* h, const mgd_patch_desc* p) {
  Context& c = h->c;
  if (c.finalized) return fail(c, "mgd_add_patch after mgd_finalize_setup");
  if (p->type < MGD_PATCH_SAT_FAR_FIELD || p->type > MGD_PATCH_SOLENOIDAL_EXCITATION)
    return fail(c, std::string("unsupported patch type for patch '") + p->name + "'");
  if (p->grid_index < 1) return fail(c, "patch grid index must be >= 1");
  std::vector<double> omega, phases;
  if (p->type == MGD_PATCH_SOLENOIDAL_EXCITATION) {
    // src/SolenoidalExcitationPatchImpl.f90:40-50 (number_of_modes clipped at 0)
    const int nM = std::max(0, p->n_modes);
    if (nM > kMaxExcitationModes)
      return fail(c, std::string("patch '") + p->name + "': more than " + std::to_string(kMaxExcitationModes) +
                         " excitation modes");
    if (nM > 0 && (!p->angular_frequencies || !p->phases))
      return fail(c, std::string("patch '") + p->name + "': the excitation modes are missing");
    if (!(p->radius > 0.0)) return fail(c, std::string("patch '") + p->name + "': radius must be positive");
    if (nM > 0) {
      omega.assign(p->angular_frequencies, p->angular_frequencies + nM);
      phases.assign(p->phases, p->phases + 3 * nM);
    }
  }
  c.patches.push_back(*p);
  c.patches.back().n_modes = std::max(0, p->n_modes);
  c.patches.back().angular_frequencies = nullptr;  // copied below; the caller's arrays may go
  c.patches.back().phases = nullptr;
  c.patchOmega.push_back(std::move(omega));
  c.patchPhases.push_back(std::move(phases));
  return 0;
}

int mgd_add_acoustic_source(mgd_ctx* h, const mgd_acoustic_source* s) {
  Context& c = h->c;
  if ((int)c.sources.size() >= MGD_MAX_SOURCES) return fail(c, "too many acoustic sources");
  c.sources.push_back(*s);
  return 0;
}

static double* fieldPtr(Context& c, DevBlock& b, int field, bool write) {
  BlockView& v = b.v;
  switch (field) {
    case MGD_FIELD_CONSERVED: return v.q;
    case MGD_FIELD_ADJOINT: return v.lam;
    case MGD_FIELD_TARGET: return (double*)v.qt;
    case MGD_FIELD_RHS: return v.rhs;
    case MGD_FIELD_CONTROL_MOLLIFIER: return (double*)v.mc;
    case MGD_FIELD_TARGET_MOLLIFIER: return (double*)v.mt;
    case MGD_FIELD_MEAN_PRESSURE: return (double*)v.meanP;
    case MGD_FIELD_METRICS: return write ? nullptr : (double*)v.metrics;
    case MGD_FIELD_JACOBIAN: return write ? nullptr : (double*)v.jac;
    case MGD_FIELD_PRESSURE: return write ? nullptr : v.prim + v.N * PrimLayout{c.nD}.p();
    case MGD_FIELD_TEMPERATURE: return write ? nullptr : v.prim + v.N * PrimLayout{c.nD}.T();
    default: return nullptr;
  }
}

int mgd_set_field(mgd_ctx* h, int block, int field, const double* host) {
  Context& c = h->c;
  if (block < 1 || block > (int)c.blocks.size()) return fail(c, "invalid block index");
  DevBlock& b = c.blocks[block - 1];
  if (c.finalized && (field == MGD_FIELD_CONTROL_MOLLIFIER || field == MGD_FIELD_TARGET_MOLLIFIER ||
                      field == MGD_FIELD_TARGET))
    return fail(c, "target state and mollifiers must be set before mgd_finalize_setup");
  double* d = fieldPtr(c, b, field, true);
  if (!d) return fail(c, "field is read-only or unknown");
  CUDA_TRY(c, cudaMemcpyAsync(d, host, (size_t)b.v.N * ncompOf(c, field) * sizeof(double), cudaMemcpyDefault, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

int mgd_get_field(mgd_ctx* h, int block, int field, double* host) {
  Context& c = h->c;
  if (block < 1 || block > (int)c.blocks.size()) return fail(c, "invalid block index");
  DevBlock& b = c.blocks[block - 1];
  const size_t n = (size_t)b.v.N * ncompOf(c, field);
  if (field == MGD_FIELD_NORM) {
    std::copy(b.hostNorm.begin(), b.hostNorm.end(), host);
    return 0;
  }
  if (field == MGD_FIELD_ARC_LENGTHS) {
    std::copy(b.hostMetricsArc.begin(), b.hostMetricsArc.end(), host);
    return 0;
  }
  double* d = fieldPtr(c, b, field, false);
  if (!d) return fail(c, "unknown field");
  CUDA_TRY(c, cudaMemcpyAsync(host, d, n * sizeof(double), cudaMemcpyDefault, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

// Patch extents with negative indices counted from the end
// (src/PatchDescriptorImpl.f90:57-63).
static void resolveExtent(const mgd_patch_desc& p, const int gs[3], int nD, int ext[6]) {
  for (int i = 0; i < 3; ++i) {
    int lo = p.extent[2 * i], hi = p.extent[2 * i + 1];
    if (i >= nD) lo = hi = 1;
    if (lo < 0) lo += gs[i] + 1;
    if (hi < 0) hi += gs[i] + 1;
    ext[2 * i] = lo;
    ext[2 * i + 1] = hi;
  }
}

template <class F>
static void forExtent(const int ext[6], const int gs[3], F f) {
  long long pi = 0;
  for (int k = ext[4]; k <= ext[5]; ++k)
    for (int j = ext[2]; j <= ext[3]; ++j)
      for (int i = ext[0]; i <= ext[1]; ++i, ++pi)
        f((long long)(i - 1) + (long long)gs[0] * ((j - 1) + (long long)gs[1] * (k - 1)), pi);
}

// Tile-shape autotuner: times each stage kernel of one RK stage under
// candidate thread-block tilings on the current state and keeps the fastest
// per kernel. Results are cached per grid shape and physics flags for the
// lifetime of the process.
static RunScalars apiScalars(Context& c);
static int setApiTime(Context& c, double time);

struct TuneKey {
  int nD, gs[3], curv, visc, diss, comp;
  bool operator<(const TuneKey& o) const {
    return std::tie(nD, gs[0], gs[1], gs[2], curv, visc, diss, comp) <
           std::tie(o.nD, o.gs[0], o.gs[1], o.gs[2], o.curv, o.visc, o.diss, o.comp);
  }
};

// Tiles of the six stage kernels of a block, shared by all contexts of the
// process (contexts may be set up from several threads): filled by the
// per-kernel autotuner at setup and replaced by mgd_tune_run.
struct Tuned {
  std::array<Tile, 6> tiles;
  int gradLanes, coreLanes;
};
static std::map<TuneKey, Tuned> g_tuneCache;
static std::mutex g_tuneCacheMutex;

static TuneKey tuneKey(const Context& c, const DevBlock& b) {
  return TuneKey{c.nD, {b.v.gs[0], b.v.gs[1], b.v.gs[2]}, b.v.curvilinear, c.phys.viscous, c.phys.dissipation,
                 c.phys.composite};
}

static void storeTuned(const Context& c, const DevBlock& b) {
  const Tile* slots[6] = {&b.tGrad, &b.tDiss, &b.tRhs, &b.tAdjA, &b.tAdjD, &b.tAdjB};
  Tuned entry;
  for (int k = 0; k < 6; ++k) entry.tiles[k] = *slots[k];
  entry.gradLanes = b.gradLanes;
  entry.coreLanes = b.coreLanes;
  std::lock_guard<std::mutex> lock(g_tuneCacheMutex);
  g_tuneCache[tuneKey(c, b)] = entry;
}

static int autotune(Context& c, DevBlock& b) {
  const TuneKey key = tuneKey(c, b);
  Tile* slots[6] = {&b.tGrad, &b.tDiss, &b.tRhs, &b.tAdjA, &b.tAdjD, &b.tAdjB};
  {
    std::lock_guard<std::mutex> lock(g_tuneCacheMutex);
    auto it = g_tuneCache.find(key);
    if (it != g_tuneCache.end()) {
      for (int k = 0; k < 6; ++k) *slots[k] = it->second.tiles[k];
      b.gradLanes = it->second.gradLanes;
      b.coreLanes = it->second.coreLanes;
      return 0;
    }
  }
  // 2D: CTAs of 128 or 256 threads. At 2D sizes a stage kernel is a single
  // wave that shares the SMs with the side-stream dissipation and, in adjoint
  // runs, the concurrent checkpoint recomputation; smaller CTAs that are
  // fastest alone fill the SMs' CTA slots (at most 32 per SM) and slow those
  // down. 3D kernels run many waves and also take 64-thread tiles.
  std::vector<std::array<int, 3>> cands;
  if (c.nD == 2)
    cands = {{128, 1, 1}, {64, 2, 1}, {32, 4, 1}, {16, 8, 1}, {8, 16, 1},
             {256, 1, 1}, {128, 2, 1}, {64, 4, 1}, {32, 8, 1}, {16, 16, 1}};
  else
    cands = {{32, 2, 2}, {32, 4, 1}, {16, 4, 2}, {16, 8, 1}, {8, 8, 2}, {32, 1, 4}, {64, 2, 1},
             {32, 2, 1}, {16, 2, 2}, {8, 4, 4}, {32, 4, 2}};
  RunScalars rs = apiScalars(c);
  if (setApiTime(c, 0.0)) return 1;
  launchPrims(c, b, b.v.q, false);
  if (c.phys.viscous) launchGradFlux(c, b, false, true, &rs, 1, false);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // kTuneReps back-to-back launches per timing, the fastest of kTunePasses
  // passes over the candidates: single timings of kernels of tens of
  // microseconds right after setup vary with the clock ramp
  constexpr int kTuneReps = 10, kTunePasses = 2;
  auto timeIt = [&](auto fn) {
    fn();
    cudaEventRecord(e0, c.stream);
    for (int r = 0; r < kTuneReps; ++r) fn();
    cudaEventRecord(e1, c.stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
  };
  const long long saved = c.launches;
  for (int k = 0; k < 6; ++k) {
    if ((k == 1 && !c.phys.dissipation) || (k == 4 && !c.phys.viscous)) continue;
    auto launch = [&]() {
      switch (k) {
        case 0: launchGradFlux(c, b, true, false, &rs, 1, false); break;
        case 1: launchDissipation(c, b, b.v.q, 1.0); break;
        case 2: launchForwardDivergence(c, b, 0, rs, true, false); break;
        case 3: launchAdjointCore(c, b, rs, 1, false); break;
        case 4: launchAdjointDiffusion(c, b); break;
        default: launchAdjointAssemble(c, b, 0, rs, 1, 0.0, true, false); break;
      }
    };
    // the gradient/flux kernel of 2D blocks also has a two-lanes-per-point form
    const int nLaneForms = (k == 0 && c.nD == 2) ? 2 : 1;
    const int nc = (int)cands.size();
    std::vector<float> ms((size_t)nLaneForms * nc, 1e30f);
    for (int r = 0; r < 20; ++r) launch();  // clocks up before the first timing
    for (int pass = 0; pass < kTunePasses; ++pass)
      for (int lf = 0; lf < nLaneForms; ++lf)
        for (int i = 0; i < nc; ++i) {
          *slots[k] = makeTile(b, cands[i][0], cands[i][1], cands[i][2]);
          if (k == 0) b.gradLanes = lf + 1;
          ms[(size_t)lf * nc + i] = std::min(ms[(size_t)lf * nc + i], timeIt(launch));
        }
    const int best = (int)(std::min_element(ms.begin(), ms.end()) - ms.begin());
    *slots[k] = makeTile(b, cands[best % nc][0], cands[best % nc][1], cands[best % nc][2]);
    if (k == 0) b.gradLanes = best / nc + 1;
  }
  c.launches = saved;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (checkLaunch(c)) return 1;
  storeTuned(c, b);
  return 0;
}

namespace mgd {

// Fastest of nCands tile shapes for one forward stage kernel (BK_GRAD,
// BK_DISS or BK_RHS) of block b, timed on its current state; b's own tiles
// are left as they were.
int autotuneTile(Context& c, DevBlock& b, int kernel, const int (*cands)[3], int nCands, Tile* best) {
  RunScalars rs = apiScalars(c);
  if (setApiTime(c, 0.0)) return 1;
  launchPrims(c, b, b.v.q, false);
  Tile* slot = kernel == BK_GRAD ? &b.tGrad : (kernel == BK_DISS ? &b.tDiss : &b.tRhs);
  const Tile saved = *slot;
  // the batched kernels have one lane per point
  const int savedLanes = b.gradLanes;
  b.gradLanes = 1;
  const long long savedLaunches = c.launches;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float bestMs = 1e30f;
  *best = saved;
  for (int k = 0; k < nCands; ++k) {
    *slot = makeTile(b, cands[k][0], cands[k][1], cands[k][2]);
    auto run = [&]() {
      if (kernel == BK_GRAD) launchGradFlux(c, b, true, false, &rs, 1, false);
      else if (kernel == BK_DISS) launchDissipation(c, b, b.v.q, 1.0);
      else launchForwardDivergence(c, b, 0, rs, true, false);
    };
    run();
    cudaEventRecord(e0, c.stream);
    for (int r = 0; r < 10; ++r) run();
    cudaEventRecord(e1, c.stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < bestMs) { bestMs = ms; *best = *slot; }
  }
  *slot = saved;
  b.gradLanes = savedLanes;
  c.launches = savedLaunches;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return checkLaunch(c);
}

}  // namespace mgd

// Patch setup of block bi (updatePatchFactories and the patch setup routines,
// src/PatchFactoryImpl.f90:161-574): patches on other blocks are skipped.
// mollifierTotals holds the control and target mollifier quadratures over all
// blocks (normalizeControlMollifier / normalizeTargetMollifier,
// src/RegionImpl.f90:459-603, sum over every block).
// Solenoidal-excitation entries of block bi (setupSolenoidalExcitationPatch,
// src/SolenoidalExcitationPatchImpl.f90:93-130): the non-hole points of each
// patch with its strength amplitude exp(-g |x - x0|^2), g = 9 / (2 radius^2),
// the offsets from the origin and the spatial functions of every mode, and a
// dense map from grid point to entry.
static int setupExcitation(Context& c, int bi, const std::vector<int>& exts) {
  DevBlock& b = c.blocks[bi];
  const long long N = b.v.N;
  const int* gs = b.v.gs;
  std::vector<int> idx;
  struct HostPatch {
    ExcPatch x;
    size_t pi;
    std::vector<double> S, dx, dy, cache;
    std::vector<int> pts;
  };
  std::vector<HostPatch> hs;
  int total = 0;
  for (size_t pi = 0; pi < c.patches.size(); ++pi) {
    const mgd_patch_desc& p = c.patches[pi];
    if (p.type != MGD_PATCH_SOLENOIDAL_EXCITATION || p.grid_index != bi + 1 || p.n_modes <= 0) continue;
    if (idx.empty()) idx.assign(N, -1);
    HostPatch h;
    h.pi = pi;
    const int nM = p.n_modes;
    const double g = 9.0 / (2.0 * p.radius * p.radius);
    const std::vector<double>& w = c.patchOmega[pi];
    const std::vector<double>& ph = c.patchPhases[pi];
    bool overlap = false;
    forExtent(&exts[6 * pi], gs, [&](long long gi, long long) {
      if (b.hostIblank[gi] == 0) return;
      if (idx[gi] >= 0) {
        overlap = true;
        return;
      }
      idx[gi] = total + (int)h.pts.size();
      h.pts.push_back((int)gi);
      const double dx = b.hostCoords[gi] - p.origin[0], dy = b.hostCoords[N + gi] - p.origin[1];
      h.dx.push_back(dx);
      h.dy.push_back(dy);
      h.S.push_back(p.amplitude * std::exp(-g * (dx * dx + dy * dy)));
    });
    if (overlap) return fail(c, "overlapping solenoidal-excitation patches are not supported");
    const long long nE = (long long)h.pts.size();
    h.cache.assign((size_t)4 * nM * nE, 0.0);
    for (long long e = 0; e < nE; ++e)
      for (int l = 0; l < nM; ++l) {
        const double a = w[l] * h.dx[e] + ph[l], d = w[l] * h.dy[e] + ph[nM + l];
        h.cache[e + nE * l] = std::sin(a);
        h.cache[e + nE * (nM + l)] = std::cos(a);
        h.cache[e + nE * (2 * nM + l)] = std::sin(d);
        h.cache[e + nE * (3 * nM + l)] = std::cos(d);
      }
    h.x.nE = (int)nE;
    h.x.off = total;
    h.x.nModes = nM;
    h.x.g = g;
    h.x.speed[0] = p.velocity[0];
    h.x.speed[1] = p.velocity[1];
    total += (int)nE;
    hs.push_back(std::move(h));
  }
  b.exc.clear();
  if (hs.empty()) return 0;
  int* dIdx = nullptr;
  double* dF = nullptr;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (x != cudaSuccess) e = x; };
  chk(devAlloc(b, &dIdx, N));
  chk(devAlloc(b, &dF, 3LL * total));
  for (HostPatch& h : hs) {
    double *w, *S, *dx, *dy, *cache;
    int* pts;
    const long long nE = h.x.nE;
    chk(devAlloc(b, &w, h.x.nModes));
    chk(devAlloc(b, &S, nE));
    chk(devAlloc(b, &dx, nE));
    chk(devAlloc(b, &dy, nE));
    chk(devAlloc(b, &cache, 4LL * h.x.nModes * nE));
    chk(devAlloc(b, &pts, nE));
    if (e != cudaSuccess) break;
    chk(cudaMemcpy(w, c.patchOmega[h.pi].data(), h.x.nModes * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(S, h.S.data(), nE * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(dx, h.dx.data(), nE * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(dy, h.dy.data(), nE * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(cache, h.cache.data(), h.cache.size() * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(pts, h.pts.data(), nE * sizeof(int), cudaMemcpyHostToDevice));
    h.x.omega = w; h.x.S = S; h.x.dx = dx; h.x.dy = dy; h.x.cache = cache; h.x.point = pts;
    b.exc.push_back(h.x);
  }
  if (e == cudaSuccess) e = cudaMemcpy(dIdx, idx.data(), N * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(c, std::string("solenoidal-excitation setup failed: ") + cudaGetErrorString(e));
  b.v.excIdx = dIdx;
  b.v.excF = dF;
  return 0;
}

static int finalizeBlock(Context& c, int bi, const double* mollifierTotals) {
  DevBlock& b = c.blocks[bi];
  const int nD = c.nD, nU = c.nU;
  const long long N = b.v.N;
  const int* gs = b.v.gs;
  std::vector<int> exts;
  for (const mgd_patch_desc& p : c.patches) {
    int e[6];
    if (p.grid_index != bi + 1) {
      exts.insert(exts.end(), 6, 0);  // keeps exts aligned with c.patches
      continue;
    }
    resolveExtent(p, gs, nD, e);
    for (int i = 0; i < nD; ++i)
      if (e[2 * i] < 1 || e[2 * i + 1] > gs[i] || e[2 * i] > e[2 * i + 1])
        return fail(c, std::string("patch '") + p.name + "' has an invalid extent");
    const bool satType = p.type == MGD_PATCH_SAT_FAR_FIELD || p.type == MGD_PATCH_SLIP_WALL ||
                         p.type == MGD_PATCH_ISOTHERMAL_WALL || p.type == MGD_PATCH_ADIABATIC_WALL ||
                         p.type == MGD_PATCH_BLOCK_INTERFACE;
    if (satType || p.type == MGD_PATCH_SPONGE) {
      const int d = std::abs(p.normal_direction);
      if (d < 1 || d > nD) return fail(c, std::string("patch '") + p.name + "' has an invalid normal direction");
      if (satType && e[2 * (d - 1)] != e[2 * (d - 1) + 1])
        return fail(c, std::string("patch '") + p.name + "' extends more than 1 grid point along its normal direction");
    }
    exts.insert(exts.end(), e, e + 6);
  }
  if (setupExcitation(c, bi, exts)) return 1;
  // sponge strengths (computeSpongeStrengths, src/PatchFactoryImpl.f90:161-374)
  std::vector<double> sponge(N, 0.0);
  for (size_t pi = 0; pi < c.patches.size(); ++pi) {
    const mgd_patch_desc& p = c.patches[pi];
    if (p.type != MGD_PATCH_SPONGE || p.grid_index != bi + 1) continue;
    const int* e = &exts[6 * pi];
    const int dir = std::abs(p.normal_direction) - 1;
    const long long st = b.v.ax[dir].stride;
    const int lo = e[2 * dir], hi = e[2 * dir + 1];
    std::vector<double> strength;
    forExtent(e, gs, [&](long long gi, long long) {
      const int i = (int)((gi / st) % gs[dir]) + 1;
      const long long line0 = gi - (long long)(i - 1) * st;
      auto curve = [&](int i1) {
        double s = 0.0;
        for (int x = 0; x < nD; ++x) {
          const double v = b.hostJmi[(size_t)N * (nD * dir + x) + line0 + (long long)(i1 - 1) * st];
          s += v * v;
        }
        return std::sqrt(s);
      };
      double num = 0.0, den = 0.0;
      if (p.normal_direction > 0) {
        for (int t = lo; t <= i - 1; ++t) num += curve(t);
        for (int t = lo; t <= hi - 1; ++t) den += curve(t);
      } else {
        for (int t = i + 1; t <= hi; ++t) num += curve(t);
        for (int t = lo + 1; t <= hi; ++t) den += curve(t);
      }
      const double s = num / den;
      strength.push_back(p.sponge_amount * std::pow(1.0 - s, (double)p.sponge_exponent));
    });
    size_t k = 0;
    forExtent(e, gs, [&](long long gi, long long) {
      if (b.hostIblank[gi] != 0) sponge[gi] += strength[k];
      ++k;
    });
  }
  // masks, actuator indices, cost-target counts, far-field entries
  std::vector<double> maskT(N, 0.0), maskA(N, 0.0), tgt(N, 0.0);
  std::vector<int> actIdx(N, -1), ffOf(3 * N, -1);
  std::vector<int> ffPoint, ffDir, ffSigned, ffKind;
  std::vector<double> ffSigInv, ffSigV, ffSigVRaw, ffWallInv, ffWallVisc, ffWallT;
  std::vector<double> qtH;  // target state on the host (isothermal wall temperatures)
  const HostOp d1 = schemeOps(c.opts.discretization_scheme).d1;
  long long actOffset = 0;
  for (size_t pi = 0; pi < c.patches.size(); ++pi) {
    const mgd_patch_desc& p = c.patches[pi];
    if (p.grid_index != bi + 1) continue;
    const int* e = &exts[6 * pi];
    if (p.type == MGD_PATCH_ACTUATOR && bi > 0)
      return fail(c, std::string("actuator patch '") + p.name + "' must lie in block 1");
    switch (p.type) {
      case MGD_PATCH_COST_TARGET:
        forExtent(e, gs, [&](long long gi, long long) {
          maskT[gi] = 1.0;
          if (b.hostIblank[gi] != 0) tgt[gi] += 1.0;
        });
        break;
      case MGD_PATCH_ACTUATOR: {
        bool overlap = false;
        forExtent(e, gs, [&](long long gi, long long k) {
          maskA[gi] = 1.0;
          if (actIdx[gi] >= 0) overlap = true;
          actIdx[gi] = (int)(actOffset + k);
        });
        if (overlap) return fail(c, "overlapping actuator patches are not supported");
        actOffset += (long long)(e[1] - e[0] + 1) * (e[3] - e[2] + 1) * (e[5] - e[4] + 1);
        break;
      }
      case MGD_PATCH_SAT_FAR_FIELD: {
        // src/FarFieldPatchImpl.f90:53-74
        const int dir = std::abs(p.normal_direction);
        const double nb = d1.norm[0];
        const double sInv = std::copysign(p.inviscid_penalty_amount, (double)p.normal_direction) / nb;
        const double sVis = c.opts.viscous ? std::copysign(p.viscous_penalty_amount, (double)p.normal_direction) / nb : 0.0;
        bool full = false;
        forExtent(e, gs, [&](long long gi, long long) {
          if (b.hostIblank[gi] == 0) return;
          int slot = 0;
          while (slot < 3 && ffOf[3 * gi + slot] >= 0) ++slot;
          if (slot == 3) { full = true; return; }
          ffOf[3 * gi + slot] = (int)ffPoint.size();
          ffPoint.push_back((int)gi);
          ffDir.push_back(dir);
          ffSigned.push_back(p.normal_direction);
          ffSigInv.push_back(sInv);
          ffSigVRaw.push_back(sVis);
          ffSigV.push_back(sVis);  // times 1/det below
          ffKind.push_back(SAT_FAR_FIELD);
          ffWallInv.push_back(0.0);
          ffWallVisc.push_back(0.0);
          ffWallT.push_back(0.0);
        });
        if (full) return fail(c, "more than three SAT patches meet at one point");
        break;
      }
      case MGD_PATCH_SLIP_WALL:
      case MGD_PATCH_ISOTHERMAL_WALL:
      case MGD_PATCH_ADIABATIC_WALL: {
        // src/ImpenetrableWallImpl.f90:3-40, src/IsothermalWallImpl.f90:3-80
        const int dir = std::abs(p.normal_direction);
        const double nb = d1.norm[0];
        const double sInv = std::copysign(p.inviscid_penalty_amount, (double)p.normal_direction) / nb;
        const bool iso = p.type == MGD_PATCH_ISOTHERMAL_WALL;
        const double sVis = (iso && c.opts.viscous) ? p.viscous_penalty_amount / nb * c.phys.reInv : 0.0;
        if (iso && p.wall_temperature <= 0.0 && qtH.empty()) {
          qtH.resize((size_t)N * nU);
          CUDA_TRY(c, cudaMemcpy(qtH.data(), b.v.qt, qtH.size() * sizeof(double), cudaMemcpyDeviceToHost));
        }
        bool full = false;
        forExtent(e, gs, [&](long long gi, long long) {
          if (b.hostIblank[gi] == 0) return;
          int slot = 0;
          while (slot < 3 && ffOf[3 * gi + slot] >= 0) ++slot;
          if (slot == 3) { full = true; return; }
          ffOf[3 * gi + slot] = (int)ffPoint.size();
          ffPoint.push_back((int)gi);
          ffDir.push_back(dir);
          ffSigned.push_back(p.normal_direction);
          ffSigInv.push_back(0.0);
          ffSigVRaw.push_back(0.0);
          ffSigV.push_back(0.0);
          ffKind.push_back(iso ? SAT_ISOTHERMAL_WALL : SAT_WALL);
          ffWallInv.push_back(sInv);   // times 1/det below
          ffWallVisc.push_back(sVis);  // times 1/det below
          double Tw = p.wall_temperature;
          if (iso && Tw <= 0.0) {
            // temperature of the target state (src/PatchFactoryImpl.f90:512-538)
            const double g = c.phys.g;
            const double v = 1.0 / qtH[gi];
            double u2 = 0.0;
            for (int d = 0; d < nD; ++d) {
              const double u = v * qtH[(size_t)N * (d + 1) + gi];
              u2 += u * u;
            }
            const double pr = (g - 1.0) * (qtH[(size_t)N * (nD + 1) + gi] - 0.5 * qtH[gi] * u2);
            Tw = g * pr / (g - 1.0) * v;
          }
          ffWallT.push_back(Tw);
        });
        if (full) return fail(c, "more than three SAT patches meet at one point");
        break;
      }
      case MGD_PATCH_BLOCK_INTERFACE: {
        // setupBlockInterfacePatch, src/BlockInterfacePatchImpl.f90:3-88; the
        // partner side is filled in by resolveInterfaces
        const int dir = std::abs(p.normal_direction);
        const double nb = d1.norm[0];
        const double sInv = std::copysign(p.inviscid_penalty_amount, (double)p.normal_direction) / nb;
        const double sVis = c.opts.viscous ? std::copysign(p.viscous_penalty_amount, (double)p.normal_direction) / nb : 0.0;
        std::vector<int>& table = c.ifacePointEntry[pi];
        table.assign((size_t)(e[1] - e[0] + 1) * (e[3] - e[2] + 1) * (e[5] - e[4] + 1), -1);
        bool full = false;
        forExtent(e, gs, [&](long long gi, long long k) {
          if (b.hostIblank[gi] == 0) return;
          int slot = 0;
          while (slot < 3 && ffOf[3 * gi + slot] >= 0) ++slot;
          if (slot == 3) { full = true; return; }
          table[k] = (int)ffPoint.size();
          ffOf[3 * gi + slot] = (int)ffPoint.size();
          ffPoint.push_back((int)gi);
          ffDir.push_back(dir);
          ffSigned.push_back(p.normal_direction);
          ffSigInv.push_back(0.0);
          ffSigVRaw.push_back(0.0);
          ffSigV.push_back(0.0);
          ffKind.push_back(SAT_INTERFACE);
          ffWallInv.push_back(sInv);   // the own inviscid penalty, kept unscaled
          ffWallVisc.push_back(sVis);  // the own viscous penalty, kept unscaled
          ffWallT.push_back(0.0);
        });
        if (full) return fail(c, "more than three SAT patches meet at one point");
        break;
      }
      default:
        break;
    }
  }
  if (bi == 0) c.actuatorPoints = actOffset;
  std::vector<int> actPts((size_t)std::max(1LL, actOffset), 0);
  for (long long p = 0; p < N; ++p)
    if (actIdx[p] >= 0) actPts[actIdx[p]] = (int)p;
  for (long long p = 0; p < N; ++p)
    if (b.hostIblank[p] == 0) { maskT[p] = 0.0; maskA[p] = 0.0; }
  // mollifier normalization (src/RegionImpl.f90:459-603, L1 norm)
  std::vector<double> mcH(N), mtH(N);
  CUDA_TRY(c, cudaMemcpy(mcH.data(), b.v.mc, N * sizeof(double), cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(mtH.data(), b.v.mt, N * sizeof(double), cudaMemcpyDeviceToHost));
  if (c.opts.enable_controller && mollifierTotals[0] != 0.0)
    for (long long p = 0; p < N; ++p) mcH[p] = mcH[p] / mollifierTotals[0];
  if (c.opts.enable_functional && mollifierTotals[1] != 0.0)
    for (long long p = 0; p < N; ++p) mtH[p] = mtH[p] / mollifierTotals[1];
  std::vector<double> wT(N), wA(N);
  for (long long p = 0; p < N; ++p) {
    wT[p] = maskT[p] * b.hostNorm[p];
    wA[p] = maskA[p] * b.hostNorm[p];
  }
  if (bi == 0) {
    c.actuatorWeights.assign((size_t)actOffset, 0.0);
    for (long long k = 0; k < actOffset; ++k) c.actuatorWeights[k] = wA[actPts[k]];
  }
  // acoustic source Gaussians exp(-9/(2 R^2) |x - x0|^2) (src/AcousticSourceImpl.f90:34-64)
  std::vector<double> srcG((size_t)N * std::max<size_t>(1, c.sources.size()), 0.0);
  for (size_t s = 0; s < c.sources.size(); ++s) {
    const mgd_acoustic_source& src = c.sources[s];
    const double gf = 9.0 / (2.0 * src.radius * src.radius);
    for (long long p = 0; p < N; ++p) {
      if (b.hostIblank[p] == 0) continue;
      double r = 0.0;
      for (int d = 0; d < nD; ++d) {
        const double x = b.hostCoords[(size_t)N * d + p] - src.location[d];
        r += x * x;
      }
      srcG[(size_t)N * s + p] = std::exp(-gf * r);
    }
  }
  BlockView& v = b.v;
  v.nSources = (int)c.sources.size();
  std::vector<int> tgtPts;
  for (long long p = 0; p < N; ++p)
    if (wT[p] != 0.0) tgtPts.push_back((int)p);
  {
    int* dT = nullptr;
    int* dA = nullptr;
    if (devAlloc(b, &dT, std::max<size_t>(1, tgtPts.size())) != cudaSuccess ||
        devAlloc(b, &dA, actPts.size()) != cudaSuccess)
      return fail(c, "device allocation failed for patch point lists");
    if (!tgtPts.empty())
      CUDA_TRY(c, cudaMemcpy(dT, tgtPts.data(), tgtPts.size() * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(dA, actPts.data(), actPts.size() * sizeof(int), cudaMemcpyHostToDevice));
    v.tgtPts = dT;
    v.nTgt = (int)tgtPts.size();
    v.actPts = dA;
    v.nAct = (int)actOffset;
  }
  CUDA_TRY(c, cudaMemcpy((void*)v.sponge, sponge.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy((void*)v.mc, mcH.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy((void*)v.mt, mtH.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy((void*)v.wT, wT.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy((void*)v.wA, wA.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy((void*)v.tgtCount, tgt.data(), N * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy((void*)v.actIdx, actIdx.data(), N * sizeof(int), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy((void*)v.ffOfPoint, ffOf.data(), 3 * N * sizeof(int), cudaMemcpyHostToDevice));
  if (!c.sources.empty())
    CUDA_TRY(c, cudaMemcpy((void*)v.srcG, srcG.data(), srcG.size() * sizeof(double), cudaMemcpyHostToDevice));
  // far-field entries
  const int nFF = (int)ffPoint.size();
  FarFieldEntries& ff = v.ff;
  ff.n = nFF;
  if (nFF > 0) {
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (x != cudaSuccess) e = x; };
    chk(devAlloc(b, &ff.point, nFF));
    chk(devAlloc(b, &ff.normalDir, nFF));
    chk(devAlloc(b, &ff.M, (size_t)nFF * nU * nU));
    chk(devAlloc(b, &ff.sigV, nFF));
    chk(devAlloc(b, &ff.sigVRaw, nFF));
    chk(devAlloc(b, &ff.visc, (size_t)nFF * nU));
    chk(devAlloc(b, &ff.viscT, (size_t)nFF * nU));
    chk(devAlloc(b, &ff.kind, nFF));
    chk(devAlloc(b, &ff.wallInv, nFF));
    chk(devAlloc(b, &ff.wallVisc, nFF));
    chk(devAlloc(b, &ff.wallT, nFF));
    chk(devAlloc(b, &ff.partnerBlock, nFF));
    chk(devAlloc(b, &ff.partnerPoint, nFF));
    chk(devAlloc(b, &ff.partnerEntry, nFF));
    chk(devAlloc(b, &ff.dirL, nFF));
    chk(devAlloc(b, &ff.dirR, nFF));
    chk(devAlloc(b, &ff.metricsR, (size_t)nFF * nD));
    chk(devAlloc(b, &ff.ifInv, (size_t)nFF * 2));
    chk(devAlloc(b, &ff.ifVis, (size_t)nFF * 2));
    chk(devAlloc(b, &ff.ifVisc, (size_t)nFF * nU));
    chk(devAlloc(b, &ff.ifAd, (size_t)nFF * nD * (nU - 1)));
    double* dSig = nullptr;
    int* dSigned = nullptr;
    chk(devAlloc(b, &dSig, nFF));
    chk(devAlloc(b, &dSigned, nFF));
    if (e != cudaSuccess) return fail(c, "device allocation failed for far-field entries");
    std::vector<double> jacH(N);
    CUDA_TRY(c, cudaMemcpy(jacH.data(), v.jac, N * sizeof(double), cudaMemcpyDeviceToHost));
    b.nInterfaceEntries = 0;
    b.hostIfaceInv.assign((size_t)nFF, 0.0);
    b.hostIfaceVis.assign((size_t)nFF, 0.0);
    for (int k = 0; k < nFF; ++k) {
      if (ffKind[k] == SAT_INTERFACE) {
        ++b.nInterfaceEntries;
        b.hostIfaceInv[k] = ffWallInv[k];
        b.hostIfaceVis[k] = ffWallVisc[k];
        ffWallInv[k] = ffWallVisc[k] = 0.0;
        continue;
      }
      ffSigV[k] = ffSigV[k] * jacH[ffPoint[k]];
      ffWallInv[k] = ffWallInv[k] * jacH[ffPoint[k]];
      ffWallVisc[k] = ffWallVisc[k] * jacH[ffPoint[k]];
    }
    b.hostFfPoint = ffPoint;
    b.hostFfSigned = ffSigned;
    if (b.nInterfaceEntries > 0) {
      std::vector<int> ifList;
      for (int k = 0; k < nFF; ++k)
        if (ffKind[k] == SAT_INTERFACE) ifList.push_back(k);
      chk(devAlloc(b, &ff.ifList, ifList.size()));
      if (e != cudaSuccess) return fail(c, "device allocation failed for the interface entries");
      CUDA_TRY(c, cudaMemcpy(ff.ifList, ifList.data(), ifList.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    CUDA_TRY(c, cudaMemcpy(ff.kind, ffKind.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.wallInv, ffWallInv.data(), nFF * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.wallVisc, ffWallVisc.data(), nFF * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.wallT, ffWallT.data(), nFF * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.point, ffPoint.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.normalDir, ffDir.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.sigV, ffSigV.data(), nFF * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.sigVRaw, ffSigVRaw.data(), nFF * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(dSig, ffSigInv.data(), nFF * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(dSigned, ffSigned.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    launchFarFieldMatricesWith(c, b, dSig, dSigned);
    if (c.opts.viscous) {
      // target viscous fluxes: primitives and stress of the target state
      launchPrims(c, b, v.qt, false);
      double* qSave = v.q;
      v.q = (double*)v.qt;
      launchGradFlux(c, b, false, true, nullptr, 0, false);
      v.q = qSave;
      launchFarFieldTargetVisc(c, b);
    }
    if (checkLaunch(c)) return 1;
    CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  }
  return 0;
}

// Point correspondence of an interface patch and its conforming patch
// (readPatchInterfaceInformation, src/InterfaceHelperImpl.f90:3-113, and the
// reordering of reshapeReceivedData, src/BlockInterfacePatchImpl.f90:785-931):
// the partner patch-local index of each patch point, or an error.
static int interfaceMap(Context& c, const int* ext, const int* extQ, const int reorder[3],
                        std::vector<long long>& out) {
  const long long g0 = ext[1] - ext[0] + 1, g1 = ext[3] - ext[2] + 1, g2 = ext[5] - ext[4] + 1;
  const long long q0 = extQ[1] - extQ[0] + 1, q1 = extQ[3] - extQ[2] + 1, q2 = extQ[5] - extQ[4] + 1;
  int o[3] = {reorder[0], reorder[1], reorder[2]};
  if (o[2] != 3) return fail(c, "interface index reordering of the third index is not supported");
  const bool transpose = std::abs(o[0]) == 2 && std::abs(o[1]) == 1;
  if (transpose) std::swap(o[0], o[1]);
  out.assign((size_t)(g0 * g1 * g2), 0);
  for (long long k = 1; k <= g2; ++k)
    for (long long j = 1; j <= g1; ++j)
      for (long long i = 1; i <= g0; ++i) {
        const long long fi = o[0] == -1 ? g0 + 1 - i : i;
        const long long fj = o[1] == -2 ? g1 + 1 - j : j;
        const long long a = transpose ? fj : fi, b = transpose ? fi : fj;
        if (a < 1 || a > q0 || b < 1 || b > q1 || k > q2) return fail(c, "block interface patches do not conform");
        out[(size_t)((i - 1) + g0 * ((j - 1) + g1 * (k - 1)))] = (a - 1) + q0 * ((b - 1) + q1 * (k - 1));
      }
  return 0;
}

// Partners of the block-interface entries of every block: conforming point,
// its entry, the partner's normal metric row, penalties and normal direction
// (the METRICS exchange of collectInterfaceData, src/BlockInterfacePatchImpl.f90:598-720).
static int resolveInterfaces(Context& c) {
  const int nP = (int)c.patches.size(), nD = c.nD;
  std::vector<int> partner(nP, -1);
  std::vector<std::array<int, 3>> reorder(nP, std::array<int, 3>{1, 2, 3});
  for (int i = 0; i < nP; ++i) {
    const mgd_patch_desc& p = c.patches[i];
    if (p.type != MGD_PATCH_BLOCK_INTERFACE || p.conforms_with[0] == 0) continue;
    for (int k = 0; k < nP; ++k)
      if (std::strncmp(c.patches[k].name, p.conforms_with, MGD_NAME_LEN) == 0) partner[i] = k;
    if (partner[i] < 0 || c.patches[partner[i]].type != MGD_PATCH_BLOCK_INTERFACE)
      return fail(c, std::string("invalid interface specification for patch '") + p.name + "'");
    for (int d = 0; d < 3; ++d) reorder[i][d] = p.interface_index[d] != 0 ? p.interface_index[d] : d + 1;
  }
  for (int i = 0; i < nP; ++i) {
    if (partner[i] < 0) continue;
    const int j = partner[i];
    if (partner[j] < 0) {
      partner[j] = i;
      for (int l = 1; l <= 3; ++l)
        for (int k = 1; k <= 3; ++k)
          if (std::abs(reorder[i][k - 1]) == l) {
            reorder[j][l - 1] = reorder[i][k - 1] < 0 ? -k : k;
            break;
          }
    } else if (partner[j] != i) {
      return fail(c, std::string("interface specification of patch '") + c.patches[j].name + "' violates commutativity");
    }
  }
  // host metrics of every block
  std::vector<std::vector<double>> metrics(c.blocks.size());
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    const long long N = c.blocks[bi].v.N;
    metrics[bi].resize((size_t)N * nD * nD);
    CUDA_TRY(c, cudaMemcpy(metrics[bi].data(), c.blocks[bi].v.metrics, metrics[bi].size() * sizeof(double),
                           cudaMemcpyDeviceToHost));
  }
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    DevBlock& b = c.blocks[bi];
    const int nFF = b.v.ff.n;
    if (b.nInterfaceEntries == 0) continue;
    std::vector<int> pBlock(nFF, 0), pPoint(nFF, 0), pEntry(nFF, 0), dirL(nFF, 0), dirR(nFF, 0);
    std::vector<double> mR((size_t)nFF * nD, 0.0), inv((size_t)nFF * 2, 0.0), vis((size_t)nFF * 2, 0.0);
    for (int i = 0; i < nP; ++i) {
      const mgd_patch_desc& p = c.patches[i];
      if (p.type != MGD_PATCH_BLOCK_INTERFACE || p.grid_index != (int)bi + 1) continue;
      if (partner[i] < 0) return fail(c, std::string("block interface patch '") + p.name + "' has no conforming patch");
      const mgd_patch_desc& q = c.patches[partner[i]];
      const int qb = q.grid_index - 1;
      DevBlock& bq = c.blocks[qb];
      int ext[6], extQ[6];
      resolveExtent(p, b.v.gs, nD, ext);
      resolveExtent(q, bq.v.gs, nD, extQ);
      std::vector<long long> map;
      if (interfaceMap(c, ext, extQ, reorder[i].data(), map)) return 1;
      const std::vector<int>& mine = c.ifacePointEntry[i];
      const std::vector<int>& theirs = c.ifacePointEntry[partner[i]];
      const long long q0 = extQ[1] - extQ[0] + 1, q1 = extQ[3] - extQ[2] + 1;
      const int qdir = std::abs(q.normal_direction);
      for (size_t k = 0; k < mine.size(); ++k) {
        const int e = mine[k];
        if (e < 0) continue;
        const long long qk = map[k];
        const int qe = theirs[(size_t)qk];
        if (qe < 0) return fail(c, std::string("block interface '") + p.name + "' meets a hole of its partner");
        const long long qi = qk % q0, qj = (qk / q0) % q1, qkk = qk / (q0 * q1);
        const long long qgi = (extQ[0] - 1 + qi) + (long long)bq.v.gs[0] * ((extQ[2] - 1 + qj) +
                              (long long)bq.v.gs[1] * (extQ[4] - 1 + qkk));
        pBlock[e] = qb;
        pPoint[e] = (int)qgi;
        pEntry[e] = qe;
        dirL[e] = p.normal_direction;
        dirR[e] = q.normal_direction;
        for (int d = 0; d < nD; ++d)
          mR[(size_t)e * nD + d] = metrics[qb][(size_t)bq.v.N * (nD * (qdir - 1) + d) + qgi];
        inv[2 * e] = b.hostIfaceInv[e];
        inv[2 * e + 1] = bq.hostIfaceInv[qe];
        vis[2 * e] = b.hostIfaceVis[e];
        vis[2 * e + 1] = bq.hostIfaceVis[qe];
      }
    }
    FarFieldEntries& ff = b.v.ff;
    CUDA_TRY(c, cudaMemcpy(ff.partnerBlock, pBlock.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.partnerPoint, pPoint.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.partnerEntry, pEntry.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.dirL, dirL.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.dirR, dirR.data(), nFF * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.metricsR, mR.data(), mR.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.ifInv, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(ff.ifVis, vis.data(), vis.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  c.hasInterfaces = false;
  for (const DevBlock& b : c.blocks) c.hasInterfaces = c.hasInterfaces || b.nInterfaceEntries > 0;
  return 0;
}

// Control and target mollifier quadratures over every block (the sums that
// normalizeControlMollifier / normalizeTargetMollifier reduce,
// src/RegionImpl.f90:459-603).
static int mollifierTotals(Context& c, double* totals) {
  totals[0] = totals[1] = 0.0;
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    DevBlock& b = c.blocks[bi];
    const long long N = b.v.N;
    std::vector<double> maskA(N, 0.0), maskT(N, 0.0), mc(N), mt(N);
    for (const mgd_patch_desc& p : c.patches) {
      if (p.grid_index != (int)bi + 1) continue;
      if (p.type != MGD_PATCH_ACTUATOR && p.type != MGD_PATCH_COST_TARGET) continue;
      int e[6];
      resolveExtent(p, b.v.gs, c.nD, e);
      forExtent(e, b.v.gs, [&](long long gi, long long) {
        (p.type == MGD_PATCH_ACTUATOR ? maskA : maskT)[gi] = 1.0;
      });
    }
    CUDA_TRY(c, cudaMemcpy(mc.data(), b.v.mc, N * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(c, cudaMemcpy(mt.data(), b.v.mt, N * sizeof(double), cudaMemcpyDeviceToHost));
    for (long long p = 0; p < N; ++p) {
      if (b.hostIblank[p] == 0) continue;
      totals[0] += maskA[p] * b.hostNorm[p] * mc[p];
      totals[1] += maskT[p] * b.hostNorm[p] * mt[p];
    }
  }
  return 0;
}

int mgd_finalize_setup(mgd_ctx* h) {
  Context& c = h->c;
  if (c.finalized) return 0;
  if (c.blocks.empty()) return fail(c, "no block");
  for (const mgd_patch_desc& p : c.patches)
    if (p.grid_index < 1 || p.grid_index > (int)c.blocks.size())
      return fail(c, std::string("patch '") + p.name + "' refers to a missing block");
  c.ifacePointEntry.assign(c.patches.size(), std::vector<int>());
  double totals[2];
  if (mollifierTotals(c, totals)) return 1;
  for (int bi = 0; bi < (int)c.blocks.size(); ++bi)
    if (finalizeBlock(c, bi, totals)) return 1;
  if (resolveInterfaces(c)) return 1;
  c.finalized = true;
  for (DevBlock& b : c.blocks)
    if (autotune(c, b)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

static RunScalars apiScalars(Context& c) {
  RunScalars r{};
  r.step = c.dCounters + 2;
  r.segBase = c.dCounters + 3;
  r.amp = c.dApiAmp;
  r.stageTime = c.dApiTime;
  r.apiForcing = c.apiForcingSet ? c.dApiForcing : nullptr;
  setStepSize(r, c.opts.time_step_size);
  r.adjointForcingSwitch = c.opts.adjoint_forcing_switch;
  r.nPartialBlocks = reductionBlocks(c.blocks[0]);
  return r;
}

static int setApiTime(Context& c, double time) {
  double amp[MGD_MAX_SOURCES] = {0};
  const double pi = 4.0 * std::atan(1.0);
  for (size_t s = 0; s < c.sources.size(); ++s) {
    const mgd_acoustic_source& src = c.sources[s];
    amp[s] = src.amplitude * std::cos(2.0 * pi * src.frequency * time + src.phase);
  }
  CUDA_TRY(c, cudaMemcpyAsync(c.dApiAmp, amp, sizeof amp, cudaMemcpyHostToDevice, c.stream));
  // pageable source: the copy completes before the call returns
  CUDA_TRY(c, cudaMemcpyAsync(c.dApiTime, &time, sizeof time, cudaMemcpyHostToDevice, c.stream));
  return 0;
}

// The per-call forward RHS adds the actuators' forcing when the caller set one
// (ActuatorPatch%updateRhs, src/ActuatorPatchImpl.f90:108-181).
static bool apiController(const Context& c) {
  return c.apiForcingSet && c.opts.enable_controller && c.opts.controller_switch;
}

static int requireReady(Context& c) {
  if (!c.finalized) return fail(c, "mgd_finalize_setup has not been called");
  return 0;
}

namespace mgd {

// One forward RK stage (rkStage 1..4) or the forward RHS alone (rkStage 0).
// The dissipation kernel runs on the side stream beside the flux kernel; both
// only read q and join before the divergence kernel updates it.
void forwardStage(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, bool api, bool controller, bool store,
                  bool functional, const Lanes* lanes) {
  const Lanes L = lanes ? *lanes : Lanes{c.stream, c.side, c.evFork[0], c.evJoin[0]};
  const int stage = api ? 1 : rkStage;
  const bool diss = c.phys.dissipation != 0, exc = !b.exc.empty();
  if (diss || exc) {
    cudaEventRecord(L.fork, L.main);
    cudaStreamWaitEvent(L.side, L.fork, 0);
    if (diss) launchDissipation(c, b, b.v.q, 1.0, L.side);
    if (exc) launchExcitation(c, b, rs, stage, false, false, L.side);
    cudaEventRecord(L.join, L.side);
  }
  launchGradFlux(c, b, true, false, &rs, stage, store, L.main);
  if (diss || exc) cudaStreamWaitEvent(L.main, L.join, 0);
  launchForwardDivergence(c, b, rkStage, rs, api, controller, L.main);
  if (rkStage > 0) launchPrims(c, b, b.v.q, false, nullptr, 0, L.main);
  if (functional) {
    if ((diss || exc) && rkStage >= 1 && rkStage <= 3) {
      // beside the next stage's flux kernel: that stage's side work queues
      // behind it and its join comes before that stage's primitives replace
      // these and before the step counter advances
      cudaEventRecord(L.fork, L.main);
      cudaStreamWaitEvent(L.side, L.fork, 0);
      launchFunctional(c, b, rs, stage, L.side);
    } else {
      launchFunctional(c, b, rs, stage, L.main);
    }
  }
}

// One adjoint RK stage (rkStage 4..1) or the adjoint RHS alone (rkStage 0).
// The wall and far-field SAT vectors, the adjoint dissipation and, when
// recording, the gradient/sensitivity kernel read lambda on the side stream
// beside the core and diffusion kernels; all join before the assembly
// kernel updates lambda.
void adjointStage(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, int stage, double apiFactor, bool api,
                  bool fromSlot, bool record, const Lanes* lanes) {
  const Lanes L = lanes ? *lanes : Lanes{c.stream, c.side, c.evFork[1], c.evJoin[1]};
  const bool exc = !b.exc.empty();
  const bool sat = b.v.ff.n > b.nInterfaceEntries;
  const bool side = c.phys.dissipation != 0 || record || exc || sat;
  if (side) {
    cudaEventRecord(L.fork, L.main);
    cudaStreamWaitEvent(L.side, L.fork, 0);
    if (sat) launchAdjointSatVectors(c, b, rs, stage, fromSlot, L.side);
    if (c.phys.dissipation) launchDissipation(c, b, b.v.lam, -1.0, L.side);
    if (record) launchGradientSensitivity(c, b, rs, stage, L.side);
    if (exc) launchExcitation(c, b, rs, stage, true, fromSlot, L.side);
    cudaEventRecord(L.join, L.side);
  }
  launchAdjointCore(c, b, rs, stage, fromSlot, L.main);
  launchAdjointDiffusion(c, b, L.main);
  if (side) cudaStreamWaitEvent(L.main, L.join, 0);
  launchAdjointAssemble(c, b, rkStage, rs, stage, apiFactor, api, fromSlot, L.main);
}

// Arrays of every block for the interface kernels.
static BlockRefs blockRefs(Context& c) {
  BlockRefs r{};
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    r.q[bi] = c.blocks[bi].v.q;
    r.lam[bi] = c.blocks[bi].v.lam;
    r.ifVisc[bi] = c.blocks[bi].v.ff.ifVisc;
    r.N[bi] = c.blocks[bi].v.N;
  }
  return r;
}

// The forward RHS (rkStage 0) or one forward RK stage of every block of a
// multi-block region: all blocks' fluxes first, then the block-interface SATs
// (which read the partner blocks), then the divergence and update of each block.
void regionForwardStage(Context& c, int rkStage, const RunScalars& rs) {
  const BlockRefs refs = blockRefs(c);
  for (DevBlock& b : c.blocks) {
    launchDissipation(c, b, b.v.q, 1.0);
    launchGradFlux(c, b, true, false, &rs, 1, false);
    launchExcitation(c, b, rs, 1, false, false);
  }
  for (DevBlock& b : c.blocks) launchInterfaceSat(c, b, refs);
  for (DevBlock& b : c.blocks) {
    // actuator patches lie in block 1
    launchForwardDivergence(c, b, rkStage, rs, true, apiController(c) && &b == &c.blocks[0]);
    if (rkStage > 0) launchPrims(c, b, b.v.q, false);
  }
}

// The adjoint RHS or one adjoint RK stage of every block (primitives and
// stress of the forward state are current): interface SATs of every block
// first, which also read the partner blocks' lambda before any update.
void regionAdjointStage(Context& c, int rkStage, const RunScalars& rs, double apiFactor) {
  const BlockRefs refs = blockRefs(c);
  for (DevBlock& b : c.blocks) launchInterfaceSatAdjoint(c, b, refs);
  for (DevBlock& b : c.blocks) {
    launchDissipation(c, b, b.v.lam, -1.0);
    launchExcitation(c, b, rs, 1, true, false);
    launchAdjointCore(c, b, rs, 1, false);
    launchAdjointSatVectors(c, b, rs, 1, false);
    launchAdjointDiffusion(c, b);
  }
  for (DevBlock& b : c.blocks) launchAdjointAssemble(c, b, rkStage, rs, 1, apiFactor, true, false);
}

}  // namespace mgd

static bool singleBlock(const Context& c) { return c.blocks.size() == 1 && !c.hasInterfaces; }

namespace mgd {
bool perCallController(const Context& c) { return apiController(c); }
const double* perCallForcing(const Context& c) { return c.apiForcingSet ? c.dApiForcing : nullptr; }
bool singleBlockRegion(const Context& c) { return singleBlock(c); }
}  // namespace mgd

int mgd_update_state(mgd_ctx* h) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  for (DevBlock& b : c.blocks) {
    launchPrims(c, b, b.v.q, false);
    if (c.phys.viscous) launchGradFlux(c, b, false, true, nullptr, 0, false);
  }
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

int mgd_check_solution_limits(mgd_ctx* h, int* within) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (!within) return fail(c, "mgd_check_solution_limits: within must not be null");
  if (!c.opts.enable_solution_limits) return fail(c, "mgd_check_solution_limits: enable_solution_limits is off");
  CUDA_TRY(c, cudaMemsetAsync(c.dLimitKey, 0xFF, sizeof(unsigned long long), c.stream));
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) launchSolutionLimits(c, c.blocks[bi], (int)bi, nullptr, 1, c.dLimitKey);
  if (checkLaunch(c)) return 1;
  double v = 0.0;
  const int st = limitOutcome(c, &v, true);
  if (st != 0 && st != MGD_SOLUTION_LIMITS) return st;
  *within = st == 0;
  return 0;
}

// The linearized RHS covers every patch type but the solenoidal excitation,
// which the reference does not linearize either.
static int refuseLinearized(Context& c) {
  for (const mgd_patch_desc& p : c.patches)
    if (p.type == MGD_PATCH_SOLENOIDAL_EXCITATION)
      // addSolenoidalExcitation has no LINEARIZED branch (src/SolenoidalExcitationPatchImpl.f90:192)
      return fail(c, "the linearized RHS does not take solenoidal-excitation patches");
  return 0;
}

// The linearized RHS (rkStage 0) or one linearized RK stage of every block:
// the perturbation in lambda about the current conserved state. The fluxes of
// every block come first, then the interface SATs (which read the partner
// blocks' perturbations and linearized viscous fluxes), then the divergence
// and update of each block.
static void linearizedStages(Context& c, int rkStage, const RunScalars& rs, double factor) {
  for (DevBlock& x : c.blocks) {
    launchPrims(c, x, x.v.q, false);
    if (c.phys.viscous) launchGradFlux(c, x, false, true, &rs, 1, false);
    if (c.phys.dissipation) launchDissipation(c, x, x.v.lam, 1.0);
    launchLinearizedFlux(c, x, rs, 1, false);
  }
  const BlockRefs refs = blockRefs(c);
  for (DevBlock& x : c.blocks) launchInterfaceSatLinearized(c, x, refs);
  for (DevBlock& x : c.blocks) launchLinearizedDivergence(c, x, rkStage, rs, factor, 1, false);
}

int mgd_compute_rhs(mgd_ctx* h, int mode, double time, double adjoint_forcing_factor) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  DevBlock& b = c.blocks[0];
  RunScalars rs = apiScalars(c);
  if (mode == MGD_FORWARD) {
    if (setApiTime(c, time)) return 1;
    for (DevBlock& x : c.blocks) launchPrims(c, x, x.v.q, false);
    if (singleBlock(c)) forwardStage(c, b, 0, rs, true, apiController(c), false, false);
    else regionForwardStage(c, 0, rs);
  } else if (mode == MGD_ADJOINT) {
    if (setApiTime(c, time)) return 1;
    for (DevBlock& x : c.blocks) {
      launchPrims(c, x, x.v.q, false);
      if (c.phys.viscous) launchGradFlux(c, x, false, true, &rs, 1, false);
    }
    if (singleBlock(c)) adjointStage(c, b, 0, rs, 1, adjoint_forcing_factor, true, false, false);
    else regionAdjointStage(c, 0, rs, adjoint_forcing_factor);
  } else if (mode == MGD_LINEARIZED) {
    if (refuseLinearized(c)) return 1;
    linearizedStages(c, 0, rs, adjoint_forcing_factor);
  } else {
    return fail(c, "mode must be MGD_FORWARD, MGD_ADJOINT or MGD_LINEARIZED");
  }
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

int mgd_update_adjoint_forcing(mgd_ctx* h, int no_adjoint_forcing) {
  // Stores the cost-target adjoint forcing of the current forward state for
  // the per-call RHS (inside runs it is evaluated in the adjoint kernel).
  Context& c = h->c;
  if (requireReady(c)) return 1;
  for (DevBlock& b : c.blocks) {
    launchPrims(c, b, b.v.q, false);
    launchStoreAdjointForcing(c, b, no_adjoint_forcing != 0);
  }
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

static int reduceToHost(Context& c, int nSlots, std::vector<double>& out) {
  const int nb = reductionBlocks(c.blocks[0]);
  if (c.stageValueCapacity < nSlots) {
    cudaFree(c.dStageValues);
    CUDA_TRY(c, cudaMalloc((void**)&c.dStageValues, (size_t)std::max(1, nSlots) * sizeof(double)));
    c.stageValueCapacity = nSlots;
  }
  launchReducePartials(c, c.dPartials, nb, nb, nSlots, c.dStageValues);
  out.resize(nSlots);
  if (nSlots > 0)
    CUDA_TRY(c, cudaMemcpyAsync(out.data(), c.dStageValues, (size_t)nSlots * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return checkLaunch(c);
}

static int ensurePartials(Context& c, long long nSlots) {
  const long long need = nSlots * reductionBlocks(c.blocks[0]);
  if (c.partialCapacity < need) {
    cudaFree(c.dPartials);
    CUDA_TRY(c, cudaMalloc((void**)&c.dPartials, (size_t)std::max(1LL, need) * sizeof(double)));
    c.partialCapacity = need;
  }
  return 0;
}

int mgd_compute_functional(mgd_ctx* h, double* value) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  double s = 0.0;
  for (DevBlock& b : c.blocks) {
    const long long N = b.v.N;
    std::vector<double> w(N), mt(N), mp(N), pr(N);
    CUDA_TRY(c, cudaMemcpy(w.data(), b.v.wT, N * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(c, cudaMemcpy(mt.data(), b.v.mt, N * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(c, cudaMemcpy(mp.data(), b.v.meanP, N * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(c, cudaMemcpy(pr.data(), b.v.prim + N * PrimLayout{c.nD}.p(), N * sizeof(double),
                           cudaMemcpyDeviceToHost));
    for (long long p = 0; p < N; ++p) {
      const double F = pr[p] - mp[p];
      s += w[p] * (F * F * mt[p]);
    }
  }
  *value = s;
  return 0;
}

int mgd_compute_sensitivity(mgd_ctx* h, double* value) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  DevBlock& b = c.blocks[0];
  const long long N = b.v.N;
  std::vector<double> w(N), mc(N), lam(N);
  CUDA_TRY(c, cudaMemcpy(w.data(), b.v.wA, N * sizeof(double), cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(mc.data(), b.v.mc, N * sizeof(double), cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(lam.data(), b.v.lam + N * (c.nD + 1), N * sizeof(double), cudaMemcpyDeviceToHost));
  double s = 0.0;
  for (long long p = 0; p < N; ++p) {
    const double F = lam[p] * mc[p];
    s += w[p] * (F * F);
  }
  *value = s;
  return 0;
}

int mgd_rk4_substep(mgd_ctx* h, int mode, double* time, double dt, int stage) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (stage < 1 || stage > 4) return fail(c, "stage must be 1..4");
  DevBlock& b = c.blocks[0];
  RunScalars rs = apiScalars(c);
  setStepSize(rs, dt);
  if (mode == MGD_FORWARD) {
    if (stage == 2 || stage == 4) *time = *time + dt / 2.0;
    if (setApiTime(c, *time)) return 1;
    for (DevBlock& x : c.blocks) launchPrims(c, x, x.v.q, false);
    if (singleBlock(c)) forwardStage(c, b, stage, rs, true, apiController(c), false, false);
    else regionForwardStage(c, stage, rs);
  } else if (mode == MGD_ADJOINT) {
    const double factor = stage == 4 ? 2.0 : (stage == 2 ? 0.5 : 1.0);
    // time of the matching forward stage: stages 4 and 2 run at the current
    // time, stages 3 and 1 half a step earlier
    if (setApiTime(c, (stage == 3 || stage == 1) ? *time - dt / 2.0 : *time)) return 1;
    for (DevBlock& x : c.blocks) {
      launchPrims(c, x, x.v.q, false);
      if (c.phys.viscous) launchGradFlux(c, x, false, true, &rs, 1, false);
    }
    if (singleBlock(c)) adjointStage(c, b, stage, rs, 1, factor, true, false, false);
    else regionAdjointStage(c, stage, rs, factor);
    if (stage == 3 || stage == 1) *time = *time - dt / 2.0;
  } else if (mode == MGD_LINEARIZED) {
    // substepLinearizedRK4 (src/RK4IntegratorImpl.f90:272-380): the perturbation
    // in lambda advances about the conserved state held, which stays fixed
    if (refuseLinearized(c)) return 1;
    if (stage == 2 || stage == 4) *time = *time + dt / 2.0;
    linearizedStages(c, stage, rs, 1.0);
  } else {
    return fail(c, "mode must be MGD_FORWARD, MGD_ADJOINT or MGD_LINEARIZED");
  }
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

int mgd_actuator_patch_size(mgd_ctx* h, long long* n) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  *n = c.actuatorPoints;
  return 0;
}

int mgd_set_control_forcing(mgd_ctx* h, const double* host, long long n_entries) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  c.nForcingEntries = 0;
  const long long n = std::max(0LL, n_entries) * c.actuatorPoints;
  if (n == 0) {
    cudaFree(c.dForcing);
    c.dForcing = nullptr;
    c.forcingCapacity = 0;
    return 0;
  }
  if (c.forcingCapacity < n) {
    cudaFree(c.dForcing);
    c.dForcing = nullptr;
    c.forcingCapacity = 0;
    CUDA_TRY(c, cudaMalloc((void**)&c.dForcing, (size_t)n * sizeof(double)));
    c.forcingCapacity = n;
  }
  CUDA_TRY(c, cudaMemcpyAsync(c.dForcing, host, (size_t)n * sizeof(double), cudaMemcpyDefault, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  c.nForcingEntries = n_entries;
  return 0;
}

int mgd_actuator_weights(mgd_ctx* h, double* out) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (c.actuatorWeights.empty()) return 0;
  CUDA_TRY(c, cudaMemcpyAsync(out, c.actuatorWeights.data(), c.actuatorWeights.size() * sizeof(double),
                              cudaMemcpyDefault, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

static const double kRkNorm[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};

static RunScalars runScalars(Context& c) {
  RunScalars r{};
  r.step = c.dCounters + 0;
  r.segBase = c.dCounters + 1;
  r.amp = c.dAmp;
  r.forcing = c.dForcing;
  r.nForcingEntries = c.nForcingEntries;
  r.nSteps = c.runSteps;
  r.P = c.actuatorPoints;
  r.gradient = c.dGradient;
  r.partials = c.dPartials;
  r.nPartialBlocks = reductionBlocks(c.blocks[0]);
  r.stageBuf = c.dStageBuf;
  r.slotStride = c.slotStride;
  r.slotFull = c.slotFull;
  r.rk = c.dStepDt;
  r.stageTime = c.dStageTime;
  setStepSize(r, c.opts.time_step_size);
  r.adjointForcingSwitch = c.opts.adjoint_forcing_switch;
  return r;
}

static int setCounters(Context& c, int step, int segBase) {
  const int v[2] = {step, segBase};
  CUDA_TRY(c, cudaMemcpyAsync(c.dCounters, v, sizeof v, cudaMemcpyHostToDevice, c.stream));
  return 0;
}

// Captures `body` into an executable graph on stream s (the context stream
// when 0). The kernels recorded during capture are counted per graph launch
// instead.
template <class F>
static int capture(Context& c, cudaGraphExec_t* exec, long long* nodes, F body, cudaStream_t s = 0) {
  if (!s) s = c.stream;
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  cudaGraph_t g = nullptr;
  const long long before = c.launches;
  CUDA_TRY(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  body();
  CUDA_TRY(c, cudaStreamEndCapture(s, &g));
  *nodes = c.launches - before;
  c.launches = before;
  CUDA_TRY(c, cudaGraphInstantiate(exec, g, 0));
  cudaGraphDestroy(g);
  return 0;
}

// Per-step step sizes of a run, the constant-CFL reduction scratch and the
// device copy of the run time.
static int ensureStepBuffers(Context& c, DevBlock& b, int nSteps) {
  if (c.stepDtCapacity < 4LL * nSteps) {
    cudaFree(c.dStepDt);
    c.dStepDt = nullptr;
    CUDA_TRY(c, cudaMalloc((void**)&c.dStepDt, (size_t)4 * nSteps * sizeof(double)));
    c.stepDtCapacity = 4LL * nSteps;
  }
  // partial minima of every block (a region's step size is the minimum over its blocks)
  int nb = 0;
  for (DevBlock& x : c.blocks) nb += timeStepBlocks(x);
  (void)b;
  if (c.dtPartialCapacity < nb) {
    cudaFree(c.dDtPartials);
    c.dDtPartials = nullptr;
    CUDA_TRY(c, cudaMalloc((void**)&c.dDtPartials, (size_t)nb * sizeof(double)));
    c.dtPartialCapacity = nb;
  }
  if (!c.dTime) CUDA_TRY(c, cudaMalloc((void**)&c.dTime, sizeof(double)));
  return 0;
}

// Stage buffer of one checkpoint segment: 4*S slots. A slot holds the stage's
// input state q and, when memory allows, also its primitive variables, stress
// and heat flux, so the adjoint stages read them instead of recomputing them.
static int ensureStageBuffer(Context& c, DevBlock& b, int S) {
  c.trajectorySteps = 0;  // the slots are about to hold recomputed segments
  const long long N = b.v.N;
  const int nD = c.nD, nU = c.nU;
  const long long qOnly = (long long)nU * N;
  const long long full = (long long)(nU + PrimLayout{nD}.count() + nD * nD + nD) * N;
  // preference: two halves of full slots (recomputation beside the adjoint),
  // one half of full slots, one half of q-only slots
  const long long options[3][3] = {{2, full, 4LL * S * full}, {1, full, 4LL * S * full}, {1, qOnly, 4LL * S * qOnly}};
  size_t freeB = 0, totalB = 0;
  CUDA_TRY(c, cudaMemGetInfo(&freeB, &totalB));
  const double budget = 0.5 * ((double)freeB + (double)c.stageBufCapacity * sizeof(double));
  int pick = 2;
  for (int k = N <= MGD_TWO_LANE_MAX_POINTS ? 0 : 1; k < 3; ++k)
    if ((double)(options[k][0] * options[k][2]) * sizeof(double) <= budget) {
      pick = k;
      break;
    }
  const long long need = options[pick][0] * options[pick][2];
  if (c.stageBufCapacity < need) {
    cudaFree(c.dStageBuf);
    c.dStageBuf = nullptr;
    c.stageBufCapacity = 0;
    CUDA_TRY(c, cudaMalloc((void**)&c.dStageBuf, (size_t)need * sizeof(double)));
    c.stageBufCapacity = need;
  }
  c.stageHalves = (int)options[pick][0];
  c.stageHalf = options[pick][2];
  c.slotStride = options[pick][1];
  c.slotFull = options[pick][1] == full ? 1 : 0;
  return 0;
}

// Stage buffer for a resident trajectory of T steps: 4 T full slots when they
// fit the budget (*resident = true), else nothing changes (*resident = false).
static int ensureTrajectoryBuffer(Context& c, DevBlock& b, int T, bool* resident) {
  *resident = false;
  c.trajectorySteps = 0;
  const long long N = b.v.N;
  const long long full = (long long)(c.nU + PrimLayout{c.nD}.count() + c.nD * c.nD + c.nD) * N;
  const long long need = 4LL * T * full;
  size_t freeB = 0, totalB = 0;
  CUDA_TRY(c, cudaMemGetInfo(&freeB, &totalB));
  const double budget = c.trajectoryMaxBytes > 0.0
                            ? c.trajectoryMaxBytes
                            : 0.5 * ((double)freeB + (double)c.stageBufCapacity * sizeof(double));
  if ((double)need * sizeof(double) > budget) return 0;
  if (c.stageBufCapacity < need) {
    cudaFree(c.dStageBuf);
    c.dStageBuf = nullptr;
    c.stageBufCapacity = 0;
    if (cudaMalloc((void**)&c.dStageBuf, (size_t)need * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();  // out of memory: fall back to checkpoints
      return 0;
    }
    c.stageBufCapacity = need;
  }
  c.stageHalves = 1;
  c.stageHalf = need;
  c.slotStride = full;
  c.slotFull = 1;
  *resident = true;
  return 0;
}

// Forward work arrays of the recomputation that runs beside the adjoint: its
// own state, primitives, fluxes, dissipation, RK buffers and SAT vectors over
// the block's grid and patch data.
static int ensureShadow(Context& c, DevBlock& b) {
  if (c.shadowReady) return 0;
  const long long N = b.v.N;
  const int nD = c.nD, nU = c.nU;
  BlockView v = b.v;
  auto alloc = [&](double** p, long long n) -> cudaError_t {
    cudaError_t e = cudaMalloc((void**)p, (size_t)std::max(1LL, n) * sizeof(double));
    if (e == cudaSuccess) c.shadowAllocations.push_back(*p);
    return e;
  };
  double* ffv = nullptr;
  cudaError_t e = cudaSuccess;
  long long nExc = 0;
  for (const ExcPatch& X : b.exc) nExc += X.nE;
  for (auto x : {alloc(&v.q, N * nU), alloc(&v.prim, N * PrimLayout{nD}.count()), alloc(&v.fhat, N * nD * nU),
                 alloc(&v.dq, N * nD * nU), alloc(&v.b1, N * nU), alloc(&v.b2, N * nU),
                 alloc(&ffv, (long long)v.ff.n * nU), alloc(&v.excF, 3 * nExc)})
    if (x != cudaSuccess) e = x;
  if (e != cudaSuccess) return fail(c, std::string("device allocation failed for the recomputation: ") +
                                           cudaGetErrorString(e));
  v.ff.visc = ffv;
  c.shadow = v;
  c.shadowReady = true;
  return 0;
}

namespace mgd {

// Run buffers and per-stage tables of a forward run of n_steps steps from t0:
// step sizes, source amplitudes, functional partials, gradient entries and,
// with snapshots, the checkpoint snapshots. Leaves the primitives of the
// initial state current.
int prepareForwardRun(Context& c, int n_steps, int save_interval, double t0, bool snapshots) {
  DevBlock& b = c.blocks[0];
  const long long N = b.v.N;
  const int nU = c.nU;
  const bool cflMode = c.opts.use_constant_cfl != 0;
  const double dt = c.opts.time_step_size;
  if (!cflMode && !(dt > 0.0)) return fail(c, "time_step_size must be positive");
  if (cflMode && !(c.opts.cfl > 0.0)) return fail(c, "cfl must be positive in constant-CFL mode");
  c.runSteps = n_steps;
  c.saveInterval = save_interval;
  c.runT0 = t0;
  c.limitViolated = false;
  if (c.opts.enable_solution_limits)
    CUDA_TRY(c, cudaMemsetAsync(c.dLimitKey, 0xFF, sizeof(unsigned long long), c.stream));
  if (ensureStepBuffers(c, b, n_steps)) return 1;
  const int nSrc = (int)c.sources.size();
  const long long nAmp = (long long)4 * n_steps * std::max(1, nSrc);
  if (c.ampCapacity < nAmp) {
    cudaFree(c.dAmp);
    CUDA_TRY(c, cudaMalloc((void**)&c.dAmp, nAmp * sizeof(double)));
    c.ampCapacity = nAmp;
  }
  if (c.stageTimeCapacity < 4LL * n_steps) {
    cudaFree(c.dStageTime);
    c.dStageTime = nullptr;
    c.stageTimeCapacity = 0;
    CUDA_TRY(c, cudaMalloc((void**)&c.dStageTime, (size_t)4 * n_steps * sizeof(double)));
    c.stageTimeCapacity = 4LL * n_steps;
  }
  if (cflMode) {
    // step sizes, stage times and source amplitudes are produced on the device
    CUDA_TRY(c, cudaMemcpyAsync(c.dTime, &t0, sizeof(double), cudaMemcpyHostToDevice, c.stream));
  } else {
    // stage times as Solver%runForward accumulates them (src/RK4IntegratorImpl.f90:95-140)
    c.stageTimes.assign((size_t)4 * n_steps, 0.0);
    double t = t0;
    for (int s = 0; s < n_steps; ++s)
      for (int i = 1; i <= 4; ++i) {
        if (i == 2 || i == 4) t = t + dt / 2.0;
        c.stageTimes[(size_t)4 * s + i - 1] = t;
      }
    c.stepDt.assign(n_steps, dt);
    std::vector<double> rk((size_t)4 * n_steps);
    for (int s = 0; s < n_steps; ++s) {
      rk[4 * s] = dt;
      rk[4 * s + 1] = dt / 6.0;
      rk[4 * s + 2] = dt / 3.0;
      rk[4 * s + 3] = dt / 2.0;
    }
    CUDA_TRY(c, cudaMemcpy(c.dStepDt, rk.data(), rk.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<double> amp(nAmp, 0.0);
    const double pi = 4.0 * std::atan(1.0);
    for (long long k = 0; k < 4LL * n_steps; ++k)
      for (int s = 0; s < nSrc; ++s) {
        const mgd_acoustic_source& src = c.sources[s];
        amp[k * nSrc + s] = src.amplitude * std::cos(2.0 * pi * src.frequency * c.stageTimes[k] + src.phase);
      }
    CUDA_TRY(c, cudaMemcpy(c.dAmp, amp.data(), nAmp * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c.dStageTime, c.stageTimes.data(), c.stageTimes.size() * sizeof(double),
                           cudaMemcpyHostToDevice));
  }
  if (snapshots) {
    const long long nSnap = n_steps / save_interval + 2;
    if (c.snapshotCapacity < nSnap * nU * N) {
      cudaFree(c.dSnapshots);
      c.dSnapshots = nullptr;
      CUDA_TRY(c, cudaMalloc((void**)&c.dSnapshots, (size_t)nSnap * nU * N * sizeof(double)));
      c.snapshotCapacity = nSnap * nU * N;
    }
  }
  if (ensurePartials(c, 4LL * n_steps)) return 1;
  const long long nGrad = 4LL * n_steps * std::max(1LL, c.actuatorPoints);
  if (c.gradientCapacity < nGrad) {
    cudaFree(c.dGradient);
    CUDA_TRY(c, cudaMalloc((void**)&c.dGradient, nGrad * sizeof(double)));
    c.gradientCapacity = nGrad;
  }
  // state%update of the initial condition
  launchPrims(c, b, b.v.q, false);
  if (snapshots) launchSnapshot(c, b, c.dSnapshots, save_interval, true);
  return checkLaunch(c);
}

// Step sizes back to the host and J = sum over steps and stages of
// w_i dt_n J_{n,i} (src/SolverImpl.f90:836-841) from the stage partials.
int finishForwardRun(Context& c, double* cost) {
  const int n_steps = c.runSteps;
  if (c.opts.use_constant_cfl) {
    std::vector<double> rk((size_t)4 * n_steps);
    CUDA_TRY(c, cudaMemcpyAsync(rk.data(), c.dStepDt, rk.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                c.stream));
    CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    c.stepDt.resize(n_steps);
    for (int s = 0; s < n_steps; ++s) c.stepDt[s] = rk[4 * s];
  }
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  double J = 0.0;
  if (c.opts.enable_functional && c.opts.functional_type == MGD_FUNCTIONAL_TERMINAL_KINETIC_ENERGY) {
    DevBlock& b = c.blocks[0];
    if (!c.dNorm) {
      CUDA_TRY(c, cudaMalloc((void**)&c.dNorm, (size_t)b.v.N * sizeof(double)));
      CUDA_TRY(c, cudaMemcpy(c.dNorm, b.hostNorm.data(), (size_t)b.v.N * sizeof(double), cudaMemcpyHostToDevice));
    }
    launchKineticEnergy(c, b, c.dNorm, c.dDtPartials, c.dTime);
    if (checkLaunch(c)) return 1;
    CUDA_TRY(c, cudaMemcpyAsync(&J, c.dTime, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  } else if (c.opts.enable_functional) {
    std::vector<double> vals;
    if (reduceToHost(c, 4 * n_steps, vals)) return 1;
    for (int s = 0; s < n_steps; ++s)
      for (int i = 0; i < 4; ++i) J = J + kRkNorm[i] * c.stepDt[s] * vals[(size_t)4 * s + i];
  }
  *cost = J;
  return 0;
}

RunScalars runScalarsOf(Context& c) { return runScalars(c); }

// After a forward run with solution limits (or a per-call check): decodes the
// first violation, if any, into the reference's message
// (src/SolverImpl.f90:231-280), sets *value = HUGE and returns
// MGD_SOLUTION_LIMITS; 0 when the state stayed inside the limits.
int limitOutcome(Context& c, double* value, bool perCall) {
  if (!c.opts.enable_solution_limits) return 0;
  unsigned long long key = kNoLimitViolation;
  CUDA_TRY(c, cudaMemcpyAsync(&key, c.dLimitKey, sizeof key, cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (key == kNoLimitViolation) return 0;
  const long long ordinal = (long long)(key >> 36);
  const int bi = (int)((key >> 33) & 7), quantity = (int)((key >> 32) & 1);
  const long long p = (long long)(key & 0xffffffffULL);
  DevBlock& b = c.blocks[bi];
  const long long N = b.v.N;
  double v = 0.0;
  const double* src = quantity == 0 ? b.v.q + p : b.v.prim + p + N * (2 + c.nD);
  CUDA_TRY(c, cudaMemcpy(&v, src, sizeof v, cudaMemcpyDeviceToHost));
  const long long i = p % b.v.gs[0] + 1, j = (p / b.v.gs[0]) % b.v.gs[1] + 1, k = p / ((long long)b.v.gs[0] * b.v.gs[1]) + 1;
  const double lo = quantity == 0 ? c.opts.minimum_density : c.opts.minimum_temperature;
  const double hi = quantity == 0 ? c.opts.maximum_density : c.opts.maximum_temperature;
  char msg[320];
  std::snprintf(msg, sizeof msg, "%s on grid %d at (%lld, %lld, %lld): %.2E out of range (%.2E, %.2E)!",
                quantity == 0 ? "Density" : "Temperature", bi + 1, i, j, k, v, lo, hi);
  std::string text = msg;
  if (!perCall) {
    std::snprintf(msg, sizeof msg, " (forward step %lld, stage %lld)", ordinal / 4 + 1, ordinal % 4 + 1);
    text += msg;
  }
  c.limitMessage = text;
  c.error = text;
  *value = std::numeric_limits<double>::max();
  return MGD_SOLUTION_LIMITS;
}

}  // namespace mgd

// ---------------------------------------------------------------------------
// Checkpointed runs of multi-block regions (block interfaces): one stream, the
// stage kernels of every block per stage, interface SATs between the flux and
// divergence kernels, per-block snapshots, stage slots and partial sums.
// ---------------------------------------------------------------------------
static int growDevice(Context& c, double** p, long long* cap, long long need) {
  if (*cap >= need) return 0;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  CUDA_TRY(c, cudaMalloc((void**)p, (size_t)std::max(1LL, need) * sizeof(double)));
  *cap = need;
  return 0;
}

static RunScalars blockRunScalars(Context& c, DevBlock& b, bool first) {
  RunScalars r = runScalars(c);
  r.partials = b.runPartials;
  r.nPartialBlocks = reductionBlocks(b);
  r.stageBuf = b.runStage;
  if (!first) {
    // actuator patches lie in block 1
    r.forcing = nullptr;
    r.nForcingEntries = 0;
    r.P = 0;
  }
  return r;
}

static BlockRefs runRefs(Context& c) {
  BlockRefs r = blockRefs(c);
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    r.stage[bi] = c.blocks[bi].runStage;
    r.slotStride[bi] = c.slotStride;
  }
  return r;
}

// Per-stage values of every block summed over the blocks (block partial
// sums reduced in a fixed order, then the blocks in order).
static int reduceRegion(Context& c, int nSlots, std::vector<double>& out) {
  out.assign(nSlots, 0.0);
  if (c.stageValueCapacity < nSlots) {
    cudaFree(c.dStageValues);
    CUDA_TRY(c, cudaMalloc((void**)&c.dStageValues, (size_t)std::max(1, nSlots) * sizeof(double)));
    c.stageValueCapacity = nSlots;
  }
  std::vector<double> v(nSlots);
  for (DevBlock& b : c.blocks) {
    const int nb = reductionBlocks(b);
    launchReducePartials(c, b.runPartials, nb, nb, nSlots, c.dStageValues);
    CUDA_TRY(c, cudaMemcpyAsync(v.data(), c.dStageValues, (size_t)nSlots * sizeof(double), cudaMemcpyDeviceToHost,
                                c.stream));
    CUDA_TRY(c, cudaStreamSynchronize(c.stream));
    for (int k = 0; k < nSlots; ++k) out[k] += v[k];
  }
  return checkLaunch(c);
}

// One forward RK stage of every block; store writes the stage slots.
// Streams of the blocks of a region, two sets (the adjoint lane and the
// recomputation lane of a checkpointed adjoint run), created once per context
// (outside any capture).
static int ensureBlockStreams(Context& c) {
  if (c.evBlockFork) return 0;
  for (size_t bi = 0; bi < c.blocks.size() && bi < MGD_MAX_BLOCKS; ++bi) {
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c.blockStreams[bi], cudaStreamNonBlocking));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c.evBlockJoin[bi], cudaEventDisableTiming));
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c.blockStreams2[bi], cudaStreamNonBlocking));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c.evBlockJoin2[bi], cudaEventDisableTiming));
  }
  CUDA_TRY(c, cudaEventCreateWithFlags(&c.evBlockFork2, cudaEventDisableTiming));
  CUDA_TRY(c, cudaEventCreateWithFlags(&c.evBlockFork, cudaEventDisableTiming));
  return 0;
}

// The streams and events one lane of a region run issues on: its main
// stream, a side stream for the dissipation and excitation branch, and one
// stream per block.
struct RegionLanes {
  cudaStream_t main, side;
  cudaEvent_t fork, join;
  cudaStream_t* blockStreams;
  cudaEvent_t blockFork;
  cudaEvent_t* blockJoin;
};

static RegionLanes mainRegionLanes(Context& c) {
  return {c.stream, c.side, c.evFork[0], c.evJoin[0], c.blockStreams, c.evBlockFork, c.evBlockJoin};
}

// The same work for every block of a region, each block on its own stream,
// forked from the lane's main stream and joined back into it (inside a
// capture the block streams become parallel branches of the graph). A
// block's stage kernels read and write only that block's arrays, so they may
// overlap; the interface kernels, which read the partner blocks, run between
// a join and the next fork.
template <class F>
static void forEachBlockConcurrently(Context& c, const RegionLanes& L, F f) {
  const int n = (int)c.blocks.size();
  if (n == 1 || !L.blockFork) {
    for (int bi = 0; bi < n; ++bi) f(bi, L.main);
    return;
  }
  cudaEventRecord(L.blockFork, L.main);
  for (int bi = 0; bi < n; ++bi) {
    cudaStreamWaitEvent(L.blockStreams[bi], L.blockFork, 0);
    f(bi, L.blockStreams[bi]);
    cudaEventRecord(L.blockJoin[bi], L.blockStreams[bi]);
  }
  for (int bi = 0; bi < n; ++bi) cudaStreamWaitEvent(L.main, L.blockJoin[bi], 0);
}

template <class F>
static void forEachBlockConcurrently(Context& c, F f) {
  forEachBlockConcurrently(c, mainRegionLanes(c), f);
}

// One forward RK stage of every block of a region on lane L: the blocks'
// views in `blocks` (the context's blocks, or the recomputation lane's
// shadows), their run scalars, and the references the interface SATs read
// the partner blocks through.
static void regionRunStage(Context& c, std::vector<DevBlock*>& blocks, std::vector<RunScalars>& rs, int i,
                           bool controller, bool store, bool functional, const RegionLanes& L,
                           const BlockRefs& refs) {
  // dissipation and excitation of every block on the side stream beside the
  // flux and interface kernels; both only read the state of the stage
  cudaEventRecord(L.fork, L.main);
  cudaStreamWaitEvent(L.side, L.fork, 0);
  for (size_t bi = 0; bi < blocks.size(); ++bi) {
    DevBlock& b = *blocks[bi];
    if (c.phys.dissipation) launchDissipation(c, b, b.v.q, 1.0, L.side);
    launchExcitation(c, b, rs[bi], i, false, false, L.side);
  }
  cudaEventRecord(L.join, L.side);
  forEachBlockConcurrently(c, L, [&](int bi, cudaStream_t s) {
    launchGradFlux(c, *blocks[bi], true, false, &rs[bi], i, store, s);
  });
  // the interface SATs read the partner blocks' fluxes: after the join
  forEachBlockConcurrently(c, L, [&](int bi, cudaStream_t s) { launchInterfaceSat(c, *blocks[bi], refs, s); });
  cudaStreamWaitEvent(L.main, L.join, 0);
  forEachBlockConcurrently(c, L, [&](int bi, cudaStream_t s) {
    DevBlock& b = *blocks[bi];
    launchForwardDivergence(c, b, i, rs[bi], false, controller && bi == 0, s);
    launchPrims(c, b, b.v.q, false, nullptr, 0, s);
    if (functional) launchFunctional(c, b, rs[bi], i, s);
  });
}

static void regionRunStage(Context& c, std::vector<RunScalars>& rs, int i, bool controller, bool store,
                           bool functional) {
  std::vector<DevBlock*> blocks;
  for (DevBlock& b : c.blocks) blocks.push_back(&b);
  regionRunStage(c, blocks, rs, i, controller, store, functional, mainRegionLanes(c), blockRefs(c));
}

static int regionRunForward(Context& c, int n_steps, int save_interval, double t0, double* cost) {
  if (c.opts.functional_type != MGD_FUNCTIONAL_SOUND) return fail(c, "multi-block runs use the SOUND functional");
  const bool cflMode = c.opts.use_constant_cfl != 0;
  if (prepareForwardRun(c, n_steps, save_interval, t0, false)) return 1;
  if (ensureBlockStreams(c)) return 1;
  const long long nSnap = n_steps / save_interval + 2;
  for (DevBlock& b : c.blocks) {
    if (growDevice(c, &b.runSnap, &b.runSnapCap, nSnap * c.nU * b.v.N)) return 1;
    if (growDevice(c, &b.runPartials, &b.runPartialCap, 4LL * n_steps * reductionBlocks(b))) return 1;
    launchPrims(c, b, b.v.q, false);
    launchSnapshot(c, b, b.runSnap, save_interval, true);
  }
  const bool controller = c.opts.enable_controller && c.opts.controller_switch && c.dForcing;
  const bool functional = c.opts.enable_functional != 0;
  // with a resident trajectory the flux kernels of every block also store
  // every stage's state, primitives, stress and heat flux (4 n_steps full
  // slots per block), which the adjoint and tangent runs then read instead
  // of recomputing checkpoint segments
  bool resident = false;
  c.trajectorySteps = 0;
  const long long fullPer = c.nU + PrimLayout{c.nD}.count() + c.nD * c.nD + c.nD;
  if (c.trajectoryStorage) {
    size_t freeB = 0, totalB = 0;
    CUDA_TRY(c, cudaMemGetInfo(&freeB, &totalB));
    long long pts = 0, held = 0;
    for (DevBlock& b : c.blocks) {
      pts += b.v.N;
      held += b.runStageCap;
    }
    const double need = 4.0 * n_steps * (double)(fullPer * pts) * sizeof(double);
    const double budget =
        c.trajectoryMaxBytes > 0.0 ? c.trajectoryMaxBytes : 0.5 * ((double)freeB + (double)held * sizeof(double));
    resident = need <= budget;
    if (resident)
      for (DevBlock& b : c.blocks)
        if (growDevice(c, &b.runStage, &b.runStageCap, 4LL * n_steps * fullPer * b.v.N)) return 1;
  }
  std::vector<RunScalars> rs;
  const bool limits = c.opts.enable_solution_limits != 0;
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    rs.push_back(blockRunScalars(c, c.blocks[bi], bi == 0));
    if (limits) rs.back().limitKey = c.dLimitKey;
    if (resident) {
      rs.back().slotFull = 1;
      rs.back().slotStride = fullPer * c.blocks[bi].v.N;
    }
  }
  if (resident) c.slotFull = 1;
  if (setCounters(c, 1, 0)) return 1;
  if (capture(c, &c.gForward, &c.nodesForward, [&]() {
        // constant CFL: the step size from every block's state at the start of the step
        if (cflMode) launchTimeStepRegion(c, c.dDtPartials, c.dStepDt, c.dCounters, c.dTime, c.dStageTime, c.dAmp);
        for (int i = 1; i <= 4; ++i) {
          // checkSolutionLimits over every block before every substep
          if (limits)
            for (size_t bi = 0; bi < c.blocks.size(); ++bi)
              launchSolutionLimits(c, c.blocks[bi], (int)bi, c.dCounters, i, c.dLimitKey);
          regionRunStage(c, rs, i, controller, resident, functional);
        }
        for (DevBlock& b : c.blocks) launchSnapshot(c, b, b.runSnap, save_interval, false);
        launchStepAdvance(c, 1);
      }))
    return 1;
  for (int s = 0; s < n_steps; ++s) CUDA_TRY(c, cudaGraphLaunch(c.gForward, c.stream));
  c.launches += (long long)n_steps * c.nodesForward;
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (cflMode) {
    // recorded step sizes for J and the adjoint
    std::vector<double> rk((size_t)4 * n_steps);
    CUDA_TRY(c, cudaMemcpy(rk.data(), c.dStepDt, rk.size() * sizeof(double), cudaMemcpyDeviceToHost));
    c.stepDt.resize(n_steps);
    for (int s = 0; s < n_steps; ++s) c.stepDt[s] = rk[4 * s];
  }
  double J = 0.0;
  if (functional) {
    std::vector<double> vals;
    if (reduceRegion(c, 4 * n_steps, vals)) return 1;
    for (int s = 0; s < n_steps; ++s)
      for (int i = 0; i < 4; ++i) J = J + kRkNorm[i] * c.stepDt[s] * vals[(size_t)4 * s + i];
  }
  *cost = J;
  c.trajectorySteps = resident ? n_steps : 0;
  if (const int st = limitOutcome(c, cost, false)) {
    c.limitViolated = st == MGD_SOLUTION_LIMITS;
    c.trajectorySteps = 0;
    return st;
  }
  return 0;
}

// The recomputation lane's forward work arrays of every block of a region
// (its own state, primitives, fluxes, dissipation, RK buffers, SAT vectors,
// interface fluxes and excitation values over the blocks' grid and patch
// data), allocated once.
static int ensureRegionShadow(Context& c) {
  if (c.regionShadow.size() == c.blocks.size()) return 0;
  c.regionShadow.clear();
  const int nD = c.nD, nU = c.nU;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](double** p, long long n) {
    const cudaError_t x = cudaMalloc((void**)p, (size_t)std::max(1LL, n) * sizeof(double));
    if (x == cudaSuccess) c.shadowAllocations.push_back(*p);
    else e = x;
  };
  for (DevBlock& b : c.blocks) {
    const long long N = b.v.N;
    BlockView v = b.v;
    long long nExc = 0;
    for (const ExcPatch& X : b.exc) nExc = std::max(nExc, (long long)X.off + X.nE);
    double *ffv = nullptr, *ifv = nullptr;
    alloc(&v.q, N * nU);
    alloc(&v.prim, N * PrimLayout{nD}.count());
    alloc(&v.fhat, N * nD * nU);
    alloc(&v.dq, N * nD * nU);
    alloc(&v.b1, N * nU);
    alloc(&v.b2, N * nU);
    alloc(&ffv, (long long)v.ff.n * nU);
    if (v.ff.ifVisc) alloc(&ifv, (long long)v.ff.n * nU);
    if (v.excF) alloc(&v.excF, 3 * nExc);
    if (e != cudaSuccess) {
      c.regionShadow.clear();
      return fail(c, std::string("device allocation failed for the recomputation: ") + cudaGetErrorString(e));
    }
    v.ff.visc = ffv;
    if (v.ff.ifVisc) v.ff.ifVisc = ifv;
    c.regionShadow.push_back(v);
  }
  return 0;
}

// Solver%runAdjoint over a multi-block region (UniformCheckpointer). With a
// resident trajectory one segment reads every stage from its slots. Else,
// when two halves of full stage slots and the recomputation lane's work
// arrays fit, segment k-1 is recomputed on the second lanes (own streams, own
// work arrays, own step counters, the other half of the slots, lowest launch
// priority) while the adjoint consumes segment k; otherwise the segments are
// recomputed in line.
static int regionRunAdjoint(Context& c, double* sensitivity) {
  if (ensureBlockStreams(c)) return 1;
  const int nU = c.nU, nD = c.nD, T = c.runSteps;
  // a resident trajectory of this run: one segment over all steps, every
  // stage read from its slot, no recomputation
  const bool resident = c.trajectorySteps == T;
  const int S = resident ? T : c.saveInterval;
  const double dtT = c.stepDt[T - 1];
  // stage slots: full (state, primitives, stress, heat flux) when they fit in
  // half the free memory, in two halves with the second lane when those fit
  size_t freeB = 0, totalB = 0;
  CUDA_TRY(c, cudaMemGetInfo(&freeB, &totalB));
  long long pts = 0, held = 0, ffEntries = 0;
  for (DevBlock& b : c.blocks) {
    pts += b.v.N;
    held += b.runStageCap;
    ffEntries += b.v.ff.n;
  }
  const long long fullPer = nU + PrimLayout{nD}.count() + nD * nD + nD;
  const double budget = 0.5 * ((double)freeB + held * 8.0);
  const double shadowBytes = c.regionShadow.size() == c.blocks.size()
                                 ? 0.0
                                 : 8.0 * ((double)pts * (4 * nU + PrimLayout{nD}.count() + 2 * nD * nU) +
                                          2.0 * ffEntries * nU);
  const bool twoLanes = !resident && pts <= MGD_TWO_LANE_MAX_POINTS &&
                        (double)(2 * 4LL * S * fullPer * pts) * sizeof(double) + shadowBytes <= budget;
  const bool full = resident || twoLanes || (double)(4LL * S * fullPer * pts) * sizeof(double) <= budget;
  const int halves = twoLanes ? 2 : 1;
  std::vector<long long> halfSize(c.blocks.size());
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    DevBlock& b = c.blocks[bi];
    halfSize[bi] = 4LL * S * (full ? fullPer : nU) * b.v.N;
    if (growDevice(c, &b.runStage, &b.runStageCap, halves * halfSize[bi])) return 1;
  }
  if (twoLanes && ensureRegionShadow(c)) return 1;
  // the slot stride differs per block: the run scalars and the references carry each block's
  c.slotFull = full ? 1 : 0;
  const bool controller = c.opts.enable_controller && c.opts.controller_switch && c.dForcing;
  int* recCounters = twoLanes ? c.dCounters + 4 : c.dCounters;
  // run scalars and references of the adjoint lane (ra) and of the
  // recomputation (rr) for each half of the slots
  std::vector<RunScalars> ra[2], rr[2];
  BlockRefs aRefs[2];
  for (int h = 0; h < halves; ++h) {
    aRefs[h] = runRefs(c);
    for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
      DevBlock& b = c.blocks[bi];
      RunScalars r = blockRunScalars(c, b, bi == 0);
      r.slotFull = c.slotFull;
      r.slotStride = (full ? fullPer : nU) * b.v.N;
      r.stageBuf = b.runStage + h * halfSize[bi];
      ra[h].push_back(r);
      r.step = recCounters;
      r.segBase = recCounters + 1;
      rr[h].push_back(r);
      aRefs[h].stage[bi] = r.stageBuf;
      aRefs[h].slotStride[bi] = r.slotStride;
    }
  }
  // the blocks the recomputation runs on, and the references its interface
  // SATs read the partners through
  std::vector<DevBlock> shadowBlocks;
  std::vector<DevBlock*> recBlocks;
  BlockRefs recRefs = blockRefs(c);
  if (twoLanes) {
    shadowBlocks = c.blocks;
    for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
      shadowBlocks[bi].v = c.regionShadow[bi];
      recRefs.q[bi] = c.regionShadow[bi].q;
      recRefs.ifVisc[bi] = c.regionShadow[bi].ff.ifVisc;
    }
    for (DevBlock& b : shadowBlocks) recBlocks.push_back(&b);
  } else {
    for (DevBlock& b : c.blocks) recBlocks.push_back(&b);
  }
  const RegionLanes recLanes =
      twoLanes ? RegionLanes{c.stream2, c.side2, c.evFork[2], c.evJoin[2], c.blockStreams2, c.evBlockFork2,
                             c.evBlockJoin2}
               : mainRegionLanes(c);
  for (DevBlock& b : c.blocks) {
    launchPrims(c, b, b.v.q, false);
    launchAdjointInitial(c, b, c.opts.adjoint_forcing_switch ? -dtT / 6.0 : 0.0);
  }
  setProgrammaticLaunch(!twoLanes);
  struct Restore {
    ~Restore() {
      setProgrammaticLaunch(true);
      setLaunchPriority(false, 0);
    }
  } restore;
  // the adjoint is the critical path: the recomputation's kernels launch at
  // the lowest priority and take the SM time the adjoint leaves
  int prioLeast = 0, prioGreatest = 0;
  cudaDeviceGetStreamPriorityRange(&prioLeast, &prioGreatest);
  long long nodesRec = 0, nodesAdj = 0;
  for (int h = 0; h < halves; ++h) {
    if (twoLanes) setLaunchPriority(true, prioLeast);
    if (!resident && capture(c, &c.gRecomputeH[h], &nodesRec, [&]() {
          for (int i = 1; i <= 4; ++i)
            regionRunStage(c, recBlocks, rr[h], i, controller, true, false, recLanes, recRefs);
          launchStepAdvanceOn(recCounters, 1, recLanes.main);
        }, recLanes.main))
      return 1;
    if (twoLanes) setLaunchPriority(true, prioGreatest);
    std::vector<RunScalars>& rs = ra[h];
    const BlockRefs& refs = aRefs[h];
    if (capture(c, &c.gAdjointH[h], &nodesAdj, [&]() {
          for (int i = 4; i >= 1; --i) {
            if (!full)
              forEachBlockConcurrently(c, [&](int bi, cudaStream_t s) {
                DevBlock& b = c.blocks[bi];
                launchPrims(c, b, nullptr, true, &rs[bi], i, s);
                if (c.phys.viscous) launchGradFlux(c, b, false, true, &rs[bi], i, false, s);
              });
            // wall and far-field SAT vectors, dissipation, excitation and
            // gradient/sensitivity of every block on the side stream (they read
            // lambda and the forward state of the stage); interface SATs, then
            // the cores and diffusion, then the assembly, each block on its own
            // stream
            cudaEventRecord(c.evFork[1], c.stream);
            cudaStreamWaitEvent(c.side, c.evFork[1], 0);
            for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
              DevBlock& b = c.blocks[bi];
              launchAdjointSatVectors(c, b, rs[bi], i, full, c.side);
              if (c.phys.dissipation) launchDissipation(c, b, b.v.lam, -1.0, c.side);
              launchExcitation(c, b, rs[bi], i, true, full, c.side);
              launchGradientSensitivity(c, b, rs[bi], i, c.side);
            }
            cudaEventRecord(c.evJoin[1], c.side);
            forEachBlockConcurrently(c, [&](int bi, cudaStream_t s) {
              launchInterfaceSatAdjoint(c, c.blocks[bi], refs, &rs[bi], i, full, s);
            });
            forEachBlockConcurrently(c, [&](int bi, cudaStream_t s) {
              DevBlock& b = c.blocks[bi];
              launchAdjointCore(c, b, rs[bi], i, full, s);
              launchAdjointDiffusion(c, b, s);
            });
            cudaStreamWaitEvent(c.stream, c.evJoin[1], 0);
            forEachBlockConcurrently(c, [&](int bi, cudaStream_t s) {
              launchAdjointAssemble(c, c.blocks[bi], i, rs[bi], i, 0.0, false, full, s);
            });
          }
          launchStepAdvance(c, -1);
        }))
      return 1;
  }
  c.nodesRecompute = nodesRec;
  c.nodesAdjoint = nodesAdj;
  const int nSeg = (T + S - 1) / S;
  // UniformCheckpointer: reload the snapshots of segment k and recompute its stages
  auto recompute = [&](int k) -> int {
    const int L = k * S, end = std::min(T, L + S);
    const int h = k % halves;
    if (twoLanes) setLaunchPriority(true, prioLeast);
    for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
      DevBlock& b = *recBlocks[bi];
      CUDA_TRY(c, cudaMemcpyAsync(b.v.q, c.blocks[bi].runSnap + (size_t)k * nU * b.v.N,
                                  (size_t)nU * b.v.N * sizeof(double), cudaMemcpyDeviceToDevice, recLanes.main));
      launchPrims(c, b, b.v.q, false, nullptr, 0, recLanes.main);
    }
    launchSetCounters(recCounters, L + 1, L, recLanes.main);
    if (twoLanes) setLaunchPriority(true, prioGreatest);
    for (int s = L + 1; s <= end; ++s) CUDA_TRY(c, cudaGraphLaunch(c.gRecomputeH[h], recLanes.main));
    c.launches += (long long)(end - L) * nodesRec;
    if (twoLanes) CUDA_TRY(c, cudaEventRecord(c.evRecDone[h], recLanes.main));
    return 0;
  };
  if (twoLanes) {
    // the second lanes start after everything issued so far on the main stream
    CUDA_TRY(c, cudaEventRecord(c.evFork[3], c.stream));
    CUDA_TRY(c, cudaStreamWaitEvent(c.stream2, c.evFork[3], 0));
  }
  if (!resident && recompute(nSeg - 1)) return 1;
  for (int k = nSeg - 1; k >= 0; --k) {
    const int L = k * S, end = std::min(T, L + S);
    const int h = k % halves;
    if (twoLanes) {
      CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.evRecDone[h], 0));
      if (k >= 1) {
        // segment k-1 reuses the half that the adjoint of segment k+1 read
        if (k + 1 <= nSeg - 1) CUDA_TRY(c, cudaStreamWaitEvent(c.stream2, c.evAdjDone[(k + 1) % 2], 0));
        if (recompute(k - 1)) return 1;
      }
    }
    launchSetCounters(c.dCounters, end, L, c.stream);
    for (int s = end; s >= L + 1; --s) CUDA_TRY(c, cudaGraphLaunch(c.gAdjointH[h], c.stream));
    c.launches += 1 + (long long)(end - L) * nodesAdj;
    if (twoLanes) CUDA_TRY(c, cudaEventRecord(c.evAdjDone[h], c.stream));
    if (!twoLanes && !resident && k >= 1 && recompute(k - 1)) return 1;
  }
  if (twoLanes) {
    // join the second lanes back into the main stream
    CUDA_TRY(c, cudaEventRecord(c.evJoin[3], c.stream2));
    CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.evJoin[3], 0));
  }
  if (checkLaunch(c)) return 1;
  std::vector<double> vals;
  if (reduceRegion(c, 4 * T, vals)) return 1;
  double sum = 0.0;
  for (int n = T; n >= 1; --n)
    for (int i = 4; i >= 1; --i) {
      const long long entry = (long long)(T - n) * 4 + (4 - i);
      sum = sum + kRkNorm[i - 1] * c.stepDt[n - 1] * vals[entry];
    }
  *sensitivity = sum;
  return 0;
}

int mgd_run_forward(mgd_ctx* h, int n_steps, int save_interval, double t0, double* cost) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (n_steps < 1) return fail(c, "n_steps must be >= 1");
  if (save_interval < 1) save_interval = n_steps;
  if (!singleBlock(c)) return regionRunForward(c, n_steps, save_interval, t0, cost);
  DevBlock& b = c.blocks[0];
  if (prepareForwardRun(c, n_steps, save_interval, t0, true)) return 1;
  const bool cflMode = c.opts.use_constant_cfl != 0;
  const bool controller = c.opts.enable_controller && c.opts.controller_switch && c.dForcing;
  const bool functional = c.opts.enable_functional != 0 && c.opts.functional_type == MGD_FUNCTIONAL_SOUND;
  // with a resident trajectory the flux kernel also stores every stage's
  // state, primitives, stress and heat flux, which the adjoint run then reads
  // instead of recomputing checkpoint segments
  bool resident = false;
  if (c.trajectoryStorage && ensureTrajectoryBuffer(c, b, n_steps, &resident)) return 1;
  RunScalars rs = runScalars(c);
  const bool limits = c.opts.enable_solution_limits != 0;
  if (limits) rs.limitKey = c.dLimitKey;
  if (setCounters(c, 1, 0)) return 1;
  if (capture(c, &c.gForward, &c.nodesForward, [&]() {
        if (cflMode) launchTimeStep(c, b, c.dDtPartials, c.dStepDt, c.dCounters, c.dTime, c.dStageTime, c.dAmp);
        for (int i = 1; i <= 4; ++i) {
          // checkSolutionLimits before every substep (src/SolverImpl.f90:812-818)
          if (limits) launchSolutionLimits(c, b, 0, c.dCounters, i, c.dLimitKey);
          forwardStage(c, b, i, rs, false, controller, resident, functional);
        }
        launchSnapshot(c, b, c.dSnapshots, save_interval, false);
        launchStepAdvance(c, 1);
      }))
    return 1;
  for (int s = 0; s < n_steps; ++s) CUDA_TRY(c, cudaGraphLaunch(c.gForward, c.stream));
  c.launches += (long long)n_steps * c.nodesForward;
  if (checkLaunch(c)) return 1;
  if (finishForwardRun(c, cost)) return 1;
  c.trajectorySteps = resident ? n_steps : 0;
  if (const int st = limitOutcome(c, cost, false)) {
    c.limitViolated = st == MGD_SOLUTION_LIMITS;
    c.trajectorySteps = 0;
    return st;
  }
  return 0;
}

// The adjoint of a forward run that stopped at a solution-limit violation
// stops too (src/SolverImpl.f90:1193-1198): HUGE and the same status.
static int limitStop(Context& c, double* value) {
  if (!c.limitViolated) return 0;
  *value = std::numeric_limits<double>::max();
  c.error = c.limitMessage;
  return MGD_SOLUTION_LIMITS;
}

int mgd_run_adjoint(mgd_ctx* h, double* sensitivity) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (c.runSteps < 1) return fail(c, "mgd_run_adjoint needs a preceding mgd_run_forward");
  if (const int st = limitStop(c, sensitivity)) return st;
  if (!singleBlock(c)) return regionRunAdjoint(c, sensitivity);
  DevBlock& b = c.blocks[0];
  const long long N = b.v.N;
  const int nU = c.nU, T = c.runSteps;
  // a resident trajectory of this run: one segment over all steps, no recomputation
  const bool resident = c.trajectorySteps == T;
  const int S = resident ? T : c.saveInterval;
  const double dtT = c.stepDt[T - 1];  // step size of the final forward step
  if (!resident && ensureStageBuffer(c, b, S)) return 1;
  const bool twoLanes = c.stageHalves == 2;
  if (twoLanes && ensureShadow(c, b)) return 1;
  const bool controller = c.opts.enable_controller && c.opts.controller_switch && c.dForcing;
  const bool full = c.slotFull != 0;
  // The recomputation of segment k-1 runs on the second lanes (own work
  // arrays, own step counters, the other half of the stage buffer) while the
  // adjoint consumes segment k; with one half they alternate on one stream.
  DevBlock rb;
  rb.desc = b.desc;
  rb.v = twoLanes ? c.shadow : b.v;
  rb.exc = b.exc;
  rb.tGrad = b.tGrad; rb.tDiss = b.tDiss; rb.tRhs = b.tRhs; rb.gradLanes = b.gradLanes; rb.coreLanes = b.coreLanes;
  rb.tAdjA = b.tAdjA; rb.tAdjD = b.tAdjD; rb.tAdjB = b.tAdjB;
  const Lanes adjLanes{c.stream, c.side, c.evFork[1], c.evJoin[1]};
  const Lanes recLanes = twoLanes ? Lanes{c.stream2, c.side2, c.evFork[2], c.evJoin[2]}
                                  : Lanes{c.stream, c.side, c.evFork[0], c.evJoin[0]};
  int* recCounters = twoLanes ? c.dCounters + 4 : c.dCounters;
  // adjoint initial condition at the final state (its primitives are current)
  const bool terminal = c.opts.functional_type == MGD_FUNCTIONAL_TERMINAL_KINETIC_ENERGY;
  launchPrims(c, b, b.v.q, false);
  if (terminal) launchKineticEnergyAdjointInitial(c, b);
  else launchAdjointInitial(c, b, c.opts.adjoint_forcing_switch ? -dtT / 6.0 : 0.0);
  long long nodesRec = 0, nodesAdj = 0;
  setProgrammaticLaunch(!twoLanes);
  struct Restore {
    ~Restore() {
      setProgrammaticLaunch(true);
      setLaunchPriority(false, 0);
    }
  } restore;
  // The adjoint is the critical path; the recomputation of the next segment
  // has slack (a segment's forward stages take less time than its adjoint
  // stages), so its kernels launch at the lowest priority and take the SM
  // time the adjoint leaves.
  int prioLeast = 0, prioGreatest = 0;
  cudaDeviceGetStreamPriorityRange(&prioLeast, &prioGreatest);
  for (int half = 0; half < c.stageHalves; ++half) {
    RunScalars ra = runScalars(c);
    if (terminal) ra.adjointForcingSwitch = 0;  // no forcing during the run
    ra.stageBuf = c.dStageBuf + half * c.stageHalf;
    RunScalars rr = ra;
    rr.step = recCounters;
    rr.segBase = recCounters + 1;
    if (twoLanes) setLaunchPriority(true, prioLeast);
    if (!resident && capture(c, &c.gRecomputeH[half], &nodesRec, [&]() {
          for (int i = 1; i <= 4; ++i) forwardStage(c, rb, i, rr, false, controller, true, false, &recLanes);
          launchStepAdvanceOn(recCounters, 1, recLanes.main);
        }, recLanes.main))
      return 1;
    if (twoLanes) setLaunchPriority(true, prioGreatest);
    if (capture(c, &c.gAdjointH[half], &nodesAdj, [&]() {
          for (int i = 4; i >= 1; --i) {
            if (!full) {
              // restore the forward state of this stage from its slot
              launchPrims(c, b, nullptr, true, &ra, i, adjLanes.main);
              if (c.phys.viscous) launchGradFlux(c, b, false, true, &ra, i, false, adjLanes.main);
            }
            adjointStage(c, b, i, ra, i, 0.0, false, full, true, &adjLanes);
          }
          launchStepAdvanceOn(c.dCounters, -1, adjLanes.main);
        }, adjLanes.main))
      return 1;
  }
  c.nodesRecompute = nodesRec + 3;
  c.nodesAdjoint = nodesAdj + 1;
  const int nSeg = (T + S - 1) / S;
  // UniformCheckpointer: reload the snapshot of segment k and recompute its stages
  auto recompute = [&](int k) -> int {
    const int L = k * S, end = std::min(T, L + S);
    const int half = k % c.stageHalves;
    CUDA_TRY(c, cudaMemcpyAsync(rb.v.q, c.dSnapshots + (size_t)k * nU * N, (size_t)nU * N * sizeof(double),
                                cudaMemcpyDeviceToDevice, recLanes.main));
    if (twoLanes) setLaunchPriority(true, prioLeast);
    launchPrims(c, rb, rb.v.q, false, nullptr, 0, recLanes.main);
    launchSetCounters(recCounters, L + 1, L, recLanes.main);
    if (twoLanes) setLaunchPriority(true, prioGreatest);
    for (int s = L + 1; s <= end; ++s) CUDA_TRY(c, cudaGraphLaunch(c.gRecomputeH[half], recLanes.main));
    c.launches += 2 + (long long)(end - L) * nodesRec;
    if (twoLanes) CUDA_TRY(c, cudaEventRecord(c.evRecDone[half], recLanes.main));
    return 0;
  };
  if (twoLanes) {
    // the second lanes start after everything issued so far on the main stream
    CUDA_TRY(c, cudaEventRecord(c.evFork[3], c.stream));
    CUDA_TRY(c, cudaStreamWaitEvent(c.stream2, c.evFork[3], 0));
  }
  if (!resident && recompute(nSeg - 1)) return 1;
  for (int k = nSeg - 1; k >= 0; --k) {
    const int L = k * S, end = std::min(T, L + S);
    const int half = k % c.stageHalves;
    if (twoLanes) {
      CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.evRecDone[half], 0));
      if (k >= 1) {
        // segment k-1 reuses the half that the adjoint of segment k+1 read
        if (k + 1 <= nSeg - 1) CUDA_TRY(c, cudaStreamWaitEvent(c.stream2, c.evAdjDone[(k + 1) % 2], 0));
        if (recompute(k - 1)) return 1;
      }
    }
    launchSetCounters(c.dCounters, end, L, c.stream);
    for (int s = end; s >= L + 1; --s) CUDA_TRY(c, cudaGraphLaunch(c.gAdjointH[half], c.stream));
    c.launches += 1 + (long long)(end - L) * nodesAdj;
    if (twoLanes) CUDA_TRY(c, cudaEventRecord(c.evAdjDone[half], c.stream));
    if (!twoLanes && k >= 1 && recompute(k - 1)) return 1;
  }
  if (twoLanes) {
    // join the second lanes back into the main stream
    CUDA_TRY(c, cudaEventRecord(c.evJoin[3], c.stream2));
    CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.evJoin[3], 0));
  }
  if (checkLaunch(c)) return 1;
  std::vector<double> vals;
  if (reduceToHost(c, 4 * T, vals)) return 1;
  double sum = 0.0;
  for (int n = T; n >= 1; --n)
    for (int i = 4; i >= 1; --i) {
      const long long entry = (long long)(T - n) * 4 + (4 - i);
      sum = sum + kRkNorm[i - 1] * c.stepDt[n - 1] * vals[entry];
    }
  *sensitivity = sum;
  return 0;
}

// Solver%runLinearized (src/SolverImpl.f90:1300-1450) over the steps of the
// last forward run: the perturbation in lambda advances with
// substepLinearizedRK4 along the forward trajectory, whose stage states the
// checkpointer provides (reverseMigrator%migrateTo, :1378-1386). Here each
// segment's stage states are recomputed from its snapshot into the stage
// slots, then the segment's linearized steps read them. With a control
// perturbation the actuators add it (src/ActuatorPatchImpl.f90:162-170), and
// the tangent of the functional, sum over stages of w_i dt times the
// functional's tangent after each stage, is reduced like J. The conserved
// state of the final step is restored at the end.
static int regionRunLinearized(Context& c, const double* delta_forcing, long long n_entries, double* delta_cost);

int mgd_run_linearized(mgd_ctx* h, const double* delta_forcing, long long n_entries, double* delta_cost) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (c.runSteps < 1) return fail(c, "mgd_run_linearized needs a preceding mgd_run_forward");
  if (const int st = limitStop(c, delta_cost)) return st;
  if (!singleBlock(c)) return regionRunLinearized(c, delta_forcing, n_entries, delta_cost);
  if (refuseLinearized(c)) return 1;
  DevBlock& b = c.blocks[0];
  const long long N = b.v.N;
  const int nU = c.nU, T = c.runSteps;
  // a resident trajectory of this run: one segment, no recomputation (and the
  // slots stay intact for a following adjoint run)
  const bool resident = c.trajectorySteps == T;
  const int S = resident ? T : c.saveInterval;
  if (!resident && ensureStageBuffer(c, b, S)) return 1;
  const bool controller = c.opts.enable_controller && c.opts.controller_switch && c.dForcing;
  const bool deltaControl = c.opts.enable_controller && c.opts.controller_switch && delta_forcing && n_entries > 0 &&
                            c.actuatorPoints > 0;
  if (deltaControl) {
    const long long n = n_entries * c.actuatorPoints;
    if (c.deltaForcingCapacity < n) {
      cudaFree(c.dDeltaForcing);
      c.dDeltaForcing = nullptr;
      c.deltaForcingCapacity = 0;
      CUDA_TRY(c, cudaMalloc((void**)&c.dDeltaForcing, (size_t)n * sizeof(double)));
      c.deltaForcingCapacity = n;
    }
    CUDA_TRY(c, cudaMemcpyAsync(c.dDeltaForcing, delta_forcing, (size_t)n * sizeof(double), cudaMemcpyDefault,
                                c.stream));
  }
  const bool functional = c.opts.enable_functional && c.opts.functional_type == MGD_FUNCTIONAL_SOUND;
  if (functional && ensurePartials(c, 4LL * T)) return 1;
  double* qFinal = nullptr;
  CUDA_TRY(c, cudaMalloc((void**)&qFinal, (size_t)nU * N * sizeof(double)));
  struct Free { double* p; ~Free() { cudaFree(p); } } freeFinal{qFinal};
  CUDA_TRY(c, cudaMemcpyAsync(qFinal, b.v.q, (size_t)nU * N * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  setProgrammaticLaunch(true);
  RunScalars rs = runScalars(c);
  rs.stageBuf = c.dStageBuf;
  // the linearized stages read the perturbation's entries as their forcing
  RunScalars rl = rs;
  rl.forcing = deltaControl ? c.dDeltaForcing : nullptr;
  rl.nForcingEntries = deltaControl ? n_entries : 0;
  cudaGraphExec_t gRec = nullptr, gLin = nullptr;
  struct Graphs {
    cudaGraphExec_t* a;
    cudaGraphExec_t* b;
    ~Graphs() {
      if (*a) cudaGraphExecDestroy(*a);
      if (*b) cudaGraphExecDestroy(*b);
    }
  } graphs{&gRec, &gLin};
  long long nodesRec = 0, nodesLin = 0;
  const Lanes lanes{c.stream, c.side, c.evFork[0], c.evJoin[0]};
  if (!resident && capture(c, &gRec, &nodesRec, [&]() {
        for (int i = 1; i <= 4; ++i) forwardStage(c, b, i, rs, false, controller, true, false, &lanes);
        launchStepAdvance(c, 1);
      }))
    return 1;
  const bool full = c.slotFull != 0;
  if (capture(c, &gLin, &nodesLin, [&]() {
        for (int i = 1; i <= 4; ++i) {
          // forward state of stage i: read from its full slot, or restored
          // from a q-only slot with its primitives, stress and heat flux
          if (!full) {
            launchPrims(c, b, nullptr, true, &rs, i);
            if (c.phys.viscous) launchGradFlux(c, b, false, true, &rs, i, false);
          }
          // the functional's tangent after the stage before (state and perturbation at this stage's start)
          if (functional) launchFunctionalTangent(c, b, rl, i, full);
          if (c.phys.dissipation) launchDissipation(c, b, b.v.lam, 1.0);
          launchLinearized(c, b, i, rl, 0.0, i, full, deltaControl);
        }
        launchStepAdvance(c, 1);
      }))
    return 1;
  const int nSeg = (T + S - 1) / S;
  for (int k = 0; k < nSeg; ++k) {
    const int L = k * S, end = std::min(T, L + S);
    if (!resident) {
      CUDA_TRY(c, cudaMemcpyAsync(b.v.q, c.dSnapshots + (size_t)k * nU * N, (size_t)nU * N * sizeof(double),
                                  cudaMemcpyDeviceToDevice, c.stream));
      launchPrims(c, b, b.v.q, false);
      launchSetCounters(c.dCounters, L + 1, L, c.stream);
      for (int s = L + 1; s <= end; ++s) CUDA_TRY(c, cudaGraphLaunch(gRec, c.stream));
    }
    launchSetCounters(c.dCounters, L + 1, L, c.stream);
    for (int s = L + 1; s <= end; ++s) CUDA_TRY(c, cudaGraphLaunch(gLin, c.stream));
    c.launches += 3 + (long long)(end - L) * (nodesRec + nodesLin);
  }
  CUDA_TRY(c, cudaMemcpyAsync(b.v.q, qFinal, (size_t)nU * N * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  launchPrims(c, b, b.v.q, false);
  double dJ = 0.0;
  if (functional) {
    // the last stage's term, at the final state: the counters stand at step T + 1
    launchFunctionalTangent(c, b, rl, 1, false);
    if (checkLaunch(c)) return 1;
    std::vector<double> vals;
    if (reduceToHost(c, 4 * T, vals)) return 1;
    for (int st = 0; st < T; ++st)
      for (int i = 0; i < 4; ++i) dJ = dJ + kRkNorm[i] * c.stepDt[st] * vals[(size_t)4 * st + i];
  }
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (delta_cost) *delta_cost = dJ;
  return 0;
}

int mgd_set_patch_control_forcing(mgd_ctx* h, const double* forcing) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (!forcing) {
    c.apiForcingSet = false;
    return 0;
  }
  if (c.actuatorPoints == 0) return fail(c, "the region has no actuator patch");
  if (!c.dApiForcing) CUDA_TRY(c, cudaMalloc((void**)&c.dApiForcing, (size_t)c.actuatorPoints * sizeof(double)));
  CUDA_TRY(c, cudaMemcpyAsync(c.dApiForcing, forcing, (size_t)c.actuatorPoints * sizeof(double), cudaMemcpyDefault,
                              c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  c.apiForcingSet = true;
  return 0;
}

int mgd_set_adjoint_nonzero_initial_condition(mgd_ctx* h, int enable) {
  h->c.adjointNonzeroIC = enable != 0;
  return 0;
}

int mgd_time_step_size(mgd_ctx* h, double* dt) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (!c.opts.use_constant_cfl) {
    *dt = c.opts.time_step_size;
    return 0;
  }
  DevBlock& b = c.blocks[0];
  if (ensureStepBuffers(c, b, std::max(1, c.runSteps))) return 1;
  launchPrims(c, b, b.v.q, false);
  launchTimeStep(c, b, c.dDtPartials, c.dTime, nullptr, nullptr, nullptr, nullptr);
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaMemcpyAsync(dt, c.dTime, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

int mgd_get_step_sizes(mgd_ctx* h, double* host, int n_steps) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  const int n = std::min(n_steps, (int)c.stepDt.size());
  std::copy(c.stepDt.begin(), c.stepDt.begin() + std::max(0, n), host);
  return 0;
}

int mgd_get_gradient(mgd_ctx* h, double* host, long long n_entries) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  const long long avail = 4LL * c.runSteps;
  const long long n = std::min(n_entries, avail) * c.actuatorPoints;
  if (n <= 0) return 0;
  CUDA_TRY(c, cudaMemcpyAsync(host, c.dGradient, (size_t)n * sizeof(double), cudaMemcpyDefault, c.stream));
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}


// ---------------------------------------------------------------------------
// files: PLOT3D solutions and grids, actuator-patch streams, device ZAXPY
// ---------------------------------------------------------------------------
static int joinIo(Context& c) {
  if (c.ioThread.joinable()) c.ioThread.join();
  const int s = c.ioStatus;
  c.ioStatus = 0;
  if (s) return fail(c, "writing a solution file failed");
  return 0;
}

int mgd_wait_io(mgd_ctx* h) { return joinIo(h->c); }

static double* fieldArray(Context& c, DevBlock& b, int field) {
  return field == MGD_FIELD_ADJOINT ? b.v.lam : (field == MGD_FIELD_CONSERVED ? b.v.q : nullptr);
}

int mgd_save_solution(mgd_ctx* h, const char* filename, int field, int timestep, double time) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (joinIo(c)) return 1;
  size_t bytes = 0;
  for (DevBlock& b : c.blocks) {
    if (!fieldArray(c, b, field)) return fail(c, "mgd_save_solution: field must be CONSERVED or ADJOINT");
    bytes += (size_t)b.v.N * c.nU * sizeof(double);
  }
  if (!c.ioStream) {
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c.ioStream, cudaStreamNonBlocking));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c.ioCopied, cudaEventDisableTiming));
  }
  if (c.ioStagingBytes < bytes) {
    if (c.ioStaging) cudaFreeHost(c.ioStaging);
    c.ioStaging = nullptr;
    c.ioStagingBytes = 0;
    CUDA_TRY(c, cudaMallocHost((void**)&c.ioStaging, bytes));
    c.ioStagingBytes = bytes;
  }
  // copy after the work issued so far; later work on the context stream waits for the copy
  CUDA_TRY(c, cudaEventRecord(c.evFork[4], c.stream));
  CUDA_TRY(c, cudaStreamWaitEvent(c.ioStream, c.evFork[4], 0));
  size_t off = 0;
  std::vector<const double*> arrays;
  std::vector<int> sizes;
  for (DevBlock& b : c.blocks) {
    const size_t n = (size_t)b.v.N * c.nU;
    CUDA_TRY(c, cudaMemcpyAsync(c.ioStaging + off, fieldArray(c, b, field), n * sizeof(double),
                                cudaMemcpyDeviceToHost, c.ioStream));
    arrays.push_back(c.ioStaging + off);
    for (int d = 0; d < 3; ++d) sizes.push_back(b.v.gs[d]);
    off += n;
  }
  CUDA_TRY(c, cudaEventRecord(c.ioCopied, c.ioStream));
  CUDA_TRY(c, cudaStreamWaitEvent(c.stream, c.ioCopied, 0));
  const std::string name(filename);
  const int nU = c.nU;
  const cudaEvent_t copied = c.ioCopied;
  const int device = c.device;
  int* status = &c.ioStatus;
  c.ioThread = std::thread([=]() {
    cudaSetDevice(device);
    if (cudaEventSynchronize(copied) != cudaSuccess) {
      *status = 1;
      return;
    }
    // plot3dAuxiliaryData: (timestep, 0, 0, time) (src/RegionImpl.f90:1736-1746, src/StateImpl.f90:372)
    const double aux[4] = {(double)timestep, 0.0, 0.0, time};
    *status = mgd_plot3d_write_solution(name.c_str(), (int)sizes.size() / 3, sizes.data(), nU, arrays.data(), aux);
  });
  return 0;
}

int mgd_load_solution(mgd_ctx* h, const char* filename, int field, double* time) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (joinIo(c)) return 1;
  std::vector<std::vector<double>> host;
  std::vector<double*> arrays;
  std::vector<int> sizes;
  for (DevBlock& b : c.blocks) {
    if (!fieldArray(c, b, field)) return fail(c, "mgd_load_solution: field must be CONSERVED or ADJOINT");
    host.emplace_back((size_t)b.v.N * c.nU);
    for (int d = 0; d < 3; ++d) sizes.push_back(b.v.gs[d]);
  }
  for (auto& v : host) arrays.push_back(v.data());
  double aux[4] = {0, 0, 0, 0};
  if (mgd_plot3d_read_solution(filename, (int)c.blocks.size(), sizes.data(), c.nU, arrays.data(), aux))
    return fail(c, std::string("cannot read PLOT3D solution file '") + filename + "' for this region");
  for (size_t bi = 0; bi < c.blocks.size(); ++bi)
    CUDA_TRY(c, cudaMemcpy(fieldArray(c, c.blocks[bi], field), host[bi].data(), host[bi].size() * sizeof(double),
                           cudaMemcpyHostToDevice));
  if (time) *time = aux[3];
  return 0;
}

int mgd_save_grid(mgd_ctx* h, const char* filename) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  std::vector<const double*> coords;
  std::vector<const int*> ib;
  std::vector<int> sizes;
  for (DevBlock& b : c.blocks) {
    coords.push_back(b.hostCoords.data());
    ib.push_back(b.hostIblank.data());
    for (int d = 0; d < 3; ++d) sizes.push_back(b.v.gs[d]);
  }
  if (mgd_plot3d_write_grid(filename, (int)c.blocks.size(), sizes.data(), c.nD, coords.data(), ib.data()))
    return fail(c, std::string("cannot write PLOT3D grid file '") + filename + "'");
  return 0;
}

// Actuator patches in bc.dat order with their point counts and offsets in an entry.
static std::vector<std::pair<const mgd_patch_desc*, long long>> actuatorPatches(Context& c) {
  std::vector<std::pair<const mgd_patch_desc*, long long>> out;
  for (const mgd_patch_desc& p : c.patches) {
    if (p.type != MGD_PATCH_ACTUATOR || p.grid_index != 1) continue;
    int e[6];
    resolveExtent(p, c.blocks[0].v.gs, c.nD, e);
    out.emplace_back(&p, (long long)(e[1] - e[0] + 1) * (e[3] - e[2] + 1) * (e[5] - e[4] + 1));
  }
  return out;
}

int mgd_save_gradient(mgd_ctx* h, const char* prefix, long long n_entries) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  const long long P = c.actuatorPoints, n = std::min(n_entries, 4LL * c.runSteps);
  if (n <= 0 || P <= 0) return fail(c, "mgd_save_gradient needs an adjoint run and an actuator patch");
  std::vector<double> g((size_t)(n * P));
  CUDA_TRY(c, cudaMemcpy(g.data(), c.dGradient, g.size() * sizeof(double), cudaMemcpyDeviceToHost));
  long long off = 0;
  for (auto& pp : actuatorPatches(c)) {
    const std::string name = std::string(prefix) + ".gradient_" + pp.first->name + ".dat";
    if (mgd_write_patch_stream(name.c_str(), g.data(), n, pp.second, P, off))
      return fail(c, "cannot write '" + name + "'");
    off += pp.second;
  }
  return 0;
}

int mgd_load_control_forcing(mgd_ctx* h, const char* prefix, long long n_entries) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  const long long P = c.actuatorPoints;
  if (n_entries <= 0 || P <= 0) return fail(c, "mgd_load_control_forcing needs entries and an actuator patch");
  std::vector<double> f((size_t)(n_entries * P));
  long long off = 0;
  for (auto& pp : actuatorPatches(c)) {
    const std::string name = std::string(prefix) + ".control_forcing_" + pp.first->name + ".dat";
    if (mgd_read_patch_stream(name.c_str(), f.data(), n_entries, pp.second, P, off))
      return fail(c, "cannot read '" + name + "'");
    off += pp.second;
  }
  return mgd_set_control_forcing(h, f.data(), n_entries);
}

int mgd_control_zaxpy(mgd_ctx* h, double a, int accumulate) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  const long long P = c.actuatorPoints, n = 4LL * c.runSteps;
  if (n <= 0 || P <= 0 || !c.dGradient) return fail(c, "mgd_control_zaxpy needs an adjoint run and an actuator patch");
  if (accumulate && c.nForcingEntries != n) return fail(c, "mgd_control_zaxpy: the current forcing has another length");
  if (c.forcingCapacity < n * P) {
    if (accumulate) return fail(c, "mgd_control_zaxpy: no forcing to accumulate into");
    cudaFree(c.dForcing);
    c.dForcing = nullptr;
    CUDA_TRY(c, cudaMalloc((void**)&c.dForcing, (size_t)(n * P) * sizeof(double)));
    c.forcingCapacity = n * P;
  }
  launchAxpy(c, c.dForcing, c.dGradient, a, n * P, accumulate != 0);
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  c.nForcingEntries = n;
  return 0;
}

// Times each kernel of one RK stage separately with CUDA events on the
// context stream, avg_ms receiving the mean duration per launch over `reps`
// launches. Forward: [gradient/flux, dissipation, divergence+RK, primitives,
// functional]; adjoint: [core, dissipation, diffusion, assembly+RK,
// gradient/sensitivity]. The state is left changed (the RK updates run).
int mgd_profile_stage_kernels(mgd_ctx* h, int mode, int reps, double* avg_ms, int* n_kernels) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (c.runSteps < 1) return fail(c, "mgd_profile_stage_kernels needs a preceding mgd_run_forward");
  DevBlock& b = c.blocks[0];
  RunScalars rs = runScalars(c);
  if (setCounters(c, 1, 0)) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const bool controller = c.opts.enable_controller && c.opts.controller_switch && c.dForcing;
  // each kernel back to back without programmatic launch: an early-launched
  // copy would wait on the SMs beside the running one and slow it
  setProgrammaticLaunch(false);
  struct Restore {
    ~Restore() { setProgrammaticLaunch(true); }
  } restore;
  auto timeIt = [&](auto fn) {
    fn();  // warm
    cudaEventRecord(e0, c.stream);
    for (int r = 0; r < reps; ++r) fn();
    cudaEventRecord(e1, c.stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return (double)ms / reps;
  };
  launchPrims(c, b, b.v.q, false);
  if (mode == MGD_FORWARD) {
    avg_ms[0] = timeIt([&] { launchGradFlux(c, b, true, false, &rs, 2, false); });
    avg_ms[1] = c.phys.dissipation ? timeIt([&] { launchDissipation(c, b, b.v.q, 1.0); }) : 0.0;
    avg_ms[2] = timeIt([&] { launchForwardDivergence(c, b, 2, rs, false, controller); });
    avg_ms[3] = timeIt([&] { launchPrims(c, b, b.v.q, false); });
    avg_ms[4] = c.opts.enable_functional ? timeIt([&] { launchFunctional(c, b, rs, 2); }) : 0.0;
  } else {
    if (c.phys.viscous) launchGradFlux(c, b, false, true, &rs, 1, false);
    avg_ms[0] = timeIt([&] { launchAdjointCore(c, b, rs, 3, false); });
    avg_ms[1] = c.phys.dissipation ? timeIt([&] { launchDissipation(c, b, b.v.lam, -1.0); }) : 0.0;
    avg_ms[2] = c.phys.viscous ? timeIt([&] { launchAdjointDiffusion(c, b); }) : 0.0;
    avg_ms[3] = timeIt([&] { launchAdjointAssemble(c, b, 3, rs, 3, 0.0, false, false); });
    avg_ms[4] = timeIt([&] { launchGradientSensitivity(c, b, rs, 3); });
    avg_ms[5] = b.v.ff.n > b.nInterfaceEntries ? timeIt([&] { launchAdjointSatVectors(c, b, rs, 3, false); }) : 0.0;
  }
  *n_kernels = mode == MGD_FORWARD ? 5 : 6;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (checkLaunch(c)) return 1;
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  return 0;
}

// Self-test of the persistent kernel's bounded grid barrier.
int mgd_selftest_grid_barrier(int n_blocks, int expected, int rounds, long long limit, int* status,
                              long long* checksum) {
  if (n_blocks < 1 || expected < 1 || rounds < 1 || limit < 1 || !status || !checksum) return 1;
  return selftestGridBarrier(n_blocks, (unsigned int)expected, rounds, limit, status, checksum) ? 1 : 0;
}

// FP64 throughput with warps_per_sm warps on every SM.
int mgd_selftest_fp64_rate(int warps_per_sm, double* lane_ops_per_clock) {
  if (warps_per_sm < 1 || warps_per_sm > 32 || !lane_ops_per_clock) return 1;
  return selftestFp64Rate(warps_per_sm, lane_ops_per_clock) ? 1 : 0;
}

// Self-test of the table-driven power function used by the viscosity law:
// evaluates x[i]^e with it (fast) and with CUDA's pow (ref) on the current device.
int mgd_selftest_pow(const double* x, int n, double e, double* fast, double* ref) {
  if (n <= 0) return 0;
  double *dx = nullptr, *df = nullptr, *dr = nullptr;
  if (cudaMalloc((void**)&dx, n * sizeof(double)) != cudaSuccess) return 1;
  cudaMalloc((void**)&df, n * sizeof(double));
  cudaMalloc((void**)&dr, n * sizeof(double));
  cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice);
  launchPowSelfTest(dx, n, e, df, dr);
  cudaMemcpy(fast, df, n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaMemcpy(ref, dr, n * sizeof(double), cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaGetLastError();
  cudaFree(dx); cudaFree(df); cudaFree(dr);
  return err == cudaSuccess ? 0 : 1;
}

// The tangent run of a multi-block region over the checkpoints of its last
// forward run (regionRunForward): per segment, every block's stage states
// are recomputed into its own slots, then the segment's linearized steps run
// with the block-interface SATs between the blocks' fluxes and divergences.
static int regionRunLinearized(Context& c, const double* delta_forcing, long long n_entries, double* delta_cost) {
  if (refuseLinearized(c)) return 1;
  if (ensureBlockStreams(c)) return 1;
  const int nU = c.nU, nD = c.nD, T = c.runSteps;
  // a resident trajectory of this run: one segment, no recomputation (and the
  // slots stay intact for a following adjoint run)
  const bool resident = c.trajectorySteps == T;
  const int S = resident ? T : c.saveInterval;
  const bool controller = c.opts.enable_controller && c.opts.controller_switch && c.dForcing;
  const bool deltaControl = c.opts.enable_controller && c.opts.controller_switch && delta_forcing && n_entries > 0 &&
                            c.actuatorPoints > 0;
  if (deltaControl) {
    const long long n = n_entries * c.actuatorPoints;
    if (c.deltaForcingCapacity < n) {
      cudaFree(c.dDeltaForcing);
      c.dDeltaForcing = nullptr;
      c.deltaForcingCapacity = 0;
      CUDA_TRY(c, cudaMalloc((void**)&c.dDeltaForcing, (size_t)n * sizeof(double)));
      c.deltaForcingCapacity = n;
    }
    CUDA_TRY(c, cudaMemcpyAsync(c.dDeltaForcing, delta_forcing, (size_t)n * sizeof(double), cudaMemcpyDefault,
                                c.stream));
  }
  const bool functional = c.opts.enable_functional && c.opts.functional_type == MGD_FUNCTIONAL_SOUND;
  // stage slots as the region's adjoint run sizes them
  size_t freeB = 0, totalB = 0;
  CUDA_TRY(c, cudaMemGetInfo(&freeB, &totalB));
  long long pts = 0, held = 0;
  for (DevBlock& b : c.blocks) {
    pts += b.v.N;
    held += b.runStageCap;
  }
  const long long fullPer = nU + PrimLayout{nD}.count() + nD * nD + nD;
  const bool full =
      resident || (double)(4LL * S * fullPer * pts) * sizeof(double) <= 0.5 * ((double)freeB + held * 8.0);
  for (DevBlock& b : c.blocks) {
    const long long stride = (full ? fullPer : nU) * b.v.N;
    if (growDevice(c, &b.runStage, &b.runStageCap, 4LL * S * stride)) return 1;
  }
  c.slotFull = full ? 1 : 0;
  std::vector<RunScalars> rs, rl;
  std::vector<double*> qFinal(c.blocks.size(), nullptr);
  struct FreeAll {
    std::vector<double*>* v;
    ~FreeAll() {
      for (double* p : *v) cudaFree(p);
    }
  } freeAll{&qFinal};
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    DevBlock& b = c.blocks[bi];
    RunScalars r = blockRunScalars(c, b, bi == 0);
    r.slotFull = c.slotFull;
    r.slotStride = (full ? fullPer : nU) * b.v.N;
    rs.push_back(r);
    RunScalars l = r;
    l.forcing = (deltaControl && bi == 0) ? c.dDeltaForcing : nullptr;
    l.nForcingEntries = (deltaControl && bi == 0) ? n_entries : 0;
    rl.push_back(l);
    CUDA_TRY(c, cudaMalloc((void**)&qFinal[bi], (size_t)nU * b.v.N * sizeof(double)));
    CUDA_TRY(c, cudaMemcpyAsync(qFinal[bi], b.v.q, (size_t)nU * b.v.N * sizeof(double), cudaMemcpyDeviceToDevice,
                                c.stream));
  }
  BlockRefs refs = runRefs(c);
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) refs.slotStride[bi] = rs[bi].slotStride;
  cudaGraphExec_t gRec = nullptr, gLin = nullptr;
  struct Graphs {
    cudaGraphExec_t* a;
    cudaGraphExec_t* b;
    ~Graphs() {
      if (*a) cudaGraphExecDestroy(*a);
      if (*b) cudaGraphExecDestroy(*b);
    }
  } graphs{&gRec, &gLin};
  long long nodesRec = 0, nodesLin = 0;
  if (!resident && capture(c, &gRec, &nodesRec, [&]() {
        for (int i = 1; i <= 4; ++i) regionRunStage(c, rs, i, controller, true, false);
        launchStepAdvance(c, 1);
      }))
    return 1;
  if (capture(c, &gLin, &nodesLin, [&]() {
        for (int i = 1; i <= 4; ++i) {
          forEachBlockConcurrently(c, [&](int bi, cudaStream_t s) {
            DevBlock& b = c.blocks[bi];
            if (!full) {
              launchPrims(c, b, nullptr, true, &rs[bi], i, s);
              if (c.phys.viscous) launchGradFlux(c, b, false, true, &rs[bi], i, false, s);
            }
            if (functional) launchFunctionalTangent(c, b, rl[bi], i, full, s);
            if (c.phys.dissipation) launchDissipation(c, b, b.v.lam, 1.0, s);
            launchLinearizedFlux(c, b, rl[bi], i, full, s);
          });
          forEachBlockConcurrently(c, [&](int bi, cudaStream_t s) {
            launchInterfaceSatLinearized(c, c.blocks[bi], refs, &rl[bi], i, full, s);
          });
          forEachBlockConcurrently(c, [&](int bi, cudaStream_t s) {
            launchLinearizedDivergence(c, c.blocks[bi], i, rl[bi], 0.0, i, deltaControl && bi == 0, s);
          });
        }
        launchStepAdvance(c, 1);
      }))
    return 1;
  const int nSeg = (T + S - 1) / S;
  for (int k = 0; k < nSeg; ++k) {
    const int L = k * S, end = std::min(T, L + S);
    if (!resident) {
      for (DevBlock& b : c.blocks) {
        CUDA_TRY(c, cudaMemcpyAsync(b.v.q, b.runSnap + (size_t)k * nU * b.v.N, (size_t)nU * b.v.N * sizeof(double),
                                    cudaMemcpyDeviceToDevice, c.stream));
        launchPrims(c, b, b.v.q, false);
      }
      launchSetCounters(c.dCounters, L + 1, L, c.stream);
      for (int s = L + 1; s <= end; ++s) CUDA_TRY(c, cudaGraphLaunch(gRec, c.stream));
      c.launches += 1 + (long long)(end - L) * nodesRec;
    }
    launchSetCounters(c.dCounters, L + 1, L, c.stream);
    for (int s = L + 1; s <= end; ++s) CUDA_TRY(c, cudaGraphLaunch(gLin, c.stream));
    c.launches += 1 + (long long)(end - L) * nodesLin;
  }
  for (size_t bi = 0; bi < c.blocks.size(); ++bi) {
    DevBlock& b = c.blocks[bi];
    CUDA_TRY(c, cudaMemcpyAsync(b.v.q, qFinal[bi], (size_t)nU * b.v.N * sizeof(double), cudaMemcpyDeviceToDevice,
                                c.stream));
    launchPrims(c, b, b.v.q, false);
    // the last stage's term, at the final state: the counters stand at step T + 1
    if (functional) launchFunctionalTangent(c, b, rl[bi], 1, false);
  }
  if (checkLaunch(c)) return 1;
  double dJ = 0.0;
  if (functional) {
    std::vector<double> vals;
    if (reduceRegion(c, 4 * T, vals)) return 1;
    for (int st = 0; st < T; ++st)
      for (int i = 0; i < 4; ++i) dJ = dJ + kRkNorm[i] * c.stepDt[st] * vals[(size_t)4 * st + i];
  }
  CUDA_TRY(c, cudaStreamSynchronize(c.stream));
  if (delta_cost) *delta_cost = dJ;
  return 0;
}

int mgd_tune_run(mgd_ctx* h, int n_steps, int save_interval, int with_adjoint, double* best_ms) {
  Context& c = h->c;
  if (requireReady(c)) return 1;
  if (n_steps < 1) return fail(c, "mgd_tune_run: n_steps must be >= 1");
  if (save_interval < 1) save_interval = n_steps;
  // the state and adjoint of every block, restored before every timed run and at the end
  std::vector<double*> saved;
  auto release = [&]() {
    for (double* p : saved) cudaFree(p);
  };
  for (auto& b : c.blocks) {
    double* p = nullptr;
    if (cudaMalloc((void**)&p, (size_t)2 * c.nU * b.v.N * sizeof(double)) != cudaSuccess) {
      release();
      return fail(c, "mgd_tune_run: out of device memory for the saved state");
    }
    saved.push_back(p);
    cudaMemcpyAsync(p, b.v.q, (size_t)c.nU * b.v.N * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(p + (size_t)c.nU * b.v.N, b.v.lam, (size_t)c.nU * b.v.N * sizeof(double),
                    cudaMemcpyDeviceToDevice, c.stream);
  }
  auto restore = [&]() {
    for (size_t i = 0; i < c.blocks.size(); ++i) {
      DevBlock& b = c.blocks[i];
      cudaMemcpyAsync(b.v.q, saved[i], (size_t)c.nU * b.v.N * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
      cudaMemcpyAsync(b.v.lam, saved[i] + (size_t)c.nU * b.v.N, (size_t)c.nU * b.v.N * sizeof(double),
                      cudaMemcpyDeviceToDevice, c.stream);
    }
    return cudaStreamSynchronize(c.stream) == cudaSuccess ? 0 : fail(c, "mgd_tune_run: state restore failed");
  };
  const long long launches = c.launches;
  // wall time of one forward (+ adjoint) run from the saved state
  auto runOnce = [&](double* ms) -> int {
    if (restore()) return 1;
    const auto t = std::chrono::steady_clock::now();
    double J = 0.0, G = 0.0;
    if (mgd_run_forward(h, n_steps, save_interval, 0.0, &J)) return 1;
    if (with_adjoint && mgd_run_adjoint(h, &G)) return 1;
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return fail(c, "mgd_tune_run: run failed");
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
    return 0;
  };
  auto timed = [&](double* ms) -> int {  // fastest of two runs
    double a = 0.0, b = 0.0;
    if (runOnce(&a) || runOnce(&b)) return 1;
    *ms = std::min(a, b);
    return 0;
  };
  std::vector<std::array<int, 3>> cands;
  // (2D also whole-warp tiles that are not powers of two: other CTA counts
  // per grid, which can spread a single wave more evenly over the SMs)
  if (c.nD == 2)
    cands = {{8, 8, 1}, {16, 4, 1}, {32, 2, 1}, {64, 1, 1}, {8, 16, 1}, {16, 8, 1},
             {32, 4, 1}, {64, 2, 1}, {128, 1, 1}, {16, 16, 1}, {32, 8, 1},
             {8, 12, 1}, {16, 6, 1}, {16, 10, 1}, {8, 20, 1}, {16, 12, 1}, {32, 6, 1},
             // one-warp tiles: four times the CTAs of the 128-point tiles, so
             // that a single wave of small grids spreads more evenly
             {8, 4, 1}, {4, 8, 1}, {16, 2, 1}};
  else
    cands = {{8, 4, 2}, {16, 2, 2}, {32, 2, 1}, {8, 8, 2}, {16, 4, 2}, {32, 2, 2}, {32, 4, 1},
             {16, 8, 1}, {8, 4, 4}, {64, 2, 1}, {16, 4, 4}};
  auto slotOf = [](DevBlock& b, int k) -> Tile& {
    Tile* s[6] = {&b.tGrad, &b.tDiss, &b.tRhs, &b.tAdjA, &b.tAdjD, &b.tAdjB};
    return *s[k];
  };
  auto setAll = [&](int k, const std::array<int, 3>& t, int lanes) {
    for (auto& b : c.blocks) {
      slotOf(b, k) = makeTile(b, t[0], t[1], t[2]);
      if (k == 0 && c.nD == 2) b.gradLanes = lanes;
      if (k == 3 && c.nD == 2) b.coreLanes = lanes;
    }
  };
  // the tiles and forms on entry, put back if a timed run fails
  struct Entry {
    std::array<Tile, 6> tiles;
    int gradLanes, coreLanes;
  };
  std::vector<Entry> entry;
  for (auto& b : c.blocks) {
    Entry e;
    for (int k = 0; k < 6; ++k) e.tiles[k] = slotOf(b, k);
    e.gradLanes = b.gradLanes;
    e.coreLanes = b.coreLanes;
    entry.push_back(e);
  }
  int rc = 0;
  double best = 0.0;
  for (int w = 0; w < 2 && !rc; ++w) rc = runOnce(&best);  // warm-up: clocks, graph buffers
  if (!rc) rc = timed(&best);
  for (int pass = 0; pass < 2 && !rc; ++pass)
    for (int k = 0; k < 6 && !rc; ++k) {
      if ((k == 1 && !c.phys.dissipation) || (k == 4 && !c.phys.viscous) || (k >= 3 && !with_adjoint)) continue;
      const Tile& cur = slotOf(c.blocks[0], k);
      std::array<int, 3> bestT = {cur.t[0], cur.t[1], cur.t[2]};
      int bestLanes = k == 3 ? c.blocks[0].coreLanes : c.blocks[0].gradLanes;
      // 2D: the gradient/flux kernel and the adjoint core also have a form
      // with one thread per point and direction
      const int forms = ((k == 0 || k == 3) && c.nD == 2) ? 2 : 1;
      for (int lf = 0; lf < forms && !rc; ++lf)
        for (const auto& t : cands) {
          setAll(k, t, lf + 1);
          double ms = 0.0;
          if ((rc = timed(&ms))) break;
          if (ms < best) {
            best = ms;
            bestT = t;
            bestLanes = lf + 1;
          }
        }
      setAll(k, bestT, bestLanes);
    }
  if (rc) {
    const std::string err = c.error;
    for (size_t i = 0; i < c.blocks.size(); ++i) {
      DevBlock& b = c.blocks[i];
      for (int k = 0; k < 6; ++k) slotOf(b, k) = entry[i].tiles[k];
      b.gradLanes = entry[i].gradLanes;
      b.coreLanes = entry[i].coreLanes;
    }
    c.error = err;
  }
  const int rr = restore();
  release();
  c.launches = launches;
  c.runSteps = 0;  // the tuning runs leave no trajectory for mgd_run_adjoint
  c.trajectorySteps = 0;
  if (rc || rr) return 1;
  for (auto& b : c.blocks) storeTuned(c, b);
  if (best_ms) *best_ms = best;
  return 0;
}
