// mgd_noalloc.cu -- a forward-RHS entry point that allocates no device memory.
//
// Who needs it: callers that must not allocate device memory at the moment
// they evaluate an RHS. Examples are a host solver that carved its whole
// device-memory budget out up front with its own pool allocator (so that a
// cudaMalloc here would fail or fragment its pool), and latency-sensitive
// loops that cannot afford cudaMalloc's implicit device synchronisation.
// mgd_forward_rhs_noalloc reads the caller's state and writes the caller's
// RHS buffer; every intermediate it needs (primitive variables,
// contravariant fluxes, the dissipation term, the SAT vectors of the
// boundary entries, the solenoidal-excitation values, the source amplitudes
// and the stage time) lives in one fixed array in device memory that is part
// of the library image, so the context's own state and run buffers stay as
// they were.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "mgd_internal.h"

using namespace mgd;

namespace {

// The scratch array. Every GPU that loads the library holds it until the
// process exits: 2^21 doubles = 16 MiB.
constexpr long long kNoAllocScratchDoubles = 1LL << 21;
static __device__ __align__(256) double g_noallocScratch[kNoAllocScratchDoubles];

// Device address of g_noallocScratch on each device. In host code the
// array's name is only a host-side stand-in, not a device address, so the
// address is obtained once per device with cudaGetSymbolAddress while that
// device is current, and passed to the kernels.
constexpr int kMaxDevices = 64;
double* g_scratchAddr[kMaxDevices] = {nullptr};
std::mutex g_scratchMutex;

cudaError_t scratchAddress(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratchMutex);
  if (!g_scratchAddr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess) return e;
    g_scratchAddr[device] = static_cast<double*>(p);
  }
  *out = g_scratchAddr[device];
  return cudaSuccess;
}

long long align32(long long n) { return (n + 31) & ~31LL; }

}  // namespace

int mgd_forward_rhs_noalloc(mgd_ctx* h, const double* q, double time, double* rhs) {
  Context& c = h->c;
  if (!c.finalized) {
    c.error = "mgd_finalize_setup has not been called";
    return 1;
  }
  if (!q || !rhs) {
    c.error = "mgd_forward_rhs_noalloc: q and rhs must be device pointers";
    return 1;
  }
  if (!singleBlockRegion(c)) {
    // regions of several blocks, or one block with block-interface patches
    // (an O-grid cut), need the interface SATs of mgd_compute_rhs
    c.error = "mgd_forward_rhs_noalloc: one block without block-interface patches per context; "
              "use mgd_compute_rhs for multi-block regions and interface patches";
    return 1;
  }
  DevBlock& b = c.blocks[0];
  const long long N = b.v.N;
  const int nD = c.nD, nU = c.nU;
  const PrimLayout L{nD};
  // scratch layout: [amplitudes, time | primitives | fluxes | dissipation |
  //                  SAT vectors | solenoidal-excitation values]
  long long nExcEntries = 0;
  for (const ExcPatch& x : b.exc) nExcEntries = std::max(nExcEntries, (long long)x.off + x.nE);
  const long long nAmp = align32(MGD_MAX_SOURCES + 1);
  const long long nPrim = align32(N * L.count());
  const long long nFlux = align32(N * nD * nU);
  const long long nDiss = align32(c.phys.composite ? N * nU : N * nD * nU);
  const long long nFF = align32((long long)b.v.ff.n * nU);
  const long long nExc = align32(3 * nExcEntries);
  const long long need = nAmp + nPrim + nFlux + nDiss + nFF + nExc;
  if (need > kNoAllocScratchDoubles) {
    c.error = "mgd_forward_rhs_noalloc: the block needs " + std::to_string(need) +
              " doubles of scratch but the fixed array holds " + std::to_string(kNoAllocScratchDoubles) +
              " (about 100k points in 2D, 55k in 3D); use mgd_compute_rhs";
    return 1;
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  double* scratch = nullptr;
  if (e == cudaSuccess) e = scratchAddress(device, &scratch);
  if (e != cudaSuccess) {
    c.error = std::string("mgd_forward_rhs_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
    return 1;
  }
  if (device != c.device) {
    c.error = "mgd_forward_rhs_noalloc: the context's device must be current";
    return 1;
  }
  // source amplitudes at `time` (AcousticSource%add, src/AcousticSourceImpl.f90:34-64)
  double amp[MGD_MAX_SOURCES] = {0};
  const double pi = 4.0 * std::atan(1.0);
  for (size_t s = 0; s < c.sources.size(); ++s) {
    const mgd_acoustic_source& src = c.sources[s];
    amp[s] = src.amplitude * std::cos(2.0 * pi * src.frequency * time + src.phase);
  }
  // the stage time follows the amplitudes (solenoidal excitation)
  double head[MGD_MAX_SOURCES + 1];
  std::memcpy(head, amp, sizeof amp);
  head[MGD_MAX_SOURCES] = time;
  e = cudaMemcpyAsync(scratch, head, sizeof head, cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) {
    c.error = std::string("mgd_forward_rhs_noalloc: ") + cudaGetErrorString(e);
    return 1;
  }
  // The existing kernels run on a view of the block whose state, output and
  // intermediates point at the caller's buffers and at the scratch array.
  // Each intermediate is written in full before it is read within this call,
  // so nothing in the array has to start at zero.
  BlockView view = b.v;
  view.q = const_cast<double*>(q);
  view.rhs = rhs;
  view.prim = scratch + nAmp;
  view.fhat = view.prim + nPrim;
  view.dq = view.fhat + nFlux;
  view.ff.visc = view.dq + nDiss;
  if (nExcEntries) view.excF = view.ff.visc + nFF;
  RunScalars rs{};
  rs.step = c.dCounters + 2;
  rs.segBase = c.dCounters + 3;
  rs.amp = scratch;
  rs.stageTime = scratch + MGD_MAX_SOURCES;
  setStepSize(rs, c.opts.time_step_size);
  rs.adjointForcingSwitch = c.opts.adjoint_forcing_switch;
  rs.nPartialBlocks = reductionBlocks(b);
  // the actuators' forcing of the per-call path, as mgd_compute_rhs adds it
  // (ActuatorPatch%updateRhs, src/ActuatorPatchImpl.f90:108-181)
  rs.apiForcing = perCallForcing(c);
  // The launchers read the block through b.v, so the view stands in for it
  // during this call. Calls on one context do not overlap (one calling
  // thread per context), so no other call sees the substitution.
  const BlockView saved = b.v;
  b.v = view;
  launchPrims(c, b, view.q, false);
  forwardStage(c, b, 0, rs, true, perCallController(c), false, false);
  b.v = saved;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) {
    c.error = std::string("mgd_forward_rhs_noalloc: ") + cudaGetErrorString(e);
    return 1;
  }
  return 0;
}
