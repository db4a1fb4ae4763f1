// mgd_kernels.cu -- FP64 kernels of the forward and discrete-adjoint RHS and
// the RK4 stage updates, plus the setup kernels (grid metrics, far-field SAT
// matrices). Stencil taps are read through the read-only cache.
//
// Forward RK stage: kGradFlux (one thread per point: gradients, stress,
// contravariant fluxes, far-field SAT vector) runs beside kDissipation (one
// thread per point and component); kForwardDivergence (one thread per point
// and component) adds the flux divergence, dissipation, SATs and sources and
// applies the RK update; kPrims refreshes the primitive variables and
// kFunctional sums the cost functional over the cost-target points.
// Adjoint RK stage: kAdjointCore (per point) beside kDissipation and
// kGradientSensitivity; kAdjointDiffusion and kAdjointAssemble (per point and
// component) finish the adjoint RHS and its RK update.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>

#include "mgd_internal.h"
#include "sbp_tables.h"

namespace mgd {


__device__ PowTables g_powTables;

static void uploadPowTables() {
  PowTables t;
  for (int j = 0; j < 128; ++j) {
    const long double F = 1.0L + (j + 0.5L) / 128.0L;
    t.invF[j] = (double)(1.0L / F);
    const long double L = -logl((long double)t.invF[j]);
    t.logFhi[j] = (double)L;
    t.logFlo[j] = (double)(L - (long double)t.logFhi[j]);
  }
  for (int j = 0; j < 64; ++j) t.exp2j[j] = (double)exp2l(j / 64.0L);
  cudaMemcpyToSymbol(g_powTables, &t, sizeof t);
}

constexpr int kBlock = 128;      // pointwise kernels
constexpr int kMaxTile = 256;    // largest stage-kernel tile
// Taps of a boundary closure row loaded together by the stage kernels: at
// 2D sizes the kernels are single waves whose edge tiles end last, so their
// closure rows issue four loads at a time; 3D kernels and the persistent
// batched kernel (NC = false, one register budget for all its phases) keep
// one at a time and the registers that saves.
template <int ND, bool NC = true>
constexpr int kClosureUnroll = (ND == 2 && NC) ? 4 : 1;

// Programmatic dependent launch: every kernel lets the next kernel in its
// stream start launching as soon as all of its own blocks are running, and
// waits for its predecessor to complete (and its memory to be visible) before
// touching memory. Kernels launched without the attribute pass straight through.
// Waiting before the trigger (early launch one kernel deep) measured about 1%
// slower in the 201x201 gradient and the batched sweep.
__device__ __forceinline__ void pdlEnter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Early launch pays off on a single stream (the forward run, batched runs);
// beside a concurrent stream the waiting blocks would hold SM slots that the
// other stream's kernels could use, so the checkpoint recomputation and the
// adjoint launch without it.
static thread_local bool t_programmaticLaunch = true;
static thread_local int t_launchPriority = 0;  // 0: the stream's own priority
static thread_local bool t_priorityOn = false;

void setProgrammaticLaunch(bool on) { t_programmaticLaunch = on; }
void setLaunchPriority(bool on, int priority) {
  t_priorityOn = on;
  t_launchPriority = priority;
}

// Attributes of a launch: programmatic stream serialization (when on) and
// the launch priority (when set).
static int launchAttributes(cudaLaunchAttribute* attr) {
  int n = 0;
  if (t_programmaticLaunch) {
    attr[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[n].val.programmaticStreamSerializationAllowed = 1;
    ++n;
  }
  if (t_priorityOn) {
    attr[n].id = cudaLaunchAttributePriority;
    attr[n].val.priority = t_launchPriority;
    ++n;
  }
  return n;
}

template <typename... KArgs, typename... Args>
static void pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  cfg.attrs = attr;
  cfg.numAttrs = launchAttributes(attr);
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// pdl with dynamic shared memory.
template <typename... KArgs, typename... Args>
static void pdlShared(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  cfg.attrs = attr;
  cfg.numAttrs = launchAttributes(attr);
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

static inline int gridFor(long long n) { return (int)((n + kBlock - 1) / kBlock); }

// rcp = floor(2^64 / d) + 1 for d >= 2 (0 for d = 1). For 32-bit x the
// quotient floor(x / d) is the high word of x * rcp: rcp d = 2^64 + e with
// 1 <= e <= d, so x rcp / 2^64 = x / d + x e / (d 2^64), and x e < 2^64 keeps
// the added term below 1/d, short of the next integer (division by invariant
// integers using multiplication, Granlund and Montgomery, 1994).
static unsigned long long reciprocal64(unsigned d) {
  if (d <= 1) return 0;
  // ~0ULL / d = floor((2^64 - 1) / d): one less than floor(2^64 / d) when d divides 2^64
  const unsigned long long f = ~0ULL / d + (((d & (d - 1)) == 0) ? 1 : 0);
  return f + 1;
}

Tile makeTile(const DevBlock& b, int tx, int ty, int tz) {
  Tile t;
  t.t[0] = tx; t.t[1] = b.v.nD >= 2 ? ty : 1; t.t[2] = b.v.nD >= 3 ? tz : 1;
  for (int d = 0; d < 3; ++d) t.n[d] = (b.v.gs[d] + t.t[d] - 1) / t.t[d];
  t.div[0] = (unsigned)t.t[0];
  t.div[1] = (unsigned)(t.t[0] * t.t[1]);
  t.div[2] = (unsigned)t.n[0];
  t.div[3] = (unsigned)(t.n[0] * t.n[1]);
  for (int k = 0; k < 4; ++k) t.rcp[k] = reciprocal64(t.div[k]);
  return t;
}


void uploadOperatorTables() {
  static bool done[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && done[dev]) return;
  OpTables t;
  std::memset(&t, 0, sizeof t);
  static double left[kSchemes][OP_COUNT][16 * 12], right[kSchemes][OP_COUNT][16 * 12];
  std::memset(left, 0, sizeof left);
  std::memset(right, 0, sizeof right);
  for (int sc = 0; sc < kSchemes; ++sc) {
    const SchemeOps so = schemeOps(sc);
    // every operator in the kernels' shapes (OpShape); the non-composite
    // transpose carries the inverse of the first-derivative norm
    HostOp ops[OP_COUNT];
    ops[OP_D1] = embed(so.d1, 8, 12, 4);
    ops[OP_D1ADJ] = embed(makeAdjoint(so.d1), 12, 16, 4);
    ops[OP_DCOMP] = embed(so.dcomp, 8, 12, 4);
    if (so.hasDissipation) {
      ops[OP_DISS] = embed(so.diss, 2, 5, 2);
      ops[OP_DISST] = embed(so.dissT, 8, 10, 2);
      foldNormInverse(ops[OP_DISST], so.d1.norm);
    }
    for (int o = 0; o < OP_COUNT; ++o) {
      const HostOp& h = ops[o];
      for (size_t j = 0; j < h.interior.size(); ++j) t.interior[sc][o][j] = h.interior[j];
      for (size_t j = 0; j < h.left.size(); ++j) left[sc][o][j] = h.left[j];
      for (size_t j = 0; j < h.right.size(); ++j) right[sc][o][j] = h.right[j];
      t.asym[sc][o] = h.asym ? 1 : 0;
    }
  }
  cudaMemcpyToSymbol(c_ops, &t, sizeof t);
  cudaMemcpyToSymbol(g_opLeft, left, sizeof left);
  cudaMemcpyToSymbol(g_opRight, right, sizeof right);
  uploadPowTables();
  if (dev < 64) done[dev] = true;
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
struct PointIndex {
  int idx[3];
  long long base[3];  // first point of the pencil through p along each axis
};

__device__ __forceinline__ PointIndex pointIndex(const BlockView& B, long long p) {
  PointIndex r;
  const long long plane = (long long)B.gs[0] * B.gs[1];
  r.idx[0] = (int)(p % B.gs[0]);
  r.idx[1] = (int)((p / B.gs[0]) % B.gs[1]);
  r.idx[2] = (int)(p / plane);
  for (int d = 0; d < 3; ++d) r.base[d] = p - (long long)r.idx[d] * B.ax[d].stride;
  return r;
}

// Grid point of this thread in tile-block b under tiling T; false when the
// tile overhangs the grid. Along each axis the tile order puts the two edge
// tiles first (0, n-1, 1, 2, ..., n-2): the edge tiles carry the boundary
// closures and the SAT work, and the block scheduler hands out low block
// indices first, so the heavy tiles spread over the SMs instead of landing,
// with the last block row, on a few of them at the end.
__device__ __forceinline__ int edgeTilesFirst(int k, int n) { return (k == 0 || n < 2) ? k : (k == 1 ? n - 1 : k - 1); }

__device__ __forceinline__ bool locateAt(const BlockView& B, const Tile& T, int b, int t, long long& p,
                                         PointIndex& r) {
  // x / d by multiply-high with the tile's reciprocals (x >= 0, 32-bit)
  auto q = [&](int x, int k) -> int {
    return T.div[k] == 1 ? x : (int)__umul64hi((unsigned long long)(unsigned)x, T.rcp[k]);
  };
  const int t0 = q(t, 0), b0 = q(b, 2);
  const int lx = t - t0 * T.t[0], lz = q(t, 1), ly = t0 - lz * T.t[1];
  const int bz0 = q(b, 3);
  const int bx = edgeTilesFirst(b - b0 * T.n[0], T.n[0]), by = edgeTilesFirst(b0 - bz0 * T.n[1], T.n[1]),
            bz = edgeTilesFirst(bz0, T.n[2]);
  r.idx[0] = bx * T.t[0] + lx;
  r.idx[1] = by * T.t[1] + ly;
  r.idx[2] = bz * T.t[2] + lz;
  if (r.idx[0] >= B.gs[0] || r.idx[1] >= B.gs[1] || r.idx[2] >= B.gs[2]) return false;
  p = r.idx[0] + (long long)B.gs[0] * (r.idx[1] + (long long)B.gs[1] * r.idx[2]);
  for (int d = 0; d < 3; ++d) r.base[d] = p - (long long)r.idx[d] * B.ax[d].stride;
  return true;
}

__device__ __forceinline__ bool locate(const BlockView& B, const Tile& T, int b, long long& p, PointIndex& r) {
  return locateAt(B, T, b, threadIdx.x, p, r);
}

// Primitive variables of one state (computeDependentVariables +
// computeTransportVariables, src/CNSHelperImpl.f90:3-177).
template <int ND>
__device__ __forceinline__ void primitives(const double* q, const Physics& P, double* out /*6+ND*/) {
  const double v = 1.0 / q[0];
  out[0] = v;
  double u2 = 0.0;
  for (int d = 0; d < ND; ++d) {
    const double u = v * q[1 + d];
    out[1 + d] = u;
    u2 = d == 0 ? u * u : u2 + u * u;
  }
  const double pr = P.gm1 * (q[ND + 1] - 0.5 * q[0] * u2);
  const double T = P.gOverGm1 * pr * v;
  out[1 + ND] = pr;
  out[2 + ND] = T;
  double mu = P.reInv;
  if (P.powerLaw) mu = fastPowPositive(P.gm1 * T, P.powerLawExponent, &g_powTables) * P.reInv;
  out[3 + ND] = mu;
  out[4 + ND] = P.laFactor * mu;
  out[5 + ND] = mu * P.prInv;
}

// Deterministic block sum of one value per thread; thread 0 gets the result.
__device__ __forceinline__ double blockSum(double v) {
  __shared__ double warpSums[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warpSums[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)((blockDim.x + 31) / 32); ++i) s += warpSums[i];
  return s;
}

// ---------------------------------------------------------------------------
// Primitive variables (State%update pointwise part, src/StateImpl.f90:466-492)
// ---------------------------------------------------------------------------
template <int ND>
__device__ __forceinline__ void primsPoint(const BlockView& B, const Physics& P, const double* __restrict__ qSrc,
                                           int copyToQ, const RunScalars& rs, int stage, int blk) {
  const long long p = (long long)blk * kBlock + threadIdx.x;
  if (p >= B.N) return;
  constexpr int nU = ND + 2;
  if (stage > 0) {
    const int slot = ((*rs.step) - (*rs.segBase) - 1) * 4 + stage - 1;
    qSrc = rs.stageBuf + (long long)slot * rs.slotStride;
  }
  double q[nU], pr[6 + ND];
  for (int c = 0; c < nU; ++c) q[c] = qSrc[p + B.N * c];
  if (copyToQ)
    for (int c = 0; c < nU; ++c) B.q[p + B.N * c] = q[c];
  primitives<ND>(q, P, pr);
  for (int c = 0; c < 6 + ND; ++c) B.prim[p + B.N * c] = pr[c];
}

template <int ND>
__global__ void __launch_bounds__(kBlock) kPrims(BlockView B, Physics P, const double* __restrict__ qSrc,
                                                 int copyToQ, RunScalars rs, int stage) {
  pdlEnter();
  primsPoint<ND>(B, P, qSrc, copyToQ, rs, stage, blockIdx.x);
}

// Forward-state arrays seen by the adjoint kernels: the block's own arrays, or
// the stage-buffer slot of the current step and stage when the checkpoint
// recomputation stored primitives, stress and heat flux with the state.
struct FwdState {
  const double* q;
  const double* prim;
  const double* tau;
  const double* hf;
};

template <int ND>
__device__ __forceinline__ FwdState forwardState(const BlockView& B, const RunScalars& rs, int stage, bool fromSlot) {
  if (!fromSlot) return {B.q, B.prim, B.tau, B.hf};
  const int slot = ((*rs.step) - (*rs.segBase) - 1) * 4 + stage - 1;
  const double* base = rs.stageBuf + (long long)slot * rs.slotStride;
  const long long N = B.N;
  const double* prim = base + (ND + 2) * N;
  const double* tau = prim + (6 + ND) * N;
  return {base, prim, tau, tau + ND * ND * N};
}

// ---------------------------------------------------------------------------
// Wall SAT vectors of one entry (addImpenetrableWallPenalty,
// src/ImpenetrableWallImpl.f90:58-213, and the viscous penalty of
// addIsothermalWallPenalty, src/IsothermalWallImpl.f90:92-260; the adiabatic
// wall adds the impenetrable penalty only, src/AdiabaticWallImpl.f90:80-160).
// Forward: sat = -s_inv J [m.rho u, (m.rho u) u, (m.rho u) v (E + p)]
//                - s_visc J [0, rho u, E - rho T_w / gamma].
// Adjoint: sat = s_inv J (A(m) - m (dp/dq))^T lambda
//                + s_visc J [-lambda_E T_w / gamma, lambda_1 .. lambda_E].
// ---------------------------------------------------------------------------
template <int ND, bool VISC>
__device__ __forceinline__ void wallSatForward(const BlockView& B, const Physics& P, int e, long long p,
                                               const double* q, const double* u, double* sat) {
  constexpr int nU = ND + 2, E = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  double mn[ND];
  for (int d = 0; d < ND; ++d) mn[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
  double nm = q[1] * mn[0];
  for (int d = 1; d < ND; ++d) nm += q[1 + d] * mn[d];
  const double s = B.ff.wallInv[e];
  sat[0] = -(s * nm);
  for (int d = 0; d < ND; ++d) sat[1 + d] = -(s * (nm * u[d]));
  sat[E] = -(s * (nm * B.prim[p + N * L.v()] * (q[E] + B.prim[p + N * L.p()])));
  if (VISC && B.ff.kind[e] == SAT_ISOTHERMAL_WALL) {
    const double sv = B.ff.wallVisc[e];
    for (int c = 1; c < E; ++c) sat[c] -= sv * q[c];
    sat[E] -= sv * (q[E] - q[0] * B.ff.wallT[e] / P.g);
  }
  (void)nU;
}

template <int ND, bool VISC>
__device__ __forceinline__ void wallSatAdjoint(const BlockView& B, const Physics& P, int e, long long p,
                                               const double* u, double T, double v, const double* lam,
                                               double* sat) {
  constexpr int nU = ND + 2, E = ND + 1;
  const long long N = B.N;
  double mn[ND];
  for (int d = 0; d < ND; ++d) mn[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
  double y[nU];
  for (int c = 0; c < nU; ++c) y[c] = 0.0;
  addFluxJacobianTransposeProduct<ND, false>(mn, u, T, v, P, 0.0, nullptr, nullptr, lam, y);
  // minus sum_l m_l (dp/dq) lambda_{1+l}, dp/dq = (gamma - 1) (|u|^2 / 2, -u, 1)
  double ml = mn[0] * lam[1];
  for (int l = 1; l < ND; ++l) ml += mn[l] * lam[1 + l];
  double u2 = u[0] * u[0];
  for (int d = 1; d < ND; ++d) u2 += u[d] * u[d];
  const double gm1 = P.g - 1.0;
  y[0] -= (0.5 * u2 * gm1) * ml;
  for (int d = 0; d < ND; ++d) y[1 + d] -= (-u[d] * gm1) * ml;
  y[E] -= gm1 * ml;
  const double s = B.ff.wallInv[e];
  for (int c = 0; c < nU; ++c) sat[c] = s * y[c];
  if (VISC && B.ff.kind[e] == SAT_ISOTHERMAL_WALL) {
    const double sv = B.ff.wallVisc[e];
    sat[0] += sv * (-lam[E] * B.ff.wallT[e] / P.g);
    for (int c = 1; c < nU; ++c) sat[c] += sv * lam[c];
  }
}

// ---------------------------------------------------------------------------
// Velocity and temperature gradients, stress and heat flux (State%update,
// src/StateImpl.f90:494-533 with Grid%computeGradient, src/GridImpl.f90:1172-1421),
// Cartesian inviscid and viscous fluxes transformed to contravariant form
// (computeRhsForward, src/RhsHelperImpl.f90:295-339), and the complete
// far-field SAT vector of each boundary point (src/FarFieldPatchImpl.f90:227-235).
// ---------------------------------------------------------------------------
enum { GF_FLUX = 1, GF_STRESS = 4, GF_STORE = 8 };

// LANES = 2 (2D only): two adjacent lanes per point. Lane d applies the
// derivative stencils along axis d and the pair swaps its three results by
// shuffle, which halves the dependent stencil loads of each thread; both
// lanes then form stress and fluxes, lane d writes the contravariant flux of
// direction d, and the stores of the stage slot and the SAT vectors are split
// between the lanes.
template <int ND, bool CURV, bool VISC, int LANES = 1, bool NC = true>
__device__ __forceinline__ void gradFluxPoint(const BlockView& B, const Physics& P, const RunScalars& rs, int flags,
                                              int stage, const Tile& T, int blk) {
  static_assert(LANES == 1 || (LANES == 2 && ND == 2), "two lanes per point only in 2D");
  const int lane = LANES == 2 ? (int)(threadIdx.x & 1) : 0;
  long long p;
  PointIndex I;
  if (!locateAt(B, T, blk, LANES == 2 ? (int)(threadIdx.x >> 1) : (int)threadIdx.x, p, I)) return;
  constexpr int nU = ND + 2, E = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  double q[nU];
  for (int c = 0; c < nU; ++c) q[c] = B.q[p + N * c];
  double* slot = nullptr;
  if (flags & GF_STORE) {
    const int s = ((*rs.step) - (*rs.segBase) - 1) * 4 + stage - 1;
    slot = rs.stageBuf + (long long)s * rs.slotStride;
    if (lane == 0)
      for (int c = 0; c < nU; ++c) slot[p + N * c] = q[c];
    if (rs.slotFull && lane == LANES - 1)
      for (int c = 0; c < 6 + ND; ++c) slot[p + N * (nU + c)] = B.prim[p + N * c];
  }
  double m[ND * ND];
  for (int c = 0; c < ND * ND; ++c) m[c] = (CURV || (c % (ND + 1)) == 0) ? B.metrics[p + N * c] : 0.0;
  double u[ND];
  for (int d = 0; d < ND; ++d) u[d] = B.prim[p + N * L.u(d)];
  double tau[ND * ND], hf[ND];
  if (VISC && (flags & (GF_FLUX | GF_STRESS))) {
    const double jac = B.jac[p];
    double du[ND][ND], dT[ND];
    if constexpr (LANES == 2) {
      const int d = lane;
      const long long bd = d ? I.base[1] : I.base[0];
      const int id = d ? I.idx[1] : I.idx[0];
      const Axis ax = d ? B.ax[1] : B.ax[0];
      const double a0 = applyOp<OP_D1, NC, kClosureUnroll<ND, NC>>(B.prim + N * L.u(0) + bd, id, ax);
      const double a1 = applyOp<OP_D1, NC, kClosureUnroll<ND, NC>>(B.prim + N * L.u(1) + bd, id, ax);
      const double aT = applyOp<OP_D1, NC, kClosureUnroll<ND, NC>>(B.prim + N * L.T() + bd, id, ax);
      const unsigned pair = 3u << (threadIdx.x & 30);
      const double b0 = __shfl_xor_sync(pair, a0, 1);
      const double b1 = __shfl_xor_sync(pair, a1, 1);
      const double bT = __shfl_xor_sync(pair, aT, 1);
      du[0][0] = d ? b0 : a0; du[0][1] = d ? a0 : b0;
      du[1][0] = d ? b1 : a1; du[1][1] = d ? a1 : b1;
      dT[0] = d ? bT : aT; dT[1] = d ? aT : bT;
    } else {
#pragma unroll
      for (int d = 0; d < ND; ++d) {
#pragma unroll
        for (int c = 0; c < ND; ++c) du[c][d] = applyOp<OP_D1, NC, kClosureUnroll<ND, NC>>(B.prim + N * L.u(c) + I.base[d], I.idx[d], B.ax[d]);
        dT[d] = applyOp<OP_D1, NC, kClosureUnroll<ND, NC>>(B.prim + N * L.T() + I.base[d], I.idx[d], B.ax[d]);
      }
    }
    double gu[ND][ND], gT[ND];
    for (int x = 0; x < ND; ++x) {
      if (CURV) {
        for (int c = 0; c < ND; ++c) {
          double s = m[x] * du[c][0];
          for (int d = 1; d < ND; ++d) s += m[ND * d + x] * du[c][d];
          gu[c][x] = jac * s;
        }
        double s = m[x] * dT[0];
        for (int d = 1; d < ND; ++d) s += m[ND * d + x] * dT[d];
        gT[x] = jac * s;
      } else {
        const double jm = jac * m[ND * x + x];
        for (int c = 0; c < ND; ++c) gu[c][x] = jm * du[c][x];
        gT[x] = jm * dT[x];
      }
    }
    const double mu = B.prim[p + N * L.mu()], la = B.prim[p + N * L.la()], kd = B.prim[p + N * L.k()];
    double div = gu[0][0];
    for (int d = 1; d < ND; ++d) div += gu[d][d];
    div = la * div;
    for (int c = 0; c < ND; ++c) {
      tau[ND * c + c] = 2.0 * mu * gu[c][c] + div;
      for (int d = c + 1; d < ND; ++d) {
        const double t = mu * (gu[c][d] + gu[d][c]);
        tau[ND * c + d] = t;
        tau[ND * d + c] = t;
      }
    }
    for (int x = 0; x < ND; ++x) hf[x] = -kd * gT[x];
    if (flags & GF_STRESS) {
      if (lane == 0)
        for (int c = 0; c < ND * ND; ++c) B.tau[p + N * c] = tau[c];
      if (lane == LANES - 1)
        for (int x = 0; x < ND; ++x) B.hf[p + N * x] = hf[x];
    }
    if (slot && rs.slotFull) {
      double* st = slot + N * (nU + 6 + ND);
      if (lane == 0)
        for (int c = 0; c < ND * ND; ++c) st[p + N * c] = tau[c];
      if (lane == LANES - 1)
        for (int x = 0; x < ND; ++x) st[p + N * (ND * ND + x)] = hf[x];
    }
  }
  if (flags & GF_FLUX) {
    const double pr = B.prim[p + N * L.p()];
    double F[nU][ND];
    for (int d = 0; d < ND; ++d) {
      F[0][d] = q[1 + d];
      for (int c = 0; c < ND; ++c) {
        double v = c < d ? q[1 + c] * u[d] : q[1 + d] * u[c];
        if (c == d) v = v + pr;
        F[1 + c][d] = v;
      }
      F[E][d] = u[d] * (q[E] + pr);
    }
    double Fv[nU][ND];
    if (VISC) {
      for (int d = 0; d < ND; ++d) {
        Fv[0][d] = 0.0;
        for (int c = 0; c < ND; ++c) Fv[1 + c][d] = tau[ND * c + d];
        double e = u[0] * tau[d];
        for (int c = 1; c < ND; ++c) e += u[c] * tau[ND * c + d];
        Fv[E][d] = e - hf[d];
      }
    }
    for (int s = 0; s < 3 && lane == 0; ++s) {
      const int e = B.ffOfPoint[3 * p + s];
      if (e < 0) continue;
      if (B.ff.kind[e] == SAT_INTERFACE) {
        // viscousFluxesL = sum_j F_v(:, j) m_L,j (src/BlockInterfacePatchImpl.f90:645-653);
        // the SAT vector itself needs the partner block (kInterfaceSat)
        if (VISC) {
          double mn[ND];
          for (int d = 0; d < ND; ++d) mn[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
          double* out = B.ff.ifVisc + (long long)e * nU;
          out[0] = 0.0;
          for (int r = 1; r < nU; ++r) {
            double f = Fv[r][0] * mn[0];
            for (int d = 1; d < ND; ++d) f += Fv[r][d] * mn[d];
            out[r] = f;
          }
        }
        continue;
      }
      if (B.ff.kind[e] != SAT_FAR_FIELD) {
        wallSatForward<ND, VISC>(B, P, e, p, q, u, B.ff.visc + (long long)e * nU);
        continue;
      }
      // sat = -sigma_inv J A+ (q - q_target) + sigma_visc J (F_v - F_v,target) . m
      const double* M = B.ff.M + (long long)e * nU * nU;
      double dqv[nU];
      for (int c = 0; c < nU; ++c) dqv[c] = q[c] - B.qt[p + N * c];
      double mn[ND];  // metric row of the normal direction, read from memory (no dynamic register index)
      for (int d = 0; d < ND; ++d) mn[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
      for (int r = 0; r < nU; ++r) {
        double t = M[r] * dqv[0];
        for (int c = 1; c < nU; ++c) t += M[r + nU * c] * dqv[c];
        double sat = -t;
        if (VISC) {
          double f = Fv[r][0] * mn[0];
          for (int d = 1; d < ND; ++d) f += Fv[r][d] * mn[d];
          sat += B.ff.sigV[e] * (f - B.ff.viscT[(long long)e * nU + r]);
        }
        B.ff.visc[(long long)e * nU + r] = sat;
      }
    }
    if (VISC)
      for (int r = 1; r < nU; ++r)
        for (int d = 0; d < ND; ++d) F[r][d] = F[r][d] - Fv[r][d];
    if constexpr (LANES == 2) {
      const int i = lane;
      for (int c = 0; c < nU; ++c) {
        const double s = CURV ? (i ? m[2] : m[0]) * F[c][0] + (i ? m[3] : m[1]) * F[c][1]
                              : (i ? m[3] : m[0]) * (i ? F[c][1] : F[c][0]);
        B.fhat[p + N * (i * nU + c)] = s;
      }
    } else {
      for (int i = 0; i < ND; ++i)
        for (int c = 0; c < nU; ++c) {
          double s;
          if (CURV) {
            s = m[ND * i] * F[c][0];
            for (int d = 1; d < ND; ++d) s += m[ND * i + d] * F[c][d];
          } else {
            s = m[ND * i + i] * F[c][i];
          }
          B.fhat[p + N * (i * nU + c)] = s;
        }
    }
  }
}

template <int ND, bool CURV, bool VISC>
__global__ void __launch_bounds__(kMaxTile) kGradFlux(BlockView B, Physics P, RunScalars rs, int flags,
                                                      int stage, Tile T) {
  pdlEnter();
  gradFluxPoint<ND, CURV, VISC>(B, P, rs, flags, stage, T, blockIdx.x);
}

template <bool CURV, bool VISC>
__global__ void __launch_bounds__(2 * kMaxTile) kGradFluxPair(BlockView B, Physics P, RunScalars rs, int flags,
                                                              int stage, Tile T) {
  pdlEnter();
  gradFluxPoint<2, CURV, VISC, 2>(B, P, rs, flags, stage, T, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Artificial dissipation (addDissipation, src/RhsHelperImpl.f90:10-87), one
// thread per point and component. Composite: dq_c = sign * amount * sum_i
// Dc_i src_c. Non-composite, first sweep: dq_{i,c} = sign * (-amount arc_i) D_i src_c.
// ---------------------------------------------------------------------------
// comp < 0: the component is blockIdx.y (a launch over (tiles, components)).
template <int ND, bool NC = true>
__device__ __forceinline__ void dissipationPoint(const BlockView& B, const Physics& P, const double* __restrict__ src,
                                                 double sign, const Tile& T, int blk, int comp = -1) {
  long long p;
  PointIndex I;
  if (!locate(B, T, blk, p, I)) return;
  constexpr int nU = ND + 2;
  const int c = comp >= 0 ? comp : (int)blockIdx.y;
  const long long N = B.N;
  const double* x = src + N * c;
  if (P.composite) {
    double s = applyOp<OP_DCOMP, NC, kClosureUnroll<ND, NC>>(x + I.base[0], I.idx[0], B.ax[0]);
    for (int d = 1; d < ND; ++d) s += applyOp<OP_DCOMP, NC, kClosureUnroll<ND, NC>>(x + I.base[d], I.idx[d], B.ax[d]);
    B.dq[p + N * c] = (sign * P.dissipationAmount) * s;
  } else {
    for (int d = 0; d < ND; ++d)
      B.dq[p + N * (d * nU + c)] =
          (sign * B.arcA[p + N * d]) * applyOp<OP_DISS, NC, kClosureUnroll<ND, NC>>(x + I.base[d], I.idx[d], B.ax[d]);
  }
}

template <int ND>
__global__ void __launch_bounds__(kMaxTile) kDissipation(BlockView B, Physics P, const double* __restrict__ src,
                                                         double sign, Tile T) {
  pdlEnter();
  dissipationPoint<ND>(B, P, src, sign, T, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Composite dissipation of 3D blocks that are PLANE-periodic along all three
// axes, with the operands staged in shared memory by the tensor memory
// accelerator (cp.async.bulk.tensor). A CTA owns a TX x TY column of points
// (32 x 8 with 16 planes per CTA ran fastest at 128^3 among 32 x 16 and
// 32 x 8 columns with 8, 16 or 32 planes) and marches through ZC planes of it: a ring of RING planes of the column
// (z - 4 .. z + 4 and the one being prefetched) feeds the z stencil, and the
// four halo strips of the current plane (4 points beyond each x and y edge,
// their coordinates wrapped, so that no copy leaves the grid or overlaps
// another) feed the x and y stencils. Each tap then reads shared memory
// instead of global memory. The arithmetic, its order included, is that of
// dissipationPoint (periodic interior stencil of each axis, x + y + z, times
// sign x amount). One elected thread issues the copies; every wait on a copy
// is bounded, and a wait that runs out sets *err, waits (bounded) for the
// CTA's copies in flight and leaves.
// ---------------------------------------------------------------------------
namespace tmadiss {
#ifndef MGD_TMA_TX
#define MGD_TMA_TX 32
#endif
#ifndef MGD_TMA_TY
#define MGD_TMA_TY 8
#endif
#ifndef MGD_TMA_ZC
#define MGD_TMA_ZC 16
#endif
constexpr int TX = MGD_TMA_TX, TY = MGD_TMA_TY, H = 4, ZC = MGD_TMA_ZC, RING = 2 * H + 2;
constexpr int PLANE = TX * TY, STRIP_X = H * TY, STRIP_Y = TX * H;
constexpr int HALO = 2 * STRIP_X + 2 * STRIP_Y;  // left, right, bottom, top
constexpr unsigned PLANE_BYTES = PLANE * 8, HALO_BYTES = HALO * 8;
constexpr size_t SMEM = (size_t)(RING * PLANE + 2 * HALO) * 8 + (RING + 2) * 8 + 128;
}  // namespace tmadiss

__device__ __forceinline__ unsigned smemAddr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbarInit(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbarExpectTx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
               : "memory");
}

// Polls the barrier's phase with the given parity; false after `limit` polls.
__device__ __forceinline__ bool mbarWait(unsigned long long* bar, unsigned parity, long long limit) {
  const unsigned a = smemAddr(bar);
  for (long long k = 0; k < limit; ++k) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// A (x, y, z, component) box of the 4D tensor map into shared memory,
// completing on the barrier.
__device__ __forceinline__ void tmaLoad4(void* dst, const CUtensorMap* map, int x, int y, int z, int c,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smemAddr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(c), "r"(smemAddr(bar))
      : "memory");
}

__global__ void __launch_bounds__(tmadiss::TX* tmadiss::TY)
    kDissipationTma3(BlockView B, Physics P, const __grid_constant__ CUtensorMap mapC,
                     const __grid_constant__ CUtensorMap mapX, const __grid_constant__ CUtensorMap mapY, double sign,
                     int* err, long long limit) {
  using namespace tmadiss;
  pdlEnter();
  extern __shared__ unsigned char smemRaw[];
  // 128-byte aligned buffers: the ring of planes, two halo sets, the barriers
  double* ring = reinterpret_cast<double*>((reinterpret_cast<size_t>(smemRaw) + 127) & ~size_t(127));
  double* halo = ring + RING * PLANE;
  unsigned long long* barC = reinterpret_cast<unsigned long long*>(halo + 2 * HALO);
  unsigned long long* barH = barC + RING;
  const int nx = B.gs[0], ny = B.gs[1], nz = B.gs[2];
  const int tilesX = nx / TX;
  const int x0 = (blockIdx.x % tilesX) * TX, y0 = (blockIdx.x / tilesX) * TY, z0 = blockIdx.y * ZC;
  const int comp = blockIdx.z;
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const bool leader = threadIdx.x == 0;
  auto wrap = [](int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); };
  // plane z0 - H + k lives in ring slot k % RING; its fills so far give the parity
  auto loadPlane = [&](int k) {
    const int slot = k % RING;
    mbarExpectTx(&barC[slot], PLANE_BYTES);
    tmaLoad4(ring + slot * PLANE, &mapC, x0, y0, wrap(z0 - H + k, nz), comp, &barC[slot]);
  };
  auto loadHalo = [&](int i) {  // the halo strips of plane z0 + i into set i % 2
    const int set = i % 2, z = z0 + i;
    double* h = halo + set * HALO;
    mbarExpectTx(&barH[set], HALO_BYTES);
    tmaLoad4(h, &mapX, wrap(x0 - H, nx), y0, z, comp, &barH[set]);
    tmaLoad4(h + STRIP_X, &mapX, wrap(x0 + TX, nx), y0, z, comp, &barH[set]);
    tmaLoad4(h + 2 * STRIP_X, &mapY, x0, wrap(y0 - H, ny), z, comp, &barH[set]);
    tmaLoad4(h + 2 * STRIP_X + STRIP_Y, &mapY, x0, wrap(y0 + TY, ny), z, comp, &barH[set]);
  };
  if (leader) {
    for (int k = 0; k < RING; ++k) mbarInit(&barC[k], 1);
    mbarInit(&barH[0], 1);
    mbarInit(&barH[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (leader) {
    for (int k = 0; k <= 2 * H; ++k) loadPlane(k);
    loadHalo(0);
  }
  const double* __restrict__ cin = c_ops.interior[B.ax[0].scheme][OP_DCOMP];
  const double f = sign * P.dissipationAmount;
  const long long N = B.N;
  // bounded drain of every copy issued up to iteration i (after a wait ran out)
  auto drain = [&](int i) {
    for (int k = 0; k < RING && k <= i + 2 * H + 1; ++k) {
      const int last = k + ((i + 2 * H + 1 - k) / RING) * RING;  // the slot's latest fill
      if (last <= i + 2 * H + 1) mbarWait(&barC[k], (last / RING) & 1, limit);
    }
    for (int j = (i > 0 ? i - 1 : 0); j <= i + 1 && j < ZC; ++j) mbarWait(&barH[j % 2], (j / 2) & 1, limit);
  };
  // Each plane's fill is waited for once, when it first enters the stencil
  // (the first iteration waits for the nine the prologue loaded); one CTA
  // barrier per iteration both closes the previous iteration's reads of the
  // buffers refilled next and votes on whether any wait ran out.
  bool ok = true;
  for (int i = 0; i < ZC; ++i) {
    if (__syncthreads_or(!ok)) {
      if (leader) atomicExch(err, 1);
      drain(i);
      return;
    }
    // prefetch the next plane of the ring and the next halo set; both buffers
    // were last read in iteration i - 1, which the barrier above closed
    if (leader && i + 1 < ZC) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      loadPlane(i + 2 * H + 1);
      loadHalo(i + 1);
    }
    for (int k = (i == 0 ? 0 : i + 2 * H); k <= i + 2 * H; ++k)
      ok = ok && mbarWait(&barC[k % RING], (k / RING) & 1, limit);
    ok = ok && mbarWait(&barH[i % 2], (i / 2) & 1, limit);
    const double* c0 = ring + ((i + H) % RING) * PLANE;
    const double* h = halo + (i % 2) * HALO;
    const int q = ty * TX + tx;
    auto xAt = [&](int d) {  // value at x offset d in [-H, H] of the current plane
      const int xx = tx + d;
      if (xx < 0) return h[ty * H + xx + H];
      if (xx >= TX) return h[STRIP_X + ty * H + xx - TX];
      return c0[ty * TX + xx];
    };
    auto yAt = [&](int d) {
      const int yy = ty + d;
      if (yy < 0) return h[2 * STRIP_X + (yy + H) * TX + tx];
      if (yy >= TY) return h[2 * STRIP_X + STRIP_Y + (yy - TY) * TX + tx];
      return c0[yy * TX + tx];
    };
    auto zAt = [&](int d) { return ring[((i + H + d) % RING) * PLANE + q]; };
    double sx = cin[H + 1] * (xAt(1) + xAt(-1));
#pragma unroll
    for (int j = 2; j <= H; ++j) sx += cin[H + j] * (xAt(j) + xAt(-j));
    sx = sx + cin[H] * c0[q];
    double sy = cin[H + 1] * (yAt(1) + yAt(-1));
#pragma unroll
    for (int j = 2; j <= H; ++j) sy += cin[H + j] * (yAt(j) + yAt(-j));
    sy = sy + cin[H] * c0[q];
    double sz = cin[H + 1] * (zAt(1) + zAt(-1));
#pragma unroll
    for (int j = 2; j <= H; ++j) sz += cin[H + j] * (zAt(j) + zAt(-j));
    sz = sz + cin[H] * c0[q];
    double s = sx;
    s += sy;
    s += sz;
    const long long p = (x0 + tx) + (long long)nx * ((y0 + ty) + (long long)ny * (z0 + i));
    B.dq[p + N * comp] = f * s;
  }
  if (__syncthreads_or(!ok)) {
    if (leader) atomicExch(err, 1);
    drain(ZC - 1);
  }
}

// Whether a block's composite dissipation can run as kDissipationTma3.
bool tmaDissipationEligible(const Context& c, const DevBlock& b) {
  using namespace tmadiss;
  if (c.nD != 3 || !c.phys.dissipation || !c.phys.composite || !c.useTmaDissipation) return false;
  for (int d = 0; d < 3; ++d)
    if (b.v.ax[d].per != 1) return false;
  return b.v.gs[0] % TX == 0 && b.v.gs[1] % TY == 0 && b.v.gs[2] % ZC == 0 && b.v.gs[0] >= TX &&
         b.v.gs[1] >= TY && b.v.gs[2] >= 2 * H + 1;
}

// The 4D (x, y, z, component) tensor map of nComp component planes of a
// block starting at base, with the given box.
static bool encodeTensorMap(const DevBlock& b, const double* base, int nComp, unsigned boxX, unsigned boxY,
                            CUtensorMap* out) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t dims[4] = {(cuuint64_t)b.v.gs[0], (cuuint64_t)b.v.gs[1], (cuuint64_t)b.v.gs[2],
                              (cuuint64_t)nComp};
  const cuuint64_t strides[3] = {(cuuint64_t)b.v.gs[0] * 8, (cuuint64_t)b.v.gs[0] * b.v.gs[1] * 8,
                                 (cuuint64_t)b.v.N * 8};
  const cuuint32_t box[4] = {boxX, boxY, 1, 1};
  const cuuint32_t elem[4] = {1, 1, 1, 1};
  return encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<double*>(base), dims, strides, box, elem,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launches kDissipationTma3 on src; false (nothing launched) when the tensor
// maps cannot be made.
static bool launchDissipationTma(Context& c, DevBlock& b, const double* src, double sign, cudaStream_t st) {
  using namespace tmadiss;
  CUtensorMap mapC, mapX, mapY;
  if (!encodeTensorMap(b, src, c.nU, TX, TY, &mapC) || !encodeTensorMap(b, src, c.nU, H, TY, &mapX) ||
      !encodeTensorMap(b, src, c.nU, TX, H, &mapY))
    return false;
  const dim3 grid((b.v.gs[0] / TX) * (b.v.gs[1] / TY), b.v.gs[2] / ZC, c.nU);
  static bool smemSet = false;
  if (!smemSet) {
    // column shapes whose buffers exceed the default 48 KB of dynamic shared memory
    if (cudaFuncSetAttribute(kDissipationTma3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM) !=
        cudaSuccess)
      return false;
    smemSet = true;
  }
  ++c.launches;
  pdlShared(kDissipationTma3, grid, TX * TY, SMEM, st, b.v, c.phys, mapC, mapX, mapY, sign, c.dKernelError,
            (long long)1 << 24);
  c.tmaLaunched = true;
  return true;
}

template <int ND, bool NC = true>
__device__ __forceinline__ double dissipationTerm(const BlockView& B, const Physics& P, const PointIndex& I,
                                                  long long p, int c) {
  constexpr int nU = ND + 2;
  const long long N = B.N;
  if (P.composite) return B.dq[p + N * c];
  double s = applyOp<OP_DISST, NC, kClosureUnroll<ND, NC>>(B.dq + N * c + I.base[0], I.idx[0], B.ax[0]);
  for (int i = 1; i < ND; ++i) s += applyOp<OP_DISST, NC, kClosureUnroll<ND, NC>>(B.dq + N * (i * nU + c) + I.base[i], I.idx[i], B.ax[i]);
  return s;
}

// ---------------------------------------------------------------------------
// Forward RHS of one component (computeRhsForward + Region%computeRhs,
// src/RhsHelperImpl.f90:330-351, src/RegionImpl.f90:1968-2023) fused with
// that component's RK4 forward stage update (src/RK4IntegratorImpl.f90:104-158).
// ---------------------------------------------------------------------------
// comp < 0: the component is blockIdx.y (a launch over (tiles, components)).
template <int ND, bool NC = true>
__device__ __forceinline__ void forwardDivergencePoint(const BlockView& B, const Physics& P, const RunScalars& rs,
                                                       int rkStage, int stage, int controller, const Tile& T,
                                                       int blk, int lin = 0, double linFactor = 0.0,
                                                       int comp = -1) {
  // after a solution-limit violation in this run the state stays as it is
  if (rkStage > 0 && rs.limitKey && *rs.limitKey != kNoLimitViolation) return;
  long long p;
  PointIndex I;
  if (!locate(B, T, blk, p, I)) return;
  constexpr int nU = ND + 2, E = ND + 1;
  const int c = comp >= 0 ? comp : (int)blockIdx.y;
  const long long N = B.N;
  double s = applyOp<OP_D1, NC, kClosureUnroll<ND, NC>>(B.fhat + N * c + I.base[0], I.idx[0], B.ax[0]);
  for (int i = 1; i < ND; ++i) s += applyOp<OP_D1, NC, kClosureUnroll<ND, NC>>(B.fhat + N * (i * nU + c) + I.base[i], I.idx[i], B.ax[i]);
  double r = -s;
  if (P.dissipation) r += dissipationTerm<ND, NC>(B, P, I, p, c);
  r = r * B.jac[p];
  for (int k = 0; k < 3; ++k) {
    const int e = B.ffOfPoint[3 * p + k];
    if (e >= 0) r += B.ff.visc[(long long)e * nU + c];
  }
  const long long kc = p + N * c;
  const double q = B.q[kc];
  const double S = B.sponge[p];
  if (lin) {
    // linearized: the sponge acts on the perturbation (q here), the cost
    // target adds its stored adjoint forcing (src/SpongePatchImpl.f90:142-158,
    // src/CostTargetPatchImpl.f90:104-133); no sources, no control
    if (nonzero(S)) r -= S * q;
    if (nonzero(linFactor) && nonzero(B.tgtCount[p])) r += linFactor * B.adjF[kc];
  } else if (nonzero(S)) {
    r -= S * (q - B.qt[kc]);
  }
  if (!lin && B.excIdx && (c == 1 || c == 2 || c == E)) {
    const int e = B.excIdx[p];
    if (e >= 0) r += B.excF[3LL * e + (c == E ? 2 : c - 1)];
  }
  if (c == E) {
    const int step = *rs.step;
    // the actuators add the control forcing, or in a tangent run its
    // perturbation (rs.forcing then holds the perturbation's entries)
    if (controller) {
      const int ai = B.actIdx[p];
      if (ai >= 0) {
        if (rs.apiForcing) {
          r += B.mc[p] * rs.apiForcing[ai];
        } else {
          const long long e = (long long)(rs.nSteps - step) * 4 + (4 - stage);
          if (e >= 0 && e < rs.nForcingEntries) r += B.mc[p] * rs.forcing[e * rs.P + ai];
        }
      }
    }
    if (!lin && B.nSources > 0) {
      const double* amp = rs.amp + ((long long)(step - 1) * 4 + (stage - 1)) * B.nSources;
      for (int k = 0; k < B.nSources; ++k) r += amp[k] * B.srcG[p + N * k];
    }
  }
  if (B.iblank[p] == 0) r = 0.0;
  if (rkStage == 0) {
    B.rhs[kc] = r;
    return;
  }
  const RkCoeffs k = rkCoeffs(rs);
  const double h6 = k.h6, h3 = k.h3, h2 = k.h2, dt = k.dt;
  switch (rkStage) {
    case 1:
      B.b1[kc] = q;
      B.b2[kc] = q + h6 * r;
      B.q[kc] = q + h2 * r;
      break;
    case 2:
      B.b2[kc] = B.b2[kc] + h3 * r;
      B.q[kc] = B.b1[kc] + h2 * r;
      break;
    case 3:
      B.b2[kc] = B.b2[kc] + h3 * r;
      B.q[kc] = B.b1[kc] + dt * r;
      break;
    default:
      B.q[kc] = B.b2[kc] + h6 * r;
      break;
  }
}

template <int ND>
__global__ void __launch_bounds__(kMaxTile) kForwardDivergence(BlockView B, Physics P, RunScalars rs, int rkStage,
                                                               int stage, int controller, Tile T, int lin,
                                                               double linFactor) {
  pdlEnter();
  forwardDivergencePoint<ND>(B, P, rs, rkStage, stage, controller, T, blockIdx.x, lin, linFactor);
}

// checkSolutionLimits (src/SolverImpl.f90:189-304) on one point: density and
// temperature strictly inside their ranges; a comparison with NaN fails, so
// non-finite values are violations too. The first violation by key wins.
template <int ND>
__global__ void __launch_bounds__(kBlock) kSolutionLimits(BlockView B, SolutionLimits L, const int* step, int stage,
                                                          int blockIndex, unsigned long long* key) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (p >= B.N) return;
  const double rho = B.q[p];
  const double T = B.prim[p + B.N * (2 + ND)];
  const int quantity = !(rho > L.rhoMin && rho < L.rhoMax) ? 0 : !(T > L.TMin && T < L.TMax) ? 1 : 2;
  if (quantity < 2) {
    const long long ordinal = step ? (long long)(*step - 1) * 4 + (stage - 1) : 0;
    atomicMin(key, limitKeyOf(ordinal, blockIndex, quantity, p));
  }
}

// Functional (AcousticNoise%compute, src/AcousticNoiseImpl.f90:123-206) of the
// state whose primitives are current: partial sums over the cost-target points,
// fixed block layout, into the slot of (step, stage).
__device__ __forceinline__ void functionalBlock(const BlockView& B, const RunScalars& rs, int stage,
                                                int pressureComp, int blk) {
  const int i = blk * kBlock + threadIdx.x;
  double v = 0.0;
  if (i < B.nTgt) {
    const long long p = B.tgtPts[i];
    const double F = B.prim[p + B.N * pressureComp] - B.meanP[p];
    v = B.wT[p] * (F * F * B.mt[p]);
  }
  const double s = blockSum(v);
  if (threadIdx.x == 0) {
    const int slot = ((*rs.step) - 1) * 4 + (stage - 1);
    rs.partials[(long long)slot * rs.nPartialBlocks + blk] = s;
  }
}

__global__ void __launch_bounds__(kBlock) kFunctional(BlockView B, RunScalars rs, int stage, int pressureComp) {
  pdlEnter();
  functionalBlock(B, rs, stage, pressureComp, blockIdx.x);
}

// Tangent of the functional at the forward state of (step, stage) along the
// perturbation in lambda: per cost-target point wT m_t 2 (p - p_mean) delta p,
// delta p = (gamma - 1)(|u|^2/2 delta rho - u . delta(rho u) + delta E). The
// state at the start of (step, stage) is the state after the stage before,
// so the block partial sum goes to that stage's slot, (step-1)*4 + stage - 2.
template <int ND>
__global__ void __launch_bounds__(kBlock) kFunctionalTangent(BlockView B, Physics P, RunScalars rs, int stage,
                                                             int fromSlot) {
  pdlEnter();
  const int slot = ((*rs.step) - 1) * 4 + (stage - 2);
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  const PrimLayout L{ND};
  const long long N = B.N;
  const int i = blockIdx.x * kBlock + threadIdx.x;
  double val = 0.0;
  if (i < B.nTgt) {
    const long long p = B.tgtPts[i];
    double u2 = 0.0, ux = 0.0;
    for (int d = 0; d < ND; ++d) {
      const double u = fs.prim[p + N * L.u(d)];
      u2 += u * u;
      ux += u * B.lam[p + N * (d + 1)];
    }
    const double dp = P.gm1 * (0.5 * u2 * B.lam[p] - ux + B.lam[p + N * (ND + 1)]);
    const double F = fs.prim[p + N * L.p()] - B.meanP[p];
    val = B.wT[p] * (2.0 * F * dp * B.mt[p]);
  }
  const double sum = blockSum(val);
  if (threadIdx.x == 0 && slot >= 0) rs.partials[(long long)slot * rs.nPartialBlocks + blockIdx.x] = sum;
}

// Gradient entry and sensitivity partial sums of lambda at an adjoint stage
// (ThermalActuator%updateGradient / computeSensitivity,
// src/ThermalActuatorImpl.f90:83-159, 383-443), over the actuator points.
__global__ void __launch_bounds__(kBlock) kGradientSensitivity(BlockView B, RunScalars rs, int stage, int energyComp) {
  pdlEnter();
  const int i = blockIdx.x * kBlock + threadIdx.x;
  const long long entry = (long long)(rs.nSteps - *rs.step) * 4 + (4 - stage);
  double v = 0.0;
  if (i < B.nAct) {
    const long long p = B.actPts[i];
    const double g = B.lam[p + B.N * energyComp] * B.mc[p];
    rs.gradient[entry * rs.P + i] = g;
    v = B.wA[p] * (g * g);
  }
  const double s = blockSum(v);
  if (threadIdx.x == 0) rs.partials[entry * rs.nPartialBlocks + blockIdx.x] = s;
}

// ---------------------------------------------------------------------------
// Adjoint core (computeRhsAdjoint, src/RhsHelperImpl.f90:398-560): adjoint
// derivatives of lambda, (A - B1)^T products formed column by column, the
// second-partial viscous diffusion B2^T with the far-field viscous adjoint
// penalty (src/RhsHelperImpl.f90:89-250) folded into the same sweep, and
// the complete far-field adjoint SAT vector (src/FarFieldPatchImpl.f90:237-257).
// ---------------------------------------------------------------------------
// The point's share of the adjoint core once the direction sums y (nU) and
// ad (nD x (nU-1)) are formed: the far-field viscous adjoint penalty and the
// interface terms added to ad, rcore and ad stored. The SAT vectors of the
// wall and far-field entries come from kAdjointSatVectors.
template <int ND, bool CURV, bool VISC>
__device__ __forceinline__ void adjointCoreFinish(const BlockView& B, long long p, const FwdState& fs,
                                                  const double* m, const double* u, const double* y,
                                                  double (*ad)[ND + 1]) {
  constexpr int nU = ND + 2, nV = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  for (int c = 0; c < nU; ++c) B.rcore[p + N * c] = y[c];
  double lp[nU];
  for (int c = 0; c < nU; ++c) lp[c] = B.lam[p + N * c];
  const double jac = B.jac[p];
  if (VISC) {
    const double mu = fs.prim[p + N * L.mu()], la = fs.prim[p + N * L.la()], kd = fs.prim[p + N * L.k()];
    for (int k = 0; k < 3; ++k) {
      const int e = B.ffOfPoint[3 * p + k];
      if (e < 0 || B.ff.kind[e] != SAT_FAR_FIELD) continue;
      const int nd = B.ff.normalDir[e] - 1;
      double mn[ND];  // metric row of the normal direction, read from memory (no dynamic register index)
      for (int d = 0; d < ND; ++d) mn[d] = CURV || d == nd ? B.metrics[p + N * (ND * nd + d)] : 0.0;
      const double sv = B.ff.sigVRaw[e];
      for (int l = 0; l < ND; ++l) {
        double t[nV];
        for (int c = 0; c < nV; ++c) t[c] = 0.0;
        if (CURV)
          secondPartialViscousTransposeProduct<ND>(u, mu, la, kd, jac, mn, m + ND * l, &lp[1], t);
        else
          secondPartialViscousTransposeProductCart<ND>(u, mu, la, kd, jac, nd, B.metrics[p + N * (ND * nd + nd)], l,
                                                       m[ND * l + l], &lp[1], t);
        for (int c = 0; c < nV; ++c) ad[l][c] += sv * t[c];
      }
    }
    for (int k = 0; k < 3; ++k) {
      const int e = B.ffOfPoint[3 * p + k];
      if (e < 0 || B.ff.kind[e] != SAT_INTERFACE) continue;
      const double* a = B.ff.ifAd + (long long)e * ND * nV;
      for (int l = 0; l < ND; ++l)
        for (int c = 0; c < nV; ++c) ad[l][c] += a[l * nV + c];
    }
    for (int j = 0; j < ND; ++j)
      for (int c = 0; c < nV; ++c) B.ad[p + N * (j * nV + c)] = ad[j][c];
  }
}

// The adjoint SAT vector of every wall and far-field entry (B.ff.visc), one
// thread per entry: the far-field adjoint SAT (src/FarFieldPatchImpl.f90:
// 237-257) and the wall SATs (src/ImpenetrableWallImpl.f90,
// src/IsothermalWallImpl.f90). They depend only on the entry's point (its
// lambda and forward state), not on the core's sums, so they run beside the
// adjoint core instead of inside it, where a few lanes of each boundary warp
// carried them while the rest of the warp waited; the assembly kernel reads
// them. Interface entries belong to kInterfaceSatAdjoint.
template <int ND, bool VISC>
__global__ void __launch_bounds__(kBlock) kAdjointSatVectors(BlockView B, Physics P, RunScalars rs, int stage,
                                                            int fromSlot) {
  pdlEnter();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= B.ff.n) return;
  const int kind = B.ff.kind[e];
  if (kind == SAT_INTERFACE) return;
  constexpr int nU = ND + 2;
  const long long N = B.N;
  const PrimLayout L{ND};
  const long long p = B.ff.point[e];
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  double u[ND];
  for (int d = 0; d < ND; ++d) u[d] = fs.prim[p + N * L.u(d)];
  const double v = fs.prim[p + N * L.v()], Tm = fs.prim[p + N * L.T()];
  double lp[nU];
  for (int c = 0; c < nU; ++c) lp[c] = B.lam[p + N * c];
  if (kind != SAT_FAR_FIELD) {
    wallSatAdjoint<ND, VISC>(B, P, e, p, u, Tm, v, lp, B.ff.visc + (long long)e * nU);
    return;
  }
  {
    double tau[ND * ND], hf[ND];
    if (VISC) {
      for (int c = 0; c < ND * ND; ++c) tau[c] = fs.tau[p + N * c];
      for (int d = 0; d < ND; ++d) hf[d] = fs.hf[p + N * d];
    }
    const double* M = B.ff.M + (long long)e * nU * nU;
    double z[nU];
    for (int c = 0; c < nU; ++c) z[c] = 0.0;
    if (VISC) {
      double mn[ND];  // metric row of the normal direction, read from memory (no dynamic register index)
      for (int d = 0; d < ND; ++d) mn[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
      firstPartialViscousTransposeProduct<ND>(mn, u, Tm, v, P.g, P.powerLawExponent, tau, hf, lp, z);
    }
    const double sv = B.ff.sigV[e];
    for (int row = 0; row < nU; ++row) {
      double t = M[nU * row] * lp[0];
      for (int c = 1; c < nU; ++c) t += M[c + nU * row] * lp[c];
      B.ff.visc[(long long)e * nU + row] = VISC ? t - sv * z[row] : t;
    }
  }
}

// One direction's share of the adjoint core at a point: w = D+_I lambda, the
// (A_I - B1_I)^T w product into y and the B2(m_I, m_j)^T w products into
// ad[j]. y and ad start from zero, so summing the directions' shares in
// direction order reproduces the per-point accumulation exactly.
template <int ND, bool CURV, bool VISC, int I>
__device__ __forceinline__ void adjointCoreDirection(const BlockView& B, const Physics& P, const PointIndex& Ix,
                                                     const double* m, const double* u, double Tm, double v,
                                                     const double* tau, const double* hf, double mu, double la,
                                                     double kd, double jac, double* y, double (*ad)[ND + 1]) {
  constexpr int nU = ND + 2, nV = ND + 1;
  const long long N = B.N;
  double w[nU];
#pragma unroll
  for (int c = 0; c < nU; ++c) w[c] = applyOp<OP_D1ADJ, true, kClosureUnroll<ND>>(B.lam + N * c + Ix.base[I], Ix.idx[I], B.ax[I]);
  for (int c = 0; c < nU; ++c) y[c] = 0.0;
  if (CURV) {
    addFluxJacobianTransposeProduct<ND, VISC>(m + ND * I, u, Tm, v, P, P.powerLawExponent, tau, hf, w, y);
  } else {
    const double nTv = VISC ? P.powerLawExponent * P.g * v / Tm : 0.0;
    addFluxJacobianTransposeProductCart<ND, VISC>(I, m[ND * I + I], u, Tm, v, P, nTv, tau, hf, w, y);
  }
  if (VISC) {
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      for (int c = 0; c < nV; ++c) ad[j][c] = 0.0;
      if (CURV)
        secondPartialViscousTransposeProduct<ND>(u, mu, la, kd, jac, m + ND * I, m + ND * j, &w[1], ad[j]);
      else
        secondPartialViscousTransposeProductCart<ND>(u, mu, la, kd, jac, I, m[ND * I + I], j, m[ND * j + j], &w[1],
                                                     ad[j]);
    }
  }
}

template <int ND, bool CURV, bool VISC>
__device__ __forceinline__ void adjointCorePoint(const BlockView& B, const Physics& P, const RunScalars& rs,
                                                 int stage, int fromSlot, const Tile& T, int blk) {
  long long p;
  PointIndex I;
  if (!locate(B, T, blk, p, I)) return;
  constexpr int nU = ND + 2, nV = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  double w[ND][nU];
#pragma unroll
  for (int i = 0; i < ND; ++i)
#pragma unroll
    for (int c = 0; c < nU; ++c) w[i][c] = applyOp<OP_D1ADJ, true, kClosureUnroll<ND>>(B.lam + N * c + I.base[i], I.idx[i], B.ax[i]);
  double m[ND * ND];
  for (int c = 0; c < ND * ND; ++c) m[c] = (CURV || (c % (ND + 1)) == 0) ? B.metrics[p + N * c] : 0.0;
  double u[ND];
  for (int d = 0; d < ND; ++d) u[d] = fs.prim[p + N * L.u(d)];
  const double v = fs.prim[p + N * L.v()], Tm = fs.prim[p + N * L.T()];
  double tau[ND * ND], hf[ND];
  if (VISC) {
    for (int c = 0; c < ND * ND; ++c) tau[c] = fs.tau[p + N * c];
    for (int d = 0; d < ND; ++d) hf[d] = fs.hf[p + N * d];
  }
  double y[nU];
  for (int c = 0; c < nU; ++c) y[c] = 0.0;
  if (CURV) {
#pragma unroll
    for (int i = 0; i < ND; ++i)
      addFluxJacobianTransposeProduct<ND, VISC>(m + ND * i, u, Tm, v, P, P.powerLawExponent, tau, hf, w[i], y);
  } else {
    const double nTv = VISC ? P.powerLawExponent * P.g * v / Tm : 0.0;
#pragma unroll
    for (int i = 0; i < ND; ++i)
      addFluxJacobianTransposeProductCart<ND, VISC>(i, m[ND * i + i], u, Tm, v, P, nTv, tau, hf, w[i], y);
  }
  double ad[ND][nV];
  if (VISC) {
    const double mu = fs.prim[p + N * L.mu()], la = fs.prim[p + N * L.la()], kd = fs.prim[p + N * L.k()];
    const double jac = B.jac[p];
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      for (int c = 0; c < nV; ++c) ad[j][c] = 0.0;
#pragma unroll
      for (int i = 0; i < ND; ++i) {
        if (CURV)
          secondPartialViscousTransposeProduct<ND>(u, mu, la, kd, jac, m + ND * i, m + ND * j, &w[i][1], ad[j]);
        else
          secondPartialViscousTransposeProductCart<ND>(u, mu, la, kd, jac, i, m[ND * i + i], j, m[ND * j + j],
                                                       &w[i][1], ad[j]);
      }
    }
  }
  adjointCoreFinish<ND, CURV, VISC>(B, p, fs, m, u, y, ad);
}

// The adjoint core with nD threads per point: thread block = tile threads x
// nD, thread (point, direction I) forms its direction's share
// (adjointCoreDirection), the shares meet in shared memory and the
// direction-0 thread of each point sums them in direction order and finishes
// the point. Twice (2D) the threads of the per-point kernel, each with a
// third of its stencil work, for grids too small to fill the GPU per point.
template <int ND, bool CURV, bool VISC>
__global__ void __launch_bounds__(2 * kMaxTile) kAdjointCoreSplit(BlockView B, Physics P, RunScalars rs, int stage,
                                                                 int fromSlot, Tile T) {
  pdlEnter();
  constexpr int nU = ND + 2, nV = ND + 1, K = nU + ND * nV;
  extern __shared__ double share[];
  const int TT = T.threads();
  const int pt = threadIdx.x % TT, dir = threadIdx.x / TT;
  long long p = 0;
  PointIndex I;
  const bool ok = locateAt(B, T, blockIdx.x, pt, p, I);
  const long long N = B.N;
  const PrimLayout L{ND};
  FwdState fs{};
  double m[ND * ND], u[ND], tau[ND * ND], hf[ND];
  double v = 0.0, Tm = 0.0;
  if (ok) {
    fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
    for (int c = 0; c < ND * ND; ++c) m[c] = (CURV || (c % (ND + 1)) == 0) ? B.metrics[p + N * c] : 0.0;
    for (int d = 0; d < ND; ++d) u[d] = fs.prim[p + N * L.u(d)];
    v = fs.prim[p + N * L.v()];
    Tm = fs.prim[p + N * L.T()];
    if (VISC) {
      for (int c = 0; c < ND * ND; ++c) tau[c] = fs.tau[p + N * c];
      for (int d = 0; d < ND; ++d) hf[d] = fs.hf[p + N * d];
    }
    double mu = 0.0, la = 0.0, kd = 0.0, jac = 0.0;
    if (VISC) {
      mu = fs.prim[p + N * L.mu()];
      la = fs.prim[p + N * L.la()];
      kd = fs.prim[p + N * L.k()];
      jac = B.jac[p];
    }
    double y[nU], ad[ND][nV];
    if (dir == 0)
      adjointCoreDirection<ND, CURV, VISC, 0>(B, P, I, m, u, Tm, v, tau, hf, mu, la, kd, jac, y, ad);
    else if (ND > 1 && dir == 1)
      adjointCoreDirection<ND, CURV, VISC, (ND > 1 ? 1 : 0)>(B, P, I, m, u, Tm, v, tau, hf, mu, la, kd, jac, y, ad);
    else
      adjointCoreDirection<ND, CURV, VISC, (ND > 2 ? 2 : 0)>(B, P, I, m, u, Tm, v, tau, hf, mu, la, kd, jac, y, ad);
    double* mine = share + (long long)dir * K * TT + pt;
    for (int c = 0; c < nU; ++c) mine[c * TT] = y[c];
    if (VISC)
      for (int j = 0; j < ND; ++j)
        for (int c = 0; c < nV; ++c) mine[(nU + j * nV + c) * TT] = ad[j][c];
  }
  __syncthreads();
  if (!ok || dir != 0) return;
  double y[nU], ad[ND][nV];
  for (int c = 0; c < nU; ++c) {
    double t = share[c * TT + pt];
    for (int i = 1; i < ND; ++i) t += share[((long long)i * K + c) * TT + pt];
    y[c] = t;
  }
  if (VISC)
    for (int j = 0; j < ND; ++j)
      for (int c = 0; c < nV; ++c) {
        const int k = nU + j * nV + c;
        double t = share[k * TT + pt];
        for (int i = 1; i < ND; ++i) t += share[((long long)i * K + k) * TT + pt];
        ad[j][c] = t;
      }
  adjointCoreFinish<ND, CURV, VISC>(B, p, fs, m, u, y, ad);
}

template <int ND, bool CURV, bool VISC>
__global__ void __launch_bounds__(kMaxTile) kAdjointCore(BlockView B, Physics P, RunScalars rs, int stage,
                                                         int fromSlot, Tile T) {
  pdlEnter();
  adjointCorePoint<ND, CURV, VISC>(B, P, rs, stage, fromSlot, T, blockIdx.x);
}

// Divergence of the adjoint viscous diffusion, one thread per point and
// momentum/energy component: t2_c = sum_j D+_j ad_{j,c} (src/RhsHelperImpl.f90:562-564).
template <int ND>
__device__ __forceinline__ void adjointDiffusionPoint(const BlockView& B, const Tile& T, int blk) {
  long long p;
  PointIndex I;
  if (!locate(B, T, blk, p, I)) return;
  constexpr int nV = ND + 1;
  const int c = blockIdx.y;
  const long long N = B.N;
  double s = applyOp<OP_D1ADJ, true, kClosureUnroll<ND>>(B.ad + N * c + I.base[0], I.idx[0], B.ax[0]);
  for (int j = 1; j < ND; ++j) s += applyOp<OP_D1ADJ, true, kClosureUnroll<ND>>(B.ad + N * (j * nV + c) + I.base[j], I.idx[j], B.ax[j]);
  B.t2[p + N * c] = s;
}

template <int ND>
__global__ void __launch_bounds__(kMaxTile) kAdjointDiffusion(BlockView B, Tile T) {
  pdlEnter();
  adjointDiffusionPoint<ND>(B, T, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Adjoint assembly of one component: the viscous primitive-to-conservative
// map (src/RhsHelperImpl.f90:566-582), dissipation, 1/det, far-field /
// sponge / cost-target terms (src/FarFieldPatchImpl.f90:237-257,
// src/SpongePatchImpl.f90:106-124, src/CostTargetPatchImpl.f90:72-136 with
// src/AcousticNoiseImpl.f90:208-280) and the RK4 adjoint stage update of
// that component (src/RK4IntegratorImpl.f90:203-266).
// ---------------------------------------------------------------------------
template <int ND, bool VISC>
__device__ __forceinline__ void adjointAssemblePoint(const BlockView& B, const Physics& P, const RunScalars& rs,
                                                     int rkStage, int stage, double apiFactor, int api, int fromSlot,
                                                     const Tile& T, int blk) {
  long long p;
  PointIndex I;
  if (!locate(B, T, blk, p, I)) return;
  constexpr int nU = ND + 2, E = ND + 1;
  const int c = blockIdx.y;
  const long long N = B.N;
  const PrimLayout L{ND};
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  double r = B.rcore[p + N * c];
  const double v = fs.prim[p + N * L.v()];
  if (VISC) {
    const double xE = P.g * v * B.t2[p + N * ND];
    if (c == E) {
      r -= xE;
    } else if (c > 0) {
      r -= v * B.t2[p + N * (c - 1)] - fs.prim[p + N * L.u(c - 1)] * xE;
    } else {
      double su = 0.0;
      for (int d = 0; d < ND; ++d) {
        const double ud = fs.prim[p + N * L.u(d)];
        const double xd = v * B.t2[p + N * d] - ud * xE;
        su = d == 0 ? ud * xd : su + ud * xd;
      }
      r += v * fs.q[p + N * E] * xE + su;
    }
  }
  if (P.dissipation) r += dissipationTerm<ND>(B, P, I, p, c);
  r = r * B.jac[p];
  for (int k = 0; k < 3; ++k) {
    const int e = B.ffOfPoint[3 * p + k];
    if (e >= 0) r += B.ff.visc[(long long)e * nU + c];
  }
  const long long kc = p + N * c;
  const double lam = B.lam[kc];
  const double S = B.sponge[p];
  if (nonzero(S)) r += S * lam;
  if (B.excIdx && c <= 2) {
    const int e = B.excIdx[p];
    if (e >= 0) r += B.excF[3LL * e + c];
  }
  const double cnt = B.tgtCount[p];
  if (api) {
    if (nonzero(cnt) && nonzero(apiFactor)) r += apiFactor * B.adjF[kc];
  } else if (nonzero(cnt)) {
    const bool finalStage = (*rs.step == 1 && stage == 1);
    // factor 0 without the adjoint forcing and at the final stage, else 2, 0.5 or 1 by stage
    if (rs.adjointForcingSwitch && !finalStage) {
      const double factor = stage == 4 ? 2.0 : (stage == 2 ? 0.5 : 1.0);
      const double F = -2.0 * B.mt[p] * P.gm1 * (fs.prim[p + N * L.p()] - B.meanP[p]);
      double f;
      if (c == E) {
        f = F;
      } else if (c > 0) {
        f = -fs.prim[p + N * L.u(c - 1)] * F;
      } else {
        double u2 = 0.0;
        for (int d = 0; d < ND; ++d) {
          const double ud = fs.prim[p + N * L.u(d)];
          u2 = d == 0 ? ud * ud : u2 + ud * ud;
        }
        f = 0.5 * u2 * F;
      }
      for (int k = 0; k < (int)cnt; ++k) r += factor * f;
    }
  }
  if (B.iblank[p] == 0) r = 0.0;
  if (rkStage == 0) {
    B.rhs[kc] = r;
    return;
  }
  const RkCoeffs k = rkCoeffs(rs);
  const double h6 = k.h6, h3 = k.h3, h2 = k.h2, dt = k.dt;
  switch (rkStage) {
    case 4:
      B.b1[kc] = lam;
      B.b2[kc] = lam - h6 * r;
      B.lam[kc] = lam - h2 * r;
      break;
    case 3:
      B.b2[kc] = B.b2[kc] - h3 * r;
      B.lam[kc] = B.b1[kc] - h2 * r;
      break;
    case 2:
      B.b2[kc] = B.b2[kc] - h3 * r;
      B.lam[kc] = B.b1[kc] - dt * r;
      break;
    default:
      B.lam[kc] = B.b2[kc] - h6 * r;
      break;
  }
}

// ---------------------------------------------------------------------------
// Linearized RHS (computeRhsLinearized, src/RhsHelperImpl.f90:598-829) of the
// perturbation held in lambda about the current state, whose primitives,
// stress and heat flux are current.
// kLinearizedTemp: temp = (delta u, gamma v (delta E - v E delta rho
// - u . (delta(rho u) - u delta rho))) into t2 (:694-710).
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(kBlock) kLinearizedTemp(BlockView B, Physics P, RunScalars rs, int stage,
                                                          int fromSlot) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (p >= B.N) return;
  constexpr int E = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  const double v = fs.prim[p + N * L.v()], x0 = B.lam[p];
  double t[ND + 1];
  double su = 0.0;
  for (int d = 0; d < ND; ++d) {
    t[d] = -fs.prim[p + N * L.u(d)] * x0 + B.lam[p + N * (1 + d)];
    su = d == 0 ? fs.prim[p + N * L.u(d)] * t[d] : su + fs.prim[p + N * L.u(d)] * t[d];
  }
  double te = -v * fs.q[p + N * E] * x0;
  te = te - su + B.lam[p + N * E];
  t[ND] = te * P.g;
  for (int c = 0; c <= ND; ++c) B.t2[p + N * c] = t[c] * v;
}

// kLinearizedFlux: per point and direction i the contravariant linearized flux
// A_i dq - (B1_i dq + (0, sum_j B2(m_i, m_j) D_j temp)) into fhat, and the
// linearized far-field SAT of each entry at the point,
// -sigma_inv J A+(q_target) dq + sigma_visc J (linearized viscous flux along
// the normal) (src/FarFieldPatchImpl.f90:258-266).
template <int ND, bool VISC>
__global__ void __launch_bounds__(kMaxTile) kLinearizedFlux(BlockView B, Physics P, RunScalars rs, int stage,
                                                            int fromSlot, Tile T) {
  pdlEnter();
  long long p;
  PointIndex I;
  if (!locate(B, T, blockIdx.x, p, I)) return;
  constexpr int nU = ND + 2, nV = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  double x[nU];
  for (int c = 0; c < nU; ++c) x[c] = B.lam[p + N * c];
  double m[ND * ND];
  for (int c = 0; c < ND * ND; ++c) m[c] = B.metrics[p + N * c];
  double u[ND];
  for (int d = 0; d < ND; ++d) u[d] = fs.prim[p + N * L.u(d)];
  const double v = fs.prim[p + N * L.v()], Tm = fs.prim[p + N * L.T()];
  double tau[ND * ND], hf[ND], dt[ND][nV];
  double mu = 0.0, la = 0.0, kd = 0.0, jac = 0.0;
  if (VISC) {
    for (int c = 0; c < ND * ND; ++c) tau[c] = fs.tau[p + N * c];
    for (int d = 0; d < ND; ++d) hf[d] = fs.hf[p + N * d];
    mu = fs.prim[p + N * L.mu()];
    la = fs.prim[p + N * L.la()];
    kd = fs.prim[p + N * L.k()];
    jac = B.jac[p];
#pragma unroll
    for (int j = 0; j < ND; ++j)
#pragma unroll
      for (int c = 0; c < nV; ++c) dt[j][c] = applyOp<OP_D1, true, kClosureUnroll<ND>>(B.t2 + N * c + I.base[j], I.idx[j], B.ax[j]);
  }
#pragma unroll
  for (int i = 0; i < ND; ++i) {
    double Ax[nU], Bx[nU];
    fluxJacobianProduct<ND, VISC>(m + ND * i, u, Tm, v, P.g, P.powerLawExponent, tau, hf, x, Ax, Bx);
    if (VISC) {
#pragma unroll
      for (int j = 0; j < ND; ++j) secondPartialViscousProduct<ND>(u, mu, la, kd, jac, m + ND * i, m + ND * j, dt[j], Bx + 1);
    }
    for (int c = 0; c < nU; ++c) B.fhat[p + N * (i * nU + c)] = VISC ? Ax[c] - Bx[c] : Ax[c];
    for (int s = 0; s < 3; ++s) {
      const int e = B.ffOfPoint[3 * p + s];
      if (e < 0 || B.ff.normalDir[e] - 1 != i) continue;
      if (B.ff.kind[e] == SAT_INTERFACE) {
        // the interface keeps its side's linearized viscous flux along its
        // normal for kInterfaceSatLinearized (src/RhsHelperImpl.f90:788-800)
        if (VISC) {
          double* out = B.ff.ifVisc + (long long)e * nU;
          out[0] = 0.0;
          for (int r = 1; r < nU; ++r) out[r] = Bx[r];
        }
        continue;
      }
      if (B.ff.kind[e] == SAT_WALL || B.ff.kind[e] == SAT_ISOTHERMAL_WALL) {
        // linearized wall penalties (src/ImpenetrableWallImpl.f90:187-191,
        // src/IsothermalWallImpl.f90:309-322): -s_inv J (A(m) - m (dp/dq)) dq,
        // and for isothermal walls -s_visc J (0, d(rho u), dE - d rho T_w / gamma)
        double Aw[nU];
        fluxJacobianProduct<ND, false>(m + ND * i, u, Tm, v, P.g, 0.0, nullptr, nullptr, x, Aw, nullptr);
        double u2 = u[0] * u[0], ux = u[0] * x[1];
        for (int d = 1; d < ND; ++d) {
          u2 += u[d] * u[d];
          ux += u[d] * x[1 + d];
        }
        const double dpx = (P.g - 1.0) * (0.5 * u2 * x[0] - ux + x[nU - 1]);
        for (int l = 0; l < ND; ++l) Aw[1 + l] -= m[ND * i + l] * dpx;
        double* sat = B.ff.visc + (long long)e * nU;
        for (int r = 0; r < nU; ++r) sat[r] = -B.ff.wallInv[e] * Aw[r];
        if (VISC && B.ff.kind[e] == SAT_ISOTHERMAL_WALL) {
          const double sv = B.ff.wallVisc[e];
          for (int r = 1; r < nU - 1; ++r) sat[r] -= sv * x[r];
          sat[nU - 1] -= sv * (x[nU - 1] - x[0] * B.ff.wallT[e] / P.g);
        }
        continue;
      }
      if (B.ff.kind[e] != SAT_FAR_FIELD) continue;
      const double* M = B.ff.M + (long long)e * nU * nU;
      for (int r = 0; r < nU; ++r) {
        double t = M[r] * x[0];
        for (int c = 1; c < nU; ++c) t += M[r + nU * c] * x[c];
        B.ff.visc[(long long)e * nU + r] = VISC ? -t + B.ff.sigV[e] * Bx[r] : -t;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Solenoidal excitation of one patch (addSolenoidalExcitation,
// src/SolenoidalExcitationPatchImpl.f90:159-278) at the stage's forward time.
// Per entry: f = S sum_l [t1 (w t4 - 2 g dy t3), t3 (w t2 - 2 g dx t1)] with
// t1..t4 = sin/cos(w (x - x0) + phi_1 - w c_x t), sin/cos(w (y - y0) + phi_2 - w c_y t)
// formed from the cached spatial functions and the temporal functions, which
// each thread block evaluates once into shared memory.
// Forward: (f_x, f_y, u . f) for the x/y momentum and energy equations.
// Adjoint: -(dR/dq)^T lambda of the energy term u . f,
// (v (u . f) lambda_E, -v f_x lambda_E, -v f_y lambda_E) for components 0..2,
// with the forward state of the stage and lambda before the stage update.
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(kBlock) kExcitation(BlockView B, ExcPatch X, RunScalars rs, int stage, int adjoint,
                                                      int fromSlot) {
  pdlEnter();
  __shared__ double tf[4 * kMaxExcitationModes];
  const int nM = X.nModes;
  const double t = rs.stageTime[(long long)(*rs.step - 1) * 4 + (stage - 1)];
  for (int l = threadIdx.x; l < nM; l += blockDim.x) {
    double sn, cs;
    sincos(X.omega[l] * X.speed[0] * t, &sn, &cs);
    tf[l] = sn;
    tf[nM + l] = cs;
    sincos(X.omega[l] * X.speed[1] * t, &sn, &cs);
    tf[2 * nM + l] = sn;
    tf[3 * nM + l] = cs;
  }
  __syncthreads();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= X.nE) return;
  const long long nE = X.nE;
  const double dx = X.dx[e], dy = X.dy[e], g2 = 2.0 * X.g;
  double f1 = 0.0, f2 = 0.0;
  for (int l = 0; l < nM; ++l) {
    const double s1 = X.cache[e + nE * l], s2 = X.cache[e + nE * (nM + l)];
    const double s3 = X.cache[e + nE * (2 * nM + l)], s4 = X.cache[e + nE * (3 * nM + l)];
    const double t1 = s1 * tf[nM + l] - s2 * tf[l];
    const double t2 = s2 * tf[nM + l] + s1 * tf[l];
    const double t3 = s3 * tf[3 * nM + l] - s4 * tf[2 * nM + l];
    const double t4 = s4 * tf[3 * nM + l] + s3 * tf[2 * nM + l];
    const double w = X.omega[l];
    f1 += t1 * (w * t4 - g2 * dy * t3);
    f2 += t3 * (w * t2 - g2 * dx * t1);
  }
  const double S = X.S[e];
  f1 = S * f1;
  f2 = S * f2;
  const long long N = B.N, p = X.point[e];
  const PrimLayout L{ND};
  double* out = B.excF + 3LL * (X.off + e);
  if (!adjoint) {
    out[0] = f1;
    out[1] = f2;
    out[2] = B.prim[p + N * L.u(0)] * f1 + B.prim[p + N * L.u(1)] * f2;
    return;
  }
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  const double vl = fs.prim[p + N * L.v()] * B.lam[p + N * (ND + 1)];
  const double uf = fs.prim[p + N * L.u(0)] * f1 + fs.prim[p + N * L.u(1)] * f2;
  out[0] = vl * uf;
  out[1] = -vl * f1;
  out[2] = -vl * f2;
}

template <int ND, bool VISC>
__global__ void __launch_bounds__(kMaxTile) kAdjointAssemble(BlockView B, Physics P, RunScalars rs, int rkStage,
                                                             int stage, double apiFactor, int api, int fromSlot,
                                                             Tile T) {
  pdlEnter();
  adjointAssemblePoint<ND, VISC>(B, P, rs, rkStage, stage, apiFactor, api, fromSlot, T, blockIdx.x);
}

// Adjoint initial condition lambda(T) = factor * adjointForcing(q(T)),
// factor = -dt/6 (loadInitialCondition ADJOINT, src/SolverImpl.f90:368-427).
template <int ND>
__global__ void __launch_bounds__(kBlock) kAdjointInitial(BlockView B, Physics P, double factor, int accumulate) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (p >= B.N) return;
  constexpr int nU = ND + 2, E = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  double r[nU];
  for (int c = 0; c < nU; ++c) r[c] = 0.0;
  const double cnt = B.tgtCount[p];
  if (cnt != 0.0 && factor != 0.0) {
    double u[ND];
    for (int d = 0; d < ND; ++d) u[d] = B.prim[p + N * L.u(d)];
    const double F = -2.0 * B.mt[p] * P.gm1 * (B.prim[p + N * L.p()] - B.meanP[p]);
    double u2 = u[0] * u[0];
    for (int d = 1; d < ND; ++d) u2 += u[d] * u[d];
    for (int k = 0; k < (int)cnt; ++k) {
      r[E] += factor * F;
      for (int d = 0; d < ND; ++d) r[1 + d] += factor * (-u[d] * F);
      r[0] += factor * (0.5 * u2 * F);
    }
  }
  for (int c = 0; c < nU; ++c) B.lam[p + N * c] = accumulate ? B.lam[p + N * c] + r[c] : r[c];
}

template <int ND>
__global__ void __launch_bounds__(kBlock) kStoreAdjointForcing(BlockView B, Physics P, int zero) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (p >= B.N) return;
  constexpr int nU = ND + 2, E = ND + 1;
  const long long N = B.N;
  const PrimLayout L{ND};
  double r[nU];
  for (int c = 0; c < nU; ++c) r[c] = 0.0;
  const double cnt = B.tgtCount[p];
  if (!zero && cnt != 0.0) {
    double u[ND];
    for (int d = 0; d < ND; ++d) u[d] = B.prim[p + N * L.u(d)];
    const double F = -2.0 * B.mt[p] * P.gm1 * (B.prim[p + N * L.p()] - B.meanP[p]);
    double u2 = u[0] * u[0];
    for (int d = 1; d < ND; ++d) u2 += u[d] * u[d];
    for (int k = 0; k < (int)cnt; ++k) {
      r[E] += F;
      for (int d = 0; d < ND; ++d) r[1 + d] += -u[d] * F;
      r[0] += 0.5 * u2 * F;
    }
  }
  for (int c = 0; c < nU; ++c) B.adjF[p + N * c] = r[c];
}

// Terminal kinetic energy: block partial sums of H det rho |u|^2 / 2 over the
// non-hole points (norm = H det), for a fixed-order final reduction.
template <int ND>
__global__ void __launch_bounds__(kBlock) kKineticEnergyPartials(BlockView B, const double* __restrict__ norm,
                                                                 double* __restrict__ partial) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  double v = 0.0;
  if (p < B.N && B.iblank[p] != 0) {
    double m2 = 0.0;
    for (int d = 0; d < ND; ++d) {
      const double m = B.q[p + B.N * (d + 1)];
      m2 += m * m;
    }
    v = norm[p] * (0.5 * m2 / B.q[p]);
  }
  const double s = blockSum(v);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// lambda(T) = H^-1 dJ/dq(T) of the terminal kinetic energy: (-|u|^2/2, u, 0).
template <int ND>
__global__ void __launch_bounds__(kBlock) kKineticEnergyAdjointInitial(BlockView B, int accumulate) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (p >= B.N) return;
  constexpr int nU = ND + 2;
  const long long N = B.N;
  double l[nU];
  for (int c = 0; c < nU; ++c) l[c] = 0.0;
  if (B.iblank[p] != 0) {
    double u2 = 0.0;
    for (int d = 0; d < ND; ++d) {
      const double u = B.q[p + N * (d + 1)] / B.q[p];
      l[1 + d] = u;
      u2 += u * u;
    }
    l[0] = -0.5 * u2;
  }
  for (int c = 0; c < nU; ++c) B.lam[p + N * c] = accumulate ? B.lam[p + N * c] + l[c] : l[c];
}

// Snapshot of the conserved variables after a completed forward step.
__global__ void kSnapshot(double* __restrict__ snap, const double* __restrict__ q, long long n,
                          const int* __restrict__ step, int saveInterval, int initial) {
  pdlEnter();
  const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
  const int s = initial ? 0 : *step;
  if (s % saveInterval != 0 || i >= n) return;
  snap[(long long)(s / saveInterval) * n + i] = q[i];
}

__global__ void kStepAdvance(int* counters, int delta) {
  pdlEnter();
  if (threadIdx.x == 0 && blockIdx.x == 0) counters[0] += delta;
}

// out[s] = sum over the first `count` block partials of slot s (row stride
// `stride`), in a fixed order.
__global__ void kReducePartials(const double* __restrict__ partials, int stride, int count, int nSlots,
                                double* __restrict__ out) {
  pdlEnter();
  const int s = blockIdx.x;
  if (s >= nSlots) return;
  double v = 0.0;
  for (int b = threadIdx.x; b < count; b += blockDim.x) v += partials[(long long)s * stride + b];
  const double t = blockSum(v);
  if (threadIdx.x == 0) out[s] = t;
}

// ---------------------------------------------------------------------------
// Block-interface SATs (addBlockInterfacePenalty, src/BlockInterfacePatchImpl.f90:
// 127-538, discrete adjoint), one thread per interface entry. Forward:
//   sat = -s_inv,L J A+(Roe(qL, qR), m_L, dirL) (qL - qR)
//         + J (s_v,L F_vL + s_v,R F_vR) on momentum and energy,
// with s_v,L/R = |s_v| signed by the normal direction of each side. Adjoint:
//   sat = s_inv,L J [A_L^T lamL + (dA_L/dqL (qL - qR))^T lamL] - s_v,L J B1(m_L)^T lamL
//       - s_inv,R J [A_R^T lamR + (dA_R/dqL (qL - qR))^T lamR] + s_v,R J B1(m_R)^T lamR,
// where A_R uses the partner's normal metric and direction and dA/dqL comes
// from evaluating A+(Roe(qL, qR)) on dual numbers seeded with qL. The adjoint
// kernel also stores the interface terms of the adjoint viscous diffusion
// (addInterfaceAdjointPenalty, src/RhsHelperImpl.f90:831-1026) for kAdjointCore.
// ---------------------------------------------------------------------------
template <int ND, bool VISC>
__global__ void __launch_bounds__(kBlock) kInterfaceSat(BlockView B, Physics P, BlockRefs R) {
  pdlEnter();
  const int e = blockIdx.x * kBlock + threadIdx.x;
  if (e >= B.ff.n || B.ff.kind[e] != SAT_INTERFACE) return;
  constexpr int nU = ND + 2;
  const long long N = B.N, p = B.ff.point[e];
  const int pb = B.ff.partnerBlock[e];
  const long long pp = B.ff.partnerPoint[e], NR = R.N[pb];
  double qL[nU], qR[nU], dq[nU], mL[ND], roe[nU], A[nU * nU];
  for (int c = 0; c < nU; ++c) {
    qL[c] = B.q[p + N * c];
    qR[c] = R.q[pb][pp + NR * c];
    dq[c] = qL[c] - qR[c];
  }
  for (int d = 0; d < ND; ++d) mL[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
  roeAverage<ND, double>(qL, qR, P.g, roe);
  incomingJacobian<ND, double>(roe, mL, P.g, B.ff.dirL[e], A);
  const double jac = B.jac[p];
  const double s = B.ff.ifInv[2 * e];
  double* sat = B.ff.visc + (long long)e * nU;
  double vL = 0.0, vR = 0.0;
  if (VISC) {
    const double a = fabs(B.ff.ifVis[2 * e]);
    vL = B.ff.dirL[e] < 0 ? -a : a;
    vR = B.ff.dirR[e] < 0 ? -a : a;
  }
  const double* fL = B.ff.ifVisc + (long long)e * nU;
  const double* fR = R.ifVisc[pb] + (long long)B.ff.partnerEntry[e] * nU;
  for (int r = 0; r < nU; ++r) {
    double t = A[r] * dq[0];
    for (int c = 1; c < nU; ++c) t += A[r + nU * c] * dq[c];
    double v = -(s * jac * t);
    if (VISC && r > 0) v += jac * (vL * fL[r] + vR * fR[r]);
    sat[r] = v;
  }
}

// Linearized block-interface SAT of one entry (src/BlockInterfacePatchImpl.f90:468-515):
// -s_inv J (A+ (dq_L - dq_R) + (dA+ along (dq_L, dq_R)) (q_L - q_R)), the
// derivative of the Roe-averaged A+ taken on one-derivative dual numbers, plus
// J (s_vL F_L + s_vR F_R) with the two sides' linearized viscous fluxes.
template <int ND, bool VISC>
__global__ void __launch_bounds__(kBlock) kInterfaceSatLinearized(BlockView B, Physics P, BlockRefs R, RunScalars rs,
                                                                   int stage, int fromSlot) {
  pdlEnter();
  const int e = blockIdx.x * kBlock + threadIdx.x;
  if (e >= B.ff.n || B.ff.kind[e] != SAT_INTERFACE) return;
  constexpr int nU = ND + 2;
  using D = DualN<1>;
  const long long N = B.N, p = B.ff.point[e];
  const int pb = B.ff.partnerBlock[e];
  const long long pp = B.ff.partnerPoint[e], NR = R.N[pb];
  // forward state of both sides: the blocks' arrays, or their stage slots in a tangent run
  const double* qLb = B.q;
  const double* qRb = R.q[pb];
  if (fromSlot) {
    const int slot = ((*rs.step) - (*rs.segBase) - 1) * 4 + stage - 1;
    qLb = rs.stageBuf + (long long)slot * rs.slotStride;
    qRb = R.stage[pb] + (long long)slot * R.slotStride[pb];
  }
  double dq[nU], dx[nU], mL[ND];
  D dL[nU], dR[nU], roe[nU];
  for (int c = 0; c < nU; ++c) {
    const double qL = qLb[p + N * c], qR = qRb[pp + NR * c];
    const double xL = B.lam[p + N * c], xR = R.lam[pb][pp + NR * c];
    dq[c] = qL - qR;
    dx[c] = xL - xR;
    dL[c] = D(qL);
    dL[c].d[0] = xL;
    dR[c] = D(qR);
    dR[c].d[0] = xR;
  }
  for (int d = 0; d < ND; ++d) mL[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
  roeAverage<ND, D>(dL, dR, P.g, roe);
  D A[nU * nU];
  incomingJacobian<ND, D>(roe, mL, P.g, B.ff.dirL[e], A);
  const double jac = B.jac[p];
  const double s = B.ff.ifInv[2 * e];
  double vL = 0.0, vR = 0.0;
  if (VISC) {
    const double a = fabs(B.ff.ifVis[2 * e]);
    vL = B.ff.dirL[e] < 0 ? -a : a;
    vR = B.ff.dirR[e] < 0 ? -a : a;
  }
  const double* fL = B.ff.ifVisc + (long long)e * nU;
  const double* fR = R.ifVisc[pb] + (long long)B.ff.partnerEntry[e] * nU;
  double* sat = B.ff.visc + (long long)e * nU;
  for (int r = 0; r < nU; ++r) {
    double t1 = A[r].v * dx[0], t2 = A[r].d[0] * dq[0];
    for (int c = 1; c < nU; ++c) {
      t1 += A[r + nU * c].v * dx[c];
      t2 += A[r + nU * c].d[0] * dq[c];
    }
    double v = -(s * jac * t1) - s * jac * t2;
    if (VISC && r > 0) v += jac * (vL * fL[r] + vR * fR[r]);
    sat[r] = v;
  }
}

// Lanes of kInterfaceSatAdjoint: one per (interface entry, left-state
// component l, side). A warp-wide FP64 instruction occupies its SM
// sub-partition's FP64 pipe for the same time whatever the number of active
// lanes, so the per-entry work is spread over 2 nU lanes (and, with one warp
// per CTA, over many sub-partitions) instead of running as 2 nU passes in one
// lane.
template <int ND>
struct InterfaceLanes {
  static constexpr int perEntry = 2 * (ND + 2);          // (l, side) pairs
  static constexpr int entriesPerWarp = 32 / perEntry;  // 4 in 2D, 3 in 3D
};

template <int ND, bool VISC>
__global__ void __launch_bounds__(32) kInterfaceSatAdjoint(BlockView B, Physics P, BlockRefs R, RunScalars rs,
                                                            int stage, int fromSlot, int nEntries) {
  pdlEnter();
  constexpr int nU = ND + 2, nV = ND + 1;
  constexpr int G = InterfaceLanes<ND>::perEntry, EW = InterfaceLanes<ND>::entriesPerWarp;
  using D = DualN<1>;
  __shared__ double part[32][nU];
  const int lane = threadIdx.x, g = lane / G, k = lane - g * G;
  const int l = k >> 1, side = k & 1;
  const int idx = blockIdx.x * EW + g;
  const bool active = g < EW && idx < nEntries;
  const int e = active ? B.ff.ifList[idx] : 0;
  const long long N = B.N;
  const PrimLayout L{ND};
  const FwdState fs = forwardState<ND>(B, rs, stage, fromSlot != 0);
  double qL[nU], qR[nU], dq[nU], lamL[nU], lamR[nU], mL[ND], mR[ND], jac = 0.0, sL = 0.0, sR = 0.0;
  long long p = 0;
  double contrib[nU];
  for (int c = 0; c < nU; ++c) contrib[c] = 0.0;
  if (active) {
    p = B.ff.point[e];
    const int pb = B.ff.partnerBlock[e];
    const long long pp = B.ff.partnerPoint[e], NR = R.N[pb];
    // forward state of both sides: the blocks' arrays, or their stage slots in a run
    const double* qRb = R.q[pb];
    if (fromSlot) {
      const int slot = ((*rs.step) - (*rs.segBase) - 1) * 4 + stage - 1;
      qRb = R.stage[pb] + (long long)slot * R.slotStride[pb];
    }
    for (int c = 0; c < nU; ++c) {
      qL[c] = fs.q[p + N * c];
      qR[c] = qRb[pp + NR * c];
      dq[c] = qL[c] - qR[c];
      lamL[c] = B.lam[p + N * c];
      lamR[c] = R.lam[pb][pp + NR * c];
    }
    for (int d = 0; d < ND; ++d) {
      mL[d] = B.metrics[p + N * (ND * (B.ff.normalDir[e] - 1) + d)];
      mR[d] = B.ff.metricsR[(long long)e * ND + d];
    }
    jac = B.jac[p];
    sL = B.ff.ifInv[2 * e] * jac;
    sR = -B.ff.ifInv[2 * e + 1] * jac;
    // This lane's share: the Roe average and one side's incoming Jacobian on
    // single-derivative dual numbers seeded with d/dq_L[l] give
    // sum_ij lambda_i (dA_ij/dq_l) dq_j into component l; the l = 0 lanes
    // also give that side's A^T lambda into every component.
    D dL[nU], dR[nU], roe[nU];
    for (int c = 0; c < nU; ++c) {
      dL[c] = D(qL[c]);
      dL[c].d[0] = c == l ? 1.0 : 0.0;
      dR[c] = D(qR[c]);
    }
    roeAverage<ND, D>(dL, dR, P.g, roe);
    D A[nU * nU];
    incomingJacobian<ND, D>(roe, side == 0 ? mL : mR, P.g, side == 0 ? B.ff.dirL[e] : B.ff.dirR[e], A);
    const double* lam = side == 0 ? lamL : lamR;
    const double sInv = side == 0 ? sL : sR;
    if (l == 0)
      for (int r = 0; r < nU; ++r) {
        double t = A[nU * r].v * lam[0];
        for (int c = 1; c < nU; ++c) t += A[c + nU * r].v * lam[c];
        contrib[r] = sInv * t;
      }
    double t = 0.0;
    for (int i = 0; i < nU; ++i) {
      double w = 0.0;
      for (int j = 0; j < nU; ++j) w += A[i + nU * j].d[0] * dq[j];
      t += w * lam[i];
    }
    contrib[l] += sInv * t;
  }
  for (int c = 0; c < nU; ++c) part[lane][c] = contrib[c];
  __syncwarp();
  if (!active || k != 0) return;
  // the entry's lanes' shares summed in lane order, then the viscous terms
  double sat[nU];
  for (int c = 0; c < nU; ++c) {
    double t = part[lane][c];
    for (int j = 1; j < G; ++j) t += part[lane + j][c];
    sat[c] = t;
  }
  double u[ND];
  for (int d = 0; d < ND; ++d) u[d] = fs.prim[p + N * L.u(d)];
  if (VISC) {
    double tau[ND * ND], hf[ND];
    const double v = fs.prim[p + N * L.v()], T = fs.prim[p + N * L.T()];
    for (int c = 0; c < ND * ND; ++c) tau[c] = fs.tau[p + N * c];
    for (int d = 0; d < ND; ++d) hf[d] = fs.hf[p + N * d];
    for (int sd = 0; sd < 2; ++sd) {
      double y[nU];
      for (int c = 0; c < nU; ++c) y[c] = 0.0;
      firstPartialViscousTransposeProduct<ND>(sd == 0 ? mL : mR, u, T, v, P.g, P.powerLawExponent, tau, hf,
                                              sd == 0 ? lamL : lamR, y);
      const double sVis = sd == 0 ? -B.ff.ifVis[2 * e] : B.ff.ifVis[2 * e + 1];
      for (int c = 0; c < nU; ++c) sat[c] += sVis * jac * y[c];
    }
  }
  for (int c = 0; c < nU; ++c) B.ff.visc[(long long)e * nU + c] = sat[c];
  if (VISC) {
    const double mu = fs.prim[p + N * L.mu()], la = fs.prim[p + N * L.la()], kd = fs.prim[p + N * L.k()];
    double* a = B.ff.ifAd + (long long)e * ND * nV;
    for (int dl = 0; dl < ND; ++dl) {
      double ml[ND];
      for (int d = 0; d < ND; ++d) ml[d] = B.metrics[p + N * (ND * dl + d)];
      double tL[nV], tR[nV];
      for (int c = 0; c < nV; ++c) tL[c] = tR[c] = 0.0;
      secondPartialViscousTransposeProduct<ND>(u, mu, la, kd, jac, mL, ml, &lamL[1], tL);
      secondPartialViscousTransposeProduct<ND>(u, mu, la, kd, jac, mR, ml, &lamR[1], tR);
      for (int c = 0; c < nV; ++c) a[dl * nV + c] = B.ff.ifVis[2 * e] * tL[c] - B.ff.ifVis[2 * e + 1] * tR[c];
    }
  }
}

// ---------------------------------------------------------------------------
// Batched forward stage kernels: thread block k works on block map[k].y of
// instance map[k].x, with that instance's grid, state, run scalars and tile.
// ---------------------------------------------------------------------------
template <int ND, bool CURV, bool VISC>
__global__ void __launch_bounds__(kBatchThreads) kGradFluxBatch(const BatchEntry* __restrict__ E,
                                                                const int2* __restrict__ map, Physics P, int stage) {
  pdlEnter();
  const int2 m = map[blockIdx.x];
  const BatchEntry& e = E[m.x];
  gradFluxPoint<ND, CURV, VISC>(e.v, P, e.rs, GF_FLUX, stage, e.tGrad, m.y);
}

template <int ND>
__global__ void __launch_bounds__(kBatchThreads) kDissipationBatch(const BatchEntry* __restrict__ E,
                                                                   const int2* __restrict__ map, Physics P) {
  pdlEnter();
  const int2 m = map[blockIdx.x];
  const BatchEntry& e = E[m.x];
  dissipationPoint<ND>(e.v, P, e.v.q, 1.0, e.tDiss, m.y);
}

template <int ND>
__global__ void __launch_bounds__(kBatchThreads) kForwardDivergenceBatch(const BatchEntry* __restrict__ E,
                                                                         const int2* __restrict__ map, Physics P,
                                                                         int rkStage) {
  pdlEnter();
  const int2 m = map[blockIdx.x];
  const BatchEntry& e = E[m.x];
  forwardDivergencePoint<ND>(e.v, P, e.rs, rkStage, rkStage, e.controller, e.tRhs, m.y, 0, 0.0);
}

template <int ND>
__global__ void __launch_bounds__(kBlock) kPrimsBatch(const BatchEntry* __restrict__ E, const int2* __restrict__ map,
                                                      Physics P) {
  pdlEnter();
  const int2 m = map[blockIdx.x];
  const BatchEntry& e = E[m.x];
  primsPoint<ND>(e.v, P, e.v.q, 0, e.rs, 0, m.y);
}

__global__ void __launch_bounds__(kBlock) kFunctionalBatch(const BatchEntry* __restrict__ E,
                                                           const int2* __restrict__ map, int stage, int pressureComp) {
  pdlEnter();
  const int2 m = map[blockIdx.x];
  const BatchEntry& e = E[m.x];
  functionalBlock(e.v, e.rs, stage, pressureComp, m.y);
}

// ---------------------------------------------------------------------------
// Bounded wait of the persistent kernels, run by thread 0 of a CTA: polls the
// monotonic counter *count (about 100 ns per poll) until it reaches `need`.
// It gives up after `limit` polls, sets *err and returns false; it also
// returns false once another CTA has set *err, so that every CTA leaves the
// kernel and the host reads the status. The acquire fence after the wait
// (which also discards the SM's L1 lines) lets the CTA's loads after its next
// CTA barrier see what the counted producers wrote before their releases
// (__threadfence, then the atomic add to *count).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool waitCount(const unsigned long long* count, unsigned long long need, long long limit,
                                          int* err) {
  volatile const unsigned long long* vc = count;
  volatile int* verr = err;
  long long polls = 0;
  bool ok = true;
  while (*vc < need) {
    if (*verr) {
      ok = false;
      break;
    }
    if (++polls > limit) {
      atomicExch(err, 1);
      ok = false;
      break;
    }
    __nanosleep(64);
  }
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
  return ok;
}

// Persistent batched forward run: every step's four RK stages for every
// instance in one launch, scheduled as a device work queue.
//
// The run is a sequence of rounds, three per RK stage, each the work of one
// stage kernel of the per-step path: A (gradient/flux tiles, dissipation
// (tile, component) units, and the functional blocks of the stage before),
// B (divergence and RK update, per (tile, component)) and C (primitives of
// the new state, per block of points); after the last stage one more A in
// which only the functional blocks of the last stage work. All units of all
// rounds form one global order, round by round (within a round the unit
// lists' order: heavy gradient/flux tiles first). CTAs draw the next chunk of
// K consecutive units of that order from one counter and work them in order.
// A unit of instance i in round r depends only on instance i's units of
// round r-1: before working, the CTA waits until done[i], the count of
// instance i's completed units, reaches the number of its units in all
// rounds before r; after the unit it adds one to done[i]. Instances
// therefore advance independently, with no grid-wide barrier, and a CTA that
// would wait for instance i's last units of a round takes units of the other
// instances meanwhile (they come between them in the order).
//
// Progress: a unit waits only for units that come earlier in the global
// order, which were drawn earlier by co-resident CTAs (cooperative launch)
// and are worked in order within a chunk; the earliest incomplete unit has
// nothing left to wait for. Every wait gives up after plan.spinLimit polls,
// sets *plan.status and leaves; the others see the status at their next poll
// and leave too.
//
// Memory order: the producer's threads write, meet at a CTA barrier, and its
// thread 0 fences and then adds to done[i] (release); the consumer's thread 0
// reads done[i], fences (acquire, which also discards the SM's L1 lines) and
// meets its threads at a CTA barrier before they read. A CTA acquires once
// per (instance, round) in a row: the inputs of a round stay unchanged until
// all of the round's units are done, and no unit of an earlier round of that
// instance is still running to load older copies. Data of round r is
// written only by round r's units and read only by later rounds' units (or
// by units of round r that write other arrays), so ordinary cached loads see
// the producers' values. The per-point arithmetic is that of the stage
// kernels, so the results equal the per-step launches'.
template <int ND, bool CURV, bool VISC>
__global__ void __launch_bounds__(kBatchThreads, persistentMinBlocks(ND))
    kBatchRunPersistent(const BatchEntry* __restrict__ E, PersistentPlan plan, Physics P, int nSteps,
                        int functional) {
  __shared__ long long sBase;
  __shared__ int sUnit, sPhase, sStep, sFStep, sStage, sInst;
  constexpr int nU = ND + 2;
  constexpr int K = MGD_PERSISTENT_CHUNK;
  const PrimLayout L{ND};
  const long long perStage = (long long)plan.nA + plan.nB + plan.nC;
  const long long nRun = 4LL * nSteps * perStage + (functional ? plan.nA : 0);
  // thread 0: the (instance, round) whose inputs this CTA last acquired
  int heldInst = -1;
  long long heldRound = -1;
  for (;;) {
    __syncthreads();  // every thread has finished the previous chunk
    if (threadIdx.x == 0) sBase = (long long)atomicAdd(plan.work, (unsigned long long)K);
    __syncthreads();
    const long long base = sBase;
    if (base >= nRun) return;
    const int nk = (int)(nRun - base < K ? nRun - base : K);
    for (int k = 0; k < nk; ++k) {
      if (threadIdx.x == 0) {
        const long long g = base + k;
        const long long s = g / perStage;
        long long off = g - s * perStage;
        int phase = 0, inst;
        if (off < plan.nA) {
          inst = plan.unitsA[off].y;
        } else if (off < plan.nA + plan.nB) {
          phase = 1;
          off -= plan.nA;
          inst = plan.unitsB[off].x;
        } else {
          phase = 2;
          off -= plan.nA + plan.nB;
          inst = plan.unitsC[off].x;
        }
        const long long round = 3 * s + phase;
        bool ok = true;
        if (inst != heldInst || round != heldRound) {
          const int4 cnt = plan.counts[inst];
          const unsigned long long need = (unsigned long long)s * (unsigned long long)(cnt.x + cnt.y + cnt.z) +
                                          (phase >= 1 ? (unsigned long long)cnt.x : 0ULL) +
                                          (phase == 2 ? (unsigned long long)cnt.y : 0ULL);
          ok = waitCount(plan.done + inst, need, plan.spinLimit, plan.status);
          heldInst = inst;
          heldRound = round;
        }
        const int step = (int)(s / 4) + 1, stage = (int)(s % 4) + 1;
        sStep = step;
        sStage = stage;
        sFStep = stage > 1 ? step : step - 1;
        sInst = inst;
        sPhase = ok ? phase : -1;
        sUnit = (int)off;
      }
      __syncthreads();
      const int phase = sPhase;
      if (phase < 0) return;
      const int u = sUnit, stage = sStage;
      if (phase == 0) {
        // round A, or the closing functional round (stage index past the run)
        const int4 w = plan.unitsA[u];
        const BatchEntry& e = E[w.y];
        const bool closing = sStep > nSteps;
        if (w.x == 0 && !closing) {
          RunScalars rs = e.rs;
          rs.step = &sStep;
          gradFluxPoint<ND, CURV, VISC, 1, false>(e.v, P, rs, GF_FLUX, stage, e.tGrad, w.z);
        } else if (w.x == 1 && !closing) {
          dissipationPoint<ND, false>(e.v, P, e.v.q, 1.0, e.tDiss, w.z, w.w);
        } else if (w.x == 2 && functional && sFStep >= 1) {
          RunScalars rs = e.rs;
          rs.step = &sFStep;
          functionalBlock(e.v, rs, stage > 1 ? stage - 1 : 4, L.p(), w.z);
        }
      } else if (phase == 1) {
        const int4 w = plan.unitsB[u];
        const BatchEntry& e = E[w.x];
        RunScalars rs = e.rs;
        rs.step = &sStep;
        forwardDivergencePoint<ND, false>(e.v, P, rs, stage, stage, e.controller, e.tRhs, w.y, 0, 0.0, w.z);
      } else {
        const int2 w = plan.unitsC[u];
        const BlockView& B = E[w.x].v;
        const long long p = (long long)w.y * kBatchThreads + threadIdx.x;
        if (p < B.N) {
          double q[nU], pr[6 + ND];
          for (int c = 0; c < nU; ++c) q[c] = B.q[p + B.N * c];
          primitives<ND>(q, P, pr);
          for (int c = 0; c < 6 + ND; ++c) B.prim[p + B.N * c] = pr[c];
        }
      }
      __syncthreads();  // the unit's writes precede the release below
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(plan.done + sInst, 1ULL);
      }
    }
  }
}

// Self-test of the persistent kernels' bounded wait: `rounds` rounds in
// which every CTA writes its round stamp, adds one to a counter (release) and
// waits until the counter reaches round x `expected`; CTA 0 then sums all
// stamps (checking that each CTA sees the others' writes after the wait), and
// a second meeting keeps the stamps of the next round from overwriting them
// early. With `expected` above the number of CTAs no round completes: every
// wait runs out after `limit` polls and the kernel returns with status 1.
__device__ __forceinline__ bool meet(unsigned long long* count, unsigned long long need, long long limit, int* err) {
  __shared__ int sOk;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(count, 1ULL);
    sOk = waitCount(count, need, limit, err);
  }
  __syncthreads();
  return sOk != 0;
}

__global__ void kBarrierSelfTest(unsigned long long* count, int* err, long long limit, unsigned int expected,
                                 int rounds, long long* stamps, long long* sum) {
  for (int r = 1; r <= rounds; ++r) {
    if (threadIdx.x == 0) stamps[blockIdx.x] = (long long)r * (blockIdx.x + 1);
    if (!meet(count, (2ULL * r - 1) * expected, limit, err)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      long long t = 0;
      for (unsigned int b = 0; b < gridDim.x; ++b) t += stamps[b];
      sum[0] += t;
    }
    if (!meet(count, 2ULL * r * expected, limit, err)) return;
  }
}

// ---------------------------------------------------------------------------
// Constant-CFL step size (computeTimeStepSize, src/CNSHelperImpl.f90:913-982):
// block minima of the advective and viscous bounds over the non-hole points,
// then one block takes the minimum and, inside a run, records it for the step,
// advances the run time over the step's stages (src/RK4IntegratorImpl.f90:95-140)
// and evaluates the acoustic-source amplitudes of those stages
// (src/AcousticSourceImpl.f90:34-64).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double blockMin(double v) {
  __shared__ double warpMins[32];
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warpMins[w] = v;
  __syncthreads();
  double s = warpMins[0];
  if (threadIdx.x == 0)
    for (int i = 1; i < (int)((blockDim.x + 31) / 32); ++i) s = fmin(s, warpMins[i]);
  return s;
}

constexpr double kHugeStep = 1.7976931348623157e308;

template <int ND>
__global__ void __launch_bounds__(kBlock) kTimeStepPartials(BlockView B, Physics P, double cfl,
                                                            double* __restrict__ partial) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  double v = kHugeStep;
  if (p < B.N && B.iblank[p] != 0) {
    const long long N = B.N;
    const PrimLayout L{ND};
    double m[ND * ND], u[ND];
    for (int c = 0; c < ND * ND; ++c) m[c] = B.metrics[p + N * c];
    for (int d = 0; d < ND; ++d) u[d] = B.prim[p + N * L.u(d)];
    const double jac = B.jac[p];
    const double a = sqrt(P.gm1 * B.prim[p + N * L.T()]);
    double w = 0.0;
    for (int j = 0; j < ND; ++j) {
      double s = 0.0;
      for (int k = 0; k < ND; ++k) s += m[ND * j + k] * m[ND * j + k];
      w = w + s;
    }
    w = a * sqrt(w);
    for (int j = 0; j < ND; ++j) {
      double s = 0.0;
      for (int k = 0; k < ND; ++k) s += u[k] * m[ND * j + k];
      w = w + fabs(s);
    }
    w = jac * w;
    v = cfl / w;
    if (P.viscous) {
      double s = 0.0;
      for (int c = 0; c < ND * ND; ++c) s += m[c] * m[c];
      const double wv = jac * jac * s * fmax(2.0 * B.prim[p + N * L.mu()], B.prim[p + N * L.k()]);
      v = fmin(v, cfl / wv);
    }
  }
  const double r = blockMin(v);
  if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

struct SourceTable {
  int n;
  double twoPi;
  double amplitude[MGD_MAX_SOURCES], frequency[MGD_MAX_SOURCES], phase[MGD_MAX_SOURCES];
};

__global__ void __launch_bounds__(256) kTimeStepFinalize(const double* __restrict__ partial, int n,
                                                         double* __restrict__ dtOut, const int* __restrict__ step,
                                                         double* __restrict__ time, double* __restrict__ stageTime,
                                                         double* __restrict__ amp, SourceTable src) {
  pdlEnter();
  double v = kHugeStep;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v = fmin(v, partial[i]);
  const double dt = blockMin(v);
  if (threadIdx.x != 0) return;
  if (!step) {
    dtOut[0] = dt;
    return;
  }
  const int s = *step;
  double* k = dtOut + 4LL * (s - 1);
  k[0] = dt;
  k[1] = dt / 6.0;
  k[2] = dt / 3.0;
  k[3] = dt / 2.0;
  double t = *time;
  for (int i = 1; i <= 4; ++i) {
    if (i == 2 || i == 4) t = t + dt / 2.0;
    if (stageTime) stageTime[(long long)(s - 1) * 4 + (i - 1)] = t;
    for (int k = 0; k < src.n; ++k) {
      const double arg = __dadd_rn(__dmul_rn(__dmul_rn(src.twoPi, src.frequency[k]), t), src.phase[k]);
      amp[((long long)(s - 1) * 4 + (i - 1)) * src.n + k] = src.amplitude[k] * cos(arg);
    }
  }
  *time = t;
}

// ---------------------------------------------------------------------------
// setup kernels (Grid%update, src/GridImpl.f90:621-1066)
// ---------------------------------------------------------------------------

// d x_c / d xi_dir for every coordinate component c (computeCoordinateDerivatives);
// PLANE periodicity shifts the wrapped coordinate by the periodic length.
template <int ND>
__global__ void kCoordinateDerivative(BlockView B, const double* __restrict__ coords, int dir,
                                      double periodicLength, double* __restrict__ out) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (p >= B.N) return;
  const PointIndex I = pointIndex(B, p);
  const Axis ax = B.ax[dir];
  for (int c = 0; c < ND; ++c) {
    const double* line = coords + B.N * c + I.base[dir];
    double s;
    if (ax.per != MGD_PERIODIC_PLANE) {
      s = applyOp<OP_D1>(line, I.idx[dir], ax);
    } else {
      const double* cin = c_ops.interior[ax.scheme][OP_D1];
      auto at = [&](int j) {
        const int k = I.idx[dir] + j;
        double x = line[(long long)wrapIndex(k, ax.n, ax.per) * ax.stride];
        if (c == dir) {
          if (k < 0) x = x - periodicLength;
          if (k >= ax.n) x = x + periodicLength;
        }
        return x;
      };
      s = cin[5] * (at(1) - at(-1));
      for (int j = 2; j <= 4; ++j) s += cin[4 + j] * (at(j) - at(-j));
    }
    out[p + B.N * c] = s;
  }
}

__global__ void kApplyD1(BlockView B, int dir, const double* __restrict__ in, double* __restrict__ out, int ncomp) {
  pdlEnter();
  const long long p = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (p >= B.N) return;
  const PointIndex I = pointIndex(B, p);
  for (int c = 0; c < ncomp; ++c) out[p + B.N * c] = applyOp<OP_D1>(in + B.N * c + I.base[dir], I.idx[dir], B.ax[dir]);
}

// Far-field SAT matrices sigma_inv * (1/det) * A+(q_target, metric_normal).
template <int ND>
__global__ void kFarFieldMatrices(BlockView B, double g, const double* __restrict__ sigInv,
                                  const int* __restrict__ signedNormal) {
  pdlEnter();
  const int e = blockIdx.x * kBlock + threadIdx.x;
  if (e >= B.ff.n) return;
  constexpr int nU = ND + 2;
  const long long p = B.ff.point[e];
  const int nd = B.ff.normalDir[e] - 1;
  double cv[nU], m[ND], A[nU * nU];
  for (int c = 0; c < nU; ++c) cv[c] = B.qt[p + B.N * c];
  for (int d = 0; d < ND; ++d) m[d] = B.metrics[p + B.N * (ND * nd + d)];
  incomingJacobian<ND>(cv, m, g, signedNormal[e], A);
  const double s = sigInv[e] * B.jac[p];
  for (int k = 0; k < nU * nU; ++k) B.ff.M[(long long)e * nU * nU + k] = s * A[k];
}

// Target viscous flux contracted with the normal metric at every far-field
// entry (updatePatchFactories, src/PatchFactoryImpl.f90:539-571); prim, tau
// and hf hold the target state's values when this runs.
template <int ND>
__global__ void kFarFieldTargetVisc(BlockView B) {
  pdlEnter();
  const int e = blockIdx.x * kBlock + threadIdx.x;
  if (e >= B.ff.n) return;
  constexpr int nU = ND + 2, E = ND + 1;
  const long long p = B.ff.point[e], N = B.N;
  const PrimLayout L{ND};
  const int nd = B.ff.normalDir[e] - 1;
  double m[ND], u[ND], tau[ND * ND], hf[ND];
  for (int d = 0; d < ND; ++d) m[d] = B.metrics[p + N * (ND * nd + d)];
  for (int d = 0; d < ND; ++d) u[d] = B.prim[p + N * L.u(d)];
  for (int c = 0; c < ND * ND; ++c) tau[c] = B.tau[p + N * c];
  for (int d = 0; d < ND; ++d) hf[d] = B.hf[p + N * d];
  double Fv[nU][ND];
  for (int d = 0; d < ND; ++d) {
    Fv[0][d] = 0.0;
    for (int c = 0; c < ND; ++c) Fv[1 + c][d] = tau[ND * c + d];
    double s = u[0] * tau[d];
    for (int c = 1; c < ND; ++c) s += u[c] * tau[ND * c + d];
    Fv[E][d] = s - hf[d];
  }
  for (int r = 0; r < nU; ++r) {
    double t = Fv[r][0] * m[0];
    for (int d = 1; d < ND; ++d) t += Fv[r][d] * m[d];
    B.ff.viscT[(long long)e * nU + r] = t;
  }
}

__global__ void kPowSelfTest(const double* __restrict__ x, int n, double e, double* __restrict__ fast,
                             double* __restrict__ ref) {
  pdlEnter();
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= n) return;
  fast[i] = fastPowPositive(x[i], e, &g_powTables);
  ref[i] = pow(x[i], e);
}

void launchPowSelfTest(const double* x, int n, double e, double* fast, double* ref) {
  uploadOperatorTables();
  kPowSelfTest<<<(n + kBlock - 1) / kBlock, kBlock>>>(x, n, e, fast, ref);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
#define MGD_LAUNCH(c) (++(c).launches)

static inline cudaStream_t on(const Context& c, cudaStream_t s) { return s ? s : c.stream; }

// Blocks of the fixed-layout reductions: one partial sum per block of the
// cost-target (functional) and actuator (sensitivity) point lists.
int reductionBlocks(const DevBlock& b) {
  return std::max({1, (b.v.nTgt + kBlock - 1) / kBlock, (b.v.nAct + kBlock - 1) / kBlock});
}

void launchPrims(Context& c, DevBlock& b, const double* qSrc, bool copyToQ, const RunScalars* rs, int stage,
                 cudaStream_t s) {
  RunScalars r{};
  if (rs) r = *rs;
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kPrims<2>, gridFor(b.v.N), kBlock, on(c, s), b.v, c.phys, qSrc, copyToQ, r, stage);
  else pdl(kPrims<3>, gridFor(b.v.N), kBlock, on(c, s), b.v, c.phys, qSrc, copyToQ, r, stage);
}

void launchGradFlux(Context& c, DevBlock& b, bool writeFlux, bool writeStress, const RunScalars* rs, int stage,
                    bool storeStage, cudaStream_t s) {
  const int flags = (writeFlux ? GF_FLUX : 0) | (writeStress ? GF_STRESS : 0) | (storeStage ? GF_STORE : 0);
  RunScalars r{};
  if (rs) r = *rs;
  const Tile T = b.tGrad;
  const bool curv = b.v.curvilinear != 0, visc = c.phys.viscous != 0;
  MGD_LAUNCH(c);
#define GF(ND, CU, VI) \
  pdl(kGradFlux<ND, CU, VI>, T.blocks(), T.threads(), on(c, s), b.v, c.phys, r, flags, stage, T)
#define GP(CU, VI) \
  pdl(kGradFluxPair<CU, VI>, T.blocks(), 2 * T.threads(), on(c, s), b.v, c.phys, r, flags, stage, T)
  if (c.nD == 2 && b.gradLanes == 2) {
    if (curv) { if (visc) GP(true, true); else GP(true, false); }
    else { if (visc) GP(false, true); else GP(false, false); }
  } else if (c.nD == 2) {
    if (curv) { if (visc) GF(2, true, true); else GF(2, true, false); }
    else { if (visc) GF(2, false, true); else GF(2, false, false); }
  } else {
    if (curv) { if (visc) GF(3, true, true); else GF(3, true, false); }
    else { if (visc) GF(3, false, true); else GF(3, false, false); }
  }
#undef GF
#undef GP
}

void launchDissipation(Context& c, DevBlock& b, const double* src, double sign, cudaStream_t s) {
  if (!c.phys.dissipation) return;
  if (tmaDissipationEligible(c, b) && launchDissipationTma(c, b, src, sign, on(c, s))) return;
  const Tile T = b.tDiss;
  const dim3 grid(T.blocks(), c.nU);
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kDissipation<2>, grid, T.threads(), on(c, s), b.v, c.phys, src, sign, T);
  else pdl(kDissipation<3>, grid, T.threads(), on(c, s), b.v, c.phys, src, sign, T);
}

void launchForwardDivergence(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, bool api, bool controller,
                             cudaStream_t s) {
  const int stage = api ? 1 : rkStage;
  const Tile T = b.tRhs;
  const dim3 grid(T.blocks(), c.nU);
  MGD_LAUNCH(c);
  if (c.nD == 2)
    pdl(kForwardDivergence<2>, grid, T.threads(), on(c, s), b.v, c.phys, rs, rkStage, stage, controller, T, 0, 0.0);
  else
    pdl(kForwardDivergence<3>, grid, T.threads(), on(c, s), b.v, c.phys, rs, rkStage, stage, controller, T, 0, 0.0);
}

void launchLinearizedFlux(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot, cudaStream_t s) {
  const cudaStream_t st = on(c, s);
  const int fsl = fromSlot ? 1 : 0;
  if (c.phys.viscous) {
    MGD_LAUNCH(c);
    if (c.nD == 2) pdl(kLinearizedTemp<2>, gridFor(b.v.N), kBlock, st, b.v, c.phys, rs, stage, fsl);
    else pdl(kLinearizedTemp<3>, gridFor(b.v.N), kBlock, st, b.v, c.phys, rs, stage, fsl);
  }
  const Tile T = b.tGrad;
  MGD_LAUNCH(c);
#define LF(ND, VISC) pdl(kLinearizedFlux<ND, VISC>, T.blocks(), T.threads(), st, b.v, c.phys, rs, stage, fsl, T)
  if (c.nD == 2) { if (c.phys.viscous) LF(2, true); else LF(2, false); }
  else { if (c.phys.viscous) LF(3, true); else LF(3, false); }
#undef LF
}

void launchInterfaceSatLinearized(Context& c, DevBlock& b, const BlockRefs& r, const RunScalars* rs, int stage,
                                  bool fromSlot, cudaStream_t s) {
  if (b.nInterfaceEntries == 0) return;
  const int G = gridFor(b.v.ff.n);
  const RunScalars x = rs ? *rs : RunScalars{};
  const int fsl = fromSlot ? 1 : 0;
  MGD_LAUNCH(c);
  if (c.nD == 2) {
    if (c.phys.viscous) pdl(kInterfaceSatLinearized<2, true>, G, kBlock, on(c, s), b.v, c.phys, r, x, stage, fsl);
    else pdl(kInterfaceSatLinearized<2, false>, G, kBlock, on(c, s), b.v, c.phys, r, x, stage, fsl);
  } else {
    if (c.phys.viscous) pdl(kInterfaceSatLinearized<3, true>, G, kBlock, on(c, s), b.v, c.phys, r, x, stage, fsl);
    else pdl(kInterfaceSatLinearized<3, false>, G, kBlock, on(c, s), b.v, c.phys, r, x, stage, fsl);
  }
}

void launchLinearizedDivergence(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, double factor, int stage,
                                bool controller, cudaStream_t s) {
  // the divergence and RK update act on the perturbation: a view with q = lambda
  BlockView v = b.v;
  v.q = b.v.lam;
  const Tile T = b.tRhs;
  const dim3 grid(T.blocks(), c.nU);
  const int ctl = controller ? 1 : 0;
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kForwardDivergence<2>, grid, T.threads(), on(c, s), v, c.phys, rs, rkStage, stage, ctl, T, 1, factor);
  else pdl(kForwardDivergence<3>, grid, T.threads(), on(c, s), v, c.phys, rs, rkStage, stage, ctl, T, 1, factor);
}

void launchLinearized(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, double factor, int stage,
                      bool fromSlot, bool controller, cudaStream_t s) {
  launchLinearizedFlux(c, b, rs, stage, fromSlot, s);
  launchLinearizedDivergence(c, b, rkStage, rs, factor, stage, controller, s);
}

void launchFunctional(Context& c, DevBlock& b, const RunScalars& rs, int stage, cudaStream_t s) {
  MGD_LAUNCH(c);
  pdl(kFunctional, reductionBlocks(b), kBlock, on(c, s), b.v, rs, stage, PrimLayout{c.nD}.p());
}

void launchExcitation(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool adjoint, bool fromSlot,
                      cudaStream_t s) {
  for (const ExcPatch& X : b.exc) {
    if (X.nE == 0) continue;
    const int grid = (X.nE + kBlock - 1) / kBlock;
    MGD_LAUNCH(c);
    if (c.nD == 2) pdl(kExcitation<2>, grid, kBlock, on(c, s), b.v, X, rs, stage, (int)adjoint, (int)fromSlot);
    else pdl(kExcitation<3>, grid, kBlock, on(c, s), b.v, X, rs, stage, (int)adjoint, (int)fromSlot);
  }
}

void launchFunctionalTangent(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot, cudaStream_t s) {
  MGD_LAUNCH(c);
  const int fsl = fromSlot ? 1 : 0;
  if (c.nD == 2) pdl(kFunctionalTangent<2>, reductionBlocks(b), kBlock, on(c, s), b.v, c.phys, rs, stage, fsl);
  else pdl(kFunctionalTangent<3>, reductionBlocks(b), kBlock, on(c, s), b.v, c.phys, rs, stage, fsl);
}

void launchGradientSensitivity(Context& c, DevBlock& b, const RunScalars& rs, int stage, cudaStream_t s) {
  MGD_LAUNCH(c);
  pdl(kGradientSensitivity, reductionBlocks(b), kBlock, on(c, s), b.v, rs, stage, c.nD + 1);
}

void launchAdjointCore(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot, cudaStream_t s) {
  const Tile T = b.tAdjA;
  const int G = T.blocks(), W = T.threads();
  cudaStream_t st = on(c, s);
  const bool curv = b.v.curvilinear != 0, visc = c.phys.viscous != 0;
  MGD_LAUNCH(c);
  if (b.coreLanes == 2 && c.nD == 2) {
    // nD threads per point; their shares meet in shared memory
    const size_t smem = (size_t)2 * (4 + 2 * 3) * W * sizeof(double);
#define ACS(CU, VI) pdlShared(kAdjointCoreSplit<2, CU, VI>, G, 2 * W, smem, st, b.v, c.phys, rs, stage, fromSlot, T)
    if (curv) { if (visc) ACS(true, true); else ACS(true, false); }
    else { if (visc) ACS(false, true); else ACS(false, false); }
#undef ACS
    return;
  }
#define AC(ND, CU, VI) pdl(kAdjointCore<ND, CU, VI>, G, W, st, b.v, c.phys, rs, stage, fromSlot, T)
  if (c.nD == 2) {
    if (curv) { if (visc) AC(2, true, true); else AC(2, true, false); }
    else { if (visc) AC(2, false, true); else AC(2, false, false); }
  } else {
    if (curv) { if (visc) AC(3, true, true); else AC(3, true, false); }
    else { if (visc) AC(3, false, true); else AC(3, false, false); }
  }
#undef AC
}

void launchAdjointSatVectors(Context& c, DevBlock& b, const RunScalars& rs, int stage, bool fromSlot,
                             cudaStream_t s) {
  const int n = b.v.ff.n;
  if (n - b.nInterfaceEntries <= 0) return;  // no wall or far-field entry
  MGD_LAUNCH(c);
  const int fs = fromSlot ? 1 : 0;
  if (c.nD == 2) {
    if (c.phys.viscous) pdl(kAdjointSatVectors<2, true>, gridFor(n), kBlock, on(c, s), b.v, c.phys, rs, stage, fs);
    else pdl(kAdjointSatVectors<2, false>, gridFor(n), kBlock, on(c, s), b.v, c.phys, rs, stage, fs);
  } else {
    if (c.phys.viscous) pdl(kAdjointSatVectors<3, true>, gridFor(n), kBlock, on(c, s), b.v, c.phys, rs, stage, fs);
    else pdl(kAdjointSatVectors<3, false>, gridFor(n), kBlock, on(c, s), b.v, c.phys, rs, stage, fs);
  }
}

void launchAdjointDiffusion(Context& c, DevBlock& b, cudaStream_t s) {
  if (!c.phys.viscous) return;
  const Tile T = b.tAdjD;
  const dim3 grid(T.blocks(), c.nU - 1);
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kAdjointDiffusion<2>, grid, T.threads(), on(c, s), b.v, T);
  else pdl(kAdjointDiffusion<3>, grid, T.threads(), on(c, s), b.v, T);
}

void launchAdjointAssemble(Context& c, DevBlock& b, int rkStage, const RunScalars& rs, int stage, double apiFactor,
                           bool api, bool fromSlot, cudaStream_t s) {
  const Tile T = b.tAdjB;
  const dim3 grid(T.blocks(), c.nU);
  const int W = T.threads();
  cudaStream_t st = on(c, s);
  MGD_LAUNCH(c);
#define AA(ND, VI) \
  pdl(kAdjointAssemble<ND, VI>, grid, W, st, b.v, c.phys, rs, rkStage, stage, apiFactor, api, fromSlot, T)
  if (c.nD == 2) {
    if (c.phys.viscous) AA(2, true); else AA(2, false);
  } else {
    if (c.phys.viscous) AA(3, true); else AA(3, false);
  }
#undef AA
}

void launchAdjointInitial(Context& c, DevBlock& b, double factor) {
  MGD_LAUNCH(c);
  const int acc = c.adjointNonzeroIC ? 1 : 0;
  if (c.nD == 2) pdl(kAdjointInitial<2>, gridFor(b.v.N), kBlock, c.stream, b.v, c.phys, factor, acc);
  else pdl(kAdjointInitial<3>, gridFor(b.v.N), kBlock, c.stream, b.v, c.phys, factor, acc);
}

void launchStoreAdjointForcing(Context& c, DevBlock& b, bool zero) {
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kStoreAdjointForcing<2>, gridFor(b.v.N), kBlock, c.stream, b.v, c.phys, zero);
  else pdl(kStoreAdjointForcing<3>, gridFor(b.v.N), kBlock, c.stream, b.v, c.phys, zero);
}

void launchSnapshot(Context& c, DevBlock& b, double* snapshots, int saveInterval, bool initial, cudaStream_t s) {
  const long long n = b.v.N * b.v.nU;
  MGD_LAUNCH(c);
  pdl(kSnapshot, gridFor(n), kBlock, on(c, s), snapshots, b.v.q, n, c.dCounters, saveInterval, initial);
}

void launchStepAdvance(Context& c, int delta, cudaStream_t s) {
  MGD_LAUNCH(c);
  pdl(kStepAdvance, 1, 32, on(c, s), c.dCounters, delta);
}

void launchReducePartials(Context& c, const double* partials, int stride, int count, int nSlots, double* out) {
  if (nSlots <= 0) return;
  MGD_LAUNCH(c);
  pdl(kReducePartials, nSlots, kBlock, c.stream, partials, stride, count, nSlots, out);
}

void launchBatchGradFlux(Context& c, const BatchLaunch& L, int stage, cudaStream_t s) {
  const int G = L.blocks[BK_GRAD], W = L.threads[BK_GRAD];
  const bool curv = c.opts.curvilinear != 0, visc = c.phys.viscous != 0;
  MGD_LAUNCH(c);
#define GFB(ND, CU, VI) pdl(kGradFluxBatch<ND, CU, VI>, G, W, s, L.entries, L.map[BK_GRAD], c.phys, stage)
  if (c.nD == 2) {
    if (curv) { if (visc) GFB(2, true, true); else GFB(2, true, false); }
    else { if (visc) GFB(2, false, true); else GFB(2, false, false); }
  } else {
    if (curv) { if (visc) GFB(3, true, true); else GFB(3, true, false); }
    else { if (visc) GFB(3, false, true); else GFB(3, false, false); }
  }
#undef GFB
}

void launchBatchDissipation(Context& c, const BatchLaunch& L, cudaStream_t s) {
  if (!c.phys.dissipation) return;
  const dim3 grid(L.blocks[BK_DISS], c.nU);
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kDissipationBatch<2>, grid, L.threads[BK_DISS], s, L.entries, L.map[BK_DISS], c.phys);
  else pdl(kDissipationBatch<3>, grid, L.threads[BK_DISS], s, L.entries, L.map[BK_DISS], c.phys);
}

void launchBatchForwardDivergence(Context& c, const BatchLaunch& L, int rkStage, cudaStream_t s) {
  const dim3 grid(L.blocks[BK_RHS], c.nU);
  MGD_LAUNCH(c);
  if (c.nD == 2)
    pdl(kForwardDivergenceBatch<2>, grid, L.threads[BK_RHS], s, L.entries, L.map[BK_RHS], c.phys, rkStage);
  else
    pdl(kForwardDivergenceBatch<3>, grid, L.threads[BK_RHS], s, L.entries, L.map[BK_RHS], c.phys, rkStage);
}

void launchBatchPrims(Context& c, const BatchLaunch& L, cudaStream_t s) {
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kPrimsBatch<2>, L.blocks[BK_PRIMS], kBlock, s, L.entries, L.map[BK_PRIMS], c.phys);
  else pdl(kPrimsBatch<3>, L.blocks[BK_PRIMS], kBlock, s, L.entries, L.map[BK_PRIMS], c.phys);
}

void launchBatchFunctional(Context& c, const BatchLaunch& L, int stage, cudaStream_t s) {
  MGD_LAUNCH(c);
  pdl(kFunctionalBatch, L.blocks[BK_FUNC], kBlock, s, L.entries, L.map[BK_FUNC], stage, PrimLayout{c.nD}.p());
}

void launchSolutionLimits(Context& c, DevBlock& b, int blockIndex, const int* step, int stage,
                          unsigned long long* key, cudaStream_t s) {
  const SolutionLimits L{c.opts.minimum_density, c.opts.maximum_density, c.opts.minimum_temperature,
                         c.opts.maximum_temperature};
  if (c.nD == 2)
    pdl(kSolutionLimits<2>, gridFor(b.v.N), kBlock, on(c, s), b.v, L, step, stage, blockIndex, key);
  else
    pdl(kSolutionLimits<3>, gridFor(b.v.N), kBlock, on(c, s), b.v, L, step, stage, blockIndex, key);
  MGD_LAUNCH(c);
}

template <int ND, bool CURV, bool VISC>
static int persistentOccupancy() {
  int perSm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kBatchRunPersistent<ND, CURV, VISC>, kBatchThreads, 0);
  return perSm;
}

int selftestGridBarrier(int nBlocks, unsigned int expected, int rounds, long long limit, int* status,
                        long long* sum) {
  unsigned long long* bar = nullptr;
  int* err = nullptr;
  long long *stamps = nullptr, *dsum = nullptr;
  cudaError_t e = cudaMalloc((void**)&bar, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void**)&err, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&stamps, (size_t)nBlocks * sizeof(long long));
  if (e == cudaSuccess) e = cudaMalloc((void**)&dsum, sizeof(long long));
  if (e == cudaSuccess) e = cudaMemset(bar, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dsum, 0, sizeof(long long));
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(nBlocks);
    cfg.blockDim = dim3(32);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kBarrierSelfTest, bar, err, limit, expected, rounds, stamps, dsum);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(status, err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sum, dsum, sizeof(long long), cudaMemcpyDeviceToHost);
  cudaFree(bar);
  cudaFree(err);
  cudaFree(stamps);
  cudaFree(dsum);
  return e == cudaSuccess ? 0 : (int)e;
}

// FP64 throughput probe: every thread runs four independent DFMA chains of
// `iters` steps and writes one value (out holds gridDim.x * blockDim.x).
__global__ void kFp64Chains(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = (x0 + x1) + (x2 + x3);
}

int selftestFp64Rate(int warpsPerSm, double* laneOpsPerClock) {
  int dev = 0, sms = 0, clockKHz = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&clockKHz, cudaDevAttrClockRate, dev);
  const int threads = 32 * warpsPerSm, iters = 4096;
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc((void**)&out, (size_t)sms * threads * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0.f;
  if (e == cudaSuccess) {
    // one CTA per SM: a warm-up launch, then the timed one
    kFp64Chains<<<sms, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e0);
    kFp64Chains<<<sms, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess)
    *laneOpsPerClock = (double)threads * iters * 4 / (ms * 1e-3) / ((double)clockKHz * 1e3);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return e == cudaSuccess ? 0 : (int)e;
}

int persistentGridSize(const Context& c) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const bool curv = c.opts.curvilinear != 0, visc = c.phys.viscous != 0;
  int perSm = 0;
  if (c.nD == 2) perSm = curv ? (visc ? persistentOccupancy<2, true, true>() : persistentOccupancy<2, true, false>())
                              : (visc ? persistentOccupancy<2, false, true>() : persistentOccupancy<2, false, false>());
  else perSm = curv ? (visc ? persistentOccupancy<3, true, true>() : persistentOccupancy<3, true, false>())
                    : (visc ? persistentOccupancy<3, false, true>() : persistentOccupancy<3, false, false>());
  return perSm * sms;
}

cudaError_t launchBatchPersistent(Context& c, const BatchEntry* entries, const PersistentPlan& plan, int nSteps,
                                  int functional, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBatchThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const bool curv = c.opts.curvilinear != 0, visc = c.phys.viscous != 0;
  MGD_LAUNCH(c);
#define PK(ND, CU, VI) cudaLaunchKernelEx(&cfg, kBatchRunPersistent<ND, CU, VI>, entries, plan, c.phys, nSteps, functional)
  if (c.nD == 2) {
    if (curv) return visc ? PK(2, true, true) : PK(2, true, false);
    return visc ? PK(2, false, true) : PK(2, false, false);
  }
  if (curv) return visc ? PK(3, true, true) : PK(3, true, false);
  return visc ? PK(3, false, true) : PK(3, false, false);
#undef PK
}

void launchStepAdvanceOn(int* counters, int delta, cudaStream_t s) { pdl(kStepAdvance, 1, 32, s, counters, delta); }

__global__ void kSetCounters(int* counters, int step, int segBase) {
  pdlEnter();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    counters[0] = step;
    counters[1] = segBase;
  }
}

void launchSetCounters(int* counters, int step, int segBase, cudaStream_t s) {
  pdl(kSetCounters, 1, 32, s, counters, step, segBase);
}

int timeStepBlocks(const DevBlock& b) { return gridFor(b.v.N); }

// z = a x + (accumulate ? z : 0) (ZAXPY, bin/ZAXPY.f90).
__global__ void kAxpy(double* __restrict__ z, const double* __restrict__ x, double a, long long n, int accumulate) {
  pdlEnter();
  const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
  if (i >= n) return;
  z[i] = accumulate ? a * x[i] + z[i] : a * x[i];
}

void launchAxpy(Context& c, double* z, const double* x, double a, long long n, bool accumulate) {
  if (n <= 0) return;
  MGD_LAUNCH(c);
  pdl(kAxpy, (unsigned)((n + kBlock - 1) / kBlock), kBlock, c.stream, z, x, a, n, accumulate ? 1 : 0);
}

void launchInterfaceSat(Context& c, DevBlock& b, const BlockRefs& r, cudaStream_t s) {
  if (b.nInterfaceEntries == 0) return;
  const int G = gridFor(b.v.ff.n);
  MGD_LAUNCH(c);
  if (c.nD == 2) {
    if (c.phys.viscous) pdl(kInterfaceSat<2, true>, G, kBlock, on(c, s), b.v, c.phys, r);
    else pdl(kInterfaceSat<2, false>, G, kBlock, on(c, s), b.v, c.phys, r);
  } else {
    if (c.phys.viscous) pdl(kInterfaceSat<3, true>, G, kBlock, on(c, s), b.v, c.phys, r);
    else pdl(kInterfaceSat<3, false>, G, kBlock, on(c, s), b.v, c.phys, r);
  }
}

void launchInterfaceSatAdjoint(Context& c, DevBlock& b, const BlockRefs& r, const RunScalars* rs, int stage,
                               bool fromSlot, cudaStream_t s) {
  if (b.nInterfaceEntries == 0) return;
  RunScalars x{};
  if (rs) x = *rs;
  const int fs = fromSlot ? 1 : 0, n = b.nInterfaceEntries;
  MGD_LAUNCH(c);
  if (c.nD == 2) {
    const int G = (n + InterfaceLanes<2>::entriesPerWarp - 1) / InterfaceLanes<2>::entriesPerWarp;
    if (c.phys.viscous) pdl(kInterfaceSatAdjoint<2, true>, G, 32, on(c, s), b.v, c.phys, r, x, stage, fs, n);
    else pdl(kInterfaceSatAdjoint<2, false>, G, 32, on(c, s), b.v, c.phys, r, x, stage, fs, n);
  } else {
    const int G = (n + InterfaceLanes<3>::entriesPerWarp - 1) / InterfaceLanes<3>::entriesPerWarp;
    if (c.phys.viscous) pdl(kInterfaceSatAdjoint<3, true>, G, 32, on(c, s), b.v, c.phys, r, x, stage, fs, n);
    else pdl(kInterfaceSatAdjoint<3, false>, G, 32, on(c, s), b.v, c.phys, r, x, stage, fs, n);
  }
}

void launchKineticEnergy(Context& c, DevBlock& b, const double* norm, double* partials, double* out) {
  const int nb = gridFor(b.v.N);
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kKineticEnergyPartials<2>, nb, kBlock, c.stream, b.v, norm, partials);
  else pdl(kKineticEnergyPartials<3>, nb, kBlock, c.stream, b.v, norm, partials);
  launchReducePartials(c, partials, nb, nb, 1, out);
}

void launchKineticEnergyAdjointInitial(Context& c, DevBlock& b) {
  MGD_LAUNCH(c);
  const int acc = c.adjointNonzeroIC ? 1 : 0;
  if (c.nD == 2) pdl(kKineticEnergyAdjointInitial<2>, gridFor(b.v.N), kBlock, c.stream, b.v, acc);
  else pdl(kKineticEnergyAdjointInitial<3>, gridFor(b.v.N), kBlock, c.stream, b.v, acc);
}

void launchTimeStep(Context& c, DevBlock& b, double* partials, double* dtOut, const int* step, double* time,
                    double* stageTime, double* amp, cudaStream_t s) {
  const int nb = timeStepBlocks(b);
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kTimeStepPartials<2>, nb, kBlock, on(c, s), b.v, c.phys, c.opts.cfl, partials);
  else pdl(kTimeStepPartials<3>, nb, kBlock, on(c, s), b.v, c.phys, c.opts.cfl, partials);
  SourceTable src{};
  src.n = (int)c.sources.size();
  src.twoPi = 2.0 * (4.0 * std::atan(1.0));
  for (int k = 0; k < src.n; ++k) {
    src.amplitude[k] = c.sources[k].amplitude;
    src.frequency[k] = c.sources[k].frequency;
    src.phase[k] = c.sources[k].phase;
  }
  MGD_LAUNCH(c);
  pdl(kTimeStepFinalize, 1, 256, on(c, s), partials, nb, dtOut, step, time, stageTime, amp, src);
}

// The same over every block of a region: each block's partial minima at its
// offset in partials, one finalize over all of them (the minimum over blocks
// of Region%getTimeStepSize, src/RegionImpl.f90:1842-1875).
void launchTimeStepRegion(Context& c, double* partials, double* dtOut, const int* step, double* time,
                          double* stageTime, double* amp, cudaStream_t s) {
  int off = 0;
  for (DevBlock& b : c.blocks) {
    const int nb = timeStepBlocks(b);
    MGD_LAUNCH(c);
    if (c.nD == 2) pdl(kTimeStepPartials<2>, nb, kBlock, on(c, s), b.v, c.phys, c.opts.cfl, partials + off);
    else pdl(kTimeStepPartials<3>, nb, kBlock, on(c, s), b.v, c.phys, c.opts.cfl, partials + off);
    off += nb;
  }
  SourceTable src{};
  src.n = (int)c.sources.size();
  src.twoPi = 2.0 * (4.0 * std::atan(1.0));
  for (int k = 0; k < src.n; ++k) {
    src.amplitude[k] = c.sources[k].amplitude;
    src.frequency[k] = c.sources[k].frequency;
    src.phase[k] = c.sources[k].phase;
  }
  MGD_LAUNCH(c);
  pdl(kTimeStepFinalize, 1, 256, on(c, s), partials, off, dtOut, step, time, stageTime, amp, src);
}

void launchCoordinateDerivative(Context& c, DevBlock& b, int dir, double* out) {
  const double* coords = b.v.q;  // caller stages the coordinates in q
  MGD_LAUNCH(c);
  if (c.nD == 2)
    pdl(kCoordinateDerivative<2>, gridFor(b.v.N), kBlock, c.stream, b.v, coords, dir, b.desc.periodic_length[dir], out);
  else
    pdl(kCoordinateDerivative<3>, gridFor(b.v.N), kBlock, c.stream, b.v, coords, dir, b.desc.periodic_length[dir], out);
}

void launchApplyD1(Context& c, DevBlock& b, int dir, const double* in, double* out, int ncomp) {
  MGD_LAUNCH(c);
  pdl(kApplyD1, gridFor(b.v.N), kBlock, c.stream, b.v, dir, in, out, ncomp);
}

void launchFarFieldTargetVisc(Context& c, DevBlock& b) {
  if (b.v.ff.n == 0) return;
  MGD_LAUNCH(c);
  if (c.nD == 2) pdl(kFarFieldTargetVisc<2>, gridFor(b.v.ff.n), kBlock, c.stream, b.v);
  else pdl(kFarFieldTargetVisc<3>, gridFor(b.v.ff.n), kBlock, c.stream, b.v);
}

// Far-field matrices from per-entry inviscid penalty and signed normal direction.
// (Wall entries get matrices too; their SAT kernels do not read them.)
void launchFarFieldMatricesWith(Context& c, DevBlock& b, const double* sigInv, const int* signedNormal) {
  if (b.v.ff.n == 0) return;
  MGD_LAUNCH(c);
  if (c.nD == 2)
    pdl(kFarFieldMatrices<2>, gridFor(b.v.ff.n), kBlock, c.stream, b.v, c.phys.g, sigInv, signedNormal);
  else
    pdl(kFarFieldMatrices<3>, gridFor(b.v.ff.n), kBlock, c.stream, b.v, c.phys.g, sigInv, signedNormal);
}

}  // namespace mgd
