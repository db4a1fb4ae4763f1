// mgd_device.cuh -- device-side building blocks: SBP operator application
// from constant-memory tables and the pointwise gas dynamics of magudi's
// CNSHelper (src/CNSHelperImpl.f90), all in FP64.
//
// Design note: on GB300 FP64 arithmetic runs on a narrow pipe while integer,
// FP32 and load/store issue slots are plentiful, so these routines minimise
// FP64 instruction count (no recomputation, algebraic sharing) and leave
// index arithmetic and loads unoptimised.
#pragma once

#include <cstdint>

namespace mgd {

enum OpId { OP_D1 = 0, OP_D1ADJ = 1, OP_DISS = 2, OP_DISST = 3, OP_DCOMP = 4, OP_COUNT = 5 };

// Compile-time shape of each operator's boundary block.
template <int OP> struct OpShape;
template <> struct OpShape<OP_D1> { static constexpr int depth = 8, width = 12, half = 4; static constexpr bool skew = true; };
template <> struct OpShape<OP_D1ADJ> { static constexpr int depth = 12, width = 16, half = 4; static constexpr bool skew = true; };
template <> struct OpShape<OP_DISS> { static constexpr int depth = 2, width = 5, half = 2; static constexpr bool skew = false; };
template <> struct OpShape<OP_DISST> { static constexpr int depth = 8, width = 10, half = 2; static constexpr bool skew = false; };
template <> struct OpShape<OP_DCOMP> { static constexpr int depth = 8, width = 12, half = 4; static constexpr bool skew = false; };

// SBP schemes (defaults/discretization_scheme): index = MGD_SBP_* (4-8, 1-2,
// 2-4, 3-6). Every scheme's operators are stored in the fixed shapes of
// OpShape (the 4-8 shapes, the largest): lower-order closures are padded
// with interior rows and their interiors with zero coefficients.
constexpr int kSchemes = 4;

struct OpTables {
  double interior[kSchemes][OP_COUNT][9];  // offsets -half..half
  int asym[kSchemes][OP_COUNT];            // general interior sum and explicit right block
};

// One copy per translation unit; only mgd_kernels.cu launches kernels and
// fills them. Interior coefficients are uniform across a warp and live in
// constant memory; boundary-closure rows differ between lanes and are read
// from global memory through L1, which serves divergent addresses at once.
static __constant__ OpTables c_ops;
static __device__ double g_opLeft[kSchemes][OP_COUNT][16 * 12];
static __device__ double g_opRight[kSchemes][OP_COUNT][16 * 12];  // explicit right blocks (asym only)

// One direction of a block: n points along it, memory stride, periodicity,
// and the block's SBP scheme.
struct Axis {
  int n;
  int per;          // 0 none, 1 plane, 2 overlap
  long long stride;
  int scheme;       // MGD_SBP_*
};

// Index of point i + j along a periodic line (fillGhostPoints for one
// process, src/MPIHelperImpl.f90:113-390): PLANE wraps with period n;
// OVERLAP skips the duplicated end point.
__device__ __forceinline__ int wrapIndex(int i, int n, int per) {
  if (i < 0) return per == 2 ? i + n - 1 : i + n;
  if (i >= n) return per == 2 ? i - n + 1 : i - n;
  return i;
}

// y_i = (Op x)_i along one axis; `line` points at element 0 of the pencil.
// Follows applyOperator_{1,2,3} (src/StencilOperatorImpl.f90:35-457):
// sum over taps left to right, boundary rows from the left block and its
// (skew-)reflection on the right.
// Load of a stencil tap: through the read-only data path (NC), or as an
// ordinary cached load (ld.global.ca) for data that the same kernel launch
// writes elsewhere (the persistent batched kernel). The read-only path lies
// outside the memory model and may serve such data stale; ordinary loads
// after the acquiring fence of a grid barrier see the other CTAs' writes and
// still share L1 lines between neighbouring points within a phase.
template <bool NC>
__device__ __forceinline__ double tap(const double* p) {
  if constexpr (NC) return __ldg(p);
  else return __ldca(p);
}

template <int OP, bool NC = true, int CU = 1>
__device__ __forceinline__ double applyOp(const double* __restrict__ line, int i, const Axis& ax) {
  using S = OpShape<OP>;
  const double* __restrict__ cin = c_ops.interior[ax.scheme][OP];
  // only the non-composite dissipation pair of SBP 3-6 is asymmetric
  const bool asym = !S::skew && (OP == OP_DISS || OP == OP_DISST) && c_ops.asym[ax.scheme][OP];
  const long long st = ax.stride;
  if (ax.per == 0) {
    if (i < S::depth) {
      // boundary closure rows: CU taps' loads in flight at a time (the sum
      // keeps its order either way)
      const double* __restrict__ row = &g_opLeft[ax.scheme][OP][i * S::width];
      double s = __ldg(row) * tap<NC>(line);
#pragma unroll CU
      for (int k = 1; k < S::width; ++k) s += __ldg(row + k) * tap<NC>(line + k * st);
      return s;
    }
    if (i >= ax.n - S::depth) {
      const int m = ax.n - 1 - i;
      const double* __restrict__ end = line + (long long)(ax.n - S::width) * st;
      if (asym) {
        // explicit right block, columns left to right
        const double* __restrict__ row = &g_opRight[ax.scheme][OP][m * S::width];
        double s = __ldg(row) * tap<NC>(end);
#pragma unroll CU
        for (int k = 1; k < S::width; ++k) s += __ldg(row + k) * tap<NC>(end + k * st);
        return s;
      }
      const double* __restrict__ row = &g_opLeft[ax.scheme][OP][m * S::width];
      // right block = reflection of the left block, negated for skew operators
      double s = __ldg(row + S::width - 1) * tap<NC>(end);
#pragma unroll CU
      for (int k = 1; k < S::width; ++k) s += __ldg(row + S::width - 1 - k) * tap<NC>(end + k * st);
      return S::skew ? -s : s;
    }
    const double* __restrict__ c = line + (long long)i * st;
    if (S::skew) {
      double s = cin[S::half + 1] * (tap<NC>(c + st) - tap<NC>(c - st));
#pragma unroll
      for (int j = 2; j <= S::half; ++j) s += cin[S::half + j] * (tap<NC>(c + j * st) - tap<NC>(c - j * st));
      return s;
    } else if (asym) {
      double s = cin[0] * tap<NC>(c - S::half * st);
#pragma unroll
      for (int j = 1 - S::half; j <= S::half; ++j) s += cin[S::half + j] * tap<NC>(c + j * st);
      return s;
    } else {
      double s = cin[S::half + 1] * (tap<NC>(c + st) + tap<NC>(c - st));
#pragma unroll
      for (int j = 2; j <= S::half; ++j) s += cin[S::half + j] * (tap<NC>(c + j * st) + tap<NC>(c - j * st));
      return s + cin[S::half] * tap<NC>(c);
    }
  }
  // periodic: interior stencil everywhere with wrapped indices
  auto at = [&](int j) { return tap<NC>(line + (long long)wrapIndex(i + j, ax.n, ax.per) * st); };
  if (asym) {
    double s = cin[0] * at(-S::half);
#pragma unroll
    for (int j = 1 - S::half; j <= S::half; ++j) s += cin[S::half + j] * at(j);
    return s;
  }
  if (S::skew) {
    double s = cin[S::half + 1] * (at(1) - at(-1));
#pragma unroll
    for (int j = 2; j <= S::half; ++j) s += cin[S::half + j] * (at(j) - at(-j));
    return s;
  } else {
    double s = cin[S::half + 1] * (at(1) + at(-1));
#pragma unroll
    for (int j = 2; j <= S::half; ++j) s += cin[S::half + j] * (at(j) + at(-j));
    return s + cin[S::half] * at(0);
  }
}

// x != 0.0 with integer operations: false for +0 and -0 only, as the
// comparison is (NaN and every other value compare unequal to zero). GB300
// runs double-precision compares on the FP64 pipe, which the stage kernels
// keep busy; integer tests leave it to the arithmetic.
__device__ __forceinline__ bool nonzero(double x) { return (__double_as_longlong(x) << 1) != 0; }

// ---------------------------------------------------------------------------
// x^n for x > 0 in FP64 with few FP64 operations, after P. T. P. Tang's
// table-driven logarithm and exponential (ACM TOMS 15(2), 1989; 16(4), 1990):
//   log x = e ln2 + log(F) + log1p(m/F - 1), F from a 128-entry table
//   exp y = 2^(k/64) exp(r), |r| <= ln2/128, 2^(j/64) from a 64-entry table.
// Exponent and mantissa are split with integer operations, which do not
// occupy the FP64 pipe. Non-positive or non-finite x falls back to pow().
// ---------------------------------------------------------------------------
struct PowTables {
  double invF[128];   // G_j = 1 / F_j rounded, F_j = 1 + (j + 1/2)/128
  double logFhi[128]; // -log G_j, high part
  double logFlo[128]; // -log G_j, low part
  double exp2j[64];   // 2^(j/64)
};

__device__ __forceinline__ double fastPowPositive(double x, double n, const PowTables* __restrict__ tab) {
  const long long bits = __double_as_longlong(x);
  const int be = (int)((bits >> 52) & 0x7FF);
  // bits <= 0: x is -0, +0 or negative (the NaNs and infinities have be == 0x7FF)
  if (bits <= 0 || be == 0 || be == 0x7FF) return pow(x, n);
  const int e = be - 1023;
  const int j = (int)((bits >> 45) & 0x7F);
  const double m = __longlong_as_double((bits & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  const double t = fma(m, __ldg(&tab->invF[j]), -1.0);  // |t| < 2^-8
  // log1p(t) - t = t^2 (-1/2 + t/3 - t^2/4 + ... - t^6/8)
  double q = -1.0 / 8.0;
  q = fma(q, t, 1.0 / 7.0);
  q = fma(q, t, -1.0 / 6.0);
  q = fma(q, t, 1.0 / 5.0);
  q = fma(q, t, -1.0 / 4.0);
  q = fma(q, t, 1.0 / 3.0);
  q = fma(q, t, -0.5);
  const double t2 = t * t;
  const double ln2hi = 6.93147180369123816490e-01, ln2lo = 1.90821492927058770002e-10;
  const double ed = (double)e;
  const double lo = fma(t2, q, fma(ed, ln2lo, __ldg(&tab->logFlo[j])));
  const double hi = fma(ed, ln2hi, __ldg(&tab->logFhi[j]));
  const double logx = hi + (t + lo);
  const double y = n * logx;
  // exp(y): y = k ln2/64 + r
  const double inv = 92.332482616893656877;  // 64 / ln 2
  const double shifter = 6755399441055744.0;   // 1.5 * 2^52: rounds to an integer
  const double kd_s = fma(y, inv, shifter);
  const long long kbits = __double_as_longlong(kd_s);
  const double kd = kd_s - shifter;
  const double l64hi = 0.01083042469326756, l64lo = 2.9815858269852933e-12;  // ln2/64 = hi + lo, hi*k exact
  double r = fma(-kd, l64hi, y);
  r = fma(-kd, l64lo, r);
  double pe = 1.0 / 720.0;
  pe = fma(pe, r, 1.0 / 120.0);
  pe = fma(pe, r, 1.0 / 24.0);
  pe = fma(pe, r, 1.0 / 6.0);
  pe = fma(pe, r, 0.5);
  pe = fma(pe * r, r, r);                      // exp(r) - 1
  const int k = (int)(kbits & 0xFFFFFFFFLL);
  const int jj = k & 63, kk = k >> 6;
  const double tj = __ldg(&tab->exp2j[jj]);
  const double res = fma(tj, pe, tj);
  // scale by 2^kk through the exponent field (result stays normal here)
  return __longlong_as_double(__double_as_longlong(res) + ((long long)kk << 52));
}

// ---------------------------------------------------------------------------
// Pointwise gas dynamics (FP64). Layouts follow the reference: metrics of
// direction i are m[nD*i + 0..nD-1]; stress tau[nD*c + d] = tau_{c,d}.
// ---------------------------------------------------------------------------

// Incoming Jacobian A+ of the inviscid flux along `metrics` for a state of
// conserved variables cv (computeIncomingJacobianOfInviscidFlux{2D,3D},
// src/CNSHelperImpl.f90:1669-2343). out(i,j) at out[i + nU*j].
// Forward-mode dual number with K directional derivatives. Evaluating the
// incoming Jacobian of a Roe-averaged state on duals seeded with the left
// state gives its exact variation with respect to that state, which the
// block-interface adjoint needs (src/CNSHelperImpl.f90:1669-2343 with
// deltaRoeAverage, src/BlockInterfacePatchImpl.f90:337-420).
template <int K>
struct DualN {
  double v;
  double d[K];
  __host__ __device__ DualN() : v(0.0) {
    for (int k = 0; k < K; ++k) d[k] = 0.0;
  }
  __host__ __device__ DualN(double x) : v(x) {
    for (int k = 0; k < K; ++k) d[k] = 0.0;
  }
};
__host__ __device__ inline double valueOf(double x) { return x; }
template <int K> __host__ __device__ inline double valueOf(const DualN<K>& x) { return x.v; }
template <int K> __host__ __device__ inline DualN<K> operator+(const DualN<K>& a, const DualN<K>& b) {
  DualN<K> r(a.v + b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int K> __host__ __device__ inline DualN<K> operator-(const DualN<K>& a, const DualN<K>& b) {
  DualN<K> r(a.v - b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int K> __host__ __device__ inline DualN<K> operator-(const DualN<K>& a) {
  DualN<K> r(-a.v);
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K> __host__ __device__ inline DualN<K> operator*(const DualN<K>& a, const DualN<K>& b) {
  DualN<K> r(a.v * b.v);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int K> __host__ __device__ inline DualN<K> operator/(const DualN<K>& a, const DualN<K>& b) {
  DualN<K> r(a.v / b.v);
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
  return r;
}
template <int K> __host__ __device__ inline DualN<K> operator+(const DualN<K>& a, double b) { return a + DualN<K>(b); }
template <int K> __host__ __device__ inline DualN<K> operator+(double a, const DualN<K>& b) { return DualN<K>(a) + b; }
template <int K> __host__ __device__ inline DualN<K> operator-(const DualN<K>& a, double b) { return a - DualN<K>(b); }
template <int K> __host__ __device__ inline DualN<K> operator-(double a, const DualN<K>& b) { return DualN<K>(a) - b; }
template <int K> __host__ __device__ inline DualN<K> operator*(const DualN<K>& a, double b) {
  DualN<K> r(a.v * b);
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
  return r;
}
template <int K> __host__ __device__ inline DualN<K> operator*(double a, const DualN<K>& b) { return b * a; }
template <int K> __host__ __device__ inline DualN<K> operator/(const DualN<K>& a, double b) { return a / DualN<K>(b); }
template <int K> __host__ __device__ inline DualN<K> operator/(double a, const DualN<K>& b) { return DualN<K>(a) / b; }
template <int K> __host__ __device__ inline DualN<K>& operator+=(DualN<K>& a, const DualN<K>& b) {
  a = a + b;
  return a;
}
__host__ __device__ inline double sqrtOf(double x) { return sqrt(x); }
template <int K> __host__ __device__ inline DualN<K> sqrtOf(const DualN<K>& a) {
  DualN<K> r(::sqrt(a.v));
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / (2.0 * r.v);
  return r;
}

// Roe average of two conserved states (computeRoeAverage,
// src/CNSHelperImpl.f90:179-351, without the variations).
template <int ND, class S>
__host__ __device__ inline void roeAverage(const S* qL, const S* qR, double g, S* roe) {
  const S sL = sqrtOf(qL[0]), sR = sqrtOf(qR[0]);
  const S vL = 1.0 / qL[0], vR = 1.0 / qR[0];
  S mL2 = qL[1] * qL[1], mR2 = qR[1] * qR[1];
  for (int d = 1; d < ND; ++d) {
    mL2 = mL2 + qL[1 + d] * qL[1 + d];
    mR2 = mR2 + qR[1 + d] * qR[1 + d];
  }
  const S hL = g * qL[ND + 1] - 0.5 * (g - 1.0) * vL * mL2;
  const S hR = g * qR[ND + 1] - 0.5 * (g - 1.0) * vR * mR2;
  roe[0] = sL * sR;
  for (int d = 0; d < ND; ++d) roe[1 + d] = (sR * qL[1 + d] + sL * qR[1 + d]) / (sL + sR);
  roe[ND + 1] = (sR * hL + sL * hR) / (sL + sR);
  S m2 = roe[1] * roe[1];
  for (int d = 1; d < ND; ++d) m2 = m2 + roe[1 + d] * roe[1 + d];
  roe[ND + 1] = (roe[ND + 1] + 0.5 * (g - 1.0) / roe[0] * m2) / g;
}

template <int ND, class S = double>
__host__ __device__ inline void incomingJacobian(const S* cv, const double* metrics, double g,
                                                 int incomingDirection, S* out) {
  constexpr int nU = ND + 2;
  double arc = 0.0;
  for (int d = 0; d < ND; ++d) arc += metrics[d] * metrics[d];
  arc = sqrt(arc);
  double nm[3];
  for (int d = 0; d < ND; ++d) nm[d] = metrics[d] / arc;
  const S v = 1.0 / cv[0];
  S u[3], u2 = 0.0;
  for (int d = 0; d < ND; ++d) u[d] = v * cv[d + 1];
  for (int d = 0; d < ND; ++d) u2 += u[d] * u[d];
  const S T = g * (v * cv[ND + 1] - 0.5 * u2);
  S U = 0.0;
  for (int d = 0; d < ND; ++d) U += nm[d] * u[d];
  const S c = sqrtOf((g - 1.0) * T);
  const S phi2 = 0.5 * (g - 1.0) * u2;
  const S rho = cv[0];
  S R[nU][nU], L[nU][nU], lam[nU];
  if constexpr (ND == 2) {
    lam[0] = U; lam[1] = U; lam[2] = U + c; lam[3] = U - c;
    R[0][0] = 1.0; R[1][0] = u[0]; R[2][0] = u[1]; R[3][0] = phi2 / (g - 1.0);
    R[0][1] = 0.0; R[1][1] = nm[1] * rho; R[2][1] = -nm[0] * rho;
    R[3][1] = rho * (nm[1] * u[0] - nm[0] * u[1]);
    R[0][2] = 1.0; R[1][2] = u[0] + nm[0] * c; R[2][2] = u[1] + nm[1] * c;
    R[3][2] = T + phi2 / (g - 1.0) + c * U;
    R[0][3] = 1.0; R[1][3] = u[0] - nm[0] * c; R[2][3] = u[1] - nm[1] * c;
    R[3][3] = T + phi2 / (g - 1.0) - c * U;
    L[0][0] = 1.0 - phi2 / (c * c);
    L[1][0] = -v * (nm[1] * u[0] - nm[0] * u[1]);
    L[2][0] = 0.5 * (phi2 / (c * c) - U / c);
    L[3][0] = 0.5 * (phi2 / (c * c) + U / c);
    L[0][1] = u[0] / T; L[1][1] = v * nm[1];
    L[2][1] = -0.5 * (u[0] / T - nm[0] / c); L[3][1] = -0.5 * (u[0] / T + nm[0] / c);
    L[0][2] = u[1] / T; L[1][2] = -v * nm[0];
    L[2][2] = -0.5 * (u[1] / T - nm[1] / c); L[3][2] = -0.5 * (u[1] / T + nm[1] / c);
    L[0][3] = -1.0 / T; L[1][3] = 0.0; L[2][3] = 0.5 / T; L[3][3] = 0.5 / T;
  } else {
    lam[0] = U; lam[1] = U; lam[2] = U; lam[3] = U + c; lam[4] = U - c;
    const S h0 = phi2 / (g - 1.0);
    const S q = 1.0 - phi2 / (c * c);
    S (*r)[nU] = R;
    r[0][0] = nm[0]; r[1][0] = nm[0] * u[0]; r[2][0] = nm[0] * u[1] + rho * nm[2];
    r[3][0] = nm[0] * u[2] - rho * nm[1];
    r[4][0] = rho * (nm[2] * u[1] - nm[1] * u[2]) + h0 * nm[0];
    r[0][1] = nm[1]; r[1][1] = nm[1] * u[0] - rho * nm[2]; r[2][1] = nm[1] * u[1];
    r[3][1] = nm[1] * u[2] + rho * nm[0];
    r[4][1] = rho * (nm[0] * u[2] - nm[2] * u[0]) + h0 * nm[1];
    r[0][2] = nm[2]; r[1][2] = nm[2] * u[0] + rho * nm[1]; r[2][2] = nm[2] * u[1] - rho * nm[0];
    r[3][2] = nm[2] * u[2];
    r[4][2] = rho * (nm[1] * u[0] - nm[0] * u[1]) + h0 * nm[2];
    r[0][3] = 1.0; r[1][3] = u[0] + nm[0] * c; r[2][3] = u[1] + nm[1] * c;
    r[3][3] = u[2] + nm[2] * c; r[4][3] = T + h0 + c * U;
    r[0][4] = 1.0; r[1][4] = u[0] - nm[0] * c; r[2][4] = u[1] - nm[1] * c;
    r[3][4] = u[2] - nm[2] * c; r[4][4] = T + h0 - c * U;
    S (*l)[nU] = L;
    l[0][0] = nm[0] * q - v * (nm[2] * u[1] - nm[1] * u[2]);
    l[1][0] = nm[1] * q - v * (nm[0] * u[2] - nm[2] * u[0]);
    l[2][0] = nm[2] * q - v * (nm[1] * u[0] - nm[0] * u[1]);
    l[3][0] = 0.5 * (phi2 / (c * c) - U / c);
    l[4][0] = 0.5 * (phi2 / (c * c) + U / c);
    l[0][1] = nm[0] * u[0] / T; l[1][1] = nm[1] * u[0] / T - v * nm[2];
    l[2][1] = nm[2] * u[0] / T + v * nm[1];
    l[3][1] = -0.5 * (u[0] / T - nm[0] / c); l[4][1] = -0.5 * (u[0] / T + nm[0] / c);
    l[0][2] = nm[0] * u[1] / T + v * nm[2]; l[1][2] = nm[1] * u[1] / T;
    l[2][2] = nm[2] * u[1] / T - v * nm[0];
    l[3][2] = -0.5 * (u[1] / T - nm[1] / c); l[4][2] = -0.5 * (u[1] / T + nm[1] / c);
    l[0][3] = nm[0] * u[2] / T - v * nm[1]; l[1][3] = nm[1] * u[2] / T + v * nm[0];
    l[2][3] = nm[2] * u[2] / T;
    l[3][3] = -0.5 * (u[2] / T - nm[2] / c); l[4][3] = -0.5 * (u[2] / T + nm[2] / c);
    l[0][4] = -nm[0] / T; l[1][4] = -nm[1] / T; l[2][4] = -nm[2] / T;
    l[3][4] = 0.5 / T; l[4][4] = 0.5 / T;
  }
  for (int k = 0; k < nU; ++k) {
    lam[k] = arc * lam[k];
    if (incomingDirection * valueOf(lam[k]) < 0.0) lam[k] = 0.0;
  }
  for (int j = 0; j < nU; ++j)
    for (int i = 0; i < nU; ++i) {
      S s = R[i][0] * lam[0] * L[0][j];
      for (int k = 1; k < nU; ++k) s += R[i][k] * lam[k] * L[k][j];
      out[i + nU * j] = s;
    }
}

// y += (A_i - B1_i)^T w for the inviscid flux Jacobian A along metric m
// (computeJacobianOfInviscidFlux{2D,3D}, src/CNSHelperImpl.f90:1098-1445) and
// the first partial viscous Jacobian B1 (computeFirstPartialViscousJacobian,
// :2412-2601), formed column by column and contracted immediately. P
// supplies g and the ratios 1/(g-1), (g-2)/(g-1) and 1/g computed once on
// the host: the per-point divisions by g - 1 and g become multiplications
// (an FP64 division is about ten FP64 instructions), which changes only
// rounding.
template <int ND, bool VISC, class Phys>
__device__ __forceinline__ void addFluxJacobianTransposeProduct(
    const double* m, const double* u, double T, double v, const Phys& P, double n,
    const double* tau, const double* hf, const double* w, double* y) {
  const double g = P.g;
  constexpr int nU = ND + 2, E = ND + 1;
  double U = m[0] * u[0];
  for (int d = 1; d < ND; ++d) U += m[d] * u[d];
  double u2 = u[0] * u[0];
  for (int d = 1; d < ND; ++d) u2 += u[d] * u[d];
  const double phi2 = 0.5 * (g - 1.0) * u2;
  // column 0 of A: (0, phi2 m_d - U u_d, U((g-2)/(g-1) phi2 - T))
  double ct[3] = {0.0, 0.0, 0.0}, t1 = 0.0, uct = 0.0, nTv = 0.0;
  if (VISC) {
    for (int a = 0; a < ND; ++a) {
      double s = m[0] * tau[ND * a];
      for (int d = 1; d < ND; ++d) s += m[d] * tau[ND * a + d];
      ct[a] = s;
    }
    double cq = m[0] * hf[0];
    for (int d = 1; d < ND; ++d) cq += m[d] * hf[d];
    uct = u[0] * ct[0];
    for (int d = 1; d < ND; ++d) uct += u[d] * ct[d];
    t1 = uct - cq;
    nTv = n * g * v / T;
  }
  // y_j += sum_i (A(i,j) - B(i,j)) w_i for each column j
  {
    // j = 0
    double s = 0.0;
    for (int d = 0; d < ND; ++d) s += (phi2 * m[d] - U * u[d]) * w[1 + d];
    s += U * (P.gm2OverGm1 * phi2 - T) * w[E];
    if (VISC) {
      const double t2 = nTv * (phi2 * P.invGm1 - T * P.invG);
      double sb = 0.0;
      for (int d = 0; d < ND; ++d) sb += t2 * ct[d] * w[1 + d];
      sb += (t2 * t1 - v * uct) * w[E];
      s -= sb;
    }
    y[0] += s;
  }
  for (int c = 0; c < ND; ++c) {
    double s = m[c] * w[0];
    for (int d = 0; d < ND; ++d) {
      const double a = d == c ? U - (g - 2.0) * u[c] * m[c] : u[d] * m[c] - (g - 1.0) * u[c] * m[d];
      s += a * w[1 + d];
    }
    s += ((T + phi2 * P.invGm1) * m[c] - (g - 1.0) * U * u[c]) * w[E];
    if (VISC) {
      const double t2 = -nTv * u[c];
      double sb = 0.0;
      for (int d = 0; d < ND; ++d) sb += t2 * ct[d] * w[1 + d];
      sb += (t2 * t1 + v * ct[c]) * w[E];
      s -= sb;
    }
    y[1 + c] += s;
  }
  {
    double s = 0.0;
    for (int d = 0; d < ND; ++d) s += (g - 1.0) * m[d] * w[1 + d];
    s += g * U * w[E];
    if (VISC) {
      double sb = 0.0;
      for (int d = 0; d < ND; ++d) sb += nTv * ct[d] * w[1 + d];
      sb += nTv * t1 * w[E];
      s -= sb;
    }
    y[E] += s;
  }
  (void)nU;
}

// y += B1^T w alone (first partial viscous Jacobian transpose product), used
// by the far-field adjoint viscous penalty (src/FarFieldPatchImpl.f90:237-257).
template <int ND>
__device__ __forceinline__ void firstPartialViscousTransposeProduct(
    const double* m, const double* u, double T, double v, double g, double n,
    const double* tau, const double* hf, const double* w, double* y) {
  constexpr int E = ND + 1;
  double u2 = u[0] * u[0];
  for (int d = 1; d < ND; ++d) u2 += u[d] * u[d];
  const double phi2 = 0.5 * (g - 1.0) * u2;
  double ct[3];
  for (int a = 0; a < ND; ++a) {
    double s = m[0] * tau[ND * a];
    for (int d = 1; d < ND; ++d) s += m[d] * tau[ND * a + d];
    ct[a] = s;
  }
  double cq = m[0] * hf[0];
  for (int d = 1; d < ND; ++d) cq += m[d] * hf[d];
  double uct = u[0] * ct[0];
  for (int d = 1; d < ND; ++d) uct += u[d] * ct[d];
  const double t1 = uct - cq, nTv = n * g * v / T;
  {
    const double t2 = nTv * (phi2 / (g - 1.0) - T / g);
    double s = 0.0;
    for (int d = 0; d < ND; ++d) s += t2 * ct[d] * w[1 + d];
    y[0] += s + (t2 * t1 - v * uct) * w[E];
  }
  for (int c = 0; c < ND; ++c) {
    const double t2 = -nTv * u[c];
    double s = 0.0;
    for (int d = 0; d < ND; ++d) s += t2 * ct[d] * w[1 + d];
    y[1 + c] += s + (t2 * t1 + v * ct[c]) * w[E];
  }
  {
    double s = 0.0;
    for (int d = 0; d < ND; ++d) s += nTv * ct[d] * w[1 + d];
    y[E] += s + nTv * t1 * w[E];
  }
}

// y += B2(m1, m2)^T w for the second partial viscous Jacobian
// (computeSecondPartialViscousJacobian{2D,3D}, src/CNSHelperImpl.f90:2636-2757);
// w and y have nD+1 entries (momentum, energy).
template <int ND>
__device__ __forceinline__ void secondPartialViscousTransposeProduct(
    const double* u, double mu, double la, double k, double jac, const double* m1,
    const double* m2, const double* w, double* y) {
  double t1 = m1[0] * m2[0], t2 = m2[0] * u[0], t3 = m1[0] * u[0];
  for (int d = 1; d < ND; ++d) {
    t1 += m1[d] * m2[d];
    t2 += m2[d] * u[d];
    t3 += m1[d] * u[d];
  }
  t2 = mu * t2;
  t3 = la * t3;
  // column c of B2 (c < ND): rows r < ND and energy row ND
  for (int c = 0; c < ND; ++c) {
    double s = 0.0;
    for (int r = 0; r < ND; ++r) {
      const double b = r == c ? mu * t1 + (mu + la) * m1[c] * m2[c]
                              : mu * m1[c] * m2[r] + la * m1[r] * m2[c];
      s += b * w[r];
    }
    s += (mu * t1 * u[c] + m1[c] * t2 + m2[c] * t3) * w[ND];
    y[c] += jac * s;
  }
  y[ND] += jac * (k * t1) * w[ND];
}

// Linearized (tangent) flux products, the non-transposed counterparts of the
// two products above (computeRhsLinearized, src/RhsHelperImpl.f90:655-775).
// Ax = A(m) x with the rows of computeJacobianOfInviscidFlux{2D,3D}
// (src/CNSHelperImpl.f90:1098-1445) contracted with x; with VISC also
// Bx = B1(m) x with the rows of computeFirstPartialViscousJacobian{2D,3D}
// (:2412-2601). Both are contravariant along the metric row m.
template <int ND, bool VISC>
__device__ __forceinline__ void fluxJacobianProduct(const double* m, const double* u, double T, double v, double g,
                                                    double n, const double* tau, const double* hf, const double* x,
                                                    double* Ax, double* Bx) {
  constexpr int E = ND + 1;
  double U = m[0] * u[0], u2 = u[0] * u[0], mx = m[0] * x[1], ux = u[0] * x[1];
  for (int d = 1; d < ND; ++d) {
    U += m[d] * u[d];
    u2 += u[d] * u[d];
    mx += m[d] * x[1 + d];
    ux += u[d] * x[1 + d];
  }
  const double phi2 = 0.5 * (g - 1.0) * u2;
  Ax[0] = mx;
  for (int d = 0; d < ND; ++d)
    Ax[1 + d] = (phi2 * m[d] - U * u[d]) * x[0] + U * x[1 + d] + u[d] * mx - (g - 1.0) * m[d] * ux +
                (g - 1.0) * m[d] * x[E];
  Ax[E] = U * ((g - 2.0) / (g - 1.0) * phi2 - T) * x[0] + (T + phi2 / (g - 1.0)) * mx - (g - 1.0) * U * ux +
          g * U * x[E];
  if (VISC) {
    double ct[3];
    for (int a = 0; a < ND; ++a) {
      double s = m[0] * tau[ND * a];
      for (int d = 1; d < ND; ++d) s += m[d] * tau[ND * a + d];
      ct[a] = s;
    }
    double cq = m[0] * hf[0], uct = u[0] * ct[0], ctx = ct[0] * x[1];
    for (int d = 1; d < ND; ++d) {
      cq += m[d] * hf[d];
      uct += u[d] * ct[d];
      ctx += ct[d] * x[1 + d];
    }
    const double t1 = uct - cq, nTv = n * g * v / T;
    const double sg = nTv * ((phi2 / (g - 1.0) - T / g) * x[0] - ux + x[E]);
    Bx[0] = 0.0;
    for (int d = 0; d < ND; ++d) Bx[1 + d] = ct[d] * sg;
    Bx[E] = t1 * sg + v * (ctx - uct * x[0]);
  }
}

// y += B2(m1, m2) x (computeSecondPartialViscousJacobian{2D,3D},
// src/CNSHelperImpl.f90:2636-2757, applied to x); x and y have nD+1 entries.
template <int ND>
__device__ __forceinline__ void secondPartialViscousProduct(const double* u, double mu, double la, double k,
                                                            double jac, const double* m1, const double* m2,
                                                            const double* x, double* y) {
  double t1 = m1[0] * m2[0], mx1 = m1[0] * x[0], mx2 = m2[0] * x[0], ux = u[0] * x[0];
  double m1u = m1[0] * u[0], m2u = m2[0] * u[0];
  for (int d = 1; d < ND; ++d) {
    t1 += m1[d] * m2[d];
    mx1 += m1[d] * x[d];
    mx2 += m2[d] * x[d];
    ux += u[d] * x[d];
    m1u += m1[d] * u[d];
    m2u += m2[d] * u[d];
  }
  for (int r = 0; r < ND; ++r) y[r] += jac * (mu * t1 * x[r] + mu * m2[r] * mx1 + la * m1[r] * mx2);
  y[ND] += jac * (mu * t1 * ux + mu * m2u * mx1 + la * m1u * mx2 + k * t1 * x[ND]);
}

// Cartesian-grid forms of the two products above, for a metric row with a
// single non-zero entry a at component K (row K of a diagonal metric). Terms
// that the general forms multiply by a zero metric entry are dropped, which
// leaves the remaining arithmetic unchanged; K, I and J are compile-time
// constants once the callers' loops are unrolled. nTv = n g v / T is passed
// in (it does not depend on the metric).
template <int ND, bool VISC, class Phys>
__device__ __forceinline__ void addFluxJacobianTransposeProductCart(
    int K, double a, const double* u, double T, double v, const Phys& P, double nTv,
    const double* tau, const double* hf, const double* w, double* y) {
  const double g = P.g;
  constexpr int E = ND + 1;
  const double U = a * u[K];
  double u2 = u[0] * u[0];
  for (int d = 1; d < ND; ++d) u2 += u[d] * u[d];
  const double phi2 = 0.5 * (g - 1.0) * u2;
  double ct[3] = {0.0, 0.0, 0.0}, t1 = 0.0, uct = 0.0;
  if (VISC) {
    for (int c = 0; c < ND; ++c) ct[c] = a * tau[ND * c + K];
    const double cq = a * hf[K];
    uct = u[0] * ct[0];
    for (int d = 1; d < ND; ++d) uct += u[d] * ct[d];
    t1 = uct - cq;
  }
  {
    double s = 0.0;
    for (int d = 0; d < ND; ++d) s += (d == K ? phi2 * a - U * u[d] : -(U * u[d])) * w[1 + d];
    s += U * (P.gm2OverGm1 * phi2 - T) * w[E];
    if (VISC) {
      const double t2 = nTv * (phi2 * P.invGm1 - T * P.invG);
      double sb = 0.0;
      for (int d = 0; d < ND; ++d) sb += t2 * ct[d] * w[1 + d];
      sb += (t2 * t1 - v * uct) * w[E];
      s -= sb;
    }
    y[0] += s;
  }
  for (int c = 0; c < ND; ++c) {
    double s;
    if (c == K) {
      s = a * w[0];
      for (int d = 0; d < ND; ++d) {
        const double q = d == c ? U - (g - 2.0) * u[c] * a : u[d] * a;
        s += q * w[1 + d];
      }
      s += ((T + phi2 * P.invGm1) * a - (g - 1.0) * U * u[c]) * w[E];
    } else {
      s = 0.0;
      for (int d = 0; d < ND; ++d) {
        if (d == c) s += U * w[1 + d];
        else if (d == K) s += -((g - 1.0) * u[c] * a) * w[1 + d];
      }
      s += -((g - 1.0) * U * u[c]) * w[E];
    }
    if (VISC) {
      const double t2 = -nTv * u[c];
      double sb = 0.0;
      for (int d = 0; d < ND; ++d) sb += t2 * ct[d] * w[1 + d];
      sb += (t2 * t1 + v * ct[c]) * w[E];
      s -= sb;
    }
    y[1 + c] += s;
  }
  {
    double s = (g - 1.0) * a * w[1 + K];
    s += g * U * w[E];
    if (VISC) {
      double sb = 0.0;
      for (int d = 0; d < ND; ++d) sb += nTv * ct[d] * w[1 + d];
      sb += nTv * t1 * w[E];
      s -= sb;
    }
    y[E] += s;
  }
}

// B2(a e_I, b e_J)^T w for diagonal metrics (second partial viscous Jacobian).
template <int ND>
__device__ __forceinline__ void secondPartialViscousTransposeProductCart(
    const double* u, double mu, double la, double k, double jac, int I, double a, int J, double b,
    const double* w, double* y) {
  const double t2 = mu * (b * u[J]);
  const double t3 = la * (a * u[I]);
  if (I != J) {
    // t1 = 0: only the (c = I, r = J) and (c = J, r = I) entries survive
    y[I] += jac * ((mu * a * b) * w[J] + (a * t2) * w[ND]);
    y[J] += jac * ((la * a * b) * w[I] + (b * t3) * w[ND]);
    return;
  }
  const double t1 = a * b;
  for (int c = 0; c < ND; ++c) {
    const double bcc = c == I ? mu * t1 + (mu + la) * a * b : mu * t1;
    const double e = c == I ? mu * t1 * u[c] + a * t2 + b * t3 : mu * t1 * u[c];
    y[c] += jac * (bcc * w[c] + e * w[ND]);
  }
  y[ND] += jac * (k * t1) * w[ND];
}

}  // namespace mgd
