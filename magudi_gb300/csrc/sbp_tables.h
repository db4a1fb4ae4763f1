// sbp_tables.h -- host construction of the SBP 4-8 operator tables that the
// kernels read from constant memory.
//
// The operator is the diagonal-norm summation-by-parts first derivative with
// an 8th-order interior and 4th-order boundary closure (free parameters
// x1 = 541/1000, x2 = -27/400, x3 = 187/250), as magudi defines it in
// src/StencilOperatorImpl.f90:1586-1743; its artificial dissipation
// (:1928-1960); and the adjoint H^-1 D^T H of getAdjointOperator (:2285-2372).
// Tables are stored row-major: row m (0-based output point from the
// boundary), column k (0-based input point from the boundary).
#pragma once

#include <vector>

namespace mgd {

struct HostOp {
  int depth = 0, width = 0, half = 0;
  bool skew = false;
  bool asym = false;             // interior stencil not (skew-)symmetric: general sum, explicit right block
  std::vector<double> interior;  // coefficients of offsets -half..half
  std::vector<double> left;      // depth x width, row-major
  std::vector<double> right;     // asym only: depth x width, row m = point n-1-m, column k = point n-width+k
  std::vector<double> norm;      // boundary norm weights (first derivative only)
  double& L(int m, int k) { return left[(size_t)m * width + k]; }
  double L(int m, int k) const { return left[(size_t)m * width + k]; }
  double& R(int m, int k) { return right[(size_t)m * width + k]; }
  double R(int m, int k) const { return right[(size_t)m * width + k]; }
  double& I(int j) { return interior[j + half]; }
  double I(int j) const { return interior[j + half]; }
  void allocate(int d, int w, int h) {
    depth = d; width = w; half = h;
    interior.assign(2 * h + 1, 0.0);
    left.assign((size_t)d * w, 0.0);
  }
};

inline HostOp makeFirstDerivative48() {
  HostOp d;
  d.depth = 8; d.width = 12; d.half = 4; d.skew = true;
  d.interior.assign(9, 0.0);
  d.left.assign(8 * 12, 0.0);
  const double c[4] = {4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0};
  for (int j = 1; j <= 4; ++j) { d.I(j) = c[j - 1]; d.I(-j) = -c[j - 1]; }
  d.norm = {1498139.0 / 5080320.0, 1107307.0 / 725760.0, 20761.0 / 80640.0,
            1304999.0 / 725760.0,  299527.0 / 725760.0,  103097.0 / 80640.0,
            670091.0 / 725760.0,   5127739.0 / 5080320.0};
  const double a = 541.0 / 1000.0, b = -27.0 / 400.0, e = 187.0 / 250.0;
  // Row 0.
  d.L(0, 0) = -2540160.0 / 1498139.0;
  d.L(0, 1) = 9.0 * (2257920.0 * a + 11289600.0 * b + 22579200.0 * e - 15849163.0) / 5992556.0;
  d.L(0, 2) = 3.0 * (-33868800.0 * a - 162570240.0 * b - 304819200.0 * e + 235236677.0) / 5992556.0;
  d.L(0, 3) = (609638400.0 * a + 2743372800.0 * b + 4572288000.0 * e - 3577778591.0) / 17977668.0;
  d.L(0, 4) = 3.0 * (-16934400.0 * a - 67737600.0 * b - 84672000.0 * e + 67906303.0) / 1498139.0;
  d.L(0, 5) = 105.0 * (967680.0 * a + 2903040.0 * b - 305821.0) / 5992556.0;
  d.L(0, 6) = 49.0 * (-1244160.0 * a + 18662400.0 * e - 13322233.0) / 17977668.0;
  d.L(0, 7) = 3.0 * (-6773760.0 * b - 33868800.0 * e + 24839327.0) / 5992556.0;
  // Row 1.
  d.L(1, 0) = 9.0 * (-2257920.0 * a - 11289600.0 * b - 22579200.0 * e + 15849163.0) / 31004596.0;
  d.L(1, 2) = 3.0 * (7257600.0 * a + 33868800.0 * b + 60963840.0 * e - 47167457.0) / 2214614.0;
  d.L(1, 3) = 3.0 * (-9676800.0 * a - 42336000.0 * b - 67737600.0 * e + 53224573.0) / 1107307.0;
  d.L(1, 4) = 7.0 * (55987200.0 * a + 217728000.0 * b + 261273600.0 * e - 211102099.0) / 13287684.0;
  d.L(1, 5) = 3.0 * (-11612160.0 * a - 33868800.0 * b + 3884117.0) / 2214614.0;
  d.L(1, 6) = 150.0 * (24192.0 * a - 338688.0 * e + 240463.0) / 1107307.0;
  d.L(1, 7) = (152409600.0 * b + 731566080.0 * e - 536324953.0) / 46506894.0;
  // Row 2.
  d.L(2, 0) = (33868800.0 * a + 162570240.0 * b + 304819200.0 * e - 235236677.0) / 1743924.0;
  d.L(2, 1) = (-7257600.0 * a - 33868800.0 * b - 60963840.0 * e + 47167457.0) / 124566.0;
  d.L(2, 3) = (24192000.0 * a + 101606400.0 * b + 152409600.0 * e - 120219461.0) / 124566.0;
  d.L(2, 4) = (-72576000.0 * a - 270950400.0 * b - 304819200.0 * e + 249289259.0) / 249132.0;
  d.L(2, 5) = 9.0 * (806400.0 * a + 2257920.0 * b - 290167.0) / 41522.0;
  d.L(2, 6) = 6.0 * (-134400.0 * a + 1693440.0 * e - 1191611.0) / 20761.0;
  d.L(2, 7) = 5.0 * (-2257920.0 * b - 10160640.0 * e + 7439833.0) / 290654.0;
  // Row 3.
  d.L(3, 0) = (-609638400.0 * a - 2743372800.0 * b - 4572288000.0 * e + 3577778591.0) / 109619916.0;
  d.L(3, 1) = 3.0 * (9676800.0 * a + 42336000.0 * b + 67737600.0 * e - 53224573.0) / 1304999.0;
  d.L(3, 2) = 3.0 * (-24192000.0 * a - 101606400.0 * b - 152409600.0 * e + 120219461.0) / 2609998.0;
  d.L(3, 4) = 9.0 * (16128000.0 * a + 56448000.0 * b + 56448000.0 * e - 47206049.0) / 5219996.0;
  d.L(3, 5) = 3.0 * (-19353600.0 * a - 50803200.0 * b + 7628371.0) / 2609998.0;
  d.L(3, 6) = 2.0 * (10886400.0 * a - 114307200.0 * e + 79048289.0) / 3914997.0;
  d.L(3, 7) = 75.0 * (1354752.0 * b + 5419008.0 * e - 3952831.0) / 18269986.0;
  // Row 4.
  d.L(4, 0) = 3.0 * (16934400.0 * a + 67737600.0 * b + 84672000.0 * e - 67906303.0) / 2096689.0;
  d.L(4, 1) = 7.0 * (-55987200.0 * a - 217728000.0 * b - 261273600.0 * e + 211102099.0) / 3594324.0;
  d.L(4, 2) = 3.0 * (72576000.0 * a + 270950400.0 * b + 304819200.0 * e - 249289259.0) / 1198108.0;
  d.L(4, 3) = 9.0 * (-16128000.0 * a - 56448000.0 * b - 56448000.0 * e + 47206049.0) / 1198108.0;
  d.L(4, 5) = 105.0 * (414720.0 * a + 967680.0 * b - 165527.0) / 1198108.0;
  d.L(4, 6) = 15.0 * (-967680.0 * a + 6773760.0 * e - 4472029.0) / 1198108.0;
  d.L(4, 7) = (-304819200.0 * b - 914457600.0 * e + 657798011.0) / 25160268.0;
  d.L(4, 8) = -2592.0 / 299527.0;
  // Row 5.
  d.L(5, 0) = 5.0 * (-967680.0 * a - 2903040.0 * b + 305821.0) / 1237164.0;
  d.L(5, 1) = (11612160.0 * a + 33868800.0 * b - 3884117.0) / 618582.0;
  d.L(5, 2) = 9.0 * (-806400.0 * a - 2257920.0 * b + 290167.0) / 206194.0;
  d.L(5, 3) = (19353600.0 * a + 50803200.0 * b - 7628371.0) / 618582.0;
  d.L(5, 4) = 35.0 * (-414720.0 * a - 967680.0 * b + 165527.0) / 1237164.0;
  d.L(5, 6) = 80640.0 * a / 103097.0;
  d.L(5, 7) = 80640.0 * b / 103097.0;
  d.L(5, 8) = 3072.0 / 103097.0;
  d.L(5, 9) = -288.0 / 103097.0;
  // Row 6.
  d.L(6, 0) = 7.0 * (1244160.0 * a - 18662400.0 * e + 13322233.0) / 8041092.0;
  d.L(6, 1) = 150.0 * (-24192.0 * a + 338688.0 * e - 240463.0) / 670091.0;
  d.L(6, 2) = 54.0 * (134400.0 * a - 1693440.0 * e + 1191611.0) / 670091.0;
  d.L(6, 3) = 2.0 * (-10886400.0 * a + 114307200.0 * e - 79048289.0) / 2010273.0;
  d.L(6, 4) = 15.0 * (967680.0 * a - 6773760.0 * e + 4472029.0) / 2680364.0;
  d.L(6, 5) = -725760.0 * a / 670091.0;
  d.L(6, 7) = 725760.0 * e / 670091.0;
  d.L(6, 8) = -145152.0 / 670091.0;
  d.L(6, 9) = 27648.0 / 670091.0;
  d.L(6, 10) = -2592.0 / 670091.0;
  // Row 7.
  d.L(7, 0) = 3.0 * (6773760.0 * b + 33868800.0 * e - 24839327.0) / 20510956.0;
  d.L(7, 1) = (-152409600.0 * b - 731566080.0 * e + 536324953.0) / 30766434.0;
  d.L(7, 2) = 45.0 * (2257920.0 * b + 10160640.0 * e - 7439833.0) / 10255478.0;
  d.L(7, 3) = 75.0 * (-1354752.0 * b - 5419008.0 * e + 3952831.0) / 10255478.0;
  d.L(7, 4) = (304819200.0 * b + 914457600.0 * e - 657798011.0) / 61532868.0;
  d.L(7, 5) = -5080320.0 * b / 5127739.0;
  d.L(7, 6) = -5080320.0 * e / 5127739.0;
  d.L(7, 8) = 4064256.0 / 5127739.0;
  d.L(7, 9) = -1016064.0 / 5127739.0;
  d.L(7, 10) = 193536.0 / 5127739.0;
  d.L(7, 11) = -18144.0 / 5127739.0;
  return d;
}

// Dense n x n matrix of an operator on a non-periodic line of n points:
// the left block, the right block by (skew-)reflection, the interior stencil.
inline std::vector<double> denseMatrix(const HostOp& op, int n) {
  std::vector<double> M((size_t)n * n, 0.0);
  for (int r = 0; r < n; ++r) {
    if (r < op.depth) {
      for (int k = 0; k < op.width; ++k) M[(size_t)r * n + k] = op.L(r, k);
    } else if (r >= n - op.depth) {
      const int m = n - 1 - r;
      if (op.asym) {
        for (int k = 0; k < op.width; ++k) M[(size_t)r * n + (n - op.width + k)] = op.R(m, k);
      } else {
        const double sgn = op.skew ? -1.0 : 1.0;
        for (int k = 0; k < op.width; ++k) M[(size_t)r * n + (n - 1 - k)] = sgn * op.L(m, k);
      }
    } else {
      for (int j = -op.half; j <= op.half; ++j) M[(size_t)r * n + r + j] = op.I(j);
    }
  }
  return M;
}

// Adjoint with respect to the H inner product: A = H^-1 D^T H. Its boundary
// block has (D.width) rows and (D.width + D.half) columns because the
// transposes of the first interior rows of D reach into it.
inline HostOp makeAdjoint(const HostOp& d) {
  HostOp a;
  a.depth = d.width;
  a.width = d.width + d.half;
  a.half = d.half;
  a.skew = d.skew;
  a.interior.assign(2 * d.half + 1, 0.0);
  for (int j = -d.half; j <= d.half; ++j) a.I(j) = d.I(-j);
  const int n = 4 * a.width;
  const std::vector<double> D = denseMatrix(d, n);
  a.left.assign((size_t)a.depth * a.width, 0.0);
  const int nn = (int)d.norm.size();
  for (int m = 0; m < a.depth; ++m)
    for (int k = 0; k < a.width; ++k) {
      double v = D[(size_t)k * n + m];  // (D^T)(m,k)
      if (m < nn) v = v / d.norm[m];
      if (k < nn) v = v * d.norm[k];
      a.L(m, k) = v;
    }
  a.norm = d.norm;
  return a;
}

// Dissipation D_d: 5-point (1, -4, 6, -4, 1); its two boundary rows repeat the
// interior stencil anchored at the boundary.
inline HostOp makeDissipation48() {
  HostOp d;
  d.depth = 2; d.width = 5; d.half = 2; d.skew = false;
  d.interior = {1.0, -4.0, 6.0, -4.0, 1.0};
  d.left.assign(2 * 5, 0.0);
  for (int m = 0; m < 2; ++m)
    for (int k = 0; k < 5; ++k) d.L(m, k) = d.interior[k];
  return d;
}

// H^-1 D_d^T: the transpose of D_d followed by the inverse of the
// first-derivative norm on the first 8 rows; the combined boundary block is
// 8 rows by 10 columns.
inline HostOp makeDissipationTransposeNormInverse48(const HostOp& d1) {
  const HostOp dd = makeDissipation48();
  HostOp t;
  t.depth = 8; t.width = 10; t.half = 2; t.skew = false;
  t.interior = dd.interior;
  const int n = 40;
  const std::vector<double> D = denseMatrix(dd, n);
  t.left.assign(8 * 10, 0.0);
  for (int m = 0; m < 8; ++m)
    for (int k = 0; k < 10; ++k) t.L(m, k) = D[(size_t)k * n + m] / d1.norm[m];
  return t;
}

// Composite dissipation: one symmetric 8th-difference operator with
// boundary closure (interior (-1, 8, -28, 56, -70, 56, -28, 8, -1)/256),
// H-self-adjoint, applied as rhs += amount * D q with no arc-length scaling
// (magudi's default composite_dissipation = true path).
inline HostOp makeCompositeDissipation48() {
  HostOp d;
  d.depth = 8; d.width = 12; d.half = 4; d.skew = false;
  d.interior = {-1.0, 8.0, -28.0, 56.0, -70.0, 56.0, -28.0, 8.0, -1.0};
  for (double& v : d.interior) v = v / 256.0;
  d.left.assign(8 * 12, 0.0);
  struct Row { int first, count; double num[9]; double den; };
  const Row rows[8] = {
      {0, 5, {-15240960.0, 60963840.0, -91445760.0, 60963840.0, -15240960.0}, 1498139.0},
      {0, 6, {8709120.0, -35562240.0, 55157760.0, -39191040.0, 11612160.0, -725760.0}, 1107307.0},
      {0, 7, {-1451520.0, 6128640.0, -10080000.0, 8064000.0, -3225600.0, 645120.0, -80640.0}, 20761.0},
      {0, 8, {8709120.0, -39191040.0, 72576000.0, -73301760.0, 46448640.0, -20321280.0, 5806080.0, -725760.0},
       1304999.0},
      {0, 9, {-2177280.0, 11612160.0, -29030400.0, 46448640.0, -52254720.0, 40642560.0, -20321280.0, 5806080.0,
              -725760.0}, 299527.0},
      {1, 9, {-80640.0, 645120.0, -2257920.0, 4515840.0, -5644800.0, 4515840.0, -2257920.0, 645120.0, -80640.0},
       103097.0},
      {2, 9, {-725760.0, 5806080.0, -20321280.0, 40642560.0, -50803200.0, 40642560.0, -20321280.0, 5806080.0,
              -725760.0}, 670091.0},
      {3, 9, {-5080320.0, 40642560.0, -142248960.0, 284497920.0, -355622400.0, 284497920.0, -142248960.0,
              40642560.0, -5080320.0}, 5127739.0}};
  for (int m = 0; m < 8; ++m)
    for (int t = 0; t < rows[m].count; ++t) d.L(m, rows[m].first + t) = rows[m].num[t] / rows[m].den / 256.0;
  return d;
}

// ---------------------------------------------------------------------------
// The lower-order schemes of defaults/discretization_scheme ("SBP 1-2",
// "SBP 2-4", "SBP 3-6"; setupOperator, src/StencilOperatorImpl.f90:1164-1585):
// first derivative, composite dissipation, and the non-composite dissipation
// and its transpose. Boundary rows are written as (row, first column,
// values), 0-based, like the reference's rhsBoundary1(k0:, m) assignments.
// ---------------------------------------------------------------------------
struct OpRow { int m, k0, n; double v[9]; };
inline void setRows(HostOp& op, const OpRow* rows, int count, double scale = 1.0) {
  for (int r = 0; r < count; ++r)
    for (int t = 0; t < rows[r].n; ++t) op.L(rows[r].m, rows[r].k0 + t) = rows[r].v[t] * scale;
}

inline HostOp makeFirstDerivative12() {  // :1164-1177
  HostOp d;
  d.allocate(1, 2, 1);
  d.skew = true;
  d.I(1) = 1.0 / 2.0; d.I(-1) = -d.I(1);
  d.norm = {1.0 / 2.0};
  d.L(0, 0) = -1.0; d.L(0, 1) = 1.0;
  return d;
}
inline HostOp makeCompositeDissipation12() {  // :1194-1210
  HostOp d;
  d.allocate(1, 2, 1);
  d.I(0) = -2.0 / 2.0; d.I(1) = 1.0 / 2.0; d.I(-1) = d.I(1);
  d.L(0, 0) = -2.0 / 2.0; d.L(0, 1) = 2.0 / 2.0;
  return d;
}

inline HostOp makeFirstDerivative24() {  // :1212-1245
  HostOp d;
  d.allocate(4, 6, 2);
  d.skew = true;
  d.I(1) = 2.0 / 3.0; d.I(2) = -1.0 / 12.0;
  for (int j = 1; j <= 2; ++j) d.I(-j) = -d.I(j);
  d.norm = {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0};
  const OpRow rows[4] = {{0, 0, 4, {-24.0 / 17.0, 59.0 / 34.0, -4.0 / 17.0, -3.0 / 34.0}},
                         {1, 0, 3, {-1.0 / 2.0, 0.0, 1.0 / 2.0}},
                         {2, 0, 5, {4.0 / 43.0, -59.0 / 86.0, 0.0, 59.0 / 86.0, -4.0 / 43.0}},
                         {3, 0, 6, {3.0 / 98.0, 0.0, -59.0 / 98.0, 0.0, 32.0 / 49.0, -4.0 / 49.0}}};
  setRows(d, rows, 4);
  return d;
}
inline HostOp makeCompositeDissipation24() {  // :1282-1317
  HostOp d;
  d.allocate(4, 6, 2);
  const double c[3] = {-6.0, 4.0, -1.0};
  for (int j = 0; j <= 2; ++j) d.I(j) = d.I(-j) = c[j] / 16.0;
  const OpRow rows[4] = {{0, 0, 3, {-96.0 / 17.0, 192.0 / 17.0, -96.0 / 17.0}},
                         {1, 0, 4, {192.0 / 59.0, -432.0 / 59.0, 288.0 / 59.0, -48.0 / 59.0}},
                         {2, 0, 5, {-96.0 / 43.0, 288.0 / 43.0, -336.0 / 43.0, 192.0 / 43.0, -48.0 / 43.0}},
                         {3, 1, 5, {-48.0 / 49.0, 192.0 / 49.0, -288.0 / 49.0, 192.0 / 49.0, -48.0 / 49.0}}};
  setRows(d, rows, 4, 1.0 / 16.0);
  return d;
}
inline HostOp makeDissipation24() {  // :1319-1329
  HostOp d;
  d.allocate(1, 3, 1);
  d.I(-1) = 1.0; d.I(0) = -2.0; d.I(1) = 1.0;
  for (int k = 0; k < 3; ++k) d.L(0, k) = d.I(k - 1);
  return d;
}
inline HostOp makeDissipationTranspose24() {  // :1331-1345
  HostOp d;
  d.allocate(3, 4, 1);
  d.I(-1) = 1.0; d.I(0) = -2.0; d.I(1) = 1.0;
  for (int m = 0; m < 3; ++m) d.L(m, 0) = d.L(m, 1) = d.I(m - 1);
  for (int m = 1; m < 3; ++m) d.L(m, 2) = d.I(m - 2);
  d.L(2, 3) = d.I(-1);
  return d;
}

inline HostOp makeFirstDerivative36() {  // :1362-1421
  HostOp d;
  d.allocate(6, 9, 3);
  d.skew = true;
  d.I(1) = 3.0 / 4.0; d.I(2) = -3.0 / 20.0; d.I(3) = 1.0 / 60.0;
  for (int j = 1; j <= 3; ++j) d.I(-j) = -d.I(j);
  d.norm = {13649.0 / 43200.0, 12013.0 / 8640.0, 2711.0 / 4320.0, 5359.0 / 4320.0, 7877.0 / 8640.0,
            43801.0 / 43200.0};
  const OpRow rows[6] = {
      {0, 0, 6, {-21600.0 / 13649.0, 104009.0 / 54596.0, 30443.0 / 81894.0, -33311.0 / 27298.0, 16863.0 / 27298.0,
                 -15025.0 / 163788.0}},
      {1, 0, 6, {-104009.0 / 240260.0, 0.0, -311.0 / 72078.0, 20229.0 / 24026.0, -24337.0 / 48052.0,
                 36661.0 / 360390.0}},
      {2, 0, 6, {-30443.0 / 162660.0, 311.0 / 32532.0, 0.0, -11155.0 / 16266.0, 41287.0 / 32532.0,
                 -21999.0 / 54220.0}},
      {3, 0, 7, {33311.0 / 107180.0, -20229.0 / 21436.0, 485.0 / 1398.0, 0.0, 4147.0 / 21436.0,
                 25427.0 / 321540.0, 72.0 / 5359.0}},
      {4, 0, 8, {-16863.0 / 78770.0, 24337.0 / 31508.0, -41287.0 / 47262.0, -4147.0 / 15754.0, 0.0,
                 342523.0 / 472620.0, -1296.0 / 7877.0, 144.0 / 7877.0}},
      {5, 0, 9, {15025.0 / 525612.0, -36661.0 / 262806.0, 21999.0 / 87602.0, -25427.0 / 262806.0,
                 -342523.0 / 525612.0, 0.0, 32400.0 / 43801.0, -6480.0 / 43801.0, 720.0 / 43801.0}}};
  setRows(d, rows, 6);
  return d;
}
inline HostOp makeCompositeDissipation36() {  // :1487-1543
  HostOp d;
  d.allocate(6, 9, 3);
  const double c[4] = {-20.0, 15.0, -6.0, 1.0};
  for (int j = 0; j <= 3; ++j) d.I(j) = d.I(-j) = c[j] / 64.0;
  const OpRow rows[6] = {
      {0, 0, 4, {-129600.0 / 13649.0, 388800.0 / 13649.0, -388800.0 / 13649.0, 129600.0 / 13649.0}},
      {1, 0, 5, {77760.0 / 12013.0, -241920.0 / 12013.0, 259200.0 / 12013.0, -103680.0 / 12013.0,
                 8640.0 / 12013.0}},
      {2, 0, 6, {-38880.0 / 2711.0, 129600.0 / 2711.0, -159840.0 / 2711.0, 90720.0 / 2711.0, -25920.0 / 2711.0,
                 4320.0 / 2711.0}},
      {3, 0, 7, {12960.0 / 5359.0, -51840.0 / 5359.0, 90720.0 / 5359.0, -95040.0 / 5359.0, 64800.0 / 5359.0,
                 -25920.0 / 5359.0, 4320.0 / 5359.0}},
      {4, 1, 7, {8640.0 / 7877.0, -51840.0 / 7877.0, 129600.0 / 7877.0, -172800.0 / 7877.0, 129600.0 / 7877.0,
                 -51840.0 / 7877.0, 8640.0 / 7877.0}},
      {5, 2, 7, {43200.0 / 43801.0, -259200.0 / 43801.0, 648000.0 / 43801.0, -864000.0 / 43801.0,
                 648000.0 / 43801.0, -259200.0 / 43801.0, 43200.0 / 43801.0}}};
  setRows(d, rows, 6, 1.0 / 64.0);
  return d;
}
// "SBP 3-6 dissipation" (:1545-1561): interior offsets -2..1, both closure
// rows repeat it, the right block is the negated reflection.
inline HostOp makeDissipation36() {
  HostOp d;
  d.allocate(2, 4, 2);
  d.asym = true;
  const double c[4] = {-1.0, 3.0, -3.0, 1.0};
  for (int j = -2; j <= 1; ++j) d.I(j) = c[j + 2];
  d.right.assign(2 * 4, 0.0);
  for (int m = 0; m < 2; ++m)
    for (int k = 0; k < 4; ++k) d.L(m, k) = c[k];
  for (int m = 0; m < 2; ++m)
    for (int k = 0; k < 4; ++k) d.R(m, k) = -d.L(m, 3 - k);
  return d;
}
// "SBP 3-6 dissipation transpose" (:1563-1585): interior offsets -1..2 and
// the reference's explicit left and right blocks.
inline HostOp makeDissipationTranspose36() {
  HostOp d;
  d.allocate(4, 6, 2);
  d.asym = true;
  const double c[4] = {1.0, -3.0, 3.0, -1.0};  // offsets -1..2
  for (int j = -1; j <= 2; ++j) d.I(j) = c[j + 1];
  auto in = [&](int j) { return c[j + 1]; };
  // rhsBoundary1(k, m): L(m - 1, k - 1)
  for (int k = 1; k <= 3; ++k)
    for (int m = 1; m <= 4; ++m) d.L(m - 1, k - 1) = in(3 - m);
  for (int m = 2; m <= 4; ++m) d.L(m - 1, 3) = in(4 - m);
  for (int m = 3; m <= 4; ++m) d.L(m - 1, 4) = in(5 - m);
  d.L(3, 5) = in(2);
  // rhsBoundary2(k, m): R(m - 1, k - 1)
  d.right.assign(4 * 6, 0.0);
  for (int m = 1; m <= 4; ++m) d.R(m - 1, 5) = d.R(m - 1, 4) = in(3 - m);
  for (int m = 2; m <= 4; ++m) d.R(m - 1, 3) = in(m - 3);
  for (int m = 3; m <= 4; ++m) d.R(m - 1, 2) = in(m - 4);
  d.R(3, 1) = in(-1);
  return d;
}

// The scheme's operators in their own shapes.
struct SchemeOps {
  HostOp d1, dcomp, diss, dissT;
  bool hasDissipation = true;  // SBP 1-2 has no non-composite dissipation
};
inline SchemeOps schemeOps(int scheme) {
  SchemeOps s;
  switch (scheme) {
    case 1:
      s.d1 = makeFirstDerivative12(); s.dcomp = makeCompositeDissipation12(); s.hasDissipation = false;
      break;
    case 2:
      s.d1 = makeFirstDerivative24(); s.dcomp = makeCompositeDissipation24();
      s.diss = makeDissipation24(); s.dissT = makeDissipationTranspose24();
      break;
    case 3:
      s.d1 = makeFirstDerivative36(); s.dcomp = makeCompositeDissipation36();
      s.diss = makeDissipation36(); s.dissT = makeDissipationTranspose36();
      break;
    default: {
      s.d1 = makeFirstDerivative48(); s.dcomp = makeCompositeDissipation48();
      s.diss = makeDissipation48();
      // "SBP 4-8 dissipation transpose" (:1942-1960) equals the transpose of "SBP 4-8 dissipation"
      HostOp t;
      t.allocate(5, 7, 2);
      for (int j = -2; j <= 2; ++j) t.I(j) = s.diss.I(j);
      const std::vector<double> D = denseMatrix(s.diss, 40);
      for (int m = 0; m < 5; ++m)
        for (int k = 0; k < 7; ++k) t.L(m, k) = D[(size_t)k * 40 + m];
      s.dissT = t;
    }
  }
  return s;
}

// An operator in the fixed shape (D rows, W columns, half-width Hf) of the
// kernels' tables: the closure rows as given, the rows from the operator's
// depth to D as its interior stencil, the interior zero-padded to Hf; an
// explicit right block likewise. The value of every output point is
// unchanged (rows between the operator's depth and D sum the same products
// in closure order).
inline HostOp embed(const HostOp& op, int D, int W, int Hf) {
  HostOp e;
  e.allocate(D, W, Hf);
  e.skew = op.skew;
  e.asym = op.asym;
  e.norm = op.norm;
  for (int j = -op.half; j <= op.half; ++j) e.I(j) = op.I(j);
  for (int m = 0; m < D; ++m) {
    if (m < op.depth) {
      for (int k = 0; k < op.width; ++k) e.L(m, k) = op.L(m, k);
    } else {
      for (int j = -op.half; j <= op.half; ++j)
        if (op.I(j) != 0.0) e.L(m, m + j) = op.I(j);
    }
  }
  if (op.asym) {
    e.right.assign((size_t)D * W, 0.0);
    for (int m = 0; m < D; ++m) {
      if (m < op.depth) {
        for (int k = 0; k < op.width; ++k) e.R(m, W - op.width + k) = op.R(m, k);
      } else {
        // point n-1-m: coefficient I(j) on point n-1-m+j = column W-1-m+j
        for (int j = -op.half; j <= op.half; ++j)
          if (op.I(j) != 0.0) e.R(m, W - 1 - m + j) = op.I(j);
      }
    }
  }
  return e;
}

// Folds the inverse of the first-derivative norm into the boundary rows of
// an operator in kernel shape (applyNormInverse after the operator).
inline void foldNormInverse(HostOp& t, const std::vector<double>& norm) {
  for (size_t m = 0; m < norm.size() && (int)m < t.depth; ++m)
    for (int k = 0; k < t.width; ++k) {
      t.L((int)m, k) = t.L((int)m, k) / norm[m];
      if (t.asym) t.R((int)m, k) = t.R((int)m, k) / norm[m];
    }
}

}  // namespace mgd
