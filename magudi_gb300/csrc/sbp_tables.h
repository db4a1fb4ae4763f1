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
  std::vector<double> interior;  // coefficients of offsets -half..half
  std::vector<double> left;      // depth x width, row-major
  std::vector<double> norm;      // boundary norm weights (first derivative only)
  double& L(int m, int k) { return left[(size_t)m * width + k]; }
  double L(int m, int k) const { return left[(size_t)m * width + k]; }
  double& I(int j) { return interior[j + half]; }
  double I(int j) const { return interior[j + half]; }
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
      const double sgn = op.skew ? -1.0 : 1.0;
      for (int k = 0; k < op.width; ++k) M[(size_t)r * n + (n - 1 - k)] = sgn * op.L(m, k);
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

}  // namespace mgd
