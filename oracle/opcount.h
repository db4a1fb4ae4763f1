// opcount.h -- test infrastructure: an FP64 value type that counts the
// arithmetic performed on it, for the operation-counting build of the CPU
// oracle (oracle/build_opcount.sh). Every double of oracle.cpp becomes a
// Real there; the counts, per section of the oracle's RHS (ORC_SECTION),
// give the algorithmic FP64 work of the reference's operation list per grid
// point, which the benchmark's roofline uses instead of counts of its own
// kernels' instructions. Single-threaded (the counting build has no OpenMP).
#pragma once

#include <cmath>

namespace oc {

enum { ADD = 0, MUL, DIV, SQRT, SPECIAL, KINDS };
constexpr int kSections = 16;
inline long long counts[kSections][KINDS];
inline int section = 0;

inline void tick(int kind) { ++counts[section][kind]; }

}  // namespace oc

struct Real {
  double v;
  Real() : v(0.0) {}
  Real(double x) : v(x) {}
  explicit operator double() const { return v; }
  Real& operator+=(Real o) { oc::tick(oc::ADD); v += o.v; return *this; }
  Real& operator-=(Real o) { oc::tick(oc::ADD); v -= o.v; return *this; }
  Real& operator*=(Real o) { oc::tick(oc::MUL); v *= o.v; return *this; }
  Real& operator/=(Real o) { oc::tick(oc::DIV); v /= o.v; return *this; }
};
inline Real operator+(Real a, Real b) { oc::tick(oc::ADD); return Real(a.v + b.v); }
inline Real operator-(Real a, Real b) { oc::tick(oc::ADD); return Real(a.v - b.v); }
inline Real operator*(Real a, Real b) { oc::tick(oc::MUL); return Real(a.v * b.v); }
inline Real operator/(Real a, Real b) { oc::tick(oc::DIV); return Real(a.v / b.v); }
// exact overloads for mixed operands (no conversion, so no ambiguity with
// other user types that a Real converts to)
#define OC_MIXED(op, kind)                                                             \
  inline Real operator op(Real a, double b) { oc::tick(kind); return Real(a.v op b); } \
  inline Real operator op(double a, Real b) { oc::tick(kind); return Real(a op b.v); }
OC_MIXED(+, oc::ADD)
OC_MIXED(-, oc::ADD)
OC_MIXED(*, oc::MUL)
OC_MIXED(/, oc::DIV)
#undef OC_MIXED
#define OC_CMP(op)                                                \
  inline bool operator op(Real a, Real b) { return a.v op b.v; } \
  inline bool operator op(Real a, double b) { return a.v op b; } \
  inline bool operator op(double a, Real b) { return a op b.v; }
OC_CMP(<)
OC_CMP(>)
OC_CMP(<=)
OC_CMP(>=)
OC_CMP(==)
OC_CMP(!=)
#undef OC_CMP
inline Real operator-(Real a) { return Real(-a.v); }
inline Real operator+(Real a) { return a; }

// unqualified calls on Real (argument-dependent lookup) count too
inline Real sqrt(Real a) { oc::tick(oc::SQRT); return Real(std::sqrt(a.v)); }
inline Real fabs(Real a) { return Real(std::fabs(a.v)); }

namespace oc {
inline int abs(int a) { return a < 0 ? -a : a; }
inline double abs(double a) { return std::fabs(a); }
inline double max(double a, double b) { return a < b ? b : a; }
inline double min(double a, double b) { return b < a ? b : a; }
inline Real abs(Real a) { return Real(std::fabs(a.v)); }
inline Real fabs(Real a) { return Real(std::fabs(a.v)); }
inline Real sqrt(Real a) { tick(SQRT); return Real(std::sqrt(a.v)); }
inline Real exp(Real a) { tick(SPECIAL); return Real(std::exp(a.v)); }
inline Real cos(Real a) { tick(SPECIAL); return Real(std::cos(a.v)); }
inline Real sin(Real a) { tick(SPECIAL); return Real(std::sin(a.v)); }
inline Real atan(Real a) { tick(SPECIAL); return Real(std::atan(a.v)); }
inline Real pow(Real a, Real b) { tick(SPECIAL); return Real(std::pow(a.v, b.v)); }
inline Real copysign(Real a, Real b) { return Real(std::copysign(a.v, b.v)); }
inline Real max(Real a, Real b) { return a.v < b.v ? b : a; }
inline Real min(Real a, Real b) { return b.v < a.v ? b : a; }
inline long long max(long long a, long long b) { return a < b ? b : a; }
inline long long min(long long a, long long b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }

// Counts inside a scope go to section `s` (the innermost scope wins).
struct Section {
  int saved;
  explicit Section(int s) : saved(section) { section = s; }
  ~Section() { section = saved; }
};
}  // namespace oc

#define ORC_SECTION(s) oc::Section orc_section_guard_(s)
