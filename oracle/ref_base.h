// ORACLE — TEST INFRASTRUCTURE ONLY. Not part of the product.
//
// Scalar CPU restatement of VecGeom's FP64 query path (shape kernels, BVH navigation),
// written from the reference's algorithms (file:line cited per function) for use as the
// parity checker of the CUDA path. The reference itself cannot be compiled here: every
// header includes <VecCore/VecCore> (VecGeom/base/Global.h:19), an external library that
// is not present, and VecGeom/base/Config.h is generated by CMake. This restatement is
// therefore pinned against the known-answer vectors of the reference's own unit tests
// (tests/golden/*.json, extracted by tests/golden/extract_unit_vectors.py).
//
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may load it.
// Build: oracle/build.py (g++ -O2 -std=c++17 -ffp-contract=off: no FMA contraction, so
// every +,-,*,/ and sqrt is rounded exactly as the reference's scalar x86-64 build does).
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>

namespace oracle {

using Precision = double;

// VecGeom/base/Math.h:27-52 (double precision branch)
constexpr double kTolerance     = 1e-9;
constexpr double kPushTolerance = 1e-6;
constexpr double kConeTolerance = 1e-7;
constexpr double kAngTolerance  = 1e-9;
constexpr double kInfLength     = DBL_MAX;  // vecCore::NumericLimits<double>::Max()
constexpr double kEpsilon       = DBL_EPSILON;
constexpr double kPi            = 3.14159265358979323846;
constexpr double kTwoPi         = 2. * kPi;
constexpr double kHalfPi        = 0.5 * kPi;
constexpr double kHalfTolerance = 0.5 * kTolerance;
constexpr double kMinimum       = DBL_MIN;

// VecGeom/base/Global.h:71-79
enum EInside : int { kInside = 1, kSurface = 2, kOutside = 3 };

// Scalar stand-ins for the vecCore::math calls used by the reference kernels.
inline double Abs(double x) { return std::fabs(x); }
inline double Sqrt(double x) { return std::sqrt(x); }
inline double Min(double a, double b) { return a < b ? a : b; }
inline double Max(double a, double b) { return a > b ? a : b; }
inline double Min3(double a, double b, double c) { return Min(a, Min(b, c)); }
inline double Max3(double a, double b, double c) { return Max(a, Max(b, c)); }
inline double CopySign(double m, double s) { return std::copysign(m, s); }
inline double Sign(double x) { return std::copysign(1.0, x); }
// VecGeom/base/Global.h:166-178
inline double NonZeroAbs(double x) { return Abs(x) + 1.0e-30; }
inline double NonZero(double x) { return x + CopySign(1.0e-30, x); }

// VecGeom/volumes/kernel/GenericKernels.h:26-82
template <bool tol> inline double MakePlusTolerant(double x, double h = kHalfTolerance) { return tol ? x + h : x; }
template <bool tol> inline double MakeMinusTolerant(double x, double h = kHalfTolerance) { return tol ? x - h : x; }
template <bool tol> inline double MakePlusTolerantSquare(double x, double t = kTolerance)
{
  return tol ? x * (x + 2.0 * t) : x * x;
}
template <bool tol> inline double MakeMinusTolerantSquare(double x, double t = kTolerance)
{
  return tol ? Abs(x * (x - 2.0 * t)) : x * x;
}

// VecGeom/base/Vector3D.h: component-wise arithmetic, left-to-right reductions.
struct Vec3 {
  double v[3];
  Vec3() : v{0., 0., 0.} {}
  Vec3(double a, double b, double c) : v{a, b, c} {}
  double &operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
  double x() const { return v[0]; }
  double y() const { return v[1]; }
  double z() const { return v[2]; }
  double Perp2() const { return v[0] * v[0] + v[1] * v[1]; }
  double Perp() const { return Sqrt(Perp2()); }
  double Mag2() const { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
  double Mag() const { return Sqrt(Mag2()); }
  double Min() const { return Min3(v[0], v[1], v[2]); }
  double Max() const { return Max3(v[0], v[1], v[2]); }
  Vec3 Abs() const { return Vec3(std::fabs(v[0]), std::fabs(v[1]), std::fabs(v[2])); }
  double Dot(Vec3 const &o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
  Vec3 Unit() const
  {
    const double m2 = Mag2();
    const double s  = Sqrt(m2 + kMinimum);
    return Vec3(v[0] / s, v[1] / s, v[2] / s);
  }
};
inline Vec3 operator+(Vec3 const &a, Vec3 const &b) { return Vec3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
inline Vec3 operator-(Vec3 const &a, Vec3 const &b) { return Vec3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline Vec3 operator*(Vec3 const &a, Vec3 const &b) { return Vec3(a[0] * b[0], a[1] * b[1], a[2] * b[2]); }
inline Vec3 operator*(double s, Vec3 const &a) { return Vec3(s * a[0], s * a[1], s * a[2]); }
inline Vec3 operator*(Vec3 const &a, double s) { return Vec3(a[0] * s, a[1] * s, a[2] * s); }
inline Vec3 operator-(Vec3 const &a) { return Vec3(-a[0], -a[1], -a[2]); }

// VecGeom/base/Transformation3D.h:54-63 (data), :751-772 generic Transform, :640-651 generic
// DoRotation, :797-826 InverseTransformKernel, :878-942 MultiplyFromRight. With
// VECGEOM_NO_SPECIALIZATION every placed volume uses the generic translation/rotation codes.
struct Transformation3D {
  double t[3]  = {0., 0., 0.};
  double r[9]  = {1., 0., 0., 0., 1., 0., 0., 0., 1.};
  bool identity = true, hasRot = false, hasTrans = false;

  static Transformation3D FromArrays(const double *tr, const double *rot)
  {
    Transformation3D m;
    for (int i = 0; i < 3; ++i) m.t[i] = tr[i];
    for (int i = 0; i < 9; ++i) m.r[i] = rot[i];
    m.SetProperties();
    return m;
  }
  // source/Transformation3D.cpp:118-126 SetProperties and :174-185 GenerateRotationCode:
  // a component counts only when |value| > kTolerance; the rotation is the identity when
  // exactly the diagonal is set and equals 1.
  void SetProperties()
  {
    hasTrans = std::fabs(t[0]) > kTolerance || std::fabs(t[1]) > kTolerance || std::fabs(t[2]) > kTolerance;
    int code = 0;
    for (int i = 0; i < 9; ++i) code |= (1 << i) * (std::fabs(r[i]) > kTolerance);
    const bool isIdRot = code == 0x111 && r[0] == 1. && r[4] == 1. && r[8] == 1.;
    hasRot   = !isIdRot;
    identity = !hasTrans && !hasRot;
  }
  Vec3 Rotate(Vec3 const &m) const
  {
    Vec3 l;
    l[0] = m[0] * r[0];
    l[1] = m[0] * r[1];
    l[2] = m[0] * r[2];
    l[0] += m[1] * r[3];
    l[1] += m[1] * r[4];
    l[2] += m[1] * r[5];
    l[0] += m[2] * r[6];
    l[1] += m[2] * r[7];
    l[2] += m[2] * r[8];
    return l;
  }
  Vec3 Transform(Vec3 const &m) const { return Rotate(Vec3(m[0] - t[0], m[1] - t[1], m[2] - t[2])); }
  Vec3 TransformDirection(Vec3 const &m) const { return Rotate(m); }
  Vec3 InverseTransform(Vec3 const &l) const
  {
    Vec3 m;
    m[0] = t[0];
    m[0] += l[0] * r[0];
    m[0] += l[1] * r[1];
    m[0] += l[2] * r[2];
    m[1] = t[1];
    m[1] += l[0] * r[3];
    m[1] += l[1] * r[4];
    m[1] += l[2] * r[5];
    m[2] = t[2];
    m[2] += l[0] * r[6];
    m[2] += l[1] * r[7];
    m[2] += l[2] * r[8];
    return m;
  }
  Vec3 InverseTransformDirection(Vec3 const &l) const
  {
    Vec3 m;
    m[0] = l[0] * r[0];
    m[0] += l[1] * r[1];
    m[0] += l[2] * r[2];
    m[1] = l[0] * r[3];
    m[1] += l[1] * r[4];
    m[1] += l[2] * r[5];
    m[2] = l[0] * r[6];
    m[2] += l[1] * r[7];
    m[2] += l[2] * r[8];
    return m;
  }
  void MultiplyFromRight(Transformation3D const &rhs)
  {
    if (rhs.identity) return;
    identity = false;
    if (rhs.hasTrans) {
      hasTrans = true;
      t[0] += r[0] * rhs.t[0];
      t[0] += r[1] * rhs.t[1];
      t[0] += r[2] * rhs.t[2];
      t[1] += r[3] * rhs.t[0];
      t[1] += r[4] * rhs.t[1];
      t[1] += r[5] * rhs.t[2];
      t[2] += r[6] * rhs.t[0];
      t[2] += r[7] * rhs.t[1];
      t[2] += r[8] * rhs.t[2];
    }
    if (rhs.hasRot) {
      hasRot = true;
      for (int row = 0; row < 3; ++row) {
        const double tx = r[3 * row], ty = r[3 * row + 1], tz = r[3 * row + 2];
        r[3 * row]     = tx * rhs.r[0];
        r[3 * row + 1] = tx * rhs.r[1];
        r[3 * row + 2] = tx * rhs.r[2];
        r[3 * row] += ty * rhs.r[3];
        r[3 * row + 1] += ty * rhs.r[4];
        r[3 * row + 2] += ty * rhs.r[5];
        r[3 * row] += tz * rhs.r[6];
        r[3 * row + 1] += tz * rhs.r[7];
        r[3 * row + 2] += tz * rhs.r[8];
      }
    }
  }
};

} // namespace oracle
