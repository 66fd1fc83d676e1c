// Exact FP64 comparisons, minima/maxima and sign products on the integer pipe.
//
// GB300 executes FP64 arithmetic at 2 results per clock per SM, and its FP64 compares
// (a < b), minima/maxima and multiplications by +-1 issue on that same narrow pipe, one
// pipe slot each like an add. The helpers below return the same values as the IEEE
// operations they replace, for every input including signed zeros, infinities and NaNs:
//
//   dlt/dle/dgt/dge/deq(a, b)  a < b, a <= b, a > b, a >= b, a == b (false if a or b is NaN)
//   dmin(a, b), dmax(a, b)     a < b ? a : b and a > b ? a : b (the operand selected as is)
//   dabs_lt/dabs_le(x, c)      fabs(x) < c, fabs(x) <= c
//   flipsign(v, s)             v * copysign(1.0, s): an IEEE product with +-1 is exact and
//                              only sets the sign, so it is v with its sign bit flipped when
//                              the sign bit of s is set (always an integer xor)
//
// Two compile-time switches, set per translation unit before this header is included:
//
// VG_FP64_INT_COMPARE (default 1): compares and min/max run on the integer pipe. Non-NaN
//   doubles are ordered like the signed integers okey(bits) = sign ? -(bits & mag) : bits, in
//   which +0 and -0 both map to 0, and NaN operands are excluded explicitly; the bit patterns
//   are read through an opaque move so that the compiler cannot turn the integer tests back
//   into floating-point compares. That is ~10-20 integer instructions in place of one FP64
//   slot: it pays in throughput-bound kernels (the SoA shape queries, 1.2-2.5x) and costs
//   latency in divergent, latency-bound ones. With 0 the names are macros for the plain IEEE
//   operators (as macros, not functions: the navigation kernels measured ~15% slower with
//   the same operators behind inline functions).
// VG_FP64_SHORTCUTS (default 1): exact shortcuts that skip FP64 work (sign products as
//   xors, nonzero() without its addition for |x| >= 2^-46, rotations about z without their
//   zero terms). They add integer work and branches, which the divergent plain-FP64
//   navigator (5% slower with them) does not recover; the other kernels do.
//
// Every function here is static (internal linkage) because the variants coexist in one
// library, one per translation unit.
#pragma once

namespace vg {
namespace f64 {

constexpr long long kMagMask = 0x7FFFFFFFFFFFFFFFLL;
constexpr long long kInfBits = 0x7FF0000000000000LL;

#ifndef VG_FP64_INT_COMPARE
#define VG_FP64_INT_COMPARE 1
#endif
#ifndef VG_FP64_SHORTCUTS
#define VG_FP64_SHORTCUTS 1
#endif

static __device__ __forceinline__ long long dbits(double x)
{
  long long r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
}
#if VG_FP64_SHORTCUTS
static __device__ __forceinline__ double flipsign(double v, double s)
{
  return __longlong_as_double(dbits(v) ^ (dbits(s) & ~kMagMask));
}
// (-copysign(1.0, s)) * v: v with its sign bit flipped when the sign bit of s is clear
static __device__ __forceinline__ double negflipsign(double v, double s)
{
  return __longlong_as_double(dbits(v) ^ (~dbits(s) & ~kMagMask));
}
#else
static __device__ __forceinline__ double flipsign(double v, double s) { return copysign(1.0, s) * v; }
static __device__ __forceinline__ double negflipsign(double v, double s) { return -copysign(1.0, s) * v; }
#endif

#if VG_FP64_INT_COMPARE
static __device__ __forceinline__ long long okey(long long b)
{
  const long long m = b >> 63;
  return ((b & kMagMask) ^ m) - m;
}
static __device__ __forceinline__ bool nnan(long long b) { return (b & kMagMask) <= kInfBits; }

static __device__ __forceinline__ bool dlt(double a, double b)
{
  const long long x = dbits(a), y = dbits(b);
  return (okey(x) < okey(y)) & nnan(x) & nnan(y);
}
static __device__ __forceinline__ bool dle(double a, double b)
{
  const long long x = dbits(a), y = dbits(b);
  return (okey(x) <= okey(y)) & nnan(x) & nnan(y);
}
static __device__ __forceinline__ bool deq(double a, double b)
{
  const long long x = dbits(a), y = dbits(b);
  return (okey(x) == okey(y)) & nnan(x) & nnan(y);
}
static __device__ __forceinline__ bool dabs_lt(double x, double c)
{
  const long long y = dbits(c);
  return ((dbits(x) & kMagMask) < okey(y)) & nnan(y);
}
static __device__ __forceinline__ bool dabs_le(double x, double c)
{
  const long long y = dbits(c);
  return ((dbits(x) & kMagMask) <= okey(y)) & nnan(y);
}
static __device__ __forceinline__ bool dgt(double a, double b) { return dlt(b, a); }
static __device__ __forceinline__ bool dge(double a, double b) { return dle(b, a); }
static __device__ __forceinline__ bool dne(double a, double b) { return !deq(a, b); }
static __device__ __forceinline__ double dmin(double a, double b) { return dlt(a, b) ? a : b; }
static __device__ __forceinline__ double dmax(double a, double b) { return dgt(a, b) ? a : b; }
#else
static __device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
static __device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
#define dlt(a, b) ((a) < (b))
#define dle(a, b) ((a) <= (b))
#define dgt(a, b) ((a) > (b))
#define dge(a, b) ((a) >= (b))
#define deq(a, b) ((a) == (b))
#define dne(a, b) ((a) != (b))
#define dabs_lt(x, c) (fabs(x) < (c))
#define dabs_le(x, c) (fabs(x) <= (c))
#endif

} // namespace f64
} // namespace vg
