/*
 * Op-counting numeric type (test infrastructure).
 *
 * Pre-included (g++ -include) ahead of the reference's sources: it defines the
 * include guard of include/data_type.h and the three typedefs that header makes
 * (include/data_type.h:4-6), with value_type replaced by CountedDouble.  Every +, -,
 * *, / and sqrt the reference executes on a value_type then bumps a counter, which
 * pins the algorithmic FLOP figure of each hot-path function exactly, as written
 * in the reference's source (an expression the source spells out twice counts
 * twice).  Comparisons, abs and negation are counted separately and are not FLOPs.
 */
#ifndef CBNS_COUNT_TYPES_H
#define CBNS_COUNT_TYPES_H
#define _DATA_TYPE_H_

#ifdef __cplusplus
#include <cmath>

struct OpCounts {
  unsigned long long add, mul, div, sqrt, cmp, other;
};
extern OpCounts g_ops;

struct CountedDouble {
  double v;
  CountedDouble() = default;
  constexpr CountedDouble(double x) : v(x) {}
  CountedDouble& operator+=(CountedDouble o) { ++g_ops.add; v += o.v; return *this; }
  CountedDouble& operator-=(CountedDouble o) { ++g_ops.add; v -= o.v; return *this; }
  CountedDouble& operator*=(CountedDouble o) { ++g_ops.mul; v *= o.v; return *this; }
  CountedDouble& operator/=(CountedDouble o) { ++g_ops.div; v /= o.v; return *this; }
  CountedDouble operator-() const { ++g_ops.other; return CountedDouble(-v); }
};
inline CountedDouble operator+(CountedDouble a, CountedDouble b) { ++g_ops.add; return a.v + b.v; }
inline CountedDouble operator-(CountedDouble a, CountedDouble b) { ++g_ops.add; return a.v - b.v; }
inline CountedDouble operator*(CountedDouble a, CountedDouble b) { ++g_ops.mul; return a.v * b.v; }
inline CountedDouble operator/(CountedDouble a, CountedDouble b) { ++g_ops.div; return a.v / b.v; }
inline bool operator<(CountedDouble a, CountedDouble b) { ++g_ops.cmp; return a.v < b.v; }
inline bool operator>(CountedDouble a, CountedDouble b) { ++g_ops.cmp; return a.v > b.v; }
inline bool operator<=(CountedDouble a, CountedDouble b) { ++g_ops.cmp; return a.v <= b.v; }
inline bool operator>=(CountedDouble a, CountedDouble b) { ++g_ops.cmp; return a.v >= b.v; }
namespace std {
inline CountedDouble sqrt(CountedDouble a) { ++g_ops.sqrt; return std::sqrt(a.v); }
inline CountedDouble abs(CountedDouble a) { ++g_ops.other; return std::fabs(a.v); }
inline CountedDouble sin(CountedDouble a) { ++g_ops.other; return std::sin(a.v); }
inline CountedDouble cos(CountedDouble a) { ++g_ops.other; return std::cos(a.v); }
}  // namespace std

typedef CountedDouble value_type;
#else
typedef double value_type;
#endif
typedef unsigned int size_type;
typedef int index_type;

#endif
