// Minimal stand-in for the Legion runtime headers, written for this project.
//
// Test infrastructure only: it lets the reference solver's own CPU task
// bodies (the `cpu_base_impl` functions of HTR's src/prometeo_*.cc) compile
// and run outside a Legion runtime.  A "region" here is a set of host
// buffers, one per field, each addressed through affine byte strides exactly
// like Realm's AffineAccessor (element at point p lives at
// base + p.x*sx + p.y*sy + p.z*sz).  Task registration, layout constraints
// and reductions are accepted and ignored.
#ifndef HTR_ORACLE_LEGION_SHIM_H
#define HTR_ORACLE_LEGION_SHIM_H

#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>
#include <algorithm>
#include <type_traits>

namespace Realm {
template <typename FT, int N, typename T> struct AffineAccessor {};
}  // namespace Realm

namespace Legion {

typedef long long coord_t;
typedef unsigned FieldID;
typedef void *Context;
typedef unsigned LayoutConstraintID;

template <int N, typename T = coord_t> struct Point;

template <typename T> struct Point<1, T> {
  T x;
  Point() : x(0) {}
  Point(T a) : x(a) {}
  operator T() const { return x; }
};

template <typename T> struct Point<3, T> {
  T x, y, z;
  Point() : x(0), y(0), z(0) {}
  Point(T a, T b, T c) : x(a), y(b), z(c) {}
  Point operator+(const Point &o) const { return Point(x + o.x, y + o.y, z + o.z); }
  Point operator-(const Point &o) const { return Point(x - o.x, y - o.y, z - o.z); }
};

template <int N, typename T = coord_t> struct Rect {
  Point<N, T> lo, hi;
  Rect() {}
  Rect(const Point<N, T> &l, const Point<N, T> &h) : lo(l), hi(h) {}
};

// An index space only knows the rectangle it spans.
struct IndexSpace {
  const Rect<3> *rect = nullptr;
};

struct LogicalRegion {
  IndexSpace is;
  IndexSpace get_index_space() const { return is; }
};

// A Domain made of one rectangle (all HTR CPU tasks use one).
struct Domain {
  Rect<3> r;
  Domain() {}
  Domain(const Rect<3> &rr) : r(rr) {}
  operator Rect<3>() const { return r; }
};

template <int N, typename T = coord_t> struct RectInDomainIterator {
  Rect<N, T> r;
  bool valid;
  RectInDomainIterator(const Domain &d) : r(d.r), valid(true) {}
  bool operator()() const { return valid; }
  RectInDomainIterator &operator++(int) { valid = false; return *this; }
  RectInDomainIterator &operator++() { valid = false; return *this; }
  const Rect<N, T> &operator*() const { return r; }
};

struct FieldBinding {
  char *base = nullptr;   // address of point (0,0,0) (may lie outside the buffer)
  coord_t stride[3] = {0, 0, 0};  // bytes
};

struct PhysicalRegion {
  std::map<FieldID, FieldBinding> fields;
  LogicalRegion lr;
  LogicalRegion get_logical_region() const { return lr; }
  const FieldBinding &field(FieldID fid) const {
    auto it = fields.find(fid);
    assert(it != fields.end() && "field not bound in shim region");
    return it->second;
  }
};

struct Future {
  double value = 0.0;
  Future() {}
  Future(double v) : value(v) {}
  template <typename T> T get_result() const {
    if constexpr (std::is_constructible_v<T, double>)
      return T(value);
    else
      return T();  // results the harness never reads (e.g. averages)
  }
};

template <typename T> struct DeferredValue {
  T v;
  DeferredValue(T x = T()) : v(x) {}
};

struct Task {
  const void *args = nullptr;
  size_t arglen = 0;
  const void *local_args = nullptr;
  size_t local_arglen = 0;
  std::vector<Future> futures;
};

struct Processor {
  enum Kind { LOC_PROC, OMP_PROC, TOC_PROC };
};

struct ProcessorConstraint {
  ProcessorConstraint(Processor::Kind) {}
};

struct TaskVariantRegistrar {
  TaskVariantRegistrar(int, const char *) {}
  template <typename C> void add_constraint(const C &) {}
  void set_leaf(bool) {}
  void add_layout_constraint_set(unsigned, LayoutConstraintID) {}
};

struct LayoutConstraintRegistrar {
  template <typename C> void add_constraint(const C &) {}
};

class Runtime {
 public:
  Domain get_index_space_domain(Context, IndexSpace is) {
    assert(is.rect != nullptr);
    return Domain(*is.rect);
  }
  template <void (*F)(const Task *, const std::vector<PhysicalRegion> &, Context, Runtime *)>
  static void preregister_task_variant(const TaskVariantRegistrar &, const char *) {}
  template <typename R, R (*F)(const Task *, const std::vector<PhysicalRegion> &, Context, Runtime *)>
  static void preregister_task_variant(const TaskVariantRegistrar &, const char *) {}
  static LayoutConstraintID preregister_layout(const LayoutConstraintRegistrar &) { return 0; }
};

enum PrivilegeMode { READ_ONLY, READ_WRITE, WRITE_ONLY, WRITE_DISCARD, REDUCE };

template <PrivilegeMode M, typename FT, int N, typename T, typename A>
class FieldAccessor {
 public:
  FieldAccessor() {}
  FieldAccessor(const PhysicalRegion &r, FieldID fid) : b(r.field(fid)) {}
  FT &operator[](const Point<3, T> &p) const {
    return *reinterpret_cast<FT *>(b.base + p.x * b.stride[0] + p.y * b.stride[1] +
                                   p.z * b.stride[2]);
  }
  FT &operator[](const Point<1, T> &p) const {
    return *reinterpret_cast<FT *>(b.base + p.x * b.stride[0]);
  }

 private:
  FieldBinding b;
};

template <typename T> class SumReduction {};
template <typename T> class MaxReduction {};
template <typename T> class MinReduction {};

template <typename REDOP, bool EXCLUSIVE, int N, typename T, typename A>
class ReductionAccessor {
 public:
  // reductions are never executed by the harness: folding into the proxy is a no-op
  struct Ref {
    template <typename V> const Ref &operator<<=(const V &) const { return *this; }
  };
  ReductionAccessor() {}
  ReductionAccessor(const PhysicalRegion &, FieldID, int) {}
  template <typename P> Ref operator[](const P &) const { return Ref(); }
};
static const int LEGION_REDOP_SUM_FLOAT64 = 0;

// Compare-and-swap helpers named by the reference's reduction operators
// (never executed by the harness: its tasks do not reduce).
namespace TypePunning {
template <typename T> struct Pointer {
  void *p;
  explicit Pointer(void *q) : p(q) {}
  operator T *() const { return static_cast<T *>(p); }
};
template <typename A, typename B> struct Alias {
  A a;
  void load(const Pointer<A> &q) { a = *static_cast<A *>(q.p); }
  A as_one() const { return a; }
  B as_two() const {
    B b;
    std::memcpy(&b, &a, sizeof(b));
    return b;
  }
  Alias &operator=(B b) {
    std::memcpy(&a, &b, sizeof(a));
    return *this;
  }
};
}  // namespace TypePunning

}  // namespace Legion

using Legion::coord_t;

#endif
