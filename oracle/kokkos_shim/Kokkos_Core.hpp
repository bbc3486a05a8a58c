// Serial Kokkos-subset shim: TEST INFRASTRUCTURE ONLY.
//
// Kokkos is not installed in this environment, so the unmodified ExaMiniMD
// sources cannot be built as shipped.  This header implements, serially and
// on the host only, exactly the subset of the Kokkos API that ExaMiniMD's
// sources call (View, subview, deep_copy, resize, parallel_for/reduce/scan
// over Range and Team policies, team scratch, atomics, BinSort/BinOp3D,
// StaticCrsGraph, UnorderedMap, Timer).  It was written from the call sites
// in ExaMiniMD (src/*.cpp, src/*/*.h), not from Kokkos sources.
//
// Semantics fixed by this shim (they define "bit-exact" for the oracle):
//  * every parallel dispatch runs serially in index order (league order for
//    teams, team_size = vector_length = 1), so every atomic in ExaMiniMD
//    resolves in loop order;
//  * BinOp3D bins a key per dimension as int((x - min) * nbin/(max - min))
//    with x the slowest index; BinSort fills each bin in ascending source
//    index (a stable counting sort);
//  * the default layout is LayoutRight (host execution space).
//
// It is built only into oracle/_ref/ref_examinimd by oracle/Makefile.ref and
// is never linked into the product library.
#ifndef EMD_KOKKOS_SHIM_CORE_HPP
#define EMD_KOKKOS_SHIM_CORE_HPP

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_ENABLE_SERIAL 1

namespace Kokkos {

// ---------------------------------------------------------------- tags
enum MemoryTraitsFlags { Unmanaged = 0x01, RandomAccess = 0x02, Atomic = 0x04, Restrict = 0x08 };
template <unsigned N> struct MemoryTraits { enum : unsigned { value = N }; };
struct LayoutLeft {};
struct LayoutRight {};
struct LayoutStride {};
struct HostSpace {};
struct Dynamic {};
struct Static {};
template <class T> struct Schedule {};
template <class T> struct IndexType {};
struct AUTO_t { constexpr AUTO_t() {} };
constexpr AUTO_t AUTO{};
struct ParallelForTag {};
struct ParallelReduceTag {};

struct Serial {
  using memory_space = HostSpace;
  using execution_space = Serial;
  using array_layout = LayoutRight;
  static int concurrency() { return 1; }
  void print_configuration(std::ostream& os, bool = false) const {
    os << "Kokkos (serial subset shim): host serial execution\n";
  }
  void fence() const {}
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;
template <class E, class M> struct Device {};

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}
inline void fence(const std::string&) {}
[[noreturn]] inline void abort(const char* msg) {
  std::fprintf(stderr, "%s\n", msg);
  std::fflush(stderr);
  std::abort();
}

namespace Profiling {
inline void pushRegion(const std::string&) {}
inline void popRegion() {}
}  // namespace Profiling

template <class T1, class T2>
struct pair {
  T1 first;
  T2 second;
  pair() : first(), second() {}
  pair(const T1& a, const T2& b) : first(a), second(b) {}
  template <class U1, class U2>
  pair(const std::pair<U1, U2>& p) : first(p.first), second(p.second) {}
  bool operator==(const pair& o) const { return first == o.first && second == o.second; }
  bool operator!=(const pair& o) const { return !(*this == o); }
};

struct ALL_t {
  constexpr ALL_t() {}
  constexpr const ALL_t& operator()() const { return *this; }
};
constexpr ALL_t ALL{};

class Timer {
  std::chrono::steady_clock::time_point t0_;

 public:
  Timer() : t0_(std::chrono::steady_clock::now()) {}
  void reset() { t0_ = std::chrono::steady_clock::now(); }
  double seconds() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }
};

template <class T> inline void atomic_add(T* p, const T& v) { *p += v; }
template <class T> inline void atomic_add(volatile T* p, const T& v) { *p += v; }
template <class T> inline T atomic_fetch_add(T* p, const T& v) { T o = *p; *p += v; return o; }
template <class T> inline T atomic_fetch_add(volatile T* p, const T& v) { T o = *p; *p += v; return o; }

// ---------------------------------------------------------------- scratch
// A bump allocator standing in for team / thread scratch memory.
struct ScratchArena {
  char* base = nullptr;
  size_t size = 0;
  size_t used = 0;
  void* get(size_t bytes) {
    size_t aligned = (used + 15) & ~size_t(15);
    if (aligned + bytes > size) Kokkos::abort("kokkos shim: scratch request exceeds the size set by set_scratch_size");
    used = aligned + bytes;
    return base + aligned;
  }
};

namespace Impl {
// Data-type analysis: T*..*[N0][N1].. -> value type, dynamic rank, static extents.
template <class T> struct DA {
  using value_type = T;
  static constexpr int nptr = 0;
  static constexpr int nstat = 0;
  static void statics(size_t*) {}
};
template <class T> struct DA<T*> {
  using value_type = typename DA<T>::value_type;
  static constexpr int nptr = DA<T>::nptr + 1;
  static constexpr int nstat = DA<T>::nstat;
  static void statics(size_t* s) { DA<T>::statics(s); }
};
template <class T, size_t N> struct DA<T[N]> {
  using value_type = typename DA<T>::value_type;
  static constexpr int nptr = DA<T>::nptr;
  static constexpr int nstat = DA<T>::nstat + 1;
  static void statics(size_t* s) { s[0] = N; DA<T>::statics(s + 1); }
};
template <class T, int R> struct AddPtr { using type = typename AddPtr<T*, R - 1>::type; };
template <class T> struct AddPtr<T, 0> { using type = T; };

template <class... P> struct HasLayoutLeft : std::false_type {};
template <class H, class... P> struct HasLayoutLeft<H, P...>
    : std::integral_constant<bool, std::is_same<H, LayoutLeft>::value || HasLayoutLeft<P...>::value> {};

struct RangeArg {
  bool is_range;
  size_t b, e;
};
inline RangeArg to_arg(const ALL_t&) { return {true, 0, size_t(-1)}; }
template <class A, class B> inline RangeArg to_arg(const std::pair<A, B>& p) { return {true, size_t(p.first), size_t(p.second)}; }
template <class A, class B> inline RangeArg to_arg(const Kokkos::pair<A, B>& p) { return {true, size_t(p.first), size_t(p.second)}; }
template <class I, class = typename std::enable_if<std::is_integral<I>::value>::type>
inline RangeArg to_arg(I i) { return {false, size_t(i), size_t(i) + 1}; }

template <class A> struct IsRangeArg : std::false_type {};
template <> struct IsRangeArg<ALL_t> : std::true_type {};
template <class A, class B> struct IsRangeArg<std::pair<A, B>> : std::true_type {};
template <class A, class B> struct IsRangeArg<Kokkos::pair<A, B>> : std::true_type {};
template <class... A> struct CountRanges { static constexpr int value = 0; };
template <class H, class... A> struct CountRanges<H, A...> {
  static constexpr int value = (IsRangeArg<typename std::decay<H>::type>::value ? 1 : 0) + CountRanges<A...>::value;
};
}  // namespace Impl

// ---------------------------------------------------------------- View
// Every View is a strided window onto (possibly shared) storage.
template <class DataType, class... Props>
class View {
 public:
  using data_type = DataType;
  using value_type = typename Impl::DA<DataType>::value_type;
  using non_const_value_type = typename std::remove_const<value_type>::type;
  using const_value_type = const non_const_value_type;
  using pointer_type = value_type*;
  using reference_type = value_type&;
  using HostMirror = View<DataType, Props...>;
  using memory_space = HostSpace;
  using execution_space = Serial;
  using size_type = size_t;
  static constexpr int Rank = Impl::DA<DataType>::nptr + Impl::DA<DataType>::nstat;
  static constexpr int rank = Rank;
  static constexpr int rank_dynamic = Impl::DA<DataType>::nptr;
  static constexpr bool layout_left = Impl::HasLayoutLeft<Props...>::value;

  value_type* ptr_ = nullptr;
  std::shared_ptr<void> track_;
  size_t ext_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  size_t str_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::string label_;

  View() { set_static_extents(); }

  // allocation: label plus the dynamic extents (trailing static extents fixed by type)
  template <class... I>
  explicit View(const std::string& label, I... dims) : label_(label) {
    set_extents(dims...);
    allocate();
  }
  template <class... I>
  explicit View(const char* label, I... dims) : View(std::string(label), dims...) {}

  // scratch placement (team/thread scratch)
  template <class... I>
  View(ScratchArena& arena, I... dims) {
    set_extents(dims...);
    compute_strides();
    ptr_ = static_cast<value_type*>(arena.get(span() * sizeof(value_type)));
  }

  // unmanaged wrap of a raw pointer
  template <class... I>
  View(value_type* p, I... dims) {
    set_extents(dims...);
    compute_strides();
    ptr_ = p;
  }

  // conversion between Views of equal rank (layout / traits / const)
  template <class D2, class... P2,
            class = typename std::enable_if<View<D2, P2...>::Rank == Rank>::type>
  View(const View<D2, P2...>& o) {
    ptr_ = o.ptr_;
    track_ = o.track_;
    for (int d = 0; d < 8; ++d) { ext_[d] = o.ext_[d]; str_[d] = o.str_[d]; }
    label_ = o.label_;
  }
  template <class D2, class... P2,
            class = typename std::enable_if<View<D2, P2...>::Rank == Rank>::type>
  View& operator=(const View<D2, P2...>& o) {
    ptr_ = o.ptr_;
    track_ = o.track_;
    for (int d = 0; d < 8; ++d) { ext_[d] = o.ext_[d]; str_[d] = o.str_[d]; }
    label_ = o.label_;
    return *this;
  }
  View(const View&) = default;
  View& operator=(const View&) = default;

  // subview constructor: View(src, index/range/ALL ...)
  template <class D2, class... P2, class A0, class... A>
  View(const View<D2, P2...>& src, const A0& a0, const A&... a) {
    static_assert(sizeof...(A) + 1 == View<D2, P2...>::Rank, "subview needs one argument per rank");
    Impl::RangeArg args[] = {Impl::to_arg(a0), Impl::to_arg(a)...};
    size_t off = 0;
    int r = 0;
    for (int d = 0; d < View<D2, P2...>::Rank; ++d) {
      size_t e = args[d].e == size_t(-1) ? src.ext_[d] : args[d].e;
      off += args[d].b * src.str_[d];
      if (args[d].is_range) {
        ext_[r] = e - args[d].b;
        str_[r] = src.str_[d];
        ++r;
      }
    }
    if (r != Rank) Kokkos::abort("kokkos shim: subview rank mismatch");
    ptr_ = src.ptr_ + off;
    track_ = src.track_;
    label_ = src.label_;
  }

  // --- extents
  size_t extent(int d) const { return d < Rank ? ext_[d] : 1; }
  int extent_int(int d) const { return int(extent(d)); }
  size_t dimension_0() const { return extent(0); }
  size_t dimension_1() const { return extent(1); }
  size_t span() const {
    size_t s = 1;
    for (int d = 0; d < Rank; ++d) s *= ext_[d];
    return s;
  }
  size_t size() const { return span(); }
  value_type* data() const { return ptr_; }
  const std::string& label() const { return label_; }
  bool span_is_contiguous() const {
    View t;
    for (int d = 0; d < Rank; ++d) t.ext_[d] = ext_[d];
    t.compute_strides();
    for (int d = 0; d < Rank; ++d)
      if (ext_[d] > 1 && t.str_[d] != str_[d]) return false;
    return true;
  }

  template <class... I>
  static size_t shmem_size(I... dims) {
    View t;
    t.set_extents(dims...);
    return ((t.span() * sizeof(value_type)) + 15) & ~size_t(15);
  }

  // --- access
  value_type& operator()() const { return ptr_[0]; }
  template <class I0>
  value_type& operator()(I0 i0) const { return ptr_[size_t(i0) * str_[0]]; }
  template <class I0, class I1>
  value_type& operator()(I0 i0, I1 i1) const { return ptr_[size_t(i0) * str_[0] + size_t(i1) * str_[1]]; }
  template <class I0, class I1, class I2>
  value_type& operator()(I0 i0, I1 i1, I2 i2) const {
    return ptr_[size_t(i0) * str_[0] + size_t(i1) * str_[1] + size_t(i2) * str_[2]];
  }
  template <class I0, class I1, class I2, class I3>
  value_type& operator()(I0 i0, I1 i1, I2 i2, I3 i3) const {
    return ptr_[size_t(i0) * str_[0] + size_t(i1) * str_[1] + size_t(i2) * str_[2] + size_t(i3) * str_[3]];
  }
  template <class I0, class I1, class I2, class I3, class I4>
  value_type& operator()(I0 i0, I1 i1, I2 i2, I3 i3, I4 i4) const {
    return ptr_[size_t(i0) * str_[0] + size_t(i1) * str_[1] + size_t(i2) * str_[2] + size_t(i3) * str_[3] +
                size_t(i4) * str_[4]];
  }
  template <class I0, class I1, class I2, class I3, class I4, class I5>
  value_type& operator()(I0 i0, I1 i1, I2 i2, I3 i3, I4 i4, I5 i5) const {
    return ptr_[size_t(i0) * str_[0] + size_t(i1) * str_[1] + size_t(i2) * str_[2] + size_t(i3) * str_[3] +
                size_t(i4) * str_[4] + size_t(i5) * str_[5]];
  }
  template <class I0>
  value_type& operator[](I0 i0) const { return ptr_[size_t(i0) * str_[0]]; }

  // flat multi-index walk used by deep_copy between layouts
  size_t offset_of_flat(size_t flat) const {
    size_t off = 0;
    for (int d = Rank - 1; d >= 0; --d) {
      size_t idx = flat % ext_[d];
      flat /= ext_[d];
      off += idx * str_[d];
    }
    return off;
  }

  // (re)allocate with new extents; keep=true preserves the overlapping region
  template <class... I>
  void reshape_alloc(bool keep, I... dims) {
    View old = *this;
    set_extents(dims...);
    allocate();
    if (keep && old.ptr_) {
      size_t lim[8];
      for (int d = 0; d < Rank; ++d) lim[d] = std::min(old.ext_[d], ext_[d]);
      size_t total = 1;
      for (int d = 0; d < Rank; ++d) total *= lim[d];
      for (size_t flat = 0; flat < total; ++flat) {
        size_t f = flat, o_off = 0, n_off = 0;
        for (int d = Rank - 1; d >= 0; --d) {
          size_t idx = f % lim[d];
          f /= lim[d];
          o_off += idx * old.str_[d];
          n_off += idx * str_[d];
        }
        const_cast<non_const_value_type*>(ptr_)[n_off] = old.ptr_[o_off];
      }
    }
  }

 private:
  void set_static_extents() {
    size_t s[8];
    Impl::DA<DataType>::statics(s);
    for (int k = 0; k < Impl::DA<DataType>::nstat; ++k) ext_[rank_dynamic + k] = s[k];
  }
  template <class... I>
  void set_extents(I... dims) {
    set_static_extents();
    size_t d[] = {size_t(dims)..., 0};
    const int nd = int(sizeof...(I));
    for (int k = 0; k < rank_dynamic; ++k) ext_[k] = k < nd ? d[k] : 0;
  }
  void compute_strides() {
    if (layout_left) {
      size_t s = 1;
      for (int d = 0; d < Rank; ++d) { str_[d] = s; s *= (ext_[d] ? ext_[d] : 1); }
    } else {
      size_t s = 1;
      for (int d = Rank - 1; d >= 0; --d) { str_[d] = s; s *= (ext_[d] ? ext_[d] : 1); }
    }
  }
  void allocate() {
    compute_strides();
    size_t n = span();
    if (n == 0) n = 1;
    auto* mem = new non_const_value_type[n]();
    track_ = std::shared_ptr<void>(mem, [](void* p) { delete[] static_cast<non_const_value_type*>(p); });
    ptr_ = mem;
  }
};

template <class V, class... A>
auto subview(const V& v, const A&... a)
    -> View<typename Impl::AddPtr<typename V::value_type, Impl::CountRanges<A...>::value>::type, LayoutStride> {
  return View<typename Impl::AddPtr<typename V::value_type, Impl::CountRanges<A...>::value>::type, LayoutStride>(v, a...);
}

template <class V>
V create_mirror_view(const V& v) { return v; }
template <class V>
V create_mirror(const V& v) {
  V m = v;
  m.reshape_alloc(false, v.extent(0), v.extent(1), v.extent(2), v.extent(3), v.extent(4), v.extent(5), v.extent(6));
  return m;
}

// deep_copy: view <- view (any layouts), view <- scalar, scalar <- rank-0 view
template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
  if (dst.ptr_ == src.ptr_) return;
  const size_t n = std::min(dst.span(), src.span());
  auto* out = const_cast<typename View<D1, P1...>::non_const_value_type*>(dst.ptr_);
  for (size_t f = 0; f < n; ++f) out[dst.offset_of_flat(f)] = src.ptr_[src.offset_of_flat(f)];
}
template <class D1, class... P1, class S,
          class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
void deep_copy(const View<D1, P1...>& dst, const S& s) {
  const size_t n = dst.span();
  auto* out = const_cast<typename View<D1, P1...>::non_const_value_type*>(dst.ptr_);
  for (size_t f = 0; f < n; ++f) out[dst.offset_of_flat(f)] = s;
}
template <class S, class D1, class... P1,
          class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
void deep_copy(S& s, const View<D1, P1...>& src) { s = src.ptr_[0]; }

template <class D, class... P, class... I>
void resize(View<D, P...>& v, I... dims) { v.reshape_alloc(true, dims...); }
template <class D, class... P, class... I>
void realloc(View<D, P...>& v, I... dims) { v.reshape_alloc(false, dims...); }

// ---------------------------------------------------------------- policies
template <class... Props>
struct RangePolicy {
  long begin_, end_;
  RangePolicy(long b, long e) : begin_(b), end_(e) {}
};
namespace Impl {
// The functor tag of a policy is its first template argument that is not a
// policy property (IndexType, Schedule, execution space).
template <class H> struct IsPolicyProp : std::false_type {};
template <class T> struct IsPolicyProp<IndexType<T>> : std::true_type {};
template <class T> struct IsPolicyProp<Schedule<T>> : std::true_type {};
template <> struct IsPolicyProp<Serial> : std::true_type {};
template <class... P> struct TagOf { using type = void; };
template <class H, class... P> struct TagOf<H, P...> {
  using type = typename std::conditional<IsPolicyProp<H>::value, typename TagOf<P...>::type, H>::type;
};
}  // namespace Impl

struct ScratchRequestTeam { size_t bytes; };
struct ScratchRequestThread { size_t bytes; };
inline ScratchRequestTeam PerTeam(size_t b) { return {b}; }
inline ScratchRequestThread PerThread(size_t b) { return {b}; }

class TeamMember {
 public:
  int league_rank_, league_size_;
  ScratchArena* team_arena_;
  ScratchArena* thread_arena_;
  int league_rank() const { return league_rank_; }
  int league_size() const { return league_size_; }
  int team_rank() const { return 0; }
  int team_size() const { return 1; }
  void team_barrier() const {}
  ScratchArena& team_scratch(int) const { return *team_arena_; }
  ScratchArena& thread_scratch(int) const { return *thread_arena_; }
  ScratchArena& team_shmem() const { return *team_arena_; }
};
struct SingleThread { const TeamMember& m; };
struct SingleTeam { const TeamMember& m; };
inline SingleThread PerThread(const TeamMember& m) { return {m}; }
inline SingleTeam PerTeam(const TeamMember& m) { return {m}; }
template <class F> void single(const SingleThread&, const F& f) { f(); }
template <class F> void single(const SingleTeam&, const F& f) { f(); }
template <class F, class T> void single(const SingleThread&, const F& f, T& v) { f(v); }

template <class... Props>
struct TeamPolicy {
  using member_type = TeamMember;
  long league_;
  size_t team_scratch_ = 0, thread_scratch_ = 0;
  TeamPolicy(long league, AUTO_t, long = 1) : league_(league) {}
  TeamPolicy(long league, long /*team*/, long /*vector*/ = 1) : league_(league) {}
  TeamPolicy(long league, long /*team*/, AUTO_t) : league_(league) {}
  template <class F, class Tag> int team_size_max(const F&, const Tag&) const { return 1; }
  template <class F, class Tag> int team_size_recommended(const F&, const Tag&) const { return 1; }
  TeamPolicy set_scratch_size(int, ScratchRequestTeam t) const { TeamPolicy p = *this; p.team_scratch_ = t.bytes; return p; }
  TeamPolicy set_scratch_size(int, ScratchRequestThread t) const { TeamPolicy p = *this; p.thread_scratch_ = t.bytes; return p; }
  TeamPolicy set_scratch_size(int, ScratchRequestTeam t, ScratchRequestThread h) const {
    TeamPolicy p = *this; p.team_scratch_ = t.bytes; p.thread_scratch_ = h.bytes; return p;
  }
};

struct TeamThreadRangeT { long b, e; };
struct ThreadVectorRangeT { long b, e; };
template <class I> TeamThreadRangeT TeamThreadRange(const TeamMember&, I n) { return {0, long(n)}; }
template <class I, class J> TeamThreadRangeT TeamThreadRange(const TeamMember&, I b, J e) { return {long(b), long(e)}; }
template <class I> ThreadVectorRangeT ThreadVectorRange(const TeamMember&, I n) { return {0, long(n)}; }
template <class I, class J> ThreadVectorRangeT ThreadVectorRange(const TeamMember&, I b, J e) { return {long(b), long(e)}; }

template <class F> void parallel_for(const TeamThreadRangeT& r, const F& f) { for (long i = r.b; i < r.e; ++i) f(i); }
template <class F> void parallel_for(const ThreadVectorRangeT& r, const F& f) { for (long i = r.b; i < r.e; ++i) f(i); }
template <class F, class T> void parallel_reduce(const TeamThreadRangeT& r, const F& f, T& result) {
  T acc = T();
  for (long i = r.b; i < r.e; ++i) f(i, acc);
  result = acc;
}
template <class F, class T> void parallel_reduce(const ThreadVectorRangeT& r, const F& f, T& result) {
  T acc = T();
  for (long i = r.b; i < r.e; ++i) f(i, acc);
  result = acc;
}
template <class F> void parallel_scan(const ThreadVectorRangeT& r, const F& f) {
  int acc = 0;
  for (long i = r.b; i < r.e; ++i) f(int(i), acc, true);
}
template <class F> void parallel_scan(const TeamThreadRangeT& r, const F& f) {
  int acc = 0;
  for (long i = r.b; i < r.e; ++i) f(int(i), acc, true);
}

namespace Impl {
template <class Tag, class F, class I>
inline void call_range(const F& f, I i, std::true_type) { f(i); }
template <class Tag, class F, class I>
inline void call_range(const F& f, I i, std::false_type) { f(Tag(), i); }
template <class Tag, class F, class I, class T>
inline void call_reduce(const F& f, I i, T& v, std::true_type) { f(i, v); }
template <class Tag, class F, class I, class T>
inline void call_reduce(const F& f, I i, T& v, std::false_type) { f(Tag(), i, v); }
template <class Tag, class F, class I, class T>
inline void call_scan(const F& f, I i, T& v, std::true_type) { f(i, v, true); }
template <class Tag, class F, class I, class T>
inline void call_scan(const F& f, I i, T& v, std::false_type) { f(Tag(), i, v, true); }
template <class Tag, class F>
inline void call_team(const F& f, const TeamMember& m, std::true_type) { f(m); }
template <class Tag, class F>
inline void call_team(const F& f, const TeamMember& m, std::false_type) { f(Tag(), m); }
template <class Tag, class F, class T>
inline void call_team_reduce(const F& f, const TeamMember& m, T& v, std::true_type) { f(m, v); }
template <class Tag, class F, class T>
inline void call_team_reduce(const F& f, const TeamMember& m, T& v, std::false_type) { f(Tag(), m, v); }
}  // namespace Impl

// parallel_for
template <class F> void parallel_for(long n, const F& f) { for (long i = 0; i < n; ++i) f(int(i)); }
template <class F> void parallel_for(const std::string&, long n, const F& f) { parallel_for(n, f); }
template <class... P, class F> void parallel_for(const RangePolicy<P...>& p, const F& f) {
  using Tag = typename Impl::TagOf<P...>::type;
  for (long i = p.begin_; i < p.end_; ++i) Impl::call_range<Tag>(f, int(i), std::is_void<Tag>());
}
template <class... P, class F> void parallel_for(const std::string&, const RangePolicy<P...>& p, const F& f) { parallel_for(p, f); }
template <class... P, class F> void parallel_for(const TeamPolicy<P...>& p, const F& f) {
  using Tag = typename Impl::TagOf<P...>::type;
  std::vector<char> team_buf(p.team_scratch_ + 16), thread_buf(p.thread_scratch_ + 16);
  ScratchArena team_arena{team_buf.data(), team_buf.size(), 0};
  ScratchArena thread_arena{thread_buf.data(), thread_buf.size(), 0};
  for (long l = 0; l < p.league_; ++l) {
    team_arena.used = 0;
    thread_arena.used = 0;
    TeamMember m{int(l), int(p.league_), &team_arena, &thread_arena};
    Impl::call_team<Tag>(f, m, std::is_void<Tag>());
  }
}
template <class... P, class F> void parallel_for(const std::string&, const TeamPolicy<P...>& p, const F& f) { parallel_for(p, f); }

// reducers
template <class T>
struct Max {
  T& ref;
  explicit Max(T& r) : ref(r) {}
};
template <class T>
struct Sum {
  T& ref;
  explicit Sum(T& r) : ref(r) {}
};

// parallel_reduce
template <class F, class T> void parallel_reduce(long n, const F& f, T& result) {
  T acc = T();
  for (long i = 0; i < n; ++i) f(int(i), acc);
  result = acc;
}
template <class F, class T> void parallel_reduce(const std::string&, long n, const F& f, T& result) { parallel_reduce(n, f, result); }
template <class F, class T> void parallel_reduce(const std::string&, long n, const F& f, Max<T> r) {
  T acc = std::numeric_limits<T>::lowest();
  for (long i = 0; i < n; ++i) f(int(i), acc);
  r.ref = acc;
}
template <class... P, class F, class T> void parallel_reduce(const RangePolicy<P...>& p, const F& f, T& result) {
  using Tag = typename Impl::TagOf<P...>::type;
  T acc = T();
  for (long i = p.begin_; i < p.end_; ++i) Impl::call_reduce<Tag>(f, int(i), acc, std::is_void<Tag>());
  result = acc;
}
template <class... P, class F, class T> void parallel_reduce(const std::string&, const RangePolicy<P...>& p, const F& f, T& result) {
  parallel_reduce(p, f, result);
}
template <class... P, class F, class T> void parallel_reduce(const TeamPolicy<P...>& p, const F& f, T& result) {
  using Tag = typename Impl::TagOf<P...>::type;
  std::vector<char> team_buf(p.team_scratch_ + 16), thread_buf(p.thread_scratch_ + 16);
  ScratchArena team_arena{team_buf.data(), team_buf.size(), 0};
  ScratchArena thread_arena{thread_buf.data(), thread_buf.size(), 0};
  T acc = T();
  for (long l = 0; l < p.league_; ++l) {
    team_arena.used = 0;
    thread_arena.used = 0;
    TeamMember m{int(l), int(p.league_), &team_arena, &thread_arena};
    Impl::call_team_reduce<Tag>(f, m, acc, std::is_void<Tag>());
  }
  result = acc;
}
template <class... P, class F, class T> void parallel_reduce(const std::string&, const TeamPolicy<P...>& p, const F& f, T& result) {
  parallel_reduce(p, f, result);
}

// parallel_scan (serial: one pass with final = true)
template <class... P, class F> void parallel_scan(const RangePolicy<P...>& p, const F& f) {
  using Tag = typename Impl::TagOf<P...>::type;
  int acc = 0;
  for (long i = p.begin_; i < p.end_; ++i) Impl::call_scan<Tag>(f, int(i), acc, std::is_void<Tag>());
}
template <class... P, class F> void parallel_scan(const std::string&, const RangePolicy<P...>& p, const F& f) { parallel_scan(p, f); }

}  // namespace Kokkos

#include "Kokkos_Sort.hpp"
#include "Kokkos_StaticCrsGraph.hpp"

#endif  // EMD_KOKKOS_SHIM_CORE_HPP
