// Minimal stand-in for Kokkos_Core.hpp (host, Serial): a row-major unmanaged
// view over a raw pointer with up to 4 extents.  Only what the reference's
// Hex8 master-element sources need to compile and run.
#pragma once
#include "Kokkos_Macros.hpp"
#include <cstddef>
#include <string>
#include <type_traits>
#include <vector>
#include <memory>
#include <iostream>
namespace Kokkos {
struct LayoutRight {};
struct MemoryUnmanaged {};
enum : unsigned { Aligned = 1 };
template <unsigned... > struct MemoryTraits {};
struct HostSpace { using scratch_memory_space = HostSpace; };
struct Serial { using scratch_memory_space = HostSpace; using memory_space = HostSpace; };
using DefaultExecutionSpace = Serial;
struct Dynamic {};
template <class> struct Schedule {};
struct AUTO_t {};
constexpr AUTO_t AUTO{};
struct PerTeam { PerTeam(size_t) {} };
struct PerThread { PerThread(size_t) {} };
struct TeamMember {
  HostSpace team_shmem() const { return {}; }
  int team_size() const { return 1; }
  int team_rank() const { return 0; }
  int league_rank() const { return 0; }
};
template <class... > struct TeamPolicy {
  using member_type = TeamMember;
  TeamPolicy(size_t, AUTO_t) {}
  TeamPolicy& set_scratch_size(int, PerTeam, PerThread) { return *this; }
};
template <class... > struct RangePolicy { RangePolicy(size_t b, size_t e) : b_(b), e_(e) {} size_t b_, e_; };
template <class P, class F> void parallel_for(const std::string&, P p, F f) { for (size_t i = p.b_; i < p.e_; ++i) f(i); }

namespace shim {
template <class T> struct rank_of { using type = T; static constexpr int value = 0; };
template <class T> struct rank_of<T*> { using type = typename rank_of<T>::type; static constexpr int value = 1 + rank_of<T>::value; };
template <class T, size_t N> struct rank_of<T[N]> { using type = typename rank_of<T>::type; static constexpr int value = 1 + rank_of<T>::value; };
}

template <class DataType, class... Props>
class View {
 public:
  using value_type = typename shim::rank_of<DataType>::type;
  static constexpr int rank = shim::rank_of<DataType>::value;
  View() = default;
  View(value_type* p, size_t n0 = 1, size_t n1 = 1, size_t n2 = 1, size_t n3 = 1)
      : p_(p), n_{n0, n1, n2, n3} {}
  View(HostSpace, size_t n0 = 1, size_t n1 = 1, size_t n2 = 1, size_t n3 = 1)
      : p_(nullptr), n_{n0, n1, n2, n3} {}
  template <class I0> value_type& operator()(I0 i) const { return p_[i]; }
  template <class I0, class I1> value_type& operator()(I0 i, I1 j) const { return p_[i * n_[1] + j]; }
  template <class I0, class I1, class I2> value_type& operator()(I0 i, I1 j, I2 k) const {
    return p_[(i * n_[1] + j) * n_[2] + k];
  }
  template <class I0> value_type& operator[](I0 i) const { return p_[i]; }
  size_t extent(int r) const { return n_[r]; }
  size_t size() const { size_t s = 1; for (int r = 0; r < rank; ++r) s *= n_[r]; return s; }
  value_type* data() const { return p_; }
  bool span_is_contiguous() const { return true; }
 private:
  value_type* p_ = nullptr;
  size_t n_[4] = {1, 1, 1, 1};
};
struct ALL_t {};
inline ALL_t ALL() { return {}; }
struct SubviewProxy {
  template <class D, class... P> operator View<D, P...>() const { return View<D, P...>(); }
};
template <class V, class... A> SubviewProxy subview(const V&, A...) { return {}; }
template <class P, class F, class R> void parallel_reduce(const std::string&, P p, F f, R& r) {
  for (size_t i = p.b_; i < p.e_; ++i) f(i, r);
}
}  // namespace Kokkos
