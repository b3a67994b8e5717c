// Stand-in for stk_simd: one double per "SIMD" lane.
#pragma once
#include <cstddef>
#include <memory>
#include <iostream>
#include <limits>
namespace stk { namespace simd {
typedef double Double;
static constexpr int ndoubles = 1;
inline bool are_any(bool b) { return b; }
inline bool are_all(bool b) { return b; }
} }
namespace non_std { template <class T, size_t A> using AlignedAllocator = std::allocator<T>; }
