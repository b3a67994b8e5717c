// Minimal stand-in for Kokkos_Macros.hpp: lets the reference's Hex8 master
// element compile on the host without Kokkos (Serial semantics only).
#pragma once
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_IMPL_MEMORY_ALIGNMENT 64
