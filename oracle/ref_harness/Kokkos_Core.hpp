// TEST INFRASTRUCTURE ONLY.
// The few Kokkos spellings that the reference's hot-path method bodies use
// directly, for a serial host build of those bodies (see ref_harness.cpp).
// Written from the public meaning of these names: lambdas capture by value,
// inline-function markers, restrict, abort and fence.
#ifndef OFX_REF_KOKKOS_CORE_HPP_
#define OFX_REF_KOKKOS_CORE_HPP_
#include <cstdio>
#include <cstdlib>
#include <string>

#define KOKKOS_LAMBDA [=]
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_RESTRICT __restrict__

namespace Kokkos {
struct LayoutRight {};
struct HostSpace {};
struct DefaultExecutionSpace {};
inline void abort(const char* msg) {
  std::fprintf(stderr, "Kokkos::abort: %s\n", msg);
  std::abort();
}
inline void fence() {}
}  // namespace Kokkos
#endif
