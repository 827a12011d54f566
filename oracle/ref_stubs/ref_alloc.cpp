// ref_alloc.cpp -- array allocation for the reference host code compiled into
// the test library (oracle test infrastructure only).
//
// The reference reads and writes one float past its trace arrays:
// deriv::adjoint reads d[i+1] for the last sample of the last trace and
// deriv::forward adds into d[n] (Born/deriv_3d.cpp:17-19, :38-40).  With the
// stock allocator that read returns heap garbage and the results change from
// run to run.  Every new[] here is zero-filled with a 64-byte zero tail, so
// the reads see 0 and the writes land in padding -- the values the oracle
// defines for those accesses.  The library links with -Bsymbolic-functions,
// so only the reference code inside it uses these operators.
#include <cstdlib>
#include <new>

void *operator new[](std::size_t n) {
  void *p = std::calloc(1, n + 64);
  if (!p) throw std::bad_alloc();
  return p;
}
void *operator new[](std::size_t n, const std::nothrow_t &) noexcept { return std::calloc(1, n + 64); }
void operator delete[](void *p) noexcept { std::free(p); }
void operator delete[](void *p, std::size_t) noexcept { std::free(p); }
void operator delete[](void *p, const std::nothrow_t &) noexcept { std::free(p); }
