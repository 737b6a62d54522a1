// One hash-family instantiation per object file: compiled once per
// (FAMILY_HASH, FAMILY_N, FAMILY_ROBUST) so the twelve variants build in
// parallel.  Each object defines cuspx_register_<hash>_<n>_<robust>().
#include "spx_launch.cuh"

#if !defined(FAMILY_HASH) || !defined(FAMILY_N) || !defined(FAMILY_ROBUST)
#error "compile with -DFAMILY_HASH=0|1 -DFAMILY_N=16|24|32 -DFAMILY_ROBUST=0|1"
#endif

#define CUSPX_CAT2(a, b, c, d) a##_##b##_##c##_##d
#define CUSPX_CAT(a, b, c, d) CUSPX_CAT2(a, b, c, d)

namespace cuspx {
#if FAMILY_HASH == 0
using FamilyHF = Sha2<FAMILY_N, FAMILY_ROBUST != 0>;
#else
using FamilyHF = Shake<FAMILY_N, FAMILY_ROBUST != 0>;
#endif

void CUSPX_CAT(register_family, FAMILY_HASH, FAMILY_N, FAMILY_ROBUST)() {
    g_family[FAMILY_HASH][FAMILY_N / 8 - 2][FAMILY_ROBUST] = Family<FamilyHF>::ops();
}
}  // namespace cuspx
