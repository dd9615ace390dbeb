// Register two-step search passes: the compiled sides, table c (the sides
// of the uneven-pair batch at s = 4, and prob mode at side 64).  Split across translation units so
// that they compile in parallel.
#define VG_PASS_TYPES_ONLY
#include "vesper_regpass.cuh"

namespace vg {

const RegEntry *find_reg_c(int mode, int d) {
    static const RegEntry table[] = {
        RegPath<VESPER_MODE_VEC, 3, 1, 9, 3>::entry(),    // 27
        RegPath<VESPER_MODE_VEC, 3, 1, 11, 3>::entry(),   // 33
        RegPath<VESPER_MODE_VEC, 3, 1, 7, 5>::entry(),    // 35
        RegPath<VESPER_MODE_VEC, 3, 1, 7, 6>::entry(),    // 42
        RegPath<VESPER_MODE_VEC, 3, 1, 11, 4>::entry(),   // 44
        RegPath<VESPER_MODE_PROB, 7, 2, 8, 8>::entry(),   // 64: prob mode on grids padded to 64^3
        RegPath<VESPER_MODE_PROB, 7, 2, 8, 4>::entry(),   // 32: prob mode, 128^3 / 64^3 pairs at s = 3
        RegPath<VESPER_MODE_PROB, 7, 2, 10, 3>::entry(),  // 30
    };
    for (const RegEntry &e : table)
        if (e.mode == mode && e.d == d) return &e;
    return nullptr;
}

}  // namespace vg
