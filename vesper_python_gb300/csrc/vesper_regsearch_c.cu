// Register two-step search passes: the compiled sides, table c (the sides
// of the uneven-pair batch at s = 4).  Split across translation units so
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
    };
    for (const RegEntry &e : table)
        if (e.mode == mode && e.d == d) return &e;
    return nullptr;
}

}  // namespace vg
