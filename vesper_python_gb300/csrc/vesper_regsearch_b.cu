// Register two-step search passes: the compiled sides, table b of two.
// Split across translation units so that they compile in parallel.
#define VG_PASS_TYPES_ONLY
#include "vesper_regpass.cuh"

namespace vg {

const RegEntry *find_reg_b(int mode, int d) {
    static const RegEntry table[] = {
        RegPath<VESPER_MODE_VEC, 3, 1, 15, 5>::entry(),   // 75: 200^3 / 100^3 pairs at s = 2
        RegPath<VESPER_MODE_VEC, 3, 1, 8, 4>::entry(),    // 32: 128^3 / 64^3 pairs at s = 3
        // the scalar modes of the 200^3 / 100^3 workload (side 75)
        RegPath<VESPER_MODE_OVERLAP, 1, 1, 15, 5>::entry(),
        RegPath<VESPER_MODE_CC, 1, 1, 15, 5>::entry(),
        RegPath<VESPER_MODE_PCC, 1, 1, 15, 5>::entry(),
        RegPath<VESPER_MODE_LAPLACIAN, 1, 1, 15, 5>::entry(),
    };
    for (const RegEntry &e : table)
        if (e.mode == mode && e.d == d) return &e;
    return nullptr;
}

}  // namespace vg
