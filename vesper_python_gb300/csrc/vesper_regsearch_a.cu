// Register two-step search passes: the compiled sides, table a of two.
// Split across translation units so that they compile in parallel.
#define VG_PASS_TYPES_ONLY
#include "vesper_regpass.cuh"

namespace vg {

const RegEntry *find_reg_a(int mode, int d) {
    static const RegEntry table[] = {
        RegPath<VESPER_MODE_VEC, 3, 1, 13, 1>::entry(),   // 128^3 / 64^3 pairs at s = 7
        RegPath<VESPER_MODE_VEC, 3, 1, 7, 4>::entry(),    // 28: 128^3 / 64^3 pairs at s = 3
        RegPath<VESPER_MODE_VEC, 3, 1, 10, 3>::entry(),   // 30
    };
    for (const RegEntry &e : table)
        if (e.mode == mode && e.d == d) return &e;
    return nullptr;
}

// the lookup vesper_search.cu uses
const RegEntry *find_reg(int mode, int d) {
    const RegEntry *e = find_reg_a(mode, d);
    if (!e) e = find_reg_b(mode, d);
    return e ? e : find_reg_c(mode, d);
}

}  // namespace vg
