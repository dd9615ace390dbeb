// Refinement sets and picks on the device, for the aligner's graph form: the
// +-5 degree refinement slots of every pair's global top-N on the 5-degree
// lattice (VESPER_1_prob_new.py:689-713), and after their search the stable
// top-N over the slots the reference's filter keeps (:739), the picked
// models' rotations, scores and linear translations, and the translations
// wrapped as get_score wraps them (:1323-1329).  Two launches replace the
// tensor arithmetic that built these per pair.
#include "vesper_common.cuh"

namespace vg {

// Slot t = (i N + k) 27 + o: offset o of top k of pair i.  The top's lattice
// row (x, y, z) plus the offset is kept where x < L, y < L and z < L / 2
// (before wrapping) and the top exists (grid index >= 0), then negative
// coordinates wrap by +L; a dropped slot gets row 0.
__global__ void k_refine_slots(const int64_t *tg, int n, int N, const int64_t *grid_rows, int ngrid,
                               const int64_t *off, int L, const float *lat, int64_t *crow, uint8_t *valid,
                               float *rmats) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * N * 27) return;
    const int o = t % 27, ik = t / 27;
    const int64_t g = tg[ik];
    const bool have = g >= 0 && g < ngrid;
    const int64_t row = grid_rows[have ? g : 0];
    const int64_t LL = (int64_t)L * L;
    int64_t c[3] = {row / LL + off[3 * o], (row / L) % L + off[3 * o + 1], row % L + off[3 * o + 2]};
    const bool v = c[0] < L && c[1] < L && c[2] < L / 2 && have;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (c[a] < 0) c[a] += L;
    const int64_t cr = v ? (c[0] * L + c[1]) * L + c[2] : 0;
    crow[t] = cr;
    valid[t] = v ? 1 : 0;
#pragma unroll
    for (int e = 0; e < 9; ++e) rmats[(size_t)t * 9 + e] = lat[cr * 9 + e];
}

// One pair: the stable top-N of scores[s nscore] over the slots s with
// valid[s] (the others read -inf), ties to the lower slot, -1 past the slots;
// then per pick k (slot 0 standing in for -1): the slot's lattice row, its
// score, its linear translation lin, the row's rotation matrix, and
// (lin / d^2, lin / d % d, lin % d) with each t > d / 2 taken as t - d.
constexpr int kPickThreads = 256;
__global__ void __launch_bounds__(kPickThreads) k_refine_pick(const float *scores, const int32_t *lin, int nscore,
                                                              const uint8_t *valid, const int64_t *crow, int nslot,
                                                              int topn, const float *lat, int d, int32_t *rtop,
                                                              int64_t *rows, float *rscore, int64_t *rlin,
                                                              float *mats, int32_t *trans) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long *red = (unsigned long long *)smem;        // [kPickThreads / 32]
    int *pick = (int *)(red + kPickThreads / 32);                 // [topn]
    uint32_t *taken = (uint32_t *)(pick + topn);                  // [ceil(nslot / 32)]
    const int nwords = (nslot + 31) >> 5;
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) taken[i] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < topn; ++k) {
        unsigned long long best = 0ull;
        for (int i = threadIdx.x; i < nslot; i += blockDim.x) {
            if (taken[i >> 5] & (1u << (i & 31))) continue;
            const float s = valid[i] ? scores[(size_t)i * nscore] : -INFINITY;
            best = max(best, make_key(s, (uint32_t)i));
        }
        best = warp_max_u64(best);
        if (lane == 0) red[warp] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long v = 0ull;
            for (int w = 0; w < kPickThreads / 32; ++w) v = max(v, red[w]);
            int idx = -1;
            if (v != 0ull) {
                idx = (int)(0xffffffffu - (uint32_t)(v & 0xffffffffull));
                taken[idx >> 5] |= 1u << (idx & 31);
            }
            pick[k] = idx;
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < topn; k += blockDim.x) {
        const int idx = pick[k];
        const int sel = idx < 0 ? 0 : idx;
        const int64_t r = crow[sel];
        const int64_t l = (int64_t)lin[(size_t)sel * nscore];
        rtop[k] = idx;
        rows[k] = r;
        rscore[k] = scores[(size_t)sel * nscore];
        rlin[k] = l;
#pragma unroll
        for (int e = 0; e < 9; ++e) mats[(size_t)k * 9 + e] = lat[r * 9 + e];
        const int64_t t[3] = {l / ((int64_t)d * d), (l / d) % d, l % d};
#pragma unroll
        for (int a = 0; a < 3; ++a) trans[k * 3 + a] = (int32_t)(2 * t[a] > d ? t[a] - d : t[a]);
    }
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_refine_slots(const int64_t *tg, int n, int topn, const int64_t *grid_rows, int ngrid,
                                   const int64_t *offsets, int lattice_n, const float *lattice, int64_t *crow,
                                   uint8_t *valid, float *rmats, void *stream) {
    if (!tg || !grid_rows || !offsets || !lattice || !crow || !valid || !rmats || n < 0 || topn < 1 || ngrid < 1 ||
        lattice_n < 1)
        return fail(VESPER_ERR_INVALID, "vesper_refine_slots: bad arguments");
    const long long total = (long long)n * topn * 27;
    if (total == 0) return VESPER_OK;
    if (total > (1ll << 30)) return fail(VESPER_ERR_UNSUPPORTED, "vesper_refine_slots: too many slots");
    k_refine_slots<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        tg, n, topn, grid_rows, ngrid, offsets, lattice_n, lattice, crow, valid, rmats);
    VG_CHECK_LAUNCH("k_refine_slots");
    return VESPER_OK;
}

extern "C" int vesper_refine_pick(const float *scores, const int32_t *lin, int nscore, const uint8_t *valid,
                                  const int64_t *crow, int nslot, int topn, const float *lattice, int d,
                                  int32_t *rtop, int64_t *rows, float *rscore, int64_t *rlin, float *mats,
                                  int32_t *trans, void *stream) {
    if (!scores || !lin || !valid || !crow || !lattice || !rtop || !rows || !rscore || !rlin || !mats || !trans ||
        nscore < 1 || nslot < 1 || topn < 1 || d < 1)
        return fail(VESPER_ERR_INVALID, "vesper_refine_pick: bad arguments");
    const size_t sm = (kPickThreads / 32) * sizeof(unsigned long long) + (size_t)topn * sizeof(int) +
                      (size_t)((nslot + 31) / 32) * sizeof(uint32_t);
    if (sm > (size_t)smem_limit()) return fail(VESPER_ERR_UNSUPPORTED, "vesper_refine_pick: too many slots");
    allow_smem(k_refine_pick, sm);
    k_refine_pick<<<1, kPickThreads, sm, (cudaStream_t)stream>>>(scores, lin, nscore, valid, crow, nslot, topn,
                                                                 lattice, d, rtop, rows, rscore, rlin, mats, trans);
    VG_CHECK_LAUNCH("k_refine_pick");
    return VESPER_OK;
}
