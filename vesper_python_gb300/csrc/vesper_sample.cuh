// Query source of the search kernels: the packed float4 query (k_pack) and
// the reference's nearest-voxel rotation gather (rot_mrc,
// VESPER_1_prob_new.py:279-354) of one destination voxel.  Shared by the
// pass kernels and the fused small-grid search.
#pragma once

#include "vesper_common.cuh"

namespace vg {

struct Src {
    const float4 *q4;     // [N]
    const float4 *p4;     // [N] or null
    const double *data;   // [N] (Laplacian needs the float64 density)
    int d;
};

__host__ __device__ inline int odd_up(int n) { return n | 1; }

// ---- pack -------------------------------------------------------------------
template <int MODE>
__global__ void k_pack(const double *data, const float *vec, const float *probs, int d, double ave, float4 *q4,
                       float4 *p4) {
    const size_t n = (size_t)d * d * d;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = data[i];
        const float m = v != 0.0 ? 1.f : 0.f;
        float4 o;
        if (MODE == VESPER_MODE_VEC || MODE == VESPER_MODE_PROB) {
            o = make_float4(vec[3 * i], vec[3 * i + 1], vec[3 * i + 2], m);
        } else {
            float val = 0.f;   // query transforms, VESPER_1_prob_new.py:548-553
            if (MODE == VESPER_MODE_OVERLAP) val = v > 0 ? 1.f : 0.f;
            if (MODE == VESPER_MODE_CC) val = v > 0 ? (float)v : 0.f;
            if (MODE == VESPER_MODE_PCC) val = v > 0 ? (float)__dsub_rn(v, ave) : 0.f;
            o = make_float4(val, 0.f, 0.f, m);
        }
        q4[i] = o;
        if (MODE == VESPER_MODE_PROB) p4[i] = make_float4(probs[i], probs[n + i], probs[2 * n + i], probs[3 * n + i]);
    }
}

// ---- gather -----------------------------------------------------------------
// Winning source (last reference row passing bounds and mask) of destination
// (x, y, z): its index, or -1.  Same rule as gather_src, reading the packed
// source once per candidate.
__device__ __forceinline__ int gather4(const float *F, int d, int x, int y, int z, const float4 *q4, float4 &out) {
    int cx[2], cy[2], cz[2];
    const int nx = gather_cands(x, d, cx), ny = gather_cands(y, d, cy), nz = gather_cands(z, d, cz);
    const float hc = 0.5f * (float)d;
    for (int a = 0; a < nz; ++a)
        for (int b = 0; b < nx; ++b)
            for (int e = 0; e < ny; ++e) {
                int ox, oy, oz;
                if (!old_index(F, d, hc, (float)cx[b] - hc, (float)cy[e] - hc, (float)cz[a] - hc, ox, oy, oz))
                    continue;
                const int i = (ox * d + oy) * d + oz;
                const float4 v = q4[i];
                if (v.w != 0.f) {
                    out = v;
                    return i;
                }
            }
    return -1;
}

// Probability channels, each with its own mask p != 0 (VESPER_1_prob_new.py:1245-1297).
__device__ __forceinline__ float4 gather_probs(const float *F, int d, int x, int y, int z, const float4 *p4) {
    int cx[2], cy[2], cz[2];
    const int nx = gather_cands(x, d, cx), ny = gather_cands(y, d, cy), nz = gather_cands(z, d, cz);
    const float hc = 0.5f * (float)d;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    bool s0 = false, s1 = false, s2 = false, s3 = false;
    for (int a = 0; a < nz; ++a)
        for (int b = 0; b < nx; ++b)
            for (int e = 0; e < ny; ++e) {
                int ox, oy, oz;
                if (!old_index(F, d, hc, (float)cx[b] - hc, (float)cy[e] - hc, (float)cz[a] - hc, ox, oy, oz))
                    continue;
                const float4 v = p4[(ox * d + oy) * d + oz];
                if (!s0 && v.x != 0.f) { o.x = v.x; s0 = true; }
                if (!s1 && v.y != 0.f) { o.y = v.y; s1 = true; }
                if (!s2 && v.z != 0.f) { o.z = v.z; s2 = true; }
                if (!s3 && v.w != 0.f) { o.w = v.w; s3 = true; }
                if (s0 && s1 && s2 && s3) return o;
            }
    return o;
}

// Single-candidate shortcut of gather_cands: the source new_pos index that
// lands on destination t, -1 for none, -2 when two rows land there (odd d,
// t = (d-1)/2) and the general enumeration is needed.
__device__ __forceinline__ int cand1(int t, int d) {
    if ((d & 1) == 0) return t;
    const int m = (d - 1) >> 1;
    if (t < m) return t;
    if (t == m) return -2;
    return t < d - 1 ? t + 1 : -1;
}

// gather4 with the rotation matrix in registers and the common case (one
// candidate row per axis) done without the candidate loops.
__device__ __forceinline__ int gather4_fast(const float (&F)[9], int d, int x, int y, int z, const float4 *q4,
                                            float4 &out) {
    const int ix = cand1(x, d), iy = cand1(y, d), iz = cand1(z, d);
    if ((ix | iy | iz) < 0) {
        if (ix == -1 || iy == -1 || iz == -1) return -1;
        return gather4(F, d, x, y, z, q4, out);
    }
    const float hc = 0.5f * (float)d;
    int ox, oy, oz;
    if (!old_index(F, d, hc, (float)ix - hc, (float)iy - hc, (float)iz - hc, ox, oy, oz)) return -1;
    const int i = (ox * d + oy) * d + oz;
    const float4 v = __ldg(q4 + i);   // read-only path: the query is not written during a search
    if (v.w == 0.f) return -1;
    out = v;
    return i;
}

// Source index of destination (x, y, z) when every axis has one candidate
// row (the common case): the voxel (its mask not yet read), -1 for none (out
// of bounds, or no row lands there), -2 when an axis has two candidate rows
// (odd d, middle index) and the general enumeration of gather4 decides.
__device__ __forceinline__ int gather_index_fast(const float (&F)[9], int d, int x, int y, int z) {
    const int ix = cand1(x, d), iy = cand1(y, d), iz = cand1(z, d);
    if ((ix | iy | iz) < 0) return (ix == -1 || iy == -1 || iz == -1) ? -1 : -2;
    const float hc = 0.5f * (float)d;
    int ox, oy, oz;
    if (!old_index(F, d, hc, (float)ix - hc, (float)iy - hc, (float)iz - hc, ox, oy, oz)) return -1;
    return (ox * d + oy) * d + oz;
}

template <int MODE>
__device__ __forceinline__ void sample(const Src &s, const float *F, int x, int y, int z, float *out);

// sample_fast for a side D known at compile time (modes V, O, C, P): the
// candidate rows, the bounds and the index arithmetic fold to constants; the
// rare multi-candidate voxels of odd sides take the general gather.  Same
// results as sample().
template <int MODE, int D>
__device__ __forceinline__ void sample_ct(const Src &s, const float (&F)[9], int x, int y, int z, float *out) {
    static_assert(MODE == VESPER_MODE_VEC || MODE == VESPER_MODE_OVERLAP || MODE == VESPER_MODE_CC ||
                  MODE == VESPER_MODE_PCC, "sample_ct: modes V, O, C, P");
    const int ix = cand1(x, D), iy = cand1(y, D), iz = cand1(z, D);
    bool hit = false;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((ix | iy | iz) < 0) {
        if (ix == -2 || iy == -2 || iz == -2) {
            if (ix != -1 && iy != -1 && iz != -1) {
                sample<MODE>(s, F, x, y, z, out);
                return;
            }
        }
    } else {
        constexpr float hc = 0.5f * (float)D;
        int ox, oy, oz;
        if (old_index(F, D, hc, (float)ix - hc, (float)iy - hc, (float)iz - hc, ox, oy, oz)) {
            v = __ldg(s.q4 + (ox * D + oy) * D + oz);
            hit = v.w != 0.f;
        }
    }
    if (MODE == VESPER_MODE_VEC) {
        float r[3] = {0.f, 0.f, 0.f};
        if (hit) rotate_vec(F, v.x, v.y, v.z, r);
        out[0] = r[0];
        out[1] = r[1];
        out[2] = r[2];
    } else {
        out[0] = hit ? v.x : 0.f;
    }
}

// Channel values of the rotated query at (x, y, z), rotation matrix in
// registers; same results as sample().
template <int MODE>
__device__ __forceinline__ void sample_fast(const Src &s, const float (&F)[9], int x, int y, int z, float *out) {
    if (MODE == VESPER_MODE_LAPLACIAN || MODE == VESPER_MODE_PROB) {
        sample<MODE>(s, F, x, y, z, out);
        return;
    }
    float4 v;
    const bool hit = gather4_fast(F, s.d, x, y, z, s.q4, v) >= 0;
    if (MODE == VESPER_MODE_VEC) {
        float r[3] = {0.f, 0.f, 0.f};
        if (hit) rotate_vec(F, v.x, v.y, v.z, r);
        out[0] = r[0];
        out[1] = r[1];
        out[2] = r[2];
    } else {
        out[0] = hit ? v.x : 0.f;
    }
}

// laplacian_filter of the rotated density at (x, y, z) from that density
// already gathered into rd[d^3] (k_rot_density): the arithmetic of sample<L>
// below, with plain reads where sample<L> gathers each of the seven values.
__device__ __forceinline__ float lap_from_rd(const double *rd, int d, int x, int y, int z) {
    auto D = [&](int xx, int yy, int zz) -> double { return rd[((size_t)xx * d + yy) * d + zz]; };
    const double c = D(x, y, z);
    double acc = 0.0;
    if (c > 0) {
        acc = __dmul_rn(-6.0, c);
        if (x + 1 < d) acc = __dadd_rn(acc, D(x + 1, y, z));
        if (x - 1 >= 0) acc = __dadd_rn(acc, D(x - 1, y, z));
        if (y + 1 < d) acc = __dadd_rn(acc, D(x, y + 1, z));
        if (y - 1 >= 0) acc = __dadd_rn(acc, D(x, y - 1, z));
        if (z + 1 < d) acc = __dadd_rn(acc, D(x, y, z + 1));
        if (z - 1 >= 0) acc = __dadd_rn(acc, D(x, y, z - 1));
    }
    return (float)acc;
}

// Channel values of the rotated query at (x, y, z): out[c] for every channel.
template <int MODE>
__device__ __forceinline__ void sample(const Src &s, const float *F, int x, int y, int z, float *out) {
    const int d = s.d;
    float4 v;
    if (MODE == VESPER_MODE_LAPLACIAN) {
        // laplacian_filter of the rotated density (VESPER_1_prob_new.py:494-526), float64
        auto D = [&](int xx, int yy, int zz) -> double {
            float4 w;
            const int i = gather4(F, d, xx, yy, zz, s.q4, w);
            return i >= 0 ? s.data[i] : 0.0;
        };
        const double c = D(x, y, z);
        double acc = 0.0;
        if (c > 0) {
            acc = __dmul_rn(-6.0, c);
            if (x + 1 < d) acc = __dadd_rn(acc, D(x + 1, y, z));
            if (x - 1 >= 0) acc = __dadd_rn(acc, D(x - 1, y, z));
            if (y + 1 < d) acc = __dadd_rn(acc, D(x, y + 1, z));
            if (y - 1 >= 0) acc = __dadd_rn(acc, D(x, y - 1, z));
            if (z + 1 < d) acc = __dadd_rn(acc, D(x, y, z + 1));
            if (z - 1 >= 0) acc = __dadd_rn(acc, D(x, y, z - 1));
        }
        out[0] = (float)acc;
        return;
    }
    const bool hit = gather4(F, d, x, y, z, s.q4, v) >= 0;
    if (MODE == VESPER_MODE_VEC || MODE == VESPER_MODE_PROB) {
        float r[3] = {0.f, 0.f, 0.f};
        if (hit) rotate_vec(F, v.x, v.y, v.z, r);
        out[0] = r[0];
        out[1] = r[1];
        out[2] = r[2];
        if (MODE == VESPER_MODE_PROB) {
            const float4 p = gather_probs(F, d, x, y, z, s.p4);
            out[3] = p.x;
            out[4] = p.y;
            out[5] = p.z;
            out[6] = p.w;
        }
    } else {
        out[0] = hit ? v.x : 0.f;
    }
}

}  // namespace vg
