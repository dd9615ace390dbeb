// Search passes with register-resident two-step line FFTs, for grid sides
// d = N1 * N2 compiled in (vesper_search.cu instantiates the sides it
// supports this way; every other side uses the radix-stage passes of
// vesper_passes.cuh).  Same inputs, outputs and layouts as those passes.
//
//   A  gather C channels of one x plane (two rows per packed complex z line),
//      z R2C (step 1 in place, step 2 + unpack into the plane), y FFT (step 1
//      in place, step 2 straight to S in global memory)
//   B  x FFT step 1 from S in global memory, step 2 + conj(T) product summed
//      per group in registers, inverse step 2 in registers, inverse step 1
//      straight to U
//   C  inverse y (step 2 from U in global memory, step 1), inverse z C2R
//      (packing + step 2, step 1 in registers) and the argmax
#pragma once

#include "vesper_passes.cuh"
#include "vesper_regfft.cuh"

namespace vg {

template <int N1, int N2>
struct RGeom {
    static constexpr int D = N1 * N2;
    static constexpr int H = D / 2 + 1;
    static constexpr int NP = (D + 1) / 2;
    static constexpr int Zp = D | 1;
    static constexpr int Hp = H | 1;
};

// Gather of the packed rows (2p, 2p+1) of NIT items, GI items per thread in
// flight: every item's source indices first, then all their loads, then the
// values (V/O/C/P modes; the rare multi-candidate voxels of odd sides take the
// general gather).  map(item, pl, p, z) gives an item's plane slot, packed
// line and z (false: skip); store(pl, p, z, v0, v1) writes its values.
template <int MODE, int NCH, int D, int GI, class Map, class Store>
__device__ __forceinline__ void gather_rows_batched(const PassA2 &a, const float (&Fr)[9], int b, int x0, int NIT,
                                                    Map map, Store store) {
    const int T = blockDim.x;
    for (int base = threadIdx.x; base < NIT; base += GI * T) {
        int src[GI][2], pl[GI], pp[GI], zz[GI];
        bool on[GI];
#pragma unroll
        for (int g = 0; g < GI; ++g) {
            const int item = base + g * T;
            on[g] = item < NIT && map(item, pl[g], pp[g], zz[g]);
            src[g][0] = src[g][1] = -1;
            if (on[g]) {
                const int x = x0 + pl[g], y0 = 2 * pp[g];
                src[g][0] = gather_index_fast(Fr, D, x, y0, zz[g]);
                if (y0 + 1 < D) src[g][1] = gather_index_fast(Fr, D, x, y0 + 1, zz[g]);
            }
        }
        float4 q[GI][2];
#pragma unroll
        for (int g = 0; g < GI; ++g)
#pragma unroll
            for (int h = 0; h < 2; ++h)
                q[g][h] = src[g][h] >= 0 ? __ldg(a.src.q4 + src[g][h]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int g = 0; g < GI; ++g) {
            if (!on[g]) continue;
            float v[2][NCH];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int y = 2 * pp[g] + h;
                if (src[g][h] == -2) {
                    sample<MODE>(a.src, Fr, x0 + pl[g], y, zz[g], v[h]);
                } else {
                    const float4 w = q[g][h];
                    const bool hit = src[g][h] >= 0 && w.w != 0.f;
                    if (MODE == VESPER_MODE_VEC) {
                        float r3[3] = {0.f, 0.f, 0.f};
                        if (hit) rotate_vec(Fr, w.x, w.y, w.z, r3);
#pragma unroll
                        for (int c = 0; c < NCH; ++c) v[h][c] = r3[c < 3 ? c : 0];
                    } else {
                        v[h][0] = hit ? w.x : 0.f;
                    }
                }
            }
            store(pl[g], pp[g], zz[g], v[0], v[1]);
        }
    }
}

// Pass A keeps, per channel, a plane of 2*NP rows of Hp complex values: packed
// z line p lives in the storage of rows 2p and 2p+1 (D <= 2 Hp elements) and is
// unpacked into exactly those two rows.
template <int N1, int N2>
__host__ __device__ inline size_t smem_ra(int cchunk) {
    using G = RGeom<N1, N2>;
    return align16(G::D * sizeof(float2)) + align16(16 * sizeof(float)) +
           (size_t)cchunk * (size_t)(2 * G::NP) * G::Hp * sizeof(float2);
}
template <int N1, int N2>
__host__ __device__ inline size_t smem_rb(int nch, int ngrp, int W) {
    using G = RGeom<N1, N2>;
    return align16(G::D * sizeof(float2)) + (size_t)(nch + ngrp) * G::D * W * sizeof(float2);
}
template <int N1, int N2>
__host__ __device__ inline size_t smem_rc(int ngrp) {
    using G = RGeom<N1, N2>;
    return align16(G::D * sizeof(float2)) + 2 * (size_t)ngrp * G::D * G::Hp * sizeof(float2) +
           3 * 32 * sizeof(unsigned long long);
}

// ---------------------------------------------------------------------------
// Resident CTAs per SM the register budget is sized for: 4 (64 registers)
// where the side's pass A fits without spills, 3 (80) for side 75 and prob,
// 2 for the Laplacian mode (its float64 stencil).
template <int MODE, int N1, int N2>
constexpr int rpass_a_ctas() {
    return MODE == VESPER_MODE_LAPLACIAN ? 2 : (N1 * N2 > 64 || MODE == VESPER_MODE_PROB) ? 3 : 4;
}

template <int MODE, int NCH, int N1, int N2>
__global__ void __launch_bounds__(256, rpass_a_ctas<MODE, N1, N2>()) k_rpass_a(const PassA2 a) {
    using G = RGeom<N1, N2>;
    constexpr int D = G::D, H = G::H, NP = G::NP, Hp = G::Hp;
    constexpr int PS = 2 * NP * Hp;   // plane stride per channel
    extern __shared__ __align__(16) unsigned char smem[];
    const int x = blockIdx.x, b = blockIdx.y, r = a.r0 + b;
    float2 *twn = (float2 *)smem;
    float *F = (float *)(smem + align16(D * sizeof(float2)));
    float2 *plane = (float2 *)(smem + align16(D * sizeof(float2)) + align16(16 * sizeof(float)));
    twiddles_n(D, twn);
    if (threadIdx.x < 9) F[threadIdx.x] = a.rotmats[(size_t)r * 9 + threadIdx.x];
    if (x == 0 && threadIdx.x < a.nscore) a.keys[(size_t)r * a.nscore + threadIdx.x] = 0ull;
    __syncthreads();
    float Fr[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Fr[i] = F[i];
    for (int c0 = 0; c0 < NCH; c0 += a.cchunk) {
        const int cn = min(a.cchunk, NCH - c0);
        // gather rows (2p, 2p+1) into packed z line p (natural z order): each
        // warp covers a tile of 4 packed lines x 8 z (8 rows x 8 z voxels, so
        // its source voxels cluster in fewer cache lines than a row of 32 z)
        constexpr int TP = (NP + 3) / 4, TZ = (D + 7) / 8;
        if constexpr (MODE == VESPER_MODE_VEC || MODE == VESPER_MODE_OVERLAP || MODE == VESPER_MODE_CC ||
                      MODE == VESPER_MODE_PCC) {
            auto map = [&](int item, int &pl, int &p, int &z) {
                const int lane = item & 31, tile = item >> 5;
                pl = 0;
                p = (tile / TZ) * 4 + (lane >> 3);
                z = (tile % TZ) * 8 + (lane & 7);
                return p < NP && z < D;
            };
            auto store = [&](int, int p, int z, const float *v0, const float *v1) {
#pragma unroll
                for (int c = 0; c < NCH; ++c)
                    if (c >= c0 && c < c0 + cn) plane[(c - c0) * PS + 2 * p * Hp + z] = make_float2(v0[c], v1[c]);
            };
            gather_rows_batched<MODE, NCH, D, 2>(a, Fr, b, x, TP * TZ * 32, map, store);
        } else
        for (int t = threadIdx.x; t < TP * TZ * 32; t += blockDim.x) {
            const int lane = t & 31, tile = t >> 5;
            const int p = (tile / TZ) * 4 + (lane >> 3), z = (tile % TZ) * 8 + (lane & 7), y0 = 2 * p;
            if (p >= NP || z >= D) continue;
            float v0[NCH], v1[NCH];
            sample_a<MODE, NCH>(a, Fr, b, x, y0, z, v0);
            if (y0 + 1 < D) {
                sample_a<MODE, NCH>(a, Fr, b, x, y0 + 1, z, v1);
            } else {
#pragma unroll
                for (int c = 0; c < NCH; ++c) v1[c] = 0.f;
            }
#pragma unroll
            for (int c = 0; c < NCH; ++c)
                if (c >= c0 && c < c0 + cn) plane[(c - c0) * PS + 2 * p * Hp + z] = make_float2(v0[c], v1[c]);
        }
        __syncthreads();
        // z step 1, in place: items (c, j2, p), p fastest
        for (int t = threadIdx.x; t < cn * N2 * NP; t += blockDim.x) {
            const int p = t % NP, cj = t / NP, j2 = cj % N2, c = cj / N2;
            float2 *line = plane + c * PS + 2 * p * Hp;
            float2 v[N1];
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1) v[j1] = line[j2 + N2 * j1];
            rdft<N1, false>(v);
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) line[j2 + N2 * k1] = (k1 && j2) ? cmul(v[k1], twn[j2 * k1]) : v[k1];
        }
        __syncthreads();
        // z step 2 + unpack into rows (2p, 2p+1), which hold line p itself: items
        // (line, q), q in [0, N1/2]; each round covers whole lines and reads
        // everything before it writes
        {
            constexpr int NQ = N1 / 2 + 1;
            const int per_round = ((int)blockDim.x / NQ) * NQ;
            const int items = cn * NP * NQ;
            for (int base = 0; base < items; base += per_round) {
                const int t = base + (int)threadIdx.x;
                const bool on = (int)threadIdx.x < per_round && t < items;
                const int q = t % NQ, cp = t / NQ, p = cp % NP, c = cp / NP;
                const int q2 = (N1 - q) % N1;
                float2 u[N2], w2[N2];
                float2 *line = plane + c * PS + 2 * p * Hp;
                if (on) {
#pragma unroll
                    for (int j2 = 0; j2 < N2; ++j2) u[j2] = line[N2 * q + j2];
                    rdft<N2, false>(u);
#pragma unroll
                    for (int j2 = 0; j2 < N2; ++j2) w2[j2] = line[N2 * q2 + j2];
                    rdft<N2, false>(w2);
                }
                __syncthreads();
                if (on) {
                    const int y = 2 * p;
                    float2 *row0 = plane + c * PS + y * Hp;
                    float2 *row1 = row0 + Hp;
#pragma unroll
                    for (int k2 = 0; k2 < N2; ++k2) {
                        const int k = q + N1 * k2;
                        if (k < H) {
                            float2 A, B;
                            unpack_pair(u[k2], (q == 0) ? u[(N2 - k2) % N2] : w2[N2 - 1 - k2], A, B);
                            row0[k] = A;
                            row1[k] = (y + 1 < D) ? B : make_float2(0.f, 0.f);
                        }
                        if (q != 0 && q2 != q) {
                            const int kb = q2 + N1 * k2;
                            if (kb < H) {
                                float2 A, B;
                                unpack_pair(w2[k2], u[N2 - 1 - k2], A, B);
                                row0[kb] = A;
                                row1[kb] = (y + 1 < D) ? B : make_float2(0.f, 0.f);
                            }
                        }
                    }
                }
                __syncthreads();
            }
        }
        // y step 1, in place: items (c, j2, kz), kz fastest
        for (int t = threadIdx.x; t < cn * N2 * H; t += blockDim.x) {
            const int kz = t % H, cj = t / H, j2 = cj % N2, c = cj / N2;
            float2 *col = plane + c * PS + kz;
            float2 v[N1];
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1) v[j1] = col[(j2 + N2 * j1) * Hp];
            rdft<N1, false>(v);
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) col[(j2 + N2 * k1) * Hp] = (k1 && j2) ? cmul(v[k1], twn[j2 * k1]) : v[k1];
        }
        __syncthreads();
        // y step 2: items (c, k1, kz), kz fastest -> S rows ky = k1 + N1 k2
        for (int t = threadIdx.x; t < cn * N1 * H; t += blockDim.x) {
            const int kz = t % H, ck = t / H, k1 = ck % N1, c = ck / N1;
            const float2 *col = plane + c * PS + kz;
            float2 u[N2];
#pragma unroll
            for (int j2 = 0; j2 < N2; ++j2) u[j2] = col[(N2 * k1 + j2) * Hp];
            rdft<N2, false>(u);
            float2 *dst = a.S + (((size_t)b * NCH + c0 + c) * D + x) * (size_t)D * H + kz;
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) dst[(size_t)(k1 + N1 * k2) * H] = u[k2];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Pass A for sides up to 32 with whole lines in registers: PL x-planes per
// CTA; one packed z line per thread (DFT + unpack in registers), then one y
// column per thread (DFT in registers, straight to S).
constexpr int kLinePlanes = 1;     // x-planes per CTA of the whole-line pass A
constexpr int kLineAThreads = 64;   // its block size (measured: 64 threads, 1 plane beat 128 and 256 threads, 2 planes)

template <int D>
struct LineGeom {
    static constexpr int H = D / 2 + 1, NP = (D + 1) / 2, Hp = H | 1;
    static constexpr int LS = 2 * Hp + 1;   // packed-line stride (odd)
    static constexpr int PS = NP * LS;      // plane stride per channel
};
template <int D, int NCH, int PL>
__host__ __device__ inline size_t smem_ra_line() {
    return 64 + (size_t)PL * NCH * LineGeom<D>::PS * sizeof(float2);
}

template <int MODE, int NCH, int N1, int N2, int PL>
__global__ void __launch_bounds__(kLineAThreads, 8) k_rpass_a_line(const PassA2 a) {
    constexpr int D = N1 * N2;
    using L = LineGeom<D>;
    constexpr int H = L::H, NP = L::NP, Hp = L::Hp, LS = L::LS, PS = L::PS;
    extern __shared__ __align__(16) unsigned char smem[];
    float *F = (float *)smem;
    float2 *buf = (float2 *)(smem + 64);   // [PL][NCH][NP][LS]
    const int x0 = blockIdx.x * PL, b = blockIdx.y, r = a.r0 + b;
    if (threadIdx.x < 9) F[threadIdx.x] = a.rotmats[(size_t)r * 9 + threadIdx.x];
    if (x0 == 0 && threadIdx.x < a.nscore) a.keys[(size_t)r * a.nscore + threadIdx.x] = 0ull;
    __syncthreads();
    float Fr[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Fr[i] = F[i];
    // gather: each warp covers a tile of 4 packed lines x 8 z of one plane
    constexpr int TP = (NP + 3) / 4, TZ = (D + 7) / 8;
    for (int t = threadIdx.x; t < PL * TP * TZ * 32; t += blockDim.x) {
        const int lane = t & 31, tile = t >> 5;
        const int pl = tile / (TP * TZ), tt = tile % (TP * TZ);
        const int p = (tt / TZ) * 4 + (lane >> 3), z = (tt % TZ) * 8 + (lane & 7), y0 = 2 * p;
        const int x = x0 + pl;
        if (p >= NP || z >= D || x >= D) continue;
        float v0[NCH], v1[NCH];
        sample_a_ct<MODE, NCH, D>(a, Fr, b, x, y0, z, v0);
        if (y0 + 1 < D) {
            sample_a_ct<MODE, NCH, D>(a, Fr, b, x, y0 + 1, z, v1);
        } else {
#pragma unroll
            for (int c = 0; c < NCH; ++c) v1[c] = 0.f;
        }
#pragma unroll
        for (int c = 0; c < NCH; ++c) buf[(pl * NCH + c) * PS + p * LS + z] = make_float2(v0[c], v1[c]);
    }
    __syncthreads();
    // z: one packed line per thread; DFT and unpack into rows 2p (offset 0)
    // and 2p + 1 (offset Hp) of the line's own storage
    for (int t = threadIdx.x; t < PL * NCH * NP; t += blockDim.x) {
        const int p = t % NP, pc = t / NP;
        if (x0 + pc / NCH >= D) continue;
        float2 *line = buf + pc * PS + p * LS;
        float2 v[D];
#pragma unroll
        for (int j = 0; j < D; ++j) v[j] = line[j];
        rdft<D, false, true>(v);   // largest prime power first (faster here)
        const bool two = 2 * p + 1 < D;
#pragma unroll
        for (int k = 0; k < H; ++k) {
            float2 A, B;
            unpack_pair(v[k], v[(D - k) % D], A, B);
            line[k] = A;
            line[Hp + k] = two ? B : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();
    // y: one column (plane, channel, kz) per thread -> S rows ky
    for (int t = threadIdx.x; t < PL * NCH * H; t += blockDim.x) {
        const int kz = t % H, pc = t / H, pl = pc / NCH, c = pc % NCH, x = x0 + pl;
        if (x >= D) continue;
        const float2 *pln = buf + pc * PS + kz;
        float2 v[D];
#pragma unroll
        for (int y = 0; y < D; ++y) v[y] = pln[(y >> 1) * LS + (y & 1) * Hp];
        rdft<D, false, true>(v);   // largest prime power first (faster here)
        float2 *dst = a.S + (((size_t)b * NCH + c) * D + x) * (size_t)D * H + kz;
#pragma unroll
        for (int ky = 0; ky < D; ++ky) dst[(size_t)ky * H] = v[ky];
    }
}

// ---------------------------------------------------------------------------
template <int NCH, int NGRP, int N1, int N2>
__global__ void __launch_bounds__(256) k_rpass_b(const PassB2 a) {
    using G = RGeom<N1, N2>;
    constexpr int D = G::D, H = G::H, dH = D * H;
    extern __shared__ __align__(16) unsigned char smem[];
    const int W = a.W, j0 = blockIdx.x * W, b = blockIdx.y;
    float2 *twn = (float2 *)smem;
    float2 *buf = (float2 *)(smem + align16(D * sizeof(float2)));   // [NCH][D][W]
    float2 *pbuf = buf + (size_t)NCH * D * W;                         // [NGRP][D][W]
    twiddles_n(D, twn);
    __syncthreads();
    const float2 *src = a.S + (size_t)b * NCH * D * dH;
    // forward step 1: items (c, j2, w) from global
    for (int t = threadIdx.x; t < NCH * N2 * W; t += blockDim.x) {
        const int w = t % W, cj = t / W, j2 = cj % N2, c = cj / N2, j = j0 + w;
        float2 v[N1];
        const float2 *s = src + (size_t)c * D * dH + j;
#pragma unroll
        for (int j1 = 0; j1 < N1; ++j1) v[j1] = j < dH ? s[(size_t)(j2 + N2 * j1) * dH] : make_float2(0.f, 0.f);
        rdft<N1, false>(v);
        float2 *col = buf + (size_t)c * D * W + w;
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) col[(j2 + N2 * k1) * W] = (k1 && j2) ? cmul(v[k1], twn[j2 * k1]) : v[k1];
    }
    __syncthreads();
    // forward step 2, product with conj(T), group sums, inverse step 2 (over
    // k2) with conjugate twiddles into pbuf rows k1 + N1 j2: items (k1, w)
    for (int t = threadIdx.x; t < N1 * W; t += blockDim.x) {
        const int w = t % W, k1 = t / W, j = j0 + w;
        float2 acc[NGRP][N2];
#pragma unroll
        for (int g = 0; g < NGRP; ++g)
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) acc[g][k2] = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            const float2 *col = buf + (size_t)c * D * W + w;
            float2 u[N2];
#pragma unroll
            for (int j2 = 0; j2 < N2; ++j2) u[j2] = col[(N2 * k1 + j2) * W];
            rdft<N2, false>(u);
            const int g = (NGRP == 2 && c >= 3) ? 1 : 0;
            if (j < dH) {
                const float2 *T = a.T + (size_t)c * D * dH + j;
#pragma unroll
                for (int k2 = 0; k2 < N2; ++k2)
                    acc[g][k2] = cadd(acc[g][k2], cmul(T[(size_t)(k1 + N1 * k2) * dH], u[k2]));
            }
        }
#pragma unroll
        for (int g = 0; g < NGRP; ++g) {
            rdft<N2, true>(acc[g]);
            float2 *col = pbuf + (size_t)g * D * W + w;
#pragma unroll
            for (int j2 = 0; j2 < N2; ++j2)
                col[(k1 + N1 * j2) * W] = (k1 && j2) ? cmulc(acc[g][j2], twn[j2 * k1]) : acc[g][j2];
        }
    }
    __syncthreads();
    // inverse step 1: items (g, j2, w) -> U rows x = j2 + N2 j1
    float2 *dst = a.U + (size_t)b * NGRP * D * dH;
    for (int t = threadIdx.x; t < NGRP * N2 * W; t += blockDim.x) {
        const int w = t % W, gj = t / W, j2 = gj % N2, g = gj / N2, j = j0 + w;
        const float2 *col = pbuf + (size_t)g * D * W + w;
        float2 v[N1];
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1] = col[(k1 + N1 * j2) * W];
        rdft<N1, true>(v);
        if (j < dH)
#pragma unroll
            for (int j1 = 0; j1 < N1; ++j1) dst[((size_t)g * D + j2 + N2 * j1) * dH + j] = v[j1];
    }
}

// ---------------------------------------------------------------------------
// Pass B for sides up to 32 with one score group: one spectrum column j =
// ky H + kz per thread, whole x lines in registers -- for every channel the
// forward x DFT of its S column, times conj(T) added into the column's sum,
// then the inverse x DFT of the sum straight to U.  No shared memory.
constexpr int kLineBThreads = 64;  // fewer idle threads in the last CTA of each rotation (measured: 64 beat 128, 256)

template <int NCH, int N1, int N2>
__global__ void __launch_bounds__(kLineBThreads) k_rpass_b_line(const PassB2 a) {
    constexpr int D = N1 * N2, H = D / 2 + 1, dH = D * H;
    const int j = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (j >= dH) return;
    const float2 *src = a.S + (size_t)b * NCH * D * dH + j;
    float2 acc[D];
#pragma unroll
    for (int k = 0; k < D; ++k) acc[k] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int c = 0; c < NCH; ++c) {
        float2 v[D];
#pragma unroll
        for (int x = 0; x < D; ++x) v[x] = src[(size_t)(c * D + x) * dH];
        rdft<D, false>(v);
        const float2 *T = a.T + (size_t)c * D * dH + j;
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k] = cadd(acc[k], cmul(T[(size_t)k * dH], v[k]));
    }
    rdft<D, true>(acc);
    float2 *dst = a.U + (size_t)b * D * dH + j;
#pragma unroll
    for (int x = 0; x < D; ++x) dst[(size_t)x * dH] = acc[x];
}

// ---------------------------------------------------------------------------
template <int NGRP, int SC, int N1, int N2>
__global__ void __launch_bounds__(256) k_rpass_c(const PassC2 a) {
    using G = RGeom<N1, N2>;
    constexpr int D = G::D, H = G::H, NP = G::NP, Zp = G::Zp, Hp = G::Hp;
    extern __shared__ __align__(16) unsigned char smem[];
    const int x = blockIdx.x, b = blockIdx.y, r = a.r0 + b;
    float2 *twn = (float2 *)smem;
    float2 *plane = (float2 *)(smem + align16(D * sizeof(float2)));   // [NGRP][D][Hp]
    float2 *rows = plane + (size_t)NGRP * D * Hp;                      // [NGRP][D][Hp]
    float2 *zbuf = plane;   // [NGRP][NP][Zp], NP * Zp <= D * Hp; plane is dead by then
    unsigned long long *red = (unsigned long long *)(rows + (size_t)NGRP * D * Hp);
    twiddles_n(D, twn);
    __syncthreads();
    // inverse y step 2 from U: items (g, k1, kz) -> plane rows k1 + N1 j2
    for (int t = threadIdx.x; t < NGRP * N1 * H; t += blockDim.x) {
        const int kz = t % H, gk = t / H, k1 = gk % N1, g = gk / N1;
        const float2 *src = a.U + (((size_t)b * NGRP + g) * D + x) * (size_t)D * H + kz;
        float2 u[N2];
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) u[k2] = src[(size_t)(k1 + N1 * k2) * H];
        rdft<N2, true>(u);
        float2 *col = plane + (size_t)g * D * Hp + kz;
#pragma unroll
        for (int j2 = 0; j2 < N2; ++j2) col[(k1 + N1 * j2) * Hp] = (k1 && j2) ? cmulc(u[j2], twn[j2 * k1]) : u[j2];
    }
    __syncthreads();
    // inverse y step 1: items (g, j2, kz) -> rows y = j2 + N2 j1 (second buffer)
    for (int t = threadIdx.x; t < NGRP * N2 * H; t += blockDim.x) {
        const int kz = t % H, gj = t / H, j2 = gj % N2, g = gj / N2;
        const float2 *col = plane + (size_t)g * D * Hp + kz;
        float2 v[N1];
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1] = col[(k1 + N1 * j2) * Hp];
        rdft<N1, true>(v);
        float2 *out = rows + (size_t)g * D * Hp + kz;
#pragma unroll
        for (int j1 = 0; j1 < N1; ++j1) out[(j2 + N2 * j1) * Hp] = v[j1];
    }
    __syncthreads();
    // z: pack rows (2p, 2p+1) into full lines (Hermitian completion, DC and
    // Nyquist imaginary parts dropped), inverse step 2: items (g, p, k1)
    for (int t = threadIdx.x; t < NGRP * NP * N1; t += blockDim.x) {
        const int k1 = t % N1, gp = t / N1, p = gp % NP, g = gp / NP, y = 2 * p;
        const float2 *pl = rows + (size_t)g * D * Hp;
        const bool hb = y + 1 < D;
        float2 u[N2];
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            const int k = k1 + N1 * k2;
            float2 Z;
            if (k < H) {
                float2 A = pl[y * Hp + k], B = hb ? pl[(y + 1) * Hp + k] : make_float2(0.f, 0.f);
                if (k == 0 || 2 * k == D) { A.y = 0.f; B.y = 0.f; }
                Z = make_float2(A.x - B.y, A.y + B.x);
            } else {
                const int kk = D - k;
                const float2 A = pl[y * Hp + kk], B = hb ? pl[(y + 1) * Hp + kk] : make_float2(0.f, 0.f);
                Z = make_float2(A.x + B.y, B.x - A.y);
            }
            u[k2] = Z;
        }
        rdft<N2, true>(u);
        float2 *zl = zbuf + ((size_t)g * NP + p) * Zp;
#pragma unroll
        for (int j2 = 0; j2 < N2; ++j2) zl[k1 + N1 * j2] = (k1 && j2) ? cmulc(u[j2], twn[j2 * k1]) : u[j2];
    }
    __syncthreads();
    // inverse z step 1 + scores: items (p, j2) over every group
    unsigned long long best[3] = {0ull, 0ull, 0ull};
    for (int t = threadIdx.x; t < NP * N2; t += blockDim.x) {
        const int p = t % NP, j2 = t / NP;
        float2 v0[N1], v1[N1];
        const float2 *zl0 = zbuf + (size_t)p * Zp;
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v0[k1] = zl0[k1 + N1 * j2];
        rdft<N1, true>(v0);
        if (NGRP == 2) {
            const float2 *zl1 = zbuf + ((size_t)NP + p) * Zp;
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) v1[k1] = zl1[k1 + N1 * j2];
            rdft<N1, true>(v1);
        }
#pragma unroll
        for (int j1 = 0; j1 < N1; ++j1) {
            const int z = j2 + N2 * j1;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int y = 2 * p + half;
                if (y >= D) break;
                const uint32_t lin = (uint32_t)((x * D + y) * D + z);
                const float s0 = half ? v0[j1].y : v0[j1].x;
                best[0] = max(best[0], make_key(s0, lin));
                if (SC >= 2) {
                    const float s1 = half ? v1[j1].y : v1[j1].x;
                    best[1] = max(best[1], make_key(s1, lin));
                    if (SC == 3) {
                        const float sv = __fdiv_rn(__fsub_rn(s0, a.mix.vave), a.mix.vstd);
                        const float sp = __fdiv_rn(__fsub_rn(s1, a.mix.pave), a.mix.pstd);
                        const float m =
                            __fadd_rn(__fmul_rn(a.mix.one_minus_alpha, sv), __fmul_rn(a.mix.alpha, sp));
                        best[2] = max(best[2], make_key(m, lin));
                    }
                }
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int s = 0; s < SC; ++s) {
        const unsigned long long v = warp_max_u64(best[s]);
        if (lane == 0) red[s * 32 + warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < SC) {
        unsigned long long v = 0ull;
        for (int w2 = 0; w2 < nw; ++w2) v = max(v, red[threadIdx.x * 32 + w2]);
        atomicMax(&a.keys[(size_t)r * a.nscore + threadIdx.x], v);
    }
}

// ---------------------------------------------------------------------------
// Pass C for sides up to 32 with one score group and one score: several
// x-planes per CTA, whole lines in registers.  Phase y: one (plane, kz) column
// per thread, its D values read from U, inverse DFT, rows y to shared memory;
// phase z: one (plane, row pair) per thread, the two rows' half spectra packed
// into one complex line (Hermitian completion, DC and Nyquist imaginary parts
// dropped), inverse DFT (real part row 2p, imaginary part row 2p + 1), the
// scores' first-index argmax keys; one barrier between the phases.  With
// several planes per CTA both phases keep most threads busy.
// Used where 4 planes divide the side (measured: side 28 0.078 -> 0.056 us per
// rotation, side 32 0.096 -> 0.079 against the two-step pass C; at side 30 it
// took 0.104-0.111 with 2 to 6 planes per CTA against the two-step's 0.093, so
// side 30 keeps the two-step kernel).  Threads: the y phase's columns rounded
// up to whole warps.
template <int D> __host__ __device__ constexpr int line_c_planes() { return 4; }
template <int D> __host__ __device__ constexpr bool line_c_used() { return D <= 32 && D % line_c_planes<D>() == 0; }
template <int D> __host__ __device__ constexpr int line_c_threads() {
    return (line_c_planes<D>() * (D / 2 + 1) + 31) / 32 * 32 > 128 ? 128
                                                                   : (line_c_planes<D>() * (D / 2 + 1) + 31) / 32 * 32;
}

template <int D, int PL>
__host__ __device__ constexpr size_t smem_rc_line() {
    return (size_t)PL * D * (D / 2 + 1) * sizeof(float2) + 2 * sizeof(unsigned long long);
}

template <int N1, int N2>
__global__ void __launch_bounds__(line_c_threads<N1 * N2>()) k_rpass_c_line(const PassC2 a) {
    constexpr int D = N1 * N2, H = D / 2 + 1, NP = (D + 1) / 2, PL = line_c_planes<D>();
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *rows = (float2 *)smem;   // [PL][D][H]
    unsigned long long *red = (unsigned long long *)(rows + (size_t)PL * D * H);   // [2]
    const int x0 = blockIdx.x * PL, b = blockIdx.y, r = a.r0 + b;
    if (threadIdx.x < 2) red[threadIdx.x] = 0ull;
    // y: inverse DFT of every (plane, kz) column
    for (int t = threadIdx.x; t < PL * H; t += blockDim.x) {
        const int pl = t / H, kz = t - pl * H, x = x0 + pl;
        if (x >= D) continue;
        const float2 *src = a.U + ((size_t)b * D + x) * (size_t)D * H + kz;
        float2 v[D];
#pragma unroll
        for (int ky = 0; ky < D; ++ky) v[ky] = src[(size_t)ky * H];
        rdft<D, true>(v);
        float2 *dst = rows + (size_t)pl * D * H + kz;
#pragma unroll
        for (int y = 0; y < D; ++y) dst[(size_t)y * H] = v[y];
    }
    __syncthreads();
    // z: row pairs (2p, 2p + 1), inverse complex DFT, scores
    unsigned long long best = 0ull;
    for (int t = threadIdx.x; t < PL * NP; t += blockDim.x) {
        const int pl = t / NP, p = t - pl * NP, x = x0 + pl, y = 2 * p;
        if (x >= D) continue;
        const float2 *r0 = rows + ((size_t)pl * D + y) * H;
        const bool hb = y + 1 < D;
        const float2 *r1 = r0 + H;
        float2 u[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            if (k < H) {
                float2 A = r0[k], B = hb ? r1[k] : make_float2(0.f, 0.f);
                if (k == 0 || 2 * k == D) { A.y = 0.f; B.y = 0.f; }
                u[k] = make_float2(A.x - B.y, A.y + B.x);
            } else {
                const float2 A = r0[D - k], B = hb ? r1[D - k] : make_float2(0.f, 0.f);
                u[k] = make_float2(A.x + B.y, B.x - A.y);
            }
        }
        rdft<D, true>(u);
        const uint32_t base = (uint32_t)((x * D + y) * D);
#pragma unroll
        for (int z = 0; z < D; ++z) {
            best = max(best, make_key(u[z].x, base + z));
            if (hb) best = max(best, make_key(u[z].y, base + D + z));
        }
    }
    best = warp_max_u64(best);
    if ((threadIdx.x & 31) == 0) atomicMax(&red[0], best);
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(&a.keys[(size_t)r * a.nscore], red[0]);
}

// ---- one compiled side of the register passes, as vesper_search.cu calls it ----
struct RegEntry {
    int mode, d;
    size_t (*sa)(int cc);
    size_t (*sb)(int nch, int ngrp, int W);
    size_t (*sc)(int ngrp);
    void (*a)(dim3, int, size_t, cudaStream_t, const PassA2 &);
    void (*b)(dim3, int, size_t, cudaStream_t, const PassB2 &);
    void (*c)(dim3, int, size_t, cudaStream_t, const PassC2 &, int nscore);
};

template <int MODE, int NCH, int NGRP, int N1, int N2>
struct RegPath {
    static void a(dim3 g, int T, size_t s, cudaStream_t st, const PassA2 &p) {
        if constexpr (N1 * N2 <= 32 && MODE != VESPER_MODE_LAPLACIAN) {
            // whole lines in registers, kLinePlanes x-planes per CTA
            constexpr int PL = kLinePlanes;
            const size_t sl = smem_ra_line<N1 * N2, NCH, PL>();
            allow_smem(k_rpass_a_line<MODE, NCH, N1, N2, PL>, sl);
            k_rpass_a_line<MODE, NCH, N1, N2, PL><<<dim3((N1 * N2 + PL - 1) / PL, g.y), kLineAThreads, sl, st>>>(p);
        } else {
            allow_smem(k_rpass_a<MODE, NCH, N1, N2>, s);
            k_rpass_a<MODE, NCH, N1, N2><<<g, T, s, st>>>(p);
        }
    }
    static void b(dim3 g, int T, size_t s, cudaStream_t st, const PassB2 &p) {
        if constexpr (N1 * N2 <= 32 && NGRP == 1) {
            constexpr int dH = N1 * N2 * (N1 * N2 / 2 + 1);
            k_rpass_b_line<NCH, N1, N2><<<dim3((dH + kLineBThreads - 1) / kLineBThreads, g.y), kLineBThreads, 0,
                                          st>>>(p);
        } else {
            allow_smem(k_rpass_b<NCH, NGRP, N1, N2>, s);
            k_rpass_b<NCH, NGRP, N1, N2><<<g, T, s, st>>>(p);
        }
    }
    static void c(dim3 g, int T, size_t s, cudaStream_t st, const PassC2 &p, int nscore) {
        if constexpr (NGRP == 1 && line_c_used<N1 * N2>()) {
            constexpr int D = N1 * N2, PL = line_c_planes<D>();
            constexpr size_t sl = smem_rc_line<D, PL>();
            allow_smem(k_rpass_c_line<N1, N2>, sl);
            k_rpass_c_line<N1, N2><<<dim3((D + PL - 1) / PL, g.y), line_c_threads<D>(), sl, st>>>(p);
        } else if constexpr (NGRP == 1) {
            // sides up to 32: a plane's steps have 45 to 160 items, so 96 threads
            // per plane leave fewer idle (measured at side 30: 0.096 us per rotation
            // with 64 threads against 0.123 with 256, 0.101 with 128; then 0.089
            // with 96 against 0.092 with 64 and 0.096 with 32)
            const int t = N1 * N2 <= 32 ? 96 : T;
            allow_smem(k_rpass_c<1, 1, N1, N2>, s);
            k_rpass_c<1, 1, N1, N2><<<g, t, s, st>>>(p);
        } else if (nscore == 1) {
            allow_smem(k_rpass_c<NGRP, 1, N1, N2>, s);
            k_rpass_c<NGRP, 1, N1, N2><<<g, T, s, st>>>(p);
        } else if (nscore == 2) {
            allow_smem(k_rpass_c<NGRP, 2, N1, N2>, s);
            k_rpass_c<NGRP, 2, N1, N2><<<g, T, s, st>>>(p);
        } else {
            allow_smem(k_rpass_c<NGRP, 3, N1, N2>, s);
            k_rpass_c<NGRP, 3, N1, N2><<<g, T, s, st>>>(p);
        }
    }
    static RegEntry entry() {
        return RegEntry{MODE, N1 * N2, &smem_ra<N1, N2>, &smem_rb<N1, N2>, &smem_rc<N1, N2>, &a, &b, &c};
    }
};

// Lookups of the tables in vesper_regsearch_{a,b,c}.cu.
const RegEntry *find_reg_a(int mode, int d);
const RegEntry *find_reg_b(int mode, int d);
const RegEntry *find_reg_c(int mode, int d);

}  // namespace vg
