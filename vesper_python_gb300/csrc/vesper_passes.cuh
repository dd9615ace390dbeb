// The three per-batch passes of the rotational search (included by
// vesper_search.cu).
//
//   pack   (once per call)  query fields -> float4 source: (vx, vy, vz, mask) for
//                           V / prob, (mode value, 0, 0, mask) for O/C/P/L, plus
//                           float4 probabilities for prob; mask = data != 0
//   A  k_pass_a   grid (d, nb)       rotate one x plane of C channels, z R2C
//                                    (two real rows per complex line), y FFT -> S
//   B  k_pass_b   grid (Nh/W, nb)    x FFT, * conj target, sum per group,
//                                    inverse x FFT -> U
//   C  k_pass_c   grid (d, nb)       inverse y, inverse z (C2R, row pairs),
//                                    scores, first-index argmax -> keys
//
// Every FFT runs over all lines of a plane at once with the division-free
// stage tables of vesper_fft.cuh; row strides are padded to odd element
// counts so that lines handled by neighbouring threads fall in distinct
// shared-memory banks.
#pragma once

#include "vesper_sample.cuh"

namespace vg {

// ---- shared-memory layout helpers ---------------------------------------------
struct PlaneGeom {
    int d, H, npairs, Zp, Hp;   // npairs = (d+1)/2 packed z lines; padded strides
};
__host__ __device__ inline PlaneGeom plane_geom(int d) {
    PlaneGeom g;
    g.d = d;
    g.H = d / 2 + 1;
    g.npairs = (d + 1) / 2;
    g.Zp = odd_up(d);
    g.Hp = odd_up(g.H);
    return g;
}
__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }
// common head: tw (float2 d) | rev (short d) | off, two (short ntab each)
__host__ __device__ inline size_t smem_head(int d, int ntab) {
    return align16((size_t)d * sizeof(float2)) + align16((size_t)d * sizeof(short)) +
           2 * align16((size_t)ntab * sizeof(short));
}
struct Head {
    float2 *tw;
    short *rev, *off, *two;
    unsigned char *rest;
};
__device__ __forceinline__ Head carve_head(unsigned char *smem, int d, int ntab) {
    Head h;
    h.tw = (float2 *)smem;
    h.rev = (short *)(smem + align16((size_t)d * sizeof(float2)));
    h.off = (short *)((unsigned char *)h.rev + align16((size_t)d * sizeof(short)));
    h.two = (short *)((unsigned char *)h.off + align16((size_t)ntab * sizeof(short)));
    h.rest = (unsigned char *)h.two + align16((size_t)ntab * sizeof(short));
    return h;
}
__device__ __forceinline__ void init_head(const FftPlan &P, const Head &h) {
    fft_tables(P, h.rev, h.tw);
    fft_stage_tables(P, h.off, h.two);
}

// ---- pass A -------------------------------------------------------------------
struct PassA2 {
    Src src;
    const float *rotmats;
    int r0, nch, cchunk, nscore;
    FftPlan P;
    float2 *S;                    // [batch][nch][d][d][H]
    unsigned long long *keys;     // [nrot][nscore]
    const double *rd;             // Laplacian mode: [batch][d^3] rotated density, or null
};

// Pass-A sample of rotation b of the batch: the Laplacian mode reads the
// batch's gathered density when it is there, every other mode gathers.
template <int MODE, int NCH>
__device__ __forceinline__ void sample_a(const PassA2 &a, const float (&F)[9], int b, int x, int y, int z,
                                         float *out) {
    if constexpr (MODE == VESPER_MODE_LAPLACIAN) {
        if (a.rd) {
            const int d = a.src.d;
            out[0] = lap_from_rd(a.rd + (size_t)b * d * d * d, d, x, y, z);
            return;
        }
    }
    sample_fast<MODE>(a.src, F, x, y, z, out);
}

// sample_a for a side known at compile time (sample_ct in modes V/O/C/P).
template <int MODE, int NCH, int D>
__device__ __forceinline__ void sample_a_ct(const PassA2 &a, const float (&F)[9], int b, int x, int y, int z,
                                            float *out) {
    if constexpr (MODE == VESPER_MODE_VEC || MODE == VESPER_MODE_OVERLAP || MODE == VESPER_MODE_CC ||
                  MODE == VESPER_MODE_PCC)
        sample_ct<MODE, D>(a.src, F, x, y, z, out);
    else
        sample_a<MODE, NCH>(a, F, b, x, y, z, out);
}

__host__ __device__ inline size_t smem_a2(int d, int ntab, int cchunk) {
    const PlaneGeom g = plane_geom(d);
    return smem_head(d, ntab) + align16(16 * sizeof(float)) +
           (size_t)cchunk * ((size_t)g.npairs * g.Zp + (size_t)d * g.Hp) * sizeof(float2);
}

template <int MODE, int NCH>
__global__ void __launch_bounds__(512) k_pass_a(const PassA2 a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const PlaneGeom g = plane_geom(a.src.d);
    const int d = g.d, H = g.H, np = g.npairs, Zp = g.Zp, Hp = g.Hp;
    const int x = blockIdx.x, b = blockIdx.y, r = a.r0 + b;
    const Head h = carve_head(smem, d, a.P.ntab);
    float *F = (float *)h.rest;
    float2 *zbuf = (float2 *)(h.rest + align16(16 * sizeof(float)));
    float2 *plane = zbuf + (size_t)a.cchunk * np * Zp;
    init_head(a.P, h);
    if (threadIdx.x < 9) F[threadIdx.x] = a.rotmats[(size_t)r * 9 + threadIdx.x];
    if (x == 0 && threadIdx.x < a.nscore) a.keys[(size_t)r * a.nscore + threadIdx.x] = 0ull;
    __syncthreads();
    float Fr[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Fr[i] = F[i];
    for (int c0 = 0; c0 < NCH; c0 += a.cchunk) {
        const int cn = min(a.cchunk, NCH - c0);
        // gather two rows (2p, 2p+1) per item into packed z lines, digit-reversed z
        for (Walk2 w(d); w.o < np; w.next()) {
            const int p = w.o, z = w.i, y0 = 2 * p;
            float v0[NCH], v1[NCH];
            sample_a<MODE, NCH>(a, Fr, b, x, y0, z, v0);
            if (y0 + 1 < d) {
                sample_a<MODE, NCH>(a, Fr, b, x, y0 + 1, z, v1);
            } else {
#pragma unroll
                for (int c = 0; c < NCH; ++c) v1[c] = 0.f;
            }
            const int rz = h.rev[z];
#pragma unroll
            for (int c = 0; c < NCH; ++c)
                if (c >= c0 && c < c0 + cn) zbuf[((c - c0) * np + p) * Zp + rz] = make_float2(v0[c], v1[c]);
        }
        __syncthreads();
        fft_lines<false>(zbuf, line_slot(cn * np, cn * np, 0, Zp), 1, a.P, h.off, h.two, h.tw);
        // unpack the two half spectra into rows rev(y) of the plane
        for (int c = 0; c < cn; ++c) {
            const float2 *zl = zbuf + (size_t)c * np * Zp;
            float2 *pl = plane + (size_t)c * d * Hp;
            for (Walk2 w(H); w.o < np; w.next()) {
                const int p = w.o, k = w.i, y = 2 * p;
                float2 A, B;
                unpack_pair(zl[p * Zp + k], zl[p * Zp + (k == 0 ? 0 : d - k)], A, B);
                pl[h.rev[y] * Hp + k] = A;
                if (y + 1 < d) pl[h.rev[y + 1] * Hp + k] = B;
            }
        }
        __syncthreads();
        fft_lines<false>(plane, line_slot(cn * H, H, d * Hp, 1), Hp, a.P, h.off, h.two, h.tw);
        for (int c = 0; c < cn; ++c) {
            float2 *dst = a.S + (((size_t)b * NCH + c0 + c) * d + x) * (size_t)d * H;
            const float2 *pl = plane + (size_t)c * d * Hp;
            for (Walk2 w(H); w.o < d; w.next()) dst[w.o * H + w.i] = pl[w.o * Hp + w.i];
        }
        __syncthreads();
    }
}

// ---- pass B -------------------------------------------------------------------
struct PassB2 {
    const float2 *S;
    const float2 *T;     // [nch][d][d][H] conj target spectrum
    float2 *U;           // [batch][ngrp][d][d][H]
    int d, nch, ngrp, split, W;
    FftPlan P;
};

// pass B on the tensor cores (split-BF16 DFTs; vesper_tcdft.cu), sides 32 and 64
bool tc_pass_b_supported(int d);
int tc_pass_b_wave(int d);   // rotations per full wave of its CTAs
int tc_pass_b(const PassB2 &a, int nb, int *err, cudaStream_t st, int stall = 0,
              uint64_t limit_ns = 200ull * 1000000);

__host__ __device__ inline size_t smem_b2(int d, int ntab, int nch, int ngrp, int W) {
    return smem_head(d, ntab) + (size_t)(nch + ngrp) * d * W * sizeof(float2);
}

#ifndef VG_PASS_TYPES_ONLY   // translation units other than vesper_search.cu need only the types
__global__ void __launch_bounds__(512) k_pass_b(const PassB2 a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int d = a.d, H = d / 2 + 1, dH = d * H, W = a.W;
    const int j0 = blockIdx.x * W, b = blockIdx.y;
    const Head h = carve_head(smem, d, a.P.ntab);
    float2 *buf = (float2 *)h.rest;
    float2 *pbuf = buf + (size_t)a.nch * d * W;
    init_head(a.P, h);
    __syncthreads();
    const float2 *src = a.S + (size_t)b * a.nch * d * dH;
    for (int c = 0; c < a.nch; ++c)
        for (Walk2 w(W); w.o < d; w.next()) {
            const int x = w.o, j = j0 + w.i;
            buf[((size_t)c * d + h.rev[x]) * W + w.i] =
                j < dH ? src[((size_t)c * d + x) * dH + j] : make_float2(0.f, 0.f);
        }
    __syncthreads();
    fft_lines<false>(buf, line_slot(a.nch * W, W, d * W, 1), W, a.P, h.off, h.two, h.tw);
    for (int g = 0; g < a.ngrp; ++g) {
        const int cb = g == 0 ? 0 : a.split, ce = g == 0 ? a.split : a.nch;
        for (Walk2 w(W); w.o < d; w.next()) {
            const int x = w.o, j = j0 + w.i;
            float2 acc = make_float2(0.f, 0.f);
            if (j < dH)
                for (int c = cb; c < ce; ++c)
                    acc = cadd(acc, cmul(a.T[((size_t)c * d + x) * dH + j], buf[((size_t)c * d + x) * W + w.i]));
            pbuf[((size_t)g * d + h.rev[x]) * W + w.i] = acc;
        }
    }
    __syncthreads();
    fft_lines<true>(pbuf, line_slot(a.ngrp * W, W, d * W, 1), W, a.P, h.off, h.two, h.tw);
    float2 *dst = a.U + (size_t)b * a.ngrp * d * dH;
    for (int g = 0; g < a.ngrp; ++g)
        for (Walk2 w(W); w.o < d; w.next()) {
            const int j = j0 + w.i;
            if (j < dH) dst[((size_t)g * d + w.o) * dH + j] = pbuf[((size_t)g * d + w.o) * W + w.i];
        }
}
#endif

// ---- pass C -------------------------------------------------------------------
struct PassC2 {
    const float2 *U;
    int d, ngrp, r0, nscore;
    FftPlan P;
    Mix mix;
    unsigned long long *keys;
};

__host__ __device__ inline size_t smem_c2(int d, int ntab, int ngrp) {
    const PlaneGeom g = plane_geom(d);
    return smem_head(d, ntab) + (size_t)ngrp * ((size_t)d * g.Hp + (size_t)g.npairs * g.Zp) * sizeof(float2) +
           3 * 32 * sizeof(unsigned long long);
}

template <int SC>
__global__ void __launch_bounds__(512) k_pass_c(const PassC2 a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const PlaneGeom g = plane_geom(a.d);
    const int d = g.d, H = g.H, np = g.npairs, Zp = g.Zp, Hp = g.Hp, ngrp = a.ngrp;
    const int x = blockIdx.x, b = blockIdx.y, r = a.r0 + b;
    const Head h = carve_head(smem, d, a.P.ntab);
    float2 *plane = (float2 *)h.rest;
    float2 *zbuf = plane + (size_t)ngrp * d * Hp;
    unsigned long long *red = (unsigned long long *)(zbuf + (size_t)ngrp * np * Zp);
    init_head(a.P, h);
    __syncthreads();
    for (int gi = 0; gi < ngrp; ++gi) {
        const float2 *src = a.U + (((size_t)b * ngrp + gi) * d + x) * (size_t)d * H;
        float2 *pl = plane + (size_t)gi * d * Hp;
        for (Walk2 w(H); w.o < d; w.next()) pl[h.rev[w.o] * Hp + w.i] = src[w.o * H + w.i];
    }
    __syncthreads();
    fft_lines<true>(plane, line_slot(ngrp * H, H, d * Hp, 1), Hp, a.P, h.off, h.two, h.tw);
    // pack row pairs (2p, 2p+1) into full-length lines: Z = A + iB, Hermitian
    // completion, DC / Nyquist imaginary parts dropped (C2R semantics)
    for (int gi = 0; gi < ngrp; ++gi) {
        const float2 *pl = plane + (size_t)gi * d * Hp;
        float2 *zl = zbuf + (size_t)gi * np * Zp;
        for (Walk2 w(d); w.o < np; w.next()) {
            const int p = w.o, k = w.i, y = 2 * p;
            const bool hb = y + 1 < d;
            float2 Z;
            if (k < H) {
                float2 A = pl[y * Hp + k], B = hb ? pl[(y + 1) * Hp + k] : make_float2(0.f, 0.f);
                if (k == 0 || 2 * k == d) { A.y = 0.f; B.y = 0.f; }
                Z = make_float2(A.x - B.y, A.y + B.x);
            } else {
                const int kk = d - k;
                const float2 A = pl[y * Hp + kk], B = hb ? pl[(y + 1) * Hp + kk] : make_float2(0.f, 0.f);
                Z = make_float2(A.x + B.y, B.x - A.y);
            }
            zl[p * Zp + h.rev[k]] = Z;
        }
    }
    __syncthreads();
    fft_lines<true>(zbuf, line_slot(ngrp * np, ngrp * np, 0, Zp), 1, a.P, h.off, h.two, h.tw);
    unsigned long long best[3] = {0ull, 0ull, 0ull};
    for (Walk2 w(d); w.o < np; w.next()) {
        const int p = w.o, z = w.i;
        const float2 z0 = zbuf[p * Zp + z];
        float2 z1 = make_float2(0.f, 0.f);
        if (SC >= 2) z1 = zbuf[(np + p) * Zp + z];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int y = 2 * p + half;
            if (y >= d) break;
            const uint32_t lin = (uint32_t)((x * d + y) * d + z);
            const float v0 = half ? z0.y : z0.x;
            best[0] = max(best[0], make_key(v0, lin));
            if (SC >= 2) {
                const float v1 = half ? z1.y : z1.x;
                best[1] = max(best[1], make_key(v1, lin));
                if (SC == 3) {
                    // find_best_trans_mixed (VESPER_1_prob_new.py:1534-1539), float32
                    const float sv = __fdiv_rn(__fsub_rn(v0, a.mix.vave), a.mix.vstd);
                    const float sp = __fdiv_rn(__fsub_rn(v1, a.mix.pave), a.mix.pstd);
                    const float m = __fadd_rn(__fmul_rn(a.mix.one_minus_alpha, sv), __fmul_rn(a.mix.alpha, sp));
                    best[2] = max(best[2], make_key(m, lin));
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

}  // namespace vg
