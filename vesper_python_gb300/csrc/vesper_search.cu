// Rotational FFT search: target spectra, batched rotate -> FFT -> correlate ->
// inverse FFT -> argmax, and the stable top-N.
//
// Data layout in HBM (per rotation b of a batch, channel c, group g):
//   S[b][c][x][ky][kz]  complex64 forward spectrum after the z and y passes
//   T[c][kx][ky][kz]    complex64 conj(target spectrum), kz in [0, d/2]
//   U[b][g][kx][ky][kz] complex64 sum over the group's channels of
//                       T_c * Q_c after the inverse x pass
// The three passes of one batch keep S and U resident in L2 (the library
// default batch keeps them well under the 129 MB L2).
#include <algorithm>
#include <mutex>

#include "vesper_common.cuh"

namespace vg {

constexpr int kThreads = 256;
constexpr int kRY = 8;          // rows per z-chunk (even: rows are paired into one complex line)
constexpr int kPairs = kRY / 2;

struct Query {
    const double *data;
    const float *vec;
    const float *probs;
    int d;
    double ave;
};

struct Mix {
    float one_minus_alpha, alpha, vave, vstd, pave, pstd;
};

__host__ __device__ inline int mode_nch(int mode) {
    return mode == VESPER_MODE_VEC ? 3 : (mode == VESPER_MODE_PROB ? 7 : 1);
}
__host__ __device__ inline int mode_ngrp(int mode) { return mode == VESPER_MODE_PROB ? 2 : 1; }

// ---------------------------------------------------------------------------
// mode fields
// ---------------------------------------------------------------------------

// Rotated query value(s) at destination (x, y, z), channels [c0, c0+cn).
// VESPER_1_prob_new.py: rot_mrc :279-354 (vec, data), rot_mrc_prob :1244-1297
// (per-channel masks), query transforms :548-555, laplacian_filter :494-526.
template <int MODE>
__device__ __forceinline__ void query_sample(const Query &q, const float *F, int x, int y, int z, int c0, int cn,
                                             float *out) {
    const int d = q.d;
    const double *data = q.data;
    float v[7];
    auto dmask = [data](int i) { return data[i] != 0.0; };
    if (MODE == VESPER_MODE_VEC || MODE == VESPER_MODE_PROB) {
        if (c0 < 3) {
            const int s = gather_src(F, d, x, y, z, dmask);
            if (s >= 0) {
                rotate_vec(F, q.vec[3 * s], q.vec[3 * s + 1], q.vec[3 * s + 2], v);
            } else {
                v[0] = v[1] = v[2] = 0.f;
            }
        }
        if (MODE == VESPER_MODE_PROB) {
            const size_t vol = (size_t)d * d * d;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                v[3 + k] = 0.f;
                if (c0 <= 3 + k && 3 + k < c0 + cn) {
                    const float *p = q.probs + k * vol;
                    const int s = gather_src(F, d, x, y, z, [p](int i) { return p[i] != 0.f; });
                    if (s >= 0) v[3 + k] = p[s];
                }
            }
        }
    } else if (MODE == VESPER_MODE_LAPLACIAN) {
        auto D = [&](int xx, int yy, int zz) -> double {
            const int s = gather_src(F, d, xx, yy, zz, dmask);
            return s >= 0 ? data[s] : 0.0;
        };
        const double cval = D(x, y, z);
        double acc = 0.0;
        if (cval > 0) {
            acc = __dmul_rn(-6.0, cval);
            if (x + 1 < d) acc = __dadd_rn(acc, D(x + 1, y, z));
            if (x - 1 >= 0) acc = __dadd_rn(acc, D(x - 1, y, z));
            if (y + 1 < d) acc = __dadd_rn(acc, D(x, y + 1, z));
            if (y - 1 >= 0) acc = __dadd_rn(acc, D(x, y - 1, z));
            if (z + 1 < d) acc = __dadd_rn(acc, D(x, y, z + 1));
            if (z - 1 >= 0) acc = __dadd_rn(acc, D(x, y, z - 1));
        }
        v[0] = (float)acc;
    } else {
        const int s = gather_src(F, d, x, y, z, dmask);
        const double val = s >= 0 ? data[s] : 0.0;
        if (MODE == VESPER_MODE_OVERLAP)
            v[0] = val > 0 ? 1.f : 0.f;
        else if (MODE == VESPER_MODE_CC)
            v[0] = val > 0 ? (float)val : 0.f;
        else
            v[0] = val > 0 ? (float)__dsub_rn(val, q.ave) : 0.f;
    }
    for (int c = 0; c < cn; ++c) out[c] = v[c0 + c];
}

// Target field of channel c at (x, y, z) in float64 (VESPER_1_prob_new.py:601-615,
// :831-838).
template <int MODE>
__device__ __forceinline__ double target_sample(const Query &q, int x, int y, int z, int c) {
    const int d = q.d;
    const size_t lin = ((size_t)x * d + y) * d + z;
    if (MODE == VESPER_MODE_VEC) return (double)q.vec[3 * lin + c];
    if (MODE == VESPER_MODE_PROB)
        return c < 3 ? (double)q.vec[3 * lin + c] : (double)q.probs[(size_t)(c - 3) * d * d * d + lin];
    const double val = q.data[lin];
    if (MODE == VESPER_MODE_OVERLAP) return val > 0 ? 1.0 : 0.0;
    if (MODE == VESPER_MODE_CC) return val > 0 ? val : 0.0;
    if (MODE == VESPER_MODE_PCC) return val > 0 ? __dsub_rn(val, q.ave) : 0.0;
    // Laplacian
    if (!(val > 0)) return 0.0;
    auto D = [&](int xx, int yy, int zz) { return q.data[((size_t)xx * d + yy) * d + zz]; };
    double acc = __dmul_rn(-6.0, val);
    if (x + 1 < d) acc = __dadd_rn(acc, D(x + 1, y, z));
    if (x - 1 >= 0) acc = __dadd_rn(acc, D(x - 1, y, z));
    if (y + 1 < d) acc = __dadd_rn(acc, D(x, y + 1, z));
    if (y - 1 >= 0) acc = __dadd_rn(acc, D(x, y - 1, z));
    if (z + 1 < d) acc = __dadd_rn(acc, D(x, y, z + 1));
    if (z - 1 >= 0) acc = __dadd_rn(acc, D(x, y, z - 1));
    return acc;
}

// ---------------------------------------------------------------------------
// shared helpers for the z pass (real rows paired into complex lines)
// ---------------------------------------------------------------------------

// After a forward FFT of line Z = a + i b, the half spectra of a and b.
template <typename C>
__device__ __forceinline__ void unpack_pair(C Zk, C Zn, C &A, C &B) {
    using R = typename Real<C>::T;
    const R h = (R)0.5;
    A = mk(h * (Zk.x + Zn.x), h * (Zk.y - Zn.y));
    B = mk(h * (Zk.y + Zn.y), -h * (Zk.x - Zn.x));
}

// ---------------------------------------------------------------------------
// Pass A (query): rotate + forward z (R2C, paired rows) + forward y.
// grid (d, nb): blockIdx.x = x plane, blockIdx.y = rotation within batch.
// ---------------------------------------------------------------------------
struct PassA {
    Query q;
    const float *rotmats;
    int r0, H, nch, cchunk, nscore;
    FftPlan P;
    float2 *S;
    unsigned long long *keys;
};

__host__ __device__ inline size_t smem_pass_a(int d, int H, int cchunk) {
    return (size_t)d * sizeof(float2) + (size_t)cchunk * d * H * sizeof(float2) +
           (size_t)cchunk * kPairs * d * sizeof(float2) + 16 * sizeof(float) + ((d * sizeof(short) + 15) & ~15);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_query_zy(const PassA a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int d = a.q.d, H = a.H, dH = d * H;
    const int x = blockIdx.x, b = blockIdx.y, r = a.r0 + b;
    float2 *tw = (float2 *)smem;
    float2 *plane = tw + d;
    float2 *zbuf = plane + (size_t)a.cchunk * dH;
    float *F = (float *)(zbuf + (size_t)a.cchunk * kPairs * d);
    short *rev = (short *)(F + 16);
    fft_tables(a.P, rev, tw);
    if (threadIdx.x < 9) F[threadIdx.x] = a.rotmats[(size_t)r * 9 + threadIdx.x];
    if (x == 0 && threadIdx.x < a.nscore) a.keys[(size_t)r * a.nscore + threadIdx.x] = 0ull;
    __syncthreads();
    for (int c0 = 0; c0 < a.nch; c0 += a.cchunk) {
        const int cn = min(a.cchunk, a.nch - c0);
        for (int y0 = 0; y0 < d; y0 += kRY) {
            for (int t = threadIdx.x; t < kRY * d; t += blockDim.x) {
                const int yy = t / d, z = t - yy * d, y = y0 + yy;
                float v[7];
                if (y < d) {
                    query_sample<MODE>(a.q, F, x, y, z, c0, cn, v);
                } else {
                    for (int c = 0; c < cn; ++c) v[c] = 0.f;
                }
                for (int c = 0; c < cn; ++c) {
                    float *dst = (float *)&zbuf[(c * kPairs + (yy >> 1)) * d + rev[z]];
                    dst[yy & 1] = v[c];
                }
            }
            __syncthreads();
            fft_run<false>(zbuf, Lines{cn * kPairs, 1, d, 0, 1}, a.P, tw, false);
            for (int t = threadIdx.x; t < cn * kPairs * H; t += blockDim.x) {
                const int line = t / H, k = t - line * H;
                const int c = line / kPairs, pr = line - c * kPairs;
                const int y = y0 + 2 * pr;
                float2 A, B;
                unpack_pair(zbuf[line * d + k], zbuf[line * d + (k == 0 ? 0 : d - k)], A, B);
                if (y < d) plane[((size_t)c * d + rev[y]) * H + k] = A;
                if (y + 1 < d) plane[((size_t)c * d + rev[y + 1]) * H + k] = B;
            }
            __syncthreads();
        }
        fft_run<false>(plane, Lines{cn * H, H, dH, 1, H}, a.P, tw, true);
        float2 *dst = a.S + (((size_t)b * a.nch + c0) * d + x) * dH;
        for (int t = threadIdx.x; t < cn * dH; t += blockDim.x) {
            const int c = t / dH, rest = t - c * dH;
            dst[(size_t)c * d * dH + rest] = plane[t];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Pass B: forward x, multiply by conj target and sum each group's channels,
// inverse x.  grid (ceil(d*H / W), nb).
// ---------------------------------------------------------------------------
struct PassB {
    const float2 *S;
    const float2 *T;
    float2 *U;
    int d, H, nch, ngrp, split, W;
    FftPlan P;
};

__host__ __device__ inline size_t smem_pass_b(int d, int nch, int ngrp, int W) {
    return (size_t)d * sizeof(float2) + (size_t)(nch + ngrp) * d * W * sizeof(float2) +
           ((d * sizeof(short) + 15) & ~15);
}

__global__ void __launch_bounds__(kThreads) k_x_corr(const PassB a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int d = a.d, dH = d * a.H, W = a.W;
    const int j0 = blockIdx.x * W, b = blockIdx.y;
    float2 *tw = (float2 *)smem;
    float2 *buf = tw + d;
    float2 *pbuf = buf + (size_t)a.nch * d * W;
    short *rev = (short *)(pbuf + (size_t)a.ngrp * d * W);
    fft_tables(a.P, rev, tw);
    __syncthreads();
    const float2 *src = a.S + (size_t)b * a.nch * d * dH;
    for (int t = threadIdx.x; t < a.nch * d * W; t += blockDim.x) {
        const int c = t / (d * W), rem = t - c * d * W, x = rem / W, w = rem - x * W, j = j0 + w;
        buf[((size_t)c * d + rev[x]) * W + w] = j < dH ? src[((size_t)c * d + x) * dH + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    fft_run<false>(buf, Lines{a.nch * W, W, d * W, 1, W}, a.P, tw, true);
    for (int t = threadIdx.x; t < a.ngrp * d * W; t += blockDim.x) {
        const int g = t / (d * W), rem = t - g * d * W, x = rem / W, w = rem - x * W, j = j0 + w;
        const int cb = g == 0 ? 0 : a.split, ce = g == 0 ? a.split : a.nch;
        float2 acc = make_float2(0.f, 0.f);
        if (j < dH)
            for (int c = cb; c < ce; ++c)
                acc = cadd(acc, cmul(a.T[((size_t)c * d + x) * dH + j], buf[((size_t)c * d + x) * W + w]));
        pbuf[((size_t)g * d + rev[x]) * W + w] = acc;
    }
    __syncthreads();
    fft_run<true>(pbuf, Lines{a.ngrp * W, W, d * W, 1, W}, a.P, tw, true);
    float2 *dst = a.U + (size_t)b * a.ngrp * d * dH;
    for (int t = threadIdx.x; t < a.ngrp * d * W; t += blockDim.x) {
        const int g = t / (d * W), rem = t - g * d * W, x = rem / W, w = rem - x * W, j = j0 + w;
        if (j < dH) dst[((size_t)g * d + x) * dH + j] = pbuf[t];
    }
}

// ---------------------------------------------------------------------------
// Pass C: inverse y, inverse z (C2R, paired rows), scores and argmax.
// grid (d, nb).  SC = number of scores kept per rotation (1, 2 or 3).
// ---------------------------------------------------------------------------
struct PassC {
    const float2 *U;
    int d, H, ngrp, r0, nscore;
    FftPlan P;
    Mix mix;
    unsigned long long *keys;
};

__host__ __device__ inline size_t smem_pass_c(int d, int H, int ngrp) {
    return (size_t)d * sizeof(float2) + (size_t)ngrp * d * H * sizeof(float2) +
           (size_t)ngrp * kPairs * d * sizeof(float2) + ((d * sizeof(short) + 15) & ~15) +
           3 * 32 * sizeof(unsigned long long);
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

template <int SC>
__global__ void __launch_bounds__(kThreads) k_inv_argmax(const PassC a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int d = a.d, H = a.H, dH = d * H, ngrp = a.ngrp;
    const int x = blockIdx.x, b = blockIdx.y, r = a.r0 + b;
    float2 *tw = (float2 *)smem;
    float2 *plane = tw + d;
    float2 *zbuf = plane + (size_t)ngrp * dH;
    short *rev = (short *)(zbuf + (size_t)ngrp * kPairs * d);
    unsigned long long *red = (unsigned long long *)((char *)rev + ((d * sizeof(short) + 15) & ~15));
    fft_tables(a.P, rev, tw);
    __syncthreads();
    const float2 *src = a.U + ((size_t)b * ngrp * d + x) * dH;
    for (int t = threadIdx.x; t < ngrp * dH; t += blockDim.x) {
        const int g = t / dH, rest = t - g * dH, ky = rest / H, kz = rest - ky * H;
        plane[((size_t)g * d + rev[ky]) * H + kz] = src[(size_t)g * d * dH + rest];
    }
    __syncthreads();
    fft_run<true>(plane, Lines{ngrp * H, H, dH, 1, H}, a.P, tw, true);
    unsigned long long best[3] = {0ull, 0ull, 0ull};
    for (int y0 = 0; y0 < d; y0 += kRY) {
        for (int t = threadIdx.x; t < ngrp * kPairs * d; t += blockDim.x) {
            const int line = t / d, k = t - line * d;
            const int g = line / kPairs, pr = line - g * kPairs, y = y0 + 2 * pr;
            const float2 *pa = plane + ((size_t)g * d + y) * H;
            const float2 *pb = pa + H;
            const bool ha = y < d, hb = y + 1 < d;
            float2 Z;
            if (k < H) {
                float2 A = ha ? pa[k] : make_float2(0.f, 0.f), B = hb ? pb[k] : make_float2(0.f, 0.f);
                if (k == 0 || 2 * k == d) { A.y = 0.f; B.y = 0.f; }
                Z = make_float2(A.x - B.y, A.y + B.x);
            } else {
                const int kk = d - k;
                const float2 A = ha ? pa[kk] : make_float2(0.f, 0.f), B = hb ? pb[kk] : make_float2(0.f, 0.f);
                Z = make_float2(A.x + B.y, B.x - A.y);
            }
            zbuf[line * d + rev[k]] = Z;
        }
        __syncthreads();
        fft_run<true>(zbuf, Lines{ngrp * kPairs, 1, d, 0, 1}, a.P, tw, false);
        for (int t = threadIdx.x; t < kRY * d; t += blockDim.x) {
            const int rr = t / d, z = t - rr * d, y = y0 + rr;
            if (y >= d) continue;
            const int pr = rr >> 1;
            const uint32_t lin = (uint32_t)((x * d + y) * d + z);
            const float2 z0 = zbuf[pr * d + z];
            const float v0 = (rr & 1) ? z0.y : z0.x;
            best[0] = max(best[0], make_key(v0, lin));
            if (SC >= 2) {
                const float2 z1 = zbuf[(kPairs + pr) * d + z];
                const float v1 = (rr & 1) ? z1.y : z1.x;
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
        __syncthreads();
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
        for (int w = 0; w < nw; ++w) v = max(v, red[threadIdx.x * 32 + w]);
        atomicMax(&a.keys[(size_t)r * a.nscore + threadIdx.x], v);
    }
}

__global__ void k_decode(const unsigned long long *keys, int n, float *scores, int32_t *lin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    scores[i] = order_float((uint32_t)(k >> 32));
    lin[i] = (int32_t)(0xffffffffu - (uint32_t)(k & 0xffffffffull));
}

// ---------------------------------------------------------------------------
// Target spectra, float64: z/y pass per (x plane, channel), then x pass.
// ---------------------------------------------------------------------------
struct TargetA {
    Query q;
    int H;
    FftPlan P;
    double2 *S;
};

__host__ __device__ inline size_t smem_target_a(int d, int H) {
    return (size_t)d * sizeof(double2) + (size_t)d * H * sizeof(double2) + (size_t)kPairs * d * sizeof(double2) +
           ((d * sizeof(short) + 15) & ~15);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_target_zy(const TargetA a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int d = a.q.d, H = a.H, dH = d * H;
    const int x = blockIdx.x, c = blockIdx.y;
    double2 *tw = (double2 *)smem;
    double2 *plane = tw + d;
    double2 *zbuf = plane + (size_t)dH;
    short *rev = (short *)(zbuf + (size_t)kPairs * d);
    fft_tables(a.P, rev, tw);
    __syncthreads();
    for (int y0 = 0; y0 < d; y0 += kRY) {
        for (int t = threadIdx.x; t < kRY * d; t += blockDim.x) {
            const int yy = t / d, z = t - yy * d, y = y0 + yy;
            const double v = y < d ? target_sample<MODE>(a.q, x, y, z, c) : 0.0;
            double *dst = (double *)&zbuf[(yy >> 1) * d + rev[z]];
            dst[yy & 1] = v;
        }
        __syncthreads();
        fft_run<false>(zbuf, Lines{kPairs, 1, d, 0, 1}, a.P, tw, false);
        for (int t = threadIdx.x; t < kPairs * H; t += blockDim.x) {
            const int pr = t / H, k = t - pr * H, y = y0 + 2 * pr;
            double2 A, B;
            unpack_pair(zbuf[pr * d + k], zbuf[pr * d + (k == 0 ? 0 : d - k)], A, B);
            if (y < d) plane[(size_t)rev[y] * H + k] = A;
            if (y + 1 < d) plane[(size_t)rev[y + 1] * H + k] = B;
        }
        __syncthreads();
    }
    fft_run<false>(plane, Lines{H, H, dH, 1, H}, a.P, tw, true);
    double2 *dst = a.S + ((size_t)c * d + x) * dH;
    for (int t = threadIdx.x; t < dH; t += blockDim.x) dst[t] = plane[t];
}

struct TargetB {
    const double2 *S;
    float2 *T;
    int d, H, W;
    FftPlan P;
};

__host__ __device__ inline size_t smem_target_b(int d, int W) {
    return (size_t)d * sizeof(double2) + (size_t)d * W * sizeof(double2) + ((d * sizeof(short) + 15) & ~15);
}

__global__ void __launch_bounds__(kThreads) k_target_x(const TargetB a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int d = a.d, dH = d * a.H, W = a.W;
    const int j0 = blockIdx.x * W, c = blockIdx.y;
    double2 *tw = (double2 *)smem;
    double2 *buf = tw + d;
    short *rev = (short *)(buf + (size_t)d * W);
    fft_tables(a.P, rev, tw);
    __syncthreads();
    const double2 *src = a.S + (size_t)c * d * dH;
    for (int t = threadIdx.x; t < d * W; t += blockDim.x) {
        const int x = t / W, w = t - x * W, j = j0 + w;
        buf[(size_t)rev[x] * W + w] = j < dH ? src[(size_t)x * dH + j] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    fft_run<false>(buf, Lines{W, W, d * W, 1, W}, a.P, tw, true);
    float2 *dst = a.T + (size_t)c * d * dH;
    for (int t = threadIdx.x; t < d * W; t += blockDim.x) {
        const int x = t / W, w = t - x * W, j = j0 + w;
        if (j < dH) {
            const double2 v = buf[t];
            dst[(size_t)x * dH + j] = make_float2((float)v.x, (float)(-v.y));
        }
    }
}

// ---------------------------------------------------------------------------
// stable top-N over strided scores
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_topn(const float *scores, int n, int stride, int topn, int32_t *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long *red = (unsigned long long *)smem;  // 32
    uint32_t *taken = (uint32_t *)(red + 32);             // ceil(n/32)
    const int nwords = (n + 31) >> 5;
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) taken[i] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < topn; ++k) {
        unsigned long long best = 0ull;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            if (taken[i >> 5] & (1u << (i & 31))) continue;
            best = max(best, make_key(scores[(size_t)i * stride], (uint32_t)i));
        }
        best = warp_max_u64(best);
        if (lane == 0) red[warp] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long v = 0ull;
            for (int w = 0; w < nw; ++w) v = max(v, red[w]);
            int idx = -1;
            if (v != 0ull) {
                idx = (int)(0xffffffffu - (uint32_t)(v & 0xffffffffull));
                taken[idx >> 5] |= 1u << (idx & 31);
            }
            out[k] = idx;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int smem_limit() {
    static int lim = 0;
    if (!lim) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
            v = 227 * 1024;
        lim = v;
    }
    return lim;
}

template <typename K>
static void allow_smem(K kernel, size_t bytes) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

static int pick_cchunk(int d, int H, int nch) {
    const size_t lim = (size_t)smem_limit();
    // prefer two CTAs per SM, then one
    for (size_t cap : {lim / 2 - 1024, lim}) {
        for (int c = nch; c >= 1; --c)
            if (smem_pass_a(d, H, c) <= cap) return c;
    }
    return 0;
}

static int pick_w(int d, int nch, int ngrp) {
    const size_t lim = (size_t)smem_limit();
    for (int W : {32, 16, 8, 4, 2, 1})
        if (smem_pass_b(d, nch, ngrp, W) <= lim / 2 - 1024) return W;
    for (int W : {8, 4, 2, 1})
        if (smem_pass_b(d, nch, ngrp, W) <= lim) return W;
    return 0;
}

static int pick_target_w(int d) {
    const size_t lim = (size_t)smem_limit();
    for (int W : {16, 8, 4, 2, 1})
        if (smem_target_b(d, W) <= lim / 2 - 1024) return W;
    return 1;
}

static int default_batch(int d, int mode) {
    const size_t H = d / 2 + 1;
    const size_t per = (size_t)(mode_nch(mode) + mode_ngrp(mode)) * d * d * H * sizeof(float2);
    const size_t budget = 64ull << 20;
    int b = (int)std::max<size_t>(1, budget / per);
    return std::min(b, 64);
}

static int check_dim(int d, int mode, FftPlan *P) {
    if (mode < 0 || mode > VESPER_MODE_PROB) return fail(VESPER_ERR_INVALID, "unknown mode %d", mode);
    if (d < 2) return fail(VESPER_ERR_INVALID, "grid side %d < 2", d);
    if (!make_plan(d, P)) return fail(VESPER_ERR_UNSUPPORTED, "grid side %d is not 2^a3^b5^c7^d(11|13)", d);
    if (d > vesper_max_dim(mode)) return fail(VESPER_ERR_UNSUPPORTED, "grid side %d above the maximum %d", d,
                                              vesper_max_dim(mode));
    return VESPER_OK;
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_max_dim(int mode) {
    int best = 0;
    for (int d = 2; d <= 256; ++d) {
        FftPlan P;
        if (!make_plan(d, &P)) continue;
        const int H = d / 2 + 1;
        const size_t lim = (size_t)smem_limit();
        const int nch = mode_nch(mode), ngrp = mode_ngrp(mode);
        if (smem_pass_a(d, H, 1) > lim || smem_pass_c(d, H, ngrp) > lim || smem_target_a(d, H) > lim ||
            smem_pass_b(d, nch, ngrp, 1) > lim)
            continue;
        best = d;
    }
    return best;
}

extern "C" int vesper_search_nscore(int mode, int with_mix) {
    if (mode == VESPER_MODE_PROB) return with_mix ? 3 : 2;
    return 1;
}

extern "C" int vesper_spectra_bytes(int dim, int mode, size_t *bytes) {
    if (!bytes) return fail(VESPER_ERR_INVALID, "bytes is NULL");
    const size_t H = dim / 2 + 1;
    *bytes = (size_t)mode_nch(mode) * dim * dim * H * sizeof(float2);
    return VESPER_OK;
}

extern "C" int vesper_target_workspace_size(int dim, int mode, size_t *bytes) {
    if (!bytes) return fail(VESPER_ERR_INVALID, "bytes is NULL");
    const size_t H = dim / 2 + 1;
    *bytes = (size_t)mode_nch(mode) * dim * dim * H * sizeof(double2) + 256;
    return VESPER_OK;
}

extern "C" int vesper_target_spectra(const double *data, const float *vec, const float *probs, int dim, int mode,
                                     double ave, void *spectra_out, void *workspace, size_t workspace_bytes,
                                     void *stream) {
    FftPlan P;
    int rc = check_dim(dim, mode, &P);
    if (rc) return rc;
    const bool need_vec = mode == VESPER_MODE_VEC || mode == VESPER_MODE_PROB;
    if ((need_vec && !vec) || (!need_vec && !data) || (mode == VESPER_MODE_PROB && !probs) || !spectra_out)
        return fail(VESPER_ERR_INVALID, "vesper_target_spectra: missing input or output pointer");
    size_t need = 0;
    vesper_target_workspace_size(dim, mode, &need);
    if (!workspace || workspace_bytes < need)
        return fail(VESPER_ERR_WORKSPACE, "vesper_target_spectra: workspace %zu < %zu bytes", workspace_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    const int H = dim / 2 + 1, nch = mode_nch(mode);
    TargetA ta{Query{data, vec, probs, dim, ave}, H, P, (double2 *)workspace};
    const size_t sa = smem_target_a(dim, H);
    dim3 ga(dim, nch);
    switch (mode) {
#define VG_TGT(M)                                                \
    case M:                                                      \
        allow_smem(k_target_zy<M>, sa);                          \
        k_target_zy<M><<<ga, kThreads, sa, st>>>(ta);            \
        break;
        VG_TGT(VESPER_MODE_VEC)
        VG_TGT(VESPER_MODE_OVERLAP)
        VG_TGT(VESPER_MODE_CC)
        VG_TGT(VESPER_MODE_PCC)
        VG_TGT(VESPER_MODE_LAPLACIAN)
        VG_TGT(VESPER_MODE_PROB)
#undef VG_TGT
    }
    VG_CHECK_LAUNCH("k_target_zy");
    const int W = pick_target_w(dim);
    TargetB tb{(const double2 *)workspace, (float2 *)spectra_out, dim, H, W, P};
    const size_t sb = smem_target_b(dim, W);
    allow_smem(k_target_x, sb);
    k_target_x<<<dim3((dim * H + W - 1) / W, nch), kThreads, sb, st>>>(tb);
    VG_CHECK_LAUNCH("k_target_x");
    return VESPER_OK;
}

extern "C" int vesper_search_workspace_size(int dim, int mode, int batch, int nrot, size_t *bytes) {
    if (!bytes) return fail(VESPER_ERR_INVALID, "bytes is NULL");
    if (batch <= 0) batch = default_batch(dim, mode);
    const size_t H = dim / 2 + 1;
    Carver cv(nullptr, 0);
    cv.take<float2>((size_t)batch * mode_nch(mode) * dim * dim * H);
    cv.take<float2>((size_t)batch * mode_ngrp(mode) * dim * dim * H);
    cv.take<unsigned long long>((size_t)std::max(nrot, 1) * 3);
    *bytes = cv.off + 256;
    return VESPER_OK;
}

// Per-pass event timing of one search (profiling entry point).
// A ring of event sets keeps kRing batches in flight: a slot's events are read
// (and its times accumulated) only when the slot is reused or at the end.
constexpr int kRing = 16;
struct PassTimer {
    cudaEvent_t ev[kRing][4][2];
    bool used[kRing][4];
    float ms[4];
};

static int search_impl(const void *spectra, const double *data, const float *vec, const float *probs, int dim,
                       int mode, double ave, const float *rotmats, int nrot, const double *mix, float *scores_out,
                       int32_t *lin_out, int batch, void *workspace, size_t workspace_bytes, void *stream,
                       PassTimer *tm) {
    FftPlan P;
    int rc = check_dim(dim, mode, &P);
    if (rc) return rc;
    if (nrot < 0) return fail(VESPER_ERR_INVALID, "nrot %d < 0", nrot);
    if (nrot == 0) return VESPER_OK;
    const bool need_vec = mode == VESPER_MODE_VEC || mode == VESPER_MODE_PROB;
    if (!spectra || !data || (need_vec && !vec) || (mode == VESPER_MODE_PROB && !probs) || !rotmats ||
        !scores_out || !lin_out)
        return fail(VESPER_ERR_INVALID, "vesper_search: missing input or output pointer");
    if (mix && mode != VESPER_MODE_PROB) return fail(VESPER_ERR_INVALID, "mix parameters need VESPER_MODE_PROB");
    if (batch <= 0) batch = default_batch(dim, mode);
    size_t need = 0;
    vesper_search_workspace_size(dim, mode, batch, nrot, &need);
    if (!workspace || workspace_bytes < need)
        return fail(VESPER_ERR_WORKSPACE, "vesper_search: workspace %zu < %zu bytes", workspace_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    const int H = dim / 2 + 1, nch = mode_nch(mode), ngrp = mode_ngrp(mode);
    const int nscore = vesper_search_nscore(mode, mix != nullptr);
    Carver cv(workspace, workspace_bytes);
    float2 *S = cv.take<float2>((size_t)batch * nch * dim * dim * H);
    float2 *U = cv.take<float2>((size_t)batch * ngrp * dim * dim * H);
    unsigned long long *keys = cv.take<unsigned long long>((size_t)nrot * 3);

    const int cchunk = pick_cchunk(dim, H, nch);
    const int W = pick_w(dim, nch, ngrp);
    if (!cchunk || !W) return fail(VESPER_ERR_UNSUPPORTED, "grid side %d does not fit shared memory", dim);
    const size_t sa = smem_pass_a(dim, H, cchunk), sb = smem_pass_b(dim, nch, ngrp, W),
                 sc = smem_pass_c(dim, H, ngrp);
    Mix mx{};
    if (mix) {
        mx.one_minus_alpha = (float)(1.0 - mix[0]);
        mx.alpha = (float)mix[0];
        mx.vstd = (float)mix[1];
        mx.vave = (float)mix[2];
        mx.pstd = (float)mix[3];
        mx.pave = (float)mix[4];
    }
    PassA pa{Query{data, vec, probs, dim, ave}, rotmats, 0, H, nch, cchunk, nscore, P, S, keys};
    PassB pb{S, (const float2 *)spectra, U, dim, H, nch, ngrp, mode == VESPER_MODE_PROB ? 3 : nch, W, P};
    PassC pc{U, dim, H, ngrp, 0, nscore, P, mx, keys};
    switch (mode) {
        case VESPER_MODE_VEC: allow_smem(k_query_zy<VESPER_MODE_VEC>, sa); break;
        case VESPER_MODE_OVERLAP: allow_smem(k_query_zy<VESPER_MODE_OVERLAP>, sa); break;
        case VESPER_MODE_CC: allow_smem(k_query_zy<VESPER_MODE_CC>, sa); break;
        case VESPER_MODE_PCC: allow_smem(k_query_zy<VESPER_MODE_PCC>, sa); break;
        case VESPER_MODE_LAPLACIAN: allow_smem(k_query_zy<VESPER_MODE_LAPLACIAN>, sa); break;
        case VESPER_MODE_PROB: allow_smem(k_query_zy<VESPER_MODE_PROB>, sa); break;
    }
    allow_smem(k_x_corr, sb);
    allow_smem(k_inv_argmax<1>, sc);
    allow_smem(k_inv_argmax<2>, sc);
    allow_smem(k_inv_argmax<3>, sc);
    const int nbx = (dim * H + W - 1) / W;
    int slot = 0;
    auto drain = [&](int sl) {
        for (int p = 0; p < 4; ++p) {
            if (!tm->used[sl][p]) continue;
            cudaEventSynchronize(tm->ev[sl][p][1]);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, tm->ev[sl][p][0], tm->ev[sl][p][1]);
            tm->ms[p] += ms;
            tm->used[sl][p] = false;
        }
    };
    auto mark = [&](int pass, int edge) {
        if (!tm) return;
        if (edge == 0 && tm->used[slot][pass]) drain(slot);
        cudaEventRecord(tm->ev[slot][pass][edge], st);
        if (edge == 1) tm->used[slot][pass] = true;
    };
    for (int r0 = 0; r0 < nrot; r0 += batch) {
        const int nb = std::min(batch, nrot - r0);
        pa.r0 = r0;
        pc.r0 = r0;
        const dim3 gplane(dim, nb);
        mark(0, 0);
        switch (mode) {
            case VESPER_MODE_VEC: k_query_zy<VESPER_MODE_VEC><<<gplane, kThreads, sa, st>>>(pa); break;
            case VESPER_MODE_OVERLAP: k_query_zy<VESPER_MODE_OVERLAP><<<gplane, kThreads, sa, st>>>(pa); break;
            case VESPER_MODE_CC: k_query_zy<VESPER_MODE_CC><<<gplane, kThreads, sa, st>>>(pa); break;
            case VESPER_MODE_PCC: k_query_zy<VESPER_MODE_PCC><<<gplane, kThreads, sa, st>>>(pa); break;
            case VESPER_MODE_LAPLACIAN: k_query_zy<VESPER_MODE_LAPLACIAN><<<gplane, kThreads, sa, st>>>(pa); break;
            case VESPER_MODE_PROB: k_query_zy<VESPER_MODE_PROB><<<gplane, kThreads, sa, st>>>(pa); break;
        }
        VG_CHECK_LAUNCH("k_query_zy");
        mark(0, 1);
        mark(1, 0);
        k_x_corr<<<dim3(nbx, nb), kThreads, sb, st>>>(pb);
        VG_CHECK_LAUNCH("k_x_corr");
        mark(1, 1);
        mark(2, 0);
        switch (nscore) {
            case 1: k_inv_argmax<1><<<gplane, kThreads, sc, st>>>(pc); break;
            case 2: k_inv_argmax<2><<<gplane, kThreads, sc, st>>>(pc); break;
            default: k_inv_argmax<3><<<gplane, kThreads, sc, st>>>(pc); break;
        }
        VG_CHECK_LAUNCH("k_inv_argmax");
        mark(2, 1);
        slot = (slot + 1) % kRing;
    }
    const int n = nrot * nscore;
    mark(3, 0);
    k_decode<<<(n + 255) / 256, 256, 0, st>>>(keys, n, scores_out, lin_out);
    VG_CHECK_LAUNCH("k_decode");
    mark(3, 1);
    if (tm)
        for (int sl = 0; sl < kRing; ++sl) drain(sl);
    return VESPER_OK;
}

extern "C" int vesper_search(const void *spectra, const double *data, const float *vec, const float *probs, int dim,
                             int mode, double ave, const float *rotmats, int nrot, const double *mix,
                             float *scores_out, int32_t *lin_out, int batch, void *workspace,
                             size_t workspace_bytes, void *stream) {
    return search_impl(spectra, data, vec, probs, dim, mode, ave, rotmats, nrot, mix, scores_out, lin_out, batch,
                       workspace, workspace_bytes, stream, nullptr);
}

extern "C" int vesper_search_profile(const void *spectra, const double *data, const float *vec, const float *probs,
                                     int dim, int mode, double ave, const float *rotmats, int nrot,
                                     const double *mix, float *scores_out, int32_t *lin_out, int batch,
                                     void *workspace, size_t workspace_bytes, void *stream, float *pass_ms,
                                     int *pass_launches) {
    if (!pass_ms || !pass_launches) return fail(VESPER_ERR_INVALID, "vesper_search_profile: NULL timing outputs");
    static PassTimer tm;   // one profiling call at a time per process
    static bool created = false;
    if (!created) {
        for (int sl = 0; sl < kRing; ++sl)
            for (int p = 0; p < 4; ++p)
                for (int e = 0; e < 2; ++e)
                    if (cudaEventCreate(&tm.ev[sl][p][e]) != cudaSuccess)
                        return fail(VESPER_ERR_CUDA, "vesper_search_profile: cudaEventCreate failed");
        created = true;
    }
    for (int sl = 0; sl < kRing; ++sl)
        for (int p = 0; p < 4; ++p) tm.used[sl][p] = false;
    for (int p = 0; p < 4; ++p) tm.ms[p] = 0.f;
    const int rc = search_impl(spectra, data, vec, probs, dim, mode, ave, rotmats, nrot, mix, scores_out, lin_out,
                               batch, workspace, workspace_bytes, stream, &tm);
    for (int p = 0; p < 4; ++p) pass_ms[p] = tm.ms[p];
    if (batch <= 0) batch = default_batch(dim, mode);
    const int nb = nrot > 0 ? (nrot + batch - 1) / batch : 0;
    pass_launches[0] = pass_launches[1] = pass_launches[2] = nb;
    pass_launches[3] = nrot > 0 ? 1 : 0;
    return rc;
}

// ---------------------------------------------------------------------------
// Search without caller-provided scratch.
//
// For callers that cannot allocate device memory themselves -- for example
// code that runs while another part of the process holds a stream capture in
// global mode (cudaMalloc then fails), or a host application that hands this
// library only pre-allocated input and output buffers under a fixed
// device-memory budget.  Its scratch is the fixed array below, which the CUDA
// module reserves on every GPU that loads this library and keeps until the
// process exits.  All calls on a device share it: calls that overlap on the
// GPU (two streams, or two host threads) race on it, so serialise them.
// ---------------------------------------------------------------------------
namespace vg {
constexpr size_t kStaticScratchBytes = 16ull << 20;   // 16 MiB
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_static_mu;
static void *g_static_ptr[kMaxDevices] = {};
}  // namespace vg

// The host-side name g_static_scratch is only a stand-in for the device array,
// so its device address is looked up once per device (with that device
// current) and cached; the first call on each device does this set-up, so make
// that first call before any stream capture.
extern "C" int vesper_search_static(const void *spectra, const double *data, const float *vec, const float *probs,
                                    int dim, int mode, double ave, const float *rotmats, int nrot, const double *mix,
                                    float *scores_out, int32_t *lin_out, void *stream) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cuda_check("vesper_search_static: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(VESPER_ERR_UNSUPPORTED, "vesper_search_static: device %d", dev);
    void *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_static_mu);
        if (!g_static_ptr[dev]) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess || !p)
                return fail(VESPER_ERR_CUDA, "vesper_search_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_static_ptr[dev] = p;
        }
        scratch = g_static_ptr[dev];
    }
    size_t need = 0;
    int rc = vesper_search_workspace_size(dim, mode, 1, nrot, &need);
    if (rc) return rc;
    if (need > kStaticScratchBytes)
        return fail(VESPER_ERR_UNSUPPORTED,
                    "vesper_search_static: dim=%d mode=%d nrot=%d needs %zu bytes of scratch, above its fixed %zu "
                    "(use vesper_search with a workspace)", dim, mode, nrot, need, (size_t)kStaticScratchBytes);
    // one rotation per pipeline step; the keys each rotation reads are zeroed by
    // its own first pass, so nothing left in the array by an earlier call matters
    return search_impl(spectra, data, vec, probs, dim, mode, ave, rotmats, nrot, mix, scores_out, lin_out, 1, scratch,
                       kStaticScratchBytes, stream, nullptr);
}

extern "C" int vesper_topn(const float *scores, int n, int stride, int topn, int32_t *idx_out, void *stream) {
    if (!scores || !idx_out || n < 0 || topn < 0 || stride < 1)
        return fail(VESPER_ERR_INVALID, "vesper_topn: bad arguments");
    if (topn == 0) return VESPER_OK;
    const size_t sm = 32 * sizeof(unsigned long long) + (size_t)((n + 31) / 32) * sizeof(uint32_t);
    if (sm > (size_t)smem_limit()) return fail(VESPER_ERR_UNSUPPORTED, "vesper_topn: n=%d too large", n);
    allow_smem(k_topn, sm);
    k_topn<<<1, 1024, sm, (cudaStream_t)stream>>>(scores, n, stride, topn, idx_out);
    VG_CHECK_LAUNCH("k_topn");
    return VESPER_OK;
}
