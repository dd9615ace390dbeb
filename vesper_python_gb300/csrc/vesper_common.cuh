// Shared host/device helpers of the VESPER GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "vesper_fft.cuh"
#include "../../include/vesper_gb300.h"

namespace vg {

// ---- error reporting (per host thread) --------------------------------------
void set_error(const char *fmt, ...);
int fail(int code, const char *fmt, ...);
int cuda_check(const char *what);

#define VG_CHECK_LAUNCH(what)                          \
    do {                                               \
        int _rc = ::vg::cuda_check(what);              \
        if (_rc != VESPER_OK) return _rc;              \
    } while (0)

// ---- FFT plans ----------------------------------------------------------------
// Factor n into supported radices (4s first, then 2, 3, 5, 7, 11, 13).  Returns
// false when n has another prime factor or more than one of 11 and 13.
bool make_plan(int n, FftPlan *plan);

// ---- workspace carving ----------------------------------------------------------
struct Carver {
    char *base;
    size_t cap, off;
    __host__ Carver(void *b, size_t c) : base((char *)b), cap(c), off(0) {}
    template <typename T>
    __host__ T *take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        T *p = (T *)(base ? base + off : nullptr);
        off += count * sizeof(T);
        return p;
    }
    __host__ bool ok() const { return off <= cap; }
};

// ---- ordering key for (score desc, index asc) ---------------------------------
// -0.0 and +0.0 compare equal (as in numpy's argmax and sorts): both map to
// the key of +0.0, so ties between them resolve by index like any other tie.
__device__ __forceinline__ uint32_t float_order(float f) {
    const uint32_t u = f == 0.f ? 0u : __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float order_float(uint32_t o) {
    const uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
    return __uint_as_float(u);
}
__device__ __forceinline__ unsigned long long make_key(float s, uint32_t lin) {
    return ((unsigned long long)float_order(s) << 32) | (unsigned long long)(0xffffffffu - lin);
}

// ---- reference gather geometry (rot_mrc, VESPER_1_prob_new.py:279-354) --------
// Candidate source new_pos indices i (per axis) that land on destination t
// after dest = int(trunc(i - d/2) + d/2), in descending order of i.  For
// even d only i = t; for odd d (m = (d-1)/2) i = t below m, {m+1, m} at m,
// t+1 above m and none at d-1.
__device__ __forceinline__ int gather_cands(int t, int d, int *c) {
    if ((d & 1) == 0) { c[0] = t; return 1; }
    const int m = (d - 1) >> 1;
    if (t < m) { c[0] = t; return 1; }
    if (t == m) { c[0] = m + 1; c[1] = m; return 2; }
    if (t < d - 1) { c[0] = t + 1; return 1; }
    return 0;
}

// old position of the new_pos row (ix, iy, iz): float32 sgemm order with an
// FMA chain over k = 0, 1, 2, then a float32 add of d/2.  F is np.flip(mtx).
__device__ __forceinline__ bool old_index(const float *F, int d, float cf, float hx, float hy, float hz,
                                          int &ox, int &oy, int &oz) {
    float o[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float acc = __fmul_rn(hx, F[a * 3 + 0]);
        acc = __fmaf_rn(hy, F[a * 3 + 1], acc);
        acc = __fmaf_rn(hz, F[a * 3 + 2], acc);
        o[a] = __fadd_rn(acc, cf);
    }
    const float df = (float)d;
    if (!(o[0] >= 0.f && o[1] >= 0.f && o[2] >= 0.f && o[0] < df && o[1] < df && o[2] < df)) return false;
    ox = (int)o[0];
    oy = (int)o[1];
    oz = (int)o[2];
    return true;
}

// Winning source voxel for destination (x, y, z): the last reference row
// (z slowest, x middle, y fastest) whose old position is in bounds and passes
// ``mask``.  Returns the source linear index or -1.
template <class Mask>
__device__ __forceinline__ int gather_src(const float *F, int d, int x, int y, int z, Mask mask) {
    int cx[2], cy[2], cz[2];
    const int nx = gather_cands(x, d, cx), ny = gather_cands(y, d, cy), nz = gather_cands(z, d, cz);
    const float cf = 0.5f * (float)d;
    const float hc = 0.5f * (float)d;
    for (int a = 0; a < nz; ++a) {
        const float hz = (float)cz[a] - hc;
        for (int b = 0; b < nx; ++b) {
            const float hx = (float)cx[b] - hc;
            for (int e = 0; e < ny; ++e) {
                const float hy = (float)cy[e] - hc;
                int ox, oy, oz;
                if (!old_index(F, d, cf, hx, hy, hz, ox, oy, oz)) continue;
                const int src = (ox * d + oy) * d + oz;
                if (mask(src)) return src;
            }
        }
    }
    return -1;
}

// rotated vector: new_vec_j = sum_k v_k F[k][j] (sgemm order, FMA chain)
__device__ __forceinline__ void rotate_vec(const float *F, float v0, float v1, float v2, float *o) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        float acc = __fmul_rn(v0, F[0 * 3 + j]);
        acc = __fmaf_rn(v1, F[1 * 3 + j], acc);
        o[j] = __fmaf_rn(v2, F[2 * 3 + j], acc);
    }
}

// ---- search-wide definitions ------------------------------------------------------
constexpr int kThreads = 256;
constexpr int kRY = 8;          // rows per z-chunk of the float64 target pass (even: rows pair up)
constexpr int kPairs = kRY / 2;

struct Query {
    const double *data;
    const float *vec;
    const float *probs;
    int d;
    double ave;
};

// prob-mode z-score mixing constants (float32, as numpy 1.21 computes them)
struct Mix {
    float one_minus_alpha, alpha, vave, vstd, pave, pstd;
};

__host__ __device__ inline int mode_nch(int mode) {
    return mode == VESPER_MODE_VEC ? 3 : (mode == VESPER_MODE_PROB ? 7 : 1);
}
__host__ __device__ inline int mode_ngrp(int mode) { return mode == VESPER_MODE_PROB ? 2 : 1; }

// After a forward FFT of line Z = a + i b, the half spectra of a and b.
template <typename C>
__device__ __forceinline__ void unpack_pair(C Zk, C Zn, C &A, C &B) {
    using R = typename Real<C>::T;
    const R h = (R)0.5;
    A = mk(h * (Zk.x + Zn.x), h * (Zk.y - Zn.y));
    B = mk(h * (Zk.y + Zn.y), -h * (Zk.x - Zn.x));
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

__host__ __device__ inline size_t smem_target_a(int d, int H) {
    return (size_t)d * sizeof(double2) + (size_t)d * H * sizeof(double2) + (size_t)kPairs * d * sizeof(double2) +
           ((d * sizeof(short) + 15) & ~15);
}
__host__ __device__ inline size_t smem_target_b(int d, int W) {
    return (size_t)d * sizeof(double2) + (size_t)d * W * sizeof(double2) + ((d * sizeof(short) + 15) & ~15);
}

// Opt-in shared memory per block of the current device (host).
inline int smem_limit() {
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

// Raise a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device.  The largest limit set so far is remembered per (device,
// kernel), so the driver call is made only when a launch needs more (the call
// costs about a microsecond of host time, and hot paths launch thousands of
// kernels).
template <typename K>
inline void allow_smem(K kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> set;
    int dev = 0;
    cudaGetDevice(&dev);
    const std::pair<int, const void *> key(dev, (const void *)kernel);
    {
        std::lock_guard<std::mutex> g(mu);
        const auto it = set.find(key);
        if (it != set.end() && it->second >= bytes) return;
    }
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess) {
        std::lock_guard<std::mutex> g(mu);
        size_t &v = set[key];
        if (bytes > v) v = bytes;
    }
}

}  // namespace vg
