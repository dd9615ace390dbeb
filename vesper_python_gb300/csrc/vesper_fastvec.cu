// fastVEC on the GPU: the Gaussian-weighted density and unit vector of every
// destination voxel of the coarse grid (doFastVEC / calc,
// VESPER_1_prob_new.py:121-142, :180-257).
//
// The reference sums, for each destination voxel at source position pos,
//   v = src[p] * exp(-1.5 |p - pos|^2 fsiv)
// over the box [int(pos - fmaxd) v 0, int(pos + fmaxd + 1) ^ S) on each axis,
// together with v * p.  Both the weight and the box factor per axis, and pos
// on axis a depends only on the destination index on that axis, so the sums
// are three successive 1-D banded contractions (z, then y, then x):
//   A0[xp][yp][z] = sum_zp wz[z][zp] src[xp][yp][zp]      A1 = same with zp wz
//   B0[xp][y][z]  = sum_yp wy[y][yp] A0                    B1 = yp wy A0, B2 = wy A1
//   D = sum_xp wx B0, Px = sum xp wx B0, Py = sum wx B1, Pz = sum wx B2
// with w = exp(-1.5 r^2 fsiv) per axis (the product of the three per-axis
// factors is the reference's exp of the sum up to rounding).  The per-voxel
// skip tests (pos inside the source, src[int(pos)] != 0) and the
// normalisation follow the reference operation by operation.
//
// Cost: S0 S1 d WB + S0 d^2 WB + d^3 WB multiply-adds (x2..4) instead of
// d^3 WB^3 exponentials, WB = band width <= 2 fmaxd + 2.
//
// Arithmetic.  The reference sums in float64, which runs at 1/64 of the
// float32 rate on this part.  The contractions therefore carry every partial
// sum as an unevaluated pair of float32 values hi + lo ("double-single" or
// float-float numbers, Dekker 1971): products by TwoProd (the rounding error
// of hi * v recovered exactly with one fmaf), sums by Knuth's TwoSum followed by
// a FastTwoSum renormalisation after every term, about 2^-46 relative per
// operation.  Every term is non-negative (the thresholded source is >= 0;
// weights and positions are positive), so nothing cancels inside a sum.  The
// weights are computed in float64 and split into pairs; each voxel's finish
// (ratios, norm, unit vector) runs in float64 on the pair sums.  Against the
// float64 restatement of the reference loop this gives densities within 1e-13
// relative and the same float32 vectors.  A pair cannot hold a weight below
// the float32 normal range to full precision, so geometries whose smallest
// band weight exp(-1.5 (fmaxd + 1)^2 fsiv) is below 2^-70 (dreso / src_width
// below about 0.8) run the same contractions in float64 instead.
#include <algorithm>
#include <cmath>

#include "vesper_common.cuh"

namespace vg {

struct AxisTables {
    // per axis a and destination index i (d entries each)
    double *pos;     // [3][d]
    int *stp;        // [3][d]
    int *len;        // [3][d] endp - stp (>= 0)
    int *idx;        // [3][d] int(pos) if 0 <= pos < S else -1
    double *w;       // [3][WB][d]  weight of band entry k
    double *wp;      // [3][WB][d]  weight * (stp + k)
    float2 *wf;      // [3][WB][d]  w as a float-float pair (hi, lo)
    float2 *wpf;     // [3][WB][d]  wp as a pair
    int *plane;      // [S0] source plane xp holds a non-zero value (written by the z stage)
    int *list;       // [S0 S1] source rows holding a non-zero value (float-float z stage)
    int *nlist;      // [1] their count
};

struct FvGeom {
    int S[3];
    int d, WB;
    double sw, dw, fsiv, fmaxd;
    double sorig[3], dorig[3];
};

// Block (i, a): destination index i on axis a; its threads share the band
// entries k (the exponentials), each computing the same position and band.
__global__ void k_fv_tables(const FvGeom g, AxisTables t) {
    const int i = blockIdx.x;
    const int a = blockIdx.y;
    if (i >= g.d) return;
    if (a == 0)   // clear the plane flags: block i takes planes i*128 + tid + m*128*d
        for (int xp = i * blockDim.x + threadIdx.x; xp < g.S[0]; xp += g.d * blockDim.x) t.plane[xp] = 0;
    if (a == 0 && i == 0 && threadIdx.x == 0) *t.nlist = 0;
    // (xyz_arr * dest_xwidth + dest_orig - src_orig) / src_xwidth
    double p = __dmul_rn((double)i, g.dw);
    p = __dadd_rn(p, g.dorig[a]);
    p = __dsub_rn(p, g.sorig[a]);
    p = __ddiv_rn(p, g.sw);
    const int o = a * g.d + i;
    int stp = __double2int_rz(__dsub_rn(p, g.fmaxd));
    if (stp < 0) stp = 0;
    int endp = __double2int_rz(__dadd_rn(__dadd_rn(p, g.fmaxd), 1.0));
    if (endp >= g.S[a]) endp = g.S[a];
    const int len = max(0, min(endp - stp, g.WB));
    if (threadIdx.x == 0) {
        t.pos[o] = p;
        t.idx[o] = (p >= 0.0 && p < (double)g.S[a]) ? (int)p : -1;
        t.stp[o] = stp;
        t.len[o] = len;
    }
    for (int k = threadIdx.x; k < g.WB; k += blockDim.x) {
        double w = 0.0;
        if (k < len) {
            double r = __dsub_rn((double)(stp + k), p);
            r = __dmul_rn(r, r);
            w = exp(__dmul_rn(__dmul_rn(-1.5, r), g.fsiv));
        }
        const size_t wo = ((size_t)a * g.WB + k) * g.d + i;
        const double wp = __dmul_rn(w, (double)(stp + k));
        t.w[wo] = w;
        t.wp[wo] = wp;
        // hi = w rounded to float32; lo = the (exact) remainder rounded to float32
        const float wh = __double2float_rn(w), wph = __double2float_rn(wp);
        t.wf[wo] = make_float2(wh, __double2float_rn(__dsub_rn(w, (double)wh)));
        t.wpf[wo] = make_float2(wph, __double2float_rn(__dsub_rn(wp, (double)wph)));
    }
}

// ---- float-float helpers (all operations explicitly rounded, so the compiler
// neither fuses nor reorders them) ------------------------------------------------
// (sh, sl) += (th, tl): TwoSum of the high parts, the low parts added to the
// error, then FastTwoSum to renormalise
__device__ __forceinline__ void ff_add(float &sh, float &sl, float th, float tl) {
    const float s = __fadd_rn(sh, th);
    const float bb = __fsub_rn(s, sh);
    float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(th, bb));
    e = __fadd_rn(e, __fadd_rn(sl, tl));
    sh = __fadd_rn(s, e);
    sl = __fsub_rn(e, __fsub_rn(sh, s));
}

// (h, l) * v for a float32 v: TwoProd of h * v, plus l * v in the low part
__device__ __forceinline__ void ff_mul_f(float h, float l, float v, float &ph, float &pl) {
    ph = __fmul_rn(h, v);
    pl = __fmaf_rn(l, v, __fmaf_rn(h, v, -ph));
}

// (ah, al) * (bh, bl): TwoProd of the high parts plus both cross terms
__device__ __forceinline__ void ff_mul(float2 a, float2 b, float &ph, float &pl) {
    ph = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -ph);
    e = __fmaf_rn(a.x, b.y, e);
    pl = __fmaf_rn(a.y, b.x, e);
}

// stage 1: contract z.  Block = RB source rows (xp, yp), all d outputs.
constexpr int kRB = 8;
__global__ void __launch_bounds__(256) k_fv_z(const float *src, const FvGeom g, const AxisTables t, double *A0,
                                              double *A1) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int S2 = g.S[2], d = g.d;
    const size_t nrows = (size_t)g.S[0] * g.S[1];
    const size_t row0 = (size_t)blockIdx.x * kRB;
    float *rows = (float *)smem;
    __shared__ int nz[kRB];   // row holds a non-zero value (thresholded maps are mostly empty rows)
    if (threadIdx.x < kRB) nz[threadIdx.x] = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < kRB * S2; e += blockDim.x) {
        const size_t r = row0 + e / S2;
        const float v = r < nrows ? src[r * S2 + (e % S2)] : 0.f;
        rows[e] = v;
        if (v != 0.f) nz[e / S2] = 1;
    }
    __syncthreads();
    const int *stp = t.stp + 2 * d, *len = t.len + 2 * d;
    const double *w = t.w + (size_t)2 * g.WB * d, *wp = t.wp + (size_t)2 * g.WB * d;
    for (int o = threadIdx.x; o < kRB * d; o += blockDim.x) {
        const int rr = o / d, z = o - rr * d;
        const size_t r = row0 + rr;
        if (r >= nrows) continue;
        if (!nz[rr]) {   // an all-zero row: the sums are +0.0, as the loop would give
            A0[r * d + z] = 0.0;
            A1[r * d + z] = 0.0;
            continue;
        }
        const float *row = rows + rr * S2 + stp[z];
        const int n = len[z];
        double s0 = 0.0, s1 = 0.0;
        for (int k = 0; k < n; ++k) {
            const double v = (double)row[k];
            s0 = fma(v, w[(size_t)k * d + z], s0);
            s1 = fma(v, wp[(size_t)k * d + z], s1);
        }
        A0[r * d + z] = s0;
        A1[r * d + z] = s1;
    }
}

// stage 2: contract y.  Block = (xp, z tile of ZT).
constexpr int kZT = 32;
__global__ void __launch_bounds__(256) k_fv_y(const FvGeom g, const AxisTables t, const double *A0, const double *A1,
                                              double *B0, double *B1, double *B2) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int S1 = g.S[1], d = g.d;
    const int xp = blockIdx.y, z0 = blockIdx.x * kZT;
    const int zn = min(kZT, d - z0);
    double *a0 = (double *)smem;
    double *a1 = a0 + (size_t)S1 * kZT;
    __shared__ int any;   // the tile holds a non-zero partial sum (planes outside the map hold none)
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < S1 * kZT; e += blockDim.x) {
        const int yp = e / kZT, zz = e - yp * kZT;
        const size_t gi = ((size_t)xp * S1 + yp) * d + z0 + zz;
        const double v0 = zz < zn ? A0[gi] : 0.0, v1 = zz < zn ? A1[gi] : 0.0;
        a0[e] = v0;
        a1[e] = v1;
        if (v0 != 0.0 || v1 != 0.0) any = 1;
    }
    __syncthreads();
    if (!any) {   // every sum is +0.0, as the loop below would give (A0, A1 >= +0.0)
        for (int o = threadIdx.x; o < d * kZT; o += blockDim.x) {
            const int y = o / kZT, zz = o - y * kZT;
            if (zz >= zn) continue;
            const size_t go = ((size_t)xp * d + y) * d + z0 + zz;
            B0[go] = 0.0;
            B1[go] = 0.0;
            B2[go] = 0.0;
        }
        return;
    }
    const int *stp = t.stp + d, *len = t.len + d;
    const double *w = t.w + (size_t)g.WB * d, *wp = t.wp + (size_t)g.WB * d;
    for (int o = threadIdx.x; o < d * kZT; o += blockDim.x) {
        const int y = o / kZT, zz = o - y * kZT;
        if (zz >= zn) continue;
        const int n = len[y], s = stp[y];
        double b0 = 0.0, b1 = 0.0, b2 = 0.0;
        for (int k = 0; k < n; ++k) {
            const double wy = __ldg(&w[(size_t)k * d + y]), wyp = __ldg(&wp[(size_t)k * d + y]);
            const double v0 = a0[(s + k) * kZT + zz], v1 = a1[(s + k) * kZT + zz];
            b0 = fma(wy, v0, b0);
            b1 = fma(wyp, v0, b1);
            b2 = fma(wy, v1, b2);
        }
        const size_t go = ((size_t)xp * d + y) * d + z0 + zz;
        B0[go] = b0;
        B1[go] = b1;
        B2[go] = b2;
    }
}

// stage 3: contract x and finish each voxel.  Block = (y, z tile of ZT/2).
constexpr int kZT3 = 16;
__global__ void __launch_bounds__(256) k_fv_x(const float *src, const FvGeom g, const AxisTables t, const double *B0,
                                              const double *B1, const double *B2, double *data_out, float *data_f32,
                                              float *vec_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int S0 = g.S[0], d = g.d;
    const int y = blockIdx.y, z0 = blockIdx.x * kZT3;
    const int zn = min(kZT3, d - z0);
    double *b0 = (double *)smem;
    double *b1 = b0 + (size_t)S0 * kZT3;
    double *b2 = b1 + (size_t)S0 * kZT3;
    for (int e = threadIdx.x; e < S0 * kZT3; e += blockDim.x) {
        const int xp = e / kZT3, zz = e - xp * kZT3;
        const size_t gi = ((size_t)xp * d + y) * d + z0 + zz;
        const bool ok = zz < zn;
        b0[e] = ok ? B0[gi] : 0.0;
        b1[e] = ok ? B1[gi] : 0.0;
        b2[e] = ok ? B2[gi] : 0.0;
    }
    __syncthreads();
    const int *stp = t.stp, *len = t.len;
    const double *w = t.w, *wp = t.wp;
    for (int o = threadIdx.x; o < d * kZT3; o += blockDim.x) {
        const int x = o / kZT3, zz = o - x * kZT3, z = z0 + zz;
        if (zz >= zn) continue;
        const size_t lin = ((size_t)x * d + y) * d + z;
        // skip tests (VESPER_1_prob_new.py:200-211)
        const int ix = t.idx[x], iy = t.idx[d + y], iz = t.idx[2 * d + z];
        bool valid = ix >= 0 && iy >= 0 && iz >= 0;
        if (valid) valid = src[((size_t)ix * g.S[1] + iy) * g.S[2] + iz] != 0.f;
        double dt = 0.0, px = 0.0, py = 0.0, pz = 0.0;
        if (valid) {
            const int n = len[x], s = stp[x];
            for (int k = 0; k < n; ++k) {
                const double wx = __ldg(&w[(size_t)k * d + x]), wxp = __ldg(&wp[(size_t)k * d + x]);
                const int e = (s + k) * kZT3 + zz;
                dt = fma(wx, b0[e], dt);
                px = fma(wxp, b0[e], px);
                py = fma(wx, b1[e], py);
                pz = fma(wx, b2[e], pz);
            }
        }
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        if (valid && dt != 0.0) {
            // VESPER_1_prob_new.py:242-255
            const double rd = __ddiv_rn(1.0, dt);
            const double t0 = __dsub_rn(__dmul_rn(px, rd), t.pos[x]);
            const double t1 = __dsub_rn(__dmul_rn(py, rd), t.pos[d + y]);
            const double t2 = __dsub_rn(__dmul_rn(pz, rd), t.pos[2 * d + z]);
            double dv = __dadd_rn(__dmul_rn(t0, t0), __dmul_rn(t1, t1));
            dv = __dsqrt_rn(__dadd_rn(dv, __dmul_rn(t2, t2)));
            if (dv == 0.0) dv = 1.0;
            const double rdv = __ddiv_rn(1.0, dv);
            v0 = (float)__dmul_rn(t0, rdv);
            v1 = (float)__dmul_rn(t1, rdv);
            v2 = (float)__dmul_rn(t2, rdv);
        }
        data_out[lin] = dt;
        if (data_f32) data_f32[lin] = (float)dt;
        vec_out[3 * lin + 0] = v0;
        vec_out[3 * lin + 1] = v1;
        vec_out[3 * lin + 2] = v2;
    }
}

// ---- float-float stages ---------------------------------------------------------

// stage 1a: list the source rows (xp, yp) that hold a non-zero value (one warp
// per row, any order: each row's sums are independent of the others) and mark
// their planes; an all-zero row's sums are +0.0, as the reference's loop gives,
// and are written here.
__global__ void __launch_bounds__(256) k_fvf_rows(const float *src, const FvGeom g, const AxisTables t,
                                                  float2 *A0, float2 *A1) {
    const int S1 = g.S[1], S2 = g.S[2], d = g.d;
    const size_t nrows = (size_t)g.S[0] * S1;
    const int lane = threadIdx.x & 31;
    for (size_t row = (size_t)blockIdx.x * 8 + (threadIdx.x >> 5); row < nrows; row += (size_t)gridDim.x * 8) {
        const float *rp = src + row * S2;
        bool nz = false;
        for (int e = lane; e < S2; e += 32) nz |= __ldg(rp + e) != 0.f;
        if (__any_sync(0xffffffffu, nz)) {
            if (lane == 0) {
                t.list[atomicAdd(t.nlist, 1)] = (int)row;
                t.plane[row / S1] = 1;
            }
        } else {
            for (int z = lane; z < d; z += 32) {
                A0[row * d + z] = make_float2(0.f, 0.f);
                A1[row * d + z] = make_float2(0.f, 0.f);
            }
        }
    }
}

// stage 1b (z).  Block b takes listed rows [b kZRows, (b + 1) kZRows), staged in
// shared memory with one extra all-zero row, together with the z axis's weight
// pairs when they fit (SW); each thread sums kFfRows of the rows for one output
// z, so every weight pair it loads serves kFfRows rows.  Blocks past the list's
// end return at once.
constexpr int kZRows = 16;
constexpr int kFfRows = 2;
constexpr int kFfBatch = 8;   // band entries loaded per round by the global-load forms
template <bool SW>
__global__ void __launch_bounds__(256) k_fvf_z(const float *src, const FvGeom g, const AxisTables t, float2 *A0,
                                               float2 *A1) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int S2 = g.S[2], d = g.d, WB = g.WB;
    const int first = blockIdx.x * kZRows;
    const int nr = min(kZRows, *t.nlist - first);
    if (nr <= 0) return;   // block-uniform
    float2 *sw = (float2 *)smem;                          // [WB][d] when SW
    float2 *swp = sw + (SW ? (size_t)WB * d : 0);         // [WB][d] when SW
    float *rows = (float *)(swp + (SW ? (size_t)WB * d : 0));   // [kZRows + 1][S2]
    const float2 *gw = t.wf + (size_t)2 * WB * d, *gwp = t.wpf + (size_t)2 * WB * d;
    if (SW)
        for (int e = threadIdx.x; e < WB * d; e += blockDim.x) {
            sw[e] = __ldg(gw + e);
            swp[e] = __ldg(gwp + e);
        }
#pragma unroll 4
    for (int e = threadIdx.x; e < (kZRows + 1) * S2; e += blockDim.x) {
        const int r = e / S2;
        rows[e] = r < nr ? __ldg(src + (size_t)t.list[first + r] * S2 + (e - r * S2)) : 0.f;
    }
    __syncthreads();
    const int ng = (nr + kFfRows - 1) / kFfRows;
    const int *stp = t.stp + 2 * d, *len = t.len + 2 * d;
    const float2 *w = SW ? sw : gw, *wp = SW ? swp : gwp;
    for (int it = threadIdx.x; it < ng * d; it += blockDim.x) {
        const int gi = it / d, z = it - gi * d;
        int off[kFfRows];
#pragma unroll
        for (int r = 0; r < kFfRows; ++r) {
            const int li = gi * kFfRows + r;
            off[r] = (li < nr ? li : kZRows) * S2 + stp[z];   // row kZRows is all zero
        }
        float s0h[kFfRows], s0l[kFfRows], s1h[kFfRows], s1l[kFfRows];
#pragma unroll
        for (int r = 0; r < kFfRows; ++r) s0h[r] = s0l[r] = s1h[r] = s1l[r] = 0.f;
        const int n = len[z];
#pragma unroll 2
        for (int k = 0; k < n; ++k) {
            const float2 a = w[(size_t)k * d + z], b = wp[(size_t)k * d + z];
#pragma unroll
            for (int r = 0; r < kFfRows; ++r) {
                const float v = rows[off[r] + k];
                float ph, pl;
                ff_mul_f(a.x, a.y, v, ph, pl);
                ff_add(s0h[r], s0l[r], ph, pl);
                ff_mul_f(b.x, b.y, v, ph, pl);
                ff_add(s1h[r], s1l[r], ph, pl);
            }
        }
#pragma unroll
        for (int r = 0; r < kFfRows; ++r) {
            const int li = gi * kFfRows + r;
            if (li < nr) {
                const size_t o = (size_t)t.list[first + li] * d + z;
                A0[o] = make_float2(s0h[r], s0l[r]);
                A1[o] = make_float2(s1h[r], s1l[r]);
            }
        }
    }
}

// stage 2 (y).  Block = (z tile of 32, source plane xp, chunk of yc consecutive
// outputs y); lanes over z, warp w sums outputs y0 + w, y0 + w + 8, ...  The
// rows of A0 and A1 that the chunk's bands cover (at most rmax, a bound the
// host derives from the geometry) and the chunk's weight pairs are first copied
// to shared memory with coalesced loads that are all in flight together; a
// block whose rows exceed rmax (rmax = 0: the slab does not fit) reads global
// memory instead, kFfBatch band entries per round.  A plane without a non-zero
// value gives +0.0.
__global__ void __launch_bounds__(256) k_fvf_y(const FvGeom g, const AxisTables t, int yc, int rmax,
                                               const float2 *A0, const float2 *A1, float2 *B0, float2 *B1,
                                               float2 *B2) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int S1 = g.S[1], d = g.d, WB = g.WB;
    const int z0 = blockIdx.x * 32, xp = blockIdx.y, y0 = blockIdx.z * yc;
    const int yn = min(yc, d - y0);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int z = z0 + lane;
    const int *stp = t.stp + d, *len = t.len + d;
    const float2 *wf = t.wf + (size_t)WB * d, *wpf = t.wpf + (size_t)WB * d;
    if (!t.plane[xp]) {
        for (int e = threadIdx.x; e < yn * 32; e += blockDim.x) {
            const int zz = z0 + (e & 31), y = y0 + (e >> 5);
            if (zz < d) {
                const size_t go = ((size_t)xp * d + y) * d + zz;
                B0[go] = B1[go] = B2[go] = make_float2(0.f, 0.f);
            }
        }
        return;
    }
    const int r0 = stp[y0];
    int r1 = r0;
    for (int y = y0; y < y0 + yn; ++y) r1 = max(r1, stp[y] + len[y]);
    const bool slab = r1 - r0 <= rmax;   // block-uniform
    float2 *s0 = (float2 *)smem;            // [rmax][32]
    float2 *s1 = s0 + (size_t)rmax * 32;    // [rmax][32]
    float2 *sw = s1 + (size_t)rmax * 32;    // [yc][WB]
    float2 *swp = sw + (size_t)yc * WB;     // [yc][WB]
    if (slab) {
#pragma unroll 4
        for (int e = threadIdx.x; e < (r1 - r0) * 32; e += blockDim.x) {
            const int r = e >> 5, zz = z0 + (e & 31);
            float2 v0 = make_float2(0.f, 0.f), v1 = v0;
            if (zz < d) {
                const size_t gi = ((size_t)xp * S1 + r0 + r) * d + zz;
                v0 = __ldg(A0 + gi);
                v1 = __ldg(A1 + gi);
            }
            s0[e] = v0;
            s1[e] = v1;
        }
        for (int e = threadIdx.x; e < yn * WB; e += blockDim.x) {
            const int yy = e / WB, k = e - yy * WB;
            sw[e] = __ldg(wf + (size_t)k * d + y0 + yy);
            swp[e] = __ldg(wpf + (size_t)k * d + y0 + yy);
        }
        __syncthreads();
    }
    for (int yy = wid; yy < yn; yy += 8) {
        const int y = y0 + yy;
        const int n = len[y], s = stp[y];
        float b0h = 0.f, b0l = 0.f, b1h = 0.f, b1l = 0.f, b2h = 0.f, b2l = 0.f;
        auto term = [&](float2 wy, float2 wyp, float2 v0, float2 v1) {
            float ph, pl;
            ff_mul(v0, wy, ph, pl);
            ff_add(b0h, b0l, ph, pl);
            ff_mul(v0, wyp, ph, pl);
            ff_add(b1h, b1l, ph, pl);
            ff_mul(v1, wy, ph, pl);
            ff_add(b2h, b2l, ph, pl);
        };
        if (slab) {
            const float2 *a0 = s0 + (size_t)(s - r0) * 32 + lane, *a1 = s1 + (size_t)(s - r0) * 32 + lane;
            const float2 *w = sw + (size_t)yy * WB, *wp = swp + (size_t)yy * WB;
#pragma unroll 2
            for (int k = 0; k < n; ++k) term(w[k], wp[k], a0[k * 32], a1[k * 32]);
        } else if (z < d) {
            const float2 *w = wf + y, *wp = wpf + y;
            const float2 *a0 = A0 + ((size_t)xp * S1 + s) * d + z, *a1 = A1 + ((size_t)xp * S1 + s) * d + z;
            int k = 0;
            for (; k + kFfBatch <= n; k += kFfBatch) {
                float2 wy[kFfBatch], wyp[kFfBatch], v0[kFfBatch], v1[kFfBatch];
#pragma unroll
                for (int u = 0; u < kFfBatch; ++u) {
                    const size_t o = (size_t)(k + u) * d;
                    wy[u] = __ldg(w + o);
                    wyp[u] = __ldg(wp + o);
                    v0[u] = __ldg(a0 + o);
                    v1[u] = __ldg(a1 + o);
                }
#pragma unroll
                for (int u = 0; u < kFfBatch; ++u) term(wy[u], wyp[u], v0[u], v1[u]);
            }
            for (; k < n; ++k) {
                const size_t o = (size_t)k * d;
                term(__ldg(w + o), __ldg(wp + o), __ldg(a0 + o), __ldg(a1 + o));
            }
        }
        if (z < d) {
            const size_t go = ((size_t)xp * d + y) * d + z;
            B0[go] = make_float2(b0h, b0l);
            B1[go] = make_float2(b1h, b1l);
            B2[go] = make_float2(b2h, b2l);
        }
    }
}

// stage 3 (x) and each voxel's finish.  Block = (z tile of 32, output y, chunk
// of xc consecutive outputs x); lanes over z, warp w sums outputs x0 + w, ...,
// from a shared-memory slab of B0, B1, B2 as in stage 2.
__global__ void __launch_bounds__(256) k_fvf_x(const float *src, const FvGeom g, const AxisTables t, int xc,
                                               int rmax, const float2 *B0, const float2 *B1, const float2 *B2,
                                               double *data_out, float *data_f32, float *vec_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int d = g.d, WB = g.WB;
    const int z0 = blockIdx.x * 32, y = blockIdx.y, x0 = blockIdx.z * xc;
    const int xn = min(xc, d - x0);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int z = z0 + lane;
    const int *stp = t.stp, *len = t.len;
    const size_t plane = (size_t)d * d;
    const int r0 = stp[x0];
    int r1 = r0;
    for (int x = x0; x < x0 + xn; ++x) r1 = max(r1, stp[x] + len[x]);
    const bool slab = r1 - r0 <= rmax;   // block-uniform
    float2 *s0 = (float2 *)smem;            // [rmax][32] each
    float2 *s1 = s0 + (size_t)rmax * 32;
    float2 *s2 = s1 + (size_t)rmax * 32;
    float2 *sw = s2 + (size_t)rmax * 32;    // [xc][WB]
    float2 *swp = sw + (size_t)xc * WB;     // [xc][WB]
    if (slab) {
#pragma unroll 4
        for (int e = threadIdx.x; e < (r1 - r0) * 32; e += blockDim.x) {
            const int r = e >> 5, zz = z0 + (e & 31);
            float2 v0 = make_float2(0.f, 0.f), v1 = v0, v2 = v0;
            if (zz < d) {
                const size_t gi = (size_t)(r0 + r) * plane + (size_t)y * d + zz;
                v0 = __ldg(B0 + gi);
                v1 = __ldg(B1 + gi);
                v2 = __ldg(B2 + gi);
            }
            s0[e] = v0;
            s1[e] = v1;
            s2[e] = v2;
        }
        for (int e = threadIdx.x; e < xn * WB; e += blockDim.x) {
            const int xx = e / WB, k = e - xx * WB;
            sw[e] = __ldg(t.wf + (size_t)k * d + x0 + xx);
            swp[e] = __ldg(t.wpf + (size_t)k * d + x0 + xx);
        }
        __syncthreads();
    }
    if (z >= d) return;   // no barrier below
    for (int xx = wid; xx < xn; xx += 8) {
        const int x = x0 + xx;
        // skip tests (VESPER_1_prob_new.py:200-211)
        const int ix = t.idx[x], iy = t.idx[d + y], iz = t.idx[2 * d + z];
        bool valid = ix >= 0 && iy >= 0 && iz >= 0;
        if (valid) valid = src[((size_t)ix * g.S[1] + iy) * g.S[2] + iz] != 0.f;
        float dh = 0.f, dl = 0.f, xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f, zh = 0.f, zl = 0.f;
        auto term = [&](float2 wx, float2 wxp, float2 v0, float2 v1, float2 v2) {
            float ph, pl;
            ff_mul(v0, wx, ph, pl);
            ff_add(dh, dl, ph, pl);
            ff_mul(v0, wxp, ph, pl);
            ff_add(xh, xl, ph, pl);
            ff_mul(v1, wx, ph, pl);
            ff_add(yh, yl, ph, pl);
            ff_mul(v2, wx, ph, pl);
            ff_add(zh, zl, ph, pl);
        };
        const int n = len[x], s = stp[x];
        if (valid && slab) {
            const size_t o = (size_t)(s - r0) * 32 + lane;
            const float2 *v0 = s0 + o, *v1 = s1 + o, *v2 = s2 + o;
            const float2 *w = sw + (size_t)xx * WB, *wp = swp + (size_t)xx * WB;
#pragma unroll 2
            for (int k = 0; k < n; ++k) term(w[k], wp[k], v0[k * 32], v1[k * 32], v2[k * 32]);
        } else if (valid) {
            const float2 *w = t.wf + x, *wp = t.wpf + x;
            const size_t b = (size_t)s * plane + (size_t)y * d + z;
            int k = 0;
            for (; k + kFfBatch <= n; k += kFfBatch) {
                float2 wx[kFfBatch], wxp[kFfBatch], v0[kFfBatch], v1[kFfBatch], v2[kFfBatch];
#pragma unroll
                for (int u = 0; u < kFfBatch; ++u) {
                    const size_t e = b + (size_t)(k + u) * plane;
                    wx[u] = __ldg(w + (size_t)(k + u) * d);
                    wxp[u] = __ldg(wp + (size_t)(k + u) * d);
                    v0[u] = __ldg(B0 + e);
                    v1[u] = __ldg(B1 + e);
                    v2[u] = __ldg(B2 + e);
                }
#pragma unroll
                for (int u = 0; u < kFfBatch; ++u) term(wx[u], wxp[u], v0[u], v1[u], v2[u]);
            }
            for (; k < n; ++k) {
                const size_t e = b + (size_t)k * plane;
                term(__ldg(w + (size_t)k * d), __ldg(wp + (size_t)k * d), __ldg(B0 + e), __ldg(B1 + e),
                     __ldg(B2 + e));
            }
        }
        const double dt = valid ? (double)dh + (double)dl : 0.0;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        if (valid && dt != 0.0) {
            // VESPER_1_prob_new.py:242-255
            const double px = (double)xh + (double)xl, py = (double)yh + (double)yl, pz = (double)zh + (double)zl;
            const double rd = __ddiv_rn(1.0, dt);
            const double t0 = __dsub_rn(__dmul_rn(px, rd), t.pos[x]);
            const double t1 = __dsub_rn(__dmul_rn(py, rd), t.pos[d + y]);
            const double t2 = __dsub_rn(__dmul_rn(pz, rd), t.pos[2 * d + z]);
            double dv = __dadd_rn(__dmul_rn(t0, t0), __dmul_rn(t1, t1));
            dv = __dsqrt_rn(__dadd_rn(dv, __dmul_rn(t2, t2)));
            if (dv == 0.0) dv = 1.0;
            const double rdv = __ddiv_rn(1.0, dv);
            v0 = (float)__dmul_rn(t0, rdv);
            v1 = (float)__dmul_rn(t1, rdv);
            v2 = (float)__dmul_rn(t2, rdv);
        }
        const size_t lin = ((size_t)x * d + y) * d + z;
        data_out[lin] = dt;
        if (data_f32) data_f32[lin] = (float)dt;
        vec_out[3 * lin + 0] = v0;
        vec_out[3 * lin + 1] = v1;
        vec_out[3 * lin + 2] = v2;
    }
}

// smallest band weight of the geometry (|r| <= fmaxd + 1 on each axis)
static bool fv_float_float(const FvGeom &g) {
    const double r = g.fmaxd + 1.0;
    return std::exp(-1.5 * r * r * g.fsiv) >= 0x1p-70;
}

// chunk size and slab rows of the y and x stages: the chunk's bands cover at
// most WB + floor((c - 1) dw / sw) + 1 source rows (stp is non-decreasing in
// the output index and steps by at most floor(dw / sw) + 1); c = 8 outputs per
// block, fewer while the slab exceeds 100 KB; rmax = 0 (global loads) when even
// one output's band does not fit
static void fvf_chunk(const FvGeom &g, int S, int narr, int *c, int *rmax, size_t *bytes) {
    for (int cc = 8; cc >= 1; cc /= 2) {
        const int r = std::min(S, g.WB + (int)((cc - 1) * g.dw / g.sw) + 2);
        const size_t b = ((size_t)narr * r * 32 + 2 * (size_t)cc * g.WB) * sizeof(float2);
        if (b <= 100 * 1024 || (cc == 1 && b <= 200 * 1024)) {
            *c = cc;
            *rmax = r;
            *bytes = b;
            return;
        }
    }
    *c = 8;
    *rmax = 0;
    *bytes = 0;
}

static void fv_geom(int sx, int sy, int sz, double src_width, const double *src_orig, int dim, double dest_width,
                    const double *dest_orig, double dreso, FvGeom *g) {
    g->S[0] = sx;
    g->S[1] = sy;
    g->S[2] = sz;
    g->d = dim;
    g->sw = src_width;
    g->dw = dest_width;
    // VESPER_1_prob_new.py:183-187
    volatile double q = dreso / src_width;
    double fs = q * 0.5;
    fs = fs * fs;
    g->fsiv = 1.0 / fs;
    g->fmaxd = q * 2.0;
    g->WB = (int)(2.0 * g->fmaxd) + 3;
    for (int a = 0; a < 3; ++a) {
        g->sorig[a] = src_orig[a];
        g->dorig[a] = dest_orig[a];
    }
}

static size_t fv_workspace(const FvGeom &g, AxisTables *t, double **A0, double **A1, double **B0, double **B1,
                           double **B2, void *base, size_t cap) {
    Carver cv(base, cap);
    const int d = g.d;
    t->pos = cv.take<double>(3 * (size_t)d);
    t->stp = cv.take<int>(3 * (size_t)d);
    t->len = cv.take<int>(3 * (size_t)d);
    t->idx = cv.take<int>(3 * (size_t)d);
    t->w = cv.take<double>(3 * (size_t)g.WB * d);
    t->wp = cv.take<double>(3 * (size_t)g.WB * d);
    t->wf = cv.take<float2>(3 * (size_t)g.WB * d);
    t->wpf = cv.take<float2>(3 * (size_t)g.WB * d);
    t->plane = cv.take<int>((size_t)g.S[0]);
    t->list = cv.take<int>((size_t)g.S[0] * g.S[1]);
    t->nlist = cv.take<int>(1);
    // the partial sums: float64, or float-float pairs of the same 8 bytes
    const size_t rows = (size_t)g.S[0] * g.S[1];
    *A0 = cv.take<double>(rows * d);
    *A1 = cv.take<double>(rows * d);
    *B0 = cv.take<double>((size_t)g.S[0] * d * d);
    *B1 = cv.take<double>((size_t)g.S[0] * d * d);
    *B2 = cv.take<double>((size_t)g.S[0] * d * d);
    return cv.off + 256;
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_fastvec_workspace_size(int sx, int sy, int sz, int dim, size_t *bytes) {
    if (!bytes || sx < 1 || sy < 1 || sz < 1 || dim < 1)
        return fail(VESPER_ERR_INVALID, "vesper_fastvec_workspace_size: bad arguments");
    // the band width depends on dreso / src_width; size for the widest band the
    // caller can ask for below (fmaxd <= 512 source voxels)
    FvGeom g{};
    g.S[0] = sx;
    g.S[1] = sy;
    g.S[2] = sz;
    g.d = dim;
    g.WB = 2 * 512 + 3;
    AxisTables t;
    double *a0, *a1, *b0, *b1, *b2;
    *bytes = fv_workspace(g, &t, &a0, &a1, &b0, &b1, &b2, nullptr, 0);
    return VESPER_OK;
}

extern "C" int vesper_fastvec(const float *src, int sx, int sy, int sz, double src_width, const double *src_orig,
                              int dim, double dest_width, const double *dest_orig, double dreso, double *data_out,
                              float *data_f32, float *vec_out, void *workspace, size_t workspace_bytes,
                              void *stream) {
    if (!src || !src_orig || !dest_orig || !data_out || !vec_out)
        return fail(VESPER_ERR_INVALID, "vesper_fastvec: missing pointer");
    if (sx < 1 || sy < 1 || sz < 1 || dim < 1) return fail(VESPER_ERR_INVALID, "vesper_fastvec: bad sizes");
    if (!(src_width > 0) || !(dreso > 0)) return fail(VESPER_ERR_INVALID, "vesper_fastvec: bad widths");
    FvGeom g;
    fv_geom(sx, sy, sz, src_width, src_orig, dim, dest_width, dest_orig, dreso, &g);
    if (g.fmaxd > 512.0) return fail(VESPER_ERR_UNSUPPORTED, "vesper_fastvec: window %.1f voxels too wide", g.fmaxd);
    AxisTables t;
    double *A0, *A1, *B0, *B1, *B2;
    const size_t need = fv_workspace(g, &t, &A0, &A1, &B0, &B1, &B2, workspace, workspace_bytes);
    if (!workspace || workspace_bytes < need)
        return fail(VESPER_ERR_WORKSPACE, "vesper_fastvec: workspace %zu < %zu bytes", workspace_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    k_fv_tables<<<dim3(dim, 3), 128, 0, st>>>(g, t);
    VG_CHECK_LAUNCH("k_fv_tables");
    const size_t nrows = (size_t)sx * sy;
    if (fv_float_float(g)) {
        const size_t srows = (size_t)(kZRows + 1) * sz * sizeof(float);
        const size_t sweights = 2 * (size_t)g.WB * dim * sizeof(float2);
        const bool zsw = srows + sweights <= 100 * 1024;   // the z weights staged in shared memory
        const size_t s1 = srows + (zsw ? sweights : 0);
        if (s1 > 200 * 1024) return fail(VESPER_ERR_UNSUPPORTED, "vesper_fastvec: source rows too long (%d)", sz);
        float2 *a0 = reinterpret_cast<float2 *>(A0), *a1 = reinterpret_cast<float2 *>(A1);
        float2 *b0 = reinterpret_cast<float2 *>(B0), *b1 = reinterpret_cast<float2 *>(B1),
               *b2 = reinterpret_cast<float2 *>(B2);
        k_fvf_rows<<<(unsigned)std::min<size_t>((nrows + 7) / 8, 4096), 256, 0, st>>>(src, g, t, a0, a1);
        VG_CHECK_LAUNCH("k_fvf_rows");
        const unsigned zb = (unsigned)((nrows + kZRows - 1) / kZRows);
        if (zsw) {
            allow_smem(k_fvf_z<true>, s1);
            k_fvf_z<true><<<zb, 256, s1, st>>>(src, g, t, a0, a1);
        } else {
            allow_smem(k_fvf_z<false>, s1);
            k_fvf_z<false><<<zb, 256, s1, st>>>(src, g, t, a0, a1);
        }
        VG_CHECK_LAUNCH("k_fvf_z");
        const unsigned zt = (unsigned)((dim + 31) / 32);
        int yc, ry, xc, rx;
        size_t sy2, sx3;
        fvf_chunk(g, sy, 2, &yc, &ry, &sy2);
        fvf_chunk(g, sx, 3, &xc, &rx, &sx3);
        allow_smem(k_fvf_y, sy2);
        k_fvf_y<<<dim3(zt, sx, (unsigned)((dim + yc - 1) / yc)), 256, sy2, st>>>(g, t, yc, ry, a0, a1, b0, b1, b2);
        VG_CHECK_LAUNCH("k_fvf_y");
        allow_smem(k_fvf_x, sx3);
        k_fvf_x<<<dim3(zt, dim, (unsigned)((dim + xc - 1) / xc)), 256, sx3, st>>>(src, g, t, xc, rx, b0, b1, b2,
                                                                                  data_out, data_f32, vec_out);
        VG_CHECK_LAUNCH("k_fvf_x");
        return VESPER_OK;
    }
    const size_t s1 = (size_t)kRB * sz * sizeof(float);
    if (s1 > 200 * 1024) return fail(VESPER_ERR_UNSUPPORTED, "vesper_fastvec: source rows too long (%d)", sz);
    allow_smem(k_fv_z, s1);
    k_fv_z<<<(unsigned)((nrows + kRB - 1) / kRB), 256, s1, st>>>(src, g, t, A0, A1);
    VG_CHECK_LAUNCH("k_fv_z");
    const size_t s2 = 2 * (size_t)sy * kZT * sizeof(double);
    const size_t s3 = 3 * (size_t)sx * kZT3 * sizeof(double);
    if (s2 > 220 * 1024 || s3 > 220 * 1024)
        return fail(VESPER_ERR_UNSUPPORTED, "vesper_fastvec: source side too large (%d, %d)", sx, sy);
    allow_smem(k_fv_y, s2);
    k_fv_y<<<dim3((dim + kZT - 1) / kZT, sx), 256, s2, st>>>(g, t, A0, A1, B0, B1, B2);
    VG_CHECK_LAUNCH("k_fv_y");
    allow_smem(k_fv_x, s3);
    k_fv_x<<<dim3((dim + kZT3 - 1) / kZT3, dim), 256, s3, st>>>(src, g, t, B0, B1, B2, data_out, data_f32, vec_out);
    VG_CHECK_LAUNCH("k_fv_x");
    return VESPER_OK;
}
