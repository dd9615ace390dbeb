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
// in float64, with w = exp(-1.5 r^2 fsiv) per axis (the product of the three
// per-axis factors is the reference's exp of the sum up to rounding).  The
// per-voxel skip tests (pos inside the source, src[int(pos)] != 0) and the
// normalisation follow the reference operation by operation.
//
// Cost: S0 S1 d WB + S0 d^2 WB + d^3 WB multiply-adds (x2..4) instead of
// d^3 WB^3 exponentials, WB = band width <= 2 fmaxd + 2.
#include <algorithm>

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
        t.w[wo] = w;
        t.wp[wo] = __dmul_rn(w, (double)(stp + k));
    }
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
    const size_t s1 = (size_t)kRB * sz * sizeof(float);
    if (s1 > 200 * 1024) return fail(VESPER_ERR_UNSUPPORTED, "vesper_fastvec: source rows too long (%d)", sz);
    cudaFuncSetAttribute(k_fv_z, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1);
    k_fv_z<<<(unsigned)((nrows + kRB - 1) / kRB), 256, s1, st>>>(src, g, t, A0, A1);
    VG_CHECK_LAUNCH("k_fv_z");
    const size_t s2 = 2 * (size_t)sy * kZT * sizeof(double);
    const size_t s3 = 3 * (size_t)sx * kZT3 * sizeof(double);
    if (s2 > 220 * 1024 || s3 > 220 * 1024)
        return fail(VESPER_ERR_UNSUPPORTED, "vesper_fastvec: source side too large (%d, %d)", sx, sy);
    cudaFuncSetAttribute(k_fv_y, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2);
    k_fv_y<<<dim3((dim + kZT - 1) / kZT, sx), 256, s2, st>>>(g, t, A0, A1, B0, B1, B2);
    VG_CHECK_LAUNCH("k_fv_y");
    cudaFuncSetAttribute(k_fv_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s3);
    k_fv_x<<<dim3((dim + kZT3 - 1) / kZT3, dim), 256, s3, st>>>(src, g, t, B0, B1, B2, data_out, data_f32, vec_out);
    VG_CHECK_LAUNCH("k_fv_x");
    return VESPER_OK;
}
