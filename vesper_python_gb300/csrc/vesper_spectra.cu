// Target spectra (float64, once per pair) and the stable top-N.
#include <algorithm>

#include "vesper_common.cuh"

namespace vg {

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
    // Laplacian (laplacian_filter, :494-526)
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

// z (R2C, paired rows) and y passes per (x plane, channel).
struct TargetA {
    Query q;
    int H;
    FftPlan P;
    double2 *S;
};

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

// x pass, conjugate, round to complex64.
struct TargetB {
    const double2 *S;
    float2 *T;
    int d, H, W;
    FftPlan P;
};

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

// Stable top-N over strided scores: N rounds of a block-wide (score, -index)
// maximum, chosen indices masked in a shared bitmap.
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

static int pick_target_w(int d) {
    const size_t lim = (size_t)smem_limit();
    for (int W : {16, 8, 4, 2, 1})
        if (smem_target_b(d, W) <= lim / 2 - 1024) return W;
    return 1;
}

}  // namespace vg

using namespace vg;

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
    if (mode < 0 || mode > VESPER_MODE_PROB) return fail(VESPER_ERR_INVALID, "unknown mode %d", mode);
    FftPlan P;
    if (dim < 2 || !make_plan(dim, &P))
        return fail(VESPER_ERR_UNSUPPORTED, "grid side %d is not 2^a3^b5^c7^d(11|13)", dim);
    const int H = dim / 2 + 1, nch = mode_nch(mode);
    if (smem_target_a(dim, H) > (size_t)smem_limit())
        return fail(VESPER_ERR_UNSUPPORTED, "grid side %d too large for the target pass", dim);
    const bool need_vec = mode == VESPER_MODE_VEC || mode == VESPER_MODE_PROB;
    if ((need_vec && !vec) || (!need_vec && !data) || (mode == VESPER_MODE_PROB && !probs) || !spectra_out)
        return fail(VESPER_ERR_INVALID, "vesper_target_spectra: missing input or output pointer");
    size_t need = 0;
    vesper_target_workspace_size(dim, mode, &need);
    if (!workspace || workspace_bytes < need)
        return fail(VESPER_ERR_WORKSPACE, "vesper_target_spectra: workspace %zu < %zu bytes", workspace_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
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
