// Materialised rotation of the query map (rot_mrc / rot_mrc_prob) and the
// float64 final-model scoring (get_score).
#include "vesper_common.cuh"

namespace vg {

// One destination voxel per thread, rotation r = blockIdx.y.
// VESPER_1_prob_new.py:279-354 (rot_mrc) and :1211-1299 (rot_mrc_prob).
__global__ void k_rot_gather(const double *data, const float *vec, const float *probs, int d, const float *rotmats,
                             double *data_out, float *vec_out, float *probs_out) {
    __shared__ float F[9];
    const int r = blockIdx.y;
    if (threadIdx.x < 9) F[threadIdx.x] = rotmats[(size_t)r * 9 + threadIdx.x];
    __syncthreads();
    const size_t vol = (size_t)d * d * d;
    const size_t lin = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (lin >= vol) return;
    const int z = (int)(lin % d), y = (int)((lin / d) % d), x = (int)(lin / ((size_t)d * d));
    const int s = gather_src(F, d, x, y, z, [data](int i) { return data[i] != 0.0; });
    double dv = 0.0;
    float o[3] = {0.f, 0.f, 0.f};
    if (s >= 0) {
        dv = data[s];
        rotate_vec(F, vec[3 * (size_t)s], vec[3 * (size_t)s + 1], vec[3 * (size_t)s + 2], o);
    }
    data_out[(size_t)r * vol + lin] = dv;
    float *vo = vec_out + ((size_t)r * vol + lin) * 3;
    vo[0] = o[0];
    vo[1] = o[1];
    vo[2] = o[2];
    if (probs) {
        for (int k = 0; k < 4; ++k) {
            const float *p = probs + k * vol;
            const int sp = gather_src(F, d, x, y, z, [p](int i) { return p[i] != 0.f; });
            probs_out[((size_t)r * 4 + k) * vol + lin] = sp >= 0 ? p[sp] : 0.f;
        }
    }
}

// ---------------------------------------------------------------------------
// get_score (VESPER_1_prob_new.py:1302-1393) in float64, one block per call.
// ---------------------------------------------------------------------------
constexpr int kRsThreads = 1024;

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        red[32] = s;
    }
    __syncthreads();
    return red[32];
}

struct RescoreArgs {
    const double *tdata;
    const float *tvec;
    double tave, tstd, tstd_norm_ave;
    const double *sdata;
    const float *svec;
    int d, tx, ty, tz;
    double *result;
    double *sco;
};

__global__ void __launch_bounds__(kRsThreads) k_rescore(const RescoreArgs a) {
    __shared__ double red[33];
    const int d = a.d;
    const size_t vol = (size_t)d * d * d;
    // search-map statistics over data > 0 (:1312-1318)
    double n2 = 0.0, s2 = 0.0, q2 = 0.0, nt = 0.0;
    for (size_t i = threadIdx.x; i < vol; i += blockDim.x) {
        const double v = a.sdata[i];
        if (v > 0) {
            n2 += 1.0;
            s2 += v;
            q2 += v * v;
        }
        if (a.tdata[i] != 0.0) nt += 1.0;
    }
    n2 = block_sum(n2, red);
    s2 = block_sum(s2, red);
    q2 = block_sum(q2, red);
    nt = block_sum(nt, red);
    const double ave2 = s2 / n2;
    const double std2 = sqrt(q2);
    double p2 = 0.0;
    for (size_t i = threadIdx.x; i < vol; i += blockDim.x) {
        const double v = a.sdata[i];
        if (v > 0) p2 += (v - ave2) * (v - ave2);
    }
    p2 = block_sum(p2, red);
    const double pstd2 = sqrt(p2);
    // overlap terms (:1333-1379): target voxel p, search voxel p + t
    double cc = 0.0, pcc = 0.0, nm = 0.0, extra = 0.0, score = 0.0;
    for (size_t i = threadIdx.x; i < vol; i += blockDim.x) {
        const int z = (int)(i % d), y = (int)((i / d) % d), x = (int)(i / ((size_t)d * d));
        const int sx = x + a.tx, sy = y + a.ty, sz = z + a.tz;
        if (sx < 0 || sy < 0 || sz < 0 || sx >= d || sy >= d || sz >= d) continue;
        const size_t j = ((size_t)sx * d + sy) * d + sz;
        const double t = a.tdata[i], s = a.sdata[j];
        const double d1 = t <= 0 ? 0.0 : t;
        const double d2 = s <= 0 ? 0.0 : d1;   // the reference's d2 = where(d2 <= 0, 0, d1)
        const double pd1 = d1 <= 0 ? 0.0 : d1 - a.tave;
        const double pd2 = d2 <= 0 ? 0.0 : d2 - ave2;
        cc += d1 * d2;
        pcc += pd1 * pd2;
        if (t > 0 && s > 0) nm += 1.0;
        if (t == 0 && s > 0) extra += 1.0;
        const double dot = (double)a.tvec[3 * i] * (double)a.svec[3 * j] +
                           (double)a.tvec[3 * i + 1] * (double)a.svec[3 * j + 1] +
                           (double)a.tvec[3 * i + 2] * (double)a.svec[3 * j + 2];
        score += dot;
        if (a.sco) a.sco[j] = dot;
    }
    cc = block_sum(cc, red);
    pcc = block_sum(pcc, red);
    nm = block_sum(nm, red);
    extra = block_sum(extra, red);
    score = block_sum(score, red);
    if (threadIdx.x == 0) {
        a.result[0] = nm;
        a.result[1] = nt + extra;
        a.result[2] = cc / (a.tstd * std2);
        a.result[3] = pcc / (a.tstd_norm_ave * pstd2);
        a.result[4] = score;
        a.result[5] = ave2;
        a.result[6] = std2;
        a.result[7] = pstd2;
    }
}

// ---- the same scores over many blocks and many models ---------------------------
// Model m = blockIdx.y, voxel chunk b = blockIdx.x.  Phase 1 sums the search
// map's statistics per chunk; a one-block reduction per model adds the chunks
// in chunk order (deterministic) and derives ave2/std2; phase 2 sums the
// centred norm and the overlap terms per chunk; a second reduction forms the
// result.  Per-voxel arithmetic is that of k_rescore.
constexpr int kRbThreads = 256;
constexpr int kRbVoxPerThread = 8;
constexpr int kRbParts = 6;   // doubles per chunk and model in the workspace

struct RescoreBatchArgs {
    const double *tdata;
    const float *tvec;
    double tave, tstd, tstd_norm_ave;
    const double *sdata;   // [nmodel][vol]
    const float *svec;     // [nmodel][vol][3]
    int d, nmodel, nchunk;
    const int32_t *trans;  // DEVICE [nmodel][3], already wrapped; NULL: (tx, ty, tz)
    int tx, ty, tz;
    double *part;          // [nmodel][nchunk][kRbParts]
    double *stats;         // [nmodel][4]: n2, ave2, std2, nt
    double *result;        // [nmodel][8]
    double *sco;           // [vol] (nmodel == 1 only) or NULL
    const double *tstats;  // DEVICE vesper_map_stats layout of the target, or NULL: tave/tstd/tstd_norm_ave
};

// Target statistics: from device memory when given (so that a captured call
// replays with new maps), else the host values.
__device__ __forceinline__ double rb_tave(const RescoreBatchArgs &a) { return a.tstats ? a.tstats[2] : a.tave; }
__device__ __forceinline__ double rb_tstd(const RescoreBatchArgs &a) { return a.tstats ? a.tstats[3] : a.tstd; }
__device__ __forceinline__ double rb_tpstd(const RescoreBatchArgs &a) {
    return a.tstats ? a.tstats[4] : a.tstd_norm_ave;
}

__device__ __forceinline__ void rb_chunk(const RescoreBatchArgs &a, size_t &lo, size_t &hi) {
    const size_t vol = (size_t)a.d * a.d * a.d;
    const size_t per = (size_t)kRbThreads * kRbVoxPerThread;
    lo = (size_t)blockIdx.x * per;
    hi = lo + per < vol ? lo + per : vol;
}

__global__ void __launch_bounds__(kRbThreads) k_rescore_p1(const RescoreBatchArgs a) {
    __shared__ double red[33];
    const int m = blockIdx.y;
    const size_t vol = (size_t)a.d * a.d * a.d;
    const double *sd = a.sdata + (size_t)m * vol;
    size_t lo, hi;
    rb_chunk(a, lo, hi);
    double n2 = 0.0, s2 = 0.0, q2 = 0.0, nt = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double v = sd[i];
        if (v > 0) {
            n2 += 1.0;
            s2 += v;
            q2 += v * v;
        }
        if (a.tdata[i] != 0.0) nt += 1.0;
    }
    n2 = block_sum(n2, red);
    s2 = block_sum(s2, red);
    q2 = block_sum(q2, red);
    nt = block_sum(nt, red);
    if (threadIdx.x == 0) {
        double *p = a.part + ((size_t)m * a.nchunk + blockIdx.x) * kRbParts;
        p[0] = n2;
        p[1] = s2;
        p[2] = q2;
        p[3] = nt;
    }
}

__global__ void k_rescore_r1(const RescoreBatchArgs a) {
    const int m = blockIdx.x;
    if (threadIdx.x != 0) return;
    double n2 = 0.0, s2 = 0.0, q2 = 0.0, nt = 0.0;
    for (int b = 0; b < a.nchunk; ++b) {
        const double *p = a.part + ((size_t)m * a.nchunk + b) * kRbParts;
        n2 += p[0];
        s2 += p[1];
        q2 += p[2];
        nt += p[3];
    }
    double *st = a.stats + (size_t)m * 4;
    st[0] = n2;
    st[1] = s2 / n2;
    st[2] = sqrt(q2);
    st[3] = nt;
}

__global__ void __launch_bounds__(kRbThreads) k_rescore_p2(const RescoreBatchArgs a) {
    __shared__ double red[33];
    const int m = blockIdx.y, d = a.d;
    const size_t vol = (size_t)d * d * d;
    const double *sd = a.sdata + (size_t)m * vol;
    const float *sv = a.svec + (size_t)m * vol * 3;
    const double ave2 = a.stats[(size_t)m * 4 + 1];
    const double tave = rb_tave(a);
    const int tx = a.trans ? a.trans[3 * m] : a.tx, ty = a.trans ? a.trans[3 * m + 1] : a.ty,
              tz = a.trans ? a.trans[3 * m + 2] : a.tz;
    size_t lo, hi;
    rb_chunk(a, lo, hi);
    double p2 = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double v = sd[i];
        if (v > 0) p2 += (v - ave2) * (v - ave2);
    }
    double cc = 0.0, pcc = 0.0, nm = 0.0, extra = 0.0, score = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int z = (int)(i % d), y = (int)((i / d) % d), x = (int)(i / ((size_t)d * d));
        const int sx = x + tx, sy = y + ty, sz = z + tz;
        if (sx < 0 || sy < 0 || sz < 0 || sx >= d || sy >= d || sz >= d) continue;
        const size_t j = ((size_t)sx * d + sy) * d + sz;
        const double t = a.tdata[i], s = sd[j];
        const double d1 = t <= 0 ? 0.0 : t;
        const double d2 = s <= 0 ? 0.0 : d1;   // the reference's d2 = where(d2 <= 0, 0, d1)
        const double pd1 = d1 <= 0 ? 0.0 : d1 - tave;
        const double pd2 = d2 <= 0 ? 0.0 : d2 - ave2;
        cc += d1 * d2;
        pcc += pd1 * pd2;
        if (t > 0 && s > 0) nm += 1.0;
        if (t == 0 && s > 0) extra += 1.0;
        const double dot = (double)a.tvec[3 * i] * (double)sv[3 * j] + (double)a.tvec[3 * i + 1] * (double)sv[3 * j + 1] +
                           (double)a.tvec[3 * i + 2] * (double)sv[3 * j + 2];
        score += dot;
        if (a.sco) a.sco[j] = dot;
    }
    p2 = block_sum(p2, red);
    cc = block_sum(cc, red);
    pcc = block_sum(pcc, red);
    nm = block_sum(nm, red);
    extra = block_sum(extra, red);
    score = block_sum(score, red);
    if (threadIdx.x == 0) {
        double *p = a.part + ((size_t)m * a.nchunk + blockIdx.x) * kRbParts;
        p[0] = p2;
        p[1] = cc;
        p[2] = pcc;
        p[3] = nm;
        p[4] = extra;
        p[5] = score;
    }
}

__global__ void k_rescore_r2(const RescoreBatchArgs a) {
    const int m = blockIdx.x;
    if (threadIdx.x != 0) return;
    double acc[kRbParts] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < a.nchunk; ++b) {
        const double *p = a.part + ((size_t)m * a.nchunk + b) * kRbParts;
        for (int k = 0; k < kRbParts; ++k) acc[k] += p[k];
    }
    const double *st = a.stats + (size_t)m * 4;
    const double pstd2 = sqrt(acc[0]);
    double *r = a.result + (size_t)m * 8;
    r[0] = acc[3];
    r[1] = st[3] + acc[4];
    r[2] = acc[1] / (rb_tstd(a) * st[2]);
    r[3] = acc[2] / (rb_tpstd(a) * pstd2);
    r[4] = acc[5];
    r[5] = st[1];
    r[6] = st[2];
    r[7] = pstd2;
}

static size_t rescore_chunks(int dim) {
    const size_t vol = (size_t)dim * dim * dim;
    const size_t per = (size_t)kRbThreads * kRbVoxPerThread;
    return (vol + per - 1) / per;
}

static int launch_rescore_batch(RescoreBatchArgs a, cudaStream_t st) {
    const dim3 g((unsigned)a.nchunk, (unsigned)a.nmodel);
    k_rescore_p1<<<g, kRbThreads, 0, st>>>(a);
    VG_CHECK_LAUNCH("k_rescore_p1");
    k_rescore_r1<<<a.nmodel, 32, 0, st>>>(a);
    VG_CHECK_LAUNCH("k_rescore_r1");
    k_rescore_p2<<<g, kRbThreads, 0, st>>>(a);
    VG_CHECK_LAUNCH("k_rescore_p2");
    k_rescore_r2<<<a.nmodel, 32, 0, st>>>(a);
    VG_CHECK_LAUNCH("k_rescore_r2");
    return VESPER_OK;
}

__global__ void k_zero_f64(double *p, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = 0.0;
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_rot_gather(const double *data, const float *vec, const float *probs, int dim,
                                 const float *rotmats, int nrot, double *data_out, float *vec_out, float *probs_out,
                                 void *stream) {
    if (!data || !vec || !rotmats || !data_out || !vec_out || (probs && !probs_out))
        return fail(VESPER_ERR_INVALID, "vesper_rot_gather: missing pointer");
    if (dim < 1 || dim > 1024 || nrot < 0) return fail(VESPER_ERR_INVALID, "vesper_rot_gather: bad sizes");
    if (nrot == 0) return VESPER_OK;
    const size_t vol = (size_t)dim * dim * dim;
    k_rot_gather<<<dim3((unsigned)((vol + 255) / 256), nrot), 256, 0, (cudaStream_t)stream>>>(
        data, vec, probs, dim, rotmats, data_out, vec_out, probs_out);
    VG_CHECK_LAUNCH("k_rot_gather");
    return VESPER_OK;
}

extern "C" int vesper_rescore_batch_workspace_size(int dim, int nmodel, size_t *bytes) {
    if (!bytes) return fail(VESPER_ERR_INVALID, "bytes is NULL");
    if (dim < 1 || nmodel < 0) return fail(VESPER_ERR_INVALID, "vesper_rescore_batch_workspace_size: bad sizes");
    *bytes = ((size_t)nmodel * rescore_chunks(dim) * kRbParts + (size_t)nmodel * 4) * sizeof(double) + 256;
    return VESPER_OK;
}

extern "C" int vesper_rescore_workspace_size(int dim, size_t *bytes) {
    return vesper_rescore_batch_workspace_size(dim, 1, bytes);
}

extern "C" int vesper_rescore_batch(const double *tdata, const float *tvec, double tave, double tstd,
                                    double tstd_norm_ave, const double *sdata, const float *svec, int dim,
                                    const int32_t *trans_dev, int nmodel, double *result_out, void *workspace,
                                    size_t workspace_bytes, void *stream) {
    if (!tdata || !tvec || !sdata || !svec || !trans_dev || !result_out)
        return fail(VESPER_ERR_INVALID, "vesper_rescore_batch: missing pointer");
    if (dim < 1 || nmodel < 0 || nmodel > 65535) return fail(VESPER_ERR_INVALID, "vesper_rescore_batch: bad sizes");
    if (nmodel == 0) return VESPER_OK;
    size_t need = 0;
    vesper_rescore_batch_workspace_size(dim, nmodel, &need);
    if (!workspace || workspace_bytes < need) return fail(VESPER_ERR_WORKSPACE, "vesper_rescore_batch: workspace");
    const int nchunk = (int)rescore_chunks(dim);
    Carver cv(workspace, workspace_bytes);
    double *part = cv.take<double>((size_t)nmodel * nchunk * kRbParts);
    double *stats = cv.take<double>((size_t)nmodel * 4);
    RescoreBatchArgs a{tdata, tvec, tave, tstd, tstd_norm_ave, sdata, svec, dim, nmodel, nchunk, trans_dev,
                       0, 0, 0, part, stats, result_out, nullptr, nullptr};
    return launch_rescore_batch(a, (cudaStream_t)stream);
}

extern "C" int vesper_rescore_batch_dev(const double *tdata, const float *tvec, const double *tstats_dev,
                                        const double *sdata, const float *svec, int dim, const int32_t *trans_dev,
                                        int nmodel, double *result_out, void *workspace, size_t workspace_bytes,
                                        void *stream) {
    if (!tstats_dev) return fail(VESPER_ERR_INVALID, "vesper_rescore_batch_dev: missing target statistics");
    if (!tdata || !tvec || !sdata || !svec || !trans_dev || !result_out)
        return fail(VESPER_ERR_INVALID, "vesper_rescore_batch_dev: missing pointer");
    if (dim < 1 || nmodel < 0 || nmodel > 65535)
        return fail(VESPER_ERR_INVALID, "vesper_rescore_batch_dev: bad sizes");
    if (nmodel == 0) return VESPER_OK;
    size_t need = 0;
    vesper_rescore_batch_workspace_size(dim, nmodel, &need);
    if (!workspace || workspace_bytes < need)
        return fail(VESPER_ERR_WORKSPACE, "vesper_rescore_batch_dev: workspace");
    const int nchunk = (int)rescore_chunks(dim);
    Carver cv(workspace, workspace_bytes);
    double *part = cv.take<double>((size_t)nmodel * nchunk * kRbParts);
    double *stats = cv.take<double>((size_t)nmodel * 4);
    RescoreBatchArgs a{tdata, tvec, 0.0, 0.0, 0.0, sdata, svec, dim, nmodel, nchunk, trans_dev,
                       0, 0, 0, part, stats, result_out, nullptr, tstats_dev};
    return launch_rescore_batch(a, (cudaStream_t)stream);
}

extern "C" int vesper_rescore(const double *tdata, const float *tvec, double tave, double tstd, double tstd_norm_ave,
                              const double *sdata, const float *svec, int dim, const int32_t *trans,
                              double *result_out, double *sco_out, void *workspace, size_t workspace_bytes,
                              void *stream) {
    if (!tdata || !tvec || !sdata || !svec || !trans || !result_out)
        return fail(VESPER_ERR_INVALID, "vesper_rescore: missing pointer");
    if (dim < 1) return fail(VESPER_ERR_INVALID, "vesper_rescore: bad dim");
    // wrap the translation to (-d/2, d/2] (:1323-1329)
    int t[3];
    for (int a = 0; a < 3; ++a) {
        t[a] = trans[a];
        if (t[a] > 0.5 * dim) t[a] -= dim;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const size_t vol = (size_t)dim * dim * dim;
    if (sco_out) {
        k_zero_f64<<<(unsigned)((vol + 255) / 256), 256, 0, st>>>(sco_out, vol);
        VG_CHECK_LAUNCH("k_zero_f64");
    }
    size_t need = 0;
    vesper_rescore_workspace_size(dim, &need);
    if (workspace && workspace_bytes >= need) {
        // many blocks: chunk partial sums in the workspace
        const int nchunk = (int)rescore_chunks(dim);
        Carver cv(workspace, workspace_bytes);
        double *part = cv.take<double>((size_t)nchunk * kRbParts);
        double *stats = cv.take<double>(4);
        RescoreBatchArgs a{tdata, tvec, tave, tstd, tstd_norm_ave, sdata, svec, dim, 1, nchunk, nullptr,
                           t[0], t[1], t[2], part, stats, result_out, sco_out};
        return launch_rescore_batch(a, st);
    }
    // no workspace: one block
    RescoreArgs a{tdata, tvec, tave, tstd, tstd_norm_ave, sdata, svec, dim, t[0], t[1], t[2], result_out, sco_out};
    k_rescore<<<1, kRsThreads, 0, st>>>(a);
    VG_CHECK_LAUNCH("k_rescore");
    return VESPER_OK;
}
