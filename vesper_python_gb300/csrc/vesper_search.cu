// Rotational FFT search: batched rotate -> FFT -> correlate -> inverse FFT ->
// argmax over every rotation of the angle grid (the rotation loops of
// search_map_fft / search_map_fft_prob).
//
// Data layout in HBM (per rotation b of a batch, channel c, group g):
//   q4[N], p4[N]        packed query source (vesper_passes.cuh, k_pack)
//   S[b][c][x][ky][kz]  complex64 forward spectrum after the z and y passes
//   T[c][kx][ky][kz]    complex64 conj(target spectrum), kz in [0, d/2]
//   U[b][g][kx][ky][kz] complex64 sum over the group's channels of
//                       T_c * Q_c after the inverse x pass
//   keys[r][s]          64-bit (score order bits, ~index) per rotation / score
// The library's default batch keeps S and U (64 MB) resident in the 129 MB L2
// across the three passes of a batch.
#include <algorithm>
#include <mutex>

#include "vesper_common.cuh"
#include "vesper_passes.cuh"
#include "vesper_regpass.cuh"

namespace vg {

__global__ void k_decode(const unsigned long long *keys, int n, float *scores, int32_t *lin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    scores[i] = order_float((uint32_t)(k >> 32));
    lin[i] = (int32_t)(0xffffffffu - (uint32_t)(k & 0xffffffffull));
}

struct SearchCfg {
    int batch, cchunk, W, threads;
    size_t sa, sb, sc;
    int path;   // 0: radix-stage passes, 1: register two-step passes
};

// ---- register two-step passes: the sides compiled in (vesper_regsearch_*.cu)
const RegEntry *find_reg(int mode, int d);

// vesper_fused.cu: 1 if a fused single-kernel search is compiled for (mode,
// side) -- launched when rc is non-null, its status stored there -- else 0.
int vesper_fused_search(int mode, int d, const Src &src, const float *rotmats, const void *spectra, int nrot,
                        int nscore, unsigned long long *keys, cudaStream_t st, int *rc);

static int default_batch(int d, int mode) {
    const size_t H = d / 2 + 1;
    const size_t per = (size_t)(mode_nch(mode) + mode_ngrp(mode)) * d * d * H * sizeof(float2);
    const size_t budget = 64ull << 20;
    int b = (int)std::max<size_t>(1, budget / per);
    return std::min(b, 2048);
}

// Shared-memory and thread-count plan of the three passes for side d.
static bool plan_passes(int d, int mode, const FftPlan &P, SearchCfg *c) {
    const size_t lim = (size_t)smem_limit();
    const int nch = mode_nch(mode), ngrp = mode_ngrp(mode);
    const PlaneGeom g = plane_geom(d);
    const int T = kThreads, T2 = 2 * kThreads;
    c->threads = T;
    c->cchunk = 0;
    for (size_t cap : {lim / 2 - 1024, lim}) {
        for (int cc = nch; cc >= 1 && !c->cchunk; --cc)
            if (smem_a2(d, P.ntab, cc) <= cap && cc * g.npairs <= T2 && cc * g.H <= T2) c->cchunk = cc;
        if (c->cchunk) break;
    }
    c->W = 0;
    for (size_t cap : {lim / 2 - 1024, lim}) {
        for (int W : {32, 16, 8, 4, 2, 1})
            if (!c->W && smem_b2(d, P.ntab, nch, ngrp, W) <= cap && nch * W <= T2) c->W = W;
        if (c->W) break;
    }
    c->sa = smem_a2(d, P.ntab, std::max(c->cchunk, 1));
    c->sb = smem_b2(d, P.ntab, nch, ngrp, std::max(c->W, 1));
    c->sc = smem_c2(d, P.ntab, ngrp);
    return c->cchunk > 0 && c->W > 0 && c->sc <= lim && ngrp * g.npairs <= T2 && ngrp * g.H <= T2;
}

static int check_dim(int d, int mode, FftPlan *P) {
    if (mode < 0 || mode > VESPER_MODE_PROB) return fail(VESPER_ERR_INVALID, "unknown mode %d", mode);
    if (d < 2) return fail(VESPER_ERR_INVALID, "grid side %d < 2", d);
    if (!make_plan(d, P)) return fail(VESPER_ERR_UNSUPPORTED, "grid side %d is not 2^a3^b5^c7^d(11|13)", d);
    if (d > vesper_max_dim(mode))
        return fail(VESPER_ERR_UNSUPPORTED, "grid side %d above the maximum %d", d, vesper_max_dim(mode));
    return VESPER_OK;
}

// A ring of event sets keeps kRing batches in flight: a slot's events are read
// (and its times accumulated) only when the slot is reused or at the end.
constexpr int kRing = 16;
struct PassTimer {
    cudaEvent_t ev[kRing][4][2];
    bool used[kRing][4];
    float ms[4];
};

template <int MODE, int NCH>
static void launch_a(dim3 grid, const SearchCfg &c, cudaStream_t st, const PassA2 &pa) {
    allow_smem(k_pass_a<MODE, NCH>, c.sa);
    k_pass_a<MODE, NCH><<<grid, c.threads, c.sa, st>>>(pa);
}

template <int MODE>
static void launch_pack(const double *data, const float *vec, const float *probs, int d, double ave, float4 *q4,
                        float4 *p4, cudaStream_t st) {
    const size_t n = (size_t)d * d * d;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_pack<MODE><<<blocks, 256, 0, st>>>(data, vec, probs, d, ave, q4, p4);
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_max_dim(int mode) {
    int best = 0;
    for (int d = 2; d <= 256; ++d) {
        FftPlan P;
        if (!make_plan(d, &P)) continue;
        SearchCfg c;
        if (!plan_passes(d, mode, P, &c)) continue;
        if (smem_target_a(d, d / 2 + 1) > (size_t)smem_limit()) continue;
        best = d;
    }
    return best;
}

extern "C" int vesper_search_nscore(int mode, int with_mix) {
    if (mode == VESPER_MODE_PROB) return with_mix ? 3 : 2;
    return 1;
}

// Laplacian mode: the rotated density of every rotation of a batch
// (rot_mrc's gather, density != 0 mask), so that pass A computes the filter
// from plain reads instead of seven gathers per voxel.
__global__ void k_rot_density(const Src s, const float *rotmats, int r0, double *rd) {
    __shared__ float F[9];
    const int b = blockIdx.y;
    if (threadIdx.x < 9) F[threadIdx.x] = rotmats[(size_t)(r0 + b) * 9 + threadIdx.x];
    __syncthreads();
    const int d = s.d;
    const size_t n = (size_t)d * d * d;
    const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int x = (int)(v / ((size_t)d * d)), y = (int)((v / d) % d), z = (int)(v % d);
    float4 w;
    const int i = gather4(F, d, x, y, z, s.q4, w);
    rd[(size_t)b * n + v] = i >= 0 ? s.data[i] : 0.0;
}

extern "C" int vesper_search_workspace_size(int dim, int mode, int batch, int nrot, size_t *bytes) {
    if (!bytes) return fail(VESPER_ERR_INVALID, "bytes is NULL");
    if (batch <= 0) batch = default_batch(dim, mode);
    const size_t H = dim / 2 + 1, N = (size_t)dim * dim * dim;
    Carver cv(nullptr, 0);
    cv.take<int>(64);   // status word (tensor-core pass B time-outs)
    cv.take<float4>(N);
    if (mode == VESPER_MODE_PROB) cv.take<float4>(N);
    cv.take<float2>((size_t)batch * mode_nch(mode) * dim * dim * H);
    cv.take<float2>((size_t)batch * mode_ngrp(mode) * dim * dim * H);
    cv.take<unsigned long long>((size_t)std::max(nrot, 1) * 3);
    if (mode == VESPER_MODE_LAPLACIAN) cv.take<double>((size_t)batch * N);
    *bytes = cv.off + 256;
    return VESPER_OK;
}

static int search_impl(const void *spectra, const double *data, const float *vec, const float *probs, int dim,
                       int mode, double ave, const float *rotmats, int nrot, const double *mix, float *scores_out,
                       int32_t *lin_out, int batch, void *workspace, size_t workspace_bytes, void *stream,
                       PassTimer *tm, const int *opts = nullptr) {
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
    SearchCfg cfg;
    if (!plan_passes(dim, mode, P, &cfg))
        return fail(VESPER_ERR_UNSUPPORTED, "grid side %d does not fit shared memory", dim);
    cfg.path = 0;
    const RegEntry *reg = find_reg(mode, dim);
    const int want_path = opts ? opts[0] : -1;
    // path 3: pass B on the tensor cores (split-BF16), passes A and C as path 1 (else 0)
    const bool tcb = want_path == 3;
    if (tcb && !tc_pass_b_supported(dim))
        return fail(VESPER_ERR_UNSUPPORTED, "tensor-core pass B: side %d (32 and 64 only)", dim);
    if (reg && want_path != 0) {
        const size_t lim = (size_t)smem_limit();
        const int nchr = mode_nch(mode), ngrr = mode_ngrp(mode);
        int cc = 0, W = 0;
        for (size_t cap : {lim / 2 - 1024, lim}) {
            for (int c = nchr; c >= 1 && !cc; --c)
                if (reg->sa(c) <= cap) cc = c;
            if (cc) break;
        }
        for (int w : {32, 16, 8, 4, 2, 1})
            if (!W && reg->sb(nchr, ngrr, w) <= lim / 2 - 1024) W = w;
        if (opts && opts[1] > 0 && opts[1] <= nchr && reg->sa(opts[1]) <= lim) cc = opts[1];
        if (opts && opts[2] > 0 && reg->sb(nchr, ngrr, opts[2]) <= lim) W = opts[2];
        if (cc && W && reg->sc(ngrr) <= lim) {
            cfg.path = 1;
            cfg.cchunk = cc;
            cfg.W = W;
            cfg.sa = reg->sa(cc);
            cfg.sb = reg->sb(nchr, ngrr, W);
            cfg.sc = reg->sc(ngrr);
        }
    } else if (opts) {
        const int nchr = mode_nch(mode), ngrr = mode_ngrp(mode);
        const size_t lim = (size_t)smem_limit();
        if (opts[1] > 0 && opts[1] <= nchr && smem_a2(dim, P.ntab, opts[1]) <= lim) {
            cfg.cchunk = opts[1];
            cfg.sa = smem_a2(dim, P.ntab, opts[1]);
        }
        if (opts[2] > 0 && smem_b2(dim, P.ntab, nchr, ngrr, opts[2]) <= lim && nchr * opts[2] <= 2 * kThreads) {
            cfg.W = opts[2];
            cfg.sb = smem_b2(dim, P.ntab, nchr, ngrr, opts[2]);
        }
    }
    if (want_path == 1 && cfg.path != 1)
        return fail(VESPER_ERR_UNSUPPORTED, "no register-FFT passes compiled for mode %d, side %d", mode, dim);
    cudaStream_t st = (cudaStream_t)stream;
    if (tcb && cudaMemsetAsync(workspace, 0, sizeof(int), st) != cudaSuccess)
        return cuda_check("vesper_search: status word");
    if (tcb) {   // batches of whole waves of tensor-core CTAs (a partial extra wave costs a full one)
        const int wave = tc_pass_b_wave(dim);
        if (batch > wave) batch = batch / wave * wave;
    }
    const int H = dim / 2 + 1, nch = mode_nch(mode), ngrp = mode_ngrp(mode);
    const size_t N = (size_t)dim * dim * dim;
    const int nscore = vesper_search_nscore(mode, mix != nullptr);
    Carver cv(workspace, workspace_bytes);
    int *status = cv.take<int>(64);
    float4 *q4 = cv.take<float4>(N);
    float4 *p4 = mode == VESPER_MODE_PROB ? cv.take<float4>(N) : nullptr;
    float2 *S = cv.take<float2>((size_t)batch * nch * dim * dim * H);
    float2 *U = cv.take<float2>((size_t)batch * ngrp * dim * dim * H);
    unsigned long long *keys = cv.take<unsigned long long>((size_t)nrot * 3);
    double *rd = mode == VESPER_MODE_LAPLACIAN ? cv.take<double>((size_t)batch * N) : nullptr;

    switch (mode) {
        case VESPER_MODE_VEC: launch_pack<VESPER_MODE_VEC>(data, vec, probs, dim, ave, q4, p4, st); break;
        case VESPER_MODE_OVERLAP: launch_pack<VESPER_MODE_OVERLAP>(data, vec, probs, dim, ave, q4, p4, st); break;
        case VESPER_MODE_CC: launch_pack<VESPER_MODE_CC>(data, vec, probs, dim, ave, q4, p4, st); break;
        case VESPER_MODE_PCC: launch_pack<VESPER_MODE_PCC>(data, vec, probs, dim, ave, q4, p4, st); break;
        case VESPER_MODE_LAPLACIAN: launch_pack<VESPER_MODE_LAPLACIAN>(data, vec, probs, dim, ave, q4, p4, st); break;
        case VESPER_MODE_PROB: launch_pack<VESPER_MODE_PROB>(data, vec, probs, dim, ave, q4, p4, st); break;
    }
    VG_CHECK_LAUNCH("k_pack");

    Mix mx{};
    if (mix) {
        mx.one_minus_alpha = (float)(1.0 - mix[0]);
        mx.alpha = (float)mix[0];
        mx.vstd = (float)mix[1];
        mx.vave = (float)mix[2];
        mx.pstd = (float)mix[3];
        mx.pave = (float)mix[4];
    }
    PassA2 pa{Src{q4, p4, data, dim}, rotmats, 0, nch, cfg.cchunk, nscore, P, S, keys, rd};
    PassB2 pb{S, (const float2 *)spectra, U, dim, nch, ngrp, mode == VESPER_MODE_PROB ? 3 : nch, cfg.W, P};
    PassC2 pc{U, dim, ngrp, 0, nscore, P, mx, keys};
    allow_smem(k_pass_b, cfg.sb);
    allow_smem(k_pass_c<1>, cfg.sc);
    allow_smem(k_pass_c<2>, cfg.sc);
    allow_smem(k_pass_c<3>, cfg.sc);
    const int nbx = (dim * H + cfg.W - 1) / cfg.W;
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
    // fused single-kernel search where it is compiled for (mode, side)
    bool fused = false;
    if (want_path == 2 || want_path < 0) {
        int frc = VESPER_OK;
        mark(0, 0);
        fused = vesper_fused_search(mode, dim, Src{q4, p4, data, dim}, rotmats, spectra, nrot, nscore, keys, st,
                                    &frc) != 0;
        if (fused && frc) return frc;
        if (fused) {
            mark(0, 1);
            slot = (slot + 1) % kRing;
        }
    }
    if (want_path == 2 && !fused)
        return fail(VESPER_ERR_UNSUPPORTED, "no fused search compiled for mode %d, side %d", mode, dim);
    for (int r0 = 0; !fused && r0 < nrot; r0 += batch) {
        const int nb = std::min(batch, nrot - r0);
        pa.r0 = r0;
        pc.r0 = r0;
        const dim3 gplane(dim, nb);
        mark(0, 0);
        if (rd) {
            k_rot_density<<<dim3((unsigned)((N + 255) / 256), nb), 256, 0, st>>>(pa.src, rotmats, r0, rd);
            VG_CHECK_LAUNCH("k_rot_density");
        }
        if (cfg.path == 1) {
            reg->a(gplane, kThreads, cfg.sa, st, pa);
            VG_CHECK_LAUNCH("k_rpass_a");
            mark(0, 1);
            mark(1, 0);
            if (tcb) {
                rc = tc_pass_b(pb, nb, status, st);
                if (rc) return rc;
            } else {
                reg->b(dim3(nbx, nb), kThreads, cfg.sb, st, pb);
                VG_CHECK_LAUNCH("k_rpass_b");
            }
            mark(1, 1);
            mark(2, 0);
            reg->c(gplane, kThreads, cfg.sc, st, pc, nscore);
            VG_CHECK_LAUNCH("k_rpass_c");
            mark(2, 1);
            slot = (slot + 1) % kRing;
            continue;
        }
        switch (mode) {
            case VESPER_MODE_VEC: launch_a<VESPER_MODE_VEC, 3>(gplane, cfg, st, pa); break;
            case VESPER_MODE_OVERLAP: launch_a<VESPER_MODE_OVERLAP, 1>(gplane, cfg, st, pa); break;
            case VESPER_MODE_CC: launch_a<VESPER_MODE_CC, 1>(gplane, cfg, st, pa); break;
            case VESPER_MODE_PCC: launch_a<VESPER_MODE_PCC, 1>(gplane, cfg, st, pa); break;
            case VESPER_MODE_LAPLACIAN: launch_a<VESPER_MODE_LAPLACIAN, 1>(gplane, cfg, st, pa); break;
            case VESPER_MODE_PROB: launch_a<VESPER_MODE_PROB, 7>(gplane, cfg, st, pa); break;
        }
        VG_CHECK_LAUNCH("k_pass_a");
        mark(0, 1);
        mark(1, 0);
        if (tcb) {
            rc = tc_pass_b(pb, nb, status, st);
            if (rc) return rc;
        } else {
            k_pass_b<<<dim3(nbx, nb), cfg.threads, cfg.sb, st>>>(pb);
            VG_CHECK_LAUNCH("k_pass_b");
        }
        mark(1, 1);
        mark(2, 0);
        switch (nscore) {
            case 1: k_pass_c<1><<<gplane, cfg.threads, cfg.sc, st>>>(pc); break;
            case 2: k_pass_c<2><<<gplane, cfg.threads, cfg.sc, st>>>(pc); break;
            default: k_pass_c<3><<<gplane, cfg.threads, cfg.sc, st>>>(pc); break;
        }
        VG_CHECK_LAUNCH("k_pass_c");
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

extern "C" int vesper_search_tuned(const void *spectra, const double *data, const float *vec, const float *probs,
                                   int dim, int mode, double ave, const float *rotmats, int nrot, const double *mix,
                                   float *scores_out, int32_t *lin_out, int batch, void *workspace,
                                   size_t workspace_bytes, void *stream, const int *opts) {
    return search_impl(spectra, data, vec, probs, dim, mode, ave, rotmats, nrot, mix, scores_out, lin_out, batch,
                       workspace, workspace_bytes, stream, nullptr, opts);
}

extern "C" int vesper_search_profile(const void *spectra, const double *data, const float *vec, const float *probs,
                                     int dim, int mode, double ave, const float *rotmats, int nrot,
                                     const double *mix, float *scores_out, int32_t *lin_out, int batch,
                                     void *workspace, size_t workspace_bytes, void *stream, float *pass_ms,
                                     int *pass_launches, const int *opts) {
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
                               batch, workspace, workspace_bytes, stream, &tm, opts);
    for (int p = 0; p < 4; ++p) pass_ms[p] = tm.ms[p];
    int path = 0, launches = 0;
    vesper_search_plan(dim, mode, batch, nrot, opts, &path, &launches);
    if (batch <= 0) batch = default_batch(dim, mode);
    const int nb = nrot > 0 ? (nrot + batch - 1) / batch : 0;
    pass_launches[0] = path == 2 ? (nrot > 0) : nb;
    pass_launches[1] = pass_launches[2] = path == 2 ? 0 : nb;
    pass_launches[3] = nrot > 0 ? 1 : 0;
    return rc;
}

extern "C" int vesper_search_plan(int dim, int mode, int batch, int nrot, const int *opts, int *path_out,
                                  int *launches_out) {
    if (!path_out || !launches_out) return fail(VESPER_ERR_INVALID, "vesper_search_plan: NULL output");
    FftPlan P;
    int rc = check_dim(dim, mode, &P);
    if (rc) return rc;
    const int want = opts ? opts[0] : -1;
    int path = 0;
    if ((want == 2 || want < 0) && vesper_fused_search(mode, dim, Src{}, nullptr, nullptr, 0, 1, nullptr, nullptr,
                                                       nullptr))
        path = 2;
    else if (want != 0 && want != 2 && find_reg(mode, dim))
        path = 1;
    if (want == 2 && path != 2) return fail(VESPER_ERR_UNSUPPORTED, "no fused search for mode %d, side %d", mode, dim);
    if (want == 3) {
        if (!tc_pass_b_supported(dim))
            return fail(VESPER_ERR_UNSUPPORTED, "tensor-core pass B: side %d (32 and 64 only)", dim);
        path = 3;
    }
    if (batch <= 0) batch = default_batch(dim, mode);
    if (path == 3) {   // as the search does: batches of whole waves of tensor-core CTAs
        const int wave = tc_pass_b_wave(dim);
        if (batch > wave) batch = batch / wave * wave;
    }
    const int nb = nrot > 0 ? (nrot + batch - 1) / batch : 0;
    *path_out = path;
    // pack + passes (+ the gathered density of each Laplacian batch) + decode
    *launches_out = nrot > 0 ? 2 + (path == 2 ? 1 : (mode == VESPER_MODE_LAPLACIAN ? 4 : 3) * nb) : 0;
    return VESPER_OK;
}

extern "C" int vesper_search_status(const void *workspace, size_t workspace_bytes, int *status_out, void *stream) {
    if (!workspace || workspace_bytes < sizeof(int) || !status_out)
        return fail(VESPER_ERR_INVALID, "vesper_search_status: bad args");
    int v = 0;
    if (cudaMemcpyAsync(&v, workspace, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess ||
        cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
        return cuda_check("vesper_search_status");
    *status_out = v;
    return VESPER_OK;
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
    // the largest pipeline batch (up to the library default) whose scratch fits
    // the array; every batch gives the same results, larger ones fewer launches
    int batch = 1;
    for (int b = default_batch(dim, mode); b > 1; b = b * 3 / 4) {
        size_t nb = 0;
        if (vesper_search_workspace_size(dim, mode, b, nrot, &nb) == VESPER_OK && nb <= kStaticScratchBytes) {
            batch = b;
            break;
        }
    }
    // the keys each rotation reads are zeroed by its own first pass, so nothing
    // left in the array by an earlier call matters
    return search_impl(spectra, data, vec, probs, dim, mode, ave, rotmats, nrot, mix, scores_out, lin_out, batch,
                       scratch, kStaticScratchBytes, stream, nullptr);
}
