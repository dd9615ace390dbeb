/*
 * CPU oracle for the VESPER alignment hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's integer/float arithmetic where the
 * exact operation order decides the result:
 *   - doFastVEC / calc         (VESPER_1_prob_new.py:121-142, :180-257)
 *   - rot_mrc / rot_pos_mtx    (VESPER_1_prob_new.py:260-354)
 *   - rot_mrc_prob             (VESPER_1_prob_new.py:1211-1299)
 *
 * Only the test-suite, the smoke check and the CPU-baseline leg of the
 * benchmark load this library, as the checker.  The product path never does.
 *
 * Build with -ffp-contract=off: the reference's scalar loops (numba, no
 * fastmath) do not contract a*b+c into FMAs, while its float32 matrix
 * products (numpy/numba '@' -> BLAS sgemm) do.  The latter are written here
 * with explicit fmaf() in the sgemm accumulation order over k = 0, 1, 2:
 *   r = fmaf(a2, b2, fmaf(a1, b1, a0 * b0)).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* One destination voxel of doFastVEC (VESPER_1_prob_new.py:195-255).
 * Returns 1 if the voxel was written (data and possibly vec). */
static int fastvec_voxel(const float *src, const int sd[3], double sw, const double sorig[3],
                         const int x, const int y, const int z, double dw, const double dorig[3],
                         double fsiv, double fmaxd, double *out_d, float out_v[3])
{
    double pos[3];
    const int xyz[3] = {x, y, z};
    for (int a = 0; a < 3; a++) {
        /* (xyz_arr * dest_xwidth + dest_orig - src_orig) / src_xwidth */
        double t = (double)xyz[a] * dw;
        t = t + dorig[a];
        t = t - sorig[a];
        pos[a] = t / sw;
    }
    if (pos[0] < 0 || pos[1] < 0 || pos[2] < 0 || pos[0] >= sd[0] || pos[1] >= sd[1] || pos[2] >= sd[2])
        return 0;
    {
        const int64_t ix = (int64_t)pos[0], iy = (int64_t)pos[1], iz = (int64_t)pos[2];
        if (src[(ix * sd[1] + iy) * sd[2] + iz] == 0.0f)
            return 0;
    }
    int stp[3], endp[3];
    for (int a = 0; a < 3; a++) {
        stp[a] = (int32_t)(pos[a] - fmaxd);        /* astype(np.int32): truncation */
        if (stp[a] < 0) stp[a] = 0;
        endp[a] = (int32_t)(pos[a] + fmaxd + 1.0);
        if (endp[a] >= sd[a]) endp[a] = sd[a];
    }
    /* calc() (VESPER_1_prob_new.py:121-142) */
    double dtotal = 0.0, p0 = 0.0, p1 = 0.0, p2 = 0.0;
    for (int xp = stp[0]; xp < endp[0]; xp++) {
        double rx = (double)xp - pos[0];
        rx = rx * rx;
        for (int yp = stp[1]; yp < endp[1]; yp++) {
            double ry = (double)yp - pos[1];
            ry = ry * ry;
            const float *row = src + ((int64_t)xp * sd[1] + yp) * sd[2];
            for (int zp = stp[2]; zp < endp[2]; zp++) {
                double rz = (double)zp - pos[2];
                rz = rz * rz;
                double d2 = rx + ry;
                d2 = d2 + rz;
                double e = -1.5 * d2;
                e = e * fsiv;
                double v = (double)row[zp] * exp(e);
                dtotal += v;
                p0 += v * (double)xp;
                p1 += v * (double)yp;
                p2 += v * (double)zp;
            }
        }
    }
    *out_d = dtotal;
    out_v[0] = out_v[1] = out_v[2] = 0.0f;
    if (dtotal == 0)
        return 1;
    const double rd = 1.0 / dtotal;
    double t0 = p0 * rd - pos[0];
    double t1 = p1 * rd - pos[1];
    double t2 = p2 * rd - pos[2];
    double dvec = t0 * t0 + t1 * t1;
    dvec = sqrt(dvec + t2 * t2);
    if (dvec == 0) dvec = 1.0;
    const double rdvec = 1.0 / dvec;
    out_v[0] = (float)(t0 * rdvec);
    out_v[1] = (float)(t1 * rdvec);
    out_v[2] = (float)(t2 * rdvec);
    return 1;
}

/*
 * doFastVEC over the whole destination grid, or over the ``n_idx`` linear
 * destination indices in ``idx`` when it is non-NULL (used for bounded CPU
 * timing samples).  src: [x][y][z] float32.  out_data: double, out_vec: float
 * x3 -- both must be zero-initialised by the caller (the reference writes
 * only the voxels that pass its checks).  nthreads <= 0 uses all threads.
 */
void orc_fastvec(const float *src, const int *sdims, double swidth, const double *sorig,
                 const int *ddims, double dwidth, const double *dorig, double dreso,
                 double *out_data, float *out_vec, const int64_t *idx, int64_t n_idx, int nthreads)
{
    const double gstep = swidth;
    double fs = (dreso / gstep) * 0.5;
    fs = fs * fs;
    const double fsiv = 1.0 / fs;
    const double fmaxd = (dreso / gstep) * 2.0;
    const int sd[3] = {sdims[0], sdims[1], sdims[2]};
    const int64_t dd1 = ddims[1], dd2 = ddims[2];
    const int64_t total = idx ? n_idx : (int64_t)ddims[0] * dd1 * dd2;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t t = 0; t < total; t++) {
        const int64_t lin = idx ? idx[t] : t;
        const int x = (int)(lin / (dd1 * dd2));
        const int y = (int)((lin / dd2) % dd1);
        const int z = (int)(lin % dd2);
        double dv;
        float vv[3];
        if (fastvec_voxel(src, sd, swidth, sorig, x, y, z, dwidth, dorig, fsiv, fmaxd, &dv, vv)) {
            out_data[lin] = dv;
            out_vec[lin * 3 + 0] = vv[0];
            out_vec[lin * 3 + 1] = vv[1];
            out_vec[lin * 3 + 2] = vv[2];
        }
    }
}

/*
 * rot_mrc / rot_mrc_prob restated as the reference's scatter, row by row.
 *
 * F is np.flip(mtx) as float32 (row-major 3x3), where mtx is the ZYX Euler
 * matrix with |m| < 1e-15 zeroed.  Rows of new_pos follow
 * meshgrid(arange(d) x3).T.reshape(-1, 3): z slowest, x middle, y fastest.
 *   old_j   = sum_k p_k F[j][k] (sgemm order, float32) + cent   (float32 add)
 *   in-bound: 0 <= old_j < d on all axes; old and new truncated to int
 *   dens mask: data[old] != 0 (per prob channel: p_c[old] != 0)
 *   new_vec_j = sum_k v_k F[k][j]  (sgemm order, float32)
 *   dest = int(trunc(new_pos) + cent)   -- later rows overwrite earlier ones
 * Outputs must be zero-initialised by the caller.  probs/out_probs may be
 * NULL (rot_mrc) or arrays of 4 channel pointers (rot_mrc_prob).
 */
void orc_rot_gather(const double *data, const float *vec, const float *const *probs, int d,
                    const float *F, double *out_data, float *out_vec, float *const *out_probs)
{
    const double cent = 0.5 * (double)d;
    const float centf = (float)cent;
    const int64_t d2 = (int64_t)d * d;
    for (int k = 0; k < d; k++)          /* z (slowest) */
        for (int i = 0; i < d; i++)      /* x */
            for (int j = 0; j < d; j++) {/* y (fastest) */
                const double pn[3] = {(double)i - cent, (double)j - cent, (double)k - cent};
                const float pf[3] = {(float)pn[0], (float)pn[1], (float)pn[2]};
                float old[3];
                for (int a = 0; a < 3; a++) {
                    float acc = pf[0] * F[a * 3 + 0];
                    acc = fmaf(pf[1], F[a * 3 + 1], acc);
                    acc = fmaf(pf[2], F[a * 3 + 2], acc);
                    old[a] = acc + centf;
                }
                if (!(old[0] >= 0 && old[1] >= 0 && old[2] >= 0 && old[0] < d && old[1] < d && old[2] < d))
                    continue;
                const int64_t oi = (int32_t)(double)old[0], oj = (int32_t)(double)old[1],
                              ok = (int32_t)(double)old[2];
                const int64_t src = (oi * d + oj) * d + ok;
                const int ni = (int)((double)(int32_t)pn[0] + cent);
                const int nj = (int)((double)(int32_t)pn[1] + cent);
                const int nk = (int)((double)(int32_t)pn[2] + cent);
                const int64_t dst = ((int64_t)ni * d + nj) * d + nk;
                if (data[src] != 0.0) {
                    const float v0 = vec[src * 3 + 0], v1 = vec[src * 3 + 1], v2 = vec[src * 3 + 2];
                    for (int a = 0; a < 3; a++) {
                        float acc = v0 * F[0 * 3 + a];
                        acc = fmaf(v1, F[1 * 3 + a], acc);
                        acc = fmaf(v2, F[2 * 3 + a], acc);
                        out_vec[dst * 3 + a] = acc;
                    }
                    out_data[dst] = data[src];
                }
                if (probs)
                    for (int c = 0; c < 4; c++)
                        if (probs[c][src] != 0.0f)
                            out_probs[c][dst] = probs[c][src];
            }
    (void)d2;
}

/*
 * Old-position table of one rotation, for index-level tests of the gather:
 * for every row of new_pos (reference row order) the float32 old position,
 * and the destination linear index.  old_out: n x 3 float, dst_out: n int64.
 */
void orc_rot_positions(int d, const float *F, float *old_out, int64_t *dst_out)
{
    const double cent = 0.5 * (double)d;
    const float centf = (float)cent;
    int64_t r = 0;
    for (int k = 0; k < d; k++)
        for (int i = 0; i < d; i++)
            for (int j = 0; j < d; j++, r++) {
                const double pn[3] = {(double)i - cent, (double)j - cent, (double)k - cent};
                const float pf[3] = {(float)pn[0], (float)pn[1], (float)pn[2]};
                for (int a = 0; a < 3; a++) {
                    float acc = pf[0] * F[a * 3 + 0];
                    acc = fmaf(pf[1], F[a * 3 + 1], acc);
                    acc = fmaf(pf[2], F[a * 3 + 2], acc);
                    old_out[r * 3 + a] = acc + centf;
                }
                const int ni = (int)((double)(int32_t)pn[0] + cent);
                const int nj = (int)((double)(int32_t)pn[1] + cent);
                const int nk = (int)((double)(int32_t)pn[2] + cent);
                dst_out[r] = ((int64_t)ni * d + nj) * d + nk;
            }
}
