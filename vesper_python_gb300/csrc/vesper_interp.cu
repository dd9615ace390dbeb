// Hole filling of probability maps sampled on every other voxel
// (interpolate, interpolation_functions.py:6-135), in place on a
// [nx][ny][nz][nch] float32 array.
//
// The reference fixes a parity (ref_x, ref_y, ref_z) from the first voxel in
// C order whose channel 0 is positive, then fills, channel by channel, every
// zero voxel whose index parity differs from the reference in one axis (x,
// then y, then z), in two axes (xy, xz, yz), then in all three, with the mean
// of its two neighbours along each differing axis.  Within a step the voxels
// written and the voxels read have different parities, so every step is one
// parallel launch; steps run in the reference's order.  The reference's loops
// stop before the last index of each axis and index i - 1 = -1 wraps to the
// last element (Python/numba negative indexing); both are kept.  Means are
// accumulated in float64 and rounded to float32 on store, as the numba
// function's float64 accumulator does.
#include <algorithm>

#include "vesper_common.cuh"

namespace vg {

// parity[0..2] of the first voxel (C order) with channel 0 > 0; first[0] holds
// its linear index (atomicMin; starts at 0xffffffffffffffff)
__global__ void k_interp_first(const float *data, long long nvox, int nch, unsigned long long *first) {
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nvox;
         v += (long long)gridDim.x * blockDim.x)
        if (data[v * nch] > 0.f) atomicMin(first, (unsigned long long)v);
}

// Step with flip mask m (bit 0: x, bit 1: y, bit 2: z): voxels whose parity
// differs from the reference exactly on the axes in m.
__global__ void k_interp_step(float *data, int nx, int ny, int nz, int nch, int m,
                              const unsigned long long *first) {
    const unsigned long long f = *first;
    if (f == ~0ull) return;   // no voxel with a positive channel 0: the caller reports it
    const long long yz = (long long)ny * nz;
    const int rx = (int)((f / (unsigned long long)yz) & 1ull);
    const int ry = (int)((f / (unsigned long long)nz % (unsigned long long)ny) & 1ull);
    const int rz = (int)((f % (unsigned long long)nz) & 1ull);
    // first index of each axis' class: the flipped parity on flipped axes
    const int sx = (m & 1) ? (rx + 1) % 2 : rx, sy = (m & 2) ? (ry + 1) % 2 : ry, sz = (m & 4) ? (rz + 1) % 2 : rz;
    // counts of range(s, n - 1, 2) for each axis
    const int kx = max(0, (nx - sx) / 2), ky = max(0, (ny - sy) / 2), kz = max(0, (nz - sz) / 2);
    const long long total = (long long)kx * ky * kz * nch;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(t % nch);
        const long long c = t / nch;
        const int kk = (int)(c % kz), jj = (int)((c / kz) % ky), ii = (int)(c / ((long long)kz * ky));
        const int i = sx + 2 * ii, j = sy + 2 * jj, k = sz + 2 * kk;
        float *p = data + (((long long)i * ny + j) * nz + k) * nch + l;
        if (*p != 0.f) continue;
        double s = 0.0;
        int n = 0;
        auto at = [&](int a, int b, int e) -> double {
            // Python negative indexing: -1 is the last element
            const int aa = a < 0 ? a + nx : a, bb = b < 0 ? b + ny : b, ee = e < 0 ? e + nz : e;
            return (double)data[(((long long)aa * ny + bb) * nz + ee) * nch + l];
        };
        // the reference's summation order: x pair, then y pair, then z pair
        if (m & 1) {
            s += at(i + 1, j, k);
            s += at(i - 1, j, k);
            n += 2;
        }
        if (m & 2) {
            s += at(i, j + 1, k);
            s += at(i, j - 1, k);
            n += 2;
        }
        if (m & 4) {
            s += at(i, j, k + 1);
            s += at(i, j, k - 1);
            n += 2;
        }
        *p = (float)(s / (double)n);
    }
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_prob_interpolate(float *data, int nx, int ny, int nz, int nch, void *workspace,
                                       size_t workspace_bytes, void *stream) {
    if (!data || nx < 1 || ny < 1 || nz < 1 || nch < 1) return fail(VESPER_ERR_INVALID, "prob_interpolate: bad args");
    if (!workspace || workspace_bytes < sizeof(unsigned long long))
        return fail(VESPER_ERR_WORKSPACE, "prob_interpolate: workspace of 8 bytes needed");
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long *first = (unsigned long long *)workspace;
    if (cudaMemsetAsync(first, 0xff, sizeof(unsigned long long), st) != cudaSuccess)
        return cuda_check("prob_interpolate: memset");
    const long long nvox = (long long)nx * ny * nz;
    k_interp_first<<<(unsigned)std::min<long long>((nvox + 255) / 256, 4096), 256, 0, st>>>(data, nvox, nch, first);
    VG_CHECK_LAUNCH("k_interp_first");
    // the reference's order of steps: x, y, z, xy, xz, yz, xyz
    const int masks[7] = {1, 2, 4, 3, 5, 6, 7};
    for (int s = 0; s < 7; ++s) {
        const long long cells = (long long)((nx + 1) / 2) * ((ny + 1) / 2) * ((nz + 1) / 2) * nch;
        const unsigned g = (unsigned)std::min<long long>((cells + 255) / 256, 65535);
        k_interp_step<<<std::max(1u, g), 256, 0, st>>>(data, nx, ny, nz, nch, masks[s], first);
        VG_CHECK_LAUNCH("k_interp_step");
    }
    return VESPER_OK;
}

extern "C" int vesper_prob_interpolate_found(const void *workspace, int *found, void *stream) {
    // host check after the call: did any voxel have a positive channel 0?
    if (!workspace || !found) return fail(VESPER_ERR_INVALID, "prob_interpolate_found: bad args");
    unsigned long long v = 0;
    if (cudaMemcpyAsync(&v, workspace, sizeof(v), cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess ||
        cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
        return cuda_check("prob_interpolate_found");
    *found = v != 0xffffffffffffffffull;
    return VESPER_OK;
}
