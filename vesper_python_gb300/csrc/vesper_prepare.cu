// Map preparation on the device: the threshold and maximum radius of
// mrc_set_vox_size (VESPER_1_prob_new.py:72-89) and the fastVEC statistics
// (VESPER_1_prob_new.py:157-161).
#include <algorithm>

#include "vesper_common.cuh"

namespace vg {

// data[data < th] = 0 (float32 compare), and the largest squared distance
// ((i-cx)^2 + (j-cy)^2) + (k-cz)^2 of a non-zero voxel, as the bits of a
// non-negative double (ordered like unsigned integers) via atomicMax, with
// the count of non-zero voxels.  One warp per source row (i, j) at a time, its
// lanes over k: the row's index arithmetic and (i-cx)^2 + (j-cy)^2 are done
// once per row (the same float64 operations in the same order per voxel).
// Warp w of nw strides over the rows.
__device__ __forceinline__ void prepare_rows(float *data, int sx, int sy, int sz, float th, double cx, double cy,
                                             double cz, unsigned long long *out, int w, int nw) {
    const int lane = threadIdx.x & 31;
    double best = -1.0;
    unsigned long long cnt = 0;
    const int nrows = sx * sy;
    for (int row = w; row < nrows; row += nw) {
        const int x = row / sy, j = row - x * sy;
        const double a = (double)x - cx, b = (double)j - cy;
        const double ab = __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
        float *rp = data + (size_t)row * sz;
        for (int k = lane; k < sz; k += 32) {
            float v = rp[k];
            if (v < th) {
                v = 0.f;
                rp[k] = 0.f;
            }
            if (v != 0.f) {
                const double c = (double)k - cz;
                const double d2 = __dadd_rn(ab, __dmul_rn(c, c));
                best = d2 > best ? d2 : best;
                ++cnt;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double v = __shfl_down_sync(0xffffffffu, best, o);
        best = v > best ? v : best;
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0 && cnt > 0) {
        atomicMax(&out[0], (unsigned long long)__double_as_longlong(best));
        atomicAdd(&out[1], cnt);
    }
}

__global__ void k_prepare(float *data, int sx, int sy, int sz, float th, double cx, double cy, double cz,
                          unsigned long long *out) {
    prepare_rows(data, sx, sy, sz, th, cx, cy, cz, out, (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5),
                 (int)((gridDim.x * blockDim.x) >> 5));
}

// The same for up to kPrepMax maps in one launch: map i takes blocks
// [first[i], first[i + 1]) and strides over its voxels with that many blocks.
constexpr int kPrepMax = 64;
struct PrepMap {
    float *data;
    unsigned long long *out;
    double c[3];
    int s[3];
    float th;
    int first;   // first block of the map; first of entry nmap = the grid size
};
struct PrepBatch {
    int nmap;
    PrepMap m[kPrepMax + 1];
};

__global__ void k_prepare_many(const __grid_constant__ PrepBatch b) {
    int i = 0;
    while (i + 1 < b.nmap && b.m[i + 1].first <= (int)blockIdx.x) ++i;
    const PrepMap &m = b.m[i];
    const int wpb = blockDim.x >> 5;
    prepare_rows(m.data, m.s[0], m.s[1], m.s[2], m.th, m.c[0], m.c[1], m.c[2], m.out,
                 (int)(blockIdx.x - m.first) * wpb + (int)(threadIdx.x >> 5), (b.m[i + 1].first - m.first) * wpb);
}

__global__ void k_init_u64(unsigned long long *p) {
    p[0] = 0ull;
    p[1] = 0ull;
}

// fastVEC statistics in float64, one block: dsum, Nact, ave, std, std_norm_ave.
constexpr int kStThreads = 1024;
__device__ __forceinline__ double st_block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        red[32] = s;
    }
    __syncthreads();
    return red[32];
}

__global__ void __launch_bounds__(kStThreads) k_stats(const double *data, size_t n, double *out) {
    __shared__ double red[33];
    double s = 0.0, cnt = 0.0, pos = 0.0, q = 0.0, np_ = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = data[i];
        s += v;
        if (v != 0.0) cnt += 1.0;
        if (v > 0.0) {
            pos += v;
            q += v * v;
            np_ += 1.0;
        }
    }
    s = st_block_sum(s, red);
    cnt = st_block_sum(cnt, red);
    pos = st_block_sum(pos, red);
    q = st_block_sum(q, red);
    np_ = st_block_sum(np_, red);
    const double ave = pos / np_;
    double p2 = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = data[i];
        if (v > 0.0) p2 += (v - ave) * (v - ave);
    }
    p2 = st_block_sum(p2, red);
    if (threadIdx.x == 0) {
        out[0] = s;
        out[1] = cnt;
        out[2] = ave;
        out[3] = sqrt(q);
        out[4] = sqrt(p2);
    }
}

// The same statistics over many blocks: per-chunk partial sums in a
// workspace, added in chunk order by one thread (deterministic), then the
// centred norm the same way.  Float64 runs at a small fraction of the float32
// rate on this part, so one block would leave the other SMs idle.
constexpr int kSmThreads = 256;
constexpr int kSmPerThread = 8;

__device__ __forceinline__ void sm_chunk(size_t n, size_t &lo, size_t &hi) {
    const size_t per = (size_t)kSmThreads * kSmPerThread;
    lo = (size_t)blockIdx.x * per;
    hi = lo + per < n ? lo + per : n;
}

__global__ void __launch_bounds__(kSmThreads) k_stats_p1(const double *data, size_t n, double *part) {
    __shared__ double red[33];
    size_t lo, hi;
    sm_chunk(n, lo, hi);
    double s = 0.0, cnt = 0.0, pos = 0.0, q = 0.0, np_ = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double v = data[i];
        s += v;
        if (v != 0.0) cnt += 1.0;
        if (v > 0.0) {
            pos += v;
            q += v * v;
            np_ += 1.0;
        }
    }
    s = st_block_sum(s, red);
    cnt = st_block_sum(cnt, red);
    pos = st_block_sum(pos, red);
    q = st_block_sum(q, red);
    np_ = st_block_sum(np_, red);
    if (threadIdx.x == 0) {
        double *p = part + (size_t)blockIdx.x * 6;
        p[0] = s;
        p[1] = cnt;
        p[2] = pos;
        p[3] = q;
        p[4] = np_;
    }
}

__global__ void k_stats_r1(const double *part, int nchunk, double *out) {
    if (threadIdx.x != 0) return;
    double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < nchunk; ++b)
        for (int k = 0; k < 5; ++k) a[k] += part[(size_t)b * 6 + k];
    out[0] = a[0];
    out[1] = a[1];
    out[2] = a[2] / a[4];
    out[3] = sqrt(a[3]);
}

__global__ void __launch_bounds__(kSmThreads) k_stats_p2(const double *data, size_t n, const double *out,
                                                         double *part) {
    __shared__ double red[33];
    size_t lo, hi;
    sm_chunk(n, lo, hi);
    const double ave = out[2];
    double p2 = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double v = data[i];
        if (v > 0.0) p2 += (v - ave) * (v - ave);
    }
    p2 = st_block_sum(p2, red);
    if (threadIdx.x == 0) part[(size_t)blockIdx.x * 6 + 5] = p2;
}

__global__ void k_stats_r2(const double *part, int nchunk, double *out) {
    if (threadIdx.x != 0) return;
    double p2 = 0.0;
    for (int b = 0; b < nchunk; ++b) p2 += part[(size_t)b * 6 + 5];
    out[4] = sqrt(p2);
}

static int stats_chunks(int dim) {
    const size_t n = (size_t)dim * dim * dim, per = (size_t)kSmThreads * kSmPerThread;
    return (int)((n + per - 1) / per);
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_prepare_map(float *data, int sx, int sy, int sz, double threshold, const double *cent,
                                  uint64_t *out2, void *stream) {
    if (!data || !cent || !out2 || sx < 1 || sy < 1 || sz < 1)
        return fail(VESPER_ERR_INVALID, "vesper_prepare_map: bad arguments");
    if ((long long)sx * sy > 0x7fffffffll) return fail(VESPER_ERR_UNSUPPORTED, "vesper_prepare_map: too many rows");
    const double th = threshold < 0 ? 0.0 : threshold;   // th < 0 leaves data unshifted (:73-79)
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long *acc = (unsigned long long *)out2;
    k_init_u64<<<1, 1, 0, st>>>(acc);
    const int blocks = std::max(1, std::min((sx * sy + 31) / 32, 152 * 16));
    k_prepare<<<blocks, 256, 0, st>>>(data, sx, sy, sz, (float)th, cent[0], cent[1], cent[2], acc);
    VG_CHECK_LAUNCH("k_prepare");
    return VESPER_OK;
}

extern "C" int vesper_prepare_maps(int nmap, float *const *data, const int *dims, const double *thresholds,
                                   const double *cents, uint64_t *out, void *stream) {
    if (nmap < 0 || (nmap > 0 && (!data || !dims || !thresholds || !cents || !out)))
        return fail(VESPER_ERR_INVALID, "vesper_prepare_maps: bad arguments");
    for (int i = 0; i < nmap; ++i)
        if (!data[i] || dims[3 * i] < 1 || dims[3 * i + 1] < 1 || dims[3 * i + 2] < 1)
            return fail(VESPER_ERR_INVALID, "vesper_prepare_maps: map %d: bad arguments", i);
        else if ((long long)dims[3 * i] * dims[3 * i + 1] > 0x7fffffffll)
            return fail(VESPER_ERR_UNSUPPORTED, "vesper_prepare_maps: map %d: too many rows", i);
    if (nmap == 0) return VESPER_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(out, 0, (size_t)nmap * 2 * sizeof(uint64_t), st) != cudaSuccess)
        return cuda_check("vesper_prepare_maps: clear");
    for (int i0 = 0; i0 < nmap; i0 += kPrepMax) {
        PrepBatch b{};
        b.nmap = std::min(kPrepMax, nmap - i0);
        int blocks = 0;
        for (int k = 0; k < b.nmap; ++k) {
            const int i = i0 + k;
            PrepMap &m = b.m[k];
            m.data = data[i];
            m.out = (unsigned long long *)out + 2 * (size_t)i;
            for (int a = 0; a < 3; ++a) {
                m.s[a] = dims[3 * i + a];
                m.c[a] = cents[3 * i + a];
            }
            m.th = (float)(thresholds[i] < 0 ? 0.0 : thresholds[i]);   // th < 0 leaves data unshifted (:73-79)
            m.first = blocks;
            const int rows = m.s[0] * m.s[1];
            blocks += std::max(1, std::min((rows + 31) / 32, 1024));   // 8 warps per block, about 4 rows per warp
        }
        b.m[b.nmap].first = blocks;
        k_prepare_many<<<blocks, 256, 0, st>>>(b);
        VG_CHECK_LAUNCH("k_prepare_many");
    }
    return VESPER_OK;
}

extern "C" int vesper_map_stats_workspace_size(int dim, size_t *bytes) {
    if (!bytes || dim < 1) return fail(VESPER_ERR_INVALID, "vesper_map_stats_workspace_size: bad arguments");
    *bytes = (size_t)stats_chunks(dim) * 6 * sizeof(double);
    return VESPER_OK;
}

extern "C" int vesper_map_stats(const double *data, int dim, double *stats_out, void *stream) {
    if (!data || !stats_out || dim < 1) return fail(VESPER_ERR_INVALID, "vesper_map_stats: bad arguments");
    k_stats<<<1, kStThreads, 0, (cudaStream_t)stream>>>(data, (size_t)dim * dim * dim, stats_out);
    VG_CHECK_LAUNCH("k_stats");
    return VESPER_OK;
}

extern "C" int vesper_map_stats_ws(const double *data, int dim, double *stats_out, void *workspace,
                                   size_t workspace_bytes, void *stream) {
    if (!data || !stats_out || dim < 1) return fail(VESPER_ERR_INVALID, "vesper_map_stats_ws: bad arguments");
    size_t need = 0;
    vesper_map_stats_workspace_size(dim, &need);
    if (!workspace || workspace_bytes < need) return fail(VESPER_ERR_WORKSPACE, "vesper_map_stats_ws: workspace");
    const size_t n = (size_t)dim * dim * dim;
    const int nc = stats_chunks(dim);
    double *part = (double *)workspace;
    cudaStream_t st = (cudaStream_t)stream;
    k_stats_p1<<<nc, kSmThreads, 0, st>>>(data, n, part);
    VG_CHECK_LAUNCH("k_stats_p1");
    k_stats_r1<<<1, 32, 0, st>>>(part, nc, stats_out);
    VG_CHECK_LAUNCH("k_stats_r1");
    k_stats_p2<<<nc, kSmThreads, 0, st>>>(data, n, stats_out, part);
    VG_CHECK_LAUNCH("k_stats_p2");
    k_stats_r2<<<1, 32, 0, st>>>(part, nc, stats_out);
    VG_CHECK_LAUNCH("k_stats_r2");
    return VESPER_OK;
}
