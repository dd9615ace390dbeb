// Learned rotation proposal: a small 3-D convolutional encoder applied to the
// target and the query vector fields, a rotational correlation of the two
// feature fields at zero translation over the angle grid, and the kernels to
// train it (backward passes, softmax cross-entropy, Adam).  Nothing in the
// reference corresponds to this: it orders the rotation grid so that only its
// best-scored fraction is correlated by vesper_search.
//
// Layouts: activations [C][d][d][d] float32 (channel-major); weights
// [Cout][Cin][27] stored as bfloat16 (3x3x3 taps, z fastest) with float32
// accumulation; biases float32.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "vesper_common.cuh"

namespace vg {

// blocks of the score backward pass (two waves of the 152 SMs at most); each
// keeps its partial gradients in shared memory and writes them to its own
// workspace slot
constexpr int kPropBlocks = 304;

// ---- convolution (3x3x3, zero padding) ----------------------------------------
__global__ void k_conv_fwd(const float *in, int cin, const __nv_bfloat16 *W, const float *bias, int cout, int d,
                           int relu, float *out) {
    const int n = d * d * d;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    const int co = blockIdx.y;
    in += (size_t)blockIdx.z * cin * n;     // map blockIdx.z of a stack
    out += (size_t)blockIdx.z * cout * n;
    if (v >= n) return;
    const int x = v / (d * d), y = (v / d) % d, z = v % d;
    float acc = bias ? bias[co] : 0.f;
    const __nv_bfloat16 *w = W + (size_t)co * cin * 27;
    for (int ci = 0; ci < cin; ++ci) {
        const float *src = in + (size_t)ci * n;
        const __nv_bfloat16 *wc = w + ci * 27;
#pragma unroll
        for (int o = 0; o < 27; ++o) {
            const int xx = x + o / 9 - 1, yy = y + (o / 3) % 3 - 1, zz = z + o % 3 - 1;
            if (xx < 0 || yy < 0 || zz < 0 || xx >= d || yy >= d || zz >= d) continue;
            acc = fmaf(__bfloat162float(wc[o]), src[(xx * d + yy) * d + zz], acc);
        }
    }
    out[(size_t)co * n + v] = relu ? fmaxf(acc, 0.f) : acc;
}

// The same layer with COG = 4 output channels and ZS consecutive z voxels per
// thread: the block's COG x cin x 27 weights sit in shared memory as float32 in
// [cin][27][channel] order (each tap's four weights are one 16-byte broadcast
// load), and for each input channel and (x, y) neighbour row the ZS + 2 input
// values of the row are loaded once, so each load feeds up to 3 x COG products
// and each weight load ZS x COG.  Taps outside the grid are skipped per voxel
// as in k_conv_fwd, in the same order (bias, then ci, then tap), so the
// results are the same bits.
constexpr int kConvCOG = 4;
constexpr int kConvZS = 4;   // measured over the prop128 step: 4 beat 2 and 1 (one voxel per thread)
template <int COG, int ZS>
__global__ void __launch_bounds__(128) k_conv_fwd_s(const float *in, int cin, const __nv_bfloat16 *W,
                                                    const float *bias, int cout, int d, int relu, float *out) {
    static_assert(COG == 4, "k_conv_fwd_s: 4 output channels per thread");
    extern __shared__ float4 wsh4[];   // [cin][27]
    float *wsh = (float *)wsh4;
    const int n = d * d * d, nzs = (d + ZS - 1) / ZS;
    const int co0 = blockIdx.y * COG;
    in += (size_t)blockIdx.z * cin * n;
    out += (size_t)blockIdx.z * cout * n;
    for (int i = threadIdx.x; i < COG * cin * 27; i += blockDim.x) {
        const int j = i / (cin * 27), t = i - j * cin * 27;   // t = ci * 27 + o
        wsh[t * COG + j] = __bfloat162float(W[(size_t)co0 * cin * 27 + i]);
    }
    __syncthreads();
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= d * d * nzs) return;
    const int x = u / (d * nzs), y = (u / nzs) % d, z0 = (u % nzs) * ZS;
    float acc[ZS][COG];
#pragma unroll
    for (int i = 0; i < ZS; ++i)
#pragma unroll
        for (int j = 0; j < COG; ++j) acc[i][j] = bias ? bias[co0 + j] : 0.f;
    for (int ci = 0; ci < cin; ++ci) {
        const float *src = in + (size_t)ci * n;
        const float4 *w = wsh4 + (size_t)ci * 27;
#pragma unroll
        for (int ox = 0; ox < 3; ++ox) {
            const int xx = x + ox - 1;
            if (xx < 0 || xx >= d) continue;
#pragma unroll
            for (int oy = 0; oy < 3; ++oy) {
                const int yy = y + oy - 1;
                if (yy < 0 || yy >= d) continue;
                const float *row = src + ((size_t)xx * d + yy) * d;
                float val[ZS + 2];
#pragma unroll
                for (int e = 0; e < ZS + 2; ++e) {
                    const int zz = z0 + e - 1;
                    val[e] = zz >= 0 && zz < d ? row[zz] : 0.f;
                }
#pragma unroll
                for (int oz = 0; oz < 3; ++oz) {
                    const float4 w4 = w[ox * 9 + oy * 3 + oz];
#pragma unroll
                    for (int i = 0; i < ZS; ++i) {
                        const int zz = z0 + i + oz - 1;
                        if (zz < 0 || zz >= d) continue;
                        const float v = val[i + oz];
                        acc[i][0] = fmaf(w4.x, v, acc[i][0]);
                        acc[i][1] = fmaf(w4.y, v, acc[i][1]);
                        acc[i][2] = fmaf(w4.z, v, acc[i][2]);
                        acc[i][3] = fmaf(w4.w, v, acc[i][3]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < ZS; ++i) {
        const int z = z0 + i;
        if (z >= d) break;
        const size_t v = ((size_t)x * d + y) * d + z;
#pragma unroll
        for (int j = 0; j < COG; ++j) out[(size_t)(co0 + j) * n + v] = relu ? fmaxf(acc[i][j], 0.f) : acc[i][j];
    }
}

// din[ci][v] = sum_co sum_o W[co][ci][o] * g[co][v - o],  g = dout (masked by
// out > 0 for a ReLU layer)
__global__ void k_conv_bwd_data(const float *dout, const float *out, int relu, const __nv_bfloat16 *W, int cin,
                                int cout, int d, float *din) {
    const int n = d * d * d;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    const int ci = blockIdx.y;
    if (v >= n) return;
    const int x = v / (d * d), y = (v / d) % d, z = v % d;
    float acc = 0.f;
    for (int co = 0; co < cout; ++co) {
        const float *g = dout + (size_t)co * n;
        const float *o_ = out + (size_t)co * n;
        const __nv_bfloat16 *wc = W + ((size_t)co * cin + ci) * 27;
#pragma unroll
        for (int o = 0; o < 27; ++o) {
            const int xx = x - (o / 9 - 1), yy = y - ((o / 3) % 3 - 1), zz = z - (o % 3 - 1);
            if (xx < 0 || yy < 0 || zz < 0 || xx >= d || yy >= d || zz >= d) continue;
            const int u = (xx * d + yy) * d + zz;
            const float gv = (relu && !(o_[u] > 0.f)) ? 0.f : g[u];
            acc = fmaf(__bfloat162float(wc[o]), gv, acc);
        }
    }
    din[(size_t)ci * n + v] = acc;
}

// dW[co][ci][o] += sum_v g[co][v] * in[ci][v + o]; db[co] += sum_v g[co][v].
// One block per (co, ci); 27 taps reduced over the voxels.
__global__ void k_conv_bwd_weight(const float *dout, const float *out, int relu, const float *in, int cin, int cout,
                                  int d, float *dW, float *db) {
    const int n = d * d * d;
    const int co = blockIdx.x / cin, ci = blockIdx.x % cin;
    __shared__ float red[28][32];
    float acc[28];
#pragma unroll
    for (int o = 0; o < 28; ++o) acc[o] = 0.f;
    const float *g = dout + (size_t)co * n;
    const float *o_ = out + (size_t)co * n;
    const float *src = in + (size_t)ci * n;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
        const float gv = (relu && !(o_[v] > 0.f)) ? 0.f : g[v];
        if (gv == 0.f) continue;
        const int x = v / (d * d), y = (v / d) % d, z = v % d;
#pragma unroll
        for (int o = 0; o < 27; ++o) {
            const int xx = x + o / 9 - 1, yy = y + (o / 3) % 3 - 1, zz = z + o % 3 - 1;
            if (xx < 0 || yy < 0 || zz < 0 || xx >= d || yy >= d || zz >= d) continue;
            acc[o] = fmaf(gv, src[(xx * d + yy) * d + zz], acc[o]);
        }
        acc[27] += gv;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 0; o < 28; ++o) {
        float s = acc[o];
        for (int k = 16; k > 0; k >>= 1) s += __shfl_down_sync(0xffffffffu, s, k);
        if (lane == 0) red[o][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x < 28) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
        if (threadIdx.x < 27)
            dW[((size_t)co * cin + ci) * 27 + threadIdx.x] += s;
        else if (ci == 0)
            db[co] += s;
    }
}

// ---- network input ---------------------------------------------------------------
// out[c][X][Y][Z], c = (vx, vy, vz, mask = data != 0), each the mean over the
// pool^3 block of voxels (pool X .. pool X + pool - 1, clipped at the grid
// edge) of the fastVEC output of one map.
__global__ void k_prop_field(const double *data, const float *vec, int d, int pool, int dp, float *out) {
    const int np = dp * dp * dp;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int X = i / (dp * dp), Y = (i / dp) % dp, Z = i % dp;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    int cnt = 0;
    for (int x = X * pool; x < min(d, X * pool + pool); ++x)
        for (int y = Y * pool; y < min(d, Y * pool + pool); ++y)
            for (int z = Z * pool; z < min(d, Z * pool + pool); ++z) {
                const size_t v = ((size_t)x * d + y) * d + z;
                acc[0] += vec[3 * v];
                acc[1] += vec[3 * v + 1];
                acc[2] += vec[3 * v + 2];
                acc[3] += data[v] != 0.0 ? 1.f : 0.f;
                ++cnt;
            }
    const float inv = 1.f / (float)cnt;
#pragma unroll
    for (int c = 0; c < 4; ++c) out[(size_t)c * np + i] = acc[c] * inv;
}

// ---- rotational correlation at zero translation --------------------------------
// Source voxel of destination v under rotation F: the reference's gather rule
// (gather_src) with every in-bounds voxel accepted.
__device__ __forceinline__ int prop_src(const float *F, int d, int v) {
    const int x = v / (d * d), y = (v / d) % d, z = v % d;
    return gather_src(F, d, x, y, z, [](int) { return true; });
}

// s[r] = sum_v sum_k ET[k][v] * EQ[k][src_r(v)]; one block per rotation.
__global__ void k_prop_score(const float *ET, const float *EQ, int K, int d, const float *rotmats, int nrot,
                             float *scores) {
    __shared__ float F[9];
    __shared__ float red[32];
    const int r = blockIdx.x;
    if (threadIdx.x < 9) F[threadIdx.x] = rotmats[(size_t)r * 9 + threadIdx.x];
    __syncthreads();
    const int n = d * d * d;
    float acc = 0.f;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
        const int s = prop_src(F, d, v);
        if (s < 0) continue;
        for (int k = 0; k < K; ++k) acc = fmaf(ET[(size_t)k * n + v], EQ[(size_t)k * n + s], acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        scores[r] = s;
    }
}

// [nmap][K][n] -> [nmap][n][K]
__global__ void k_vmajor(const float *in, int K, int n, float *out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t per = (size_t)K * n;
    if (i >= per) return;
    const size_t m = blockIdx.y;
    const int v = (int)(i / K), k = (int)(i % K);
    out[m * per + i] = in[m * per + (size_t)k * n + v];
}

// The same scores from voxel-major features (K a multiple of 4): one voxel's
// K channels are K/4 float4 loads, so the gathered query voxel costs whole
// 32-byte sectors instead of K scattered words.
template <int K4>
__global__ void k_prop_score_vm(const float4 *ET, const float4 *EQ, int d, const float *rotmats, float *scores) {
    __shared__ float F[9];
    __shared__ float red[32];
    const int r = blockIdx.x;
    if (threadIdx.x < 9) F[threadIdx.x] = rotmats[(size_t)r * 9 + threadIdx.x];
    __syncthreads();
    const int n = d * d * d;
    float acc = 0.f;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
        const int s = prop_src(F, d, v);
        if (s < 0) continue;
#pragma unroll
        for (int j = 0; j < K4; ++j) {
            const float4 a = __ldg(ET + (size_t)v * K4 + j), b = __ldg(EQ + (size_t)s * K4 + j);
            acc = fmaf(a.x, b.x, acc);
            acc = fmaf(a.y, b.y, acc);
            acc = fmaf(a.z, b.z, acc);
            acc = fmaf(a.w, b.w, acc);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        scores[r] = t;
    }
}

// [nmap][K][n] float32 -> [nmap][n][K] float16 (the inference features)
__global__ void k_vmajor_f16(const float *in, int K, int n, __half *out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t per = (size_t)K * n;
    if (i >= per) return;
    const size_t m = blockIdx.y;
    const int v = (int)(i / K), k = (int)(i % K);
    out[m * per + i] = __float2half_rn(in[m * per + (size_t)k * n + (size_t)v]);
}

// Scores of RPB rotations per block from float16 voxel-major features, K8
// groups of 8 channels (one 16-byte load per voxel and group): each target
// voxel's features are loaded once for the block's RPB rotations, the
// gathered query voxel once per rotation; products accumulate in float32.
template <int K8, int RPB>
__global__ void __launch_bounds__(256) k_prop_score_f16(const uint4 *ET, const uint4 *EQ, int d,
                                                        const float *rotmats, int nrot, float *scores) {
    __shared__ float F[RPB][9];
    __shared__ float red[RPB][32];
    const int r0 = blockIdx.x * RPB;
    if (threadIdx.x < 9 * RPB) {
        const int j = threadIdx.x / 9, e = threadIdx.x % 9;
        F[j][e] = r0 + j < nrot ? rotmats[(size_t)(r0 + j) * 9 + e] : 0.f;
    }
    __syncthreads();
    const int n = d * d * d;
    float acc[RPB];
#pragma unroll
    for (int j = 0; j < RPB; ++j) acc[j] = 0.f;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
        float2 t[K8][4];
#pragma unroll
        for (int g = 0; g < K8; ++g) {
            const uint4 a = __ldg(ET + (size_t)v * K8 + g);
            t[g][0] = __half22float2(*(const __half2 *)&a.x);
            t[g][1] = __half22float2(*(const __half2 *)&a.y);
            t[g][2] = __half22float2(*(const __half2 *)&a.z);
            t[g][3] = __half22float2(*(const __half2 *)&a.w);
        }
#pragma unroll
        for (int j = 0; j < RPB; ++j) {
            if (r0 + j >= nrot) break;
            const int s = prop_src(F[j], d, v);
            if (s < 0) continue;
#pragma unroll
            for (int g = 0; g < K8; ++g) {
                const uint4 b = __ldg(EQ + (size_t)s * K8 + g);
                const float2 q0 = __half22float2(*(const __half2 *)&b.x), q1 = __half22float2(*(const __half2 *)&b.y);
                const float2 q2 = __half22float2(*(const __half2 *)&b.z), q3 = __half22float2(*(const __half2 *)&b.w);
                float a = acc[j];
                a = fmaf(t[g][0].x, q0.x, a);
                a = fmaf(t[g][0].y, q0.y, a);
                a = fmaf(t[g][1].x, q1.x, a);
                a = fmaf(t[g][1].y, q1.y, a);
                a = fmaf(t[g][2].x, q2.x, a);
                a = fmaf(t[g][2].y, q2.y, a);
                a = fmaf(t[g][3].x, q3.x, a);
                a = fmaf(t[g][3].y, q3.y, a);
                acc[j] = a;
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < RPB; ++j) {
        float a = acc[j];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) red[j][warp] = a;
    }
    __syncthreads();
    if (threadIdx.x < RPB && r0 + (int)threadIdx.x < nrot) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
        scores[r0 + threadIdx.x] = t;
    }
}

// Source voxel of every (rotation, destination voxel) of a small grid, as
// int16 (-1: none): the rotation grid is fixed, so the gather geometry is
// computed once and then streamed from HBM (nrot * d^3 * 2 bytes) instead of
// being recomputed for every map pair.
__global__ void k_prop_srcmap(int d, const float *rotmats, int nrot, int16_t *out) {
    __shared__ float F[9];
    const int r = blockIdx.y;
    if (threadIdx.x < 9) F[threadIdx.x] = rotmats[(size_t)r * 9 + threadIdx.x];
    __syncthreads();
    const int n = d * d * d;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    out[(size_t)r * n + v] = (int16_t)prop_src(F, d, v);
}

// Scores from float16 voxel-major features and a precomputed source map:
// RPB rotations per block, each target voxel's features loaded once for them.
template <int K8, int RPB>
__global__ void __launch_bounds__(256) k_prop_score_map(const uint4 *ET, const uint4 *EQ, int d,
                                                        const int16_t *srcmap, int nrot, float *scores) {
    __shared__ float red[RPB][32];
    const int r0 = blockIdx.x * RPB;
    const int n = d * d * d;
    float acc[RPB];
#pragma unroll
    for (int j = 0; j < RPB; ++j) acc[j] = 0.f;
    for (int v = threadIdx.x; v < n; v += blockDim.x) {
        int sj[RPB];
#pragma unroll
        for (int j = 0; j < RPB; ++j) sj[j] = r0 + j < nrot ? (int)__ldg(srcmap + (size_t)(r0 + j) * n + v) : -1;
        float2 t[K8][4];
#pragma unroll
        for (int g = 0; g < K8; ++g) {
            const uint4 a = __ldg(ET + (size_t)v * K8 + g);
            t[g][0] = __half22float2(*(const __half2 *)&a.x);
            t[g][1] = __half22float2(*(const __half2 *)&a.y);
            t[g][2] = __half22float2(*(const __half2 *)&a.z);
            t[g][3] = __half22float2(*(const __half2 *)&a.w);
        }
#pragma unroll
        for (int j = 0; j < RPB; ++j) {
            const int s = sj[j];
            if (s < 0) continue;
#pragma unroll
            for (int g = 0; g < K8; ++g) {
                const uint4 b = __ldg(EQ + (size_t)s * K8 + g);
                const float2 q0 = __half22float2(*(const __half2 *)&b.x), q1 = __half22float2(*(const __half2 *)&b.y);
                const float2 q2 = __half22float2(*(const __half2 *)&b.z), q3 = __half22float2(*(const __half2 *)&b.w);
                float a = acc[j];
                a = fmaf(t[g][0].x, q0.x, a);
                a = fmaf(t[g][0].y, q0.y, a);
                a = fmaf(t[g][1].x, q1.x, a);
                a = fmaf(t[g][1].y, q1.y, a);
                a = fmaf(t[g][2].x, q2.x, a);
                a = fmaf(t[g][2].y, q2.y, a);
                a = fmaf(t[g][3].x, q3.x, a);
                a = fmaf(t[g][3].y, q3.y, a);
                acc[j] = a;
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < RPB; ++j) {
        float a = acc[j];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) red[j][warp] = a;
    }
    __syncthreads();
    if (threadIdx.x < RPB && r0 + (int)threadIdx.x < nrot) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
        scores[r0 + threadIdx.x] = t;
    }
}

// The same scores with the query's features staged in shared memory: block
// (pair p, chunk c) scores rotations [c kScChunk, (c + 1) kScChunk) of pair p,
// so each rotation's gathers are shared-memory loads instead of scattered L1
// lines, and the blocks of one chunk (consecutive in launch order, pair index
// fastest) read that chunk of the gather map while it is in L2.  Row n of the
// staged features is zero and stands for "no source voxel" (the product of a
// finite feature with +0 adds nothing).  Thread t sums voxels t, t + 256, ...
// in the order of k_prop_score_map and the reduction is the same, so the scores
// are bit-identical to it.  Pair p reads ET + p pstride and EQ + p pstride
// (uint4 units) and writes scores + p nrot.
constexpr int kScChunk = 32;
constexpr int kScRPB = 8;

// c + a.lo * b.lo, then + a.hi * b.hi, for packed float16 pairs a, b: each step
// one fma.rn.f32.f16 (float16 operands, float32 addend and result, one
// rounding), which equals fmaf on the operands converted to float32 (the
// conversion is exact and the product of two float16 values is exact in
// float32).
__device__ __forceinline__ float fma_h2_f32(uint32_t a, uint32_t b, float c) {
    float d;
    asm("{\n\t.reg .f16 al, ah, bl, bh;\n\t"
        "mov.b32 {al, ah}, %1;\n\t"
        "mov.b32 {bl, bh}, %2;\n\t"
        "fma.rn.f32.f16 %0, al, bl, %3;\n\t"
        "fma.rn.f32.f16 %0, ah, bh, %0;\n\t}"
        : "=f"(d) : "r"(a), "r"(b), "f"(c));
    return d;
}
template <int K8>
__global__ void __launch_bounds__(256) k_prop_score_map_s(const uint4 *ET, const uint4 *EQ, size_t pstride,
                                                          int npair, int d, const int16_t *srcmap, int nrot,
                                                          float *scores) {
    extern __shared__ uint4 sq[];   // [n + 1][K8]
    __shared__ float red[kScRPB][8];
    const int n = d * d * d;
    const int p = blockIdx.x % npair, c = blockIdx.x / npair;
    const uint4 *et = ET + (size_t)p * pstride, *eq = EQ + (size_t)p * pstride;
    for (int e = threadIdx.x; e < n * K8; e += blockDim.x) sq[e] = __ldg(eq + e);
    if (threadIdx.x < K8) sq[(size_t)n * K8 + threadIdx.x] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rend = min(nrot, (c + 1) * kScChunk);
    for (int r0 = c * kScChunk; r0 < rend; r0 += kScRPB) {
        float acc[kScRPB];
#pragma unroll
        for (int j = 0; j < kScRPB; ++j) acc[j] = 0.f;
        for (int v = threadIdx.x; v < n; v += blockDim.x) {
            int sj[kScRPB];
#pragma unroll
            for (int j = 0; j < kScRPB; ++j) {
                const int s = r0 + j < rend ? (int)__ldg(srcmap + (size_t)(r0 + j) * n + v) : -1;
                sj[j] = s < 0 ? n : s;
            }
            uint4 t[K8];
#pragma unroll
            for (int g = 0; g < K8; ++g) t[g] = __ldg(et + (size_t)v * K8 + g);
#pragma unroll
            for (int j = 0; j < kScRPB; ++j) {
#pragma unroll
                for (int g = 0; g < K8; ++g) {
                    const uint4 b = sq[(size_t)sj[j] * K8 + g];
                    float a = acc[j];
                    a = fma_h2_f32(t[g].x, b.x, a);
                    a = fma_h2_f32(t[g].y, b.y, a);
                    a = fma_h2_f32(t[g].z, b.z, a);
                    a = fma_h2_f32(t[g].w, b.w, a);
                    acc[j] = a;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < kScRPB; ++j) {
            float a = acc[j];
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if (lane == 0) red[j][warp] = a;
        }
        __syncthreads();
        if (threadIdx.x < kScRPB && r0 + (int)threadIdx.x < rend) {
            float t = 0.f;
            for (int w = 0; w < 8; ++w) t += red[threadIdx.x][w];
            scores[(size_t)p * nrot + r0 + threadIdx.x] = t;
        }
        __syncthreads();   // red is rewritten by the next group
    }
}

// Partial gradients of the correlation for channels [k0, k0 + kc): block b
// takes rotations [b*chunk, (b+1)*chunk) and writes part[b][0][k][v] =
// sum_r g_r EQ[k][src_r(v)] and part[b][1][k][s] = sum_r g_r ET[k][v] summed
// over the v with src_r(v) = s, accumulated in shared memory.
__global__ void k_prop_score_bwd(const float *ET, const float *EQ, int K, int k0, int kc, int d,
                                 const float *rotmats, int nrot, const float *gs, int chunk, float *part) {
    extern __shared__ __align__(16) float sm[];
    const int n = d * d * d;
    float *gT = sm;             // [kc][n]
    float *gQ = sm + kc * n;    // [kc][n]
    __shared__ float F[9];
    for (int i = threadIdx.x; i < 2 * kc * n; i += blockDim.x) sm[i] = 0.f;
    const int r0 = blockIdx.x * chunk, r1 = min(nrot, r0 + chunk);
    for (int r = r0; r < r1; ++r) {
        __syncthreads();
        if (threadIdx.x < 9) F[threadIdx.x] = rotmats[(size_t)r * 9 + threadIdx.x];
        __syncthreads();
        const float g = gs[r];
        if (g == 0.f) continue;
        for (int v = threadIdx.x; v < n; v += blockDim.x) {
            const int s = prop_src(F, d, v);
            if (s < 0) continue;
            for (int k = 0; k < kc; ++k) {
                gT[k * n + v] = fmaf(g, EQ[(size_t)(k0 + k) * n + s], gT[k * n + v]);
                atomicAdd(&gQ[k * n + s], g * ET[(size_t)(k0 + k) * n + v]);
            }
        }
    }
    __syncthreads();
    float *dst = part + (size_t)blockIdx.x * 2 * K * n;
    for (int i = threadIdx.x; i < 2 * kc * n; i += blockDim.x) {
        const int half = i / (kc * n), rem = i % (kc * n);
        dst[(size_t)half * K * n + (size_t)k0 * n + rem] = sm[i];
    }
}

__global__ void k_sum_parts(const float *part, int nparts, int len, float *out_a, float *out_b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * len) return;
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += part[(size_t)p * 2 * len + i];
    if (i < len)
        out_a[i] += s;
    else
        out_b[i - len] += s;
}

// ---- loss ---------------------------------------------------------------------
// Block-wide sum / max of one value per thread (blockDim a multiple of 32).
__device__ float block_sum(float v, float *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float t = 0.f;
    for (int w = 0; w < nw; ++w) t += red[w];
    return t;
}
__device__ float block_max(float v, float *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float t = -INFINITY;
    for (int w = 0; w < nw; ++w) t = fmaxf(t, red[w]);
    return t;
}

// Standardised scores u = (s - mean) / std over the rotations, p =
// softmax(u / tau), loss += -sum q log p, and the gradient with respect to s
// through the standardisation:
//   gu = (p - q) / tau,  gs = (gu - mean(gu) - u * mean(gu * u)) / std.
// One block; three passes over the n scores.
__global__ void k_softmax_ce(const float *s, const float *q, int n, float tau, float *loss, float *g) {
    __shared__ float red[32];
    float a = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a += s[i];
    const float mu = block_sum(a, red) / (float)n;
    a = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float t = s[i] - mu;
        a = fmaf(t, t, a);
    }
    const float sd = sqrtf(block_sum(a, red) / (float)n) + 1e-6f;
    const float inv = 1.f / sd;
    float m = -INFINITY;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, (s[i] - mu) * inv / tau);
    m = block_max(m, red);
    a = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a += expf((s[i] - mu) * inv / tau - m);
    const float lz = logf(block_sum(a, red));
    float l = 0.f, sg = 0.f, sgu = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float u = (s[i] - mu) * inv;
        const float lp = u / tau - m - lz;
        l -= q[i] * lp;
        const float gu = (expf(lp) - q[i]) / tau;
        g[i] = gu;
        sg += gu;
        sgu = fmaf(gu, u, sgu);
    }
    l = block_sum(l, red);
    const float mg = block_sum(sg, red) / (float)n;
    const float mgu = block_sum(sgu, red) / (float)n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float u = (s[i] - mu) * inv;
        g[i] = (g[i] - mg - u * mgu) * inv;
    }
    if (threadIdx.x == 0) *loss += l;
}

// ---- Adam (float32 master weights, bfloat16 copies for the convolutions) ------
__global__ void k_adam(float *w, float *m, float *v, const float *g, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2, float gscale, __nv_bfloat16 *wbf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * gscale;
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
    if (wbf) wbf[i] = __float2bfloat16(w[i]);
}

// ---- top-k subset: indices of the k largest scores (ties to lower index) --------
// One block: the k-th largest order-preserving key by a most-significant-digit
// radix select (four passes of 8 bits over per-warp shared histograms), then
// an ordered compaction.  The keys sit in shared memory when they fit
// (skeys), else they are re-read from global memory each pass.
constexpr int kTkWarps = 1024 / 32;
__global__ void __launch_bounds__(1024) k_topk_subset(const float *s, int n, int k, int32_t *idx, int skeys) {
    extern __shared__ uint32_t dyn[];
    uint32_t *hist = dyn;                       // [kTkWarps][256] per-warp digit counts
    uint32_t *keys = dyn + kTkWarps * 256;      // [n] when skeys
    __shared__ unsigned int cnt;
    __shared__ int ncount[1024 / 32];
    __shared__ uint32_t sel_digit, sel_need;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s += (size_t)blockIdx.x * n;     // block b: score row b
    idx += (size_t)blockIdx.x * k;
    if (skeys) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = float_order(s[i]);
    }
    __syncthreads();
    auto key = [&](int i) -> uint32_t { return skeys ? keys[i] : float_order(s[i]); };
    // digits from the top: prefix/mask select the keys that still compete;
    // need = how many of the k still have to come from them
    uint32_t prefix = 0u, mask = 0u, need = (uint32_t)k;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < kTkWarps * 256; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
        uint32_t *hw = hist + warp * 256;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const uint32_t kv = key(i);
            if ((kv & mask) == prefix) atomicAdd(&hw[(kv >> shift) & 255u], 1u);
        }
        __syncthreads();
        // fold the warps' histograms into the first one
        for (int b = threadIdx.x; b < 256; b += blockDim.x) {
            uint32_t t = 0;
            for (int w = 0; w < kTkWarps; ++w) t += hist[w * 256 + b];
            hist[b] = t;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t cum = 0, d = 0, nd = need;
            for (int b = 255; b >= 0; --b) {
                const uint32_t c = hist[b];
                if (cum + c >= need) {
                    d = (uint32_t)b;
                    nd = need - cum;
                    break;
                }
                cum += c;
            }
            sel_digit = d;
            sel_need = nd;
        }
        __syncthreads();
        prefix |= sel_digit << shift;
        mask |= 255u << shift;
        need = sel_need;
        __syncthreads();
    }
    const uint32_t t = prefix;   // the k-th largest key: count(key > t) < k <= count(key >= t)
    // strictly above the threshold first, then ties in index order, k in total
    if (threadIdx.x == 0) cnt = 0u;
    __syncthreads();
    unsigned int above = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) above += key(i) > t;
    for (int o = 16; o > 0; o >>= 1) above += __shfl_down_sync(0xffffffffu, above, o);
    if (lane == 0) atomicAdd(&cnt, above);
    __syncthreads();
    const int n_above = (int)cnt;
    // one ordered compaction: every index above the threshold and the first
    // (k - n_above) ties, in ascending index order
    const int ties_wanted = k - n_above;
    int base_sel = 0, base_tie = 0;
    for (int start = 0; start < n; start += blockDim.x) {
        const int i = start + threadIdx.x;
        const uint32_t kv = i < n ? key(i) : 0u;
        const int is_above = i < n && kv > t, is_tie = i < n && kv == t;
        const unsigned lower = (1u << lane) - 1u;
        // tie positions first (warp ballot, then a prefix over the warps)
        const unsigned mt = __ballot_sync(0xffffffffu, is_tie);
        if (lane == 0) ncount[warp] = __popc(mt);
        __syncthreads();
        int pt = 0, tt = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            if (w < warp) pt += ncount[w];
            tt += ncount[w];
        }
        const int sel = is_above || (is_tie && base_tie + pt + __popc(mt & lower) < ties_wanted);
        __syncthreads();
        const unsigned ms = __ballot_sync(0xffffffffu, sel);
        if (lane == 0) ncount[warp] = __popc(ms);
        __syncthreads();
        int ps = 0, ts = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            if (w < warp) ps += ncount[w];
            ts += ncount[w];
        }
        if (sel) idx[base_sel + ps + __popc(ms & lower)] = i;
        base_sel += ts;
        base_tie += tt;
        __syncthreads();
    }
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_prop_field(const double *data, const float *vec, int d, int pool, float *out, void *stream) {
    if (!data || !vec || !out || d < 1 || pool < 1) return fail(VESPER_ERR_INVALID, "prop_field: bad args");
    const int dp = (d + pool - 1) / pool;
    const int np = dp * dp * dp;
    k_prop_field<<<(np + 127) / 128, 128, 0, (cudaStream_t)stream>>>(data, vec, d, pool, dp, out);
    VG_CHECK_LAUNCH("k_prop_field");
    return VESPER_OK;
}

extern "C" int vesper_prop_conv_fwd(const float *in, int cin, const void *W, const float *bias, int cout, int d,
                                    int relu, int nmap, float *out, void *stream) {
    if (!in || !W || !out || cin < 1 || cout < 1 || d < 1 || nmap < 1 || nmap > 65535)
        return fail(VESPER_ERR_INVALID, "conv_fwd: bad args");
    const int n = d * d * d;
    // 4 output channels per thread (8 measured 10 % slower over the encoder), 4 z voxels
    constexpr int COG = kConvCOG, ZS = kConvZS;
    const size_t sm = (size_t)COG * cin * 27 * sizeof(float);
    if (cout % COG == 0 && sm <= (size_t)smem_limit()) {
        const int nu = d * d * ((d + ZS - 1) / ZS);
        allow_smem(k_conv_fwd_s<COG, ZS>, sm);
        k_conv_fwd_s<COG, ZS><<<dim3((nu + 127) / 128, cout / COG, nmap), 128, sm, (cudaStream_t)stream>>>(
            in, cin, (const __nv_bfloat16 *)W, bias, cout, d, relu, out);
        VG_CHECK_LAUNCH("k_conv_fwd_s");
        return VESPER_OK;
    }
    k_conv_fwd<<<dim3((n + 127) / 128, cout, nmap), 128, 0, (cudaStream_t)stream>>>(
        in, cin, (const __nv_bfloat16 *)W, bias, cout, d, relu, out);
    VG_CHECK_LAUNCH("k_conv_fwd");
    return VESPER_OK;
}

extern "C" int vesper_prop_conv_bwd(const float *dout, const float *out, int relu, const float *in, const void *W,
                                    int cin, int cout, int d, float *din, float *dW, float *db, void *stream) {
    if (!dout || !out || !in || !W || !dW || !db || cin < 1 || cout < 1 || d < 1)
        return fail(VESPER_ERR_INVALID, "conv_bwd: bad args");
    const int n = d * d * d;
    cudaStream_t st = (cudaStream_t)stream;
    if (din) {
        k_conv_bwd_data<<<dim3((n + 127) / 128, cin), 128, 0, st>>>(dout, out, relu, (const __nv_bfloat16 *)W, cin,
                                                                    cout, d, din);
        VG_CHECK_LAUNCH("k_conv_bwd_data");
    }
    k_conv_bwd_weight<<<cout * cin, 256, 0, st>>>(dout, out, relu, in, cin, cout, d, dW, db);
    VG_CHECK_LAUNCH("k_conv_bwd_weight");
    return VESPER_OK;
}

extern "C" int vesper_prop_score(const float *ET, const float *EQ, int K, int d, const float *rotmats, int nrot,
                                 float *scores, void *stream) {
    if (!ET || !EQ || !rotmats || !scores || K < 1 || d < 1 || nrot < 0)
        return fail(VESPER_ERR_INVALID, "prop_score: bad args");
    if (nrot == 0) return VESPER_OK;
    k_prop_score<<<nrot, 256, 0, (cudaStream_t)stream>>>(ET, EQ, K, d, rotmats, nrot, scores);
    VG_CHECK_LAUNCH("k_prop_score");
    return VESPER_OK;
}

extern "C" int vesper_prop_vmajor(const float *in, int K, int d, int nmap, float *out, void *stream) {
    if (!in || !out || K < 1 || d < 1 || nmap < 1 || nmap > 65535) return fail(VESPER_ERR_INVALID, "vmajor: bad args");
    const size_t per = (size_t)K * d * d * d;
    k_vmajor<<<dim3((unsigned)((per + 255) / 256), nmap), 256, 0, (cudaStream_t)stream>>>(in, K, d * d * d, out);
    VG_CHECK_LAUNCH("k_vmajor");
    return VESPER_OK;
}

extern "C" int vesper_prop_score_vm(const float *ET, const float *EQ, int K, int d, const float *rotmats, int nrot,
                                    float *scores, void *stream) {
    if (!ET || !EQ || !rotmats || !scores || d < 1 || nrot < 0 || K < 4 || K % 4 || K > 32)
        return fail(VESPER_ERR_INVALID, "prop_score_vm: bad args (K a multiple of 4, <= 32)");
    if (((uintptr_t)ET | (uintptr_t)EQ) & 15) return fail(VESPER_ERR_INVALID, "prop_score_vm: 16-byte alignment");
    if (nrot == 0) return VESPER_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const float4 *a = (const float4 *)ET, *b = (const float4 *)EQ;
    switch (K / 4) {
        case 1: k_prop_score_vm<1><<<nrot, 256, 0, st>>>(a, b, d, rotmats, scores); break;
        case 2: k_prop_score_vm<2><<<nrot, 256, 0, st>>>(a, b, d, rotmats, scores); break;
        case 4: k_prop_score_vm<4><<<nrot, 256, 0, st>>>(a, b, d, rotmats, scores); break;
        case 8: k_prop_score_vm<8><<<nrot, 256, 0, st>>>(a, b, d, rotmats, scores); break;
        default: return fail(VESPER_ERR_UNSUPPORTED, "prop_score_vm: K = %d", K);
    }
    VG_CHECK_LAUNCH("k_prop_score_vm");
    return VESPER_OK;
}

extern "C" int vesper_prop_vmajor_f16(const float *in, int K, int d, int nmap, void *out, void *stream) {
    if (!in || !out || K < 1 || d < 1 || nmap < 1 || nmap > 65535)
        return fail(VESPER_ERR_INVALID, "vmajor_f16: bad args");
    const size_t per = (size_t)K * d * d * d;
    k_vmajor_f16<<<dim3((unsigned)((per + 255) / 256), nmap), 256, 0, (cudaStream_t)stream>>>(in, K, d * d * d,
                                                                                              (__half *)out);
    VG_CHECK_LAUNCH("k_vmajor_f16");
    return VESPER_OK;
}

extern "C" int vesper_prop_score_f16(const void *ET, const void *EQ, int K, int d, const float *rotmats, int nrot,
                                     float *scores, void *stream) {
    if (!ET || !EQ || !rotmats || !scores || d < 1 || nrot < 0 || K < 8 || K % 8 || K > 32)
        return fail(VESPER_ERR_INVALID, "prop_score_f16: bad args (K a multiple of 8, <= 32)");
    if (((uintptr_t)ET | (uintptr_t)EQ) & 15) return fail(VESPER_ERR_INVALID, "prop_score_f16: 16-byte alignment");
    if (nrot == 0) return VESPER_OK;
    cudaStream_t st = (cudaStream_t)stream;
    constexpr int RPB = 4;
    const unsigned nb = (unsigned)((nrot + RPB - 1) / RPB);
    const uint4 *a = (const uint4 *)ET, *b = (const uint4 *)EQ;
    switch (K / 8) {
        case 1: k_prop_score_f16<1, RPB><<<nb, 256, 0, st>>>(a, b, d, rotmats, nrot, scores); break;
        case 2: k_prop_score_f16<2, RPB><<<nb, 256, 0, st>>>(a, b, d, rotmats, nrot, scores); break;
        case 4: k_prop_score_f16<4, RPB><<<nb, 256, 0, st>>>(a, b, d, rotmats, nrot, scores); break;
        default: return fail(VESPER_ERR_UNSUPPORTED, "prop_score_f16: K = %d", K);
    }
    VG_CHECK_LAUNCH("k_prop_score_f16");
    return VESPER_OK;
}

extern "C" int vesper_prop_srcmap(int d, const float *rotmats, int nrot, void *srcmap_out, void *stream) {
    if (!rotmats || !srcmap_out || d < 1 || nrot < 0 || nrot > 65535)
        return fail(VESPER_ERR_INVALID, "prop_srcmap: bad args");
    if ((long long)d * d * d > 32767) return fail(VESPER_ERR_UNSUPPORTED, "prop_srcmap: d^3 above int16");
    if (nrot == 0) return VESPER_OK;
    const int n = d * d * d;
    k_prop_srcmap<<<dim3((n + 255) / 256, nrot), 256, 0, (cudaStream_t)stream>>>(d, rotmats, nrot,
                                                                                (int16_t *)srcmap_out);
    VG_CHECK_LAUNCH("k_prop_srcmap");
    return VESPER_OK;
}

// launch of k_prop_score_map_s for npair pairs, or false when the query's
// features do not fit in shared memory
static bool score_map_staged(const uint4 *et, const uint4 *eq, size_t pstride, int npair, int K8, int d,
                             const int16_t *m, int nrot, float *scores, cudaStream_t st) {
    const int n = d * d * d;
    const size_t sm = ((size_t)n + 1) * K8 * sizeof(uint4);
    if (sm > (size_t)smem_limit()) return false;
    const unsigned nb = (unsigned)(npair * ((nrot + kScChunk - 1) / kScChunk));
    switch (K8) {
        case 1:
            allow_smem(k_prop_score_map_s<1>, sm);
            k_prop_score_map_s<1><<<nb, 256, sm, st>>>(et, eq, pstride, npair, d, m, nrot, scores);
            return true;
        case 2:
            allow_smem(k_prop_score_map_s<2>, sm);
            k_prop_score_map_s<2><<<nb, 256, sm, st>>>(et, eq, pstride, npair, d, m, nrot, scores);
            return true;
        case 4:
            allow_smem(k_prop_score_map_s<4>, sm);
            k_prop_score_map_s<4><<<nb, 256, sm, st>>>(et, eq, pstride, npair, d, m, nrot, scores);
            return true;
    }
    return false;
}

extern "C" int vesper_prop_score_map(const void *ET, const void *EQ, int K, int d, const void *srcmap, int nrot,
                                     float *scores, void *stream) {
    if (!ET || !EQ || !srcmap || !scores || d < 1 || nrot < 0 || K < 8 || K % 8 || K > 32)
        return fail(VESPER_ERR_INVALID, "prop_score_map: bad args (K a multiple of 8, <= 32)");
    if (((uintptr_t)ET | (uintptr_t)EQ) & 15) return fail(VESPER_ERR_INVALID, "prop_score_map: 16-byte alignment");
    if (nrot == 0) return VESPER_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const uint4 *a = (const uint4 *)ET, *b = (const uint4 *)EQ;
    const int16_t *m = (const int16_t *)srcmap;
    if (score_map_staged(a, b, 0, 1, K / 8, d, m, nrot, scores, st)) {
        VG_CHECK_LAUNCH("k_prop_score_map_s");
        return VESPER_OK;
    }
    constexpr int RPB = 4;
    const unsigned nb = (unsigned)((nrot + RPB - 1) / RPB);
    switch (K / 8) {
        case 1: k_prop_score_map<1, RPB><<<nb, 256, 0, st>>>(a, b, d, m, nrot, scores); break;
        case 2: k_prop_score_map<2, RPB><<<nb, 256, 0, st>>>(a, b, d, m, nrot, scores); break;
        case 4: k_prop_score_map<4, RPB><<<nb, 256, 0, st>>>(a, b, d, m, nrot, scores); break;
        default: return fail(VESPER_ERR_UNSUPPORTED, "prop_score_map: K = %d", K);
    }
    VG_CHECK_LAUNCH("k_prop_score_map");
    return VESPER_OK;
}

extern "C" int vesper_prop_score_map_many(const void *VM, int npair, int K, int d, const void *srcmap, int nrot,
                                          float *scores, void *stream) {
    if (!VM || !srcmap || !scores || npair < 0 || d < 1 || nrot < 0 || K < 8 || K % 8 || K > 32)
        return fail(VESPER_ERR_INVALID, "prop_score_map_many: bad args (K a multiple of 8, <= 32)");
    if ((uintptr_t)VM & 15) return fail(VESPER_ERR_INVALID, "prop_score_map_many: 16-byte alignment");
    if (npair == 0 || nrot == 0) return VESPER_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int K8 = K / 8;
    const size_t per = (size_t)d * d * d * K8;   // uint4 per map
    const uint4 *vm = (const uint4 *)VM;
    const int16_t *m = (const int16_t *)srcmap;
    if (score_map_staged(vm, vm + per, 2 * per, npair, K8, d, m, nrot, scores, st)) {
        VG_CHECK_LAUNCH("k_prop_score_map_s");
        return VESPER_OK;
    }
    for (int i = 0; i < npair; ++i) {
        const int rc = vesper_prop_score_map(vm + 2 * i * per, vm + (2 * i + 1) * per, K, d, srcmap, nrot,
                                             scores + (size_t)i * nrot, stream);
        if (rc != VESPER_OK) return rc;
    }
    return VESPER_OK;
}

extern "C" int vesper_prop_score_bwd_workspace(int K, int d, size_t *bytes) {
    if (!bytes) return fail(VESPER_ERR_INVALID, "bytes is NULL");
    *bytes = (size_t)kPropBlocks * 2 * K * d * d * d * sizeof(float);
    return VESPER_OK;
}

extern "C" int vesper_prop_score_bwd(const float *ET, const float *EQ, int K, int d, const float *rotmats, int nrot,
                                     const float *gscores, float *gET, float *gEQ, void *workspace,
                                     size_t workspace_bytes, void *stream) {
    if (!ET || !EQ || !rotmats || !gscores || !gET || !gEQ || K < 1 || d < 1 || nrot < 1)
        return fail(VESPER_ERR_INVALID, "prop_score_bwd: bad args");
    const int n = d * d * d;
    // channels per launch: the largest divisor of K whose two [kc][n] float
    // buffers fit in shared memory
    int kc = K;
    while (kc > 0 && (K % kc != 0 || (size_t)2 * kc * n * sizeof(float) > (size_t)smem_limit())) --kc;
    if (kc < 1) return fail(VESPER_ERR_UNSUPPORTED, "prop_score_bwd: d^3 too large for shared memory");
    const size_t sm = (size_t)2 * kc * n * sizeof(float);
    const int nblk = std::min(kPropBlocks, nrot);
    const int chunk = (nrot + nblk - 1) / nblk;
    size_t need = 0;
    vesper_prop_score_bwd_workspace(K, d, &need);
    if (!workspace || workspace_bytes < need) return fail(VESPER_ERR_WORKSPACE, "prop_score_bwd: workspace");
    cudaStream_t st = (cudaStream_t)stream;
    allow_smem(k_prop_score_bwd, sm);
    for (int k0 = 0; k0 < K; k0 += kc) {
        k_prop_score_bwd<<<nblk, 256, sm, st>>>(ET, EQ, K, k0, kc, d, rotmats, nrot, gscores, chunk,
                                                (float *)workspace);
        VG_CHECK_LAUNCH("k_prop_score_bwd");
    }
    const int len = K * n;
    k_sum_parts<<<(2 * len + 255) / 256, 256, 0, st>>>((const float *)workspace, nblk, len, gET, gEQ);
    VG_CHECK_LAUNCH("k_sum_parts");
    return VESPER_OK;
}

extern "C" int vesper_prop_softmax_ce(const float *scores, const float *target, int n, float tau, float *loss,
                                      float *gscores, void *stream) {
    if (!scores || !target || !loss || !gscores || n < 1 || !(tau > 0))
        return fail(VESPER_ERR_INVALID, "softmax_ce: bad args");
    k_softmax_ce<<<1, 1024, 0, (cudaStream_t)stream>>>(scores, target, n, tau, loss, gscores);
    VG_CHECK_LAUNCH("k_softmax_ce");
    return VESPER_OK;
}

extern "C" int vesper_prop_adam(float *w, float *m, float *v, const float *g, int n, float lr, float b1, float b2,
                                float eps, int step, float gscale, void *wbf16, void *stream) {
    if (!w || !m || !v || !g || n < 0 || step < 1) return fail(VESPER_ERR_INVALID, "adam: bad args");
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(w, m, v, g, n, lr, b1, b2, eps, c1, c2, gscale,
                                                              (__nv_bfloat16 *)wbf16);
    VG_CHECK_LAUNCH("k_adam");
    return VESPER_OK;
}

extern "C" int vesper_topk_subset_batch(const float *scores, int nbatch, int n, int k, int32_t *idx_out,
                                        void *stream) {
    if (!scores || !idx_out || nbatch < 1 || nbatch > 65535 || n < 1 || k < 1 || k > n)
        return fail(VESPER_ERR_INVALID, "topk_subset: bad args");
    const size_t hb = (size_t)kTkWarps * 256 * sizeof(uint32_t);
    const size_t kb = (size_t)n * sizeof(uint32_t);
    const int skeys = hb + kb <= (size_t)smem_limit() - 4096 ? 1 : 0;
    const size_t sm = hb + (skeys ? kb : 0);
    allow_smem(k_topk_subset, sm);
    k_topk_subset<<<nbatch, 1024, sm, (cudaStream_t)stream>>>(scores, n, k, idx_out, skeys);
    VG_CHECK_LAUNCH("k_topk_subset");
    return VESPER_OK;
}

extern "C" int vesper_topk_subset(const float *scores, int n, int k, int32_t *idx_out, void *stream) {
    return vesper_topk_subset_batch(scores, 1, n, k, idx_out, stream);
}
