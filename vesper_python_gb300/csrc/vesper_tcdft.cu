// Search pass B on the 5th-generation tensor cores: the x-axis DFT of every
// channel, the product with the conjugate target spectrum, the sum per score
// group and the inverse x-axis DFT, as dense split-BF16 contractions with
// float32 accumulation in TMEM (grids of side 32 and 64).
//
// Pass B of the FP32 search (k_pass_b, k_rpass_b) computes, for rotation b,
// group g and column j = ky * H + kz of the (x, ky, kz) spectrum,
//   U[b][g][x][j] = sum_k e^{+2 pi i k x / d} sum_{c in g} T[c][k][j] X_c[k][j],
//   X_c[k][j] = sum_x e^{-2 pi i k x / d} S[b][c][x][j]          (T conjugated).
// Here each column j is one row of an M = 128 tile (one TMEM lane), and a
// length-d complex DFT is the real GEMM  X = A * B^T  with
//   A[row][2x] = Re S, A[row][2x + 1] = Im S          (K = 2d),
//   B[2k][2x] = cos t, B[2k][2x + 1] = sin t, B[2k + 1][2x] = -sin t,
//   B[2k + 1][2x + 1] = cos t,  t = 2 pi (k x mod d) / d  (N = 2d).
// The inverse uses the same matrix: IDFT(u) = conj(DFT(conj u)).
//
// Split-BF16: a float32 value v is held as hi = bf16(v), lo = bf16(v - hi);
// each product is hi_a hi_b + hi_a lo_b + lo_a hi_b (three MMAs into one
// float32 accumulator; lo_a lo_b, about 2^-16 of the product, is dropped).
// The operands keep about 16 significant bits, so a transform carries relative
// errors near 1e-5 of the line's magnitude, against near 1e-7 for the float32
// FFT.
//
// One CTA = one M tile of 128 rows, 256 threads: threads t and t + 128 own row
// t (TMEM lane t), each half of its elements.  A CTA runs its tiles (the
// channels of each group, then the group's inverse) as a pipeline: a TMA box
// brings a channel's S lines to shared memory, the CTA writes the split
// operand, one thread issues the 3 * K / 16 MMAs into one of two TMEM
// accumulators and commits them to an mbarrier, and while they run every
// thread reads back the previous tile (tcgen05.ld) and multiplies it by the
// target spectrum into the group sum in registers, and the next box loads.
// The results carry the split-BF16 error described above: measured against a
// float64 oracle, a few 1e-6 of the largest correlation score.  Waits are
// bounded (200 ms of global time unless the caller gives a limit); a time-out
// sets *err, and the CTA waits once more, frees its TMEM and returns
// (vesper_tc_pass_b_stall_test runs that path on purpose).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <type_traits>

#include "vesper_common.cuh"
#define VG_PASS_TYPES_ONLY
#include "vesper_passes.cuh"
#include "vesper_tcdft.cuh"

namespace vg {

constexpr int kTcRows = 128;                     // M: columns j per CTA
constexpr int kTcThreads = 256;                  // two threads per row: each takes half of its elements

template <int D>
struct TcGeom {
    static constexpr int K = 2 * D;                                  // = N
    static constexpr uint32_t SBO = (uint32_t)(K / 8) * 128;         // 8-row group stride
    static constexpr size_t B_BYTES = (size_t)K * K * 2;             // one split of the DFT matrix
    static constexpr size_t A_BYTES = (size_t)kTcRows * K * 2;       // one split of the tile
    static constexpr uint32_t TMEM_COLS = 2 * K;                     // two accumulator buffers (128 or 256)
    static constexpr size_t STAGE_BYTES = (size_t)D * kTcRows * 8;   // one TMA box: D x 128 complex
    // + 64 bytes of barriers and TMEM slot, + 4 KB that no operand uses: every
    // address an MMA could form from these descriptors stays inside the block
    static constexpr size_t SMEM = 2 * B_BYTES + 2 * A_BYTES + STAGE_BYTES + 64 + 4096;
};

// The real-form DFT matrix, hi then lo, in the K-major core-matrix layout,
// written into shared memory by every CTA (no table in device memory).  Entry
// (n, k) is c, s, -s or c of the angle 2 pi m / D, m = (n/2)(k/2) mod D, so the
// D cosines and sines are computed once (float64 sincospi, then split into
// bf16 hi + lo of the float64 value) and the K^2 entries looked up.
template <int D>
__device__ void tc_build_table(unsigned char *bh, unsigned char *bl, __nv_bfloat16 (*tw)[D], int tid, int nthr) {
    constexpr int K = TcGeom<D>::K;
    for (int m = tid; m < D; m += nthr) {
        double s, c;
        sincospi(2.0 * (double)m / (double)D, &s, &c);
        const double v[3] = {c, s, -s};
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            const __nv_bfloat16 hi = __double2bfloat16(v[e]);
            tw[2 * e][m] = hi;
            tw[2 * e + 1][m] = __double2bfloat16(v[e] - (double)__bfloat162float(hi));
        }
    }
    __syncthreads();
    for (int i = tid; i < K * K; i += nthr) {
        const int n = i / K, k = i % K;
        const int m = ((n >> 1) * (k >> 1)) % D;
        // c, s for even rows; -s, c for odd rows
        const int e = (n & 1) == 0 ? ((k & 1) == 0 ? 0 : 1) : ((k & 1) == 0 ? 2 : 0);
        const uint32_t off = tc::kmajor_off(n, k, K);
        *(__nv_bfloat16 *)(bh + off) = tw[2 * e][m];
        *(__nv_bfloat16 *)(bl + off) = tw[2 * e + 1][m];
    }
}

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// (re, im) split into packed hi and lo bf16 pairs (re in the low half)
__device__ __forceinline__ void split_pair(float re, float im, uint32_t &h, uint32_t &l) {
    const __nv_bfloat16 hr = __float2bfloat16_rn(re), hi_ = __float2bfloat16_rn(im);
    const __nv_bfloat16 lr = __float2bfloat16_rn(re - __bfloat162float(hr));
    const __nv_bfloat16 li = __float2bfloat16_rn(im - __bfloat162float(hi_));
    h = pack_bf16(hr, hi_);
    l = pack_bf16(lr, li);
}

// elements x0 .. x0 + 3 (x0 a multiple of 4) of this thread's row into the hi
// and lo tiles: one 16-byte chunk of a core-matrix row each, so eight rows of a
// warp fill one 128-byte shared-memory wavefront
__device__ __forceinline__ void put_split4(unsigned char *ah, unsigned char *al, int row, int x0, int K, float2 v0,
                                           float2 v1, float2 v2, float2 v3) {
    uint4 h, l;
    split_pair(v0.x, v0.y, h.x, l.x);
    split_pair(v1.x, v1.y, h.y, l.y);
    split_pair(v2.x, v2.y, h.z, l.z);
    split_pair(v3.x, v3.y, h.w, l.w);
    const uint32_t off = tc::kmajor_off(row, 2 * x0, K);
    *(uint4 *)(ah + off) = h;
    *(uint4 *)(al + off) = l;
}

// MMAs of one tile: D = A * B^T over K, split-BF16 (hi hi + hi lo + lo hi)
template <int D>
__device__ __forceinline__ void issue_split_mma(uint32_t tmem, const unsigned char *ah, const unsigned char *al,
                                                const unsigned char *bh, const unsigned char *bl, uint64_t *mbar) {
    using G = TcGeom<D>;
    constexpr uint32_t idesc = tc::idesc_bf16(kTcRows, G::K);
    const uint32_t sah = tc::smem_addr(ah), sal = tc::smem_addr(al);
    const uint32_t sbh = tc::smem_addr(bh), sbl = tc::smem_addr(bl);
#pragma unroll
    for (int s = 0; s < G::K / 16; ++s) {
        const uint32_t o = (uint32_t)s * 2 * tc::kLBO;
        tc::mma_bf16(tmem, tc::smem_desc(sah + o, tc::kLBO, G::SBO), tc::smem_desc(sbh + o, tc::kLBO, G::SBO), idesc,
                     s > 0 ? 1u : 0u);
        tc::mma_bf16(tmem, tc::smem_desc(sah + o, tc::kLBO, G::SBO), tc::smem_desc(sbl + o, tc::kLBO, G::SBO), idesc,
                     1u);
        tc::mma_bf16(tmem, tc::smem_desc(sal + o, tc::kLBO, G::SBO), tc::smem_desc(sbh + o, tc::kLBO, G::SBO), idesc,
                     1u);
    }
    tc::mma_commit(mbar);
}

template <int D>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tcb(const PassB2 a, const __grid_constant__ CUtensorMap tmS, int *err, int stall,
          uint64_t limit_ns) {
    using G = TcGeom<D>;
    constexpr int K = G::K;
    constexpr int H = D / 2 + 1;
    constexpr int dH = D * H;
    constexpr int DH2 = D / 2;                     // elements of a row per thread
    extern __shared__ __align__(16) unsigned char smem[];   // 16-byte alignment suffices without swizzle
    unsigned char *bh = smem, *bl = smem + G::B_BYTES;
    unsigned char *ah = smem + 2 * G::B_BYTES, *al = ah + G::A_BYTES;
    float2 *stage = (float2 *)(al + G::A_BYTES);            // [D][128]: one TMA box of S
    uint64_t *mbar_mma = (uint64_t *)((unsigned char *)stage + G::STAGE_BYTES);
    uint64_t *mbar_tma = mbar_mma + 1;
    uint32_t *tslot = (uint32_t *)(mbar_mma + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = tid & (kTcRows - 1), half = tid >> 7;   // warps w and w + 4 share TMEM lanes 32 (w % 4) ..
    const int j0 = blockIdx.x * kTcRows, j = j0 + row;
    const int b = blockIdx.y;
    const bool live = j < dH;

    // the DFT matrix (hi, lo) into shared memory
    {
        __shared__ __nv_bfloat16 tw[6][D];
        tc_build_table<D>(bh, bl, tw, tid, kTcThreads);
    }
    if (tid == 0) {
        tc::mbar_init(mbar_mma, 1);
        tc::mbar_init(mbar_tma, 1);
    }
    if (warp == 0) tc::tmem_alloc(tslot, G::TMEM_COLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);   // this warp's 32 lanes
    uint32_t pm = 0, pt = 0;   // phases of the MMA and TMA barriers
    bool ok = true;
    if (stall) {   // failure self-test: a wait that nothing completes (no copy was issued)
        const bool got = tc::mbar_wait(mbar_tma, pt, limit_ns);
        pt ^= 1u;
        ok = __syncthreads_and(got ? 1 : 0) != 0;
    }

    // Tiles of one CTA, in order: the channels of group 0, its inverse, then
    // (two groups) the channels of group 1 and its inverse.  Tile t's MMAs
    // accumulate in TMEM buffer t & 1.
    const int n0 = a.ngrp == 1 ? a.nch : a.split;
    const int ntiles = a.nch + a.ngrp;
    auto is_inv = [&](int t) { return t == n0 || t == a.nch + 1; };
    auto chan = [&](int t) { return t < n0 ? t : t - 1; };

    auto load_s = [&](int t) {   // one thread: the S box of channel tile t into the stage
        tc::fence_smem_async();
        tc::mbar_expect_tx(mbar_tma, (uint32_t)G::STAGE_BYTES);
        tc::tma_load_3d(stage, &tmS, j0, 0, b * a.nch + chan(t), mbar_tma);
    };

    float ur[DH2], ui[DH2];   // group sum at frequencies half * D/2 + [0, D/2) of this row
#pragma unroll
    for (int x = 0; x < DH2; ++x) ur[x] = ui[x] = 0.f;
    float2 *U = a.U + (size_t)b * a.ngrp * D * dH;

    // read-back of tile t (its MMAs have completed): a channel's spectrum times
    // the conjugate target into the group sum, or an inverse into U
    auto epilogue = [&](int t) {
        const uint32_t tb = trow + (uint32_t)((t & 1) * K);
        if (!is_inv(t)) {
            // this thread's D/2 target values first: one L2 round trip for all
            const float2 *tc_ = a.T + (size_t)chan(t) * D * dH + (size_t)half * DH2 * dH + j;
            float2 tv[DH2];
#pragma unroll
            for (int kq = 0; kq < DH2; ++kq) tv[kq] = live ? __ldg(tc_ + (size_t)kq * dH) : make_float2(0.f, 0.f);
#pragma unroll
            for (int qq = 0; qq < K / 32; ++qq) {
                const int q = half * (K / 32) + qq;
                float v[16];
                tc::tmem_ld16(tb + (uint32_t)(q * 16), v);
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int kq = qq * 8 + e;
                    ur[kq] = fmaf(tv[kq].x, v[2 * e], fmaf(-tv[kq].y, v[2 * e + 1], ur[kq]));
                    ui[kq] = fmaf(tv[kq].x, v[2 * e + 1], fmaf(tv[kq].y, v[2 * e], ui[kq]));
                }
            }
        } else {
            float2 *ug = U + (size_t)(t == n0 ? 0 : 1) * D * dH + j;
#pragma unroll
            for (int qq = 0; qq < K / 32; ++qq) {
                const int q = half * (K / 32) + qq;
                float v[16];
                tc::tmem_ld16(tb + (uint32_t)(q * 16), v);
                if (live) {
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        ug[(size_t)(q * 8 + e) * dH] = make_float2(v[2 * e], -v[2 * e + 1]);
                }
            }
        }
        tc::fence_before_sync();
    };

    if (tid == 0 && ok) load_s(0);
    int pending = -1;   // tile whose read-back is still to do
    for (int t = 0; t < ntiles && ok; ++t) {
        if (!is_inv(t)) {
            const bool got = tc::mbar_wait(mbar_tma, pt, limit_ns);
            pt ^= 1u;
            ok = __syncthreads_and(got ? 1 : 0) != 0;
            if (!ok) break;
#pragma unroll 2
            for (int xq = 0; xq < DH2; xq += 4) {
                const int x = half * DH2 + xq;
                put_split4(ah, al, row, x, K, stage[x * kTcRows + row], stage[(x + 1) * kTcRows + row],
                           stage[(x + 2) * kTcRows + row], stage[(x + 3) * kTcRows + row]);
            }
        } else {
            if (pending >= 0) {   // the group sum needs the last channel's read-back
                epilogue(pending);
                pending = -1;
            }
            // inverse DFT of the group sum: conj(DFT(conj u))
#pragma unroll
            for (int kq = 0; kq < DH2; kq += 4) {
                put_split4(ah, al, row, half * DH2 + kq, K, make_float2(ur[kq], -ui[kq]),
                           make_float2(ur[kq + 1], -ui[kq + 1]), make_float2(ur[kq + 2], -ui[kq + 2]),
                           make_float2(ur[kq + 3], -ui[kq + 3]));
            }
#pragma unroll
            for (int kq = 0; kq < DH2; ++kq) ur[kq] = ui[kq] = 0.f;
        }
        tc::fence_smem_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_split_mma<D>(tmem + (uint32_t)((t & 1) * K), ah, al, bh, bl, mbar_mma);
            if (t + 1 < ntiles && !is_inv(t + 1)) load_s(t + 1);   // the stage was read above
        }
        if (pending >= 0) epilogue(pending);   // overlaps this tile's MMAs
        pending = t;
        const bool got = tc::mbar_wait(mbar_mma, pm, limit_ns);
        pm ^= 1u;
        tc::fence_after_sync();
        ok = __syncthreads_and(got ? 1 : 0) != 0;   // MMAs done: the operand tile is free
    }
    if (ok && pending >= 0) epilogue(pending);
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // work of the timed-out step may still run: wait for both barriers
        // once more (bounded) before the TMEM goes back
        tc::mbar_wait(mbar_mma, pm ^ 1u, limit_ns);
        tc::mbar_wait(mbar_tma, pt ^ 1u, limit_ns);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, G::TMEM_COLS);
}

// ---- host ---------------------------------------------------------------------

bool tc_pass_b_supported(int d) { return d == 32 || d == 64; }

// rotations per full wave of pass-B CTAs on this device (column tiles of 128
// per rotation; CTAs resident per SM by shared memory), at least 1
int tc_pass_b_wave(int d) {
    if (!tc_pass_b_supported(d)) return 1;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) return 1;
    const size_t sm = d == 32 ? TcGeom<32>::SMEM : TcGeom<64>::SMEM;
    const int per_sm = std::max(1, (int)((size_t)smem_limit() / (sm + 1024)));
    const int dH = d * (d / 2 + 1);
    const int tiles = (dH + kTcRows - 1) / kTcRows;
    return std::max(1, nsm * per_sm / tiles);
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// [planes][D][dH] complex64 (8-byte elements) in boxes of 128 x D x 1; columns
// past dH read as zeros
static bool box_map(CUtensorMap *m, const void *base, int D, int dH, int planes) {
    const auto fn = encode_tiled();
    if (!fn || ((uintptr_t)base & 15u)) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)dH, (cuuint64_t)D, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)dH * 8, (cuuint64_t)D * dH * 8};
    const cuuint32_t box[3] = {(cuuint32_t)kTcRows, (cuuint32_t)D, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void *>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// pass B of nb rotations on the tensor cores; err: device int, set to 1 when
// a wait timed out (left untouched otherwise)
int tc_pass_b(const PassB2 &a, int nb, int *err, cudaStream_t st, int stall, uint64_t limit_ns) {
    if (nb < 1 || nb > 65535 || !err) return fail(VESPER_ERR_INVALID, "tc pass B: bad batch");
    auto run = [&](auto dc) -> int {
        constexpr int D = decltype(dc)::value;
        constexpr size_t sm = TcGeom<D>::SMEM;
        allow_smem(k_tcb<D>, sm);
        const int dH = D * (D / 2 + 1);
        CUtensorMap tmS;
        if ((dH * 8) % 16 || !box_map(&tmS, a.S, D, dH, nb * a.nch))
            return fail(VESPER_ERR_CUDA, "tc pass B: tensor map (driver entry point or alignment)");
        k_tcb<D><<<dim3((dH + kTcRows - 1) / kTcRows, nb), kTcThreads, sm, st>>>(a, tmS, err, stall, limit_ns);
        VG_CHECK_LAUNCH("k_tcb");
        return VESPER_OK;
    };
    if (a.d == 32) return run(std::integral_constant<int, 32>{});
    if (a.d == 64) return run(std::integral_constant<int, 64>{});
    return fail(VESPER_ERR_UNSUPPORTED, "tc pass B: side %d (32 and 64 only)", a.d);
}

}  // namespace vg

using namespace vg;

extern "C" int vesper_tc_pass_b_stall_test(const void *S, const void *T, void *U, int d, int nch, int ngrp,
                                           int split, int limit_ms, int *err, void *stream) {
    if (!S || !T || !U || !err || nch < 1 || ngrp < 1 || ngrp > 2 || split < 1 || split > nch || limit_ms < 1 ||
        limit_ms > 1000)
        return fail(VESPER_ERR_INVALID, "vesper_tc_pass_b_stall_test: bad args");
    if (ngrp == 2 && split >= nch) return fail(VESPER_ERR_INVALID, "vesper_tc_pass_b_stall_test: empty second group");
    PassB2 a{};
    a.S = (const float2 *)S;
    a.T = (const float2 *)T;
    a.U = (float2 *)U;
    a.d = d;
    a.nch = nch;
    a.ngrp = ngrp;
    a.split = ngrp == 1 ? nch : split;
    return tc_pass_b(a, 1, err, (cudaStream_t)stream, 1, (uint64_t)limit_ms * 1000000ull);
}

extern "C" int vesper_tc_pass_b(const void *S, const void *T, void *U, int d, int nch, int ngrp, int split,
                                int nbatch, int *err, void *stream) {
    if (!S || !T || !U || !err || nch < 1 || ngrp < 1 || ngrp > 2 || split < 1 || split > nch)
        return fail(VESPER_ERR_INVALID, "vesper_tc_pass_b: bad args");
    if (ngrp == 2 && split >= nch) return fail(VESPER_ERR_INVALID, "vesper_tc_pass_b: empty second group");
    PassB2 a{};
    a.S = (const float2 *)S;
    a.T = (const float2 *)T;
    a.U = (float2 *)U;
    a.d = d;
    a.nch = nch;
    a.ngrp = ngrp;
    a.split = ngrp == 1 ? nch : split;
    return tc_pass_b(a, nbatch, err, (cudaStream_t)stream);
}
