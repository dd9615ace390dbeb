// Fused small-grid search: one CTA correlates a whole rotation in shared
// memory -- gather the rotated query, forward R2C FFT over z, y and x, product
// with the target spectra, channel sum, inverse FFT back to the d^3 score
// volume and the first-index argmax -- with no intermediate in global memory
// and one launch for every rotation of the grid (a persistent grid-stride
// loop over rotations).  Each line FFT runs whole in one thread's registers
// (rdft<D>, D <= 32), so D is a compile-time side; the sides and modes
// compiled are in the table at the end (mode V for the sides 8 to 24, the scalar
// modes O/C/P/L for 12 <= D <= 16, the grids of 128^3/64^3 pairs at s = 7).  It computes the same quantities as the three-pass
// search (vesper_search.cu) in a different FFT order, so scores agree to
// float32 rounding, not bit for bit.
//
// Shared memory per channel: one [D][2*NP][Hp] complex volume (x, y, kz),
// NP = ceil(D/2), Hp = (D/2+1)|1.  The packed z line (rows 2p, 2p+1 as real
// and imaginary parts) of plane x is stored in the space of its own output
// rows 2p and 2p+1 (D <= 2*Hp), so the z transform and its unpacking run in
// place, each line read whole into registers before it is written.
#include <algorithm>

#include "vesper_regfft.cuh"
#include "vesper_sample.cuh"

namespace vg {

constexpr int kFusedThreads = 256;

template <int D>
struct FGeom {
    static constexpr int H = D / 2 + 1;
    static constexpr int NP = (D + 1) / 2;
    static constexpr int Hp = H | 1;
    static constexpr int RS = 2 * NP * Hp;   // plane stride (one x)
    static constexpr int CS = D * RS;        // channel stride
};

template <int NCH, int D>
constexpr size_t fused_smem() {
    return 64 + 32 * sizeof(unsigned long long) + (size_t)NCH * FGeom<D>::CS * sizeof(float2);
}

struct FusedArgs {
    Src src;
    const float *rotmats;
    const float2 *T;   // conj target spectra [NCH][D][D][H] (kx, ky, kz)
    int nrot;
    int nscore;
    unsigned long long *keys;
};

// CTAs per SM the register budget is sized for, as many as the side's shared
// volume allows without spilling: 4 (64 registers) up to side 13, 3 up to
// 15, 2 for 16 to 20, 1 above and for the Laplacian mode (its float64
// stencil needs the registers).
template <int MODE, int D>
constexpr int fused_ctas() {
    return MODE == VESPER_MODE_LAPLACIAN ? 1 : D <= 13 ? 4 : D <= 15 ? 3 : D <= 20 ? 2 : 1;
}

template <int MODE, int NCH, int D>
__global__ void __launch_bounds__(kFusedThreads, fused_ctas<MODE, D>()) k_fused(const FusedArgs a) {
    using G = FGeom<D>;
    constexpr int H = G::H, NP = G::NP, Hp = G::Hp, RS = G::RS, CS = G::CS;
    extern __shared__ __align__(16) unsigned char smem[];
    float *F = (float *)smem;
    unsigned long long *red = (unsigned long long *)(smem + 64);
    float2 *V = (float2 *)(smem + 64 + 32 * sizeof(unsigned long long));
    for (int r = blockIdx.x; r < a.nrot; r += gridDim.x) {
        if (threadIdx.x < 9) F[threadIdx.x] = a.rotmats[(size_t)r * 9 + threadIdx.x];
        __syncthreads();
        float Fr[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) Fr[i] = F[i];
        // 1. gather: packed z line p of plane x <- rows (2p, 2p+1); items (x, p, z)
        for (int t = threadIdx.x; t < D * NP * D; t += blockDim.x) {
            const int z = t % D, xp = t / D, p = xp % NP, x = xp / NP, y0 = 2 * p;
            float v0[NCH], v1[NCH];
            sample_fast<MODE>(a.src, Fr, x, y0, z, v0);
            if (y0 + 1 < D) {
                sample_fast<MODE>(a.src, Fr, x, y0 + 1, z, v1);
            } else {
#pragma unroll
                for (int c = 0; c < NCH; ++c) v1[c] = 0.f;
            }
#pragma unroll
            for (int c = 0; c < NCH; ++c) V[c * CS + x * RS + 2 * p * Hp + z] = make_float2(v0[c], v1[c]);
        }
        __syncthreads();
        // 2. z FFT of each packed line, unpacked in place into rows 2p, 2p+1
        for (int t = threadIdx.x; t < NCH * D * NP; t += blockDim.x) {
            const int p = t % NP, cx = t / NP;
            float2 *line = V + cx * RS + 2 * p * Hp;
            float2 v[D];
#pragma unroll
            for (int j = 0; j < D; ++j) v[j] = line[j];
            rdft<D, false>(v);
            const bool hb = 2 * p + 1 < D;
#pragma unroll
            for (int k = 0; k < H; ++k) {
                float2 A, B;
                unpack_pair(v[k], v[(D - k) % D], A, B);
                line[k] = A;
                line[Hp + k] = hb ? B : make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
        // 3. y FFT: items (c, x, kz)
        for (int t = threadIdx.x; t < NCH * D * H; t += blockDim.x) {
            const int kz = t % H, cx = t / H;
            float2 *col = V + cx * RS + kz;
            float2 v[D];
#pragma unroll
            for (int j = 0; j < D; ++j) v[j] = col[j * Hp];
            rdft<D, false>(v);
#pragma unroll
            for (int j = 0; j < D; ++j) col[j * Hp] = v[j];
        }
        __syncthreads();
        // 4. x FFT and product with the conjugate target spectrum: items (c, ky, kz)
        for (int t = threadIdx.x; t < NCH * D * H; t += blockDim.x) {
            const int kz = t % H, cy = t / H, ky = cy % D, c = cy / D;
            float2 *col = V + c * CS + ky * Hp + kz;
            const float2 *Tc = a.T + ((size_t)c * D * D + ky) * H + kz;
            float2 v[D];
#pragma unroll
            for (int j = 0; j < D; ++j) v[j] = col[j * RS];
            rdft<D, false>(v);
#pragma unroll
            for (int k = 0; k < D; ++k) col[k * RS] = cmul(Tc[(size_t)k * D * H], v[k]);
        }
        __syncthreads();
        // 5. channel sum and inverse x FFT into channel 0: items (ky, kz)
        for (int t = threadIdx.x; t < D * H; t += blockDim.x) {
            const int kz = t % H, ky = t / H;
            float2 *col = V + ky * Hp + kz;
            float2 v[D];
#pragma unroll
            for (int k = 0; k < D; ++k) {
                float2 s = col[k * RS];
#pragma unroll
                for (int c = 1; c < NCH; ++c) s = cadd(s, col[c * CS + k * RS]);
                v[k] = s;
            }
            rdft<D, true>(v);
#pragma unroll
            for (int x = 0; x < D; ++x) col[x * RS] = v[x];
        }
        __syncthreads();
        // 6. inverse y FFT: items (x, kz)
        for (int t = threadIdx.x; t < D * H; t += blockDim.x) {
            const int kz = t % H, x = t / H;
            float2 *col = V + x * RS + kz;
            float2 v[D];
#pragma unroll
            for (int k = 0; k < D; ++k) v[k] = col[k * Hp];
            rdft<D, true>(v);
#pragma unroll
            for (int y = 0; y < D; ++y) col[y * Hp] = v[y];
        }
        __syncthreads();
        // 7. inverse z C2R of rows (2p, 2p+1) as one complex line (Hermitian
        // completion, DC and Nyquist imaginary parts dropped) and the argmax
        unsigned long long best = 0ull;
        for (int t = threadIdx.x; t < D * NP; t += blockDim.x) {
            const int p = t % NP, x = t / NP, y = 2 * p;
            const bool hb = y + 1 < D;
            const float2 *r0 = V + x * RS + y * Hp;
            const float2 *r1 = r0 + Hp;
            float2 u[D];
#pragma unroll
            for (int k = 0; k < D; ++k) {
                if (k < H) {
                    float2 A = r0[k], B = hb ? r1[k] : make_float2(0.f, 0.f);
                    if (k == 0 || 2 * k == D) {
                        A.y = 0.f;
                        B.y = 0.f;
                    }
                    u[k] = make_float2(A.x - B.y, A.y + B.x);
                } else {
                    const float2 A = r0[D - k], B = hb ? r1[D - k] : make_float2(0.f, 0.f);
                    u[k] = make_float2(A.x + B.y, B.x - A.y);
                }
            }
            rdft<D, true>(u);
            const uint32_t lin0 = (uint32_t)((x * D + y) * D);
#pragma unroll
            for (int z = 0; z < D; ++z) {
                best = max(best, make_key(u[z].x, lin0 + z));
                if (hb) best = max(best, make_key(u[z].y, lin0 + D + z));
            }
        }
        best = warp_max_u64(best);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long v = 0ull;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = max(v, red[w]);
            a.keys[(size_t)r * a.nscore] = v;
        }
        __syncthreads();
    }
}

template <int MODE, int NCH, int D>
static int launch_fused(const FusedArgs &a, cudaStream_t st) {
    constexpr size_t sm = fused_smem<NCH, D>();
    if (sm > (size_t)smem_limit()) return fail(VESPER_ERR_UNSUPPORTED, "fused search: side %d too large", D);
    allow_smem(k_fused<MODE, NCH, D>, sm);
    // resident CTAs of the whole GPU, queried once per device
    static std::mutex mu;
    static std::map<int, int> slots;
    int dev = 0;
    cudaGetDevice(&dev);
    int cap = 0;
    {
        std::lock_guard<std::mutex> g(mu);
        const auto it = slots.find(dev);
        if (it != slots.end()) cap = it->second;
    }
    if (cap == 0) {
        int per_sm = 0, nsm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused<MODE, NCH, D>, kFusedThreads, sm);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cap = std::max(per_sm, 1) * std::max(nsm, 1);
        std::lock_guard<std::mutex> g(mu);
        slots[dev] = cap;
    }
    const int grid = std::max(1, std::min(a.nrot, cap));
    k_fused<MODE, NCH, D><<<grid, kFusedThreads, sm, st>>>(a);
    VG_CHECK_LAUNCH("k_fused");
    return VESPER_OK;
}

struct FusedEntry {
    int mode, d;
    size_t smem;
    int (*run)(const FusedArgs &, cudaStream_t);
};

template <int MODE, int NCH, int D>
constexpr FusedEntry fused_entry() {
    return FusedEntry{MODE, D, fused_smem<NCH, D>(), &launch_fused<MODE, NCH, D>};
}

static const FusedEntry kFused[] = {
    fused_entry<VESPER_MODE_VEC, 3, 8>(),  fused_entry<VESPER_MODE_VEC, 3, 9>(),
    fused_entry<VESPER_MODE_VEC, 3, 11>(),
    fused_entry<VESPER_MODE_VEC, 3, 10>(), fused_entry<VESPER_MODE_VEC, 3, 12>(),
    fused_entry<VESPER_MODE_VEC, 3, 13>(), fused_entry<VESPER_MODE_VEC, 3, 14>(),
    fused_entry<VESPER_MODE_VEC, 3, 15>(), fused_entry<VESPER_MODE_VEC, 3, 16>(),
    fused_entry<VESPER_MODE_VEC, 3, 18>(), fused_entry<VESPER_MODE_VEC, 3, 20>(),
    fused_entry<VESPER_MODE_VEC, 3, 21>(), fused_entry<VESPER_MODE_VEC, 3, 22>(),
    fused_entry<VESPER_MODE_VEC, 3, 24>(),
#define VG_FUSED_SCALAR(D)                                                                              \
    fused_entry<VESPER_MODE_OVERLAP, 1, D>(), fused_entry<VESPER_MODE_CC, 1, D>(),                       \
        fused_entry<VESPER_MODE_PCC, 1, D>(), fused_entry<VESPER_MODE_LAPLACIAN, 1, D>()
    VG_FUSED_SCALAR(12), VG_FUSED_SCALAR(13), VG_FUSED_SCALAR(14), VG_FUSED_SCALAR(15), VG_FUSED_SCALAR(16),
#undef VG_FUSED_SCALAR
};

// Internal entry used by vesper_search.cu: returns 1 if a fused kernel is
// compiled for (mode, d) and fits this device (launching it and storing its
// status in *rc when rc is non-null), 0 if not.
int vesper_fused_search(int mode, int d, const Src &src, const float *rotmats, const void *spectra, int nrot,
                        int nscore, unsigned long long *keys, cudaStream_t st, int *rc) {
    for (const FusedEntry &e : kFused) {
        if (e.mode != mode || e.d != d) continue;
        if (e.smem > (size_t)smem_limit()) return 0;
        if (rc) *rc = e.run(FusedArgs{src, rotmats, (const float2 *)spectra, nrot, nscore, keys}, st);
        return 1;
    }
    return 0;
}

}  // namespace vg
