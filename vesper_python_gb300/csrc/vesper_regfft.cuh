// Register-resident DFTs and the two-step line FFT.
//
// rdft<N, INV>(a): an N-point DFT of a[0..N) held in registers, natural order
// in and out, N <= 32 with prime factors 2, 3, 5, 7, 11, 13.  N with two
// coprime factors N = P * M (P the power of N's smallest prime) is split by
// the prime-factor (Good-Thomas) mapping: input n = (M n1 + P n2) mod N, P-point
// DFTs over n1, M-point DFTs over n2, output k = the residue pair (k mod P,
// k mod M) -- no twiddle multiplications.  A prime power N is split N = P * M
// (P the first radix) decimation-in-time: M-point DFTs of the P interleaved
// sub-sequences, twiddles W_N^{r k} from a constant table, then P-point DFTs.
// All indices are compile-time, so nothing spills to memory and the index
// maps are register renamings.
//
// Two-step line FFT of length n = N1 * N2 (both <= 32):
//   X[k1 + N1 k2] = sum_j2 W_N2^{j2 k2} W_n^{j2 k1} sum_j1 x[j2 + N2 j1] W_N1^{j1 k1}
// step 1 (per j2): an N1-point DFT of the stride-N2 sub-sequence, times
// W_n^{j2 k1}; step 2 (per k1): an N2-point DFT.  The inverse runs the same two
// steps in the opposite order with conjugate twiddles.  Each step is one
// shared-memory round trip, against one per radix stage in vesper_fft.cuh.
#pragma once

#include "vesper_fft.cuh"
#include "vesper_twiddles.cuh"

namespace vg {

template <int N> __host__ __device__ constexpr int first_radix() {
    return (N % 4 == 0 && N > 4) ? 4 : N % 2 == 0 ? 2 : N % 3 == 0 ? 3 : N % 5 == 0 ? 5 : N % 7 == 0 ? 7
           : N % 11 == 0 ? 11 : 13;
}
template <int N> __host__ __device__ constexpr bool leaf_dft() {
    return N == 2 || N == 3 || N == 4 || N == 5 || N == 7 || N == 11 || N == 13;
}

// The P of a coprime split N = P * M when N has two prime factors, else 0: the
// power of N's smallest prime (LF false) or N's largest prime power (LF true).
// Both give the same DFT; the order changes the registers the compiler keeps
// live (measured: largest first is faster in pass A at sides 28 and 30,
// smallest first in passes B and C).
template <int N, bool LF = false> __host__ __device__ constexpr int pfa_first() {
    int best = 0;
    const int ps[6] = {2, 3, 5, 7, 11, 13};
    for (int i = 0; i < 6; ++i) {
        if (N % ps[i]) continue;
        int P = 1;
        while (N % (P * ps[i]) == 0) P *= ps[i];
        if (P == N) return 0;
        if (!LF) return P;
        if (P > best) best = P;
    }
    return best;
}
// x with (a x) mod b == 1, for coprime a, b (b > 1)
__host__ __device__ constexpr int inv_mod(int a, int b) {
    for (int x = 1; x < b; ++x)
        if ((a * x) % b == 1) return x;
    return 0;
}

template <int N, bool INV, bool LF = false>
__device__ __forceinline__ void rdft(float2 *a) {
    if constexpr (N == 1) {
        return;
    } else if constexpr (leaf_dft<N>()) {
        Dft<N, INV, float2>::run(a);
    } else if constexpr (pfa_first<N, LF>() != 0) {
        constexpr int P = pfa_first<N, LF>(), M = N / P;
        constexpr int cp = M * inv_mod(M % P, P), cm = P * inv_mod(P % M, M);   // CRT weights of k1, k2
        float2 b[M][P];
#pragma unroll
        for (int n2 = 0; n2 < M; ++n2)
#pragma unroll
            for (int n1 = 0; n1 < P; ++n1) b[n2][n1] = a[(M * n1 + P * n2) % N];
#pragma unroll
        for (int n2 = 0; n2 < M; ++n2) rdft<P, INV, LF>(b[n2]);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
            float2 c[M];
#pragma unroll
            for (int n2 = 0; n2 < M; ++n2) c[n2] = b[n2][k1];
            rdft<M, INV, LF>(c);
#pragma unroll
            for (int k2 = 0; k2 < M; ++k2) a[(k1 * cp + k2 * cm) % N] = c[k2];
        }
    } else {
        constexpr int P = first_radix<N>(), M = N / P;
        float2 b[P][M];
#pragma unroll
        for (int r = 0; r < P; ++r)
#pragma unroll
            for (int m = 0; m < M; ++m) b[r][m] = a[r + P * m];
#pragma unroll
        for (int r = 0; r < P; ++r) rdft<M, INV, LF>(b[r]);
#pragma unroll
        for (int r = 1; r < P; ++r)
#pragma unroll
            for (int k = 1; k < M; ++k) {
                const float2 w = c_rtw[rtw_off<N>() + r * k];
                b[r][k] = INV ? cmulc(b[r][k], w) : cmul(b[r][k], w);
            }
#pragma unroll
        for (int k = 0; k < M; ++k) {
            float2 c[P];
#pragma unroll
            for (int r = 0; r < P; ++r) c[r] = b[r][k];
            Dft<P, INV, float2>::run(c);
#pragma unroll
            for (int q = 0; q < P; ++q) a[k + M * q] = c[q];
        }
    }
}

// W_n^m, m < n, in shared memory (forward sign); computed per CTA.
__device__ __forceinline__ void twiddles_n(int n, float2 *tw) {
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
        float s, c;
        sincospif(-2.0f * (float)m / (float)n, &s, &c);
        tw[m] = make_float2(c, s);
    }
}

}  // namespace vg
