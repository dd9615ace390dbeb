// Mixed-radix in-place FFT on batches of lines held in shared memory.
//
// Lengths are the grid sides the reference produces with pyFFTW's
// next_fast_len (VESPER_1_prob_new.py:97): 2^a 3^b 5^c 7^d 11^e 13^f, e+f<=1.
// Each transform is a decimation-in-time Cooley-Tukey FFT done in place:
// the caller writes element i of a line at position fft_pos(i) (mixed-radix
// digit reversal), the stages run from the innermost radix outwards, and the
// output comes out in natural order.  Stage s with radix p combines p
// sub-transforms of length L into one of length L*p:
//   X[j + L q] = sum_r W_{Lp}^{r j} W_p^{r q} Y_r[j],  Y_r at [r L, (r+1) L)
// Forward uses W_n = exp(-2 pi i / n) (FFTW_FORWARD), inverse exp(+2 pi i / n)
// without normalisation (FFTW_BACKWARD).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vg {

constexpr int kMaxStages = 12;

struct FftPlan {
    int n;
    int nst;
    int rad[kMaxStages];   // radix of stage s, stage 0 innermost
    int st0[kMaxStages];   // start of stage s in the butterfly tables (sum of n / rad over earlier stages)
    int ntab;              // total butterfly-table entries
};

// ---- complex helpers (float2 / double2) -----------------------------------
template <typename C> struct Real;
template <> struct Real<float2> { using T = float; };
template <> struct Real<double2> { using T = double; };

__device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {  // a * conj(b)
    return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C, typename R> __device__ __forceinline__ C cscale(C a, R s) { return mk(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C> __device__ __forceinline__ C rot90(C a) {
    return INV ? mk(-a.y, a.x) : mk(a.y, -a.x);
}

// ---- plan helpers ----------------------------------------------------------
__device__ __forceinline__ int fft_pos(int i, const FftPlan &P) {
    int pos = 0, size = P.n;
    for (int s = P.nst - 1; s >= 0; --s) {
        const int p = P.rad[s];
        size /= p;
        pos += (i % p) * size;
        i /= p;
    }
    return pos;
}

// Twiddle table: stage s occupies [L_s - 1, L_{s+1} - 1); entry (j, r) at
// (L_s - 1) + j (p_s - 1) + (r - 1) holds exp(-2 pi i r j / L_{s+1}).
__device__ __forceinline__ void tw_value(int idx, const FftPlan &P, float2 &w) {
    int L = 1;
    for (int s = 0; s < P.nst; ++s) {
        const int p = P.rad[s];
        const int Ln = L * p;
        if (idx < Ln - 1) {
            const int local = idx - (L - 1);
            const int j = local / (p - 1);
            const int r = local % (p - 1) + 1;
            float sv, cv;
            sincospif(-2.0f * (float)(r * j) / (float)Ln, &sv, &cv);
            w = make_float2(cv, sv);
            return;
        }
        L = Ln;
    }
    w = make_float2(1.f, 0.f);
}
__device__ __forceinline__ void tw_value(int idx, const FftPlan &P, double2 &w) {
    int L = 1;
    for (int s = 0; s < P.nst; ++s) {
        const int p = P.rad[s];
        const int Ln = L * p;
        if (idx < Ln - 1) {
            const int local = idx - (L - 1);
            const int j = local / (p - 1);
            const int r = local % (p - 1) + 1;
            double sv, cv;
            sincospi(-2.0 * (double)(r * j) / (double)Ln, &sv, &cv);
            w = make_double2(cv, sv);
            return;
        }
        L = Ln;
    }
    w = make_double2(1.0, 0.0);
}

// Fill rev[n] (digit-reversed positions) and tw[n-1]; caller syncs.
template <typename C>
__device__ void fft_tables(const FftPlan &P, short *rev, C *tw) {
    for (int i = threadIdx.x; i < P.n; i += blockDim.x) rev[i] = (short)fft_pos(i, P);
    for (int i = threadIdx.x; i < P.n - 1; i += blockDim.x) tw_value(i, P, tw[i]);
}

// ---- small DFT butterflies --------------------------------------------------
// constants cos/sin(2 pi k / p), k = 1 .. (p-1)/2
struct K7 {
    __host__ __device__ static constexpr double c(int k) {
        return k == 1 ? 0.6234898018587336 : k == 2 ? -0.22252093395631434 : -0.900968867902419;
    }
    __host__ __device__ static constexpr double s(int k) {
        return k == 1 ? 0.7818314824680298 : k == 2 ? 0.9749279121818236 : 0.43388373911755823;
    }
};
struct K11 {
    __host__ __device__ static constexpr double c(int k) {
        return k == 1 ? 0.8412535328311812 : k == 2 ? 0.41541501300188644 : k == 3 ? -0.142314838273285
             : k == 4 ? -0.654860733945285 : -0.9594929736144974;
    }
    __host__ __device__ static constexpr double s(int k) {
        return k == 1 ? 0.5406408174555976 : k == 2 ? 0.9096319953545183 : k == 3 ? 0.9898214418809328
             : k == 4 ? 0.7557495743542583 : 0.28173255684142967;
    }
};
struct K13 {
    __host__ __device__ static constexpr double c(int k) {
        return k == 1 ? 0.8854560256532099 : k == 2 ? 0.5680647467311559 : k == 3 ? 0.120536680255323
             : k == 4 ? -0.35460488704253545 : k == 5 ? -0.7485107481711012 : -0.970941817426052;
    }
    __host__ __device__ static constexpr double s(int k) {
        return k == 1 ? 0.4647231720437685 : k == 2 ? 0.8229838658936564 : k == 3 ? 0.992708874098054
             : k == 4 ? 0.9350162426854148 : k == 5 ? 0.6631226582407952 : 0.23931566428755768;
    }
};

template <int P, bool INV, typename C> struct Dft;

template <bool INV, typename C> struct Dft<2, INV, C> {
    __device__ static void run(C *a) {
        const C t = a[1];
        a[1] = csub(a[0], t);
        a[0] = cadd(a[0], t);
    }
};
template <bool INV, typename C> struct Dft<3, INV, C> {
    __device__ static void run(C *a) {
        using R = typename Real<C>::T;
        const R c = (R)-0.5, s = (R)0.8660254037844386;
        const C t1 = cadd(a[1], a[2]);
        const C t2 = csub(a[0], cscale(t1, (R)0.5));
        const C t3 = cscale(rot90<INV>(csub(a[1], a[2])), s);
        (void)c;
        a[0] = cadd(a[0], t1);
        a[1] = cadd(t2, t3);
        a[2] = csub(t2, t3);
    }
};
template <bool INV, typename C> struct Dft<4, INV, C> {
    __device__ static void run(C *a) {
        const C s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
        const C s13 = cadd(a[1], a[3]), d13 = rot90<INV>(csub(a[1], a[3]));
        a[0] = cadd(s02, s13);
        a[2] = csub(s02, s13);
        a[1] = cadd(d02, d13);
        a[3] = csub(d02, d13);
    }
};
template <bool INV, typename C> struct Dft<5, INV, C> {
    __device__ static void run(C *a) {
        using R = typename Real<C>::T;
        const R c1 = (R)0.30901699437494745, c2 = (R)-0.8090169943749473;
        const R s1 = (R)0.9510565162951535, s2 = (R)0.5877852522924732;
        const C s14 = cadd(a[1], a[4]), d14 = rot90<INV>(csub(a[1], a[4]));
        const C s23 = cadd(a[2], a[3]), d23 = rot90<INV>(csub(a[2], a[3]));
        const C a0 = a[0];
        const C r1 = cadd(a0, cadd(cscale(s14, c1), cscale(s23, c2)));
        const C r2 = cadd(a0, cadd(cscale(s14, c2), cscale(s23, c1)));
        const C i1 = cadd(cscale(d14, s1), cscale(d23, s2));
        const C i2 = csub(cscale(d14, s2), cscale(d23, s1));
        a[0] = cadd(a0, cadd(s14, s23));
        a[1] = cadd(r1, i1);
        a[4] = csub(r1, i1);
        a[2] = cadd(r2, i2);
        a[3] = csub(r2, i2);
    }
};
// generic odd prime p: y_m = a0 + sum_k (a_k + a_{p-k}) cos(2 pi k m / p) -/+ i (a_k - a_{p-k}) sin(...)
template <int P, typename KT, bool INV, typename C> struct DftOdd {
    __device__ static void run(C *a) {
        using R = typename Real<C>::T;
        constexpr int H = (P - 1) / 2;
        C sp[H], dm[H];
#pragma unroll
        for (int k = 1; k <= H; ++k) {
            sp[k - 1] = cadd(a[k], a[P - k]);
            dm[k - 1] = rot90<INV>(csub(a[k], a[P - k]));
        }
        const C a0 = a[0];
        C y0 = a0;
#pragma unroll
        for (int k = 0; k < H; ++k) y0 = cadd(y0, sp[k]);
#pragma unroll
        for (int m = 1; m <= H; ++m) {
            C re = a0, im = mk((R)0, (R)0);
#pragma unroll
            for (int k = 1; k <= H; ++k) {
                const int km = (k * m) % P;
                const int idx = km <= H ? km : P - km;
                const R cv = (R)KT::c(idx);
                const R sv = km <= H ? (R)KT::s(idx) : -(R)KT::s(idx);
                re = cadd(re, cscale(sp[k - 1], cv));
                im = cadd(im, cscale(dm[k - 1], sv));
            }
            a[m] = cadd(re, im);
            a[P - m] = csub(re, im);
        }
        a[0] = y0;
    }
};
template <bool INV, typename C> struct Dft<7, INV, C> : DftOdd<7, K7, INV, C> {};
template <bool INV, typename C> struct Dft<11, INV, C> : DftOdd<11, K11, INV, C> {};
template <bool INV, typename C> struct Dft<13, INV, C> : DftOdd<13, K13, INV, C> {};

template <int P, bool INV, typename C>
__device__ __forceinline__ void butterfly(C *base, int estride, const C *tw) {
    C a[P];
    a[0] = base[0];
#pragma unroll
    for (int r = 1; r < P; ++r) {
        const C v = base[r * estride];
        a[r] = INV ? cmulc(v, tw[r - 1]) : cmul(v, tw[r - 1]);
    }
    Dft<P, INV, C>::run(a);
#pragma unroll
    for (int r = 0; r < P; ++r) base[r * estride] = a[r];
}

// Line geometry: line l starts at (l / nin) * so + (l % nin) * si; element e of
// a line sits at base + e * es.
struct Lines {
    int count, nin, so, si, es;
    __device__ __forceinline__ int base(int l) const { return (l / nin) * so + (l % nin) * si; }
};

// Run every stage of an n-point FFT over ``g.count`` lines of ``buf``.  With
// lines_fast, consecutive threads take consecutive lines (use when lines are
// adjacent in memory); otherwise consecutive butterflies of one line.
template <bool INV, typename C>
__device__ void fft_run(C *buf, const Lines &g, const FftPlan &P, const C *tw, bool lines_fast) {
    int L = 1;
    for (int s = 0; s < P.nst; ++s) {
        const int p = P.rad[s];
        const int Ln = L * p;
        const int nbf = P.n / p;
        const int total = g.count * nbf;
        const C *tws = tw + (L - 1);
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            int line, bf;
            if (lines_fast) {
                line = t % g.count;
                bf = t / g.count;
            } else {
                bf = t % nbf;
                line = t / nbf;
            }
            const int j = bf % L;
            const int blk = bf / L;
            C *b = buf + g.base(line) + (blk * Ln + j) * g.es;
            const int es = L * g.es;
            const C *w = tws + j * (p - 1);
            switch (p) {
                case 2: butterfly<2, INV>(b, es, w); break;
                case 3: butterfly<3, INV>(b, es, w); break;
                case 4: butterfly<4, INV>(b, es, w); break;
                case 5: butterfly<5, INV>(b, es, w); break;
                case 7: butterfly<7, INV>(b, es, w); break;
                case 11: butterfly<11, INV>(b, es, w); break;
                case 13: butterfly<13, INV>(b, es, w); break;
                default: break;
            }
        }
        __syncthreads();
        L = Ln;
    }
}

// ---------------------------------------------------------------------------
// Division-free line FFTs.  Per CTA, stage tables give for butterfly bf of
// stage s its element offset inside the line (blk * L * p + j) and the offset
// of its twiddles in tw[]; each thread owns one line (two when there are more
// lines than threads) and a fixed stride through that line's butterflies, so
// the inner loops carry no integer division.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fft_stage_tables(const FftPlan &P, short *off, short *two) {
    int L = 1;
    for (int s = 0; s < P.nst; ++s) {
        const int p = P.rad[s], nbf = P.n / p;
        for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
            const int j = bf % L, blk = bf / L;
            off[P.st0[s] + bf] = (short)(blk * L * p + j);
            two[P.st0[s] + bf] = (short)((L - 1) + j * (p - 1));
        }
        L *= p;
    }
}

struct LineSlot {
    int base0, base1;   // element offsets of the thread's lines
    int sub0, nsub;     // first butterfly and butterfly stride inside line 0
    bool a0, a1;
};

// Line l starts at (l / nin) * so + (l % nin) * si.  Supports count <= 2 * blockDim.
__device__ __forceinline__ LineSlot line_slot(int count, int nin, int so, int si) {
    LineSlot s;
    const int T = blockDim.x, t = threadIdx.x;
    if (count >= T) {
        s.nsub = 1;
        s.sub0 = 0;
        s.a0 = true;
        s.base0 = (t / nin) * so + (t % nin) * si;
        const int l1 = t + T;
        s.a1 = l1 < count;
        s.base1 = s.a1 ? (l1 / nin) * so + (l1 % nin) * si : 0;
    } else {
        s.nsub = T / count;
        const int l = t % count;
        s.sub0 = t / count;
        s.a0 = s.sub0 < s.nsub;
        s.a1 = false;
        s.base0 = (l / nin) * so + (l % nin) * si;
        s.base1 = 0;
    }
    return s;
}

template <int P, bool INV, typename C>
__device__ __forceinline__ void stage_loop(C *buf, const LineSlot &ls, int es, int esL, int nbf, const short *off,
                                           const short *two, const C *tw) {
    if (ls.a0)
        for (int bf = ls.sub0; bf < nbf; bf += ls.nsub) butterfly<P, INV>(buf + ls.base0 + off[bf] * es, esL, tw + two[bf]);
    if (ls.a1)
        for (int bf = 0; bf < nbf; ++bf) butterfly<P, INV>(buf + ls.base1 + off[bf] * es, esL, tw + two[bf]);
}

template <bool INV, typename C>
__device__ void fft_lines(C *buf, const LineSlot &ls, int es, const FftPlan &P, const short *off, const short *two,
                          const C *tw) {
    int L = 1;
    for (int s = 0; s < P.nst; ++s) {
        const int p = P.rad[s];
        const int nbf = P.n / p, esL = L * es;
        const short *o = off + P.st0[s], *w = two + P.st0[s];
        switch (p) {
            case 2: stage_loop<2, INV>(buf, ls, es, esL, nbf, o, w, tw); break;
            case 3: stage_loop<3, INV>(buf, ls, es, esL, nbf, o, w, tw); break;
            case 4: stage_loop<4, INV>(buf, ls, es, esL, nbf, o, w, tw); break;
            case 5: stage_loop<5, INV>(buf, ls, es, esL, nbf, o, w, tw); break;
            case 7: stage_loop<7, INV>(buf, ls, es, esL, nbf, o, w, tw); break;
            case 11: stage_loop<11, INV>(buf, ls, es, esL, nbf, o, w, tw); break;
            case 13: stage_loop<13, INV>(buf, ls, es, esL, nbf, o, w, tw); break;
            default: break;
        }
        __syncthreads();
        L *= p;
    }
}

// Walk a flattened 2-D index space (rows of ``inner`` items) in steps of
// blockDim.x without division: (o, i) advances by (T / inner, T % inner).
struct Walk2 {
    int o, i, so, si, inner;
    __device__ __forceinline__ Walk2(int inner_) : inner(inner_) {
        const int T = blockDim.x, t = threadIdx.x;
        o = t / inner_;
        i = t % inner_;
        so = T / inner_;
        si = T % inner_;
    }
    __device__ __forceinline__ void next() {
        o += so;
        i += si;
        if (i >= inner) {
            i -= inner;
            ++o;
        }
    }
};

}  // namespace vg
