// Library-wide host helpers: error reporting, FFT plans, small queries.
#include <cstring>
#include <string>

#include "vesper_common.cuh"

namespace vg {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_check(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(VESPER_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return VESPER_OK;
}

bool make_plan(int n, FftPlan *plan) {
    if (n < 1) return false;
    int rad[64], k = 0, m = n;
    while (m % 4 == 0) { rad[k++] = 4; m /= 4; }
    while (m % 2 == 0) { rad[k++] = 2; m /= 2; }
    int big = 0;
    const int primes[] = {3, 5, 7, 11, 13};
    for (int p : primes)
        while (m % p == 0) {
            if (p >= 11) ++big;
            rad[k++] = p;
            m /= p;
        }
    if (m != 1 || big > 1 || k > kMaxStages) return false;
    plan->n = n;
    plan->nst = k;
    int acc = 0;
    for (int i = 0; i < k; ++i) {
        plan->rad[i] = rad[i];
        plan->st0[i] = acc;
        acc += n / rad[i];
    }
    plan->ntab = acc;
    if (n == 1) { plan->nst = 0; plan->ntab = 0; }
    return true;
}

}  // namespace vg

extern "C" int vesper_version(void) { return 100; }

extern "C" const char *vesper_last_error(void) { return vg::g_last_error.c_str(); }

extern "C" int vesper_fast_len_ok(int n) {
    vg::FftPlan p;
    return (n >= 2 && vg::make_plan(n, &p)) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// FP32 FMA throughput probe: the measured denominator of the search kernels'
// FP32 roofline.  Every thread runs kChains independent fmaf chains for
// ``iters`` steps (2 flops each); the sum is stored only when it equals a
// value no chain reaches, so the chains stay live without a store per thread.
// ---------------------------------------------------------------------------
namespace vg {
constexpr int kChains = 16;

__global__ void k_fma_peak(float *out, int iters) {
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = (threadIdx.x + 1) * 1e-6f + k * 1e-7f;
    const float b = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == -1.0f) out[blockIdx.x] = s;
}
}  // namespace vg

extern "C" int vesper_fp32_peak_probe(int blocks, int threads, int iters, float *out, double *flops_out,
                                      void *stream) {
    if (blocks < 1 || threads < 32 || threads > 1024 || threads % 32 || iters < 1 || !out || !flops_out)
        return vg::fail(VESPER_ERR_INVALID, "vesper_fp32_peak_probe: bad arguments");
    vg::k_fma_peak<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters);
    *flops_out = 2.0 * vg::kChains * (double)iters * threads * blocks;
    return vg::cuda_check("k_fma_peak");
}
