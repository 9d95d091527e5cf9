// k_diag.cu -- device self-checks and pipe-rate probes (not on the
// simulation path): the bit-level conversions and grid index of the
// split-precision kernels against the hardware / FP64 forms, and the
// throughput of the FP64 pipe, the converters and the FP32 FMA pipe, which
// decide where the split path may spend FP64 work.
#include "simmd_internal.cuh"

namespace simmd {

// self-check: f2d / d2f_rn against the converter, bit for bit, and the
// integer grid index against its FP64 form
__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__global__ void k_check_conversions(long long n, unsigned long long seed, unsigned long long* bad)
{
    unsigned long long nbad = 0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = mix64(seed + 0x9e3779b97f4a7c15ull * (unsigned long long)(k + 1));
        // widening: any float pattern
        const float f = __uint_as_float((unsigned)h);
        if (__double_as_longlong(f2d(f)) != __double_as_longlong((double)f)) nbad++;
        // narrowing: a double in the float range (exponent drawn over it and
        // a little beyond), the dropped bits often a tie or next to one
        unsigned long long b = h;
        const unsigned long long ef = 880ull + ((h >> 52) % 288ull);
        b = (b & 0x800fffffffffffffull) | (ef << 52);
        const int kind = (int)((h >> 40) & 7ull);
        if (kind == 0) b = (b & ~0x1fffffffull) | 0x10000000ull;          // exact tie
        else if (kind == 1) b = (b & ~0x1fffffffull) | 0x0fffffffull;     // just below
        else if (kind == 2) b = (b & ~0x1fffffffull) | 0x10000001ull;     // just above
        else if (kind == 3) b = (b & ~0xfffffffffffffull) | 0xfffffe0000000ull | (h & 0x1fffffffull);  // carry
        const double x = __longlong_as_double((long long)(kind == 4 ? h : b));  // kind 4: any pattern
        const float a = d2f_rn(x), c = (float)x;
        if (__float_as_uint(a) != __float_as_uint(c) && !(a != a && c != c)) nbad++;
        // grid index: the FP64 form floor(x/h + 0.5) clamped to [0, 1023]
        RepDesc dd = {};
        const int hk = -(int)((h >> 20) & 7ull);  // h = 2^0 .. 2^-7
        dd.h = __longlong_as_double((long long)(1023 + hk) << 52);
        const double inv_h = __longlong_as_double((long long)(1023 - hk) << 52);
        const int gk = (int)((h >> 24) & 7ull);
        double xg;
        if (gk == 0) xg = __longlong_as_double((long long)h);  // any pattern
        else if (gk == 1) xg = ((double)(long long)((h >> 27) % 2300ull) * 0.5 - 50.0) * dd.h;  // ties
        else if (gk == 2) xg = __longlong_as_double(0x3fdfffffffffffffll) * dd.h;  // 0.5 - 2^-54
        else xg = ((double)(long long)(h >> 11) * 0x1.0p-53 * 1100.0 - 30.0) * dd.h;
        const double q = floor(xg * inv_h + 0.5);
        const int gref = (q == q) ? (int)fmax(fmin(q, 1023.0), 0.0) : 0;
        if (grid_index(xg, dd) != gref) nbad++;
    }
    if (nbad) atomicAdd(bad, nbad);
}

void launch_check_conversions_impl(long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t s)
{
    k_check_conversions<<<1024, 256, 0, s>>>(n, seed, bad);
}

// ---------------------------------------------------------------------------
// pipe rates: RATE_ITERS x 4 independent chains per thread
// ---------------------------------------------------------------------------
constexpr int RATE_ITERS = 2048;

template <int OP>
__global__ void k_rate(double* out, double a, float af)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double r = 0.0;
    if (OP == 0) {  // FP64 add
        double x0 = tid, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
        for (int i = 0; i < RATE_ITERS; i++) {
            x0 = __dadd_rn(x0, a);
            x1 = __dadd_rn(x1, a);
            x2 = __dadd_rn(x2, a);
            x3 = __dadd_rn(x3, a);
        }
        r = x0 + x1 + x2 + x3;
    } else if (OP == 1 || OP == 2) {  // float -> double: converter, bit operations
        float f0 = (float)tid, f1 = f0 + 1.f, f2 = f0 + 2.f, f3 = f0 + 3.f;
        long long acc = 0;
        for (int i = 0; i < RATE_ITERS; i++) {
            if (OP == 1)
                acc ^= __double_as_longlong((double)f0) ^ __double_as_longlong((double)f1) ^
                       __double_as_longlong((double)f2) ^ __double_as_longlong((double)f3);
            else
                acc ^= __double_as_longlong(f2d(f0)) ^ __double_as_longlong(f2d(f1)) ^ __double_as_longlong(f2d(f2)) ^
                       __double_as_longlong(f2d(f3));
            f0 += af;
            f1 += af;
            f2 += af;
            f3 += af;
        }
        r = (double)acc;
    } else if (OP == 3 || OP == 4) {  // double -> float: converter, bit operations
        long long b0 = __double_as_longlong(1.0 + tid * 1e-7), b1 = b0 + 977, b2 = b0 + 1931, b3 = b0 + 2897;
        const long long step = __double_as_longlong(a) & 0xffffll;
        unsigned acc = 0;
        for (int i = 0; i < RATE_ITERS; i++) {
            const double d0 = __longlong_as_double(b0), d1 = __longlong_as_double(b1), d2 = __longlong_as_double(b2),
                         d3 = __longlong_as_double(b3);
            if (OP == 3)
                acc ^= __float_as_uint((float)d0) ^ __float_as_uint((float)d1) ^ __float_as_uint((float)d2) ^
                       __float_as_uint((float)d3);
            else
                acc ^= __float_as_uint(d2f_rn(d0)) ^ __float_as_uint(d2f_rn(d1)) ^ __float_as_uint(d2f_rn(d2)) ^
                       __float_as_uint(d2f_rn(d3));
            b0 += step;
            b1 += step;
            b2 += step;
            b3 += step;
        }
        r = (double)acc;
    } else {  // FP32 FMA
        float x0 = (float)tid, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
        for (int i = 0; i < RATE_ITERS; i++) {
            x0 = fmaf(x0, af, af);
            x1 = fmaf(x1, af, af);
            x2 = fmaf(x2, af, af);
            x3 = fmaf(x3, af, af);
        }
        r = (double)(x0 + x1 + x2 + x3);
    }
    out[tid] = r;  // one slot per thread: keeps the chains live
}

// out[k] = G operations per second of probe k (0 FP64 add, 1/2 float->double
// converter / bits, 3/4 double->float converter / bits, 5 FP32 FMA); out
// holds blocks*threads doubles of scratch
int run_pipe_rates(int blocks, int threads, double* scratch, double* gops, cudaStream_t s)
{
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return 1;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return 1;
    }
    int err = 0;
    const double ops = (double)blocks * threads * RATE_ITERS * 4.0;
    for (int rep = 0; rep < 2 && !err; rep++)  // the first pass warms up
        for (int k = 0; k < 6 && !err; k++) {
            cudaEventRecord(e0, s);
            switch (k) {
            case 0: k_rate<0><<<blocks, threads, 0, s>>>(scratch, 1e-9, 1e-3f); break;
            case 1: k_rate<1><<<blocks, threads, 0, s>>>(scratch, 1e-9, 1e-3f); break;
            case 2: k_rate<2><<<blocks, threads, 0, s>>>(scratch, 1e-9, 1e-3f); break;
            case 3: k_rate<3><<<blocks, threads, 0, s>>>(scratch, 3.0e-300, 1e-3f); break;
            case 4: k_rate<4><<<blocks, threads, 0, s>>>(scratch, 3.0e-300, 1e-3f); break;
            default: k_rate<5><<<blocks, threads, 0, s>>>(scratch, 1e-9, 0.999f); break;
            }
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
                err = 1;
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep == 1) gops[k] = ms > 0.f ? ops / ((double)ms * 1e6) : 0.0;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return err;
}

}  // namespace simmd
